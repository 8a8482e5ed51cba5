// OpenMM CUDA-platform kernels for CharmmGBSWForce and CharmmGBMVForce on
// the gbx C ABI (include/gbx.h).
//
// They implement the plugin's kernel interfaces (openmmapi/include/openmm/
// charmmKernels.h:49-129 in the reference plugin) and replace its CUDA
// kernel (platforms/cuda/src/CharmmCudaKernels.cpp:845-993): one gbx_context
// per force instance, evaluated on OpenMM's own device buffers -- posq
// (float4, or double4 in double precision), the 64-bit fixed-point force
// buffer and the energy buffer (float in single precision) -- on the
// context's current stream.  OpenMM's atom reordering is handed to the
// library as an atom order, so parameters stay in atom order and results do
// not depend on it.  Calls never synchronise the stream; a lookup table that
// outgrew its buffers in one step is reported by a later step as an
// OpenMMException rather than passing silently.
#pragma once

#include <string>
#include <vector>

#include "CudaContext.h"
#include "gbx.h"
#include "openmm/charmmKernels.h"

namespace GB300 {

// State and per-step work shared by both force kernels.
class GbxForceState {
 public:
  explicit GbxForceState(OpenMM::CudaContext& cu) : cu(cu) {}
  ~GbxForceState();
  GbxForceState(const GbxForceState&) = delete;
  GbxForceState& operator=(const GbxForceState&) = delete;

  void create(const gbx_config& cfg, int numAtoms);
  void setParameters(const std::vector<double>& charge, const std::vector<double>& radius);
  void setGlobals(double alpha0, double alpha1);
  void createCustom(const gbx_config& cfg, int numAtoms, const gbx_custom& custom);
  void setCustomParameters(const std::vector<double>& params);  // [n][num_params]
  void setCustomGlobal(int index, const std::string& name, double value);
  void setBox(double a, double b, double c);
  // One evaluation on OpenMM's buffers; the energy is added to OpenMM's
  // energy buffer, so the kernel returns 0 as the reference CUDA kernel does.
  double execute(bool includeForces, bool includeEnergy);
  void check(gbx_status status, const char* what) const;

  OpenMM::CudaContext& cu;
  gbx_context* handle = nullptr;
  int numAtoms = 0;

 private:
  bool orderSet = false;
  double globals[2] = {0.0, 0.0};
  std::vector<double> customGlobals;
  double box[3] = {0.0, 0.0, 0.0};
};

class GB300CalcCharmmGBSWForceKernel : public OpenMM::CalcCharmmGBSWForceKernel {
 public:
  GB300CalcCharmmGBSWForceKernel(std::string name, const OpenMM::Platform& platform, OpenMM::CudaContext& cu)
      : OpenMM::CalcCharmmGBSWForceKernel(name, platform), state(cu) {}
  void initialize(const OpenMM::System& system, const OpenMM::CharmmGBSWForce& force) override;
  double execute(OpenMM::ContextImpl& context, bool includeForces, bool includeEnergy) override;
  void copyParametersToContext(OpenMM::ContextImpl& context, const OpenMM::CharmmGBSWForce& force) override;

 private:
  void copyParameters(const OpenMM::CharmmGBSWForce& force);
  GbxForceState state;
  bool periodic = false;
};

class GB300CalcCharmmGBMVForceKernel : public OpenMM::CalcCharmmGBMVForceKernel {
 public:
  GB300CalcCharmmGBMVForceKernel(std::string name, const OpenMM::Platform& platform, OpenMM::CudaContext& cu)
      : OpenMM::CalcCharmmGBMVForceKernel(name, platform), state(cu) {}
  void initialize(const OpenMM::System& system, const OpenMM::CharmmGBMVForce& force) override;
  double execute(OpenMM::ContextImpl& context, bool includeForces, bool includeEnergy) override;
  void copyParametersToContext(OpenMM::ContextImpl& context, const OpenMM::CharmmGBMVForce& force) override;

 private:
  void copyParameters(const OpenMM::CharmmGBMVForce& force);
  GbxForceState state;
  int chargeIndex = -1, radiusIndex = -1;
  std::string alphaNames[2];
  bool custom = false;                    // expressions outside the canonical set
  std::vector<std::string> globalNames;   // the force's global parameters (custom)
  std::vector<std::string> paramDerivNames;  // addEnergyParameterDerivative (custom)
};

// Whether the force uses the canonical CHARMM expression set (parameters q
// and radius, integrals I4 {4} and I7 {7}, the computed value B and the
// self and pair energy terms), which the library's fixed kernels evaluate;
// other sets are compiled for the device (gbx_create_custom).  Throws for
// what neither path supports (CustomIntegral, a missing "radius", an
// integral of order below 2).
bool isCanonicalGBMVForce(const OpenMM::CharmmGBMVForce& force, int& chargeIndex, int& radiusIndex);

}  // namespace GB300
