// Stand-in for the plugin's openmm/charmmKernels.h (test infrastructure):
// the two kernel interfaces of charmmKernels.h:49-129 in the reference
// plugin, which a GB300 kernel implements.
#pragma once
#include <string>

#include "openmm/CharmmGBMVForce.h"
#include "openmm/CharmmGBSWForce.h"
#include "openmm/KernelImpl.h"
#include "openmm/System.h"
#include "openmm/internal/ContextImpl.h"

namespace OpenMM {
class CalcCharmmGBMVForceKernel : public KernelImpl {
 public:
  static std::string Name() { return "CalcCharmmGBMVForce"; }
  CalcCharmmGBMVForceKernel(std::string name, const Platform& platform) : KernelImpl(name, platform) {}
  virtual void initialize(const System& system, const CharmmGBMVForce& force) = 0;
  virtual double execute(ContextImpl& context, bool includeForces, bool includeEnergy) = 0;
  virtual void copyParametersToContext(ContextImpl& context, const CharmmGBMVForce& force) = 0;
};

class CalcCharmmGBSWForceKernel : public KernelImpl {
 public:
  static std::string Name() { return "CalcCharmmGBSWForce"; }
  CalcCharmmGBSWForceKernel(std::string name, const Platform& platform) : KernelImpl(name, platform) {}
  virtual void initialize(const System& system, const CharmmGBSWForce& force) = 0;
  virtual double execute(ContextImpl& context, bool includeForces, bool includeEnergy) = 0;
  virtual void copyParametersToContext(ContextImpl& context, const CharmmGBSWForce& force) = 0;
};
}  // namespace OpenMM
