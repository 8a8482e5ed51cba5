// Stand-in for OpenMM's CUDA platform CudaContext (test infrastructure): the
// members a force kernel reads each step, settable by a test driver.
#pragma once
#include <cuda.h>

#include <map>
#include <string>
#include <vector>

#include "CudaArray.h"

namespace OpenMM {
// OpenMM returns the box edges as CUDA's double4 (x, y, z, unused).
struct BoxSize {
  double x, y, z, w;
};

class CudaContext {
 public:
  void setAsCurrent() { ++current_calls; }
  CudaArray& getPosq() { return posq; }
  CudaArray& getForce() { return force; }
  CudaArray& getEnergyBuffer() { return energy; }
  int getNumAtoms() const { return numAtoms; }
  int getPaddedNumAtoms() const { return paddedNumAtoms; }
  bool getUseDoublePrecision() const { return useDouble; }
  bool getUseMixedPrecision() const { return useMixed; }
  const std::vector<int>& getAtomIndex() const { return atomIndex; }
  bool getAtomsWereReordered() const { return reordered; }
  BoxSize getPeriodicBoxSize() const { return box; }
  CUstream getCurrentStream() { return stream; }
  // energy parameter derivatives: the names a force registers, and the
  // context's workspace for derivatives formed outside its own kernels
  void addEnergyParameterDerivative(const std::string& name) { paramDerivNames.push_back(name); }
  std::map<std::string, double>& getEnergyParamDerivWorkspace() { return paramDerivWorkspace; }

  // test controls
  CudaArray posq, force, energy;
  int numAtoms = 0, paddedNumAtoms = 0;
  bool useDouble = false, useMixed = false, reordered = false;
  std::vector<int> atomIndex;
  BoxSize box{2.0, 2.0, 2.0, 0.0};
  CUstream stream = nullptr;
  int current_calls = 0;
  std::vector<std::string> paramDerivNames;
  std::map<std::string, double> paramDerivWorkspace;
};
}  // namespace OpenMM
