// Stand-in for OpenMM's openmm/internal/ContextImpl.h (test infrastructure):
// the system, the platform data and the global parameters.
#pragma once
#include <map>
#include <string>

#include "openmm/OpenMMException.h"
#include "openmm/System.h"

namespace OpenMM {
class ContextImpl {
 public:
  ContextImpl(System& system, void* platformData) : system_(system), data_(platformData) {}
  const System& getSystem() const { return system_; }
  void* getPlatformData() { return data_; }
  double getParameter(const std::string& name) const {
    auto it = params_.find(name);
    if (it == params_.end()) throw OpenMMException("Called getParameter() with invalid parameter name: " + name);
    return it->second;
  }
  void setParameter(const std::string& name, double value) { params_[name] = value; }

 private:
  System& system_;
  void* data_;
  std::map<std::string, double> params_;
};
}  // namespace OpenMM
