// Stand-in for OpenMM's openmm/KernelImpl.h (test infrastructure).
#pragma once
#include <string>

#include "openmm/Platform.h"

namespace OpenMM {
class KernelImpl {
 public:
  KernelImpl(std::string name, const Platform& platform) : name_(name), platform_(&platform) {}
  virtual ~KernelImpl() = default;
  const std::string& getName() const { return name_; }
  const Platform& getPlatform() { return *platform_; }

 private:
  std::string name_;
  const Platform* platform_;
};
}  // namespace OpenMM
