// Stand-in for OpenMM's openmm/KernelFactory.h (test infrastructure).
#pragma once
#include <string>

#include "openmm/KernelImpl.h"

namespace OpenMM {
class ContextImpl;

class KernelFactory {
 public:
  virtual ~KernelFactory() = default;
  virtual KernelImpl* createKernelImpl(std::string name, const Platform& platform, ContextImpl& context) const = 0;
};
}  // namespace OpenMM
