// Stand-in for OpenMM's openmm/Platform.h (test infrastructure): a registry
// of platforms and the kernel factories registered on them.
#pragma once
#include <map>
#include <string>
#include <vector>

namespace OpenMM {
class KernelFactory;

class Platform {
 public:
  virtual ~Platform() = default;
  static std::vector<Platform*>& registry() {
    static std::vector<Platform*> r;
    return r;
  }
  static int getNumPlatforms() { return (int)registry().size(); }
  static Platform& getPlatform(int index) { return *registry()[index]; }
  static void registerPlatform(Platform* p) { registry().push_back(p); }
  void registerKernelFactory(const std::string& name, KernelFactory* factory) { factories[name] = factory; }
  std::map<std::string, KernelFactory*> factories;
};
}  // namespace OpenMM
