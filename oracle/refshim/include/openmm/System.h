#ifndef REFSHIM_SYSTEM_H
#define REFSHIM_SYSTEM_H
#include <vector>
#include "../Vec3.h"
namespace OpenMM {
class System {
 public:
  explicit System(int n = 0) : n_(n) {}
  int getNumParticles() const { return n_; }
 private:
  int n_;
};
}  // namespace OpenMM
#endif
