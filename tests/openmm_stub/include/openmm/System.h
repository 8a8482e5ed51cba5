// Stand-in for OpenMM's openmm/System.h (test infrastructure).
#pragma once
#include "openmm/Vec3.h"

namespace OpenMM {
class System {
 public:
  int addParticle(double) { return n_++; }
  int getNumParticles() const { return n_; }
  void setDefaultPeriodicBoxVectors(const Vec3& a, const Vec3& b, const Vec3& c) {
    a_ = a;
    b_ = b;
    c_ = c;
  }
  void getDefaultPeriodicBoxVectors(Vec3& a, Vec3& b, Vec3& c) const {
    a = a_;
    b = b_;
    c = c_;
  }

 private:
  int n_ = 0;
  Vec3 a_{2.0, 0.0, 0.0}, b_{0.0, 2.0, 0.0}, c_{0.0, 0.0, 2.0};
};
}  // namespace OpenMM
