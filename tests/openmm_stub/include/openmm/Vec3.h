// Stand-in for OpenMM's openmm/Vec3.h (test infrastructure).
#pragma once

namespace OpenMM {
class Vec3 {
 public:
  Vec3() : d{0.0, 0.0, 0.0} {}
  Vec3(double x, double y, double z) : d{x, y, z} {}
  double operator[](int k) const { return d[k]; }
  double& operator[](int k) { return d[k]; }

 private:
  double d[3];
};
}  // namespace OpenMM
