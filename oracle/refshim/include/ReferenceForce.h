// Stand-in for OpenMM's ReferenceForce distance helpers (getDeltaR returns
// b - a with R2 = dot and R = sqrt(R2)).  Written for this repository.
#ifndef REFSHIM_REFERENCEFORCE_H
#define REFSHIM_REFERENCEFORCE_H
#include <cmath>
#include "Vec3.h"
namespace OpenMM {
class ReferenceForce {
 public:
  static const int XIndex = 0, YIndex = 1, ZIndex = 2, R2Index = 3, RIndex = 4, LastDeltaRIndex = 5;
  static void getDeltaR(const Vec3& a, const Vec3& b, double* d) {
    d[XIndex] = b[0] - a[0];
    d[YIndex] = b[1] - a[1];
    d[ZIndex] = b[2] - a[2];
    d[R2Index] = d[XIndex] * d[XIndex] + d[YIndex] * d[YIndex] + d[ZIndex] * d[ZIndex];
    d[RIndex] = std::sqrt(d[R2Index]);
  }
  static void getDeltaRPeriodic(const Vec3& a, const Vec3& b, const Vec3* box, double* d) {
    Vec3 diff = b - a;
    diff -= box[2] * std::floor(diff[2] / box[2][2] + 0.5);
    diff -= box[1] * std::floor(diff[1] / box[1][1] + 0.5);
    diff -= box[0] * std::floor(diff[0] / box[0][0] + 0.5);
    d[XIndex] = diff[0];
    d[YIndex] = diff[1];
    d[ZIndex] = diff[2];
    d[R2Index] = diff.dot(diff);
    d[RIndex] = std::sqrt(d[R2Index]);
  }
};
}  // namespace OpenMM
#endif
