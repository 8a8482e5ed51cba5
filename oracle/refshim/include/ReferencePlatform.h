#ifndef REFSHIM_REFERENCEPLATFORM_H
#define REFSHIM_REFERENCEPLATFORM_H
#include "Vec3.h"
namespace OpenMM {
class ReferencePlatform {
 public:
  class PlatformData {
   public:
    Vec3* periodicBoxVectors;
  };
};
}  // namespace OpenMM
#endif
