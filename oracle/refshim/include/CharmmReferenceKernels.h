// Stand-in for the reference's CharmmReferenceKernels.h: the real one pulls
// in Lepton and the OpenMM kernel framework, none of which the GBSW engine
// needs.  It only has to provide what CharmmReferenceGBSW.h expects in scope.
#ifndef REFSHIM_CHARMMREFERENCEKERNELS_H
#define REFSHIM_CHARMMREFERENCEKERNELS_H
#include <cassert>
#include <vector>
#include "Vec3.h"
#include "ReferenceNeighborList.h"
#endif
