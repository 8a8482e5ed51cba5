#ifndef REFSHIM_NEIGHBORLIST_H
#define REFSHIM_NEIGHBORLIST_H
#include <utility>
#include <vector>
namespace OpenMM {
typedef std::vector<std::pair<int, int> > NeighborList;
}
#endif
