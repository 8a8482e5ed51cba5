#ifndef REFSHIM_UNITS_H
#define REFSHIM_UNITS_H
namespace OpenMM {
static const double NmPerAngstrom = 0.1;
static const double AngstromsPerNm = 10.0;
}
#endif
