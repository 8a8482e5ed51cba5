#ifndef REFSHIM_REALTYPE_H
#define REFSHIM_REALTYPE_H
// OpenMM 7.x value of 1/(4 pi eps0) in kJ nm / (mol e^2).
#define ONE_4PI_EPS0 138.935456
#endif
