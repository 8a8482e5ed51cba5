// C entry points around the reference's own CPU classes, compiled in place
// from the reference tree by oracle/Makefile.ref.  TEST INFRASTRUCTURE ONLY:
// used to pin the FP64 oracle and to write the golden fixtures.  Nothing here
// is part of the product.
#include <cmath>
#include <cstring>
#include <iostream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "Vec3.h"
#include "ReferenceNeighborList.h"
#include "ReferencePlatform.h"
#include "openmm/OpenMMException.h"
#include "openmm/System.h"
#include "openmm/internal/ContextImpl.h"
#include "openmm/CharmmGBMVForce.h"
#include "openmm/internal/CharmmQuadrature.h"

// The table arrays are private members; read them for comparison.
#define private public
#define protected public
#include "CharmmReferenceKernels.h"
#include "CharmmReferenceGBSW.h"
#include "CustomGBIntegral.h"
#include "GBSWIntegral.h"
#include "GBMVIntegralTypeI.h"
#include "GBMVIntegralTypeII.h"
#undef private
#undef protected

using OpenMM::Vec3;

static std::vector<Vec3> to_vec3(int n, const double* p) {
  std::vector<Vec3> v(n);
  for (int i = 0; i < n; ++i) v[i] = Vec3(p[3 * i], p[3 * i + 1], p[3 * i + 2]);
  return v;
}

extern "C" {

int ref_gauss_legendre(double x0, double x1, int n, double* x, double* w) {
  std::vector<std::vector<double> > g = CharmmQuadrature::GaussLegendre(x0, x1, n);
  for (int i = 0; i < n; ++i) {
    x[i] = g[i][0];
    w[i] = g[i][1];
  }
  return 0;
}

// Lebedev rule by rule index; returns the number of points written to xyzw.
int ref_lebedev(int rule, double* xyzw, int cap) {
  std::vector<std::vector<double> > s = CharmmQuadrature::Lebedev(rule);
  if ((int)s.size() > cap) return -1;
  for (size_t i = 0; i < s.size(); ++i)
    for (int k = 0; k < 4; ++k) xyzw[4 * i + k] = s[i][k];
  return (int)s.size();
}

// Copy of the quadrature a CharmmReferenceGBSW instance builds (q*5: x y z r w).
int ref_gbsw_quadrature(double* out, int cap) {
  OpenMM::CharmmReferenceGBSW g(1);
  if ((int)g._quad.size() > cap) return -1;
  for (size_t q = 0; q < g._quad.size(); ++q)
    for (int k = 0; k < 5; ++k) out[5 * q + k] = g._quad[q][k];
  return (int)g._quad.size();
}

namespace {
// CharmmGBSWForce on the Reference platform: energy, forces (added to zero),
// Born radii.  A fresh engine per call (the reference does not reset its
// accumulators between calls).  cutoff < 0 means NoCutoff; box (rectangular
// edge lengths) non-null means CutoffPeriodic.
double gbsw_run(int n, const double* pos, const double* charge, const double* radius, double cutoff,
                const double* box, double* forces, double* born) {
  std::vector<Vec3> x = to_vec3(n, pos);
  std::vector<double> q(charge, charge + n), R(radius, radius + n), sf(n, 1.0);
  Vec3 vectors[3] = {Vec3(0, 0, 0), Vec3(0, 0, 0), Vec3(0, 0, 0)};
  if (box)
    for (int k = 0; k < 3; ++k) vectors[k][k] = box[k];
  OpenMM::NeighborList nl;
  OpenMM::CharmmReferenceGBSW g(n);
  g.setAtomicRadii(R);
  g.setScaledRadiusFactors(sf);
  g.setSolventDielectric(80.0);
  g.setSoluteDielectric(1.0);
  g.setNeighborList(nl);
  if (cutoff > 0) {
    g.setUseCutoff(cutoff);
    // every pair i<j: the engine itself drops r > cutoff (by minimum image when periodic)
    for (int i = 0; i < n; ++i)
      for (int j = i + 1; j < n; ++j) nl.push_back(std::make_pair(i, j));
  } else {
    g.setNoCutoff();
  }
  if (box) g.setPeriodic(vectors);
  else g.setNoPeriodic();
  std::vector<Vec3> f(n);
  double e = g.computeEnergyForces(x, q, f);
  for (int i = 0; i < n; ++i)
    for (int k = 0; k < 3; ++k) forces[3 * i + k] = f[i][k];
  if (born) {
    OpenMM::CharmmReferenceGBSW g2(n);
    g2.setAtomicRadii(R);
    g2.setScaledRadiusFactors(sf);
    if (box) {  // the engine wants a cutoff before a box; Born radii do not use it
      g2.setUseCutoff(cutoff);
      g2.setPeriodic(vectors);
    } else {
      g2.setNoCutoff();
      g2.setNoPeriodic();
    }
    g2.computeLookupTable(x);
    std::vector<double> b(n);
    g2.computeBornRadiiFast(x, q, b);
    for (int i = 0; i < n; ++i) born[i] = b[i];
  }
  return e;
}
}  // namespace

double ref_gbsw_energy_forces(int n, const double* pos, const double* charge, const double* radius,
                              double cutoff, double* forces, double* born) {
  return gbsw_run(n, pos, charge, radius, cutoff, nullptr, forces, born);
}

// The same with a rectangular periodic box (CutoffPeriodic).
double ref_gbsw_energy_forces_periodic(int n, const double* pos, const double* charge, const double* radius,
                                       double cutoff, const double* box, double* forces, double* born) {
  return gbsw_run(n, pos, charge, radius, cutoff, box, forces, born);
}

// Lookup table of CharmmReferenceGBSW: dims[3], min[3], counts[ncell] and the
// concatenated lists (ascending cell order).  Returns total entries or -needed.
long ref_gbsw_table(int n, const double* pos, const double* radius, int* dims, double* mn, int* counts,
                    long counts_cap, int* atoms, long atoms_cap) {
  std::vector<Vec3> x = to_vec3(n, pos);
  OpenMM::CharmmReferenceGBSW g(n);
  g.setAtomicRadii(std::vector<double>(radius, radius + n));
  g.computeLookupTable(x);
  long ncell = (long)g._lookupTable.size();
  for (int k = 0; k < 3; ++k) {
    dims[k] = g._lookupTableNumberOfGridPoints[k];
    mn[k] = g._lookupTableMinCoordinate[k];
  }
  long total = 0;
  for (long c = 0; c < ncell; ++c) total += (long)g._lookupTable[c].size();
  if (ncell > counts_cap || total > atoms_cap) return -total - 1;
  long o = 0;
  for (long c = 0; c < ncell; ++c) {
    counts[c] = (int)g._lookupTable[c].size();
    for (int a : g._lookupTable[c]) atoms[o++] = a;
  }
  return total;
}

struct IntegralRun {
  OpenMM::CustomGBIntegral* impl = nullptr;
  OpenMM::CharmmGBMVForce force;
  Vec3 box[3];
  OpenMM::ReferencePlatform::PlatformData data;
  OpenMM::ContextImpl* ctx = nullptr;
  ~IntegralRun() {
    delete impl;
    delete ctx;
  }
};

// type: 0 GBSWIntegral, 1 GBMVIntegralTypeI, 2 GBMVIntegralTypeII.
// box != NULL supplies the context's periodic box (the GBMV classes always
// read it; GBSWIntegral only with CutoffPeriodic).
static IntegralRun* make_integral(int type, int n, const double* radius, int n_int, const int* orders,
                                  const double* box, bool periodic = false) {
  IntegralRun* r = new IntegralRun();
  if (periodic) r->force.method = OpenMM::CharmmGBMVForce::CutoffPeriodic;  // minimum-image distances
  for (int i = 0; i < n; ++i) r->force.particles.push_back(std::vector<double>(1, radius[i]));
  for (int k = 0; k < n_int; ++k) r->force.integralOrders.push_back(std::vector<int>(1, orders[k]));
  double b[3] = {10.0, 10.0, 10.0};
  if (box) memcpy(b, box, sizeof(b));
  r->box[0] = Vec3(b[0], 0, 0);
  r->box[1] = Vec3(0, b[1], 0);
  r->box[2] = Vec3(0, 0, b[2]);
  r->data.periodicBoxVectors = r->box;
  r->ctx = new OpenMM::ContextImpl(&r->data);
  if (type == 0) r->impl = new OpenMM::GBSWIntegral();
  else if (type == 1) r->impl = new OpenMM::GBMVIntegralTypeI();
  else r->impl = new OpenMM::GBMVIntegralTypeII();
  OpenMM::System sys(n);
  r->impl->initialize(sys, r->force);
  return r;
}

// Integrals [n_int*n] and, if grads != NULL, the dense gradient
// [n_int][n][n][3] the reference produces.
int ref_integral_evaluate(int type, int n, const double* pos, const double* radius, int n_int, const int* orders,
                          const double* box, double* integrals, double* grads) {
  try {
    IntegralRun* r = make_integral(type, n, radius, n_int, orders, box);
    std::vector<Vec3> x = to_vec3(n, pos);
    std::vector<double> I(n_int * n), G((size_t)n_int * n * n * 3);
    r->impl->BeforeComputation(*r->ctx, x);
    r->impl->evaluate(*r->ctx, x, I, G, true);
    memcpy(integrals, I.data(), sizeof(double) * I.size());
    if (grads) memcpy(grads, G.data(), sizeof(double) * G.size());
    delete r;
    return 0;
  } catch (std::exception& e) {
    std::cerr << "ref_integral_evaluate: " << e.what() << std::endl;
    return -1;
  }
}

// The same for a CharmmGBMVForce with CutoffPeriodic: the integral classes
// then measure point-to-atom distances by minimum image (and GBSWIntegral
// switches to the box-sampled table).
int ref_integral_evaluate_periodic(int type, int n, const double* pos, const double* radius, int n_int,
                                   const int* orders, const double* box, double* integrals) {
  try {
    IntegralRun* r = make_integral(type, n, radius, n_int, orders, box, true);
    std::vector<Vec3> x = to_vec3(n, pos);
    std::vector<double> I(n_int * n), G((size_t)n_int * n * n * 3);
    r->impl->BeforeComputation(*r->ctx, x);
    r->impl->evaluate(*r->ctx, x, I, G, false);
    memcpy(integrals, I.data(), sizeof(double) * I.size());
    delete r;
    return 0;
  } catch (std::exception& e) {
    std::cerr << "ref_integral_evaluate_periodic: " << e.what() << std::endl;
    return -1;
  }
}

// The integral classes' table after BeforeComputation: dims, min, step,
// counts (capped) and lists.
long ref_integral_table(int type, int n, const double* pos, const double* radius, const double* box, int* dims,
                        double* mn, double* step, int* counts, long counts_cap, int* atoms, long atoms_cap) {
  int orders[1] = {4};
  IntegralRun* r = make_integral(type, n, radius, 1, orders, box);
  std::vector<Vec3> x = to_vec3(n, pos);
  r->impl->BeforeComputation(*r->ctx, x);
  OpenMM::CustomGBIntegral* b = r->impl;
  long ncell = (long)b->_lookupTableNumAtoms.size();
  for (int k = 0; k < 3; ++k) {
    dims[k] = b->_lookupTableNumberOfGridPoints[k];
    mn[k] = b->_lookupTableMinCoordinate[k];
    step[k] = b->_periodic ? b->_lookupTableGridStep[k] : b->_lookupTableGridLength;
  }
  long total = 0;
  for (long c = 0; c < ncell; ++c) total += b->_lookupTableNumAtoms[c];
  if (ncell > counts_cap || total > atoms_cap) {
    delete r;
    return -total - 1;
  }
  long o = 0;
  for (long c = 0; c < ncell; ++c) {
    counts[c] = b->_lookupTableNumAtoms[c];
    for (int m = 0; m < counts[c]; ++m) atoms[o++] = b->_lookupTable[c][m];
  }
  delete r;
  return total;
}

}  // extern "C"
