/*
 * FP64 CPU oracle for the CHARMM GBSW / GBMV hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  The CUDA path's results are compared against
 * it; nothing in the product links, loads or calls it.  Only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg use it.
 *
 * It restates the reference's CPU algorithms (file:line citations are into
 * the reference project ymwangg/OpenMMCustomGBIntegralForce) in plain C with
 * double arithmetic, parameterised where the reference hard-codes constants,
 * and without the reference's O(N^2) gradient storage.  It is pinned against
 * the reference classes compiled in place (oracle/refshim) and against the
 * golden vectors in tests/golden.
 *
 * Build with -ffp-contract=off so that no multiply-add is fused: the lookup
 * table membership tests must round exactly as the reference's do.
 */
#ifndef GBX_ORACLE_H
#define GBX_ORACLE_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_GBSW = 0, ORC_GBMV1 = 1, ORC_GBMV2 = 2 };
enum {
  ORC_TABLE_STANDALONE = 0, /* CharmmReferenceGBSW.cpp:440-552 (uniform pad, uncapped) */
  ORC_TABLE_GRID = 1,       /* CustomGBIntegral.cpp:162-228,310-324 (per-atom pad, capped) */
  ORC_TABLE_PERIODIC = 2    /* CustomGBIntegral.cpp:45-160,284-309 (box-sampled, capped) */
};

typedef struct {
  int model;          /* ORC_GBSW / ORC_GBMV1 / ORC_GBMV2 */
  /* tensor-product quadrature, index q = ir*nS + is */
  int nq;
  const double* qoff; /* [nq*3] */
  const double* qrad; /* [nq]   */
  const double* qw;   /* [nq]   */
  /* integrals: order n -> weight w / r^(n-2) (GBSWIntegral.cpp:96,144) */
  int n_int;
  int orders[4];
  /* lookup table */
  int table_mode;
  double h;           /* grid length (0.15 nm) */
  double buffer;      /* standalone: 0.20; grid: 0.04 GBSW / 0.21 GBMV */
  int cap;            /* per-cell cap, <= 0 means uncapped */
  double box[3];      /* periodic-sampled table only */
  /* volume-model constants */
  double sw;          /* GBSW switching half-width 0.03 nm */
  double gamma0, beta, lambda, p1, p2, s0;
  /* energy */
  double r0;          /* eta = 0.05 nm */
  double alpha0, alpha1;
  double pref;        /* -ONE_4PI_EPS0*(1-1/80), CharmmReferenceGBSW.cpp:177-178 */
  int use_cutoff;
  double cutoff;
  int cutoff_chain_quirk; /* drop chain-rule terms for |xi-xk|>rc, CharmmReferenceGBSW.cpp:291-292 */
  int skip_empty;     /* GBSW: empty list -> point skipped (V=1) */
  int standalone_sums; /* accumulate as CharmmReferenceGBSW.cpp:586-589 ((w*f)/(r*r), (w*f)/r^5 by
                          repeated products) instead of GBSWIntegral.cpp:144-145 (w/pow(r,n-2))*f */
  int nthreads;       /* OpenMP threads, <= 0 -> all */
  int atom_stride;    /* timing samples: only atoms i % stride == 0 run their
                         points, chain rule and pair rows (<= 1: all atoms).
                         The results are then partial; the cost scales by stride. */
  int periodic;       /* CutoffPeriodic (rectangular box[3]): every distance by minimum
                         image (ReferenceForce::getDeltaRPeriodic, CharmmReferenceGBSW.cpp:
                         242-243,287-288,620-621,647-648), the standalone table's query
                         point wrapped once per axis (:522-535) */
} orc_config;

typedef struct {
  int mode;
  int dims[3];
  double min[3], max[3], step[3], box[3];
  double pad;       /* standalone: uniform membership radius */
  int64_t ncell;
  int32_t* count;   /* [ncell] entries kept (capped) */
  int64_t* start;   /* [ncell+1] CSR offsets into atoms */
  int32_t* atoms;   /* ascending insertion order per cell */
  int64_t dropped;  /* insertions refused by the cap */
  int64_t oob;      /* membership hits whose flat index fell outside the table */
  int wrap;         /* standalone table of a periodic system: queries wrap once per axis */
} orc_table;

typedef struct {
  double volume_evals;   /* (point, listed atom) pairs visited, reference order */
  double shell_evals;    /* of which inside the switching shell (GBSW) */
  double points;         /* (atom, quadrature point) pairs with a non-empty list */
  double active_points;  /* points with 0 < V < 1 (GBSW) */
  double chain_pairs;    /* (point, atom) pairs in the chain rule */
  double pairs;          /* pair-term pairs evaluated */
} orc_work;

int orc_table_build(const orc_config* cfg, int n, const double* pos, const double* radius, orc_table* t);
void orc_table_free(orc_table* t);
/* flat cell index of a point or -1 for "no list" (outside the grid) */
int64_t orc_table_query(const orc_table* t, const double p[3]);

/* Integrals I_k[k*n+i] (GBSWIntegral.cpp:119-157, GBMVIntegralTypeI.cpp:111-152,
 * GBMVIntegralTypeII.cpp:116-160). */
int orc_integrals(const orc_config* cfg, const orc_table* t, int n, const double* pos,
                  const double* radius, double* integrals, orc_work* work);

/* Chain rule: forces[j] -= sum_{i,k} dEdI[k*n+i] * dI_k[i]/dx_j, accumulated
 * point by point instead of through the dense N x N x 3 gradient. */
int orc_integral_chain(const orc_config* cfg, const orc_table* t, int n, const double* pos,
                       const double* radius, const double* dEdI, double* forces, orc_work* work);

/* Full energy + forces for the canonical CHARMM GB expression:
 *   1/B = alpha0 (1/r0 - I4) + alpha1 (1/(4 r0^4) - I7)^(1/4)
 *   E   = sum_{i<j} pref q_i q_j / f_ij + 1/2 sum_i pref q_i^2 / B_i
 * (CharmmReferenceGBSW.cpp:169-299, 554-674).  Requires n_int == 2 with orders
 * {4, 7}.  Optional outputs may be NULL.  Adjoint outputs: dE/dq, dE/dR_in,
 * dE/dalpha[2]. */
int orc_energy_forces(const orc_config* cfg, int n, const double* pos, const double* charge,
                      const double* radius, double* energy, double* forces, double* born,
                      double* integrals, double* dEdB, double* dEdq, double* dEdR,
                      double* dEdalpha, orc_work* work);

/* The pair term alone for given Born radii B (CharmmReferenceGBSW.cpp:237-283):
 * pair energy (self terms included), pair forces [n*3], dE/dB, dE/dq, all
 * ADDED to; outputs other than energy may be NULL. */
int orc_pair_terms(const orc_config* cfg, int n, const double* pos, const double* charge, const double* B,
                   double* energy, double* forces, double* dEdB, double* dEdq, orc_work* work);

#ifdef __cplusplus
}
#endif
#endif
