/*
 * FP64 CPU oracle for the CHARMM GBSW / GBMV hot path -- TEST INFRASTRUCTURE.
 * See gbx_oracle.h for the contract.  Every function cites the reference file
 * and lines it restates (paths within ymwangg/OpenMMCustomGBIntegralForce).
 */
#include "gbx_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_MAX_LIST 4096

/* ReferenceForce::getDeltaR(a, b): b - a, R2 = dot, R = sqrt(R2) (OpenMM). */
static inline double delta_r(const double* a, const double* b, double d[3]) {
  d[0] = b[0] - a[0];
  d[1] = b[1] - a[1];
  d[2] = b[2] - a[2];
  double r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
  return sqrt(r2);
}

/* The same, by minimum image in a rectangular box when the system is periodic
 * (ReferenceForce::getDeltaRPeriodic: d -= L floor(d / L + 1/2) per axis). */
static inline double delta_cfg(const orc_config* cfg, const double* a, const double* b, double d[3]) {
  if (!cfg->periodic) return delta_r(a, b, d);
  for (int k = 2; k >= 0; --k) {
    d[k] = b[k] - a[k];
    d[k] -= cfg->box[k] * floor(d[k] / cfg->box[k] + 0.5);
  }
  double r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
  return sqrt(r2);
}

/* ------------------------------------------------------------------------- */
/* Lookup tables                                                             */
/* ------------------------------------------------------------------------- */

typedef struct {
  int64_t* counts; /* uncapped insertion attempts per cell (pass 1) */
  int32_t* fill;   /* kept entries per cell (pass 2) */
} build_scratch;

/* Emit callback: pass 1 counts, pass 2 fills.  Insertion follows atom order
 * and, within an atom, the reference's loop order. */
static inline void emit(orc_table* t, build_scratch* s, int pass, int64_t idx, int atom, int cap) {
  if (idx < 0 || idx >= t->ncell) {
    if (pass == 1) t->oob++;
    return;
  }
  if (pass == 1) {
    s->counts[idx]++;
    return;
  }
  if (cap > 0 && s->fill[idx] >= cap) {
    t->dropped++;
    return;
  }
  t->atoms[t->start[idx] + s->fill[idx]] = atom;
  s->fill[idx]++;
}

/* CharmmReferenceGBSW::computeLookupTable (CharmmReferenceGBSW.cpp:440-514). */
static void table_standalone_pass(const orc_config* cfg, int n, const double* pos, const double* radius,
                                  orc_table* t, build_scratch* s, int pass) {
  (void)radius;
  const double h = cfg->h;
  const int ny = t->dims[1], nz = t->dims[2];
  const double pad = t->pad;
  for (int a = 0; a < n; ++a) {
    const double* c = pos + 3 * a;
    int b[3], e[3];
    for (int k = 0; k < 3; ++k) {
      b[k] = (int)floor((c[k] - pad - t->min[k]) / h);
      e[k] = (int)ceil((c[k] + pad - t->min[k]) / h);
    }
    for (int i = b[0]; i <= e[0]; ++i)
      for (int j = b[1]; j <= e[1]; ++j)
        for (int k = b[2]; k <= e[2]; ++k) {
          int64_t idx = (int64_t)i * ny * nz + (int64_t)j * nz + k;
          double gp[3] = {t->min[0] + i * h, t->min[1] + j * h, t->min[2] + k * h};
          double d0 = gp[0] - c[0], d1 = gp[1] - c[1], d2 = gp[2] - c[2];
          if (sqrt(d0 * d0 + d1 * d1 + d2 * d2) < pad) emit(t, s, pass, idx, a, 0);
        }
  }
}

/* CustomGBIntegral::computeLookupTable, non-periodic branch
 * (CustomGBIntegral.cpp:162-228). */
static void table_grid_pass(const orc_config* cfg, int n, const double* pos, const double* radius,
                            orc_table* t, build_scratch* s, int pass) {
  const double h = cfg->h;
  const int ny = t->dims[1], nz = t->dims[2];
  for (int a = 0; a < n; ++a) {
    const double pad = radius[a] + sqrt(3.0) / 2.0 * h + cfg->buffer;
    const double* c = pos + 3 * a;
    int b[3], e[3];
    for (int k = 0; k < 3; ++k) {
      b[k] = (int)floor((c[k] - pad - t->min[k]) / h);
      e[k] = (int)ceil((c[k] + pad - t->min[k]) / h);
    }
    for (int i = b[0]; i <= e[0]; ++i)
      for (int j = b[1]; j <= e[1]; ++j)
        for (int k = b[2]; k <= e[2]; ++k) {
          int64_t idx = (int64_t)i * ny * nz + (int64_t)j * nz + k;
          double gp[3] = {t->min[0] + i * h, t->min[1] + j * h, t->min[2] + k * h};
          double d0 = gp[0] - c[0], d1 = gp[1] - c[1], d2 = gp[2] - c[2];
          if (d0 * d0 + d1 * d1 + d2 * d2 < pad * pad) emit(t, s, pass, idx, a, cfg->cap);
        }
  }
}

/* CustomGBIntegral::computeLookupTable, periodic branch
 * (CustomGBIntegral.cpp:45-160): box-sized grid centred on the centre of
 * geometry; each atom walks sample points at the grid step from
 * x - pad - L to x + pad + L and tests the *sample* against pad. */
static void table_periodic_pass(const orc_config* cfg, int n, const double* pos, const double* radius,
                                orc_table* t, build_scratch* s, int pass) {
  const int ny = t->dims[1], nz = t->dims[2];
  const double* step = t->step;
  const double dx = t->box[0], dy = t->box[1], dz = t->box[2];
  double L = step[0] > step[1] ? step[0] : step[1];
  L = L > step[2] ? L : step[2];
  for (int a = 0; a < n; ++a) {
    const double pad = radius[a] + sqrt(3.0) / 2.0 * L + cfg->buffer;
    const double* c = pos + 3 * a;
    double bc[3], ec[3];
    for (int k = 0; k < 3; ++k) {
      bc[k] = (c[k] - pad - L);
      ec[k] = (c[k] + pad + L);
    }
    for (double x = bc[0]; x < ec[0]; x += step[0])
      for (double y = bc[1]; y < ec[1]; y += step[1])
        for (double z = bc[2]; z < ec[2]; z += step[2]) {
          double x0 = x - dx * floor((x - t->min[0]) / dx);
          double y0 = y - dy * floor((y - t->min[1]) / dy);
          double z0 = z - dz * floor((z - t->min[2]) / dz);
          int ix = (int)floor((x0 - t->min[0]) / step[0]);
          int iy = (int)floor((y0 - t->min[1]) / step[1]);
          int iz = (int)floor((z0 - t->min[2]) / step[2]);
          double ddx = x - c[0], ddy = y - c[1], ddz = z - c[2];
          if (ddx * ddx + ddy * ddy + ddz * ddz < pad * pad) {
            int64_t idx = (int64_t)ix * ny * nz + (int64_t)iy * nz + iz;
            if (ix < 0 || iy < 0 || iz < 0 || ix >= t->dims[0] || iy >= ny || iz >= nz) idx = -1;
            emit(t, s, pass, idx, a, cfg->cap);
          }
        }
  }
}

int orc_table_build(const orc_config* cfg, int n, const double* pos, const double* radius, orc_table* t) {
  memset(t, 0, sizeof(*t));
  t->mode = cfg->table_mode;
  if (n <= 0) return -1;
  if (cfg->periodic && cfg->table_mode == ORC_TABLE_STANDALONE) {
    t->wrap = 1;  /* the table itself is built from the raw coordinates (:440-514) */
    for (int k = 0; k < 3; ++k) t->box[k] = cfg->box[k];
  }
  if (cfg->table_mode == ORC_TABLE_STANDALONE || cfg->table_mode == ORC_TABLE_GRID) {
    double mn[3], mx[3];
    for (int k = 0; k < 3; ++k) mn[k] = mx[k] = pos[k];
    double maxR = 0.0;
    for (int a = 0; a < n; ++a) {
      for (int k = 0; k < 3; ++k) {
        mn[k] = fmin(mn[k], pos[3 * a + k]);
        mx[k] = fmax(mx[k], pos[3 * a + k]);
      }
      maxR = fmax(maxR, radius[a]);
    }
    double pad;
    if (cfg->table_mode == ORC_TABLE_STANDALONE) /* CharmmReferenceGBSW.cpp:454-455 */
      pad = cfg->buffer + maxR + cfg->sw + sqrt(3.0) / 2.0 * cfg->h + 1e-6;
    else /* CustomGBIntegral.cpp:174-175: fixed 0.03 nm stands in for the radius */
      pad = 0.03 + sqrt(3.0) / 2.0 * cfg->h + cfg->buffer;
    int64_t ncell = 1;
    for (int k = 0; k < 3; ++k) {
      mn[k] -= pad;
      mx[k] += pad;
      double length = mx[k] - mn[k];
      if (cfg->table_mode == ORC_TABLE_GRID && length > 1000) return -2; /* :182-183 */
      t->dims[k] = (int)ceil(length / cfg->h) + 1;
      t->min[k] = mn[k];
      t->max[k] = mn[k] + (t->dims[k] - 1) * cfg->h;
      ncell *= t->dims[k];
    }
    t->step[0] = t->step[1] = t->step[2] = cfg->h;
    t->pad = pad;
    t->ncell = ncell;
  } else {
    /* CustomGBIntegral.cpp:45-115 */
    double cog[3] = {0, 0, 0};
    for (int a = 0; a < n; ++a)
      for (int k = 0; k < 3; ++k) cog[k] += pos[3 * a + k];
    for (int k = 0; k < 3; ++k) cog[k] /= n;
    int64_t ncell = 1;
    for (int k = 0; k < 3; ++k) {
      double d = cfg->box[k];
      t->box[k] = d;
      t->min[k] = cog[k] - d / 2.0;
      t->max[k] = cog[k] + d / 2.0;
      t->dims[k] = (int)ceil(d / cfg->h) + 1;
      t->step[k] = d / t->dims[k];
      ncell *= t->dims[k];
    }
    t->ncell = ncell;
  }
  build_scratch s;
  s.counts = (int64_t*)calloc((size_t)t->ncell, sizeof(int64_t));
  s.fill = (int32_t*)calloc((size_t)t->ncell, sizeof(int32_t));
  t->count = (int32_t*)calloc((size_t)t->ncell, sizeof(int32_t));
  t->start = (int64_t*)calloc((size_t)t->ncell + 1, sizeof(int64_t));
  if (!s.counts || !s.fill || !t->count || !t->start) return -3;
  for (int pass = 1; pass <= 2; ++pass) {
    if (pass == 2) {
      int64_t acc = 0;
      for (int64_t c = 0; c < t->ncell; ++c) {
        t->start[c] = acc;
        int64_t kept = s.counts[c];
        if (cfg->cap > 0 && kept > cfg->cap) kept = cfg->cap;
        acc += kept;
      }
      t->start[t->ncell] = acc;
      t->atoms = (int32_t*)malloc(sizeof(int32_t) * (size_t)(acc > 0 ? acc : 1));
      if (!t->atoms) return -3;
    }
    if (cfg->table_mode == ORC_TABLE_STANDALONE) table_standalone_pass(cfg, n, pos, radius, t, &s, pass);
    else if (cfg->table_mode == ORC_TABLE_GRID) table_grid_pass(cfg, n, pos, radius, t, &s, pass);
    else table_periodic_pass(cfg, n, pos, radius, t, &s, pass);
  }
  for (int64_t c = 0; c < t->ncell; ++c) t->count[c] = s.fill[c];
  free(s.counts);
  free(s.fill);
  return 0;
}

void orc_table_free(orc_table* t) {
  free(t->count);
  free(t->start);
  free(t->atoms);
  memset(t, 0, sizeof(*t));
}

/* getLookupTableAtomList: CharmmReferenceGBSW.cpp:516-552 (non-periodic),
 * CustomGBIntegral.cpp:310-324 (grid) and :284-309 (periodic). */
int64_t orc_table_query(const orc_table* t, const double p[3]) {
  const int nx = t->dims[0], ny = t->dims[1], nz = t->dims[2];
  if (t->mode == ORC_TABLE_PERIODIC) {
    int id[3];
    for (int k = 0; k < 3; ++k) {
      double d = t->box[k];
      double x0 = p[k] - floor((p[k] - t->min[k]) / d) * d;
      id[k] = (int)((x0 - t->min[k]) / t->step[k]);
    }
    if (id[0] < 0 || id[1] < 0 || id[2] < 0 || id[0] >= nx || id[1] >= ny || id[2] >= nz) return -1;
    return (int64_t)id[0] * (ny * nz) + (int64_t)id[1] * nz + id[2];
  }
  int id[3];
  double pt[3] = {p[0], p[1], p[2]};
  if (t->wrap)  /* CharmmReferenceGBSW.cpp:522-528: at most one box length per axis */
    for (int k = 0; k < 3; ++k) {
      if (pt[k] < t->min[k]) pt[k] += t->box[k];
      if (pt[k] > t->max[k]) pt[k] -= t->box[k];
    }
  for (int k = 0; k < 3; ++k) {
    if (pt[k] < t->min[k] || pt[k] > t->max[k]) return -1;
    id[k] = (int)floor((pt[k] - t->min[k]) / t->step[k]);
  }
  return (int64_t)id[0] * (ny * nz) + (int64_t)id[1] * nz + id[2];
}

/* ------------------------------------------------------------------------- */
/* Per-point volume state                                                    */
/* ------------------------------------------------------------------------- */

typedef struct {
  int n_list;
  const int32_t* list;
  double V;          /* GBSW: solvent fraction; GBMV: solute fraction 1/(1+p) */
  double presum;     /* GBMV: p = exp(beta (S - lambda)) */
  double sum1, sum2, sum3, vec[3]; /* GBMV-II */
  double evals, shell;
} point_state;

static inline double gbsw_radius(double R) { return (R + 0.03) * 0.9520; }

/* GBSW volume: CharmmReferenceGBSW.cpp:616-639 / GBSWIntegral.cpp:187-224. */
static double vol_gbsw(const orc_config* cfg, const double* pos, const double* radius, const double p[3],
                       point_state* st) {
  const double sw = cfg->sw, sw3 = sw * sw * sw;
  double V = 1.0;
  for (int l = 0; l < st->n_list; ++l) {
    int j = st->list[l];
    double d[3];
    double r = delta_cfg(cfg, p, pos + 3 * j, d);
    double Rj = gbsw_radius(radius[j]);
    double dr = r - Rj;
    double dr3 = dr * dr * dr;
    st->evals += 1;
    if (r <= Rj - sw) {
      return 0.0;
    } else if (r >= Rj + sw) {
      continue;
    } else {
      st->shell += 1;
      V *= 0.5 + 3.0 / (4.0 * sw) * dr - 1.0 / (4.0 * sw3) * dr3;
    }
  }
  return V;
}

/* GBMV-I pre-sum: GBMVIntegralTypeI.cpp:155-173. */
static double presum_gbmv1(const orc_config* cfg, const double* pos, const double* radius, const double p[3],
                           point_state* st) {
  double sum = 0.0;
  for (int l = 0; l < st->n_list; ++l) {
    int j = st->list[l];
    double d[3];
    double r = delta_cfg(cfg, p, pos + 3 * j, d);
    double r4 = r * r * r * r;
    double R = radius[j];
    double R4 = R * R * R * R;
    double gam = cfg->gamma0 * log(cfg->lambda) / (R4);
    sum += exp(gam * r4);
    st->evals += 1;
  }
  return exp(cfg->beta * (sum - cfg->lambda));
}

/* GBMV-II pre-sum: GBMVIntegralTypeII.cpp:163-191. */
static double presum_gbmv2(const orc_config* cfg, const double* pos, const double* radius, const double p[3],
                           point_state* st) {
  if (st->n_list == 0) return 0;
  st->sum1 = 0.0;
  st->sum2 = 0.0;
  st->vec[0] = st->vec[1] = st->vec[2] = 0.0;
  for (int l = 0; l < st->n_list; ++l) {
    int j = st->list[l];
    double d[3];
    double r = delta_cfg(cfg, p, pos + 3 * j, d);
    double r2 = r * r;
    double R = radius[j];
    double R2 = R * R;
    double C = cfg->p1 * R * 10 + cfg->p2;
    double F = C / (C + r2 * 100 - R2 * 100);
    F = F * F;
    st->sum1 += F;
    st->sum2 += r2 * (F * F);
    st->vec[0] += d[0] * F;
    st->vec[1] += d[1] * F;
    st->vec[2] += d[2] * F;
    st->evals += 1;
  }
  st->sum3 = sqrt(st->vec[0] * st->vec[0] + st->vec[1] * st->vec[1] + st->vec[2] * st->vec[2]);
  double S = cfg->s0 * st->sum1 * st->sum2 / (st->sum3 * st->sum3);
  return exp(cfg->beta * (S - cfg->lambda));
}

/* Evaluate the point; returns 0 if the point is skipped (GBSW empty list). */
static int point_eval(const orc_config* cfg, const orc_table* t, const double* pos, const double* radius,
                      const double p[3], point_state* st) {
  memset(st, 0, sizeof(*st));
  int64_t c = orc_table_query(t, p);
  if (c >= 0) {
    st->n_list = t->count[c];
    st->list = t->atoms + t->start[c];
  }
  if (cfg->model == ORC_GBSW) {
    if (st->n_list == 0) {
      st->V = 1.0;
      return cfg->skip_empty ? 0 : 1;
    }
    st->V = vol_gbsw(cfg, pos, radius, p, st);
    return 1;
  }
  if (c < 0 && cfg->model == ORC_GBMV1) {
    /* point off the table: the reference's periodic query never misses, the
     * grid query returns before touching the (uninitialised) list pointer;
     * an empty sum is the consistent reading. */
    st->n_list = 0;
  }
  if (cfg->model == ORC_GBMV1) {
    st->presum = presum_gbmv1(cfg, pos, radius, p, st);
    st->V = 1.0 / (1.0 + st->presum);
  } else {
    st->presum = presum_gbmv2(cfg, pos, radius, p, st);
    st->V = (st->n_list == 0 ? 0 : 1.0 / (1.0 + st->presum)); /* TypeII.cpp:140 */
  }
  return 1;
}

/* fraction entering the integral: GBSW integrates 1 - V (GBSWIntegral.cpp:145),
 * GBMV integrates V (GBMVIntegralTypeI.cpp:140). */
static inline double integrand(const orc_config* cfg, const point_state* st) {
  return cfg->model == ORC_GBSW ? 1.0 - st->V : st->V;
}

/* Gradient of the integrand wrt delta_j = x_j - p for list entry l, and wrt the
 * input radius R_j.  GBSW: GBSWIntegral.cpp:271-314 (negated: integrand is
 * 1-V); GBMV-I: TypeI.cpp:195-224; GBMV-II: TypeII.cpp:221-282.  Returns 0
 * when the atom contributes nothing. */
static int point_grad(const orc_config* cfg, const double* pos, const double* radius, const double p[3],
                      const point_state* st, int l, double g[3], double* gR) {
  int j = st->list[l];
  double d[3];
  double r = delta_cfg(cfg, p, pos + 3 * j, d);
  if (cfg->model == ORC_GBSW) {
    if (st->V == 0) return 0;
    const double sw = cfg->sw, sw3 = sw * sw * sw;
    double Rj = gbsw_radius(radius[j]);
    double dr = r - Rj;
    double dr2 = dr * dr, dr3 = dr * dr * dr;
    if (!(r > Rj - sw && r < Rj + sw)) return 0;
    double u = 0.5 + 3.0 / (4.0 * sw) * dr - 1.0 / (4.0 * sw3) * dr3;
    double du = 3.0 / (4.0 * sw) - 3.0 / (4.0 * sw3) * dr2;
    double f = (du * st->V / u) / r; /* dV/d delta = f * delta */
    for (int k = 0; k < 3; ++k) g[k] = -d[k] * f;
    /* dV/dR_j = (V/u) * du * d(dr)/dR = -(V/u) du 0.952 ; integrand 1-V */
    *gR = (st->V / u) * du * 0.9520;
    return 1;
  }
  if (cfg->model == ORC_GBMV1) {
    double ps = st->presum;
    double dVdS = -1.0 / ((1.0 + ps) * (1.0 + ps)) * (cfg->beta * ps);
    double r3 = r * r * r, r4 = r3 * r;
    double R = radius[j];
    double R4 = R * R * R * R;
    double gam = cfg->gamma0 * log(cfg->lambda) / (R4);
    double e = exp(gam * r4);
    double f2 = dVdS * gam * e * (4.0 * r3);
    for (int k = 0; k < 3; ++k) g[k] = d[k] / r * f2;
    *gR = dVdS * e * r4 * (-4.0 * gam / R);
    return 1;
  }
  /* GBMV-II */
  if (st->n_list == 0) return 0;
  double ps = st->presum;
  double factor = -1.0 / ((1.0 + ps) * (1.0 + ps)) * (cfg->beta * ps) * cfg->s0;
  double r2 = r * r;
  double R = radius[j];
  double R2 = R * R;
  double C = cfg->p1 * R * 10 + cfg->p2;
  double T = (C + r2 * 100 - R2 * 100);
  double F = C / T;
  F = F * F;
  double dFf = -400.0 * C * C / (T * T * T);
  double s3sq = st->sum3 * st->sum3;
  double tmp1 = dFf * st->sum2 / s3sq * factor;
  double tmp2 = 2.0 * F * (F + dFf * r2) / s3sq * st->sum1 * factor;
  double tmp3 = -2.0 / (s3sq * s3sq) * st->sum1 * st->sum2 * factor;
  double vd = st->vec[0] * d[0] + st->vec[1] * d[1] + st->vec[2] * d[2];
  for (int k = 0; k < 3; ++k)
    g[k] = d[k] * tmp1 + d[k] * tmp2 + tmp3 * (st->vec[k] * F + vd * dFf * d[k]);
  /* dF/dR with C' = 10 P1, T' = 10 P1 - 200 R */
  double Cp = 10.0 * cfg->p1, Tp = 10.0 * cfg->p1 - 200.0 * R;
  double dFdR = 2.0 * (C / T) * (Cp * T - C * Tp) / (T * T);
  double ds1 = dFdR, ds2 = r2 * 2.0 * F * dFdR, ds3sq = 2.0 * vd * dFdR;
  /* S = s0 s1 s2 / s3^2 -> dV = factor/s0 * dS, factor already holds s0 */
  *gR = factor * (ds1 * st->sum2 / s3sq + st->sum1 * ds2 / s3sq - st->sum1 * st->sum2 * ds3sq / (s3sq * s3sq));
  return 1;
}

static inline double order_weight(const orc_config* cfg, int k, int q) {
  return cfg->qw[q] / pow(cfg->qrad[q], cfg->orders[k] - 2);
}

static int nthreads_of(const orc_config* cfg) {
#ifdef _OPENMP
  return cfg->nthreads > 0 ? cfg->nthreads : omp_get_max_threads();
#else
  (void)cfg;
  return 1;
#endif
}

/* GBSWIntegral::evaluate etc.: q outer / atom inner in the reference; the sum
 * for one atom runs over q in ascending order either way. */
int orc_integrals(const orc_config* cfg, const orc_table* t, int n, const double* pos, const double* radius,
                  double* integrals, orc_work* work) {
  if (cfg->standalone_sums && (cfg->n_int != 2 || cfg->orders[0] != 4 || cfg->orders[1] != 7)) return -4;
  memset(integrals, 0, sizeof(double) * (size_t)cfg->n_int * n);
  double evals = 0, shell = 0, pts = 0, act = 0;
#pragma omp parallel for schedule(static) num_threads(nthreads_of(cfg)) reduction(+ : evals, shell, pts, act)
  for (int i = 0; i < n; ++i) {
    if (cfg->atom_stride > 1 && i % cfg->atom_stride) continue;
    for (int q = 0; q < cfg->nq; ++q) {
      double p[3];
      for (int k = 0; k < 3; ++k) p[k] = pos[3 * i + k] + cfg->qoff[3 * q + k];
      point_state st;
      if (!point_eval(cfg, t, pos, radius, p, &st)) continue;
      evals += st.evals;
      shell += st.shell;
      pts += 1;
      if (st.V > 0 && st.V < 1) act += 1;
      double f = integrand(cfg, &st);
      if (cfg->standalone_sums) {
        const double r = cfg->qrad[q], w = cfg->qw[q];
        const double r5 = r * r * r * r * r;
        integrals[i] += w * f / (r * r);
        integrals[n + i] += w * f / r5;
      } else {
        for (int k = 0; k < cfg->n_int; ++k) integrals[k * n + i] += order_weight(cfg, k, q) * f;
      }
    }
  }
  if (work) {
    work->volume_evals += evals;
    work->shell_evals += shell;
    work->points += pts;
    work->active_points += act;
  }
  return 0;
}

/* Shared chain-rule walk: for each point, c = sum_k dEdI_k[i] * w/r^(n-2);
 * F_j -= c * dphi/dx_j for every contributing list atom j != i, F_i gets the
 * opposite (the point moves with atom i).  dEdR[j] += c * dphi/dR_j (j == i
 * included: atom i's own radius shapes its own points). */
static int chain_walk(const orc_config* cfg, const orc_table* t, int n, const double* pos, const double* radius,
                      const double* dEdI, double* forces, double* dEdR, orc_work* work) {
  const int nt = nthreads_of(cfg);
  double* fbuf = (double*)calloc((size_t)nt * n * 3, sizeof(double));
  double* rbuf = dEdR ? (double*)calloc((size_t)nt * n, sizeof(double)) : NULL;
  if (!fbuf || (dEdR && !rbuf)) return -3;
  double pairs = 0;
#pragma omp parallel num_threads(nt) reduction(+ : pairs)
  {
#ifdef _OPENMP
    int tid = omp_get_thread_num();
#else
    int tid = 0;
#endif
    double* F = fbuf + (size_t)tid * n * 3;
    double* DR = rbuf ? rbuf + (size_t)tid * n : NULL;
#pragma omp for schedule(static)
    for (int i = 0; i < n; ++i) {
      if (cfg->atom_stride > 1 && i % cfg->atom_stride) continue;
      for (int q = 0; q < cfg->nq; ++q) {
        double c = 0.0;
        for (int k = 0; k < cfg->n_int; ++k) c += dEdI[k * n + i] * order_weight(cfg, k, q);
        double p[3];
        for (int k = 0; k < 3; ++k) p[k] = pos[3 * i + k] + cfg->qoff[3 * q + k];
        point_state st;
        if (!point_eval(cfg, t, pos, radius, p, &st)) continue;
        for (int l = 0; l < st.n_list; ++l) {
          int j = st.list[l];
          double g[3], gR = 0.0;
          if (!point_grad(cfg, pos, radius, p, &st, l, g, &gR)) continue;
          pairs += 1;
          if (DR) DR[j] += c * gR;
          if (j == i) continue;
          /* dphi/dx_j = g, dphi/dx_i = -g */
          int keep_j = 1;
          if (cfg->use_cutoff && cfg->cutoff_chain_quirk) {
            double dd[3];
            if (delta_cfg(cfg, pos + 3 * i, pos + 3 * j, dd) > cfg->cutoff) keep_j = 0;
          }
          for (int k = 0; k < 3; ++k) {
            if (keep_j) F[3 * j + k] -= c * g[k];
            F[3 * i + k] += c * g[k];
          }
        }
      }
    }
  }
  for (int tid = 0; tid < nt; ++tid) {
    for (int a = 0; a < 3 * n; ++a) forces[a] += fbuf[(size_t)tid * n * 3 + a];
    if (dEdR)
      for (int a = 0; a < n; ++a) dEdR[a] += rbuf[(size_t)tid * n + a];
  }
  free(fbuf);
  free(rbuf);
  if (work) work->chain_pairs += pairs;
  return 0;
}

int orc_integral_chain(const orc_config* cfg, const orc_table* t, int n, const double* pos, const double* radius,
                       const double* dEdI, double* forces, orc_work* work) {
  return chain_walk(cfg, t, n, pos, radius, dEdI, forces, NULL, work);
}

/* ------------------------------------------------------------------------- */
/* Canonical energy + forces                                                 */
/* ------------------------------------------------------------------------- */

/* The GB pair term for given Born radii, CharmmReferenceGBSW.cpp:237-283:
 * every pair j >= i (the self term halved), energy, pair forces, dE/dB and
 * dE/dq ADDED to the outputs (any of them may be NULL except energy). */
int orc_pair_terms(const orc_config* cfg, int n, const double* pos, const double* charge, const double* B,
                   double* energy, double* forces, double* dEdB_out, double* dEdq_out, orc_work* work) {
  const double pref = cfg->pref;
  double E = 0.0, npairs = 0;
  const int nt = nthreads_of(cfg);
  double* dbbuf = (double*)calloc((size_t)nt * n, sizeof(double));
  double* fbuf = (double*)calloc((size_t)nt * n * 3, sizeof(double));
  double* qbuf = (double*)calloc((size_t)nt * n, sizeof(double));
  if (!dbbuf || !fbuf || !qbuf) return -3;
#pragma omp parallel num_threads(nt) reduction(+ : E, npairs)
  {
#ifdef _OPENMP
    int tid = omp_get_thread_num();
#else
    int tid = 0;
#endif
    double* DB = dbbuf + (size_t)tid * n;
    double* FF = fbuf + (size_t)tid * n * 3;
    double* DQ = qbuf + (size_t)tid * n;
#pragma omp for schedule(dynamic, 16)
    for (int i = 0; i < n; ++i) {
      if (cfg->atom_stride > 1 && i % cfg->atom_stride) continue;
      for (int j = i; j < n; ++j) {
        double d[3];
        double r = delta_cfg(cfg, pos + 3 * i, pos + 3 * j, d);
        if (cfg->use_cutoff && r > cfg->cutoff) continue;
        npairs += 1;
        double qi = charge[i], qj = charge[j], Ri = B[i], Rj = B[j];
        double D = (r * r) / (4.0 * Ri * Rj);
        double ex = exp(-D);
        double f = sqrt(r * r + Ri * Rj * ex);
        double e = pref * qi * qj / f;
        if (i != j) {
          E += e;
          DQ[i] += pref * qj / f;
          DQ[j] += pref * qi / f;
        } else {
          E += 0.5 * e;
          DQ[i] += pref * qi / f;
        }
        double dGdr = -0.25 * pref * (qi * qj * (4.0 - ex)) / (f * f * f);
        for (int k = 0; k < 3; ++k) {
          double f1 = (-d[k]) * (-dGdr);
          FF[3 * i + k] += f1;
          FF[3 * j + k] -= f1;
        }
        if (i == j) {
          DB[i] += -0.5 * pref * qi * qj / (Ri * Ri);
        } else {
          double common = -0.5 * pref * ((qi * qj * ex) / (f * f * f));
          DB[i] += common * (Rj + (r * r) / (4.0 * Ri));
          DB[j] += common * (Ri + (r * r) / (4.0 * Rj));
        }
      }
    }
  }
  for (int tid = 0; tid < nt; ++tid) {
    for (int a = 0; a < n; ++a) {
      if (dEdB_out) dEdB_out[a] += dbbuf[(size_t)tid * n + a];
      if (dEdq_out) dEdq_out[a] += qbuf[(size_t)tid * n + a];
    }
    if (forces)
      for (int a = 0; a < 3 * n; ++a) forces[a] += fbuf[(size_t)tid * n * 3 + a];
  }
  free(dbbuf);
  free(fbuf);
  free(qbuf);
  if (work) work->pairs += npairs;
  *energy += E;
  return 0;
}

int orc_energy_forces(const orc_config* cfg, int n, const double* pos, const double* charge, const double* radius,
                      double* energy, double* forces, double* born, double* integrals_out, double* dEdB_out,
                      double* dEdq, double* dEdR, double* dEdalpha, orc_work* work) {
  if (cfg->n_int != 2 || cfg->orders[0] != 4 || cfg->orders[1] != 7) return -4;
  orc_table t;
  int rc = orc_table_build(cfg, n, pos, radius, &t);
  if (rc) return rc;
  double* I = (double*)calloc((size_t)2 * n, sizeof(double));
  double* B = (double*)calloc((size_t)n, sizeof(double));
  double* dEdB = (double*)calloc((size_t)n, sizeof(double));
  double* F = (double*)calloc((size_t)3 * n, sizeof(double));
  double* dq = (double*)calloc((size_t)n, sizeof(double));
  if (!I || !B || !dEdB || !F || !dq) return -3;
  double E = 0.0;
  orc_integrals(cfg, &t, n, pos, radius, I, work);
  /* Born radii, CharmmReferenceGBSW.cpp:591-593 */
  const double eta = cfg->r0, eta4 = eta * eta * eta * eta;
  for (int i = 0; i < n; ++i) {
    double inv = cfg->alpha0 * (1.0 / eta - I[i]) + cfg->alpha1 * pow((1.0 / (4.0 * eta4) - I[n + i]), 1.0 / 4.0);
    B[i] = 1.0 / inv;
  }
  rc = orc_pair_terms(cfg, n, pos, charge, B, &E, F, dEdB, dq, work);
  if (rc) return rc;
  /* chain rule through the integrals: dE/dI4 = dE/dB * B^2 alpha0,
   * dE/dI7 = dE/dB * B^2 alpha1/4 (..)^(-3/4)  (CharmmReferenceGBSW.cpp:597-611) */
  double* dEdI = (double*)calloc((size_t)2 * n, sizeof(double));
  double da0 = 0.0, da1 = 0.0;
  for (int i = 0; i < n; ++i) {
    double t7 = (1.0 / (4.0 * eta4) - I[n + i]);
    dEdI[i] = dEdB[i] * B[i] * B[i] * cfg->alpha0;
    dEdI[n + i] = dEdB[i] * B[i] * B[i] * (1.0 / 4.0) * cfg->alpha1 * pow(t7, -3.0 / 4.0);
    da0 += dEdB[i] * (-B[i] * B[i]) * (1.0 / eta - I[i]);
    da1 += dEdB[i] * (-B[i] * B[i]) * pow(t7, 1.0 / 4.0);
  }
  double* dR = dEdR ? (double*)calloc((size_t)n, sizeof(double)) : NULL;
  chain_walk(cfg, &t, n, pos, radius, dEdI, F, dR, work);
  if (energy) *energy = E;
  if (forces) memcpy(forces, F, sizeof(double) * 3 * n);
  if (born) memcpy(born, B, sizeof(double) * n);
  if (integrals_out) memcpy(integrals_out, I, sizeof(double) * 2 * n);
  if (dEdB_out) memcpy(dEdB_out, dEdB, sizeof(double) * n);
  if (dEdq) memcpy(dEdq, dq, sizeof(double) * n);
  if (dEdR) {
    memcpy(dEdR, dR, sizeof(double) * n);
    free(dR);
  }
  if (dEdalpha) {
    dEdalpha[0] = da0;
    dEdalpha[1] = da1;
  }
  free(I);
  free(B);
  free(dEdB);
  free(F);
  free(dq);
  free(dEdI);
  orc_table_free(&t);
  return 0;
}
