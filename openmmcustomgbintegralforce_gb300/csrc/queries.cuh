// Cell queries and inline list entries shared by the volume translation
// units: the reference table's query (FP32 with an exact FP64 path within a
// guard band of every cell face, CharmmReferenceGBSW.cpp:539-549,
// CustomGBIntegral.cpp:284-324), its minimum-image and wrapped variants, and
// the exact GBSW table's query.  Internal linkage in each unit.
#pragma once

#include "gbx_internal.cuh"

namespace gbx {
namespace {

struct Quad {
  const float4* qv;     // (vx, vy, vz, r)
  const float2* qw;     // (w/r^2, w/r^5)
  const double* qoff;   // FP64 offsets [3Q]
};

// Inline list entries of either table.
struct Entries {
  const TableGeom* geom;
  const int2* cell;    // (count, start); exact table: count -1 marks a buried cell
  const float4* e;     // (x, y, z, main model parameter)
  const float2* par;   // secondary model parameters (reference table only)
  const int* index;    // atom index of each entry
  long long cell_cap;  // cells allocated: a geometry with more (a table that
                       // outgrew its buffers, not yet resized) is never indexed
  const TightCell* first; // exact table: each cell's first list entry and record (else nullptr)
  long long entry_cap;    // entries allocated: a table with more was not sorted
                          // this step, its cell records are an earlier step's
  const TableGeom* wrap;  // exact table of a periodic system: the reference's
                          // standalone grid, whose edges decide a point's move
};

// Cells a query may index: none when the table outgrew either buffer this
// step (the build then wrote no cell record, and the records left in place
// may belong to another geometry).
__device__ __forceinline__ long long usable_cells(const Entries& t) {
  return t.geom->total > t.entry_cap ? -1 : t.cell_cap;
}

// ---------------------------------------------------------------------------
// Cell queries
// ---------------------------------------------------------------------------

// Reference table: FP64 query as the reference (separately rounded).
__device__ long long query_exact(const TableGeom& g, const float4 xi, const double* qoff, int q) {
  const double x[3] = {(double)xi.x, (double)xi.y, (double)xi.z};
  int id[3];
  for (int k = 0; k < 3; ++k) {
    const double p = __dadd_rn(x[k], qoff[3 * q + k]);
    if (g.mode == GBX_TABLE_PERIODIC) {
      const double d = g.box[k];
      const double x0 = __dsub_rn(p, __dmul_rn(floor(__ddiv_rn(__dsub_rn(p, g.min[k]), d)), d));
      id[k] = (int)(__ddiv_rn(__dsub_rn(x0, g.min[k]), g.step[k]));
      if (id[k] < 0 || id[k] >= g.dims[k]) return -1;
    } else {
      if (p < g.min[k] || p > g.max[k]) return -1;
      id[k] = (int)floor(__ddiv_rn(__dsub_rn(p, g.min[k]), g.step[k]));
    }
  }
  return (long long)id[0] * ((long long)g.dims[1] * g.dims[2]) + (long long)id[1] * g.dims[2] + id[2];
}

struct RefQuery {
  float rel[3];  // (x_i - min) / step, cell units
  float inv[3];
  float invdims[3];  // periodic table: 1 / dims, the box in cell units being dims
  float eps;     // guard band in cell units
  bool off;      // the geometry has more cells than are allocated: no cell
  const TableGeom* g;
  const double* qoff;
  __device__ __forceinline__ void init(const TableGeom& geom, const float4 xi, const double* qo, long long cap) {
    g = &geom;
    qoff = qo;
    off = geom.ncell > cap;
    const double x[3] = {(double)xi.x, (double)xi.y, (double)xi.z};
    const int dmax = max(geom.dims[0], max(geom.dims[1], geom.dims[2]));
    for (int k = 0; k < 3; ++k) {
      rel[k] = (float)((x[k] - geom.min[k]) * geom.inv_step[k]);
      inv[k] = (float)geom.inv_step[k];
      invdims[k] = 1.0f / (float)geom.dims[k];
    }
    eps = 1e-4f + 64.0f * (float)dmax * 5.96e-8f;
  }
  __device__ __forceinline__ void init(const Entries& t, const float4 xi, const double* qo) {
    init(*t.geom, xi, qo, usable_cells(t));
  }
  __device__ __forceinline__ long long cell(const float4 xi, const float4 v, int q) const {
    bool unsafe;
    const long long c = cell_fast(v, unsafe);
    return unsafe ? query_exact(*g, xi, qoff, q) : c;
  }
  // The FP32 query alone; unsafe: the point lies within the guard band of a
  // cell face or grid edge and needs the exact query (the result is then -1).
  __device__ __forceinline__ long long cell_fast(const float4 v, bool& unsafe) const {
    unsafe = false;
    if (off) return -1;
    const TableGeom& G = *g;
    float t[3] = {fmaf(v.x, inv[0], rel[0]), fmaf(v.y, inv[1], rel[1]), fmaf(v.z, inv[2], rel[2])};
    int id[3];
    bool safe = true;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      if (G.mode == GBX_TABLE_PERIODIC) {
        // the box-sampled grid spans the box (step = box / dims): moving the
        // point by whole boxes (CustomGBIntegral.cpp:284-309) is a shift by
        // whole multiples of dims in cell units; a point within the guard
        // band of a box edge takes the exact path
        const float W = (float)G.dims[k];
        const float nb = floorf(t[k] * invdims[k]);
        t[k] = fmaf(-nb, W, t[k]);
        if (t[k] < eps || t[k] > W - eps) safe = false;
      }
      const float f = floorf(t[k]);
      const float fr = t[k] - f;
      id[k] = (int)f;
      if (fr < eps || fr > 1.0f - eps) safe = false;
      if (G.mode == GBX_TABLE_PERIODIC) {
        if (id[k] < 0 || id[k] >= G.dims[k]) safe = false;
      } else {
        if (t[k] < -eps || t[k] > (float)(G.dims[k] - 1) + eps) return -1;
        if (t[k] < eps || t[k] > (float)(G.dims[k] - 1) - eps) safe = false;
      }
    }
    if (!safe) {
      unsafe = true;
      return -1;
    }
    return (long long)id[0] * ((long long)G.dims[1] * G.dims[2]) + (long long)id[1] * G.dims[2] + id[2];
  }
  // x_j - p formed as (x_j - x_i) - v: the FP32 difference of nearby atoms is exact
  __device__ __forceinline__ float3 delta(const float4 a, const float4 xi, const float4 v) const {
    return make_float3((a.x - xi.x) - v.x, (a.y - xi.y) - v.y, (a.z - xi.z) - v.z);
  }
};

// A box-sampled (periodic-branch) table of a CutoffPeriodic system: the
// reference query, distances by minimum image (the integral classes with
// CutoffPeriodic, GBMVIntegralTypeI.cpp:59-62, TypeII.cpp:64-67,
// GBSWIntegral.cpp:63-68).
struct MinImageQuery : RefQuery {
  float L[3], iL[3];
  __device__ __forceinline__ void init(const TableGeom& geom, const float4 xi, const double* qo, long long cap) {
    RefQuery::init(geom, xi, qo, cap);
    for (int k = 0; k < 3; ++k) {
      L[k] = (float)geom.box[k];
      iL[k] = (float)geom.inv_box[k];
    }
  }
  __device__ __forceinline__ void init(const Entries& t, const float4 xi, const double* qo) {
    init(*t.geom, xi, qo, usable_cells(t));
  }
  __device__ __forceinline__ float3 delta(const float4 a, const float4 xi, const float4 v) const {
    float d[3] = {(a.x - xi.x) - v.x, (a.y - xi.y) - v.y, (a.z - xi.z) - v.z};
#pragma unroll
    for (int k = 0; k < 3; ++k) d[k] = fmaf(-L[k], floorf(fmaf(d[k], iL[k], 0.5f)), d[k]);
    return make_float3(d[0], d[1], d[2]);
  }
};

// Standalone table of a periodic system (CutoffPeriodic): the point is moved
// by one box length along each axis where it lies below the grid's lower
// edge, then back where it lies above the upper edge, and misses if it is
// still off the grid (CharmmReferenceGBSW.cpp:522-535); FP64 as the reference.
__device__ long long query_exact_wrap(const TableGeom& g, const float4 xi, const double* qoff, int q) {
  const double x[3] = {(double)xi.x, (double)xi.y, (double)xi.z};
  int id[3];
  for (int k = 0; k < 3; ++k) {
    double p = __dadd_rn(x[k], qoff[3 * q + k]);
    if (p < g.min[k]) p = __dadd_rn(p, g.box[k]);
    if (p > g.max[k]) p = __dsub_rn(p, g.box[k]);
    if (p < g.min[k] || p > g.max[k]) return -1;
    id[k] = (int)floor(__ddiv_rn(__dsub_rn(p, g.min[k]), g.step[k]));
  }
  return (long long)id[0] * ((long long)g.dims[1] * g.dims[2]) + (long long)id[1] * g.dims[2] + id[2];
}

// The same wrap in FP32 cell units, with the exact query wherever a point
// lies within the guard band of a grid edge or a cell face; distances by
// minimum image in the rectangular box (ReferenceForce::getDeltaRPeriodic:
// d -= L floor(d / L + 1/2)).
struct PeriodicQuery {
  float rel[3];   // (x_i - min) / step, cell units
  float inv[3];
  float wrap[3];  // box edge in cell units
  float L[3], iL[3];
  float eps;
  bool off;
  const TableGeom* g;
  const double* qoff;
  __device__ __forceinline__ void init(const TableGeom& geom, const float4 xi, const double* qo, long long cap) {
    g = &geom;
    qoff = qo;
    off = geom.ncell > cap;
    const double x[3] = {(double)xi.x, (double)xi.y, (double)xi.z};
    const int dmax = max(geom.dims[0], max(geom.dims[1], geom.dims[2]));
    for (int k = 0; k < 3; ++k) {
      rel[k] = (float)((x[k] - geom.min[k]) * geom.inv_step[k]);
      inv[k] = (float)geom.inv_step[k];
      wrap[k] = (float)(geom.box[k] * geom.inv_step[k]);
      L[k] = (float)geom.box[k];
      iL[k] = (float)geom.inv_box[k];
    }
    eps = 1e-4f + 64.0f * (float)(dmax + wrap[0] + wrap[1] + wrap[2]) * 5.96e-8f;
  }
  __device__ __forceinline__ void init(const Entries& t, const float4 xi, const double* qo) {
    init(*t.geom, xi, qo, usable_cells(t));
  }
  __device__ __forceinline__ long long cell(const float4 xi, const float4 v, int q) const {
    if (off) return -1;
    const TableGeom& G = *g;
    const float t0[3] = {fmaf(v.x, inv[0], rel[0]), fmaf(v.y, inv[1], rel[1]), fmaf(v.z, inv[2], rel[2])};
    int id[3];
    bool safe = true;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const float hi = (float)(G.dims[k] - 1);
      float t = t0[k];
      if (t < -eps) t += wrap[k];
      else if (t < eps) safe = false;
      if (t > hi + eps) t -= wrap[k];
      else if (t > hi - eps) safe = false;
      if (safe && (t < -eps || t > hi + eps)) return -1;
      const float f = floorf(t);
      const float fr = t - f;
      id[k] = (int)f;
      if (fr < eps || fr > 1.0f - eps || t < eps || t > hi - eps) safe = false;
    }
    if (!safe) return query_exact_wrap(G, xi, qoff, q);
    return (long long)id[0] * ((long long)G.dims[1] * G.dims[2]) + (long long)id[1] * G.dims[2] + id[2];
  }
  __device__ __forceinline__ float3 delta(const float4 a, const float4 xi, const float4 v) const {
    float d[3] = {(a.x - xi.x) - v.x, (a.y - xi.y) - v.y, (a.z - xi.z) - v.z};
#pragma unroll
    for (int k = 0; k < 3; ++k) d[k] = fmaf(-L[k], floorf(fmaf(d[k], iL[k], 0.5f)), d[k]);
    return make_float3(d[0], d[1], d[2]);
  }
};

// Exact GBSW table: FP32 query; the table's membership margin covers a
// point landing in a neighbouring cell.
struct TightQuery {
  float xr[3];
  float inv_h;
  int dims[3];
  __device__ __forceinline__ void init(const TableGeom& g, const float4 xi, const double*, long long cap) {
    xr[0] = (float)((double)xi.x - g.min[0]);
    xr[1] = (float)((double)xi.y - g.min[1]);
    xr[2] = (float)((double)xi.z - g.min[2]);
    inv_h = (float)g.inv_step[0];
    const bool off = g.ncell > cap;  // more cells than allocated: no cell
    dims[0] = off ? 0 : g.dims[0];
    dims[1] = off ? 0 : g.dims[1];
    dims[2] = off ? 0 : g.dims[2];
  }
  __device__ __forceinline__ void init(const Entries& t, const float4 xi, const double* qo) {
    init(*t.geom, xi, qo, usable_cells(t));
  }
  // 32-bit arithmetic: the exact table holds fewer than 2^31 cells (checked
  // when it is sized); one unsigned compare per axis tests both bounds
  __device__ __forceinline__ int cell_at(float ox, float oy, float oz) const {
    const int cx = (int)floorf((xr[0] + ox) * inv_h);
    const int cy = (int)floorf((xr[1] + oy) * inv_h);
    const int cz = (int)floorf((xr[2] + oz) * inv_h);
    if ((unsigned)cx >= (unsigned)dims[0] || (unsigned)cy >= (unsigned)dims[1] || (unsigned)cz >= (unsigned)dims[2])
      return -1;
    return (cx * dims[1] + cy) * dims[2] + cz;
  }
  __device__ __forceinline__ int cell(const float4, const float4 v, int) const { return cell_at(v.x, v.y, v.z); }
  __device__ __forceinline__ float3 delta(const float4 a, const float4 xi, const float4 v) const {
    return make_float3((a.x - xi.x) - v.x, (a.y - xi.y) - v.y, (a.z - xi.z) - v.z);
  }
};

// The reference's move of a point off the standalone grid of a periodic
// system (query_exact_wrap) in FP64, as shifts: false if the point misses.
__device__ bool wrap_shift_exact(const TableGeom& g, const float4 xi, const double* qoff, int q, float sh[3]) {
  const double x[3] = {(double)xi.x, (double)xi.y, (double)xi.z};
  for (int k = 0; k < 3; ++k) {
    double p = __dadd_rn(x[k], qoff[3 * q + k]);
    double s = 0.0;
    if (p < g.min[k]) {
      p = __dadd_rn(p, g.box[k]);
      s = g.box[k];
    }
    if (p > g.max[k]) {
      p = __dsub_rn(p, g.box[k]);
      s -= g.box[k];
    }
    if (p < g.min[k] || p > g.max[k]) return false;
    sh[k] = (float)s;
  }
  return true;
}

// Exact GBSW table of a periodic system (CutoffPeriodic).  The reference
// moves a point lying off its standalone grid by one box edge along each
// axis, and reads the list of the cell the moved point p' falls in
// (CharmmReferenceGBSW.cpp:522-535).  That list holds every atom within
// reach of p', at distances below half a box edge (the table is only used
// when the grid's pad plus a cell diagonal is below half the shortest edge),
// so minimum-image distances are the distances to p' and V(p) is the exact
// product at p'.  This query makes the reference's move (FP32 with the FP64
// decision within a guard band of the grid's edges) and looks p' up in the
// exact table; distances are by minimum image.
struct PeriodicTightQuery : TightQuery {
  float xw[3];    // x_i - the standalone grid's lower edge (nm)
  float span[3];  // the standalone grid's extent (nm)
  float L[3], iL[3];
  float eps;
  const TableGeom* wg;
  const double* qoff;
  __device__ __forceinline__ void init(const Entries& t, const float4 xi, const double* qo) {
    TightQuery::init(*t.geom, xi, qo, usable_cells(t));
    const TableGeom& W = *t.wrap;
    wg = t.wrap;
    qoff = qo;
    float ext = 0.0f;
    const double x[3] = {(double)xi.x, (double)xi.y, (double)xi.z};
    for (int k = 0; k < 3; ++k) {
      xw[k] = (float)(x[k] - W.min[k]);
      span[k] = (float)(W.max[k] - W.min[k]);
      L[k] = (float)W.box[k];
      iL[k] = (float)W.inv_box[k];
      ext = fmaxf(ext, fabsf(xw[k]) + span[k] + L[k]);
    }
    // FP32 rounding of x_i - min + v (+- L), with room to spare
    eps = 1e-5f + 16.0f * 1.1920929e-7f * (ext + 4.0f);
  }
  __device__ __forceinline__ int cell(const float4 xi, const float4 v, int q) const {
    const float vv[3] = {v.x, v.y, v.z};
    float sh[3];
    bool safe = true;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      float a = xw[k] + vv[k];
      float s = 0.0f;
      bool sk = fabsf(a) >= eps;
      if (a < 0.0f) {
        a += L[k];
        s = L[k];
      }
      sk = sk && fabsf(a - span[k]) >= eps;
      if (a > span[k]) {
        a -= L[k];
        s -= L[k];
      }
      sk = sk && fabsf(a) >= eps && fabsf(a - span[k]) >= eps;
      if (sk && (a < 0.0f || a > span[k])) return -1;  // off the grid on this axis: a miss
      safe = safe && sk;
      sh[k] = s;
    }
    if (!safe && !wrap_shift_exact(*wg, xi, qoff, q, sh)) return -1;
    return cell_at(v.x + sh[0], v.y + sh[1], v.z + sh[2]);
  }
  __device__ __forceinline__ float3 delta(const float4 a, const float4 xi, const float4 v) const {
    float d[3] = {(a.x - xi.x) - v.x, (a.y - xi.y) - v.y, (a.z - xi.z) - v.z};
#pragma unroll
    for (int k = 0; k < 3; ++k) d[k] = fmaf(-L[k], floorf(fmaf(d[k], iL[k], 0.5f)), d[k]);
    return make_float3(d[0], d[1], d[2]);
  }
};

// The exact table's query types (cell records with the first entry, lists
// in aligned pairs, buried cells).
template <class Q>
struct IsTight {
  static constexpr bool value = false;
};
template <>
struct IsTight<TightQuery> {
  static constexpr bool value = true;
};
template <>
struct IsTight<PeriodicTightQuery> {
  static constexpr bool value = true;
};

// s = p / (1 + p) with p = exp(beta (S - lambda)): the solvent fraction
__device__ __forceinline__ float logistic_solvent(float beta, float lambda, float S, float& p) {
  p = __expf(beta * (S - lambda));
  return __fdividef(p, 1.0f + p);
}

}  // namespace
}  // namespace gbx
