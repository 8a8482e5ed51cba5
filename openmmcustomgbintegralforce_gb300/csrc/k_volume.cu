// Born-radius integrals and the chain rule through every quadrature point.
//
// Work decomposition: one warp = 32 consecutive atoms x one chunk of
// quadrature points; all lanes visit the same point index q at the same
// time, so the quadrature data is a warp-uniform broadcast and the 32 points
// x_i + v_q sit as close together as the atoms themselves, which keeps the
// cell lists they read hot in L1.
//
// Integrals.  The reference accumulates I_n = sum_q w_q/r_q^(n-2) * (1 - V_q)
// (GBSWIntegral.cpp:142-146) and then forms 1/r0 - I4 and 1/(4 r0^4) - I7,
// which cancel to ~3 and ~4 significant digits -- fatal in FP32.  Here the
// kernels accumulate the complement J_n = sum_q w_q/r_q^(n-2) * s_q, with s_q
// the solvent fraction (GBSW: V_q; GBMV: 1 - V_q = p/(1+p)), all terms >= 0,
// and the host supplies the FP64 constants S_n = sum_q w_q/r_q^(n-2), so that
// I_n = S_n - J_n and 1/r0 - I4 = (1/r0 - S4) + J4 without cancellation.
//
// Cell query.  The reference picks a point's cell with FP64 arithmetic
// (CharmmReferenceGBSW.cpp:539-549, CustomGBIntegral.cpp:284-324).  The kernel
// computes it in FP32 and redoes it in FP64 only when the FP32 coordinate
// lies within a guard band of a cell face, so every point reads the same list
// as the reference.
#include <math.h>

#include "gbx_internal.cuh"

namespace gbx {
namespace {

constexpr int kThreads = 128;

struct Quad {
  const float4* qv;     // (vx, vy, vz, r)
  const float2* qw;     // (w/r^2, w/r^5)
  const double* qoff;   // FP64 offsets [3Q]
};

struct Table {
  const TableGeom* geom;
  const int* count;
  const int* start;
  const int* entries;
};

// FP64 query exactly as the reference (separately rounded operations).
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

// Per-lane precomputed query state.
struct QueryState {
  float rel[3];    // (x_i - min) / step in FP32 (cell units)
  float inv[3];    // 1 / step
  float eps;       // guard band in cell units
};

__device__ __forceinline__ QueryState make_query(const TableGeom& g, const float4 xi) {
  QueryState s;
  const double x[3] = {(double)xi.x, (double)xi.y, (double)xi.z};
  int dmax = max(g.dims[0], max(g.dims[1], g.dims[2]));
  for (int k = 0; k < 3; ++k) {
    s.rel[k] = (float)((x[k] - g.min[k]) / g.step[k]);
    s.inv[k] = (float)(1.0 / g.step[k]);
  }
  // FP32 error of rel + v*inv is a few ulp of the largest cell coordinate
  s.eps = 1e-4f + 64.0f * (float)dmax * 5.96e-8f;
  return s;
}

__device__ __forceinline__ long long query_cell(const TableGeom& g, const QueryState& s, const float4 xi,
                                                const float4 v, const double* qoff, int q) {
  const float t[3] = {fmaf(v.x, s.inv[0], s.rel[0]), fmaf(v.y, s.inv[1], s.rel[1]), fmaf(v.z, s.inv[2], s.rel[2])};
  int id[3];
  bool safe = true;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const float f = floorf(t[k]);
    const float fr = t[k] - f;
    id[k] = (int)f;
    if (fr < s.eps || fr > 1.0f - s.eps) safe = false;
    if (g.mode == GBX_TABLE_PERIODIC) {
      if (id[k] < 0 || id[k] >= g.dims[k]) safe = false;  // wraps: exact path
    } else {
      // outside [min, max] -> no list; max = min + (dims-1) step
      if (t[k] < -s.eps || t[k] > (float)(g.dims[k] - 1) + s.eps) return -1;
      if (t[k] < s.eps || t[k] > (float)(g.dims[k] - 1) - s.eps) safe = false;
    }
  }
  if (!safe) return query_exact(g, xi, qoff, q);
  return (long long)id[0] * ((long long)g.dims[1] * g.dims[2]) + (long long)id[1] * g.dims[2] + id[2];
}

// ---------------------------------------------------------------------------
// Volume models.  d = x_j - p (point to atom), formed as (x_j - x_i) - v so
// the FP32 difference of nearby atoms is exact.
// ---------------------------------------------------------------------------

// Work counters for roofline accounting: compiled out unless requested.
template <bool ON>
struct Work {
  __device__ __forceinline__ void eval() {}
  __device__ __forceinline__ void shell() {}
};
template <>
struct Work<true> {
  unsigned long long e = 0, s = 0;
  __device__ __forceinline__ void eval() { ++e; }
  __device__ __forceinline__ void shell() { ++s; }
};

// GBSW volume, CharmmReferenceGBSW.cpp:616-639 / GBSWIntegral.cpp:187-224:
// V = prod_j u_j over the switching shell, 0 as soon as an atom buries the point.
template <class W>
__device__ __forceinline__ float gbsw_volume(const ModelConst& m, const float4* __restrict__ pos,
                                             const int* __restrict__ list, int cnt, const float4 xi, const float4 v,
                                             W& wk) {
  float V = 1.0f;
  for (int l = 0; l < cnt; ++l) {
    const int j = __ldg(list + l);
    const float4 a = __ldg(pos + j);
    const float dx = (a.x - xi.x) - v.x, dy = (a.y - xi.y) - v.y, dz = (a.z - xi.z) - v.z;
    const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
    const float lo = a.w - m.sw, hi = a.w + m.sw;
    wk.eval();
    if (r2 <= lo * lo) return 0.0f;
    if (r2 < hi * hi) {
      wk.shell();
      const float dr = sqrtf(r2) - a.w;
      V *= fmaf(dr, fmaf(-m.c3 * dr, dr, m.c1), 0.5f);
    }
  }
  return V;
}

// The same volume reading inline (x, y, z, R') entries of the exact table.
template <class W>
__device__ __forceinline__ float gbsw_volume_inline(const ModelConst& m, const float4* __restrict__ list, int cnt,
                                                    const float4 xi, const float4 v, W& wk) {
  float V = 1.0f;
  for (int l = 0; l < cnt; ++l) {
    const float4 a = __ldg(list + l);
    const float dx = (a.x - xi.x) - v.x, dy = (a.y - xi.y) - v.y, dz = (a.z - xi.z) - v.z;
    const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
    const float lo = a.w - m.sw, hi = a.w + m.sw;
    wk.eval();
    if (r2 <= lo * lo) return 0.0f;
    if (r2 < hi * hi) {
      wk.shell();
      const float dr = sqrtf(r2) - a.w;
      V *= fmaf(dr, fmaf(-m.c3 * dr, dr, m.c1), 0.5f);
    }
  }
  return V;
}

// GBMV-I, GBMVIntegralTypeI.cpp:155-173: S = sum_j exp(gamma_j r^4).
template <class W>
__device__ __forceinline__ float gbmv1_sum(const float4* __restrict__ pos, const int* __restrict__ list, int cnt,
                                           const float4 xi, const float4 v, W& wk) {
  float S = 0.0f;
  for (int l = 0; l < cnt; ++l) {
    const int j = __ldg(list + l);
    const float4 a = __ldg(pos + j);
    const float dx = (a.x - xi.x) - v.x, dy = (a.y - xi.y) - v.y, dz = (a.z - xi.z) - v.z;
    const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
    S += __expf(a.w * (r2 * r2));
    wk.eval();
  }
  return S;
}

struct Gbmv2State {
  float s1, s2, vx, vy, vz;
};

// GBMV-II, GBMVIntegralTypeII.cpp:163-191.
template <class W>
__device__ __forceinline__ Gbmv2State gbmv2_sums(const float4* __restrict__ pos, const float2* __restrict__ par,
                                                 const int* __restrict__ list, int cnt, const float4 xi,
                                                 const float4 v, W& wk) {
  Gbmv2State s{0.f, 0.f, 0.f, 0.f, 0.f};
  for (int l = 0; l < cnt; ++l) {
    const int j = __ldg(list + l);
    const float4 a = __ldg(pos + j);
    const float K = __ldg(&par[j].x);
    const float dx = (a.x - xi.x) - v.x, dy = (a.y - xi.y) - v.y, dz = (a.z - xi.z) - v.z;
    const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
    float F = __fdividef(a.w, fmaf(100.0f, r2, K));
    F = F * F;
    s.s1 += F;
    s.s2 = fmaf(r2, F * F, s.s2);
    s.vx = fmaf(dx, F, s.vx);
    s.vy = fmaf(dy, F, s.vy);
    s.vz = fmaf(dz, F, s.vz);
    wk.eval();
  }
  return s;
}

__device__ __forceinline__ float logistic_solvent(float beta, float lambda, float S, float& p) {
  p = __expf(beta * (S - lambda));
  return __fdividef(p, 1.0f + p);
}

__device__ __forceinline__ float gbmv2_S(const ModelConst& m, const Gbmv2State& s) {
  const float s3sq = fmaf(s.vx, s.vx, fmaf(s.vy, s.vy, s.vz * s.vz));
  return m.s0 * s.s1 * s.s2 / s3sq;
}

// ---------------------------------------------------------------------------
// Integral kernel
// ---------------------------------------------------------------------------
template <int MODEL, bool COUNT>
__global__ void __launch_bounds__(kThreads) integral_kernel(const float4* __restrict__ pos,
                                                            const float2* __restrict__ par, int n, Table tab,
                                                            Quad quad, ModelConst m, int chunk, int n_chunks,
                                                            float* __restrict__ Jpart,
                                                            unsigned long long* __restrict__ work) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) / kWarp;
  const int lane = threadIdx.x % kWarp;
  const int n_groups = (n + kWarp - 1) / kWarp;
  if (warp >= n_groups * n_chunks) return;
  const int g = warp % n_groups, c = warp / n_groups;
  const int i = g * kWarp + lane;
  const bool active = i < n;
  const TableGeom geom = *tab.geom;
  const float4 xi = active ? pos[i] : pos[0];
  const QueryState qs = make_query(geom, xi);
  const int q0 = c * chunk, q1 = min(m.nq, q0 + chunk);
  float J4 = 0.0f, J7 = 0.0f;
  Work<COUNT> wk;
  for (int q = q0; q < q1; ++q) {
    const float4 v = quad.qv[q];
    const float2 w = quad.qw[q];
    long long cell = query_cell(geom, qs, xi, v, quad.qoff, q);
    int cnt = 0;
    const int* list = nullptr;
    if (cell >= 0) {
      cnt = tab.count[cell];
      list = tab.entries + tab.start[cell];
    }
    float s;
    if (MODEL == GBX_MODEL_GBSW) {
      s = gbsw_volume(m, pos, list, cnt, xi, v, wk);
    } else if (MODEL == GBX_MODEL_GBMV1) {
      float p;
      s = logistic_solvent(m.beta, m.lambda, gbmv1_sum(pos, list, cnt, xi, v, wk), p);
    } else {
      if (cnt == 0) {
        s = 1.0f;  // empty list: V = 0 (GBMVIntegralTypeII.cpp:140)
      } else {
        float p;
        s = logistic_solvent(m.beta, m.lambda, gbmv2_S(m, gbmv2_sums(pos, par, list, cnt, xi, v, wk)), p);
      }
    }
    J4 = fmaf(w.x, s, J4);
    J7 = fmaf(w.y, s, J7);
  }
  if (active) {
    Jpart[(size_t)c * n + i] = J4;
    Jpart[((size_t)n_chunks + c) * n + i] = J7;
  }
  if constexpr (COUNT) {
    unsigned long long e = wk.e, sh = wk.s;
    for (int off = 16; off > 0; off >>= 1) {
      e += __shfl_xor_sync(0xffffffffu, e, off);
      sh += __shfl_xor_sync(0xffffffffu, sh, off);
    }
    if (lane == 0) {
      atomicAdd(&work[0], e);
      atomicAdd(&work[1], sh);
    }
  }
}

// ---------------------------------------------------------------------------
// Chain-rule kernel: F_k -= c * ds/dx_k, F_i += c * ds/dx_k with
// c = dE/dJ4_i w/r^2 + dE/dJ7_i w/r^5 (GBSWIntegral.cpp:271-314,
// GBMVIntegralTypeI.cpp:195-224, GBMVIntegralTypeII.cpp:221-282).  With ADJ,
// also dE/dR_k += c * ds/dR_k for every list atom (i's own radius included).
// ---------------------------------------------------------------------------
template <int MODEL, bool ADJ>
__global__ void __launch_bounds__(kThreads) chain_kernel(const float4* __restrict__ pos,
                                                         const float2* __restrict__ par, int n, Table tab,
                                                         Quad quad, ModelConst m, int chunk, int n_chunks,
                                                         const float2* __restrict__ dEdJ,
                                                         unsigned long long* __restrict__ force, int stride,
                                                         unsigned long long* __restrict__ dEdR) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) / kWarp;
  const int lane = threadIdx.x % kWarp;
  const int n_groups = (n + kWarp - 1) / kWarp;
  if (warp >= n_groups * n_chunks) return;
  const int g = warp % n_groups, c = warp / n_groups;
  const int i = g * kWarp + lane;
  const bool active = i < n;
  const TableGeom geom = *tab.geom;
  const float4 xi = active ? pos[i] : pos[0];
  const float2 de = active ? dEdJ[i] : make_float2(0.f, 0.f);
  const QueryState qs = make_query(geom, xi);
  const int q0 = c * chunk, q1 = min(m.nq, q0 + chunk);
  float fix = 0.f, fiy = 0.f, fiz = 0.f;
  Work<false> dummy;
  const bool quirk = m.cutoff_chain_quirk && m.cutoff2 > 0.0f;
  for (int q = q0; q < q1 && active; ++q) {
    const float4 v = quad.qv[q];
    const float2 w = quad.qw[q];
    const float cq = fmaf(de.x, w.x, de.y * w.y);
    if (cq == 0.0f) continue;
    long long cell = query_cell(geom, qs, xi, v, quad.qoff, q);
    int cnt = 0;
    const int* list = nullptr;
    if (cell >= 0) {
      cnt = tab.count[cell];
      list = tab.entries + tab.start[cell];
    }
    if (cnt == 0) continue;
    if (MODEL == GBX_MODEL_GBSW) {
      const float V = gbsw_volume(m, pos, list, cnt, xi, v, dummy);
      if (V == 0.0f) continue;
      for (int l = 0; l < cnt; ++l) {
        const int k = __ldg(list + l);
        const float4 a = __ldg(pos + k);
        const float dx = (a.x - xi.x) - v.x, dy = (a.y - xi.y) - v.y, dz = (a.z - xi.z) - v.z;
        const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
        const float lo = a.w - m.sw, hi = a.w + m.sw;
        if (!(r2 > lo * lo && r2 < hi * hi)) continue;
        const float r = sqrtf(r2);
        const float dr = r - a.w;
        const float u = fmaf(dr, fmaf(-m.c3 * dr, dr, m.c1), 0.5f);
        const float du = fmaf(-3.0f * m.c3 * dr, dr, m.c1);
        const float Vu = __fdividef(V, u);
        if (ADJ) red_add_fixed(&dEdR[k], cq * Vu * du * (-0.9520f));
        if (k == i) continue;
        const float gs = cq * Vu * du / r;  // c * ds/d(delta) / delta
        if (!quirk || ((a.x - xi.x) * (a.x - xi.x) + (a.y - xi.y) * (a.y - xi.y) + (a.z - xi.z) * (a.z - xi.z)) <=
                          m.cutoff2) {
          red_add_fixed(&force[k], -gs * dx);
          red_add_fixed(&force[k + stride], -gs * dy);
          red_add_fixed(&force[k + 2 * stride], -gs * dz);
        }
        fix = fmaf(gs, dx, fix);
        fiy = fmaf(gs, dy, fiy);
        fiz = fmaf(gs, dz, fiz);
      }
    } else if (MODEL == GBX_MODEL_GBMV1) {
      float p;
      const float S = gbmv1_sum(pos, list, cnt, xi, v, dummy);
      logistic_solvent(m.beta, m.lambda, S, p);
      const float dsdS = __fdividef(m.beta * p, (1.0f + p) * (1.0f + p));
      const float cS = cq * dsdS;
      if (cS == 0.0f) continue;
      for (int l = 0; l < cnt; ++l) {
        const int k = __ldg(list + l);
        const float4 a = __ldg(pos + k);
        const float dx = (a.x - xi.x) - v.x, dy = (a.y - xi.y) - v.y, dz = (a.z - xi.z) - v.z;
        const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
        const float r4 = r2 * r2;
        const float e = __expf(a.w * r4);
        if (ADJ) {
          const float R = __ldg(&par[k].x);
          red_add_fixed(&dEdR[k], cS * e * r4 * (-4.0f * a.w / R));
        }
        if (k == i) continue;
        const float gs = cS * 4.0f * a.w * e * r2;
        red_add_fixed(&force[k], -gs * dx);
        red_add_fixed(&force[k + stride], -gs * dy);
        red_add_fixed(&force[k + 2 * stride], -gs * dz);
        fix = fmaf(gs, dx, fix);
        fiy = fmaf(gs, dy, fiy);
        fiz = fmaf(gs, dz, fiz);
      }
    } else {
      const Gbmv2State st = gbmv2_sums(pos, par, list, cnt, xi, v, dummy);
      const float s3sq = fmaf(st.vx, st.vx, fmaf(st.vy, st.vy, st.vz * st.vz));
      float p;
      logistic_solvent(m.beta, m.lambda, m.s0 * st.s1 * st.s2 / s3sq, p);
      const float dsdS = __fdividef(m.beta * p, (1.0f + p) * (1.0f + p));
      const float cS = cq * dsdS * m.s0;
      if (cS == 0.0f) continue;
      const float inv3 = 1.0f / s3sq;
      const float t1 = st.s2 * inv3;             // d s1 term
      const float t2 = st.s1 * inv3;             // d s2 term
      const float t3 = -st.s1 * st.s2 * inv3 * inv3;  // d s3^2 term
      for (int l = 0; l < cnt; ++l) {
        const int k = __ldg(list + l);
        const float4 a = __ldg(pos + k);
        const float2 pk = __ldg(par + k);
        const float dx = (a.x - xi.x) - v.x, dy = (a.y - xi.y) - v.y, dz = (a.z - xi.z) - v.z;
        const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
        const float T = fmaf(100.0f, r2, pk.x);
        const float CT = __fdividef(a.w, T);
        const float F = CT * CT;
        const float dFf = -400.0f * CT * CT * __fdividef(1.0f, T);  // dF/d(delta) = dFf * delta
        const float vd = st.vx * dx + st.vy * dy + st.vz * dz;
        if (ADJ) {
          const float R = pk.y;
          const float Cp = 10.0f * m.p1, Tp = Cp - 200.0f * R;
          const float dFdR = 2.0f * CT * __fdividef(Cp * T - a.w * Tp, T * T);
          const float val = t1 * dFdR + t2 * (r2 * 2.0f * F * dFdR) + t3 * (2.0f * vd * dFdR);
          red_add_fixed(&dEdR[k], cS * val);
        }
        if (k == i) continue;
        // dS/d(delta_k) / s0 = t1 dFf d + t2 2F(F + dFf r2) d + t3 2 (F v + vd dFf d)
        const float sc = t1 * dFf + t2 * 2.0f * F * fmaf(dFf, r2, F) + t3 * 2.0f * vd * dFf;
        const float gx = cS * fmaf(sc, dx, t3 * 2.0f * F * st.vx);
        const float gy = cS * fmaf(sc, dy, t3 * 2.0f * F * st.vy);
        const float gz = cS * fmaf(sc, dz, t3 * 2.0f * F * st.vz);
        red_add_fixed(&force[k], -gx);
        red_add_fixed(&force[k + stride], -gy);
        red_add_fixed(&force[k + 2 * stride], -gz);
        fix += gx;
        fiy += gy;
        fiz += gz;
      }
    }
  }
  if (active) {
    red_add_fixed(&force[i], fix);
    red_add_fixed(&force[i + stride], fiy);
    red_add_fixed(&force[i + 2 * stride], fiz);
  }
}

// ---------------------------------------------------------------------------
// GBSW on the exact table (k_tight.cu).  One warp per (atom, quadrature
// chunk), lanes over quadrature points: the atom is warp-uniform, the
// per-atom sums are fixed-shape warp reductions, and the atoms a warp's
// lanes scatter forces to in one instruction are spread around the sphere.
// ---------------------------------------------------------------------------
struct TightTable {
  const TableGeom* geom;
  const int* count;   // -1: buried cell
  const int* start;
  const float4* entry;
  const int* index;
};

struct TightQuery {
  float xr[3];  // atom position relative to the grid origin
  float inv_h;
  int dims[3];
};

__device__ __forceinline__ TightQuery make_tight_query(const TableGeom& g, const float4 xi) {
  TightQuery t;
  t.xr[0] = (float)((double)xi.x - g.min[0]);
  t.xr[1] = (float)((double)xi.y - g.min[1]);
  t.xr[2] = (float)((double)xi.z - g.min[2]);
  t.inv_h = (float)(1.0 / g.step[0]);
  t.dims[0] = g.dims[0];
  t.dims[1] = g.dims[1];
  t.dims[2] = g.dims[2];
  return t;
}

// cell of x_i + v, or -1 outside the grid (no shell reaches there)
__device__ __forceinline__ long long tight_cell(const TightQuery& t, const float4 v) {
  const int cx = (int)floorf((t.xr[0] + v.x) * t.inv_h);
  const int cy = (int)floorf((t.xr[1] + v.y) * t.inv_h);
  const int cz = (int)floorf((t.xr[2] + v.z) * t.inv_h);
  if (cx < 0 || cy < 0 || cz < 0 || cx >= t.dims[0] || cy >= t.dims[1] || cz >= t.dims[2]) return -1;
  return ((long long)cx * t.dims[1] + cy) * t.dims[2] + cz;
}

template <bool COUNT>
__global__ void __launch_bounds__(kThreads) tight_integral_kernel(const float4* __restrict__ pos, int n,
                                                                  TightTable tab, Quad quad, ModelConst m,
                                                                  int chunk, int n_chunks,
                                                                  float* __restrict__ Jpart,
                                                                  unsigned long long* __restrict__ work) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) / kWarp;
  const int lane = threadIdx.x % kWarp;
  if (warp >= n * n_chunks) return;
  const int i = warp % n, c = warp / n;
  const TableGeom& geom = *tab.geom;
  const float4 xi = pos[i];
  const TightQuery tq = make_tight_query(geom, xi);
  const int q0 = c * chunk, q1 = min(m.nq, q0 + chunk);
  float J4 = 0.0f, J7 = 0.0f;
  Work<COUNT> wk;
  for (int q = q0 + lane; q < q1; q += kWarp) {
    const float4 v = quad.qv[q];
    const float2 w = quad.qw[q];
    const long long cell = tight_cell(tq, v);
    float V = 1.0f;
    if (cell >= 0) {
      const int cnt = tab.count[cell];
      if (cnt < 0) {
        V = 0.0f;
      } else if (cnt > 0) {
        V = gbsw_volume_inline(m, tab.entry + tab.start[cell], cnt, xi, v, wk);
      }
    }
    J4 = fmaf(w.x, V, J4);
    J7 = fmaf(w.y, V, J7);
  }
  for (int off = 16; off > 0; off >>= 1) {
    J4 += __shfl_xor_sync(0xffffffffu, J4, off);
    J7 += __shfl_xor_sync(0xffffffffu, J7, off);
  }
  if (lane == 0) {
    Jpart[(size_t)c * n + i] = J4;
    Jpart[((size_t)n_chunks + c) * n + i] = J7;
  }
  if constexpr (COUNT) {
    unsigned long long e = wk.e, sh = wk.s;
    for (int off = 16; off > 0; off >>= 1) {
      e += __shfl_xor_sync(0xffffffffu, e, off);
      sh += __shfl_xor_sync(0xffffffffu, sh, off);
    }
    if (lane == 0) {
      atomicAdd(&work[0], e);
      atomicAdd(&work[1], sh);
    }
  }
}

template <bool ADJ>
__global__ void __launch_bounds__(kThreads) tight_chain_kernel(const float4* __restrict__ pos, int n,
                                                               TightTable tab, Quad quad, ModelConst m, int chunk,
                                                               int n_chunks, const float2* __restrict__ dEdJ,
                                                               unsigned long long* __restrict__ force, int stride,
                                                               unsigned long long* __restrict__ dEdR) {
  constexpr int kKeep = 4;  // in-shell entries remembered from the first pass
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) / kWarp;
  const int lane = threadIdx.x % kWarp;
  if (warp >= n * n_chunks) return;
  const int i = warp % n, c = warp / n;
  const TableGeom& geom = *tab.geom;
  const float4 xi = pos[i];
  const float2 de = dEdJ[i];
  const TightQuery tq = make_tight_query(geom, xi);
  const int q0 = c * chunk, q1 = min(m.nq, q0 + chunk);
  const bool quirk = m.cutoff_chain_quirk && m.cutoff2 > 0.0f;
  float fix = 0.f, fiy = 0.f, fiz = 0.f;
  for (int q = q0 + lane; q < q1; q += kWarp) {
    const float4 v = quad.qv[q];
    const float2 w = quad.qw[q];
    const float cq = fmaf(de.x, w.x, de.y * w.y);
    const long long cell = tight_cell(tq, v);
    if (cell < 0 || cq == 0.0f) continue;
    const int cnt = tab.count[cell];
    if (cnt <= 0) continue;  // buried (V = 0) or no shell (V = 1): no gradient
    const int s = tab.start[cell];
    // pass 1: volume, remembering the first in-shell entries
    float V = 1.0f;
    int keep[kKeep];
    int nk = 0, nshell = 0;
    for (int l = 0; l < cnt; ++l) {
      const float4 a = __ldg(tab.entry + s + l);
      const float dx = (a.x - xi.x) - v.x, dy = (a.y - xi.y) - v.y, dz = (a.z - xi.z) - v.z;
      const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
      const float lo = a.w - m.sw, hi = a.w + m.sw;
      if (r2 <= lo * lo) {
        V = 0.0f;
        break;
      }
      if (r2 < hi * hi) {
        const float dr = sqrtf(r2) - a.w;
        V *= fmaf(dr, fmaf(-m.c3 * dr, dr, m.c1), 0.5f);
        if (nk < kKeep) keep[nk++] = l;
        ++nshell;
      }
    }
    if (V == 0.0f || nshell == 0) continue;
    // pass 2: d V / d x_k = (V / u_k) u'_k d_k / r_k for each in-shell atom k
    const int scan = nshell <= kKeep ? nk : cnt;
    for (int t = 0; t < scan; ++t) {
      const int l = nshell <= kKeep ? keep[t] : t;
      const float4 a = __ldg(tab.entry + s + l);
      const float dx = (a.x - xi.x) - v.x, dy = (a.y - xi.y) - v.y, dz = (a.z - xi.z) - v.z;
      const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
      const float lo = a.w - m.sw, hi = a.w + m.sw;
      if (!(r2 > lo * lo && r2 < hi * hi)) continue;
      const float r = sqrtf(r2);
      const float dr = r - a.w;
      const float u = fmaf(dr, fmaf(-m.c3 * dr, dr, m.c1), 0.5f);
      const float du = fmaf(-3.0f * m.c3 * dr, dr, m.c1);
      const float Vu = __fdividef(V, u);
      const int k = __ldg(tab.index + s + l);
      if (ADJ) red_add_fixed(&dEdR[k], cq * Vu * du * (-0.9520f));
      if (k == i) continue;
      const float gs = cq * Vu * du / r;
      const float ex = a.x - xi.x, ey = a.y - xi.y, ez = a.z - xi.z;
      if (!quirk || fmaf(ex, ex, fmaf(ey, ey, ez * ez)) <= m.cutoff2) {
        red_add_fixed(&force[k], -gs * dx);
        red_add_fixed(&force[k + stride], -gs * dy);
        red_add_fixed(&force[k + 2 * stride], -gs * dz);
      }
      fix = fmaf(gs, dx, fix);
      fiy = fmaf(gs, dy, fiy);
      fiz = fmaf(gs, dz, fiz);
    }
  }
  for (int off = 16; off > 0; off >>= 1) {
    fix += __shfl_xor_sync(0xffffffffu, fix, off);
    fiy += __shfl_xor_sync(0xffffffffu, fiy, off);
    fiz += __shfl_xor_sync(0xffffffffu, fiz, off);
  }
  if (lane == 0) {
    red_add_fixed(&force[i], fix);
    red_add_fixed(&force[i + stride], fiy);
    red_add_fixed(&force[i + 2 * stride], fiz);
  }
}

int tight_blocks(const Context* ctx) {
  const long long warps = (long long)ctx->n * ctx->n_chunks;
  return (int)((warps * kWarp + kThreads - 1) / kThreads);
}

template <int MODEL>
gbx_status launch_integrals_t(Context* ctx, const float4* pos, const ModelConst& m, const Table& t,
                              const Quad& qd, bool count_work) {
  const int n_groups = (ctx->n + kWarp - 1) / kWarp;
  const int chunk = (m.nq + ctx->n_chunks - 1) / ctx->n_chunks;
  const long long warps = (long long)n_groups * ctx->n_chunks;
  const int blocks = (int)((warps * kWarp + kThreads - 1) / kThreads);
  if (count_work)
    integral_kernel<MODEL, true><<<blocks, kThreads, 0, ctx->stream>>>(pos, ctx->d_par, ctx->n, t, qd, m, chunk,
                                                                        ctx->n_chunks, ctx->d_J, ctx->d_work);
  else
    integral_kernel<MODEL, false><<<blocks, kThreads, 0, ctx->stream>>>(pos, ctx->d_par, ctx->n, t, qd, m, chunk,
                                                                         ctx->n_chunks, ctx->d_J, nullptr);
  return GBX_OK;
}

template <int MODEL, bool ADJ>
gbx_status launch_chain_t(Context* ctx, const float4* pos, const ModelConst& m, const Table& t, const Quad& qd,
                          unsigned long long* force, int stride) {
  const int n_groups = (ctx->n + kWarp - 1) / kWarp;
  const int chunk = (m.nq + ctx->n_chunks - 1) / ctx->n_chunks;
  const long long warps = (long long)n_groups * ctx->n_chunks;
  const int blocks = (int)((warps * kWarp + kThreads - 1) / kThreads);
  chain_kernel<MODEL, ADJ><<<blocks, kThreads, 0, ctx->stream>>>(pos, ctx->d_par, ctx->n, t, qd, m, chunk,
                                                                  ctx->n_chunks, ctx->d_dEdJ, force, stride,
                                                                  ctx->d_dEdR_fx);
  return GBX_OK;
}

}  // namespace

gbx_status launch_integrals(Context* ctx, const float4* pos, bool count_work) {
  const ModelConst m = make_model_const(ctx);
  if (ctx->use_tight) {
    const TightTable tt{ctx->d_tgeom, ctx->d_tcount, ctx->d_tstart, ctx->d_tentry, ctx->d_tindex};
    const Quad qd{ctx->d_qv, ctx->d_qw, ctx->d_qoff};
    const int chunk = (m.nq + ctx->n_chunks - 1) / ctx->n_chunks;
    if (count_work)
      tight_integral_kernel<true><<<tight_blocks(ctx), kThreads, 0, ctx->stream>>>(pos, ctx->n, tt, qd, m, chunk,
                                                                                   ctx->n_chunks, ctx->d_J,
                                                                                   ctx->d_work);
    else
      tight_integral_kernel<false><<<tight_blocks(ctx), kThreads, 0, ctx->stream>>>(pos, ctx->n, tt, qd, m, chunk,
                                                                                    ctx->n_chunks, ctx->d_J,
                                                                                    nullptr);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
      ctx->last_error = std::string("integral launch: ") + cudaGetErrorString(e);
      return GBX_ERR_CUDA;
    }
    return GBX_OK;
  }
  const Table t{ctx->d_geom, ctx->d_cell_count, ctx->d_cell_start, ctx->d_entries};
  const Quad qd{ctx->d_qv, ctx->d_qw, ctx->d_qoff};
  gbx_status s;
  switch (ctx->cfg.model) {
    case GBX_MODEL_GBSW: s = launch_integrals_t<GBX_MODEL_GBSW>(ctx, pos, m, t, qd, count_work); break;
    case GBX_MODEL_GBMV1: s = launch_integrals_t<GBX_MODEL_GBMV1>(ctx, pos, m, t, qd, count_work); break;
    default: s = launch_integrals_t<GBX_MODEL_GBMV2>(ctx, pos, m, t, qd, count_work); break;
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    ctx->last_error = std::string("integral launch: ") + cudaGetErrorString(e);
    return GBX_ERR_CUDA;
  }
  return s;
}

gbx_status launch_chain(Context* ctx, const float4* pos, unsigned long long* force, int stride, bool adjoint) {
  const ModelConst m = make_model_const(ctx);
  if (ctx->use_tight) {
    const TightTable tt{ctx->d_tgeom, ctx->d_tcount, ctx->d_tstart, ctx->d_tentry, ctx->d_tindex};
    const Quad qd{ctx->d_qv, ctx->d_qw, ctx->d_qoff};
    const int chunk = (m.nq + ctx->n_chunks - 1) / ctx->n_chunks;
    if (adjoint)
      tight_chain_kernel<true><<<tight_blocks(ctx), kThreads, 0, ctx->stream>>>(
          pos, ctx->n, tt, qd, m, chunk, ctx->n_chunks, ctx->d_dEdJ, force, stride, ctx->d_dEdR_fx);
    else
      tight_chain_kernel<false><<<tight_blocks(ctx), kThreads, 0, ctx->stream>>>(
          pos, ctx->n, tt, qd, m, chunk, ctx->n_chunks, ctx->d_dEdJ, force, stride, ctx->d_dEdR_fx);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
      ctx->last_error = std::string("chain launch: ") + cudaGetErrorString(e);
      return GBX_ERR_CUDA;
    }
    return GBX_OK;
  }
  const Table t{ctx->d_geom, ctx->d_cell_count, ctx->d_cell_start, ctx->d_entries};
  const Quad qd{ctx->d_qv, ctx->d_qw, ctx->d_qoff};
  gbx_status s;
  switch (ctx->cfg.model * 2 + (adjoint ? 1 : 0)) {
    case 0: s = launch_chain_t<GBX_MODEL_GBSW, false>(ctx, pos, m, t, qd, force, stride); break;
    case 1: s = launch_chain_t<GBX_MODEL_GBSW, true>(ctx, pos, m, t, qd, force, stride); break;
    case 2: s = launch_chain_t<GBX_MODEL_GBMV1, false>(ctx, pos, m, t, qd, force, stride); break;
    case 3: s = launch_chain_t<GBX_MODEL_GBMV1, true>(ctx, pos, m, t, qd, force, stride); break;
    case 4: s = launch_chain_t<GBX_MODEL_GBMV2, false>(ctx, pos, m, t, qd, force, stride); break;
    default: s = launch_chain_t<GBX_MODEL_GBMV2, true>(ctx, pos, m, t, qd, force, stride); break;
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    ctx->last_error = std::string("chain launch: ") + cudaGetErrorString(e);
    return GBX_ERR_CUDA;
  }
  return s;
}

}  // namespace gbx
