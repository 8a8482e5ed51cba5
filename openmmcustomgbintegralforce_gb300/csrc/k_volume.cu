// Born-radius integrals and the chain rule through every quadrature point.
//
// Work decomposition: one warp = one atom i x one chunk of quadrature
// points.  GBSW integrals: lanes over points, each lane walking its point's
// list and refilling from a per-warp queue; the GBSW chain rule: lanes over
// the shaping entries of recorded points; GBMV integrals: two lanes per
// point; the GBMV chain rule: the warp on one point at a time, lanes over
// its list.  The atom is warp-uniform, every per-atom sum is a fixed-shape
// warp reduction (bit-reproducible), the quadrature data is read coalesced,
// and lists are stored inline (x, y, z, model parameter) so there is no
// dependent index -> position gather.
//
// Integrals.  The reference accumulates I_n = sum_q w_q/r_q^(n-2) * (1 - V_q)
// (GBSWIntegral.cpp:142-146) and then forms 1/r0 - I4 and 1/(4 r0^4) - I7,
// which cancel to a few significant digits -- fatal in FP32.  The kernels
// accumulate the complement J_n = sum_q w_q/r_q^(n-2) * s_q, with s_q the
// solvent fraction (GBSW: V_q; GBMV: 1 - V_q = p/(1+p)), all terms >= 0; the
// host supplies the FP64 constants S_n = sum_q w_q/r_q^(n-2), so that
// I_n = S_n - J_n and 1/r0 - I4 = (1/r0 - S4) + J4 without cancellation.
//
// Tables.  GBMV and the integral-class GBSW read the reference's own table,
// whose list contents define the result: the point's cell is computed in
// FP32 and redone in FP64 exactly as the reference does
// (CharmmReferenceGBSW.cpp:539-549, CustomGBIntegral.cpp:284-324) whenever
// the FP32 coordinate lies within a guard band of a cell face.  The
// standalone GBSW model reads the exact table of k_tight.cu instead, except
// in a periodic box, where it reads the reference table through a query that
// wraps the point as the reference does and measures minimum-image distances.
#include <math.h>

#include <type_traits>

#include "gbx_internal.cuh"
#include "queries.cuh"

namespace gbx {
namespace {

constexpr int kThreads = 128;

// Work counters for roofline accounting: compiled out unless requested.
template <bool ON>
struct Work {
  __device__ __forceinline__ void eval() {}
  __device__ __forceinline__ void shell() {}
};
template <>
struct Work<true> {
  unsigned long long e = 0, s = 0;    // the volume pass: list walk with the first-burying-atom exit
  unsigned long long fe = 0, fs = 0;  // the chain pass: every listed atom of every point
  __device__ __forceinline__ void eval() { ++e; }
  __device__ __forceinline__ void shell() { ++s; }
};

// ---------------------------------------------------------------------------
// Volume models on inline entries.  d = x_j - p comes from the query's
// delta(): (x_j - x_i) - v, so the FP32 difference of nearby atoms is exact,
// and in a periodic system its minimum image.
// ---------------------------------------------------------------------------

// GBSW, CharmmReferenceGBSW.cpp:616-639 / GBSWIntegral.cpp:187-224: V is the
// product of u_j over the switching shells, 0 once an atom buries the point.
template <class Q, class W>
__device__ __forceinline__ float gbsw_volume(const Q& qy, const ModelConst& m, const float4* __restrict__ list,
                                             int cnt, const float4 xi, const float4 v, W& wk) {
  float V = 1.0f;
  for (int l = 0; l < cnt; ++l) {
    const float4 a = __ldg(list + l);
    const float3 d = qy.delta(a, xi, v);
    const float r2 = fmaf(d.x, d.x, fmaf(d.y, d.y, d.z * d.z));
    const float lo = a.w - m.sw, hi = a.w + m.sw;
    wk.eval();
    if (r2 <= lo * lo) return 0.0f;
    if (r2 < hi * hi) {
      wk.shell();
      const float dr = r2 * rsqrtf(r2) - a.w;
      V *= fmaf(dr, fmaf(-m.c3 * dr, dr, m.c1), 0.5f);
    }
  }
  return V;
}

// GBMV-I, GBMVIntegralTypeI.cpp:155-173: S = sum_j exp(gamma_j r^4).
template <class Q, class W>
__device__ __forceinline__ float gbmv1_sum(const Q& qy, const float4* __restrict__ list, int cnt, const float4 xi,
                                           const float4 v, W& wk) {
  float S = 0.0f;
  for (int l = 0; l < cnt; ++l) {
    const float4 a = __ldg(list + l);
    const float3 d = qy.delta(a, xi, v);
    const float r2 = fmaf(d.x, d.x, fmaf(d.y, d.y, d.z * d.z));
    S += __expf(a.w * (r2 * r2));
    wk.eval();
  }
  return S;
}

struct Gbmv2State {
  float s1, s2, vx, vy, vz;
};

// GBMV-II, GBMVIntegralTypeII.cpp:163-191:
// F_j = (C_j / (C_j + 100 r^2 - 100 R_j^2))^2, sums of F, r^2 F^2 and F d.
template <class Q, class W>
__device__ __forceinline__ Gbmv2State gbmv2_sums(const Q& qy, const float4* __restrict__ list,
                                                 const float2* __restrict__ par,
                                                 int cnt, const float4 xi, const float4 v, W& wk) {
  Gbmv2State s{0.f, 0.f, 0.f, 0.f, 0.f};
  for (int l = 0; l < cnt; ++l) {
    const float4 a = __ldg(list + l);
    const float K = __ldg(&par[l].x);
    const float3 d = qy.delta(a, xi, v);
    const float r2 = fmaf(d.x, d.x, fmaf(d.y, d.y, d.z * d.z));
    float F = __fdividef(a.w, fmaf(100.0f, r2, K));
    F = F * F;
    s.s1 += F;
    s.s2 = fmaf(r2, F * F, s.s2);
    s.vx = fmaf(d.x, F, s.vx);
    s.vy = fmaf(d.y, F, s.vy);
    s.vz = fmaf(d.z, F, s.vz);
    wk.eval();
  }
  return s;
}

__device__ __forceinline__ float gbmv2_S(const ModelConst& m, const Gbmv2State& s) {
  const float s3sq = fmaf(s.vx, s.vx, fmaf(s.vy, s.vy, s.vz * s.vz));
  return m.s0 * s.s1 * s.s2 / s3sq;
}

// Chain-pass work of one point, counted only for roofline accounting: the
// reference chain kernel (reduceIntegralForce.cu:45-65) visits the whole cell
// list of every point, with the derivative work inside the switching shell.
template <int MODEL, class Q>
__device__ __forceinline__ void count_chain_work(const Q& qy, const ModelConst& m, const Entries& t, long long cell,
                                                 const float4 xi, const float4 v, Work<true>& wk) {
  if (cell < 0) return;
  const int2 cs = __ldg(t.cell + cell);
  if (cs.x <= 0) return;
  wk.fe += cs.x;
  if constexpr (MODEL != GBX_MODEL_GBSW) {
    wk.fs += cs.x;
  } else {
    for (int l = 0; l < cs.x; ++l) {
      const float4 a = __ldg(t.e + cs.y + l);
      const float3 d = qy.delta(a, xi, v);
      const float r2 = fmaf(d.x, d.x, fmaf(d.y, d.y, d.z * d.z));
      const float lo = a.w - m.sw, hi = a.w + m.sw;
      wk.fs += (r2 > lo * lo && r2 < hi * hi) ? 1 : 0;
    }
  }
}

template <int MODEL, class Q, class W>
__device__ __forceinline__ float solvent_fraction(const Q& qy, const ModelConst& m, const Entries& t, long long cell,
                                                  const float4 xi, const float4 v, W& wk) {
  int cnt = 0, s = 0;
  if (cell >= 0) {
    const int2 cs = __ldg(t.cell + cell);
    cnt = cs.x;
    if (cnt < 0) return 0.0f;  // buried cell (exact table)
    s = cs.y;
  }
  if (MODEL == GBX_MODEL_GBSW) return cnt > 0 ? gbsw_volume(qy, m, t.e + s, cnt, xi, v, wk) : 1.0f;
  float p;
  if (MODEL == GBX_MODEL_GBMV1) return logistic_solvent(m.beta, m.lambda, gbmv1_sum(qy, t.e + s, cnt, xi, v, wk), p);
  if (cnt == 0) return 1.0f;  // empty list: V = 0 (GBMVIntegralTypeII.cpp:140)
  return logistic_solvent(m.beta, m.lambda, gbmv2_S(m, gbmv2_sums(qy, t.e + s, t.par + s, cnt, xi, v, wk)), p);
}

// ---------------------------------------------------------------------------
// Integral kernel: J4 = sum w/r^2 s, J7 = sum w/r^5 s per (atom, chunk).
// ---------------------------------------------------------------------------
// GBMV point state kept for the chain rule (saves it re-summing every list):
// GBMV-I S at state[i Q + q]; GBMV-II s1, s2, vx, vy, vz in five planes of N Q.
template <int MODEL, class Q, class W>
__device__ __forceinline__ float gbmv_fraction_keep(const Q& qy, const ModelConst& m, const Entries& t, long long cell,
                                                    const float4 xi, const float4 v, W& wk, float* state,
                                                    size_t idx, size_t plane) {
  int cnt = 0, s = 0;
  if (cell >= 0) {
    const int2 cs = __ldg(t.cell + cell);
    cnt = cs.x;
    s = cs.y;
  }
  float p;
  if constexpr (MODEL == GBX_MODEL_GBMV1) {
    const float S = gbmv1_sum(qy, t.e + s, cnt, xi, v, wk);
    state[idx] = S;
    return logistic_solvent(m.beta, m.lambda, S, p);
  } else {
    if (cnt == 0) return 1.0f;  // empty list: V = 0 (GBMVIntegralTypeII.cpp:140)
    const Gbmv2State st = gbmv2_sums(qy, t.e + s, t.par + s, cnt, xi, v, wk);
    state[idx] = st.s1;
    state[idx + plane] = st.s2;
    state[idx + 2 * plane] = st.vx;
    state[idx + 3 * plane] = st.vy;
    state[idx + 4 * plane] = st.vz;
    return logistic_solvent(m.beta, m.lambda, gbmv2_S(m, st), p);
  }
}

template <int MODEL, class Q, bool COUNT>
__global__ void __launch_bounds__(kThreads) integral_kernel(const float4* __restrict__ pos, int n, Entries tab,
                                                            Quad quad, ModelConst m, int chunk, int n_chunks,
                                                            float* __restrict__ Jpart,
                                                            unsigned long long* __restrict__ work,
                                                            float* __restrict__ state) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) / kWarp;
  const int lane = threadIdx.x % kWarp;
  if (warp >= n * n_chunks) return;
  const int i = warp % n, c = warp / n;
  const float4 xi = pos[i];
  Q query;
  query.init(tab, xi, quad.qoff);
  const int q0 = c * chunk, q1 = min(m.nq, q0 + chunk);
  float J4 = 0.0f, J7 = 0.0f;
  Work<COUNT> wk;
  for (int q = q0 + lane; q < q1; q += kWarp) {
    const float4 v = quad.qv[q];
    const float2 w = quad.qw[q];
    const long long cell = query.cell(xi, v, q);
    float s;
    if constexpr (MODEL != GBX_MODEL_GBSW)
      s = state ? gbmv_fraction_keep<MODEL>(query, m, tab, cell, xi, v, wk, state, (size_t)i * m.nq + q, (size_t)n * m.nq)
                : solvent_fraction<MODEL>(query, m, tab, cell, xi, v, wk);
    else
      s = solvent_fraction<MODEL>(query, m, tab, cell, xi, v, wk);
    if constexpr (COUNT) count_chain_work<MODEL>(query, m, tab, cell, xi, v, wk);
    J4 = fmaf(w.x, s, J4);
    J7 = fmaf(w.y, s, J7);
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
    unsigned long long e = wk.e, sh = wk.s, fe = wk.fe, fs = wk.fs;
    for (int off = 16; off > 0; off >>= 1) {
      e += __shfl_xor_sync(0xffffffffu, e, off);
      sh += __shfl_xor_sync(0xffffffffu, sh, off);
      fe += __shfl_xor_sync(0xffffffffu, fe, off);
      fs += __shfl_xor_sync(0xffffffffu, fs, off);
    }
    if (lane == 0) {
      atomicAdd(&work[0], e);
      atomicAdd(&work[1], sh);
      atomicAdd(&work[2], fe);
      atomicAdd(&work[3], fs);
    }
  }
}

// GBMV integrals with kGroup lanes per point: the group reads consecutive
// entries of the point's list (kGroup x 16 contiguous bytes per load instead
// of one line per lane), each lane sums every kGroup-th entry and the group
// combines its partial sums by shuffles in a fixed order.  The point's sums
// are kept for the chain rule as in integral_kernel.  Two lanes per point
// measured fastest (GBMV-II, 10k atoms: 1.27 ms against 1.64 ms for one lane,
// 1.47 ms for four and 2.0 ms for eight).
constexpr int kGroup = 2;

template <int MODEL, class Q>
__global__ void __launch_bounds__(kThreads) gbmv_integral_kernel(const float4* __restrict__ pos, int n, Entries tab,
                                                                 Quad quad, ModelConst m, int chunk, int n_chunks,
                                                                 float* __restrict__ Jpart, float* __restrict__ state) {
  constexpr int kPer = kWarp / kGroup;  // points per warp step
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) / kWarp;
  const int lane = threadIdx.x % kWarp;
  if (warp >= n * n_chunks) return;
  const int i = warp % n, c = warp / n;
  const int g = lane / kGroup, r = lane % kGroup;
  const float4 xi = pos[i];
  Q query;
  query.init(tab, xi, quad.qoff);
  const int q0 = c * chunk, q1 = min(m.nq, q0 + chunk);
  const size_t plane = (size_t)n * m.nq;
  float J4 = 0.0f, J7 = 0.0f;
  for (int base = q0; base < q1; base += kPer) {
    const int q = base + g;
    int cnt = 0, s = 0;
    float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
    if (q < q1) {
      v = quad.qv[q];
      const long long cell = query.cell(xi, v, q);
      if (cell >= 0) {
        const int2 cs = __ldg(tab.cell + cell);
        cnt = cs.x;
        s = cs.y;
      }
    }
    float S1 = 0.f, S2 = 0.f, Vx = 0.f, Vy = 0.f, Vz = 0.f;
    for (int l = r; l < cnt; l += kGroup) {
      const float4 a = __ldg(tab.e + s + l);
      const float3 d = query.delta(a, xi, v);
      const float r2 = fmaf(d.x, d.x, fmaf(d.y, d.y, d.z * d.z));
      if constexpr (MODEL == GBX_MODEL_GBMV1) {
        S1 += __expf(a.w * (r2 * r2));
      } else {
        float F = __fdividef(a.w, fmaf(100.0f, r2, __ldg(&tab.par[s + l].x)));
        F = F * F;
        S1 += F;
        S2 = fmaf(r2, F * F, S2);
        Vx = fmaf(d.x, F, Vx);
        Vy = fmaf(d.y, F, Vy);
        Vz = fmaf(d.z, F, Vz);
      }
    }
#pragma unroll
    for (int off = 1; off < kGroup; off <<= 1) {
      S1 += __shfl_xor_sync(0xffffffffu, S1, off);
      if constexpr (MODEL != GBX_MODEL_GBMV1) {
        S2 += __shfl_xor_sync(0xffffffffu, S2, off);
        Vx += __shfl_xor_sync(0xffffffffu, Vx, off);
        Vy += __shfl_xor_sync(0xffffffffu, Vy, off);
        Vz += __shfl_xor_sync(0xffffffffu, Vz, off);
      }
    }
    if (r == 0 && q < q1) {
      const size_t idx = (size_t)i * m.nq + q;
      float p, sf;
      if constexpr (MODEL == GBX_MODEL_GBMV1) {
        if (state) state[idx] = S1;
        sf = logistic_solvent(m.beta, m.lambda, S1, p);
      } else if (cnt == 0) {
        sf = 1.0f;  // empty list: V = 0 (GBMVIntegralTypeII.cpp:140)
      } else {
        const Gbmv2State st{S1, S2, Vx, Vy, Vz};
        if (state) {
          state[idx] = st.s1;
          state[idx + plane] = st.s2;
          state[idx + 2 * plane] = st.vx;
          state[idx + 3 * plane] = st.vy;
          state[idx + 4 * plane] = st.vz;
        }
        sf = logistic_solvent(m.beta, m.lambda, gbmv2_S(m, st), p);
      }
      const float2 w = quad.qw[q];
      J4 = fmaf(w.x, sf, J4);
      J7 = fmaf(w.y, sf, J7);
    }
  }
  for (int off = 16; off > 0; off >>= 1) {
    J4 += __shfl_xor_sync(0xffffffffu, J4, off);
    J7 += __shfl_xor_sync(0xffffffffu, J7, off);
  }
  if (lane == 0) {
    Jpart[(size_t)c * n + i] = J4;
    Jpart[((size_t)n_chunks + c) * n + i] = J7;
  }
}

// ---------------------------------------------------------------------------
// GBSW integral pass that also records which points the chain rule needs:
// (q, V, mask) for every point with V > 0 shaped by an atom other than i,
// bit l of mask set for each such in-shell list entry l.  The chain rule
// then visits only those entries, with lanes spread over them.  Warp w owns
// records [w R, (w + 1) R), filled in the order points finish; count[w] =
// points recorded, or -1 - needed when they did not fit or a list was longer
// than 64 (the chain rule walks that warp's lists instead).  Records are
// stored evict-first: they are read once, and the lookup table must stay in
// L2.
// ---------------------------------------------------------------------------
struct ShellSink {
  int4* rec;
  int* st;             // the point's list start, beside each record
  int* count;          // [warps]
  unsigned* max_seen;  // largest per-warp need of this call
  int R;               // records per warp
};

__device__ __forceinline__ float shell_g(const ModelConst& m, float V, float dr) {
  const float u = fmaf(dr, fmaf(-m.c3 * dr, dr, m.c1), 0.5f);
  const float du = fmaf(-3.0f * m.c3 * dr, dr, m.c1);
  return __fdividef(V, u) * du;
}

// x << n with PTX semantics: a shift of 32 or more gives 0 (two 32-bit
// halves of the 64-bit mask, each set without a branch on l).
__device__ __forceinline__ unsigned shl_clamped(unsigned x, unsigned n) {
  unsigned r;
  asm("shl.b32 %0, %1, %2;" : "=r"(r) : "r"(x), "r"(n));
  return r;
}

// True if list entry l is atom i itself: its inline position is bitwise
// atom i's, and only then is the index read.
__device__ __forceinline__ bool is_self(const float4 a, const float4 xi, const int* __restrict__ index, int l, int i) {
  return a.x == xi.x && a.y == xi.y && a.z == xi.z && __ldg(index + l) == i;
}

// GBSW integrals with lanes refilled from a ring queue.  A warp classifies
// kRefill points at a time (empty cell: V = 1; buried cell or buried by the
// list's first entry: V = 0) and queues the points that have a list whenever
// fewer than kRefillBelow are pending;
// every lane evaluates list entries of its own point and takes the next
// queued point as soon as its own is finished, so a long list keeps one lane
// busy instead of the whole warp waiting on it, and lanes idle only at the
// end of the warp's quadrature range.  The walk per point is the sequential one of gbsw_volume
// (same order, same early exit).  J is summed in an order fixed by the input
// alone, so runs are bit-reproducible.
constexpr int kStage = 256;        // ring entries per warp (a power of two)
constexpr int kRefill = 128;       // points classified per refill
constexpr int kRefillBelow = 64;   // refill when fewer entries are pending
static_assert(kRefillBelow - 1 + kRefill <= kStage, "ring overwrite");
constexpr int kEnt = 2;            // list entries per lane step, loaded one step ahead (3 and 4 measured slower)
static_assert(kEnt == 2, "the exact table's lists are read in aligned pairs");

// Persistent: a grid of resident blocks whose warps take (atom, chunk) items
// from `next_item` one at a time, so a warp that finishes a cheap item (a
// buried or exposed atom) takes the next instead of idling until the slowest
// warp of its block is done.  Each item's results depend on the item alone.
template <class Q, bool EMIT>
__global__ void __launch_bounds__(kThreads) gbsw_integral_kernel(const float4* __restrict__ pos, int n, Entries tab,
                                                                 Quad quad, ModelConst m, int chunk, int n_chunks,
                                                                 float* __restrict__ Jpart, ShellSink sink,
                                                                 unsigned* __restrict__ next_item) {
  __shared__ int3 s_queue[kThreads / kWarp][kStage];  // (q, list start, list length)
  __shared__ int s_long[kThreads / kWarp];  // a shaping entry beyond list position 63
  // the exact table: lists start at even entries and each cell's record sits
  // beside its first entry, so both are read 32 bytes at a time
  constexpr bool kTight = IsTight<Q>::value;
  const int lane = threadIdx.x % kWarp;
  const int wib = threadIdx.x / kWarp;
  const unsigned lt = (1u << lane) - 1u;
  for (;;) {
  unsigned item = 0;
  if (lane == 0) item = atomicAdd(next_item, 1u);
  const int warp = (int)__shfl_sync(0xffffffffu, item, 0);
  if (warp >= n * n_chunks) return;
  if (lane == 0) s_long[wib] = 0;
  __syncwarp();
  int3* queue = s_queue[wib];
  int fill = 0;  // warp-uniform: points recorded so far (may exceed R)
  const int i = warp % n, c = warp / n;
  int4* region = EMIT ? sink.rec + (size_t)warp * sink.R : nullptr;
  const float4 xi = pos[i];
  Q query;
  query.init(tab, xi, quad.qoff);
  const int q0 = c * chunk, q1 = min(m.nq, q0 + chunk);
  float J4 = 0.0f, J7 = 0.0f;
  int head = 0, tail = 0;  // warp-uniform ring positions: taken, queued
  int next = q0;           // warp-uniform: first point not yet classified
  if constexpr (kTight) {
    // Radial shells well inside atom i's own burying sphere (r below
    // R'_i - w by more than FP32 rounding of |v|^2 can reach) hold only
    // points with V = 0: the exact table lists atom i in every cell they
    // fall in, so the walk would end on it at the latest.  V = 0 adds
    // nothing to J and records nothing, so they are skipped unclassified.
    const float lo = xi.w - m.sw;
    const int nrad = m.nq / m.nshell;
    int inner = 0;  // the leading shells that lie inside
    for (int r0 = 0; r0 < nrad; r0 += kWarp) {
      const int ir = r0 + lane;
      const bool in = ir < nrad && quad.qv[ir * m.nshell].w * (1.0f + 1.0f / 1024.0f) < lo;
      const unsigned out = __ballot_sync(0xffffffffu, !in);
      inner = r0 + (out ? __ffs(out) - 1 : kWarp);
      if (out) break;
    }
    next = max(q0, inner * m.nshell);
  }
  int q = 0, s = 0, cnt = 0, l = 0;
  float4 an[kEnt];  // the next kEnt list entries
#pragma unroll
  for (int u = 0; u < kEnt; ++u) an[u] = make_float4(0.f, 0.f, 0.f, 0.f);
  bool has = false;
  unsigned sm_lo = 0u, sm_hi = 0u;  // bit l of (hi:lo): in-shell entry l is not atom i
  float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
  float2 w = make_float2(0.f, 0.f);
  float V = 1.0f;
  while (true) {
    if (tail - head < kRefillBelow && next < q1) {
      // classify the next kRefill points into the ring (at most
      // kRefillBelow - 1 + kRefill entries are ever pending: no overwrite)
#pragma unroll 4
      for (int k = 0; k < kRefill / kWarp; ++k) {
        const int qc = next + k * kWarp + lane;
        int2 cs = make_int2(-1, 0);
        if (qc < q1) {
          const float4 vc = quad.qv[qc];
          const long long cell = query.cell(xi, vc, qc);
          float4 a0 = make_float4(0.f, 0.f, 0.f, 0.f);
          if constexpr (kTight) {
            // the exact table keeps each cell's first entry beside its
            // record: one load, not one after the other
            cs = make_int2(0, 0);
            if (cell >= 0) {
              const Float4x2 r = ldg_pair(tab.first + cell);
              a0 = r.a;
              cs = make_int2(__float_as_int(r.b.x), __float_as_int(r.b.y));
            }
          } else {
            cs = cell >= 0 ? __ldg(tab.cell + cell) : make_int2(0, 0);
          }
          if (cs.x == 0) {
            const float2 wc = quad.qw[qc];
            J4 += wc.x;
            J7 += wc.y;
          } else if (cs.x > 0) {
            // the list's first entry, the likeliest burying atom, buries most
            // listed points: V = 0 adds nothing, the point is not queued
            if constexpr (!kTight) a0 = __ldg(tab.e + cs.y);
            const float3 d = query.delta(a0, xi, vc);
            const float r2 = fmaf(d.x, d.x, fmaf(d.y, d.y, d.z * d.z));
            const float lo = a0.w - m.sw;
            if (r2 <= lo * lo) cs.x = -1;
          }
        }
        const unsigned qm = __ballot_sync(0xffffffffu, cs.x > 0);
        if (cs.x > 0) queue[(tail + __popc(qm & lt)) & (kStage - 1)] = make_int3(qc, cs.y, cs.x);
        tail += __popc(qm);
      }
      next += kRefill;
      __syncwarp();
    }
    const unsigned need = __ballot_sync(0xffffffffu, !has);
    if (!has) {
      const int idx = head + __popc(need & lt);
      if (idx < tail) {
        const int3 e = queue[idx & (kStage - 1)];
        q = e.x;
        s = e.y;
        cnt = e.z;
        l = 0;
        sm_lo = 0u;
        sm_hi = 0u;
        V = 1.0f;
        has = true;
        v = quad.qv[q];
        w = quad.qw[q];
        if constexpr (kTight) {
          const Float4x2 p = ldg_pair(tab.e + s);
          an[0] = p.a;
          an[1] = p.b;
        } else {
#pragma unroll
          for (int u = 0; u < kEnt; ++u)
            if (u < cnt) an[u] = __ldg(tab.e + s + u);
        }
      }
    }
    head = min(head + __popc(need), tail);
    if (__ballot_sync(0xffffffffu, has) == 0u) {
      if (next >= q1) break;
      continue;
    }
    bool fin = false;
    if (has) {
      // kEnt list entries per step (entries l .. l + kEnt - 1 were loaded one step ahead)
      float4 cur[kEnt];
#pragma unroll
      for (int u = 0; u < kEnt; ++u) cur[u] = an[u];
      if constexpr (kTight) {
        // l is even here (a point advances kEnt entries per step until it
        // ends); a pair past an odd list's end reads its padding entry
        if (l + kEnt < cnt) {
          const Float4x2 p = ldg_pair(tab.e + s + l + kEnt);
          an[0] = p.a;
          an[1] = p.b;
        }
      } else {
#pragma unroll
        for (int u = 0; u < kEnt; ++u)
          if (l + kEnt + u < cnt) an[u] = __ldg(tab.e + s + l + kEnt + u);
      }
#pragma unroll
      for (int u = 0; u < kEnt; ++u) {
        if (fin) break;
        const float4 a = cur[u];
        const float3 d = query.delta(a, xi, v);
        const float r2 = fmaf(d.x, d.x, fmaf(d.y, d.y, d.z * d.z));
        const float lo = a.w - m.sw, hi = a.w + m.sw;
        if (r2 <= lo * lo) {
          V = 0.0f;
          fin = true;
        } else {
          if (r2 < hi * hi) {
            const float dr = r2 * rsqrtf(r2) - a.w;
            V *= fmaf(dr, fmaf(-m.c3 * dr, dr, m.c1), 0.5f);
            if (EMIT && !is_self(a, xi, tab.index + s, l, i)) {
              sm_lo |= shl_clamped(1u, (unsigned)l);
              sm_hi |= shl_clamped(1u, (unsigned)(l - 32));
              if (l >= 64) s_long[wib] = 1;
            }
          }
          fin = ++l == cnt;
        }
      }
    }
    if (fin) {
      J4 = fmaf(w.x, V, J4);
      J7 = fmaf(w.y, V, J7);
      has = false;
    }
    if (EMIT) {
      // slots in finishing order (the chain rule's sums do not depend on it)
      const bool emit = fin && (sm_lo | sm_hi) != 0u && V != 0.0f;
      const unsigned em = __ballot_sync(0xffffffffu, emit);
      if (emit) {
        const int slot = fill + __popc(em & lt);
        if (slot < sink.R) {
          __stcs(region + slot, make_int4(q, __float_as_int(V), (int)sm_lo, (int)sm_hi));
          __stcs(sink.st + (size_t)warp * sink.R + slot, s);
        }
      }
      fill += __popc(em);
    }
  }
  for (int off = 16; off > 0; off >>= 1) {
    J4 += __shfl_xor_sync(0xffffffffu, J4, off);
    J7 += __shfl_xor_sync(0xffffffffu, J7, off);
  }
  __syncwarp();
  if (lane == 0) {
    Jpart[(size_t)c * n + i] = J4;
    Jpart[((size_t)n_chunks + c) * n + i] = J7;
    if (EMIT) {
      sink.count[warp] = fill <= sink.R && !s_long[wib] ? fill : -1 - fill;
      if (fill > 0) atomicMax(sink.max_seen, (unsigned)fill);
    }
  }
  __syncwarp();  // the ring and the long-list flag are reused by the next item
  }
}

// ---------------------------------------------------------------------------
// Chain rule: with c = dE/dJ4_i w/r^2 + dE/dJ7_i w/r^5 for a point of atom i,
// F_k -= c ds/dx_k for every atom k shaping the point and F_i gets the
// opposite (the point moves with atom i) -- GBSWIntegral.cpp:271-314,
// GBMVIntegralTypeI.cpp:195-224, GBMVIntegralTypeII.cpp:221-282, and the
// Born-radius prefactor of CharmmReferenceGBSW.cpp:597-611 folded into
// dE/dJ.  With ADJ also dE/dR_k += c ds/dR_k for every shaping atom
// (atom i's own radius included).
// ---------------------------------------------------------------------------
struct ChainOut {
  unsigned long long* force;
  int stride;
  unsigned long long* dEdR;
  bool quirk;  // drop F_k beyond the cutoff (CharmmReferenceGBSW.cpp:291-292)
  float cutoff2;
};

// Records of the emitting integral pass (rec == nullptr: none this call).
struct ChainRecords {
  const int4* rec;  // (q, V, mask low, mask high) per recorded point
  const int* st;    // the point's list start
  const int* count;
  int R;
  const float* state;  // GBMV point state of the integral pass (nullptr: re-sum the lists)
};

// A component whose fixed-point value is 0 (|g| < 2^-33, common for distant
// GBMV atoms) changes nothing: its reduction is skipped, the result is the
// same bits.
__device__ __forceinline__ void push_force(const ChainOut& o, int k, float gx, float gy, float gz) {
  const long long fx = float_to_fixed_split(-gx), fy = float_to_fixed_split(-gy), fz = float_to_fixed_split(-gz);
  if (fx) atomicAdd(&o.force[k], (unsigned long long)fx);
  if (fy) atomicAdd(&o.force[k + o.stride], (unsigned long long)fy);
  if (fz) atomicAdd(&o.force[k + 2 * o.stride], (unsigned long long)fz);
}

// GBSW: the force -g on a shaping atom k (unless the cutoff quirk drops it)
// and +g on atom i, as one fixed-point integer triple: atom i gets the
// negation of what k gets, so the pair's momentum balances exactly and one
// conversion serves both.  The caller loads k together with the entry, so
// the two reads overlap instead of the index waiting on the arithmetic.
__device__ __forceinline__ void push_shaping(const ChainOut& o, int k, bool push, float gx, float gy, float gz,
                                             long long& fix, long long& fiy, long long& fiz) {
  const long long fx = float_to_fixed_split(-gx), fy = float_to_fixed_split(-gy), fz = float_to_fixed_split(-gz);
  if (push) {
    if (fx) atomicAdd(&o.force[k], (unsigned long long)fx);
    if (fy) atomicAdd(&o.force[k + o.stride], (unsigned long long)fy);
    if (fz) atomicAdd(&o.force[k + 2 * o.stride], (unsigned long long)fz);
  }
  fix -= fx;
  fiy -= fy;
  fiz -= fz;
}

template <int MODEL, class Q, bool ADJ>
__global__ void __launch_bounds__(kThreads) chain_kernel(const float4* __restrict__ pos, int n, Entries tab,
                                                         Quad quad, ModelConst m, int chunk, int n_chunks,
                                                         const float2* __restrict__ dEdJ, ChainOut out,
                                                         ChainRecords rr) {
  constexpr int kWalkKeep = 4;  // GBSW: in-shell entries remembered from the volume pass
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) / kWarp;
  const int lane = threadIdx.x % kWarp;
  if (warp >= n * n_chunks) return;
  const int i = warp % n, c = warp / n;
  const float4 xi = pos[i];
  const float2 de = dEdJ[i];
  // F_i as fixed-point integers: every contribution is rounded on its own, so
  // the record and the list-walk paths give the same bits
  long long fix = 0, fiy = 0, fiz = 0;
  Q query;
  query.init(tab, xi, quad.qoff);
  const int npts = rr.count ? rr.count[warp] : -1;
  if (MODEL == GBX_MODEL_GBSW && !ADJ && npts >= 0) {
    // recorded points, 32 at a time; lanes over their shaping entries
    const int4* region = rr.rec + (size_t)warp * rr.R;
    const int* sregion = rr.st + (size_t)warp * rr.R;
    // the next batch's records and list starts, loaded one batch ahead
    int4 prn = make_int4(0, 0, 0, 0);
    int psn = 0;
    if (lane < npts) {
      prn = __ldcs(region + lane);
      psn = __ldcs(sregion + lane);
    }
    for (int b = 0; b < npts; b += kWarp) {
      unsigned mlo = 0u, mhi = 0u;
      int st = 0;
      float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
      float V = 0.0f, cq = 0.0f;
      const int4 pr = prn;
      const int ps = psn;
      if (b + kWarp + lane < npts) {
        prn = __ldcs(region + b + kWarp + lane);
        psn = __ldcs(sregion + b + kWarp + lane);
      }
      if (b + lane < npts) {
        V = __int_as_float(pr.y);
        mlo = (unsigned)pr.z;
        mhi = (unsigned)pr.w;
        v = quad.qv[pr.x];
        const float2 w = quad.qw[pr.x];
        cq = fmaf(de.x, w.x, de.y * w.y);
        st = ps;  // written by the integral pass beside the record
      }
      const int len = __popc(mlo) + __popc(mhi);
      int incl = len;
      for (int off = 1; off < kWarp; off <<= 1) {
        const int u = __shfl_up_sync(0xffffffffu, incl, off);
        if (lane >= off) incl += u;
      }
      const int total = __shfl_sync(0xffffffffu, incl, kWarp - 1);
      for (int r = 0; r < total; r += kWarp) {
        const int p = r + lane;
        int o = 0;  // owner: the points whose entries end at or before p
        for (int step = 16; step > 0; step >>= 1)
          if (__shfl_sync(0xffffffffu, incl, o + step - 1) <= p) o += step;
        const int oend = __shfl_sync(0xffffffffu, incl, o), olen = __shfl_sync(0xffffffffu, len, o);
        const unsigned olo = __shfl_sync(0xffffffffu, mlo, o), ohi = __shfl_sync(0xffffffffu, mhi, o);
        const int ost = __shfl_sync(0xffffffffu, st, o);
        const float4 ov = make_float4(__shfl_sync(0xffffffffu, v.x, o), __shfl_sync(0xffffffffu, v.y, o),
                                      __shfl_sync(0xffffffffu, v.z, o), 0.0f);
        const float oV = __shfl_sync(0xffffffffu, V, o), ocq = __shfl_sync(0xffffffffu, cq, o);
        if (p >= total) continue;
        const int nth = p - (oend - olen);  // nth shaping entry of the owner
        const int nlo = __popc(olo);
        const int l = nth < nlo ? (int)__fns(olo, 0, nth + 1) : 32 + (int)__fns(ohi, 0, nth - nlo + 1);
        const int e = ost + l;
        const float4 a = __ldg(tab.e + e);
        const int k = __ldg(tab.index + e);
        const float3 d = query.delta(a, xi, ov);
        const float r2 = fmaf(d.x, d.x, fmaf(d.y, d.y, d.z * d.z));
        // the same expressions as the list walk below
        const float g = shell_g(m, oV, r2 * rsqrtf(r2) - a.w);
        const float gs = ocq * g * rsqrtf(r2);
        const float gx = gs * d.x, gy = gs * d.y, gz = gs * d.z;
        const float3 dd = query.delta(a, xi, make_float4(0.f, 0.f, 0.f, 0.f));  // x_k - x_i
        const float ex = dd.x, ey = dd.y, ez = dd.z;
        push_shaping(out, k, !out.quirk || fmaf(ex, ex, fmaf(ey, ey, ez * ez)) <= out.cutoff2, gx, gy, gz,
                     fix, fiy, fiz);
      }
    }
  } else {
    const int q0 = c * chunk, q1 = min(m.nq, q0 + chunk);
    for (int q = q0 + lane; q < q1; q += kWarp) {
      const float4 v = quad.qv[q];
      const float2 w = quad.qw[q];
      const float cq = fmaf(de.x, w.x, de.y * w.y);
      if (cq == 0.0f) continue;
      const long long cell = query.cell(xi, v, q);
      if (cell < 0) continue;
      const int2 cs = __ldg(tab.cell + cell);
      const int cnt = cs.x;
      if (cnt <= 0) continue;  // buried or empty: no atom shapes the point
      const int s = cs.y;
      const float4* E = tab.e + s;
      if (MODEL == GBX_MODEL_GBSW) {
        float V = 1.0f;
        int keep[kWalkKeep];
        int nk = 0, nshell = 0;
        for (int l = 0; l < cnt; ++l) {
          const float4 a = __ldg(E + l);
          const float3 d = query.delta(a, xi, v);
          const float r2 = fmaf(d.x, d.x, fmaf(d.y, d.y, d.z * d.z));
          const float lo = a.w - m.sw, hi = a.w + m.sw;
          if (r2 <= lo * lo) {
            V = 0.0f;
            break;
          }
          if (r2 < hi * hi) {
            const float dr = r2 * rsqrtf(r2) - a.w;
            V *= fmaf(dr, fmaf(-m.c3 * dr, dr, m.c1), 0.5f);
            if (nk < kWalkKeep) keep[nk++] = l;
            ++nshell;
          }
        }
        if (V == 0.0f || nshell == 0) continue;
        const int scan = nshell <= kWalkKeep ? nk : cnt;
        for (int t = 0; t < scan; ++t) {
          const int l = nshell <= kWalkKeep ? keep[t] : t;
          const float4 a = __ldg(E + l);
          const float3 d = query.delta(a, xi, v);
          const float r2 = fmaf(d.x, d.x, fmaf(d.y, d.y, d.z * d.z));
          const float lo = a.w - m.sw, hi = a.w + m.sw;
          if (!(r2 > lo * lo && r2 < hi * hi)) continue;
          // the same expressions as the record path (shell_g, then c g / r)
          const float g = shell_g(m, V, r2 * rsqrtf(r2) - a.w);
          const int k = __ldg(tab.index + s + l);
          // dV/dR_k = -(V/u) u' dR'/dR with R' = (R + 0.03) 0.952
          if (ADJ) red_add_fixed(&out.dEdR[k], cq * g * (-0.9520f));
          if (k == i) continue;
          const float gs = cq * g * rsqrtf(r2);
          const float gx = gs * d.x, gy = gs * d.y, gz = gs * d.z;
          const float3 dd = query.delta(a, xi, make_float4(0.f, 0.f, 0.f, 0.f));  // x_k - x_i
          const float ex = dd.x, ey = dd.y, ez = dd.z;
          push_shaping(out, k, !out.quirk || fmaf(ex, ex, fmaf(ey, ey, ez * ez)) <= out.cutoff2, gx,
                       gy, gz, fix, fiy, fiz);
        }
      } else if (MODEL == GBX_MODEL_GBMV1) {
        Work<false> wk;
        float p;
        const float Ssum = rr.state ? rr.state[(size_t)i * m.nq + q] : gbmv1_sum(query, E, cnt, xi, v, wk);
        logistic_solvent(m.beta, m.lambda, Ssum, p);
        const float cS = cq * __fdividef(m.beta * p, (1.0f + p) * (1.0f + p));  // c ds/dS
        if (cS == 0.0f) continue;
        float px = 0.f, py = 0.f, pz = 0.f;
        for (int l = 0; l < cnt; ++l) {
          const float4 a = __ldg(E + l);
          const float3 d = query.delta(a, xi, v);
          const float r2 = fmaf(d.x, d.x, fmaf(d.y, d.y, d.z * d.z));
          const float r4 = r2 * r2;
          const float e = __expf(a.w * r4);
          const int k = __ldg(tab.index + s + l);
          if (ADJ) red_add_fixed(&out.dEdR[k], cS * e * r4 * (-4.0f * a.w / __ldg(&tab.par[s + l].x)));
          if (k == i) continue;
          const float gs = cS * 4.0f * a.w * e * r2;  // dS/d(delta) = 4 gamma e r^2 delta
          const float gx = gs * d.x, gy = gs * d.y, gz = gs * d.z;
          push_force(out, k, gx, gy, gz);
          px += gx;
          py += gy;
          pz += gz;
        }
        // the point's pull on its own atom: summed in FP32 over the list, then fixed point
        fix += float_to_fixed(px);
        fiy += float_to_fixed(py);
        fiz += float_to_fixed(pz);
      } else {
        Work<false> wk;
        Gbmv2State st;
        if (rr.state) {
          const size_t idx = (size_t)i * m.nq + q, plane = (size_t)n * m.nq;
          st = Gbmv2State{rr.state[idx], rr.state[idx + plane], rr.state[idx + 2 * plane], rr.state[idx + 3 * plane],
                          rr.state[idx + 4 * plane]};
        } else {
          st = gbmv2_sums(query, E, tab.par + s, cnt, xi, v, wk);
        }
        const float s3sq = fmaf(st.vx, st.vx, fmaf(st.vy, st.vy, st.vz * st.vz));
        float p;
        logistic_solvent(m.beta, m.lambda, m.s0 * st.s1 * st.s2 / s3sq, p);
        const float cS = cq * __fdividef(m.beta * p, (1.0f + p) * (1.0f + p)) * m.s0;
        if (cS == 0.0f) continue;
        const float inv3 = 1.0f / s3sq;
        const float t1 = st.s2 * inv3;                  // d s1 term
        const float t2 = st.s1 * inv3;                  // d s2 term
        const float t3 = -st.s1 * st.s2 * inv3 * inv3;  // d s3^2 term
        float px = 0.f, py = 0.f, pz = 0.f;
        for (int l = 0; l < cnt; ++l) {
          const float4 a = __ldg(E + l);
          const float2 pk = __ldg(tab.par + s + l);
          const float3 d = query.delta(a, xi, v);
          const float r2 = fmaf(d.x, d.x, fmaf(d.y, d.y, d.z * d.z));
          const float T = fmaf(100.0f, r2, pk.x);
          const float CT = __fdividef(a.w, T);
          const float F = CT * CT;
          const float dFf = -400.0f * F * __fdividef(1.0f, T);  // dF/d(delta) = dFf delta
          const float vd = st.vx * d.x + st.vy * d.y + st.vz * d.z;
          const int k = __ldg(tab.index + s + l);
          if (ADJ) {
            const float R = pk.y;
            const float Cp = 10.0f * m.p1, Tp = Cp - 200.0f * R;
            const float dFdR = 2.0f * CT * __fdividef(Cp * T - a.w * Tp, T * T);
            red_add_fixed(&out.dEdR[k], cS * (t1 * dFdR + t2 * (r2 * 2.0f * F * dFdR) + t3 * (2.0f * vd * dFdR)));
          }
          if (k == i) continue;
          // dS/d(delta_k) / s0 = t1 dFf d + t2 2F (F + dFf r^2) d + 2 t3 (F v + vd dFf d)
          const float sc = t1 * dFf + t2 * 2.0f * F * fmaf(dFf, r2, F) + t3 * 2.0f * vd * dFf;
          const float gx = cS * fmaf(sc, d.x, t3 * 2.0f * F * st.vx);
          const float gy = cS * fmaf(sc, d.y, t3 * 2.0f * F * st.vy);
          const float gz = cS * fmaf(sc, d.z, t3 * 2.0f * F * st.vz);
          push_force(out, k, gx, gy, gz);
          px += gx;
          py += gy;
          pz += gz;
        }
        fix += float_to_fixed(px);
        fiy += float_to_fixed(py);
        fiz += float_to_fixed(pz);
      }
    }
  }
  for (int off = 16; off > 0; off >>= 1) {
    fix += __shfl_xor_sync(0xffffffffu, fix, off);
    fiy += __shfl_xor_sync(0xffffffffu, fiy, off);
    fiz += __shfl_xor_sync(0xffffffffu, fiz, off);
  }
  if (lane == 0) {
    atomicAdd(&out.force[i], (unsigned long long)fix);
    atomicAdd(&out.force[i + out.stride], (unsigned long long)fiy);
    atomicAdd(&out.force[i + 2 * out.stride], (unsigned long long)fiz);
  }
}

// GBMV chain rule with the warp cooperating on one point at a time: the
// point's sums come from the integral pass, lanes read consecutive entries of
// its list (coalesced; GBMV visits whole lists of nearly equal length), push
// their atom's force and accumulate the point's pull on atom i.  Lanes first
// take 32 points' cells together, then the warp walks those points in turn.
template <int MODEL, class Q, bool ADJ>
// Six blocks per SM (at most 80 registers): the occupancy this latency-bound
// kernel was measured fastest at; left to itself the compiler takes 87.
__global__ void __launch_bounds__(kThreads, 6) gbmv_chain_kernel(const float4* __restrict__ pos, int n, Entries tab,
                                                              Quad quad, ModelConst m, int chunk, int n_chunks,
                                                              const float2* __restrict__ dEdJ, ChainOut out,
                                                              const float* __restrict__ state) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) / kWarp;
  const int lane = threadIdx.x % kWarp;
  if (warp >= n * n_chunks) return;
  const int i = warp % n, c = warp / n;
  const float4 xi = pos[i];
  const float2 de = dEdJ[i];
  Q query;
  query.init(tab, xi, quad.qoff);
  const int q0 = c * chunk, q1 = min(m.nq, q0 + chunk);
  const size_t plane = (size_t)n * m.nq;
  long long fix = 0, fiy = 0, fiz = 0;
  for (int base = q0; base < q1; base += kWarp) {
    // lane t takes point base + t: its cell, its state (coalesced) and the
    // point's factors of the chain rule, which the warp then broadcasts
    const int qm = base + lane;
    float4 vm = make_float4(0.f, 0.f, 0.f, 0.f);
    int cntm = 0, sm = 0;
    float cSm = 0.0f;                    // c ds/dS (0: nothing to push)
    float t1m = 0.f, t2m = 0.f, t3m = 0.f;  // GBMV-II: d s1, d s2, d s3^2 factors
    float vxm = 0.f, vym = 0.f, vzm = 0.f;
    if (qm < q1) {
      vm = quad.qv[qm];
      const float2 w = quad.qw[qm];
      const float cq = fmaf(de.x, w.x, de.y * w.y);
      const long long cell = query.cell(xi, vm, qm);
      if (cell >= 0) {
        const int2 cs = __ldg(tab.cell + cell);
        cntm = cs.x;
        sm = cs.y;
      }
      if (cntm > 0 && cq != 0.0f) {
        const size_t idx = (size_t)i * m.nq + qm;
        float p;
        if constexpr (MODEL == GBX_MODEL_GBMV1) {
          logistic_solvent(m.beta, m.lambda, state[idx], p);
          cSm = cq * __fdividef(m.beta * p, (1.0f + p) * (1.0f + p));
        } else {
          const Gbmv2State st{state[idx], state[idx + plane], state[idx + 2 * plane], state[idx + 3 * plane],
                              state[idx + 4 * plane]};
          const float s3sq = fmaf(st.vx, st.vx, fmaf(st.vy, st.vy, st.vz * st.vz));
          logistic_solvent(m.beta, m.lambda, m.s0 * st.s1 * st.s2 / s3sq, p);
          cSm = cq * __fdividef(m.beta * p, (1.0f + p) * (1.0f + p)) * m.s0;
          const float inv3 = 1.0f / s3sq;
          t1m = st.s2 * inv3;
          t2m = st.s1 * inv3;
          t3m = -st.s1 * st.s2 * inv3 * inv3;
          vxm = st.vx;
          vym = st.vy;
          vzm = st.vz;
        }
      }
    }
    float px = 0.f, py = 0.f, pz = 0.f;  // this lane's share of the points' pull on atom i
    const int np = min(kWarp, q1 - base);
    for (int t = 0; t < np; ++t) {
      const int cnt = __shfl_sync(0xffffffffu, cntm, t), s = __shfl_sync(0xffffffffu, sm, t);
      const float cS = __shfl_sync(0xffffffffu, cSm, t);
      if (cnt <= 0 || cS == 0.0f) continue;
      const float4 v = make_float4(__shfl_sync(0xffffffffu, vm.x, t), __shfl_sync(0xffffffffu, vm.y, t),
                                   __shfl_sync(0xffffffffu, vm.z, t), 0.f);
      if constexpr (MODEL == GBX_MODEL_GBMV1) {
        for (int l = lane; l < cnt; l += kWarp) {
          const float4 a = __ldg(tab.e + s + l);
          const float3 d = query.delta(a, xi, v);
          const float r2 = fmaf(d.x, d.x, fmaf(d.y, d.y, d.z * d.z));
          const float r4 = r2 * r2;
          const float e = __expf(a.w * r4);
          const int k = __ldg(tab.index + s + l);
          if (ADJ) red_add_fixed(&out.dEdR[k], cS * e * r4 * (-4.0f * a.w / __ldg(&tab.par[s + l].x)));
          if (k == i) continue;
          const float gs = cS * 4.0f * a.w * e * r2;  // dS/d(delta) = 4 gamma e r^2 delta
          const float gx = gs * d.x, gy = gs * d.y, gz = gs * d.z;
          push_force(out, k, gx, gy, gz);
          px += gx;
          py += gy;
          pz += gz;
        }
      } else {
        const float t1 = __shfl_sync(0xffffffffu, t1m, t), t2 = __shfl_sync(0xffffffffu, t2m, t),
                    t3 = __shfl_sync(0xffffffffu, t3m, t);
        const Gbmv2State st{0.f, 0.f, __shfl_sync(0xffffffffu, vxm, t), __shfl_sync(0xffffffffu, vym, t),
                            __shfl_sync(0xffffffffu, vzm, t)};
        for (int l = lane; l < cnt; l += kWarp) {
          const float4 a = __ldg(tab.e + s + l);
          const float2 pk = __ldg(tab.par + s + l);
          const float3 d = query.delta(a, xi, v);
          const float r2 = fmaf(d.x, d.x, fmaf(d.y, d.y, d.z * d.z));
          const float T = fmaf(100.0f, r2, pk.x);
          const float CT = __fdividef(a.w, T);
          const float F = CT * CT;
          const float dFf = -400.0f * F * __fdividef(1.0f, T);  // dF/d(delta) = dFf delta
          const float vd = st.vx * d.x + st.vy * d.y + st.vz * d.z;
          const int k = __ldg(tab.index + s + l);
          if (ADJ) {
            const float R = pk.y;
            const float Cp = 10.0f * m.p1, Tp = Cp - 200.0f * R;
            const float dFdR = 2.0f * CT * __fdividef(Cp * T - a.w * Tp, T * T);
            red_add_fixed(&out.dEdR[k], cS * (t1 * dFdR + t2 * (r2 * 2.0f * F * dFdR) + t3 * (2.0f * vd * dFdR)));
          }
          if (k == i) continue;
          const float sc = t1 * dFf + t2 * 2.0f * F * fmaf(dFf, r2, F) + t3 * 2.0f * vd * dFf;
          const float gx = cS * fmaf(sc, d.x, t3 * 2.0f * F * st.vx);
          const float gy = cS * fmaf(sc, d.y, t3 * 2.0f * F * st.vy);
          const float gz = cS * fmaf(sc, d.z, t3 * 2.0f * F * st.vz);
          push_force(out, k, gx, gy, gz);
          px += gx;
          py += gy;
          pz += gz;
        }
      }
    }
    fix += float_to_fixed(px);
    fiy += float_to_fixed(py);
    fiz += float_to_fixed(pz);
  }
  for (int off = 16; off > 0; off >>= 1) {
    fix += __shfl_xor_sync(0xffffffffu, fix, off);
    fiy += __shfl_xor_sync(0xffffffffu, fiy, off);
    fiz += __shfl_xor_sync(0xffffffffu, fiz, off);
  }
  if (lane == 0) {
    atomicAdd(&out.force[i], (unsigned long long)fix);
    atomicAdd(&out.force[i + out.stride], (unsigned long long)fiy);
    atomicAdd(&out.force[i + 2 * out.stride], (unsigned long long)fiz);
  }
}

Entries entries_of(const Context* ctx) {
  if (ctx->use_tight)
    return Entries{ctx->d_tgeom,     ctx->d_tcell,   ctx->d_tentry,
                   nullptr,          ctx->d_tindex,  ctx->tcell_cap,
                   ctx->d_tfirst,    ctx->tentry_cap, ctx->cfg.periodic ? ctx->d_wgeom : nullptr};
  return Entries{ctx->d_geom,    ctx->d_cell2,    ctx->d_entry4, ctx->d_entry_par, ctx->d_entries, ctx->cell_cap,
                 nullptr,        ctx->entry_cap};
}

int volume_blocks(const Context* ctx) {
  const long long warps = (long long)ctx->n * ctx->n_chunks;
  return (int)((warps * kWarp + kThreads - 1) / kThreads);
}

template <int MODEL, class Q>
void launch_integrals_t(Context* ctx, const float4* pos, const ModelConst& m, bool count_work) {
  if (MODEL != GBX_MODEL_GBSW && !count_work && ctx->gbmv_cells) {
    launch_gbmv_cells_integral(ctx, pos, m);
    return;
  }
  const Entries t = entries_of(ctx);
  const Quad qd{ctx->d_qv, ctx->d_qw, ctx->d_qoff};
  const int chunk = (m.nq + ctx->n_chunks - 1) / ctx->n_chunks;
  const ShellSink sink{ctx->d_srec, ctx->d_srec_st, ctx->d_rcount, ctx->d_rmax, ctx->srec_R};
  if (MODEL == GBX_MODEL_GBSW && !count_work) {
    // persistent grid: the resident blocks of every SM (or fewer, for few items)
    if (ctx->integral_grid == 0) {
      int per_sm = 0;
      if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, gbsw_integral_kernel<Q, true>, kThreads, 0) !=
              cudaSuccess ||
          per_sm < 1)
        per_sm = 1;
      ctx->integral_grid = per_sm * ctx->sms;
    }
    const int grid = std::min(volume_blocks(ctx), ctx->integral_grid);
    cudaMemsetAsync(ctx->d_next_item, 0, sizeof(unsigned), ctx->stream);
    if (ctx->records)
      gbsw_integral_kernel<Q, true><<<grid, kThreads, 0, ctx->stream>>>(pos, ctx->n, t, qd, m, chunk, ctx->n_chunks,
                                                                         ctx->d_J, sink, ctx->d_next_item);
    else
      gbsw_integral_kernel<Q, false><<<grid, kThreads, 0, ctx->stream>>>(pos, ctx->n, t, qd, m, chunk, ctx->n_chunks,
                                                                          ctx->d_J, sink, ctx->d_next_item);
  }
  else if (count_work)
    integral_kernel<MODEL, Q, true><<<volume_blocks(ctx), kThreads, 0, ctx->stream>>>(
        pos, ctx->n, t, qd, m, chunk, ctx->n_chunks, ctx->d_J, ctx->d_work, ctx->d_pstate);
  else if constexpr (MODEL != GBX_MODEL_GBSW)
    gbmv_integral_kernel<MODEL, Q><<<volume_blocks(ctx), kThreads, 0, ctx->stream>>>(
        pos, ctx->n, t, qd, m, chunk, ctx->n_chunks, ctx->d_J, ctx->d_pstate);
  else
    integral_kernel<MODEL, Q, false><<<volume_blocks(ctx), kThreads, 0, ctx->stream>>>(
        pos, ctx->n, t, qd, m, chunk, ctx->n_chunks, ctx->d_J, nullptr, ctx->d_pstate);
  ++ctx->launches;
}

template <int MODEL, class Q, bool ADJ>
void launch_chain_t(Context* ctx, const float4* pos, const ModelConst& m, unsigned long long* force, int stride) {
  if (MODEL != GBX_MODEL_GBSW && ctx->gbmv_cells) {
    launch_gbmv_cells_chain(ctx, pos, m, force, stride, ADJ);
    return;
  }
  const Entries t = entries_of(ctx);
  const Quad qd{ctx->d_qv, ctx->d_qw, ctx->d_qoff};
  const int chunk = (m.nq + ctx->n_chunks - 1) / ctx->n_chunks;
  ChainOut o{force, stride, ctx->d_dEdR_fx, m.cutoff_chain_quirk && m.cutoff2 > 0.0f, m.cutoff2};
  const bool records = MODEL == GBX_MODEL_GBSW && !ADJ && ctx->records;
  const ChainRecords rr{records ? ctx->d_srec : nullptr, records ? ctx->d_srec_st : nullptr,
                        records ? ctx->d_rcount : nullptr, ctx->srec_R,
                        MODEL == GBX_MODEL_GBSW ? nullptr : ctx->d_pstate};
  bool coop = false;
  if constexpr (MODEL != GBX_MODEL_GBSW) {
    coop = ctx->d_pstate != nullptr;
    if (coop)
      gbmv_chain_kernel<MODEL, Q, ADJ><<<volume_blocks(ctx), kThreads, 0, ctx->stream>>>(
          pos, ctx->n, t, qd, m, chunk, ctx->n_chunks, ctx->d_dEdJ, o, ctx->d_pstate);
  }
  if (!coop)
    chain_kernel<MODEL, Q, ADJ><<<volume_blocks(ctx), kThreads, 0, ctx->stream>>>(pos, ctx->n, t, qd, m, chunk,
                                                                                  ctx->n_chunks, ctx->d_dEdJ, o, rr);
  ++ctx->launches;
}

gbx_status launch_status(Context* ctx, const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    ctx->last_error = std::string(what) + ": " + cudaGetErrorString(e);
    return GBX_ERR_CUDA;
  }
  return GBX_OK;
}

}  // namespace

gbx_status launch_binning(Context* ctx, const float4* pos, bool count_work) {
  ctx->gbmv_cells = ctx->cfg.model != GBX_MODEL_GBSW && !count_work && gbmv_cells_apply(ctx);
  if (!ctx->gbmv_cells) return GBX_OK;
  launch_gbmv_cells_bin(ctx, pos, make_model_const(ctx));
  return launch_status(ctx, "point binning launch");
}

gbx_status launch_integrals(Context* ctx, const float4* pos, bool count_work) {
  const ModelConst m = make_model_const(ctx);
  if (ctx->use_tight && ctx->cfg.periodic) {
    launch_integrals_t<GBX_MODEL_GBSW, PeriodicTightQuery>(ctx, pos, m, count_work);
  } else if (ctx->use_tight) {
    launch_integrals_t<GBX_MODEL_GBSW, TightQuery>(ctx, pos, m, count_work);
  } else if (ctx->cfg.periodic && ctx->cfg.table_mode == GBX_TABLE_STANDALONE) {
    launch_integrals_t<GBX_MODEL_GBSW, PeriodicQuery>(ctx, pos, m, count_work);
  } else if (ctx->cfg.periodic) {
    switch (ctx->cfg.model) {
      case GBX_MODEL_GBSW: launch_integrals_t<GBX_MODEL_GBSW, MinImageQuery>(ctx, pos, m, count_work); break;
      case GBX_MODEL_GBMV1: launch_integrals_t<GBX_MODEL_GBMV1, MinImageQuery>(ctx, pos, m, count_work); break;
      default: launch_integrals_t<GBX_MODEL_GBMV2, MinImageQuery>(ctx, pos, m, count_work); break;
    }
  } else {
    switch (ctx->cfg.model) {
      case GBX_MODEL_GBSW: launch_integrals_t<GBX_MODEL_GBSW, RefQuery>(ctx, pos, m, count_work); break;
      case GBX_MODEL_GBMV1: launch_integrals_t<GBX_MODEL_GBMV1, RefQuery>(ctx, pos, m, count_work); break;
      default: launch_integrals_t<GBX_MODEL_GBMV2, RefQuery>(ctx, pos, m, count_work); break;
    }
  }
  return launch_status(ctx, "integral launch");
}

gbx_status launch_chain(Context* ctx, const float4* pos, unsigned long long* force, int stride, bool adjoint) {
  const ModelConst m = make_model_const(ctx);
  if (ctx->use_tight && ctx->cfg.periodic) {
    if (adjoint) launch_chain_t<GBX_MODEL_GBSW, PeriodicTightQuery, true>(ctx, pos, m, force, stride);
    else launch_chain_t<GBX_MODEL_GBSW, PeriodicTightQuery, false>(ctx, pos, m, force, stride);
  } else if (ctx->use_tight) {
    if (adjoint) launch_chain_t<GBX_MODEL_GBSW, TightQuery, true>(ctx, pos, m, force, stride);
    else launch_chain_t<GBX_MODEL_GBSW, TightQuery, false>(ctx, pos, m, force, stride);
  } else if (ctx->cfg.periodic && ctx->cfg.table_mode == GBX_TABLE_STANDALONE) {
    if (adjoint) launch_chain_t<GBX_MODEL_GBSW, PeriodicQuery, true>(ctx, pos, m, force, stride);
    else launch_chain_t<GBX_MODEL_GBSW, PeriodicQuery, false>(ctx, pos, m, force, stride);
  } else if (ctx->cfg.periodic) {
    switch (ctx->cfg.model * 2 + (adjoint ? 1 : 0)) {
      case 0: launch_chain_t<GBX_MODEL_GBSW, MinImageQuery, false>(ctx, pos, m, force, stride); break;
      case 1: launch_chain_t<GBX_MODEL_GBSW, MinImageQuery, true>(ctx, pos, m, force, stride); break;
      case 2: launch_chain_t<GBX_MODEL_GBMV1, MinImageQuery, false>(ctx, pos, m, force, stride); break;
      case 3: launch_chain_t<GBX_MODEL_GBMV1, MinImageQuery, true>(ctx, pos, m, force, stride); break;
      case 4: launch_chain_t<GBX_MODEL_GBMV2, MinImageQuery, false>(ctx, pos, m, force, stride); break;
      default: launch_chain_t<GBX_MODEL_GBMV2, MinImageQuery, true>(ctx, pos, m, force, stride); break;
    }
  } else {
    switch (ctx->cfg.model * 2 + (adjoint ? 1 : 0)) {
      case 0: launch_chain_t<GBX_MODEL_GBSW, RefQuery, false>(ctx, pos, m, force, stride); break;
      case 1: launch_chain_t<GBX_MODEL_GBSW, RefQuery, true>(ctx, pos, m, force, stride); break;
      case 2: launch_chain_t<GBX_MODEL_GBMV1, RefQuery, false>(ctx, pos, m, force, stride); break;
      case 3: launch_chain_t<GBX_MODEL_GBMV1, RefQuery, true>(ctx, pos, m, force, stride); break;
      case 4: launch_chain_t<GBX_MODEL_GBMV2, RefQuery, false>(ctx, pos, m, force, stride); break;
      default: launch_chain_t<GBX_MODEL_GBMV2, RefQuery, true>(ctx, pos, m, force, stride); break;
    }
  }
  return launch_status(ctx, "chain launch");
}

}  // namespace gbx
