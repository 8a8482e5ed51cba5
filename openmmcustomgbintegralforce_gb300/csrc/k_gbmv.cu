// GBMV-I / GBMV-II integrals and chain rule, processed cell by cell.
//
// Every quadrature point of the GBMV models reads the whole (capped) list of
// the lookup-table cell it falls in (GBMVIntegralTypeI.cpp:111-173,
// GBMVIntegralTypeII.cpp:116-191), and a cell is shared by a few hundred
// points of many atoms.  Instead of each point gathering its list through
// L1, the points are binned by cell and one warp takes one cell: it stages
// the cell's list in shared memory once, and then every lane evaluates its
// own point against entries that all lanes read at the same address (a
// shared-memory broadcast).
//
//   bin      warp per (atom, quadrature chunk), lanes over points: the
//            point's cell (the reference query, exact near cell faces),
//            a slot in the cell by one atomic per point, four points per
//            lane in flight; points whose cell has no list get their
//            solvent fraction here
//   scan     points per cell -> each cell's first slot
//   fill     point ids into their cell's slots
//   integral warp per cell: sorts the cell's point ids (the slots were
//            handed out by atomics, in no fixed order) so that every later
//            sum over the cell's points has an order fixed by the input
//            (cells of more than kSortMax points keep the atomic order and
//            the chain rule reduces each of their contributions on its own);
//            per point the list sums in list order, the solvent fraction by
//            point id, and the point's sums by slot for the chain rule
//   reduce   warp per (atom, chunk): J4, J7 over the solvent fractions in
//            quadrature order (the integral pass's partition, so the Born
//            radii are assembled as before)
//   chain    warp per cell, lanes as 4 points x 8 lanes of entry pairs
//            (packed FP32x2, two entries per instruction; the integral pass
//            likewise evaluates two entries per instruction): each lane
//            keeps the pull of its entries in registers over all of the
//            cell's points (one fixed-point reduction per cell and entry
//            instead of one per point and entry); the point's own pull is
//            summed across its 8 lanes and then over consecutive points of
//            the same atom (the sorted order keeps them together) before one
//            reduction per run
//
// Distances are formed in the cell's frame: entries as x_j - c0 and the
// point as (x_i - c0) + v_q, c0 the cell's corner, so every operand of the
// FP32 difference is within a few tenths of a nanometre of the cell.
#include <math.h>

#include "gbx_internal.cuh"
#include "queries.cuh"
#include "scan.cuh"

namespace gbx {
namespace {

constexpr int kBinThreads = 128;
constexpr int kCellWarps = 4;           // warps (cells) per block in the cell passes
constexpr int kCellThreads = kCellWarps * kWarp;
constexpr int kMaxList = 64;            // longest list the cell passes stage (the GBMV table cap)
constexpr int kSortMax = 16 * kWarp;    // cells of up to 512 points are sorted in registers
constexpr int kChainPts = 4;            // points per chain sub-step
constexpr int kChainEnt = kWarp / kChainPts;  // entry lanes per point
constexpr int kEntPerLane = kMaxList / kChainEnt;
static_assert(kChainPts * kChainEnt == kWarp, "chain lane split");

struct CellPoints {
  int* count;   // [cells] points binned into the cell
  int* start;   // [cells + 1] first slot
  int* order;   // [points] point id per slot, sorted within each cell by the integral pass
  int* cell;    // [points] the point's cell or -1
  int* rank;    // [points] the point's slot within its cell (atomic order)
  float* sval;  // [points] solvent fraction by point id
  float* state; // [planes][points] the point's sums by slot (GBMV-I: S; GBMV-II: s1, s2, vx, vy, vz)
  size_t plane;
};

// Point sums of a list for one point (lists in ascending atom order).
struct Sums {
  float s1, s2, vx, vy, vz;
};

// Minimum image for a box-sampled table of a periodic system (CutoffPeriodic:
// GBMVIntegralTypeI.cpp:59-62, TypeII.cpp:64-67); nothing otherwise.
template <bool PER>
struct Image {
  float L[3], iL[3];
  __device__ __forceinline__ void init(const TableGeom& g) {
    if (PER)
      for (int k = 0; k < 3; ++k) {
        L[k] = (float)g.box[k];
        iL[k] = (float)g.inv_box[k];
      }
  }
  __device__ __forceinline__ void apply2(float2& dx, float2& dy, float2& dz) const {
    if (PER) {
      dx = make_float2(fmaf(-L[0], floorf(fmaf(dx.x, iL[0], 0.5f)), dx.x), fmaf(-L[0], floorf(fmaf(dx.y, iL[0], 0.5f)), dx.y));
      dy = make_float2(fmaf(-L[1], floorf(fmaf(dy.x, iL[1], 0.5f)), dy.x), fmaf(-L[1], floorf(fmaf(dy.y, iL[1], 0.5f)), dy.y));
      dz = make_float2(fmaf(-L[2], floorf(fmaf(dz.x, iL[2], 0.5f)), dz.x), fmaf(-L[2], floorf(fmaf(dz.y, iL[2], 0.5f)), dz.y));
    }
  }
  __device__ __forceinline__ float3 apply(float3 d) const {
    if (PER) {
      d.x = fmaf(-L[0], floorf(fmaf(d.x, iL[0], 0.5f)), d.x);
      d.y = fmaf(-L[1], floorf(fmaf(d.y, iL[1], 0.5f)), d.y);
      d.z = fmaf(-L[2], floorf(fmaf(d.z, iL[2], 0.5f)), d.z);
    }
    return d;
  }
};

__device__ __forceinline__ float3 cell_corner(const TableGeom& g, int cell) {
  const int d12 = g.dims[1] * g.dims[2];
  const int ix = cell / d12, r = cell - ix * d12;
  const int iy = r / g.dims[2], iz = r - iy * g.dims[2];
  return make_float3((float)(g.min[0] + ix * g.step[0]), (float)(g.min[1] + iy * g.step[1]),
                     (float)(g.min[2] + iz * g.step[2]));
}

// The solvent fraction of a point whose cell has no list: GBMV-I S = 0;
// GBMV-II an empty list gives V = 0 (GBMVIntegralTypeII.cpp:140).
template <int MODEL>
__device__ __forceinline__ float empty_list_fraction(const ModelConst& m) {
  if (MODEL == GBX_MODEL_GBMV2) return 1.0f;
  float p;
  return logistic_solvent(m.beta, m.lambda, 0.0f, p);
}

// One binned point: its slot in its cell, or (no list) its solvent fraction.
template <int MODEL>
__device__ __forceinline__ void bin_point(const CellPoints& cp, const Entries& tab, const ModelConst& m, size_t p,
                                          long long cell) {
  const int cnt = cell >= 0 ? __ldg(&tab.cell[cell].x) : 0;
  if (cnt > 0) {
    cp.cell[p] = (int)cell;
    cp.rank[p] = atomicAdd(&cp.count[cell], 1);
  } else {
    cp.cell[p] = -1;
    cp.sval[p] = empty_list_fraction<MODEL>(m);
  }
}

template <int MODEL, class Q>
__global__ void __launch_bounds__(kBinThreads) gbmv_bin_kernel(const float4* __restrict__ pos, int n, Entries tab,
                                                               Quad quad, ModelConst m, int chunk, int n_chunks,
                                                               CellPoints cp) {
  // kBinBatch points per lane per step: their cell queries, list-count loads
  // and slot atomics are issued back to back.  A point within the FP32
  // query's guard band (about one in 500) needs the FP64 query; those are
  // queued per warp and resolved kBinDefer at a time with every lane busy,
  // instead of stalling the warp for each one (FP64 runs at a small fraction
  // of the FP32 rate on this part, whatever the number of active lanes).
  constexpr int kBinBatch = 4;
  constexpr int kBinDefer = 256;
  static_assert(kBinDefer >= 2 * kBinBatch * kWarp, "deferred queue");
  __shared__ int s_defer[kBinThreads / kWarp][kBinDefer];
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) / kWarp;
  const int lane = threadIdx.x % kWarp;
  const int wib = threadIdx.x / kWarp;
  if (warp >= n * n_chunks) return;
  const int i = warp % n, c = warp / n;
  const float4 xi = pos[i];
  Q query;
  query.init(tab, xi, quad.qoff);
  const int q0 = c * chunk, q1 = min(m.nq, q0 + chunk);
  const unsigned lt = (1u << lane) - 1u;
  int* defer = s_defer[wib];
  int ndef = 0;  // warp-uniform
  auto flush = [&]() {
    __syncwarp();
    for (int k = lane; k < ndef; k += kWarp) {
      const int q = defer[k];
      bin_point<MODEL>(cp, tab, m, (size_t)i * m.nq + q, query.cell(xi, quad.qv[q], q));
    }
    __syncwarp();
    ndef = 0;
  };
  for (int base = q0; base < q1; base += kBinBatch * kWarp) {
    long long cell[kBinBatch];
    int cnt[kBinBatch];
    bool late[kBinBatch];
#pragma unroll
    for (int u = 0; u < kBinBatch; ++u) {
      const int q = base + u * kWarp + lane;
      cell[u] = -1;
      cnt[u] = 0;
      late[u] = false;
      if (q < q1) cell[u] = query.cell_fast(quad.qv[q], late[u]);
      const unsigned dm = __ballot_sync(0xffffffffu, late[u]);
      if (late[u]) defer[ndef + __popc(dm & lt)] = q;
      ndef += __popc(dm);
    }
#pragma unroll
    for (int u = 0; u < kBinBatch; ++u)
      if (cell[u] >= 0) cnt[u] = __ldg(&tab.cell[cell[u]].x);
    // one slot atomic per listed point (the warp's points mostly fall in
    // distinct cells: aggregating them by __match_any_sync measured slower)
    int slot[kBinBatch];
#pragma unroll
    for (int u = 0; u < kBinBatch; ++u) {
      slot[u] = 0;
      if (cell[u] >= 0 && cnt[u] > 0) slot[u] = atomicAdd(&cp.count[cell[u]], 1);
    }
#pragma unroll
    for (int u = 0; u < kBinBatch; ++u) {
      const int q = base + u * kWarp + lane;
      const size_t p = (size_t)i * m.nq + q;
      if (cell[u] >= 0 && cnt[u] > 0) {
        cp.cell[p] = (int)cell[u];
        cp.rank[p] = slot[u];
      } else if (q < q1 && !late[u]) {
        cp.cell[p] = -1;
        cp.sval[p] = empty_list_fraction<MODEL>(m);
      }
    }
    if (ndef > kBinDefer - kBinBatch * kWarp) flush();
  }
  if (ndef > 0) flush();
}

__global__ void gbmv_fill_kernel(long long npts, CellPoints cp) {
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= npts) return;
  const int c = cp.cell[p];
  if (c >= 0) cp.order[cp.start[c] + cp.rank[p]] = (int)p;
}

// The table's cell count for the point scan (which writes its total into
// its own geometry record, not the table's).
__global__ void copy_ncell_kernel(const TableGeom* __restrict__ table, TableGeom* __restrict__ pg, long long cap) {
  pg->ncell = table->ncell <= cap ? table->ncell : 0;
  pg->total = 0;
}

// Bitonic sort of 32 E keys held E per lane, element lane E + r in key[r].
template <int E>
__device__ __forceinline__ void warp_bitonic_sort(int (&key)[E], int lane) {
#pragma unroll
  for (int k = 2; k <= kWarp * E; k <<= 1) {
#pragma unroll
    for (int j = k >> 1; j > 0; j >>= 1) {
      if (j < E) {
#pragma unroll
        for (int r = 0; r < E; ++r) {
          const int rp = r ^ j;
          if (rp > r) {
            const bool up = ((lane * E + r) & k) == 0;
            const int a = key[r], b = key[rp];
            key[r] = up ? min(a, b) : max(a, b);
            key[rp] = up ? max(a, b) : min(a, b);
          }
        }
      } else {
        const int lj = j / E;
        const bool lower = (lane & lj) == 0;
#pragma unroll
        for (int r = 0; r < E; ++r) {
          const bool up = ((lane * E + r) & k) == 0;
          const int o = __shfl_xor_sync(0xffffffffu, key[r], lj);
          key[r] = (up == lower) ? min(key[r], o) : max(key[r], o);
        }
      }
    }
  }
}

template <int E>
__device__ __forceinline__ void sort_slots(int* __restrict__ order, int P, int lane) {
  int key[E];
#pragma unroll
  for (int r = 0; r < E; ++r) {
    const int e = lane * E + r;
    key[r] = e < P ? order[e] : 0x7fffffff;
  }
  warp_bitonic_sort<E>(key, lane);
#pragma unroll
  for (int r = 0; r < E; ++r) {
    const int e = lane * E + r;
    if (e < P) order[e] = key[r];
  }
}

// Sorts the cell's point ids in place (cells of more than kSortMax points
// keep the atomic order; the chain rule then takes an order-free path).
__device__ __noinline__ void sort_cell(int* order, int P, int lane) {
  if (P <= kWarp) sort_slots<1>(order, P, lane);
  else if (P <= 2 * kWarp) sort_slots<2>(order, P, lane);
  else if (P <= 4 * kWarp) sort_slots<4>(order, P, lane);
  else if (P <= 8 * kWarp) sort_slots<8>(order, P, lane);
  else if (P <= kSortMax) sort_slots<16>(order, P, lane);
}

// Hardware reciprocal (PTX rcp.approx, relative error below 2^-22; the
// denominators here are >= 1 in magnitude, never subnormal).
__device__ __forceinline__ float rcp_ftz(float x) {
  float y;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float2 bc2(float v) { return make_float2(v, v); }
__device__ __forceinline__ float2 rcp2(float2 t) { return make_float2(rcp_ftz(t.x), rcp_ftz(t.y)); }

// The cell's list staged in shared memory, one array per field, so that four
// consecutive entries load as one float4 (two pairs) and each pair feeds
// packed FP32x2 arithmetic (__ffma2_rn and friends: one instruction for two
// entries, each half rounded as its scalar form).  A list whose length is
// not a multiple of four is padded with entries whose every contribution is
// exactly zero (C = 0 for GBMV-II, gamma = 0 for GBMV-I's chain;
// T = 100 r^2 + 1 >= 1), index -1.
struct __align__(16) CellList {
  float x[kMaxList], y[kMaxList], z[kMaxList];  // x_j - c0
  float w[kMaxList];    // GBMV-II C_j | GBMV-I gamma_j
  float k[kMaxList];    // GBMV-II C_j - 100 R_j^2 | GBMV-I R_j
  float r[kMaxList];    // GBMV-II R_j
  int idx[kMaxList];    // atom index
};

__device__ __forceinline__ float2 ld2(const float* p) { return *reinterpret_cast<const float2*>(p); }
__device__ __forceinline__ float4 ld4(const float* p) { return *reinterpret_cast<const float4*>(p); }
__device__ __forceinline__ float2 lo2(float4 v) { return make_float2(v.x, v.y); }
__device__ __forceinline__ float2 hi2(float4 v) { return make_float2(v.z, v.w); }

template <bool PER>
__device__ __forceinline__ void stage_list(CellList& L, const Entries& tab, int2 cs, int cnt, float3 c0, int lane) {
  const int cnt4 = (cnt + 3) & ~3;
  for (int l = lane; l < cnt4; l += kWarp) {
    if (l < cnt) {
      const float4 a = __ldg(tab.e + cs.y + l);
      const float2 pk = __ldg(tab.par + cs.y + l);
      L.x[l] = a.x - c0.x;
      L.y[l] = a.y - c0.y;
      L.z[l] = a.z - c0.z;
      L.w[l] = a.w;
      L.k[l] = pk.x;
      L.r[l] = pk.y;
      L.idx[l] = __ldg(tab.index + cs.y + l);
    } else {
      L.x[l] = L.y[l] = L.z[l] = 0.0f;
      L.w[l] = 0.0f;
      L.k[l] = 1.0f;
      L.r[l] = 1.0f;
      L.idx[l] = -1;
    }
  }
}

template <int MODEL, bool PER>
__global__ void __launch_bounds__(kCellThreads) gbmv_cell_integral_kernel(const float4* __restrict__ pos, Entries tab,
                                                                          Quad quad, ModelConst m, CellPoints cp) {
  __shared__ CellList s_list[kCellWarps];
  const int w = threadIdx.x / kWarp, lane = threadIdx.x % kWarp;
  const long long cell = (long long)blockIdx.x * kCellWarps + w;
  const TableGeom& G = *tab.geom;
  if (cell >= G.ncell || cell >= tab.cell_cap) return;
  const int P = cp.count[cell];
  if (P == 0) return;
  const int2 cs = __ldg(tab.cell + cell);
  const int cnt = min(cs.x, kMaxList);
  const float3 c0 = cell_corner(G, (int)cell);
  Image<PER> img;
  img.init(G);
  CellList& L = s_list[w];
  stage_list<PER>(L, tab, cs, cnt, c0, lane);
  const int start = cp.start[cell];
  int* order = cp.order + start;
  if (P > 1) sort_cell(order, P, lane);
  __syncwarp();
  // GBMV-II's padding entries add exactly zero; GBMV-I's (e^0 = 1) do not,
  // so its last (cnt mod 4) entries are taken one at a time
  const int nquad = MODEL == GBX_MODEL_GBMV2 ? (cnt + 3) >> 2 : cnt >> 2;
  for (int base = 0; base < P; base += kWarp) {
    const int k = base + lane;
    const bool valid = k < P;
    const int p = valid ? order[k] : 0;
    const int i = p / m.nq, q = p - i * m.nq;
    const float4 xi = __ldg(pos + i), v = __ldg(quad.qv + q);
    const float px = (xi.x - c0.x) + v.x, py = (xi.y - c0.y) + v.y, pz = (xi.z - c0.z) + v.z;
    const float2 npx = bc2(-px), npy = bc2(-py), npz = bc2(-pz);
    float2 s1 = bc2(0.f), s2 = bc2(0.f), vx = bc2(0.f), vy = bc2(0.f), vz = bc2(0.f);
    auto pair = [&](float2 ex, float2 ey, float2 ez, float2 ew, float2 ek) {
      float2 dx = __fadd2_rn(ex, npx), dy = __fadd2_rn(ey, npy), dz = __fadd2_rn(ez, npz);
      img.apply2(dx, dy, dz);
      const float2 r2 = __ffma2_rn(dx, dx, __ffma2_rn(dy, dy, __fmul2_rn(dz, dz)));
      if (MODEL == GBX_MODEL_GBMV1) {
        const float2 g = __fmul2_rn(ew, __fmul2_rn(r2, r2));
        s1 = __fadd2_rn(s1, make_float2(__expf(g.x), __expf(g.y)));
      } else {
        const float2 T = __ffma2_rn(bc2(100.0f), r2, ek);
        float2 F = __fmul2_rn(ew, rcp2(T));
        F = __fmul2_rn(F, F);
        s1 = __fadd2_rn(s1, F);
        s2 = __ffma2_rn(r2, __fmul2_rn(F, F), s2);
        vx = __ffma2_rn(dx, F, vx);
        vy = __ffma2_rn(dy, F, vy);
        vz = __ffma2_rn(dz, F, vz);
      }
    };
    for (int j = 0; j < nquad; ++j) {
      const int l = 4 * j;
      const float4 X = ld4(L.x + l), Y = ld4(L.y + l), Z = ld4(L.z + l), W = ld4(L.w + l);
      const float4 K4 = MODEL == GBX_MODEL_GBMV2 ? ld4(L.k + l) : make_float4(0.f, 0.f, 0.f, 0.f);
      pair(lo2(X), lo2(Y), lo2(Z), lo2(W), lo2(K4));
      pair(hi2(X), hi2(Y), hi2(Z), hi2(W), hi2(K4));
    }
    Sums s{s1.x + s1.y, s2.x + s2.y, vx.x + vx.y, vy.x + vy.y, vz.x + vz.y};
    if (MODEL == GBX_MODEL_GBMV1) {
      for (int l = 4 * nquad; l < cnt; ++l) {
        const float3 d = img.apply(make_float3(L.x[l] - px, L.y[l] - py, L.z[l] - pz));
        const float r2 = fmaf(d.x, d.x, fmaf(d.y, d.y, d.z * d.z));
        s.s1 += __expf(L.w[l] * (r2 * r2));
      }
    }
    if (valid) {
      float pl, S;
      if (MODEL == GBX_MODEL_GBMV1) {
        S = s.s1;
      } else {
        const float s3sq = fmaf(s.vx, s.vx, fmaf(s.vy, s.vy, s.vz * s.vz));
        S = m.s0 * s.s1 * s.s2 / s3sq;
      }
      cp.sval[p] = logistic_solvent(m.beta, m.lambda, S, pl);
      float* st = cp.state + start + k;
      st[0] = s.s1;
      if (MODEL == GBX_MODEL_GBMV2) {
        st[cp.plane] = s.s2;
        st[2 * cp.plane] = s.vx;
        st[3 * cp.plane] = s.vy;
        st[4 * cp.plane] = s.vz;
      }
    }
  }
}

// J4, J7 per (atom, chunk) over the solvent fractions, in quadrature order.
__global__ void __launch_bounds__(kBinThreads) gbmv_reduce_kernel(int n, Quad quad, int nq, int chunk, int n_chunks,
                                                                  const float* __restrict__ sval,
                                                                  float* __restrict__ Jpart) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) / kWarp;
  const int lane = threadIdx.x % kWarp;
  if (warp >= n * n_chunks) return;
  const int i = warp % n, c = warp / n;
  const int q0 = c * chunk, q1 = min(nq, q0 + chunk);
  const float* s = sval + (size_t)i * nq;
  float J4 = 0.0f, J7 = 0.0f;
  for (int q = q0 + lane; q < q1; q += kWarp) {
    const float sf = s[q];
    const float2 w = __ldg(quad.qw + q);
    J4 = fmaf(w.x, sf, J4);
    J7 = fmaf(w.y, sf, J7);
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

struct CellChainOut {
  unsigned long long* force;
  int stride;
  unsigned long long* dEdR;
};

__device__ __forceinline__ void add_fixed3(const CellChainOut& o, int k, float gx, float gy, float gz) {
  const long long fx = float_to_fixed(gx), fy = float_to_fixed(gy), fz = float_to_fixed(gz);
  if (fx) atomicAdd(&o.force[k], (unsigned long long)fx);
  if (fy) atomicAdd(&o.force[k + o.stride], (unsigned long long)fy);
  if (fz) atomicAdd(&o.force[k + 2 * o.stride], (unsigned long long)fz);
}

// One fixed-point reduction (skipped when the value rounds to zero).
__device__ __forceinline__ void add_fixed_one(unsigned long long* a, int k, float v) {
  const long long r = float_to_fixed(v);
  if (r) atomicAdd(&a[k], (unsigned long long)r);
}

// One point's chain-rule factors (the point's own lanes read them from
// shared memory): its position in the cell frame and the factors of the
// gradient with c ds/dS folded in.  GBMV-II: with u_j = F_j / T_j and
// vd = v . d_j, the pull on entry j is
//   g_j = [-400 u_j (A + C vd) + B F_j (F_j - 400 u_j r_j^2)] d_j + F_j C v
// with A = c ds/dS s0 s2 / |v|^2, B = 2 c ds/dS s0 s1 / |v|^2,
// C = -2 c ds/dS s0 s1 s2 / |v|^4 (the d s1, d s2 and d |v|^2 factors).
// GBMV-I: g_j = A e_j r_j^2 d_j with A = 4 c ds/dS gamma_j
// folded per entry.
struct __align__(16) PointChain {
  float2 npx, npy, npz;  // minus the point's position in the cell frame, in both halves
  float2 A, B, C;        // GBMV-I: A only
  float2 vx, vy, vz;
  float cS;
  int i;
};

template <int MODEL, bool PER, bool ADJ>
__global__ void __launch_bounds__(kCellThreads) gbmv_cell_chain_kernel(const float4* __restrict__ pos, Entries tab,
                                                                       Quad quad, ModelConst m, CellPoints cp,
                                                                       const float2* __restrict__ dEdJ,
                                                                       CellChainOut out) {
  __shared__ CellList s_list[kCellWarps];
  __shared__ PointChain s_pt[kCellWarps][kWarp];
  __shared__ float3 s_own[kCellWarps][kWarp];
  const int w = threadIdx.x / kWarp, lane = threadIdx.x % kWarp;
  const long long cell = (long long)blockIdx.x * kCellWarps + w;
  const TableGeom& G = *tab.geom;
  if (cell >= G.ncell || cell >= tab.cell_cap) return;
  const int P = cp.count[cell];
  if (P == 0) return;
  const int2 cs = __ldg(tab.cell + cell);
  const int cnt = min(cs.x, kMaxList);
  const float3 c0 = cell_corner(G, (int)cell);
  Image<PER> img;
  img.init(G);
  CellList& L = s_list[w];
  stage_list<PER>(L, tab, cs, cnt, c0, lane);
  const int start = cp.start[cell];
  const int* order = cp.order + start;
  const float* state = cp.state + start;
  // cells too dense to sort keep the atomic slot order: every contribution
  // is then reduced on its own (integer sums, independent of the order)
  const bool sorted = P <= kSortMax;
  // lane (ps, es): point ps of each group of kChainPts, entry pairs es, es +
  // kChainEnt, ... (entries 2 j and 2 j + 1 of pair j)
  const int ps = lane / kChainEnt, es = lane % kChainEnt;
  constexpr int kPairsPerLane = kEntPerLane / 2;
  float2 acc[kPairsPerLane][3];
  float2 accR[kPairsPerLane];
#pragma unroll
  for (int e = 0; e < kPairsPerLane; ++e) {
    acc[e][0] = acc[e][1] = acc[e][2] = bc2(0.f);
    accR[e] = bc2(0.f);
  }
  PointChain* pts = s_pt[w];
  const float Cp = 10.0f * m.p1;
  for (int base = 0; base < P; base += kWarp) {
    // lane t prepares point base + t
    int np;
    {
      const int k = base + lane;
      PointChain pc;
      pc.cS = 0.0f;
      pc.i = -1;
      pc.npx = pc.npy = pc.npz = pc.A = pc.B = pc.C = bc2(0.f);
      pc.vx = pc.vy = pc.vz = bc2(0.f);
      if (k < P) {
        const int p = order[k];
        const int i = p / m.nq, q = p - i * m.nq;
        const float4 xi = __ldg(pos + i), v = __ldg(quad.qv + q);
        const float2 wq = __ldg(quad.qw + q);
        const float2 de = __ldg(dEdJ + i);
        const float cq = fmaf(de.x, wq.x, de.y * wq.y);
        pc.i = i;
        pc.npx = bc2(-((xi.x - c0.x) + v.x));
        pc.npy = bc2(-((xi.y - c0.y) + v.y));
        pc.npz = bc2(-((xi.z - c0.z) + v.z));
        float pl;
        if (MODEL == GBX_MODEL_GBMV1) {
          logistic_solvent(m.beta, m.lambda, state[k], pl);
          pc.cS = cq * __fdividef(m.beta * pl, (1.0f + pl) * (1.0f + pl));
          pc.A = bc2(4.0f * pc.cS);
        } else {
          const float s1 = state[k], s2 = state[k + cp.plane], vx = state[k + 2 * cp.plane],
                      vy = state[k + 3 * cp.plane], vz = state[k + 4 * cp.plane];
          const float s3sq = fmaf(vx, vx, fmaf(vy, vy, vz * vz));
          logistic_solvent(m.beta, m.lambda, m.s0 * s1 * s2 / s3sq, pl);
          pc.cS = cq * __fdividef(m.beta * pl, (1.0f + pl) * (1.0f + pl)) * m.s0;
          const float inv3 = 1.0f / s3sq;
          const float A = pc.cS * (s2 * inv3), B = 2.0f * pc.cS * (s1 * inv3),
                      C = 2.0f * pc.cS * (-s1 * s2 * inv3 * inv3);
          pc.A = bc2(A);
          pc.B = bc2(B);
          pc.C = bc2(C);
          pc.vx = bc2(vx);
          pc.vy = bc2(vy);
          pc.vz = bc2(vz);
        }
      }
      // only points with a nonzero factor pull on anything (a saturated
      // solvent fraction gives exact zeros): they are packed in order, so
      // the sums see the same nonzero terms in the same order
      const unsigned lm = __ballot_sync(0xffffffffu, pc.cS != 0.0f);
      if (pc.cS != 0.0f) pts[__popc(lm & ((1u << lane) - 1u))] = pc;
      np = __popc(lm);
    }
    __syncwarp();
    for (int sub = 0; sub < np; sub += kChainPts) {
      const int t = sub + ps;
      const PointChain& pc = pts[t < np ? t : 0];
      const bool live = t < np && pc.cS != 0.0f;
      float2 ox = bc2(0.f), oy = bc2(0.f), oz = bc2(0.f);
      if (live) {
        const int pi = pc.i;
        // entries l and l + 1 as one pair, accumulated into acc[e]
        auto pair = [&](int e, int l, float2 ex, float2 ey, float2 ez, float2 aw, float2 ek, float2 er, int2 kj) {
          float2 dx = __fadd2_rn(ex, pc.npx), dy = __fadd2_rn(ey, pc.npy), dz = __fadd2_rn(ez, pc.npz);
          img.apply2(dx, dy, dz);
          const float2 r2 = __ffma2_rn(dx, dx, __ffma2_rn(dy, dy, __fmul2_rn(dz, dz)));
          // atom i's own entry moves with the point: no force from it
          const float2 own = make_float2(kj.x != pi ? 1.0f : 0.0f, kj.y != pi ? 1.0f : 0.0f);
          float2 gx, gy, gz;
          if (MODEL == GBX_MODEL_GBMV1) {
            const float2 r4 = __fmul2_rn(r2, r2);
            const float2 g = __fmul2_rn(aw, r4);
            const float2 ex2 = make_float2(__expf(g.x), __expf(g.y));
            if (ADJ) {
              // dS/dR_j = -4 gamma_j e_j r^4 / R_j (gamma ~ R^-4); padding: gamma = 0
              const float2 dr = __fmul2_rn(__fmul2_rn(__fmul2_rn(bc2(pc.cS), ex2), r4),
                                           make_float2(-4.0f * aw.x / ek.x, -4.0f * aw.y / ek.y));
              accR[e] = __fadd2_rn(accR[e], dr);
              if (!sorted) {
                if (l < cnt) add_fixed_one(out.dEdR, kj.x, dr.x);
                if (l + 1 < cnt) add_fixed_one(out.dEdR, kj.y, dr.y);
              }
            }
            // dS/d(delta) = 4 gamma e r^2 delta
            const float2 gs = __fmul2_rn(__fmul2_rn(__fmul2_rn(__fmul2_rn(pc.A, aw), ex2), r2), own);
            gx = __fmul2_rn(gs, dx);
            gy = __fmul2_rn(gs, dy);
            gz = __fmul2_rn(gs, dz);
          } else {
            const float2 T = __ffma2_rn(bc2(100.0f), r2, ek);
            const float2 rT = rcp2(T);
            const float2 CT = __fmul2_rn(aw, rT);
            const float2 F = __fmul2_rn(CT, CT);
            const float2 u = __fmul2_rn(F, rT);  // dF/d(delta) = -400 u delta
            const float2 vd = __ffma2_rn(pc.vx, dx, __ffma2_rn(pc.vy, dy, __fmul2_rn(pc.vz, dz)));
            if (ADJ) {
              // dF/dR_j with T = C_j + 100 (r^2 - R_j^2), C_j = 10 p1 R_j + p2 (nm -> A):
              // c ds/dS (s2 dF + s1 d(r^2 F^2) + d|v|^2) / |v|^2 as pc.A, pc.B, pc.C carry them
              const float2 Tp = __ffma2_rn(bc2(-200.0f), er, bc2(Cp));
              const float2 num = __ffma2_rn(bc2(Cp), T, __fmul2_rn(make_float2(-aw.x, -aw.y), Tp));
              const float2 dFdR = __fmul2_rn(__fmul2_rn(__fmul2_rn(bc2(2.0f), CT), num), __fmul2_rn(rT, rT));
              const float2 fac = __ffma2_rn(pc.C, vd, __ffma2_rn(pc.B, __fmul2_rn(r2, F), pc.A));
              const float2 dr = __fmul2_rn(dFdR, fac);
              accR[e] = __fadd2_rn(accR[e], dr);
              if (!sorted) {
                if (l < cnt) add_fixed_one(out.dEdR, kj.x, dr.x);
                if (l + 1 < cnt) add_fixed_one(out.dEdR, kj.y, dr.y);
              }
            }
            // g = [-400 u (A + C vd) + B F (F - 400 u r^2)] delta + F C v
            const float2 m400u = __fmul2_rn(bc2(-400.0f), u);
            const float2 sc = __fmul2_rn(
                __ffma2_rn(m400u, __ffma2_rn(pc.C, vd, pc.A), __fmul2_rn(__fmul2_rn(pc.B, F), __ffma2_rn(m400u, r2, F))),
                own);
            const float2 FC = __fmul2_rn(__fmul2_rn(F, own), pc.C);
            gx = __ffma2_rn(sc, dx, __fmul2_rn(FC, pc.vx));
            gy = __ffma2_rn(sc, dy, __fmul2_rn(FC, pc.vy));
            gz = __ffma2_rn(sc, dz, __fmul2_rn(FC, pc.vz));
          }
          if (sorted) {
            acc[e][0] = __fadd2_rn(acc[e][0], gx);
            acc[e][1] = __fadd2_rn(acc[e][1], gy);
            acc[e][2] = __fadd2_rn(acc[e][2], gz);
          } else {
            if (l < cnt && kj.x != pi) add_fixed3(out, kj.x, -gx.x, -gy.x, -gz.x);
            if (l + 1 < cnt && kj.y != pi) add_fixed3(out, kj.y, -gx.y, -gy.y, -gz.y);
          }
          ox = __fadd2_rn(ox, gx);
          oy = __fadd2_rn(oy, gy);
          oz = __fadd2_rn(oz, gz);
        };
#pragma unroll
        for (int e = 0; e < kPairsPerLane; ++e) {
          const int l = 2 * (es + e * kChainEnt);
          if (l < cnt) {
            const float2 R2 = ADJ && MODEL == GBX_MODEL_GBMV2 ? ld2(L.r + l) : bc2(0.f);
            pair(e, l, ld2(L.x + l), ld2(L.y + l), ld2(L.z + l), ld2(L.w + l), ld2(L.k + l), R2,
                 *reinterpret_cast<const int2*>(L.idx + l));
          }
        }
      }
      // the point's own pull, summed over its entry lanes
      float px_ = ox.x + ox.y, py_ = oy.x + oy.y, pz_ = oz.x + oz.y;
#pragma unroll
      for (int off = 1; off < kChainEnt; off <<= 1) {
        px_ += __shfl_xor_sync(0xffffffffu, px_, off);
        py_ += __shfl_xor_sync(0xffffffffu, py_, off);
        pz_ += __shfl_xor_sync(0xffffffffu, pz_, off);
      }
      if (es == 0 && t < np) s_own[w][t] = make_float3(px_, py_, pz_);
    }
    __syncwarp();
    // owner forces of these points: runs of one atom summed, one reduction per run
    {
      float3 o = lane < np ? s_own[w][lane] : make_float3(0.f, 0.f, 0.f);
      const int key = lane < np ? pts[lane].i : -1 - lane;
      if (sorted) {
#pragma unroll
        for (int off = 1; off < kWarp; off <<= 1) {
          const float yx = __shfl_up_sync(0xffffffffu, o.x, off);
          const float yy = __shfl_up_sync(0xffffffffu, o.y, off);
          const float yz = __shfl_up_sync(0xffffffffu, o.z, off);
          const int ky = __shfl_up_sync(0xffffffffu, key, off);
          if (lane >= off && ky == key) {
            o.x += yx;
            o.y += yy;
            o.z += yz;
          }
        }
        const int kn = __shfl_down_sync(0xffffffffu, key, 1);
        if (lane < np && (lane == np - 1 || kn != key)) add_fixed3(out, key, o.x, o.y, o.z);
      } else if (lane < np) {
        add_fixed3(out, key, o.x, o.y, o.z);
      }
    }
    __syncwarp();
  }
  if (!sorted) return;
  // the entries' pull over all of the cell's points: summed over the point
  // lanes, one fixed-point reduction per entry
#pragma unroll
  for (int e = 0; e < kPairsPerLane; ++e) {
#pragma unroll
    for (int off = kChainEnt; off < kWarp; off <<= 1) {
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        acc[e][c].x += __shfl_xor_sync(0xffffffffu, acc[e][c].x, off);
        acc[e][c].y += __shfl_xor_sync(0xffffffffu, acc[e][c].y, off);
      }
      if (ADJ) {
        accR[e].x += __shfl_xor_sync(0xffffffffu, accR[e].x, off);
        accR[e].y += __shfl_xor_sync(0xffffffffu, accR[e].y, off);
      }
    }
    const int l = 2 * (es + e * kChainEnt);
    if (ps == 0) {
      for (int h = 0; h < 2; ++h) {
        if (l + h >= cnt) break;
        const int kj = L.idx[l + h];
        add_fixed3(out, kj, h ? -acc[e][0].y : -acc[e][0].x, h ? -acc[e][1].y : -acc[e][1].x,
                   h ? -acc[e][2].y : -acc[e][2].x);
        if (ADJ) add_fixed_one(out.dEdR, kj, h ? accR[e].y : accR[e].x);
      }
    }
  }
}

}  // namespace

// The cell passes apply to the GBMV models on a table capped at kMaxList.
bool gbmv_cells_apply(const Context* ctx) {
  const gbx_config& c = ctx->cfg;
  return c.model != GBX_MODEL_GBSW && c.table_cap >= 1 && c.table_cap <= kMaxList && ctx->d_pcell != nullptr &&
         ctx->d_pcount != nullptr &&
         (long long)ctx->n * (c.n_radial * c.lebedev_order) < 0x7fffffffLL;
}

namespace {
Entries gbmv_entries(const Context* ctx) {
  return Entries{ctx->d_geom, ctx->d_cell2, ctx->d_entry4, ctx->d_entry_par, ctx->d_entries, ctx->cell_cap, nullptr,
                 ctx->entry_cap};
}
}  // namespace

gbx_status launch_gbmv_cells_bin(Context* ctx, const float4* pos, const ModelConst& m) {
  cudaStream_t st = ctx->stream;
  const Entries t = gbmv_entries(ctx);
  const Quad qd{ctx->d_qv, ctx->d_qw, ctx->d_qoff};
  const int chunk = (m.nq + ctx->n_chunks - 1) / ctx->n_chunks;
  const long long npts = (long long)ctx->n * m.nq;
  const CellPoints cp{ctx->d_pcount, ctx->d_pstart, ctx->d_porder, ctx->d_pcell, ctx->d_prank,
                      ctx->d_sval,   ctx->d_pstate, (size_t)npts};
  const long long warps = (long long)ctx->n * ctx->n_chunks;
  const int bin_blocks = (int)((warps * kWarp + kBinThreads - 1) / kBinThreads);
  const long long cells = ctx->cell_cap;
  cudaMemsetAsync(ctx->d_pcount, 0, sizeof(int) * cells, st);
  const bool per = ctx->cfg.periodic != 0;
  if (m.model == GBX_MODEL_GBMV1) {
    if (per) gbmv_bin_kernel<GBX_MODEL_GBMV1, MinImageQuery><<<bin_blocks, kBinThreads, 0, st>>>(pos, ctx->n, t, qd, m, chunk, ctx->n_chunks, cp);
    else gbmv_bin_kernel<GBX_MODEL_GBMV1, RefQuery><<<bin_blocks, kBinThreads, 0, st>>>(pos, ctx->n, t, qd, m, chunk, ctx->n_chunks, cp);
  } else {
    if (per) gbmv_bin_kernel<GBX_MODEL_GBMV2, MinImageQuery><<<bin_blocks, kBinThreads, 0, st>>>(pos, ctx->n, t, qd, m, chunk, ctx->n_chunks, cp);
    else gbmv_bin_kernel<GBX_MODEL_GBMV2, RefQuery><<<bin_blocks, kBinThreads, 0, st>>>(pos, ctx->n, t, qd, m, chunk, ctx->n_chunks, cp);
  }
  copy_ncell_kernel<<<1, 1, 0, st>>>(ctx->d_geom, ctx->d_pgeom, cells);
  launch_scan<false>(ctx->d_pcount, ctx->d_pgeom, ctx->d_pblock_sums, ctx->d_pstart, nullptr, cells, 0x7fffffffffffLL,
                     ctx->d_status, st);
  gbmv_fill_kernel<<<(int)((npts + 255) / 256), 256, 0, st>>>(npts, cp);
  ctx->launches += 6;  // bin, ncell copy, three scan phases, fill
  return GBX_OK;
}

gbx_status launch_gbmv_cells_integral(Context* ctx, const float4* pos, const ModelConst& m) {
  cudaStream_t st = ctx->stream;
  const Entries t = gbmv_entries(ctx);
  const Quad qd{ctx->d_qv, ctx->d_qw, ctx->d_qoff};
  const int chunk = (m.nq + ctx->n_chunks - 1) / ctx->n_chunks;
  const long long npts = (long long)ctx->n * m.nq;
  const CellPoints cp{ctx->d_pcount, ctx->d_pstart, ctx->d_porder, ctx->d_pcell, ctx->d_prank,
                      ctx->d_sval,   ctx->d_pstate, (size_t)npts};
  const long long warps = (long long)ctx->n * ctx->n_chunks;
  const int bin_blocks = (int)((warps * kWarp + kBinThreads - 1) / kBinThreads);
  const int cell_blocks = (int)((ctx->cell_cap + kCellWarps - 1) / kCellWarps);
  const bool per = ctx->cfg.periodic != 0;
  if (m.model == GBX_MODEL_GBMV1) {
    if (per) gbmv_cell_integral_kernel<GBX_MODEL_GBMV1, true><<<cell_blocks, kCellThreads, 0, st>>>(pos, t, qd, m, cp);
    else gbmv_cell_integral_kernel<GBX_MODEL_GBMV1, false><<<cell_blocks, kCellThreads, 0, st>>>(pos, t, qd, m, cp);
  } else {
    if (per) gbmv_cell_integral_kernel<GBX_MODEL_GBMV2, true><<<cell_blocks, kCellThreads, 0, st>>>(pos, t, qd, m, cp);
    else gbmv_cell_integral_kernel<GBX_MODEL_GBMV2, false><<<cell_blocks, kCellThreads, 0, st>>>(pos, t, qd, m, cp);
  }
  gbmv_reduce_kernel<<<bin_blocks, kBinThreads, 0, st>>>(ctx->n, qd, m.nq, chunk, ctx->n_chunks, ctx->d_sval,
                                                         ctx->d_J);
  ctx->launches += 2;  // integral, reduce
  return GBX_OK;
}

gbx_status launch_gbmv_cells_chain(Context* ctx, const float4* pos, const ModelConst& m, unsigned long long* force,
                                   int stride, bool adjoint) {
  cudaStream_t st = ctx->stream;
  const Entries t = gbmv_entries(ctx);
  const Quad qd{ctx->d_qv, ctx->d_qw, ctx->d_qoff};
  const long long npts = (long long)ctx->n * m.nq;
  const CellPoints cp{ctx->d_pcount, ctx->d_pstart, ctx->d_porder, ctx->d_pcell, ctx->d_prank,
                      ctx->d_sval,   ctx->d_pstate, (size_t)npts};
  const CellChainOut o{force, stride, ctx->d_dEdR_fx};
  const int cell_blocks = (int)((ctx->cell_cap + kCellWarps - 1) / kCellWarps);
  const bool per = ctx->cfg.periodic != 0;
  const int sel = (m.model == GBX_MODEL_GBMV1 ? 0 : 4) + (per ? 2 : 0) + (adjoint ? 1 : 0);
  switch (sel) {
    case 0: gbmv_cell_chain_kernel<GBX_MODEL_GBMV1, false, false><<<cell_blocks, kCellThreads, 0, st>>>(pos, t, qd, m, cp, ctx->d_dEdJ, o); break;
    case 1: gbmv_cell_chain_kernel<GBX_MODEL_GBMV1, false, true><<<cell_blocks, kCellThreads, 0, st>>>(pos, t, qd, m, cp, ctx->d_dEdJ, o); break;
    case 2: gbmv_cell_chain_kernel<GBX_MODEL_GBMV1, true, false><<<cell_blocks, kCellThreads, 0, st>>>(pos, t, qd, m, cp, ctx->d_dEdJ, o); break;
    case 3: gbmv_cell_chain_kernel<GBX_MODEL_GBMV1, true, true><<<cell_blocks, kCellThreads, 0, st>>>(pos, t, qd, m, cp, ctx->d_dEdJ, o); break;
    case 4: gbmv_cell_chain_kernel<GBX_MODEL_GBMV2, false, false><<<cell_blocks, kCellThreads, 0, st>>>(pos, t, qd, m, cp, ctx->d_dEdJ, o); break;
    case 5: gbmv_cell_chain_kernel<GBX_MODEL_GBMV2, false, true><<<cell_blocks, kCellThreads, 0, st>>>(pos, t, qd, m, cp, ctx->d_dEdJ, o); break;
    case 6: gbmv_cell_chain_kernel<GBX_MODEL_GBMV2, true, false><<<cell_blocks, kCellThreads, 0, st>>>(pos, t, qd, m, cp, ctx->d_dEdJ, o); break;
    default: gbmv_cell_chain_kernel<GBX_MODEL_GBMV2, true, true><<<cell_blocks, kCellThreads, 0, st>>>(pos, t, qd, m, cp, ctx->d_dEdJ, o); break;
  }
  ++ctx->launches;
  return GBX_OK;
}

}  // namespace gbx
