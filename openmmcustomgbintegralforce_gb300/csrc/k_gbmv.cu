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
//            a slot in the cell by one atomic per distinct cell per warp;
//            points whose cell has no list get their solvent fraction here
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
//   chain    warp per cell, lanes as 4 points x 8 list entries: each lane
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
        iL[k] = (float)(1.0 / g.box[k]);
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

template <int MODEL, class Q>
__global__ void __launch_bounds__(kBinThreads) gbmv_bin_kernel(const float4* __restrict__ pos, int n, Entries tab,
                                                               Quad quad, ModelConst m, int chunk, int n_chunks,
                                                               CellPoints cp) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) / kWarp;
  const int lane = threadIdx.x % kWarp;
  if (warp >= n * n_chunks) return;
  const int i = warp % n, c = warp / n;
  const float4 xi = pos[i];
  Q query;
  query.init(*tab.geom, xi, quad.qoff, usable_cells(tab));
  const int q0 = c * chunk, q1 = min(m.nq, q0 + chunk);
  const unsigned lt = (1u << lane) - 1u;
  for (int base = q0; base < q1; base += kWarp) {
    const int q = base + lane;
    const bool valid = q < q1;
    long long cell = -1;
    int cnt = 0;
    if (valid) {
      cell = query.cell(xi, quad.qv[q], q);
      if (cell >= 0) cnt = __ldg(&tab.cell[cell].x);
    }
    const bool listed = valid && cell >= 0 && cnt > 0;
    const unsigned lm = __ballot_sync(0xffffffffu, listed);
    const size_t p = (size_t)i * m.nq + q;
    if (listed) {
      // one atomic per distinct cell among the warp's points
      const unsigned peers = __match_any_sync(lm, (int)cell);
      const int leader = __ffs(peers) - 1;
      int r0 = 0;
      if (lane == leader) r0 = atomicAdd(&cp.count[cell], __popc(peers));
      r0 = __shfl_sync(peers, r0, leader);
      cp.cell[p] = (int)cell;
      cp.rank[p] = r0 + __popc(peers & lt);
    } else if (valid) {
      cp.cell[p] = -1;
      cp.sval[p] = empty_list_fraction<MODEL>(m);
    }
  }
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

template <int MODEL, bool PER>
__global__ void __launch_bounds__(kCellThreads) gbmv_cell_integral_kernel(const float4* __restrict__ pos, Entries tab,
                                                                          Quad quad, ModelConst m, CellPoints cp) {
  __shared__ float4 s_e[kCellWarps][kMaxList];
  __shared__ float s_k[kCellWarps][kMaxList];
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
  for (int l = lane; l < cnt; l += kWarp) {
    const float4 a = __ldg(tab.e + cs.y + l);
    s_e[w][l] = make_float4(a.x - c0.x, a.y - c0.y, a.z - c0.z, a.w);
    if (MODEL == GBX_MODEL_GBMV2) s_k[w][l] = __ldg(&tab.par[cs.y + l].x);
  }
  const int start = cp.start[cell];
  int* order = cp.order + start;
  if (P > 1) sort_cell(order, P, lane);
  __syncwarp();
  const float4* E = s_e[w];
  const float* K = s_k[w];
  for (int base = 0; base < P; base += kWarp) {
    const int k = base + lane;
    const bool valid = k < P;
    const int p = valid ? order[k] : 0;
    const int i = p / m.nq, q = p - i * m.nq;
    const float4 xi = __ldg(pos + i), v = __ldg(quad.qv + q);
    const float px = (xi.x - c0.x) + v.x, py = (xi.y - c0.y) + v.y, pz = (xi.z - c0.z) + v.z;
    Sums s{0.f, 0.f, 0.f, 0.f, 0.f};
    for (int l = 0; l < cnt; ++l) {
      const float4 a = E[l];
      const float3 d = img.apply(make_float3(a.x - px, a.y - py, a.z - pz));
      const float r2 = fmaf(d.x, d.x, fmaf(d.y, d.y, d.z * d.z));
      if (MODEL == GBX_MODEL_GBMV1) {
        s.s1 += __expf(a.w * (r2 * r2));
      } else {
        float F = __fdividef(a.w, fmaf(100.0f, r2, K[l]));
        F = F * F;
        s.s1 += F;
        s.s2 = fmaf(r2, F * F, s.s2);
        s.vx = fmaf(d.x, F, s.vx);
        s.vy = fmaf(d.y, F, s.vy);
        s.vz = fmaf(d.z, F, s.vz);
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

// dE/dR_k of one contribution: kept in the entry's register sum, or (cells
// too dense to sort) reduced on its own.
__device__ __forceinline__ void add_dEdR(const CellChainOut& o, int k, bool sorted, float& acc, float v) {
  if (sorted) {
    acc += v;
  } else {
    const long long r = float_to_fixed(v);
    if (r) atomicAdd(&o.dEdR[k], (unsigned long long)r);
  }
}

// One point's chain-rule factors (the point's own lanes read them from
// shared memory): its position in the cell frame and the factors of the
// gradient with c ds/dS folded in.  GBMV-II: with u_j = F_j / T_j and
// vd = v . d_j, the pull on entry j is
//   g_j = [-400 u_j (A + C vd) + B F_j (F_j - 400 u_j r_j^2)] d_j + F_j Cv
// with A = c ds/dS s0 s2 / |v|^2, B = 2 c ds/dS s0 s1 / |v|^2,
// C = -2 c ds/dS s0 s1 s2 / |v|^4 (the d s1, d s2 and d |v|^2 factors) and
// Cv = C v.  GBMV-I: g_j = A e_j r_j^2 d_j with A = 4 c ds/dS gamma_j
// folded per entry.
struct PointChain {
  float px, py, pz, cS, A, B, C, vx, vy, vz, cvx, cvy, cvz;
  int i;
};

template <int MODEL, bool PER, bool ADJ>
__global__ void __launch_bounds__(kCellThreads) gbmv_cell_chain_kernel(const float4* __restrict__ pos, Entries tab,
                                                                       Quad quad, ModelConst m, CellPoints cp,
                                                                       const float2* __restrict__ dEdJ,
                                                                       CellChainOut out) {
  __shared__ float4 s_e[kCellWarps][kMaxList];
  __shared__ float4 s_par[kCellWarps][kMaxList];  // (GBMV-II K | GBMV-I R, R, atom index, -)
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
  for (int l = lane; l < cnt; l += kWarp) {
    const float4 a = __ldg(tab.e + cs.y + l);
    s_e[w][l] = make_float4(a.x - c0.x, a.y - c0.y, a.z - c0.z, a.w);
    const float2 pk = __ldg(tab.par + cs.y + l);
    s_par[w][l] = make_float4(pk.x, pk.y, __int_as_float(__ldg(tab.index + cs.y + l)), 0.0f);
  }
  const int start = cp.start[cell];
  const int* order = cp.order + start;
  const float* state = cp.state + start;
  // cells too dense to sort keep the atomic slot order: every contribution
  // is then reduced on its own (integer sums, independent of the order)
  const bool sorted = P <= kSortMax;
  const int ps = lane / kChainEnt, es = lane % kChainEnt;
  float acc[kEntPerLane][3];
  float accR[kEntPerLane];
#pragma unroll
  for (int e = 0; e < kEntPerLane; ++e) {
    acc[e][0] = acc[e][1] = acc[e][2] = 0.0f;
    accR[e] = 0.0f;
  }
  PointChain* pts = s_pt[w];
  for (int base = 0; base < P; base += kWarp) {
    // lane t prepares point base + t
    {
      const int k = base + lane;
      PointChain pc;
      pc.cS = 0.0f;
      pc.i = -1;
      pc.px = pc.py = pc.pz = pc.A = pc.B = pc.C = pc.vx = pc.vy = pc.vz = pc.cvx = pc.cvy = pc.cvz = 0.0f;
      if (k < P) {
        const int p = order[k];
        const int i = p / m.nq, q = p - i * m.nq;
        const float4 xi = __ldg(pos + i), v = __ldg(quad.qv + q);
        const float2 wq = __ldg(quad.qw + q);
        const float2 de = __ldg(dEdJ + i);
        const float cq = fmaf(de.x, wq.x, de.y * wq.y);
        pc.i = i;
        pc.px = (xi.x - c0.x) + v.x;
        pc.py = (xi.y - c0.y) + v.y;
        pc.pz = (xi.z - c0.z) + v.z;
        float pl;
        if (MODEL == GBX_MODEL_GBMV1) {
          logistic_solvent(m.beta, m.lambda, state[k], pl);
          pc.cS = cq * __fdividef(m.beta * pl, (1.0f + pl) * (1.0f + pl));
          pc.A = 4.0f * pc.cS;
        } else {
          const float s1 = state[k], s2 = state[k + cp.plane], vx = state[k + 2 * cp.plane],
                      vy = state[k + 3 * cp.plane], vz = state[k + 4 * cp.plane];
          const float s3sq = fmaf(vx, vx, fmaf(vy, vy, vz * vz));
          logistic_solvent(m.beta, m.lambda, m.s0 * s1 * s2 / s3sq, pl);
          pc.cS = cq * __fdividef(m.beta * pl, (1.0f + pl) * (1.0f + pl)) * m.s0;
          const float inv3 = 1.0f / s3sq;
          pc.A = pc.cS * (s2 * inv3);
          pc.B = 2.0f * pc.cS * (s1 * inv3);
          pc.C = 2.0f * pc.cS * (-s1 * s2 * inv3 * inv3);
          pc.vx = vx;
          pc.vy = vy;
          pc.vz = vz;
          pc.cvx = pc.C * vx;
          pc.cvy = pc.C * vy;
          pc.cvz = pc.C * vz;
        }
      }
      pts[lane] = pc;
    }
    __syncwarp();
    const int np = min(kWarp, P - base);
    for (int sub = 0; sub < np; sub += kChainPts) {
      const int t = sub + ps;
      const PointChain pc = pts[t < np ? t : 0];
      const bool live = t < np && pc.cS != 0.0f;
      float ox = 0.f, oy = 0.f, oz = 0.f;
      if (live) {
#pragma unroll
        for (int e = 0; e < kEntPerLane; ++e) {
          const int l = es + e * kChainEnt;
          if (l < cnt) {
            const float4 a = s_e[w][l];
            const float4 pk = s_par[w][l];
            const int kj = __float_as_int(pk.z);
            const float3 d = img.apply(make_float3(a.x - pc.px, a.y - pc.py, a.z - pc.pz));
            const float r2 = fmaf(d.x, d.x, fmaf(d.y, d.y, d.z * d.z));
            float gx, gy, gz;
            if (MODEL == GBX_MODEL_GBMV1) {
              const float r4 = r2 * r2;
              const float ex = __expf(a.w * r4);
              if (ADJ) add_dEdR(out, kj, sorted, accR[e], pc.cS * ex * r4 * (-4.0f * a.w / pk.x));
              const float gs = pc.A * a.w * ex * r2;  // dS/d(delta) = 4 gamma e r^2 delta
              gx = gs * d.x;
              gy = gs * d.y;
              gz = gs * d.z;
            } else {
              const float T = fmaf(100.0f, r2, pk.x);
              const float rT = __fdividef(1.0f, T);
              const float CT = a.w * rT;
              const float F = CT * CT;
              const float u = F * rT;  // dF/d(delta) = -400 u delta
              const float vd = fmaf(pc.vx, d.x, fmaf(pc.vy, d.y, pc.vz * d.z));
              if (ADJ) {
                const float R = pk.y;
                const float Cp = 10.0f * m.p1, Tp = Cp - 200.0f * R;
                const float dFdR = 2.0f * CT * __fdividef(Cp * T - a.w * Tp, T * T);
                // c ds/dS (s2 dF + s1 d(r^2 F^2) + d|v|^2) / |v|^2 terms, as pc.A, pc.B, pc.C carry them
                add_dEdR(out, kj, sorted, accR[e], dFdR * (pc.A + pc.B * (r2 * F) + pc.C * vd));
              }
              const float sc = -400.0f * u * fmaf(pc.C, vd, pc.A) + pc.B * F * fmaf(-400.0f * u, r2, F);
              gx = fmaf(sc, d.x, F * pc.cvx);
              gy = fmaf(sc, d.y, F * pc.cvy);
              gz = fmaf(sc, d.z, F * pc.cvz);
            }
            if (kj != pc.i) {  // atom i's own entry moves with the point: no force
              if (sorted) {
                acc[e][0] += gx;
                acc[e][1] += gy;
                acc[e][2] += gz;
              } else {
                add_fixed3(out, kj, -gx, -gy, -gz);
              }
              ox += gx;
              oy += gy;
              oz += gz;
            }
          }
        }
      }
      // the point's own pull, summed over its entry lanes
#pragma unroll
      for (int off = 1; off < kChainEnt; off <<= 1) {
        ox += __shfl_xor_sync(0xffffffffu, ox, off);
        oy += __shfl_xor_sync(0xffffffffu, oy, off);
        oz += __shfl_xor_sync(0xffffffffu, oz, off);
      }
      if (es == 0 && t < np) s_own[w][t] = make_float3(ox, oy, oz);
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
  // the entries' pull over all of the cell's points: summed over the point
  // lanes, one fixed-point reduction per entry
#pragma unroll
  for (int e = 0; e < kEntPerLane; ++e) {
#pragma unroll
    for (int off = kChainEnt; off < kWarp; off <<= 1) {
      acc[e][0] += __shfl_xor_sync(0xffffffffu, acc[e][0], off);
      acc[e][1] += __shfl_xor_sync(0xffffffffu, acc[e][1], off);
      acc[e][2] += __shfl_xor_sync(0xffffffffu, acc[e][2], off);
      if (ADJ) accR[e] += __shfl_xor_sync(0xffffffffu, accR[e], off);
    }
    const int l = es + e * kChainEnt;
    if (ps == 0 && l < cnt) {
      const int kj = __float_as_int(s_par[w][l].z);
      if (sorted) add_fixed3(out, kj, -acc[e][0], -acc[e][1], -acc[e][2]);
      if (ADJ && sorted) {
        const long long r = float_to_fixed(accR[e]);
        if (r) atomicAdd(&out.dEdR[kj], (unsigned long long)r);
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
  const long long cells = ctx->cell_cap;
  const int cell_blocks = (int)((cells + kCellWarps - 1) / kCellWarps);
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
  if (m.model == GBX_MODEL_GBMV1) {
    if (per) gbmv_cell_integral_kernel<GBX_MODEL_GBMV1, true><<<cell_blocks, kCellThreads, 0, st>>>(pos, t, qd, m, cp);
    else gbmv_cell_integral_kernel<GBX_MODEL_GBMV1, false><<<cell_blocks, kCellThreads, 0, st>>>(pos, t, qd, m, cp);
  } else {
    if (per) gbmv_cell_integral_kernel<GBX_MODEL_GBMV2, true><<<cell_blocks, kCellThreads, 0, st>>>(pos, t, qd, m, cp);
    else gbmv_cell_integral_kernel<GBX_MODEL_GBMV2, false><<<cell_blocks, kCellThreads, 0, st>>>(pos, t, qd, m, cp);
  }
  gbmv_reduce_kernel<<<bin_blocks, kBinThreads, 0, st>>>(ctx->n, qd, m.nq, chunk, ctx->n_chunks, ctx->d_sval,
                                                         ctx->d_J);
  ctx->launches += 8;  // bin, ncell copy, three scan phases, fill, integral, reduce
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
