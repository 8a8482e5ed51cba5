// Pairwise GB energy, pair forces and dE/dB (CharmmReferenceGBSW.cpp:237-283;
// CharmmReferenceGBMV.cpp:268-347 with the canonical energy terms).
//
//   D = r^2 / (4 B_i B_j),  f = sqrt(r^2 + B_i B_j e^-D),  e_ij = pref q_i q_j / f
//   E = sum_{i<j} e_ij + 1/2 sum_i pref q_i^2 / B_i
//
// Each thread owns one atom i and streams every j through shared memory
// (warp-uniform broadcast reads).  Only i-side quantities are accumulated, so
// every ordered pair is visited once from each end: twice the pair
// arithmetic of a symmetric tile scheme, but no j-side accumulators, no
// shuffles and no per-tile atomics, and every per-atom sum runs in a fixed
// sequential order.  Per-tile FP32 partial sums are folded into FP64.
#include <algorithm>

#include "gbx_internal.cuh"

namespace gbx {
namespace {

constexpr int kPairThreads = 256;
constexpr int kJTile = 256;

struct PairArgs {
  const float4* pos;    // x, y, z, (model parameter)
  const float* charge;
  const float2* born;   // B, 1/B
  int n;
  int segments;         // j-range split
  float pref;
  float cutoff2;        // <= 0: none
  unsigned long long* force;
  int stride;
  unsigned long long* dEdB;
  double* energy_part;  // one per (i-block, segment)
  unsigned long long* dEdq;  // adjoint: sum_j pref q_j / f_ij (+ self)
};

template <bool CUTOFF, bool ADJ>
__global__ void __launch_bounds__(kPairThreads) pair_kernel(PairArgs a) {
  __shared__ float4 s_pos[kJTile];  // x, y, z, q
  __shared__ float2 s_born[kJTile];
  __shared__ double s_red[kPairThreads / kWarp];
  const int iblk = blockIdx.x;
  const int seg = blockIdx.y;
  const int i = iblk * kPairThreads + threadIdx.x;
  const bool active = i < a.n;
  const int jper = (((a.n + a.segments - 1) / a.segments) + kJTile - 1) / kJTile * kJTile;
  const int j0 = seg * jper, j1 = min(a.n, j0 + jper);
  float4 xi = make_float4(0.f, 0.f, 0.f, 0.f);
  float qi = 0.f, Bi = 1.f, invBi = 1.f;
  if (active) {
    xi = a.pos[i];
    qi = a.charge[i];
    const float2 b = a.born[i];
    Bi = b.x;
    invBi = b.y;
  }
  const float pq = a.pref * qi;
  const float kD = 0.25f * 1.4426950408889634f * invBi;  // D log2(e) = r^2 kD / B_j
  const float kB = 0.25f * invBi;
  double Fx = 0, Fy = 0, Fz = 0, dB = 0, E = 0, dQ = 0;
  for (int jt = j0; jt < j1; jt += kJTile) {
    __syncthreads();
    {
      const int j = jt + threadIdx.x;
      if (j < j1) {
        const float4 p = a.pos[j];
        s_pos[threadIdx.x] = make_float4(p.x, p.y, p.z, a.charge[j]);
        s_born[threadIdx.x] = a.born[j];
      } else {
        s_pos[threadIdx.x] = make_float4(0.f, 0.f, 0.f, 0.f);
        s_born[threadIdx.x] = make_float2(1.f, 1.f);
      }
    }
    __syncthreads();
    const int cnt = min(kJTile, j1 - jt);
    float fx = 0.f, fy = 0.f, fz = 0.f, db = 0.f, e = 0.f, dq = 0.f;
#pragma unroll 4
    for (int jj = 0; jj < cnt; ++jj) {
      const float4 pj = s_pos[jj];
      const float2 bj = s_born[jj];
      const float dx = pj.x - xi.x, dy = pj.y - xi.y, dz = pj.z - xi.z;
      const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
      bool skip = (jt + jj == i);
      if (CUTOFF) skip = skip || (r2 > a.cutoff2);
      if (skip) continue;
      const float ex = exp2f(-r2 * kD * bj.y);
      const float BB = Bi * bj.x;
      const float f2 = fmaf(BB, ex, r2);
      const float invf = rsqrtf(f2);
      const float invf3 = invf * invf * invf;
      const float pqq = pq * pj.w;
      e = fmaf(pqq, invf, e);
      if (ADJ) dq = fmaf(a.pref * pj.w, invf, dq);
      // force on i: d * dG/dr / r with dG/dr / r = -1/4 pref q q (4 - e^-D) / f^3
      const float g = -0.25f * pqq * (4.0f - ex) * invf3;
      fx = fmaf(g, dx, fx);
      fy = fmaf(g, dy, fy);
      fz = fmaf(g, dz, fz);
      // dE/dB_i: -1/2 pref q q e^-D / f^3 (B_j + r^2 / (4 B_i))
      db = fmaf(-0.5f * pqq * ex * invf3, fmaf(r2, kB, bj.x), db);
    }
    Fx += fx;
    Fy += fy;
    Fz += fz;
    dB += db;
    E += 0.5 * (double)e;  // every pair is visited from both ends
    if (ADJ) dQ += dq;
  }
  if (active && seg == 0) {
    // self term: 1/2 pref q_i^2 / B_i, dE/dB_i = -1/2 pref q_i^2 / B_i^2
    E += 0.5 * (double)pq * qi * invBi;
    dB += -0.5 * (double)pq * qi * invBi * invBi;
    if (ADJ) dQ += (double)pq * invBi;
  }
  if (active) {
    red_add_fixed_d(&a.force[i], Fx);
    red_add_fixed_d(&a.force[i + a.stride], Fy);
    red_add_fixed_d(&a.force[i + 2 * a.stride], Fz);
    red_add_fixed_d(&a.dEdB[i], dB);
    if (ADJ) red_add_fixed_d(&a.dEdq[i], dQ);
  }
  // deterministic block reduction of the energy
  for (int off = 16; off > 0; off >>= 1) E += __shfl_xor_sync(0xffffffffu, E, off);
  if (threadIdx.x % kWarp == 0) s_red[threadIdx.x / kWarp] = E;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0;
    for (int w = 0; w < kPairThreads / kWarp; ++w) s += s_red[w];
    a.energy_part[seg * gridDim.x + iblk] = s;
  }
}

// ---------------------------------------------------------------------------
// Symmetric scheme (the context path): every unordered pair once.  A warp
// owns an i-block of 128 atoms (four per lane: 128 b + 32 u + lane)
// and a run of 32-atom j-tiles above the block.  A j-tile's atoms and their
// force / dE/dB accumulators rotate one lane per step through shuffles, so
// after 32 steps every (i, j) pair of the tile was evaluated once and each
// lane again holds the complete j-side sums of its own j atom.  Pairs inside
// an i-block, and the self terms, are done by pair_block_kernel.  Every sum
// runs in a fixed order; i- and j-side sums are rounded to fixed point once
// per tile and added as integers.
// ---------------------------------------------------------------------------
constexpr int kNI = 4;          // i-atoms per lane
constexpr int kSymI = kWarp * kNI;  // atoms per i-block (one warp)
constexpr int kSymChunkMax = 8;  // j-tiles per warp unit, at most (16 and 32 measured slower at 50k: ragged tails)
constexpr int kSymThreads = 128;

struct SymArgs {
  const float4* pos;
  const float* charge;
  const float2* born;
  int n;
  float pref;
  float cutoff2;  // <= 0: none
  unsigned long long* force;
  int stride;
  unsigned long long* dEdB;
  unsigned long long* dEdq;
  unsigned long long* energy;  // fixed point (2^-32), summed as integers
  const float4* tile_box;      // cutoff: [2 * ntiles] (lower, upper) corner of each 32-atom tile
  const int* perm;             // cutoff: slot k holds atom perm[k] (spatial order); nullptr: identity
  float3 L, iL;  // periodic: box edges and their inverses (minimum image)
  int nblocks, ntiles, chunks;
  int chunk;  // j-tiles per warp unit
};

struct PAtom {
  float x, y, z, q, B, invB;
};

struct PAcc {
  float fx, fy, fz, db, dq;
};

__device__ __forceinline__ PAtom load_patom(const SymArgs& a, int k) {
  PAtom t{0.f, 0.f, 0.f, 0.f, 1.f, 1.f};  // padding atom: no charge
  if (k < a.n) {
    if (a.perm) k = a.perm[k];
    const float4 p = a.pos[k];
    const float2 b = a.born[k];
    t = PAtom{p.x, p.y, p.z, a.charge[k], b.x, b.y};
  }
  return t;
}

// Hardware 2^x and 1/sqrt(x) (PTX ex2.approx / rsqrt.approx, relative error
// below 2^-22; subnormal results and inputs flush to zero, which e^-D and
// 1/f never need).
__device__ __forceinline__ float ex2_ftz(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

__device__ __forceinline__ float rsqrt_ftz(float x) {
  float y;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// One pair.  kDi = -log2(e) / (4 B_i), kBi = 1 / (4 B_i), pqi = pref q_i.
// Adds dG/dx_i to ai (force on i: g d, d = x_j - x_i) and dG/dB_i / (-1/2)
// to ai.db; with SYM also the j side to aj.
// Minimum image in a rectangular box: d - L floor(d / L + 1/2)
// (ReferenceForce::getDeltaRPeriodic).
__device__ __forceinline__ float min_image(float d, float L, float iL) { return fmaf(-L, floorf(fmaf(d, iL, 0.5f)), d); }

template <bool SYM, bool CUTOFF, bool ADJ, bool PER = false>
__device__ __forceinline__ void gb_pair(const PAtom& I, float pqi, float kDi, float kBi, const PAtom& J, float kBj,
                                       float pref, float cutoff2, PAcc& ai, PAcc& aj, float& esum,
                                       float3 L = float3{}, float3 iL = float3{}) {
  float dx = J.x - I.x, dy = J.y - I.y, dz = J.z - I.z;
  if (PER) {
    dx = min_image(dx, L.x, iL.x);
    dy = min_image(dy, L.y, iL.y);
    dz = min_image(dz, L.z, iL.z);
  }
  const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
  if (CUTOFF && r2 > cutoff2) return;
  const float ex = ex2_ftz(r2 * (kDi * J.invB));  // e^-D, D = r^2 / (4 B_i B_j)
  const float invf = rsqrt_ftz(fmaf(I.B * J.B, ex, r2));
  const float e = pqi * J.q * invf;
  esum += e;
  const float c = e * invf * invf;  // pref q_i q_j / f^3
  const float cex = c * ex;
  const float g = fmaf(0.25f, cex, -c);  // c (e^-D / 4 - 1)
  ai.fx = fmaf(g, dx, ai.fx);
  ai.fy = fmaf(g, dy, ai.fy);
  ai.fz = fmaf(g, dz, ai.fz);
  ai.db = fmaf(cex, fmaf(r2, kBi, J.B), ai.db);
  if (ADJ) ai.dq = fmaf(pref * J.q, invf, ai.dq);
  if (SYM) {
    aj.fx = fmaf(-g, dx, aj.fx);
    aj.fy = fmaf(-g, dy, aj.fy);
    aj.fz = fmaf(-g, dz, aj.fz);
    aj.db = fmaf(cex, fmaf(r2, kBj, I.B), aj.db);
    if (ADJ) aj.dq = fmaf(pref * I.q, invf, aj.dq);
  }
}

// Two i atoms (the halves of each float2) against one j atom, in the packed
// FP32x2 instructions: one issue slot does both halves' arithmetic, each half
// rounded exactly as the scalar gb_pair rounds it.  Both sides are summed as
// -g d (exact negations of the scalar form's terms): that is the force on j
// as it stands and the force on i negated; the j side in two halves that are
// added once per tile.  With a cutoff, a pair beyond it gets 1/f = 0, which
// turns every one of its terms into a zero that leaves the sums unchanged.
struct PAtom2 {
  float2 nx, ny, nz;  // -x, -y, -z
  float2 B, pq, kD, kB;
};

struct PAcc2 {
  float2 fx, fy, fz, db, dq;
};

struct PJ2 {  // one j atom, broadcast to both halves
  float2 x, y, z, q, B, invB, kB, pq;
};

__device__ __forceinline__ float2 bcast2(float v) { return make_float2(v, v); }

template <bool CUTOFF, bool ADJ, bool PER>
__device__ __forceinline__ void gb_pair2(const PAtom2& I, const PJ2& J, float cutoff2, PAcc2& ai, PAcc2& aj,
                                        float2& esum, float3 L, float3 iL) {
  float2 dx = __fadd2_rn(J.x, I.nx), dy = __fadd2_rn(J.y, I.ny), dz = __fadd2_rn(J.z, I.nz);
  if (PER) {
    dx = make_float2(min_image(dx.x, L.x, iL.x), min_image(dx.y, L.x, iL.x));
    dy = make_float2(min_image(dy.x, L.y, iL.y), min_image(dy.y, L.y, iL.y));
    dz = make_float2(min_image(dz.x, L.z, iL.z), min_image(dz.y, L.z, iL.z));
  }
  const float2 r2 = __ffma2_rn(dx, dx, __ffma2_rn(dy, dy, __fmul2_rn(dz, dz)));
  const float2 arg = __fmul2_rn(r2, __fmul2_rn(I.kD, J.invB));
  const float2 ex = make_float2(ex2_ftz(arg.x), ex2_ftz(arg.y));
  const float2 f2 = __ffma2_rn(__fmul2_rn(I.B, J.B), ex, r2);
  float2 invf = make_float2(rsqrt_ftz(f2.x), rsqrt_ftz(f2.y));
  if (CUTOFF) {
    if (r2.x > cutoff2) invf.x = 0.0f;
    if (r2.y > cutoff2) invf.y = 0.0f;
  }
  const float2 e = __fmul2_rn(__fmul2_rn(I.pq, J.q), invf);
  esum = __fadd2_rn(esum, e);
  const float2 c = __fmul2_rn(__fmul2_rn(e, invf), invf);
  const float2 cex = __fmul2_rn(c, ex);
  const float2 gn = __ffma2_rn(bcast2(-0.25f), cex, c);  // -g = c (1 - e^-D / 4)
  ai.fx = __ffma2_rn(gn, dx, ai.fx);
  ai.fy = __ffma2_rn(gn, dy, ai.fy);
  ai.fz = __ffma2_rn(gn, dz, ai.fz);
  ai.db = __ffma2_rn(cex, __ffma2_rn(r2, I.kB, J.B), ai.db);
  if (ADJ) ai.dq = __ffma2_rn(J.pq, invf, ai.dq);
  aj.fx = __ffma2_rn(gn, dx, aj.fx);
  aj.fy = __ffma2_rn(gn, dy, aj.fy);
  aj.fz = __ffma2_rn(gn, dz, aj.fz);
  aj.db = __ffma2_rn(cex, __ffma2_rn(r2, J.kB, I.B), aj.db);
  if (ADJ) aj.dq = __ffma2_rn(I.pq, invf, aj.dq);
}

struct PFixed {
  long long fx = 0, fy = 0, fz = 0, db = 0, dq = 0;
  __device__ __forceinline__ void add(const PAcc& v) {
    fx += float_to_fixed(v.fx);
    fy += float_to_fixed(v.fy);
    fz += float_to_fixed(v.fz);
    db += float_to_fixed(-0.5f * v.db);
    dq += float_to_fixed(v.dq);
  }
};

template <bool ADJ>
__device__ __forceinline__ void push_atom(const SymArgs& a, int k, const PFixed& f) {
  if (k >= a.n) return;
  if (a.perm) k = a.perm[k];
  atomicAdd(&a.force[k], (unsigned long long)f.fx);
  atomicAdd(&a.force[k + a.stride], (unsigned long long)f.fy);
  atomicAdd(&a.force[k + 2 * a.stride], (unsigned long long)f.fz);
  atomicAdd(&a.dEdB[k], (unsigned long long)f.db);
  if (ADJ) atomicAdd(&a.dEdq[k], (unsigned long long)f.dq);
}

__device__ __forceinline__ double warp_sum(double v) {
  for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
  return v;
}

constexpr float kLog2e = 1.4426950408889634f;

// Bounding box of each 32-atom tile (cutoff path), one warp per tile.
__global__ void __launch_bounds__(kSymThreads) tile_box_kernel(const float4* __restrict__ pos, const int* __restrict__ perm,
                                                               int n, int ntiles, float4* __restrict__ box) {
  const int t = (blockIdx.x * blockDim.x + threadIdx.x) / kWarp;
  const int lane = threadIdx.x % kWarp;
  if (t >= ntiles) return;
  const int k = kWarp * t + lane;
  float lo[3], hi[3];
  if (k < n) {
    const float4 p = pos[perm[k]];
    lo[0] = hi[0] = p.x;
    lo[1] = hi[1] = p.y;
    lo[2] = hi[2] = p.z;
  } else {  // padding: the tile's first atom
    const float4 p = pos[perm[kWarp * t]];
    lo[0] = hi[0] = p.x;
    lo[1] = hi[1] = p.y;
    lo[2] = hi[2] = p.z;
  }
  for (int off = 16; off > 0; off >>= 1)
    for (int d = 0; d < 3; ++d) {
      lo[d] = fminf(lo[d], __shfl_xor_sync(0xffffffffu, lo[d], off));
      hi[d] = fmaxf(hi[d], __shfl_xor_sync(0xffffffffu, hi[d], off));
    }
  if (lane == 0) {
    box[2 * t] = make_float4(lo[0], lo[1], lo[2], 0.f);
    box[2 * t + 1] = make_float4(hi[0], hi[1], hi[2], 0.f);
  }
}

// Squared distance between two boxes (0 if they overlap).
__device__ __forceinline__ float box_gap2(const float4 alo, const float4 ahi, const float4 blo, const float4 bhi) {
  const float gx = fmaxf(0.f, fmaxf(blo.x - ahi.x, alo.x - bhi.x));
  const float gy = fmaxf(0.f, fmaxf(blo.y - ahi.y, alo.y - bhi.y));
  const float gz = fmaxf(0.f, fmaxf(blo.z - ahi.z, alo.z - bhi.z));
  return fmaf(gx, gx, fmaf(gy, gy, gz * gz));
}

__device__ __forceinline__ float2 shfl2(float2 v, int src) {
  return make_float2(__shfl_sync(0xffffffffu, v.x, src), __shfl_sync(0xffffffffu, v.y, src));
}

// The plain form is capped at 96 registers (five blocks per SM); the cutoff
// and adjoint forms keep their wider register sets.  PER: minimum image in a
// periodic box, every tile pair evaluated.
template <bool CUTOFF, bool ADJ, bool PER = false>
__global__ void __launch_bounds__(kSymThreads, (CUTOFF || ADJ) ? 1 : 5) pair_sym_kernel(SymArgs a) {
  static_assert(kNI % 2 == 0, "i atoms are paired into float2 halves");
  constexpr int kNH = kNI / 2;
  const int unit = (blockIdx.x * blockDim.x + threadIdx.x) / kWarp;
  const int lane = threadIdx.x % kWarp;
  if (unit >= a.nblocks * a.chunks) return;
  const int b = unit / a.chunks, ch = unit % a.chunks;
  const int jt0 = kNI * b + kNI + ch * a.chunk;
  const int jt1 = min(a.ntiles, jt0 + a.chunk);
  // the i atoms' fixed-point sums, lane-private in shared memory (touched
  // once per tile; in registers they would cost a quarter of the occupancy)
  constexpr int kNF = ADJ ? 5 : 4;
  __shared__ long long s_si[kSymThreads / kWarp][kNI * kNF][kWarp];
  long long(*si)[kWarp] = s_si[threadIdx.x / kWarp];
  double E = 0.0;
  if (jt0 < jt1) {
#pragma unroll
    for (int f = 0; f < kNI * kNF; ++f) si[f][lane] = 0;
    PAtom2 I[kNH];  // half h, slot s: atom 128 b + 32 (2 h + s) + lane
#pragma unroll
    for (int h = 0; h < kNH; ++h) {
      const PAtom p0 = load_patom(a, kSymI * b + kWarp * (2 * h) + lane);
      const PAtom p1 = load_patom(a, kSymI * b + kWarp * (2 * h + 1) + lane);
      I[h].nx = make_float2(-p0.x, -p1.x);
      I[h].ny = make_float2(-p0.y, -p1.y);
      I[h].nz = make_float2(-p0.z, -p1.z);
      I[h].B = make_float2(p0.B, p1.B);
      I[h].pq = make_float2(a.pref * p0.q, a.pref * p1.q);
      I[h].kD = make_float2(-0.25f * kLog2e * p0.invB, -0.25f * kLog2e * p1.invB);
      I[h].kB = make_float2(0.25f * p0.invB, 0.25f * p1.invB);
    }
    const int src = (lane + 1) % kWarp;
    float4 ilo = make_float4(0.f, 0.f, 0.f, 0.f), ihi = ilo;
    if (CUTOFF && !PER) {  // the i-block's box: the union of its tiles
      ilo = make_float4(3e38f, 3e38f, 3e38f, 0.f);
      ihi = make_float4(-3e38f, -3e38f, -3e38f, 0.f);
      for (int u = 0; u < kNI; ++u) {
        const int t = min(kNI * b + u, a.ntiles - 1);
        const float4 l = a.tile_box[2 * t], h = a.tile_box[2 * t + 1];
        ilo = make_float4(fminf(ilo.x, l.x), fminf(ilo.y, l.y), fminf(ilo.z, l.z), 0.f);
        ihi = make_float4(fmaxf(ihi.x, h.x), fmaxf(ihi.y, h.y), fmaxf(ihi.z, h.z), 0.f);
      }
    }
    for (int jt = jt0; jt < jt1; ++jt) {
      if (CUTOFF && !PER && box_gap2(ilo, ihi, a.tile_box[2 * jt], a.tile_box[2 * jt + 1]) > a.cutoff2) continue;
      PAtom J = load_patom(a, kWarp * jt + lane);
      const float2 z2 = make_float2(0.f, 0.f);
      PAcc2 ai[kNH], aj{z2, z2, z2, z2, z2};
#pragma unroll
      for (int h = 0; h < kNH; ++h) ai[h] = PAcc2{z2, z2, z2, z2, z2};
      float2 et = z2;
#pragma unroll 2
      for (int t = 0; t < kWarp; ++t) {
        const PJ2 J2{bcast2(J.x), bcast2(J.y), bcast2(J.z), bcast2(J.q), bcast2(J.B), bcast2(J.invB),
                     bcast2(0.25f * J.invB), bcast2(a.pref * J.q)};
#pragma unroll
        for (int h = 0; h < kNH; ++h) gb_pair2<CUTOFF, ADJ, PER>(I[h], J2, a.cutoff2, ai[h], aj, et, a.L, a.iL);
        J.x = __shfl_sync(0xffffffffu, J.x, src);
        J.y = __shfl_sync(0xffffffffu, J.y, src);
        J.z = __shfl_sync(0xffffffffu, J.z, src);
        J.q = __shfl_sync(0xffffffffu, J.q, src);
        J.B = __shfl_sync(0xffffffffu, J.B, src);
        J.invB = __shfl_sync(0xffffffffu, J.invB, src);
        aj.fx = shfl2(aj.fx, src);
        aj.fy = shfl2(aj.fy, src);
        aj.fz = shfl2(aj.fz, src);
        aj.db = shfl2(aj.db, src);
        if (ADJ) aj.dq = shfl2(aj.dq, src);
      }
      PFixed sj;
      sj.add(PAcc{aj.fx.x + aj.fx.y, aj.fy.x + aj.fy.y, aj.fz.x + aj.fz.y, aj.db.x + aj.db.y, aj.dq.x + aj.dq.y});
      push_atom<ADJ>(a, kWarp * jt + lane, sj);
#pragma unroll
      for (int h = 0; h < kNH; ++h) {
        const float2 v[5] = {ai[h].fx, ai[h].fy, ai[h].fz, ai[h].db, ai[h].dq};
#pragma unroll
        for (int f = 0; f < kNF; ++f) {
          const float sc = f < 3 ? -1.0f : f == 3 ? -0.5f : 1.0f;  // force: negated sums; dE/dB: -1/2 db
          si[(2 * h) * kNF + f][lane] += float_to_fixed(sc * v[f].x);
          si[(2 * h + 1) * kNF + f][lane] += float_to_fixed(sc * v[f].y);
        }
      }
      E += (double)et.x + (double)et.y;
    }
#pragma unroll
    for (int u = 0; u < kNI; ++u) {
      PFixed su;
      su.fx = si[u * kNF][lane];
      su.fy = si[u * kNF + 1][lane];
      su.fz = si[u * kNF + 2][lane];
      su.db = si[u * kNF + 3][lane];
      if (ADJ) su.dq = si[u * kNF + 4][lane];
      push_atom<ADJ>(a, kSymI * b + kWarp * u + lane, su);
    }
  }
  E = warp_sum(E);
  if (lane == 0 && E != 0.0) atomicAdd(a.energy, (unsigned long long)__double2ll_rn(E * kFixedScale));
}

// Pairs inside each i-block (i side only, each ordered pair once: lane t of
// slot h broadcasts its atom to the warp) and the self terms 1/2 pref q^2 / B.
// A warp per (i-block, slot h, half of the slot's lanes): the partial sums
// are separate fixed-point reductions, so small systems get eight times the
// warps.
constexpr int kBlockSplit = 2;  // warps per broadcast slot
template <bool CUTOFF, bool ADJ, bool PER = false>
__global__ void __launch_bounds__(kSymThreads) pair_block_kernel(SymArgs a) {
  const int wid = (blockIdx.x * blockDim.x + threadIdx.x) / kWarp;
  const int b = wid / (kNI * kBlockSplit), h = (wid / kBlockSplit) % kNI, part = wid % kBlockSplit;
  const int lane = threadIdx.x % kWarp;
  if (b >= a.nblocks) return;
  PAtom I[kNI];
  float pq[kNI], kD[kNI], kB[kNI], e[kNI];
  PAcc ai[kNI], dummy{0.f, 0.f, 0.f, 0.f, 0.f};
#pragma unroll
  for (int u = 0; u < kNI; ++u) {
    I[u] = load_patom(a, kSymI * b + kWarp * u + lane);
    pq[u] = a.pref * I[u].q;
    kD[u] = -0.25f * kLog2e * I[u].invB;
    kB[u] = 0.25f * I[u].invB;
    ai[u] = PAcc{0.f, 0.f, 0.f, 0.f, 0.f};
    e[u] = 0.0f;
  }
  // slot h's atoms, selected without indexing the register array
  PAtom src = I[0];
#pragma unroll
  for (int u = 1; u < kNI; ++u)
    if (h == u) src = I[u];
  for (int t = part * (kWarp / kBlockSplit); t < (part + 1) * (kWarp / kBlockSplit); ++t) {
    const PAtom J{__shfl_sync(0xffffffffu, src.x, t), __shfl_sync(0xffffffffu, src.y, t),
                  __shfl_sync(0xffffffffu, src.z, t), __shfl_sync(0xffffffffu, src.q, t),
                  __shfl_sync(0xffffffffu, src.B, t), __shfl_sync(0xffffffffu, src.invB, t)};
#pragma unroll
    for (int u = 0; u < kNI; ++u)
      if (h != u || t != lane)
        gb_pair<false, CUTOFF, ADJ, PER>(I[u], pq[u], kD[u], kB[u], J, 0.f, a.pref, a.cutoff2, ai[u], dummy, e[u],
                                         a.L, a.iL);
  }
  double E = 0.0;
#pragma unroll
  for (int u = 0; u < kNI; ++u) {
    PFixed su;
    su.add(ai[u]);
    if (h == 0 && part == 0) {  // the self terms, once
      su.db += float_to_fixed(-0.5f * pq[u] * I[u].q * I[u].invB * I[u].invB);
      if (ADJ) su.dq += float_to_fixed(pq[u] * I[u].invB);
    }
    push_atom<ADJ>(a, kSymI * b + kWarp * u + lane, su);
    E += 0.5 * (double)e[u] + (h == 0 && part == 0 ? 0.5 * (double)pq[u] * I[u].q * I[u].invB : 0.0);
  }
  E = warp_sum(E);
  if (lane == 0 && E != 0.0) atomicAdd(a.energy, (unsigned long long)__double2ll_rn(E * kFixedScale));
}

// ---------------------------------------------------------------------------
// Spatial order for the cutoff pair term: atoms are binned into cubic cells
// (1 nm, grown so that the grid holds at most kMaxSortCells cells) and, within
// a cell, kept in ascending atom order, so the permutation depends on the
// input alone.  32 consecutive slots then form a compact tile whose bounding
// box is far from most others, and the cutoff culls those tile pairs.
// ---------------------------------------------------------------------------
struct SortGeom {
  float lo[3];
  float inv_cell;
  int dims[3];
  int ncell;
};

constexpr int kBoxThreads = 1024;
constexpr int kSortSeg = 512;  // atoms per cell ranked in shared memory

__global__ void __launch_bounds__(kBoxThreads) sort_geom_kernel(const float4* __restrict__ pos, int n,
                                                                SortGeom* __restrict__ g) {
  __shared__ float s_lo[3][kBoxThreads / kWarp], s_hi[3][kBoxThreads / kWarp];
  float lo[3] = {3e38f, 3e38f, 3e38f}, hi[3] = {-3e38f, -3e38f, -3e38f};
  for (int k = threadIdx.x; k < n; k += blockDim.x) {
    const float4 p = pos[k];
    lo[0] = fminf(lo[0], p.x), hi[0] = fmaxf(hi[0], p.x);
    lo[1] = fminf(lo[1], p.y), hi[1] = fmaxf(hi[1], p.y);
    lo[2] = fminf(lo[2], p.z), hi[2] = fmaxf(hi[2], p.z);
  }
  for (int off = 16; off > 0; off >>= 1)
    for (int d = 0; d < 3; ++d) {
      lo[d] = fminf(lo[d], __shfl_xor_sync(0xffffffffu, lo[d], off));
      hi[d] = fmaxf(hi[d], __shfl_xor_sync(0xffffffffu, hi[d], off));
    }
  if (threadIdx.x % kWarp == 0)
    for (int d = 0; d < 3; ++d) {
      s_lo[d][threadIdx.x / kWarp] = lo[d];
      s_hi[d][threadIdx.x / kWarp] = hi[d];
    }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x / kWarp); ++w)
      for (int d = 0; d < 3; ++d) {
        s_lo[d][0] = fminf(s_lo[d][0], s_lo[d][w]);
        s_hi[d][0] = fmaxf(s_hi[d][0], s_hi[d][w]);
      }
    float cell = 1.0f;
    for (;;) {
      long long tot = 1;
      int dims[3];
      for (int d = 0; d < 3; ++d) {
        const float span = (s_hi[d][0] - s_lo[d][0]) / cell;
        // non-finite or huge spans (invalid positions) collapse to one cell row
        dims[d] = (span >= 0.0f && span < (float)kMaxSortCells) ? (int)span + 1 : 1;
        tot *= dims[d];
      }
      if (tot <= kMaxSortCells || cell > 1e6f) {
        for (int d = 0; d < 3; ++d) {
          g->lo[d] = s_lo[d][0];
          g->dims[d] = dims[d];
        }
        g->inv_cell = 1.0f / cell;
        g->ncell = (int)tot;
        break;
      }
      cell *= 1.25f;
    }
  }
}

__device__ __forceinline__ int sort_cell(const SortGeom& g, const float4 p) {
  int c[3];
  const float x[3] = {p.x, p.y, p.z};
  for (int d = 0; d < 3; ++d) c[d] = min(g.dims[d] - 1, max(0, (int)((x[d] - g.lo[d]) * g.inv_cell)));
  return (c[0] * g.dims[1] + c[1]) * g.dims[2] + c[2];
}

__global__ void sort_count_kernel(const float4* __restrict__ pos, int n, const SortGeom* __restrict__ g,
                                  int* __restrict__ cell_of, int* __restrict__ count) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const int c = sort_cell(*g, pos[k]);
  cell_of[k] = c;
  atomicAdd(&count[c], 1);
}

// Exclusive scan of the cell counts, one block (at most kMaxSortCells cells).
__global__ void __launch_bounds__(kBoxThreads) sort_scan_kernel(const int* __restrict__ count,
                                                                const SortGeom* __restrict__ g,
                                                                int* __restrict__ start, int* __restrict__ cursor) {
  __shared__ int s_warp[kBoxThreads / kWarp];
  __shared__ int s_carry;
  const int ncell = g->ncell;
  const int lane = threadIdx.x % kWarp, wib = threadIdx.x / kWarp;
  if (threadIdx.x == 0) s_carry = 0;
  __syncthreads();
  for (int base = 0; base < ncell; base += blockDim.x) {
    const int c = base + threadIdx.x;
    const int v = c < ncell ? count[c] : 0;
    int incl = v;
    for (int off = 1; off < kWarp; off <<= 1) {
      const int u = __shfl_up_sync(0xffffffffu, incl, off);
      if (lane >= off) incl += u;
    }
    if (lane == kWarp - 1) s_warp[wib] = incl;
    __syncthreads();
    if (threadIdx.x == 0) {
      int acc = 0;
      for (int w = 0; w < (int)(blockDim.x / kWarp); ++w) {
        const int t = s_warp[w];
        s_warp[w] = acc;
        acc += t;
      }
    }
    __syncthreads();
    const int excl = s_carry + s_warp[wib] + incl - v;
    if (c < ncell) {
      start[c] = excl;
      cursor[c] = 0;
    }
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) s_carry = excl + v;
    __syncthreads();
  }
}

__global__ void sort_scatter_kernel(const int* __restrict__ cell_of, int n, const int* __restrict__ start,
                                    int* __restrict__ cursor, int* __restrict__ perm) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const int c = cell_of[k];
  perm[start[c] + atomicAdd(&cursor[c], 1)] = k;
}

// Each cell's atoms in ascending atom order: ranks from the scatter's output
// (arbitrary order within a cell) into perm, out of place.
__global__ void __launch_bounds__(kSymThreads) sort_cells_by_atom_kernel(const int* __restrict__ count,
                                                                         const int* __restrict__ start,
                                                                         const SortGeom* __restrict__ g,
                                                                         const int* __restrict__ unsorted,
                                                                         int* __restrict__ perm) {
  __shared__ int s_buf[kSymThreads / kWarp][kSortSeg];
  const int lane = threadIdx.x % kWarp, wib = threadIdx.x / kWarp;
  const int ncell = g->ncell;
  int* buf = s_buf[wib];
  for (int c = (blockIdx.x * blockDim.x + threadIdx.x) / kWarp; c < ncell; c += gridDim.x * blockDim.x / kWarp) {
    const int cnt = count[c], s = start[c];
    const int* src = unsorted + s;
    if (cnt <= kSortSeg) {
      for (int p = lane; p < cnt; p += kWarp) buf[p] = src[p];
      __syncwarp();
      src = buf;
    }
    for (int p = lane; p < cnt; p += kWarp) {
      const int v = src[p];
      int r = 0;
      for (int q = 0; q < cnt; ++q) r += src[q] < v;  // atom indices are distinct
      perm[s + r] = v;
    }
    __syncwarp();
  }
}

SymArgs sym_args(int n) {
  SymArgs a{};
  a.n = n;
  a.nblocks = (n + kSymI - 1) / kSymI;
  a.ntiles = (n + kWarp - 1) / kWarp;
  // j-tiles per unit: long runs amortise the i-block setup, but small
  // systems need short ones to give ~8k working warps
  const long long visits = (long long)a.nblocks * a.ntiles / 2;
  a.chunk = (int)std::max(2LL, std::min((long long)kSymChunkMax, visits / 8192));
  a.chunks = (a.ntiles + a.chunk - 1) / a.chunk;
  return a;
}

}  // namespace

int pair_energy_parts(int n, int segments) { return ((n + kPairThreads - 1) / kPairThreads) * segments; }

int pair_segments(int n, int sms) {
  // enough CTAs for ~2 waves on the device's SMs with 8 resident CTAs each
  const int iblocks = (n + kPairThreads - 1) / kPairThreads;
  int s = (2 * sms * 8 + iblocks - 1) / iblocks;
  const int max_s = (n + kJTile - 1) / kJTile;
  if (s > max_s) s = max_s;
  if (s < 1) s = 1;
  return s;
}

// The same kernel on caller-supplied buffers (used by the allocation-free
// entry point): energy_part needs pair_energy_parts(n, pair_segments(n, sms))
// doubles and dEdB must be zero on entry.
cudaError_t launch_pair_raw(const float4* pos, const float* charge, const float2* born, int n, int sms, float pref,
                            float cutoff2, unsigned long long* force, int stride, unsigned long long* dEdB,
                            double* energy_part, cudaStream_t stream) {
  PairArgs a;
  a.pos = pos;
  a.charge = charge;
  a.born = born;
  a.n = n;
  a.segments = pair_segments(n, sms);
  a.pref = pref;
  a.cutoff2 = cutoff2;
  a.force = force;
  a.stride = stride;
  a.dEdB = dEdB;
  a.energy_part = energy_part;
  a.dEdq = nullptr;
  dim3 grid((n + kPairThreads - 1) / kPairThreads, a.segments);
  if (cutoff2 > 0) pair_kernel<true, false><<<grid, kPairThreads, 0, stream>>>(a);
  else pair_kernel<false, false><<<grid, kPairThreads, 0, stream>>>(a);
  return cudaGetLastError();
}

gbx_status launch_pair(Context* ctx, const float4* pos, unsigned long long* force, int stride, bool adjoint) {
  SymArgs a = sym_args(ctx->n);
  a.pos = pos;
  a.charge = ctx->d_charge;
  a.born = reinterpret_cast<const float2*>(ctx->d_bornf);
  a.pref = (float)ctx->cfg.prefactor;
  a.cutoff2 = ctx->cfg.cutoff > 0 ? (float)(ctx->cfg.cutoff * ctx->cfg.cutoff) : 0.0f;
  a.force = force;
  a.stride = stride;
  a.dEdB = ctx->d_dEdB_fx;
  a.dEdq = ctx->d_dEdq_fx;
  a.energy = ctx->d_energy_fx;
  a.tile_box = ctx->d_tile_box;
  a.perm = nullptr;
  const int wpb = kSymThreads / kWarp;
  const int gu = (a.nblocks * a.chunks + wpb - 1) / wpb, gb = (a.nblocks * kNI * kBlockSplit + wpb - 1) / wpb;
  cudaStream_t st = ctx->stream;
  cudaMemsetAsync(ctx->d_energy_fx, 0, sizeof(unsigned long long), st);
  if (ctx->cfg.periodic) {
    // minimum image, every tile pair evaluated (bounding boxes do not wrap)
    a.L = make_float3((float)ctx->cfg.box[0], (float)ctx->cfg.box[1], (float)ctx->cfg.box[2]);
    a.iL = make_float3((float)(1.0 / ctx->cfg.box[0]), (float)(1.0 / ctx->cfg.box[1]), (float)(1.0 / ctx->cfg.box[2]));
    if (adjoint) {
      pair_sym_kernel<true, true, true><<<gu, kSymThreads, 0, st>>>(a);
      pair_block_kernel<true, true, true><<<gb, kSymThreads, 0, st>>>(a);
    } else {
      pair_sym_kernel<true, false, true><<<gu, kSymThreads, 0, st>>>(a);
      pair_block_kernel<true, false, true><<<gb, kSymThreads, 0, st>>>(a);
    }
    ctx->launches += 2;
  } else if (a.cutoff2 > 0) {
    // spatial order, then tile boxes over it
    const int n = a.n, nb = (n + 255) / 256;
    SortGeom* sg = reinterpret_cast<SortGeom*>(ctx->d_sgeom);
    sort_geom_kernel<<<1, kBoxThreads, 0, st>>>(pos, n, sg);
    cudaMemsetAsync(ctx->d_scount, 0, sizeof(int) * kMaxSortCells, st);
    sort_count_kernel<<<nb, 256, 0, st>>>(pos, n, sg, ctx->d_cell_of, ctx->d_scount);
    sort_scan_kernel<<<1, kBoxThreads, 0, st>>>(ctx->d_scount, sg, ctx->d_sstart, ctx->d_scursor);
    sort_scatter_kernel<<<nb, 256, 0, st>>>(ctx->d_cell_of, n, ctx->d_sstart, ctx->d_scursor, ctx->d_perm_tmp);
    sort_cells_by_atom_kernel<<<ctx->sms * 8, kSymThreads, 0, st>>>(ctx->d_scount, ctx->d_sstart, sg, ctx->d_perm_tmp,
                                                               ctx->d_perm);
    ctx->launches += 5;
    a.perm = ctx->d_perm;
    tile_box_kernel<<<(a.ntiles + wpb - 1) / wpb, kSymThreads, 0, st>>>(pos, ctx->d_perm, a.n, a.ntiles,
                                                                        ctx->d_tile_box);
    ++ctx->launches;
    if (adjoint) {
      pair_sym_kernel<true, true><<<gu, kSymThreads, 0, st>>>(a);
      ++ctx->launches;
      pair_block_kernel<true, true><<<gb, kSymThreads, 0, st>>>(a);
      ++ctx->launches;
    } else {
      pair_sym_kernel<true, false><<<gu, kSymThreads, 0, st>>>(a);
      ++ctx->launches;
      pair_block_kernel<true, false><<<gb, kSymThreads, 0, st>>>(a);
      ++ctx->launches;
    }
  } else {
    if (adjoint) {
      pair_sym_kernel<false, true><<<gu, kSymThreads, 0, st>>>(a);
      ++ctx->launches;
      pair_block_kernel<false, true><<<gb, kSymThreads, 0, st>>>(a);
      ++ctx->launches;
    } else {
      pair_sym_kernel<false, false><<<gu, kSymThreads, 0, st>>>(a);
      ++ctx->launches;
      pair_block_kernel<false, false><<<gb, kSymThreads, 0, st>>>(a);
      ++ctx->launches;
    }
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    ctx->last_error = std::string("pair launch: ") + cudaGetErrorString(e);
    return GBX_ERR_CUDA;
  }
  return GBX_OK;
}

}  // namespace gbx
