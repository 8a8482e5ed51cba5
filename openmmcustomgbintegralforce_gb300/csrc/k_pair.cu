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

}  // namespace

int pair_energy_parts(int n, int segments) { return ((n + kPairThreads - 1) / kPairThreads) * segments; }

int pair_segments(int n) {
  // enough CTAs for ~2 waves on 152 SMs with 8 resident CTAs each
  const int iblocks = (n + kPairThreads - 1) / kPairThreads;
  int s = (2 * 152 * 8 + iblocks - 1) / iblocks;
  const int max_s = (n + kJTile - 1) / kJTile;
  if (s > max_s) s = max_s;
  if (s < 1) s = 1;
  return s;
}

// The same kernel on caller-supplied buffers (used by the allocation-free
// entry point): energy_part needs pair_energy_parts(n, pair_segments(n))
// doubles and dEdB must be zero on entry.
cudaError_t launch_pair_raw(const float4* pos, const float* charge, const float2* born, int n, float pref,
                            float cutoff2, unsigned long long* force, int stride, unsigned long long* dEdB,
                            double* energy_part, cudaStream_t stream) {
  PairArgs a;
  a.pos = pos;
  a.charge = charge;
  a.born = born;
  a.n = n;
  a.segments = pair_segments(n);
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
  PairArgs a;
  a.pos = pos;
  a.charge = ctx->d_charge;
  a.born = reinterpret_cast<const float2*>(ctx->d_bornf);
  a.n = ctx->n;
  a.segments = pair_segments(ctx->n);
  a.pref = (float)ctx->cfg.prefactor;
  a.cutoff2 = ctx->cfg.cutoff > 0 ? (float)(ctx->cfg.cutoff * ctx->cfg.cutoff) : 0.0f;
  a.force = force;
  a.stride = stride;
  a.dEdB = ctx->d_dEdB_fx;
  a.energy_part = ctx->d_energy_part;
  a.dEdq = ctx->d_dEdq_fx;
  dim3 grid((ctx->n + kPairThreads - 1) / kPairThreads, a.segments);
  if (a.cutoff2 > 0) {
    if (adjoint) pair_kernel<true, true><<<grid, kPairThreads, 0, ctx->stream>>>(a);
    else pair_kernel<true, false><<<grid, kPairThreads, 0, ctx->stream>>>(a);
  } else {
    if (adjoint) pair_kernel<false, true><<<grid, kPairThreads, 0, ctx->stream>>>(a);
    else pair_kernel<false, false><<<grid, kPairThreads, 0, ctx->stream>>>(a);
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    ctx->last_error = std::string("pair launch: ") + cudaGetErrorString(e);
    return GBX_ERR_CUDA;
  }
  return GBX_OK;
}

}  // namespace gbx
