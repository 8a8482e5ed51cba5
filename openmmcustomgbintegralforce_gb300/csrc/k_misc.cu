// Small per-atom kernels: model constants, position staging, FP64 Born-radius
// assembly, dE/dB -> dE/dJ conversion and the deterministic energy reduction.
#include <math.h>

#include "gbx_internal.cuh"

namespace gbx {

ModelConst make_model_const(const Context* ctx) {
  const gbx_config& c = ctx->cfg;
  ModelConst m{};
  m.model = c.model;
  m.table_mode = c.table_mode;
  m.cap = c.table_cap;
  m.skip_empty = c.skip_empty;
  m.nq = c.n_radial * c.lebedev_order;
  m.nshell = c.lebedev_order;
  m.cutoff_chain_quirk = c.cutoff_chain_quirk;
  const double w = c.switch_width;
  m.sw = (float)w;
  m.c1 = (float)(3.0 / (4.0 * w));
  m.c3 = (float)(1.0 / (4.0 * w * w * w));
  m.gamma0_lnlambda = (float)(c.gamma0 * log(c.lambda));
  m.beta = (float)c.beta;
  m.lambda = (float)c.lambda;
  m.s0 = (float)c.s0;
  m.p1 = (float)c.p1;
  m.p2 = (float)c.p2;
  m.cutoff2 = c.cutoff > 0 ? (float)(c.cutoff * c.cutoff) : 0.0f;
  m.pref = (float)c.prefactor;
  m.h = c.grid_length;
  m.buffer = c.table_buffer;
  m.cutoff = c.cutoff;
  return m;
}

namespace {

// Internal positions: x, y, z and the model's main per-atom parameter in .w
// (GBSW: R' = (R + 0.03) 0.952, CharmmReferenceGBSW.cpp:625; GBMV-I:
// gamma_j = gamma0 ln(lambda) / R^4, GBMVIntegralTypeI.cpp:168; GBMV-II:
// C_j = 10 P1 R + P2, GBMVIntegralTypeII.cpp:179), from the caller's float4
// or double4 positions (OpenMM's single / double precision posq).  With an
// atom order set, internal atom i is read from the caller's slot slot_of[i].
template <bool DBL>
__global__ void stage_positions_kernel(const void* __restrict__ in, int n, const int* __restrict__ slot_of,
                                       const float* __restrict__ wpar, float4* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int k = slot_of ? slot_of[i] : i;
  float x, y, z;
  if (DBL) {
    const double4 p = static_cast<const double4*>(in)[k];
    x = (float)p.x;
    y = (float)p.y;
    z = (float)p.z;
  } else {
    const float4 p = static_cast<const float4*>(in)[k];
    x = p.x;
    y = p.y;
    z = p.z;
  }
  out[i] = make_float4(x, y, z, wpar[i]);
}

// The caller's outputs of a call that ran on internal buffers: forces added
// to the caller's slots (each slot written by one thread), the energy added
// to a float.
__global__ void finish_outputs_kernel(int n, const int* __restrict__ slot_of,
                                      const unsigned long long* __restrict__ fint, unsigned long long* __restrict__ fout,
                                      int stride, const double* __restrict__ e_int, float* __restrict__ e_float) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i == 0 && e_float) *e_float += (float)*e_int;
  if (i >= n || !fout) return;
  const int k = slot_of ? slot_of[i] : i;
  for (int c = 0; c < 3; ++c) fout[(size_t)c * stride + k] += fint[(size_t)c * n + i];
}

// The call's device status, published to mapped host memory so that a later
// call can read it without synchronising: counts of table overflows and of
// non-finite results, and the largest table seen (cells, list entries).
__global__ void publish_status_kernel(const unsigned* __restrict__ status, const TableGeom* __restrict__ geom,
                                      unsigned long long* __restrict__ dev, StatusRecord* host) {
  const unsigned st = *status;
  if (st & (kStatusTableCells | kStatusTableEntries | kStatusSegmentTooLong)) ++dev[1];
  if (st & kStatusNonFinite) ++dev[2];
  const unsigned long long c = (unsigned long long)geom->ncell, e = (unsigned long long)geom->total;
  if (c > dev[3]) dev[3] = c;
  if (e > dev[4]) dev[4] = e;
  ++dev[0];
  volatile StatusRecord* h = host;
  h->overflows = dev[1];
  h->nonfinite = dev[2];
  h->max_cells = dev[3];
  h->max_entries = dev[4];
  __threadfence_system();
  h->seq = dev[0];
}

__global__ void born_kernel(int n, int n_chunks, const float* __restrict__ J, double S4, double S7, double C4,
                            double C7, double alpha0, double alpha1, double* __restrict__ born,
                            float2* __restrict__ bornf, double* __restrict__ dBdJ, double* __restrict__ dBda,
                            double* __restrict__ integrals, unsigned* __restrict__ status) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double J4 = 0.0, J7 = 0.0;
  for (int c = 0; c < n_chunks; ++c) {
    J4 += (double)J[(size_t)c * n + i];
    J7 += (double)J[((size_t)n_chunks + c) * n + i];
  }
  // 1/r0 - I4 = C4 + J4 and 1/(4 r0^4) - I7 = C7 + J7 (CharmmReferenceGBSW.cpp:591-593)
  const double t4 = C4 + J4, t7 = C7 + J7;
  const double q7 = sqrt(sqrt(t7));
  const double inv = alpha0 * t4 + alpha1 * q7;
  const double B = 1.0 / inv;
  born[i] = B;
  bornf[i] = make_float2((float)B, (float)inv);
  const double B2 = B * B;
  dBdJ[2 * i] = -B2 * alpha0;
  dBdJ[2 * i + 1] = -B2 * alpha1 * 0.25 * q7 / t7;  // t7^(-3/4) = t7^(1/4) / t7
  dBda[2 * i] = -B2 * t4;
  dBda[2 * i + 1] = -B2 * q7;
  integrals[i] = S4 - J4;
  integrals[n + i] = S7 - J7;
  if (!isfinite(B) || !(B > 0.0)) atomicOr(status, kStatusNonFinite);
}

__global__ void chain_prep_kernel(int n, const unsigned long long* __restrict__ dEdB_fx,
                                  const double* __restrict__ dBdJ, const double* __restrict__ dBda,
                                  float2* __restrict__ dEdJ, double* __restrict__ alpha_terms) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double g = fixed_to_double(dEdB_fx[i]);
  dEdJ[i] = make_float2((float)(g * dBdJ[2 * i]), (float)(g * dBdJ[2 * i + 1]));
  if (alpha_terms) {
    alpha_terms[2 * i] = g * dBda[2 * i];
    alpha_terms[2 * i + 1] = g * dBda[2 * i + 1];
  }
}

constexpr int kRedThreads = 1024;

// One block; fixed reduction shape, so the result is bit-reproducible.
__global__ void __launch_bounds__(kRedThreads) energy_reduce_kernel(const double* __restrict__ parts, int nparts,
                                                                    const unsigned long long* __restrict__ energy_fx,
                                                                    double* __restrict__ energy,
                                                                    const double* __restrict__ alpha_terms, int n,
                                                                    double* __restrict__ alpha_grad) {
  __shared__ double s[3][kRedThreads];
  double e = 0, a0 = 0, a1 = 0;
  {
    // four independent chains (loads in flight), combined in a fixed order
    double e4[4] = {0, 0, 0, 0};
    int k = threadIdx.x;
    for (; k + 3 * kRedThreads < nparts; k += 4 * kRedThreads)
      for (int u = 0; u < 4; ++u) e4[u] += parts[k + u * kRedThreads];
    for (; k < nparts; k += kRedThreads) e4[0] += parts[k];
    e = (e4[0] + e4[1]) + (e4[2] + e4[3]);
  }
  if (alpha_terms)
    for (int k = threadIdx.x; k < n; k += kRedThreads) {
      a0 += alpha_terms[2 * k];
      a1 += alpha_terms[2 * k + 1];
    }
  s[0][threadIdx.x] = e;
  s[1][threadIdx.x] = a0;
  s[2][threadIdx.x] = a1;
  __syncthreads();
  for (int stride = kRedThreads / 2; stride > 0; stride >>= 1) {
    if (threadIdx.x < stride)
      for (int k = 0; k < 3; ++k) s[k][threadIdx.x] += s[k][threadIdx.x + stride];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    if (energy) *energy += s[0][0] + (energy_fx ? fixed_to_double(*energy_fx) : 0.0);
    if (alpha_grad) {
      alpha_grad[0] = s[1][0];
      alpha_grad[1] = s[2][0];
    }
  }
}

}  // namespace

gbx_status launch_stage_positions(Context* ctx, const void* posq) {
  const int n = ctx->n;
  const int* slot_of = ctx->in_permuted ? ctx->d_slot_of : nullptr;
  if (ctx->in_double)
    stage_positions_kernel<true><<<(n + 255) / 256, 256, 0, ctx->stream>>>(posq, n, slot_of, ctx->d_wpar, ctx->d_pos);
  else
    stage_positions_kernel<false><<<(n + 255) / 256, 256, 0, ctx->stream>>>(posq, n, slot_of, ctx->d_wpar, ctx->d_pos);
  ++ctx->launches;
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    ctx->last_error = std::string("stage launch: ") + cudaGetErrorString(e);
    return GBX_ERR_CUDA;
  }
  return GBX_OK;
}

gbx_status launch_finish_outputs(Context* ctx, unsigned long long* force, int stride, float* energy_float) {
  const int n = ctx->n;
  finish_outputs_kernel<<<(n + 255) / 256, 256, 0, ctx->stream>>>(
      n, ctx->in_permuted ? ctx->d_slot_of : nullptr, ctx->d_force_fx, force, stride, ctx->d_energy, energy_float);
  ++ctx->launches;
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    ctx->last_error = std::string("output launch: ") + cudaGetErrorString(e);
    return GBX_ERR_CUDA;
  }
  return GBX_OK;
}

gbx_status launch_publish_status(Context* ctx) {
  publish_status_kernel<<<1, 1, 0, ctx->stream>>>(ctx->d_status, ctx->use_tight ? ctx->d_tgeom : ctx->d_geom,
                                                  ctx->d_pub, ctx->h_pub_dev);
  ++ctx->launches;
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    ctx->last_error = std::string("status launch: ") + cudaGetErrorString(e);
    return GBX_ERR_CUDA;
  }
  return GBX_OK;
}

gbx_status launch_born(Context* ctx) {
  const int n = ctx->n;
  born_kernel<<<(n + 255) / 256, 256, 0, ctx->stream>>>(
      n, ctx->n_chunks, ctx->d_J, ctx->S4, ctx->S7, ctx->C4, ctx->C7, ctx->alpha0, ctx->alpha1, ctx->d_born,
      reinterpret_cast<float2*>(ctx->d_bornf), ctx->d_dBdJ, ctx->d_dBdJ + 2 * (size_t)n, ctx->d_integrals,
      ctx->d_status);
  ++ctx->launches;
  cudaMemsetAsync(ctx->d_dEdB_fx, 0, sizeof(unsigned long long) * n, ctx->stream);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    ctx->last_error = std::string("born launch: ") + cudaGetErrorString(e);
    return GBX_ERR_CUDA;
  }
  return GBX_OK;
}

gbx_status launch_chain_prep(Context* ctx, bool adjoint) {
  const int n = ctx->n;
  chain_prep_kernel<<<(n + 255) / 256, 256, 0, ctx->stream>>>(
      n, ctx->d_dEdB_fx, ctx->d_dBdJ, ctx->d_dBdJ + 2 * (size_t)n, ctx->d_dEdJ,
      adjoint ? ctx->d_dBdJ + 4 * (size_t)n : nullptr);
  ++ctx->launches;
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    ctx->last_error = std::string("chain prep launch: ") + cudaGetErrorString(e);
    return GBX_ERR_CUDA;
  }
  return GBX_OK;
}

// Device adjoint outputs: fixed-point sums to FP64, forces as [n][3].
__global__ void adjoint_out_kernel(int n, int stride, const unsigned long long* __restrict__ force_fx,
                                   const unsigned long long* __restrict__ dq_fx,
                                   const unsigned long long* __restrict__ dR_fx, const double* __restrict__ e_in,
                                   const double* __restrict__ a_in, double* __restrict__ forces,
                                   double* __restrict__ dEdq, double* __restrict__ dEdR, double* __restrict__ energy,
                                   double* __restrict__ dEdalpha) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i == 0) {
    if (energy) *energy = *e_in;
    if (dEdalpha) {
      dEdalpha[0] = a_in[0];
      dEdalpha[1] = a_in[1];
    }
  }
  if (i >= n) return;
  if (forces)
    for (int k = 0; k < 3; ++k) forces[3 * (size_t)i + k] = fixed_to_double(force_fx[(size_t)k * stride + i]);
  if (dEdq) dEdq[i] = fixed_to_double(dq_fx[i]);
  if (dEdR) dEdR[i] = fixed_to_double(dR_fx[i]);
}

gbx_status launch_adjoint_out(Context* ctx, double* energy, double* forces, double* dEdq, double* dEdR,
                              double* dEdalpha) {
  const int n = ctx->n;
  adjoint_out_kernel<<<(n + 255) / 256, 256, 0, ctx->stream>>>(n, n, ctx->d_force_fx, ctx->d_dEdq_fx, ctx->d_dEdR_fx,
                                                               ctx->d_energy, ctx->d_alpha_grad, forces, dEdq, dEdR,
                                                               energy, dEdalpha);
  ++ctx->launches;
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    ctx->last_error = std::string("adjoint output launch: ") + cudaGetErrorString(e);
    return GBX_ERR_CUDA;
  }
  return GBX_OK;
}

gbx_status launch_energy_reduce(Context* ctx, double* energy, bool adjoint) {
  energy_reduce_kernel<<<1, kRedThreads, 0, ctx->stream>>>(ctx->d_energy_part, ctx->energy_parts, ctx->d_energy_fx,
                                                           energy,
                                                           adjoint ? ctx->d_dBdJ + 4 * (size_t)ctx->n : nullptr,
                                                           ctx->n, adjoint ? ctx->d_alpha_grad : nullptr);
  ++ctx->launches;
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    ctx->last_error = std::string("energy reduce launch: ") + cudaGetErrorString(e);
    return GBX_ERR_CUDA;
  }
  return GBX_OK;
}

}  // namespace gbx
