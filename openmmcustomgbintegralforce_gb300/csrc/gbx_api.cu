// C-ABI entry points (include/gbx.h): context lifecycle, parameters, the
// execute pipeline and result queries.  No exception crosses this boundary.
#include <math.h>
#include <omp.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <cctype>
#include <cmath>
#include <new>
#include <string>
#include <vector>

#include "gbx_internal.cuh"
#include "lebedev_rules.h"

using gbx::Context;

namespace {

#define GBX_CUDA(call)                                                                   \
  do {                                                                                   \
    cudaError_t e_ = (call);                                                             \
    if (e_ != cudaSuccess) {                                                             \
      ctx->last_error = std::string(#call ": ") + cudaGetErrorString(e_);                \
      return e_ == cudaErrorMemoryAllocation ? GBX_ERR_OUT_OF_MEMORY : GBX_ERR_CUDA;     \
    }                                                                                    \
  } while (0)

#define GBX_TRY(expr)                 \
  do {                                \
    gbx_status s_ = (expr);           \
    if (s_ != GBX_OK) return s_;      \
  } while (0)

// Gauss-Legendre by Newton iteration on the Legendre recurrence (Numerical
// Recipes gauleg, the procedure CharmmQuadrature.h:47-75 follows, with the
// same operation order so the rule is bit-identical to the reference's).
void gauss_legendre(double x0, double x1, int n, std::vector<double>& x, std::vector<double>& w) {
  const double eps = 3.0e-14;
  const double pi = 3.14159265358979323846264338327950;
  x.assign(n, 0.0);
  w.assign(n, 0.0);
  const int m = (n + 1) / 2;
  const double xm = 0.5 * (x1 + x0), xl = 0.5 * (x1 - x0);
  for (int i = 1; i <= m; ++i) {
    double z = cos(pi * (i - 0.25) / (n + 0.5)), z1 = 0.0, pp = 0.0;
    bool first = true;
    while (first || fabs(z - z1) > eps) {
      first = false;
      double p1 = 1.0, p2 = 0.0, p3;
      for (int j = 1; j <= n; ++j) {
        p3 = p2;
        p2 = p1;
        p1 = ((2.0 * j - 1.0) * z * p2 - (j - 1.0) * p3) / j;
      }
      pp = n * (z * p1 - p2) / (z * z - 1.0);
      z1 = z;
      z = z1 - p1 / pp;
    }
    x[i - 1] = xm - xl * z;
    x[n - i] = xm + xl * z;
    w[i - 1] = 2.0 * xl / ((1.0 - z * z) * pp * pp);
    w[n - i] = w[i - 1];
  }
}

const double* lebedev_rule(int order) {
  for (int k = 0; k < gbx_lebedev::kNumRules; ++k)
    if (gbx_lebedev::kRules[k].order == order) return gbx_lebedev::kRules[k].xyzw;
  return nullptr;
}

// The lookup table's buffers are sized: a call can run unchecked (a host
// call then reads the status word with its results; a device call replays its
// CUDA graph).
bool tables_sized(const Context* ctx) {
  return ctx->use_tight ? ctx->tight_valid && ctx->tcell_cap > 0 && ctx->tentry_cap > 0
                        : ctx->cell_cap > 0 && ctx->entry_cap > 0;
}

void drop_graph(Context* ctx) {
  if (ctx->graph) cudaGraphExecDestroy(ctx->graph);
  if (ctx->host_graph) cudaGraphExecDestroy(ctx->host_graph);
  ctx->graph = ctx->host_graph = nullptr;
  ctx->graph_kernels = ctx->host_graph_kernels = 0;
  ctx->host_graph_forces = -1;
  ++ctx->epoch;
}

template <class T>
gbx_status dalloc(Context* ctx, T** p, size_t count) {
  drop_graph(ctx);  // a captured graph holds the old pointers
  if (*p) cudaFree(*p);
  *p = nullptr;
  if (count == 0) count = 1;
  GBX_CUDA(cudaMalloc((void**)p, sizeof(T) * count));
  return GBX_OK;
}

gbx_status validate_config(const gbx_config& c, std::string& why) {
  if (c.model < GBX_MODEL_GBSW || c.model > GBX_MODEL_GBMV2) return why = "unknown model", GBX_ERR_INVALID_ARGUMENT;
  if (c.table_mode < GBX_TABLE_STANDALONE || c.table_mode > GBX_TABLE_PERIODIC)
    return why = "unknown table mode", GBX_ERR_INVALID_ARGUMENT;
  if (c.n_radial < 1 || c.n_radial > 256) return why = "n_radial must be in [1, 256]", GBX_ERR_INVALID_ARGUMENT;
  if (!lebedev_rule(c.lebedev_order)) return why = "unsupported Lebedev order", GBX_ERR_INVALID_ARGUMENT;
  if (!(c.r0 > 0 && c.r1 > c.r0)) return why = "need 0 < r0 < r1", GBX_ERR_INVALID_ARGUMENT;
  if (!(c.grid_length > 0)) return why = "grid_length must be > 0", GBX_ERR_INVALID_ARGUMENT;
  if (!(c.table_buffer >= 0)) return why = "table_buffer must be >= 0", GBX_ERR_INVALID_ARGUMENT;
  if (c.model == GBX_MODEL_GBSW && !(c.switch_width > 0)) return why = "switch_width must be > 0", GBX_ERR_INVALID_ARGUMENT;
  if (c.table_mode == GBX_TABLE_PERIODIC)
    for (int k = 0; k < 3; ++k)
      if (!(c.box[k] > 0)) return why = "periodic table needs a positive box", GBX_ERR_INVALID_ARGUMENT;
  if (c.table_cap > gbx::kMaxSortSegment) return why = "table_cap too large", GBX_ERR_INVALID_ARGUMENT;
  for (int k = 0; k < 2; ++k)
    if (c.integral_orders[k] != 0 && c.integral_orders[k] < 2)
      return why = "integral orders must be >= 2", GBX_ERR_INVALID_ARGUMENT;
  if (c.periodic) {  // CutoffPeriodic (CharmmReferenceGBSW.cpp:147-159, CharmmReferenceGBMV.cpp:138-149)
    // the standalone GBSW table (wrapped query) or the box-sampled table of the integral classes
    if (c.table_mode == GBX_TABLE_GRID || (c.table_mode == GBX_TABLE_STANDALONE && c.model != GBX_MODEL_GBSW))
      return why = "CutoffPeriodic needs the standalone GBSW table or the box-sampled table", GBX_ERR_UNSUPPORTED;
    if (!(c.cutoff > 0)) return why = "CutoffPeriodic needs a cutoff", GBX_ERR_INVALID_ARGUMENT;
    for (int k = 0; k < 3; ++k)
      if (!(c.box[k] >= 2.0 * c.cutoff) || !isfinite(c.box[k]))
        return why = "each box edge must be at least twice the cutoff", GBX_ERR_INVALID_ARGUMENT;
  }
  return GBX_OK;
}

gbx_status upload_quadrature(Context* ctx) {
  const gbx_config& c = ctx->cfg;
  std::vector<double> xr, wr;
  gauss_legendre(c.r0, c.r1, c.n_radial, xr, wr);
  const double* leb = lebedev_rule(c.lebedev_order);
  const int nS = c.lebedev_order, Q = c.n_radial * nS;
  ctx->q_off.assign(3 * (size_t)Q, 0.0);
  ctx->q_rad.assign(Q, 0.0);
  ctx->q_w.assign(Q, 0.0);
  std::vector<float4> qv(Q);
  std::vector<float2> qw(Q);
  double S4 = 0.0, S7 = 0.0;
  for (int i = 0; i < c.n_radial; ++i)
    for (int j = 0; j < nS; ++j) {
      const int q = i * nS + j;
      const double r = xr[i];
      for (int k = 0; k < 3; ++k) ctx->q_off[3 * q + k] = r * leb[4 * j + k];
      ctx->q_rad[q] = r;
      ctx->q_w[q] = wr[i] * leb[4 * j + 3];
      // weights of the two integrals, w / r^(n-2) (GBSWIntegral.cpp:96,144); orders 4 and 7 unless
      // set (kept as the repeated products of the reference's 4 and 7: the same bits)
      const double w4 = c.integral_orders[0] > 0 && c.integral_orders[0] != 4
                            ? ctx->q_w[q] / std::pow(r, (double)(c.integral_orders[0] - 2))
                            : ctx->q_w[q] / (r * r);
      const double w7 = c.integral_orders[1] > 0 && c.integral_orders[1] != 7
                            ? ctx->q_w[q] / std::pow(r, (double)(c.integral_orders[1] - 2))
                            : ctx->q_w[q] / (r * r * r * r * r);
      S4 += w4;
      S7 += w7;
      qv[q] = make_float4((float)ctx->q_off[3 * q], (float)ctx->q_off[3 * q + 1], (float)ctx->q_off[3 * q + 2], (float)r);
      qw[q] = make_float2((float)w4, (float)w7);
    }
  ctx->S4 = S4;
  ctx->S7 = S7;
  const double r0 = c.r0;
  ctx->C4 = 1.0 / r0 - S4;
  ctx->C7 = 1.0 / (4.0 * r0 * r0 * r0 * r0) - S7;
  GBX_TRY(dalloc(ctx, &ctx->d_qv, Q));
  GBX_TRY(dalloc(ctx, &ctx->d_qw, Q));
  GBX_TRY(dalloc(ctx, &ctx->d_qoff, 3 * (size_t)Q));
  GBX_CUDA(cudaMemcpy(ctx->d_qv, qv.data(), sizeof(float4) * Q, cudaMemcpyHostToDevice));
  GBX_CUDA(cudaMemcpy(ctx->d_qw, qw.data(), sizeof(float2) * Q, cudaMemcpyHostToDevice));
  GBX_CUDA(cudaMemcpy(ctx->d_qoff, ctx->q_off.data(), sizeof(double) * 3 * Q, cudaMemcpyHostToDevice));
  return GBX_OK;
}

// The volume kernels run one warp per (atom, chunk of quadrature points)
// with lanes over points: enough warps for ~48 per SM on the device's SMs;
// chunks of at most 896 points while that keeps under ~400 warps per SM (a
// whole 32 x 110 atom per warp left the last waves ragged: buried and
// surface atoms differ several-fold in work; measured best at 4 chunks for
// 10,000 atoms and 2 for 50,000); >= 64 points (2 per lane) per chunk.
int choose_chunks(int n, int Q, int sms) {
  int c = (sms * 48 + n - 1) / n;
  c = std::max(c, std::min((Q + 895) / 896, (sms * 400 + n - 1) / n));
  c = std::max(1, std::min(c, std::max(1, Q / 64)));
  return c;
}

gbx_status alloc_atom_buffers(Context* ctx) {
  const int n = ctx->n;
  const int Q = ctx->cfg.n_radial * ctx->cfg.lebedev_order;
  ctx->n_chunks = choose_chunks(n, Q, ctx->sms);
  GBX_TRY(dalloc(ctx, &ctx->d_radius, n));
  GBX_TRY(dalloc(ctx, &ctx->d_charge, n));
  GBX_TRY(dalloc(ctx, &ctx->d_par, n));
  GBX_TRY(dalloc(ctx, &ctx->d_wpar, n));
  GBX_TRY(dalloc(ctx, &ctx->d_pos, n));
  GBX_TRY(dalloc(ctx, &ctx->d_reduce, gbx::table_geom_scratch_doubles(n)));
  GBX_TRY(dalloc(ctx, &ctx->d_J, 2 * (size_t)ctx->n_chunks * n));
  GBX_TRY(dalloc(ctx, &ctx->d_born, n));
  GBX_TRY(dalloc(ctx, &ctx->d_bornf, 2 * (size_t)n));
  GBX_TRY(dalloc(ctx, &ctx->d_dBdJ, 6 * (size_t)n));
  GBX_TRY(dalloc(ctx, &ctx->d_integrals, 2 * (size_t)n));
  GBX_TRY(dalloc(ctx, &ctx->d_dEdB_fx, n));
  GBX_TRY(dalloc(ctx, &ctx->d_dEdJ, n));
  ctx->energy_parts = 0;  // the pair kernels add the energy to d_energy_fx
  GBX_TRY(dalloc(ctx, &ctx->d_energy_part, 1));
  GBX_TRY(dalloc(ctx, &ctx->d_energy_fx, 1));
  GBX_TRY(dalloc(ctx, &ctx->d_tile_box, 2 * (((size_t)n + 31) / 32)));
  if (ctx->cfg.model != GBX_MODEL_GBSW) {
    GBX_TRY(dalloc(ctx, &ctx->d_pstate, (size_t)n * Q * (ctx->cfg.model == GBX_MODEL_GBMV1 ? 1 : 5)));
    GBX_TRY(dalloc(ctx, &ctx->d_pcell, (size_t)n * Q));
    GBX_TRY(dalloc(ctx, &ctx->d_prank, (size_t)n * Q));
    GBX_TRY(dalloc(ctx, &ctx->d_porder, (size_t)n * Q));
    GBX_TRY(dalloc(ctx, &ctx->d_sval, (size_t)n * Q));
    GBX_TRY(dalloc(ctx, &ctx->d_pgeom, 1));
  }
  if (ctx->cfg.cutoff > 0) {
    GBX_TRY(dalloc(ctx, &ctx->d_perm, n));
    GBX_TRY(dalloc(ctx, &ctx->d_perm_tmp, n));
    GBX_TRY(dalloc(ctx, &ctx->d_cell_of, n));
    GBX_TRY(dalloc(ctx, &ctx->d_scount, gbx::kMaxSortCells));
    GBX_TRY(dalloc(ctx, &ctx->d_sstart, gbx::kMaxSortCells));
    GBX_TRY(dalloc(ctx, &ctx->d_scursor, gbx::kMaxSortCells));
    GBX_TRY(dalloc(ctx, &ctx->d_sgeom, 2));
  }
  GBX_TRY(dalloc(ctx, &ctx->d_force_fx, 3 * (size_t)n));
  GBX_TRY(dalloc(ctx, &ctx->d_energy, 1));
  GBX_TRY(dalloc(ctx, &ctx->d_dEdR_fx, n));
  GBX_TRY(dalloc(ctx, &ctx->d_dEdq_fx, n));
  GBX_TRY(dalloc(ctx, &ctx->d_alpha_grad, 2));
  GBX_TRY(dalloc(ctx, &ctx->d_status, 1));
  GBX_TRY(dalloc(ctx, &ctx->d_work, 4));
  GBX_TRY(dalloc(ctx, &ctx->d_rmax, 1));
  GBX_TRY(dalloc(ctx, &ctx->d_next_item, 1));
  GBX_TRY(dalloc(ctx, &ctx->d_geom, 1));
  GBX_TRY(dalloc(ctx, &ctx->d_tgeom, 1));
  GBX_TRY(dalloc(ctx, &ctx->d_wgeom, 1));
  GBX_CUDA(cudaMemset(ctx->d_status, 0, sizeof(unsigned)));
  GBX_CUDA(cudaMemset(ctx->d_work, 0, sizeof(unsigned long long) * 4));
  GBX_CUDA(cudaMallocHost((void**)&ctx->h_pos, sizeof(float4) * n));
  GBX_CUDA(cudaMallocHost((void**)&ctx->h_force_fx, sizeof(unsigned long long) * 3 * n));
  GBX_CUDA(cudaMallocHost((void**)&ctx->h_rmax, sizeof(unsigned)));
  *ctx->h_rmax = 0;
  GBX_CUDA(cudaMallocHost((void**)&ctx->h_status, sizeof(unsigned)));
  GBX_CUDA(cudaMallocHost((void**)&ctx->h_energy, sizeof(double)));
  GBX_CUDA(cudaEventCreateWithFlags(&ctx->srec_ev, cudaEventDisableTiming));
  GBX_TRY(dalloc(ctx, &ctx->d_pub, 5));
  GBX_CUDA(cudaMemset(ctx->d_pub, 0, sizeof(unsigned long long) * 5));
  GBX_CUDA(cudaHostAlloc((void**)&ctx->h_pub, sizeof(gbx::StatusRecord), cudaHostAllocMapped));
  memset(ctx->h_pub, 0, sizeof(gbx::StatusRecord));
  GBX_CUDA(cudaHostGetDevicePointer((void**)&ctx->h_pub_dev, ctx->h_pub, 0));
  return GBX_OK;
}

// (Re)allocates the chain-record buffer for R records per warp, within half
// of the free device memory; on failure the context runs without records.
gbx_status alloc_records(Context* ctx, int R) {
  drop_graph(ctx);  // a captured graph holds the old pointers
  if (ctx->d_srec) {
    GBX_CUDA(cudaStreamSynchronize(ctx->stream));
    cudaFree(ctx->d_srec);
    cudaFree(ctx->d_srec_st);
  }
  ctx->d_srec = nullptr;
  ctx->d_srec_st = nullptr;
  ctx->srec_R = 0;
  const long long warps = (long long)ctx->n * ctx->n_chunks;
  if (R <= 0) return GBX_OK;
  if (warps != ctx->srec_warps || !ctx->d_rcount) {
    GBX_TRY(dalloc(ctx, &ctx->d_rcount, (size_t)warps));
    ctx->srec_warps = warps;
  }
  size_t free_b = 0, total_b = 0;
  GBX_CUDA(cudaMemGetInfo(&free_b, &total_b));
  const long long fit = (long long)(free_b / 2 / (sizeof(int4) + sizeof(int))) / warps;
  if ((long long)R > fit) R = (int)(fit / 32 * 32);
  if (R <= 0 || cudaMalloc((void**)&ctx->d_srec, sizeof(int4) * (size_t)warps * R) != cudaSuccess ||
      cudaMalloc((void**)&ctx->d_srec_st, sizeof(int) * (size_t)warps * R) != cudaSuccess) {
    (void)cudaGetLastError();
    if (ctx->d_srec) cudaFree(ctx->d_srec);
    ctx->d_srec = nullptr;
    ctx->d_srec_st = nullptr;
    ctx->srec_auto = false;
    return GBX_OK;
  }
  ctx->srec_R = R;
  return GBX_OK;
}

// Decides whether this call records the GBSW chain rule's work and sizes the
// per-warp regions from the largest need the device reported (read without
// blocking; first guess half a warp's points).  Warps whose records do not
// fit walk their lists in the chain rule instead, with the same result.
gbx_status prepare_records(Context* ctx, bool wanted) {
  ctx->records = false;
  if (!wanted || ctx->cfg.model != GBX_MODEL_GBSW) return GBX_OK;
  const long long warps = (long long)ctx->n * ctx->n_chunks;
  if (ctx->srec_auto) {
    long long need = 0;
    if (ctx->srec_pending) {
      const cudaError_t q = cudaEventQuery(ctx->srec_ev);
      if (q == cudaSuccess) {
        ctx->srec_pending = false;
        const long long seen = *ctx->h_rmax;
        if (seen > ctx->srec_R) need = seen + seen / 8 + 32;
      } else if (q == cudaErrorNotReady) {
        (void)cudaGetLastError();
      } else {
        GBX_CUDA(q);
      }
    }
    if ((ctx->srec_R == 0 || warps != ctx->srec_warps) && need == 0 && !ctx->srec_pending) {
      const long long points = ((long long)ctx->q_w.size() + ctx->n_chunks - 1) / ctx->n_chunks;
      need = points / 2 + 32;
    }
    if (need > 0x40000000LL) need = 0x40000000LL;
    if (need > ctx->srec_R || (need > 0 && warps != ctx->srec_warps))
      GBX_TRY(alloc_records(ctx, (int)((need + 31) / 32 * 32)));
  }
  if (ctx->srec_R == 0 || warps != ctx->srec_warps) return GBX_OK;
  ctx->records = true;
  GBX_CUDA(cudaMemsetAsync(ctx->d_rmax, 0, sizeof(unsigned), ctx->stream));
  return GBX_OK;
}

gbx_status grow_table(Context* ctx, long long cells, long long entries) {
  if (cells > ctx->cell_cap) {
    const long long cap = cells + cells / 4 + 1024;
    GBX_TRY(dalloc(ctx, &ctx->d_cell_count, cap));
    GBX_TRY(dalloc(ctx, &ctx->d_cell_start, cap + 1));
    GBX_TRY(dalloc(ctx, &ctx->d_cell_cursor, cap));
    GBX_TRY(dalloc(ctx, &ctx->d_cell2, cap));
    GBX_TRY(dalloc(ctx, &ctx->d_block_sums, cap / (1024 * 8) + 2));
    if (ctx->cfg.model != GBX_MODEL_GBSW) {
      GBX_TRY(dalloc(ctx, &ctx->d_pcount, cap));
      GBX_TRY(dalloc(ctx, &ctx->d_pstart, cap + 1));
      GBX_TRY(dalloc(ctx, &ctx->d_pblock_sums, cap / (1024 * 8) + 2));
    }
    ctx->cell_cap = cap;
  }
  if (entries > ctx->entry_cap) {
    const long long cap = entries + entries / 4 + 4096;
    if (cap > 0x7fffffffLL) {
      ctx->last_error = "lookup table would exceed 2^31 entries";
      return GBX_ERR_TABLE_TOO_LARGE;
    }
    GBX_TRY(dalloc(ctx, &ctx->d_entries, cap));
    GBX_TRY(dalloc(ctx, &ctx->d_entry4, cap));
    GBX_TRY(dalloc(ctx, &ctx->d_entry_par, cap));
    ctx->entry_cap = cap;
  }
  return GBX_OK;
}

// Build the table; on a capacity miss read the needed sizes back, grow and
// rebuild.  Synchronises the stream when `check` is set.
gbx_status build_table_checked(Context* ctx, bool check) {
  for (int attempt = 0; attempt < 3; ++attempt) {
    GBX_CUDA(cudaMemsetAsync(ctx->d_status, 0, sizeof(unsigned), ctx->stream));
    GBX_TRY(gbx::launch_table_build(ctx, ctx->d_pos));
    if (!check && ctx->cell_cap > 0 && ctx->entry_cap > 0) {
      ctx->table_valid = true;
      return GBX_OK;
    }
    unsigned st = 0;
    gbx::TableGeom g;
    GBX_CUDA(cudaMemcpyAsync(&st, ctx->d_status, sizeof(unsigned), cudaMemcpyDeviceToHost, ctx->stream));
    GBX_CUDA(cudaMemcpyAsync(&g, ctx->d_geom, sizeof(g), cudaMemcpyDeviceToHost, ctx->stream));
    GBX_CUDA(cudaStreamSynchronize(ctx->stream));
    if (st & gbx::kStatusSegmentTooLong) {
      ctx->last_error = "a lookup-table cell holds more atoms than the sort supports";
      return GBX_ERR_TABLE_TOO_LARGE;
    }
    const bool cells_short = (st & gbx::kStatusTableCells) != 0;
    const bool entries_short = (st & gbx::kStatusTableEntries) != 0;
    if (!cells_short && !entries_short) {
      ctx->table_valid = true;
      return GBX_OK;
    }
    if (cells_short && g.ncell <= 1) {
      ctx->last_error = "lookup table dimension is too large, check atom positions";
      return GBX_ERR_TABLE_TOO_LARGE;
    }
    if (g.ncell > (long long)1 << 31) {
      ctx->last_error = "lookup grid would exceed 2^31 cells";
      return GBX_ERR_TABLE_TOO_LARGE;
    }
    // the entry count is only known once the cell array was large enough
    long long entries = cells_short ? (long long)ctx->n * 64 : g.total;
    GBX_TRY(grow_table(ctx, g.ncell, std::max(entries, (long long)ctx->n)));
  }
  ctx->last_error = "lookup table did not fit after resizing";
  return GBX_ERR_TABLE_TOO_LARGE;
}

gbx_status grow_tight(Context* ctx, long long cells, long long entries) {
  if (cells > ctx->tcell_cap) {
    const long long cap = cells + cells / 4 + 1024;
    GBX_TRY(dalloc(ctx, &ctx->d_tcount, cap));
    GBX_TRY(dalloc(ctx, &ctx->d_tstart, cap + 1));
    GBX_TRY(dalloc(ctx, &ctx->d_tcursor, cap));
    GBX_TRY(dalloc(ctx, &ctx->d_tburied, cap));
    GBX_TRY(dalloc(ctx, &ctx->d_tcell, cap));
    GBX_TRY(dalloc(ctx, &ctx->d_tfirst, cap));
    GBX_TRY(dalloc(ctx, &ctx->d_tblock_sums, cap / (1024 * 8) + 2));
    ctx->tcell_cap = cap;
  }
  if (entries > ctx->tentry_cap) {
    const long long cap = entries + entries / 4 + 4096;
    if (cap > 0x7fffffffLL) {
      ctx->last_error = "exact table would exceed 2^31 entries";
      return GBX_ERR_TABLE_TOO_LARGE;
    }
    GBX_TRY(dalloc(ctx, &ctx->d_tentry, cap));
    GBX_TRY(dalloc(ctx, &ctx->d_tindex, cap));
    ctx->tentry_cap = cap;
  }
  return GBX_OK;
}

// Exact-table counterpart of build_table_checked.
gbx_status build_tight_checked(Context* ctx, bool check) {
  for (int attempt = 0; attempt < 3; ++attempt) {
    GBX_CUDA(cudaMemsetAsync(ctx->d_status, 0, sizeof(unsigned), ctx->stream));
    GBX_TRY(gbx::launch_tight_build(ctx, ctx->d_pos));
    if (!check && ctx->tcell_cap > 0 && ctx->tentry_cap > 0) return GBX_OK;
    unsigned st = 0;
    gbx::TableGeom g;
    GBX_CUDA(cudaMemcpyAsync(&st, ctx->d_status, sizeof(unsigned), cudaMemcpyDeviceToHost, ctx->stream));
    GBX_CUDA(cudaMemcpyAsync(&g, ctx->d_tgeom, sizeof(g), cudaMemcpyDeviceToHost, ctx->stream));
    GBX_CUDA(cudaStreamSynchronize(ctx->stream));
    if (st & gbx::kStatusSegmentTooLong) {
      ctx->last_error = "an exact-table cell holds more atoms than the sort supports";
      return GBX_ERR_TABLE_TOO_LARGE;
    }
    const bool cells_short = (st & gbx::kStatusTableCells) != 0;
    const bool entries_short = (st & gbx::kStatusTableEntries) != 0;
    if (!cells_short && !entries_short) {
      ctx->tight_valid = true;
      return GBX_OK;
    }
    if (cells_short && (g.ncell <= ctx->tcell_cap || g.ncell > ((long long)1 << 31))) {
      ctx->last_error = "exact table geometry out of range, check atom positions";
      return GBX_ERR_TABLE_TOO_LARGE;
    }
    long long entries = cells_short ? (long long)ctx->n * 128 : g.total;
    GBX_TRY(grow_tight(ctx, g.ncell, std::max(entries, (long long)ctx->n)));
  }
  ctx->last_error = "exact table did not fit after resizing";
  return GBX_ERR_TABLE_TOO_LARGE;
}

gbx_status run_pipeline(Context* ctx, const float4* posq, unsigned long long* force, int stride, double* energy,
                        bool check, bool adjoint, bool count_work, bool forces = true) {
  int stage = 0;
  auto mark = [&]() -> gbx_status {
    if (ctx->timing) GBX_CUDA(cudaEventRecord(ctx->ev[stage], ctx->stream));
    ++stage;
    return GBX_OK;
  };
  GBX_TRY(mark());
  GBX_TRY(gbx::launch_stage_positions(ctx, posq));
  GBX_TRY(mark());
  ctx->table_valid = false;
  if (ctx->use_tight) GBX_TRY(build_tight_checked(ctx, check || !ctx->tight_valid));
  else GBX_TRY(build_table_checked(ctx, check));
  if (count_work) GBX_CUDA(cudaMemsetAsync(ctx->d_work, 0, sizeof(unsigned long long) * 4, ctx->stream));
  const bool chain = forces || adjoint;
  GBX_TRY(prepare_records(ctx, chain && !adjoint && !count_work));
  GBX_TRY(mark());
  GBX_TRY(gbx::launch_binning(ctx, ctx->d_pos, count_work));
  GBX_TRY(mark());
  GBX_TRY(gbx::launch_integrals(ctx, ctx->d_pos, count_work));
  GBX_TRY(mark());
  if (ctx->custom) {
    // expressions outside the canonical set: values, single and pair terms, dE/dJ
    GBX_TRY(mark());
    GBX_TRY(gbx::launch_custom_energy(ctx, ctx->d_pos, force, stride));
    GBX_TRY(mark());
    GBX_TRY(gbx::launch_custom_chain_prep(ctx, force, stride));
    GBX_TRY(mark());
    if (chain) GBX_TRY(gbx::launch_chain(ctx, ctx->d_pos, force, stride, false));
    GBX_TRY(mark());
    GBX_TRY(gbx::launch_energy_reduce(ctx, energy, false));
    GBX_TRY(mark());
    GBX_TRY(gbx::launch_publish_status(ctx));
    ctx->have_result = true;
    if (check) {
      unsigned st = 0;
      GBX_CUDA(cudaMemcpyAsync(&st, ctx->d_status, sizeof(unsigned), cudaMemcpyDeviceToHost, ctx->stream));
      GBX_CUDA(cudaStreamSynchronize(ctx->stream));
      if (st & gbx::kStatusNonFinite) {
        ctx->last_error = "non-finite computed value";
        return GBX_ERR_NONFINITE;
      }
    }
    return GBX_OK;
  }
  GBX_TRY(gbx::launch_born(ctx));
  if (adjoint) {
    GBX_CUDA(cudaMemsetAsync(ctx->d_dEdq_fx, 0, sizeof(unsigned long long) * ctx->n, ctx->stream));
    GBX_CUDA(cudaMemsetAsync(ctx->d_dEdR_fx, 0, sizeof(unsigned long long) * ctx->n, ctx->stream));
  }
  GBX_TRY(mark());
  GBX_TRY(gbx::launch_pair(ctx, ctx->d_pos, force, stride, adjoint));
  GBX_TRY(mark());
  GBX_TRY(gbx::launch_chain_prep(ctx, adjoint));
  GBX_TRY(mark());
  if (chain) GBX_TRY(gbx::launch_chain(ctx, ctx->d_pos, force, stride, adjoint));
  if (ctx->records && ctx->srec_auto && !ctx->srec_pending) {
    GBX_CUDA(cudaMemcpyAsync(ctx->h_rmax, ctx->d_rmax, sizeof(unsigned), cudaMemcpyDeviceToHost, ctx->stream));
    GBX_CUDA(cudaEventRecord(ctx->srec_ev, ctx->stream));
    ctx->srec_pending = true;
  }
  GBX_TRY(mark());
  GBX_TRY(gbx::launch_energy_reduce(ctx, energy, adjoint));
  GBX_TRY(mark());
  GBX_TRY(gbx::launch_publish_status(ctx));
  ctx->have_result = true;
  if (check) {
    unsigned st = 0;
    GBX_CUDA(cudaMemcpyAsync(&st, ctx->d_status, sizeof(unsigned), cudaMemcpyDeviceToHost, ctx->stream));
    GBX_CUDA(cudaStreamSynchronize(ctx->stream));
    if (st & gbx::kStatusNonFinite) {
      ctx->last_error = "non-finite Born radius";
      return GBX_ERR_NONFINITE;
    }
  }
  return GBX_OK;
}

void set_model_params(Context* ctx, std::vector<float>& wpar, std::vector<float2>& par) {
  const gbx_config& c = ctx->cfg;
  const int n = ctx->n;
  wpar.resize(n);
  par.resize(n);
  for (int i = 0; i < n; ++i) {
    const double R = ctx->radius[i];
    if (c.model == GBX_MODEL_GBSW) {
      wpar[i] = (float)((R + 0.03) * 0.9520);  // CharmmReferenceGBSW.cpp:625
      par[i] = make_float2((float)R, 0.0f);
    } else if (c.model == GBX_MODEL_GBMV1) {
      wpar[i] = (float)(c.gamma0 * log(c.lambda) / (R * R * R * R));  // GBMVIntegralTypeI.cpp:168
      par[i] = make_float2((float)R, 0.0f);
    } else {
      const double C = c.p1 * R * 10 + c.p2;  // GBMVIntegralTypeII.cpp:179
      wpar[i] = (float)C;
      par[i] = make_float2((float)(C - 100.0 * R * R), (float)R);
    }
  }
}

// Reads the status the device published for earlier unchecked calls (no
// synchronisation).  A call whose lookup table outgrew its buffers ran
// without the volume terms: *stale tells the caller to run this call checked
// (which grows the buffers) and report it.  Buffers are also grown ahead of
// need once the largest table seen reaches 90 % of them.
gbx_status poll_status(Context* ctx, bool* stale, bool* nonfinite) {
  *stale = *nonfinite = false;
  if (!ctx->h_pub) return GBX_OK;
  const volatile gbx::StatusRecord* r = ctx->h_pub;
  const unsigned long long ov = r->overflows, nf = r->nonfinite, mc = r->max_cells, me = r->max_entries;
  if (ov > ctx->pub_seen_overflows) {
    ctx->pub_seen_overflows = ov;
    *stale = true;
  }
  if (nf > ctx->pub_seen_nonfinite) {
    ctx->pub_seen_nonfinite = nf;
    *nonfinite = true;
  }
  if (!tables_sized(ctx)) return GBX_OK;
  const long long cap = ctx->use_tight ? ctx->tcell_cap : ctx->cell_cap;
  const long long ecap = ctx->use_tight ? ctx->tentry_cap : ctx->entry_cap;
  const long long want_c = (long long)(mc + mc / 9 + 1), want_e = (long long)(me + me / 9 + 1);
  if ((mc > 0 && want_c > cap) || (me > 0 && want_e > ecap)) {
    if (want_c > ((long long)1 << 31) || want_e > 0x7fffffffLL) return GBX_OK;  // a checked call reports it
    GBX_CUDA(cudaStreamSynchronize(ctx->stream));
    if (ctx->use_tight) GBX_TRY(grow_tight(ctx, std::max(want_c, cap), std::max(want_e, ecap)));
    else GBX_TRY(grow_table(ctx, std::max(want_c, cap), std::max(want_e, ecap)));
  }
  return GBX_OK;
}

}  // namespace

namespace gbx {
gbx_status pipeline(Context* ctx, const float4* posq, unsigned long long* force, int stride, double* energy, bool check,
                    bool adjoint, bool count_work, bool forces) {
  return run_pipeline(ctx, posq, force, stride, energy, check, adjoint, count_work, forces);
}

gbx_status set_chunks(Context* ctx, int chunks) {
  const int Q = ctx->cfg.n_radial * ctx->cfg.lebedev_order;
  chunks = std::max(1, std::min(chunks, std::max(1, Q / 32)));
  if (chunks == ctx->n_chunks) return GBX_OK;
  GBX_CUDA(cudaDeviceSynchronize());
  ctx->n_chunks = chunks;
  GBX_TRY(dalloc(ctx, &ctx->d_J, 2 * (size_t)chunks * ctx->n));
  ctx->srec_pending = false;
  ctx->srec_auto = true;  // record regions are per warp: sized again by the next call
  return alloc_records(ctx, 0);
}

gbx_status fix_chain_records(Context* ctx) {
  // freeze the record regions at the largest need seen so far (no further
  // event queries: the call sequence can be captured in a CUDA graph); a
  // size the caller fixed (or an earlier freeze) stands
  if (!ctx->srec_auto) return GBX_OK;
  if (ctx->srec_pending) {
    GBX_CUDA(cudaEventSynchronize(ctx->srec_ev));
    ctx->srec_pending = false;
  }
  const long long seen = ctx->h_rmax ? *ctx->h_rmax : 0;
  ctx->srec_auto = false;
  if (ctx->cfg.model != GBX_MODEL_GBSW) return alloc_records(ctx, 0);
  const int want = (int)((seen + seen / 4 + 64 + 31) / 32 * 32);
  if (ctx->srec_R >= want && ctx->srec_R > 0) return GBX_OK;
  return alloc_records(ctx, want);
}

void choose_table(Context* ctx) {
  const gbx_config& c = ctx->cfg;
  bool tight = ctx->tight_eligible;
  if (tight && c.periodic) {
    // the standalone grid lists atoms out to its pad from a cell's grid point
    // (CharmmReferenceGBSW.cpp:454-455), so up to the pad plus a cell
    // diagonal from a point; the exact table at the moved point equals the
    // reference only while that is below half of every box edge, where the
    // minimum image of every listed atom is the atom itself
    double rmax = 0.0;
    for (double r : ctx->radius) rmax = std::max(rmax, r);
    const double reach = c.table_buffer + (rmax + 0.03) + c.switch_width + 1.5 * sqrt(3.0) * c.grid_length + 1e-3;
    tight = reach < 0.5 * std::min(c.box[0], std::min(c.box[1], c.box[2]));
  }
  if (tight == ctx->use_tight) return;
  drop_graph(ctx);
  ctx->use_tight = tight;
  ctx->tight_valid = false;
  ctx->table_valid = false;
}
}  // namespace gbx

extern "C" {

const char* gbx_status_string(gbx_status s) {
  switch (s) {
    case GBX_OK: return "ok";
    case GBX_ERR_INVALID_ARGUMENT: return "invalid argument";
    case GBX_ERR_CUDA: return "CUDA error";
    case GBX_ERR_OUT_OF_MEMORY: return "out of device memory";
    case GBX_ERR_UNSUPPORTED: return "unsupported";
    case GBX_ERR_NONFINITE: return "non-finite result";
    case GBX_ERR_TABLE_TOO_LARGE: return "lookup table too large";
    case GBX_ERR_NOT_READY: return "no result yet";
    case GBX_ERR_TIMEOUT: return "device wait timed out";
    case GBX_ERR_EXCEEDS_STATIC_SCRATCH: return "more atoms than the static scratch of gbx_pair_noalloc holds (65536)";
    case GBX_ERR_STALE_RESULT: return "an earlier unchecked call lacked the volume terms (its lookup table outgrew its buffers)";
  }
  return "unknown status";
}

int gbx_version(void) { return 10000; }

gbx_status gbx_config_preset(int preset, gbx_config* cfg) {
  if (!cfg) return GBX_ERR_INVALID_ARGUMENT;
  memset(cfg, 0, sizeof(*cfg));
  cfg->n_radial = 24;
  cfg->r0 = 0.05;   // CharmmReferenceGBSW.cpp:27-28, GBSWIntegral.cpp:31-34
  cfg->r1 = 2.0;
  cfg->grid_length = 0.15;
  cfg->switch_width = 0.03;
  cfg->gamma0 = 0.44;
  cfg->alpha0 = -0.180;  // CharmmReferenceGBSW.cpp:559-560
  cfg->alpha1 = 1.817;
  cfg->prefactor = -138.935456 * (1.0 - 1.0 / 80.0);  // CharmmReferenceGBSW.cpp:177-178
  cfg->cutoff = 0.0;
  cfg->skip_empty = 1;
  cfg->box[0] = cfg->box[1] = cfg->box[2] = 10.0;
  switch (preset) {
    case GBX_PRESET_CHARMM_GBSW:
      cfg->model = GBX_MODEL_GBSW;
      cfg->lebedev_order = 38;
      cfg->table_mode = GBX_TABLE_STANDALONE;
      cfg->table_buffer = 0.20;  // CharmmReferenceGBSW.cpp:47
      cfg->table_cap = 0;
      cfg->cutoff_chain_quirk = 1;
      return GBX_OK;
    case GBX_PRESET_GBSW_INTEGRAL:
      cfg->model = GBX_MODEL_GBSW;
      cfg->lebedev_order = 26;
      cfg->table_mode = GBX_TABLE_GRID;
      cfg->table_buffer = 0.04;  // GBSWIntegral.cpp:60
      cfg->table_cap = 64;       // CustomGBIntegral.cpp:15
      return GBX_OK;
    case GBX_PRESET_GBMV1:
      cfg->model = GBX_MODEL_GBMV1;
      cfg->lebedev_order = 26;
      cfg->table_mode = GBX_TABLE_PERIODIC;
      cfg->table_buffer = 0.21;  // GBMVIntegralTypeI.cpp:56
      cfg->table_cap = 64;
      cfg->beta = -100;  // GBMVIntegralTypeI.cpp:22-24
      cfg->lambda = 0.1;
      cfg->skip_empty = 0;
      return GBX_OK;
    case GBX_PRESET_GBMV2:
      cfg->model = GBX_MODEL_GBMV2;
      cfg->lebedev_order = 26;
      cfg->table_mode = GBX_TABLE_PERIODIC;
      cfg->table_buffer = 0.21;
      cfg->table_cap = 64;
      cfg->beta = -20;  // GBMVIntegralTypeII.cpp:23-28
      cfg->lambda = 0.5;
      cfg->p1 = 0.45;
      cfg->p2 = 1.25;
      cfg->s0 = 0.7;
      cfg->skip_empty = 0;
      return GBX_OK;
  }
  return GBX_ERR_INVALID_ARGUMENT;
}

gbx_status gbx_create(const gbx_config* cfg, int num_atoms, gbx_context** out) {
  if (!cfg || !out || num_atoms < 1) return GBX_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  std::string why;
  gbx_status s = validate_config(*cfg, why);
  if (s != GBX_OK) return s;
  Context* ctx = new (std::nothrow) Context();
  if (!ctx) return GBX_ERR_OUT_OF_MEMORY;
  ctx->cfg = *cfg;
  ctx->n = num_atoms;
  ctx->alpha0 = (float)cfg->alpha0;
  ctx->alpha1 = (float)cfg->alpha1;
  if (cudaGetDevice(&ctx->device) != cudaSuccess ||
      cudaDeviceGetAttribute(&ctx->sms, cudaDevAttrMultiProcessorCount, ctx->device) != cudaSuccess ||
      ctx->sms < 1) {
    delete ctx;
    return GBX_ERR_CUDA;
  }
  // the exact table serves GBSW on a standalone table; a periodic system
  // only while the box is wide enough for its parameters (choose_table)
  ctx->tight_eligible = cfg->model == GBX_MODEL_GBSW && cfg->table_mode == GBX_TABLE_STANDALONE &&
                        cfg->table_policy == GBX_TABLE_POLICY_AUTO;
  ctx->use_tight = ctx->tight_eligible && !cfg->periodic;
  ctx->tight_h = cfg->tight_grid_length > 0 ? cfg->tight_grid_length : 0.1;
  s = upload_quadrature(ctx);
  if (s == GBX_OK) s = alloc_atom_buffers(ctx);
  if (s == GBX_OK && cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamNonBlocking) != cudaSuccess)
    s = GBX_ERR_CUDA;
  ctx->stream = ctx->own_stream;
  if (s != GBX_OK) {
    gbx_destroy(reinterpret_cast<gbx_context*>(ctx));
    return s;
  }
  // neutral defaults: zero charge, 0.15 nm radius
  ctx->charge.assign(num_atoms, 0.0);
  ctx->radius.assign(num_atoms, 0.15);
  s = gbx_set_particle_parameters(reinterpret_cast<gbx_context*>(ctx), ctx->charge.data(), ctx->radius.data());
  if (s != GBX_OK) {
    gbx_destroy(reinterpret_cast<gbx_context*>(ctx));
    return s;
  }
  *out = reinterpret_cast<gbx_context*>(ctx);
  return GBX_OK;
}

gbx_status gbx_destroy(gbx_context* handle) {
  Context* ctx = reinterpret_cast<Context*>(handle);
  if (!ctx) return GBX_ERR_INVALID_ARGUMENT;
  drop_graph(ctx);
  gbx::custom_destroy(ctx);
  void* ptrs[] = {ctx->d_qv, ctx->d_qw, ctx->d_qoff, ctx->d_radius, ctx->d_charge, ctx->d_par, ctx->d_wpar,
                  ctx->d_geom, ctx->d_cell_count, ctx->d_cell_start, ctx->d_cell_cursor, ctx->d_entries,
                  ctx->d_block_sums, ctx->d_reduce, ctx->d_pos, ctx->d_J, ctx->d_born, ctx->d_bornf, ctx->d_dBdJ,
                  ctx->d_integrals, ctx->d_dEdB_fx, ctx->d_dEdJ, ctx->d_energy_part, ctx->d_force_fx,
                  ctx->d_energy, ctx->d_dEdR_fx, ctx->d_dEdq_fx, ctx->d_alpha_grad, ctx->d_status, ctx->d_work,
                  ctx->d_tgeom, ctx->d_wgeom, ctx->d_tcount, ctx->d_tstart, ctx->d_tcursor, ctx->d_tburied,
                  ctx->d_tblock_sums, ctx->d_tentry, ctx->d_tindex, ctx->d_entry4, ctx->d_entry_par,
                  ctx->d_cell2, ctx->d_tcell, ctx->d_tfirst, ctx->d_srec, ctx->d_srec_st, ctx->d_rcount, ctx->d_rmax, ctx->d_next_item, ctx->d_energy_fx, ctx->d_tile_box, ctx->d_perm,
                  ctx->d_perm_tmp, ctx->d_cell_of, ctx->d_scount, ctx->d_sstart, ctx->d_scursor, ctx->d_sgeom, ctx->d_pstate,
                  ctx->d_pcell, ctx->d_prank, ctx->d_porder, ctx->d_sval, ctx->d_pcount, ctx->d_pstart,
                  ctx->d_pblock_sums, ctx->d_pgeom, ctx->d_slot_of, ctx->d_pub};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  for (int k = 0; k <= Context::kStages; ++k)
    if (ctx->ev[k]) cudaEventDestroy(ctx->ev[k]);
  if (ctx->h_pos) cudaFreeHost(ctx->h_pos);
  if (ctx->h_force_fx) cudaFreeHost(ctx->h_force_fx);
  if (ctx->h_rmax) cudaFreeHost(ctx->h_rmax);
  if (ctx->h_status) cudaFreeHost(ctx->h_status);
  if (ctx->h_energy) cudaFreeHost(ctx->h_energy);
  if (ctx->h_pub) cudaFreeHost(ctx->h_pub);
  if (ctx->srec_ev) cudaEventDestroy(ctx->srec_ev);
  if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
  delete ctx;
  return GBX_OK;
}

gbx_status gbx_last_error(const gbx_context* handle, char* buf, size_t len) {
  const Context* ctx = reinterpret_cast<const Context*>(handle);
  if (!ctx || !buf || len == 0) return GBX_ERR_INVALID_ARGUMENT;
  strncpy(buf, ctx->last_error.c_str(), len - 1);
  buf[len - 1] = 0;
  return GBX_OK;
}

gbx_status gbx_set_particle_parameters(gbx_context* handle, const double* charge, const double* radius) {
  Context* ctx = reinterpret_cast<Context*>(handle);
  if (!ctx || !charge || !radius) return GBX_ERR_INVALID_ARGUMENT;
  drop_graph(ctx);
  const int n = ctx->n;
  for (int i = 0; i < n; ++i) {
    if (!isfinite(charge[i]) || !isfinite(radius[i]) || !(radius[i] > 0)) {
      ctx->last_error = "charges must be finite and radii finite and > 0 (particle " + std::to_string(i) + ")";
      return GBX_ERR_INVALID_ARGUMENT;
    }
  }
  ctx->charge.assign(charge, charge + n);
  ctx->radius.assign(radius, radius + n);
  std::vector<float> qf(n), wpar;
  std::vector<float2> par;
  for (int i = 0; i < n; ++i) qf[i] = (float)charge[i];
  set_model_params(ctx, wpar, par);
  GBX_CUDA(cudaMemcpy(ctx->d_radius, radius, sizeof(double) * n, cudaMemcpyHostToDevice));
  GBX_CUDA(cudaMemcpy(ctx->d_charge, qf.data(), sizeof(float) * n, cudaMemcpyHostToDevice));
  GBX_CUDA(cudaMemcpy(ctx->d_wpar, wpar.data(), sizeof(float) * n, cudaMemcpyHostToDevice));
  GBX_CUDA(cudaMemcpy(ctx->d_par, par.data(), sizeof(float2) * n, cudaMemcpyHostToDevice));
  gbx::choose_table(ctx);
  return GBX_OK;
}

gbx_status gbx_set_global_parameters(gbx_context* handle, double alpha0, double alpha1) {
  Context* ctx = reinterpret_cast<Context*>(handle);
  if (!ctx || !isfinite(alpha0) || !isfinite(alpha1)) return GBX_ERR_INVALID_ARGUMENT;
  drop_graph(ctx);
  ctx->cfg.alpha0 = alpha0;
  ctx->cfg.alpha1 = alpha1;
  ctx->alpha0 = (float)alpha0;
  ctx->alpha1 = (float)alpha1;
  return GBX_OK;
}

gbx_status gbx_set_box(gbx_context* handle, const double box[3]) {
  Context* ctx = reinterpret_cast<Context*>(handle);
  if (!ctx || !box) return GBX_ERR_INVALID_ARGUMENT;
  drop_graph(ctx);
  for (int k = 0; k < 3; ++k)
    if (!(box[k] > 0) || !isfinite(box[k]) || (ctx->cfg.periodic && !(box[k] >= 2.0 * ctx->cfg.cutoff))) {
      ctx->last_error = ctx->cfg.periodic ? "each box edge must be positive and at least twice the cutoff"
                                          : "box edges must be positive";
      return GBX_ERR_INVALID_ARGUMENT;
    }
  for (int k = 0; k < 3; ++k) ctx->cfg.box[k] = box[k];
  gbx::choose_table(ctx);
  return GBX_OK;
}

}  // extern "C"

namespace {
// A copy of a gbx_custom with owned strings, checked for what the device path supports.
gbx_status custom_spec_of(const gbx_custom* cu, gbx::gbx_custom_spec& spec, std::string& why) {
  if (!cu || cu->num_integrals < 1 || cu->num_integrals > 2 || cu->num_params < 1 || cu->num_values < 0 ||
      cu->num_terms < 1 || cu->num_globals < 0)
    return why = "need 1 or 2 integrals, parameters and energy terms", GBX_ERR_INVALID_ARGUMENT;
  auto str = [](const char* s) { return std::string(s ? s : ""); };
  for (int k = 0; k < cu->num_params; ++k) spec.params.push_back(str(cu->param_names[k]));
  for (int k = 0; k < cu->num_globals; ++k) {
    spec.globals.push_back(str(cu->global_names[k]));
    spec.global_values.push_back(cu->global_values[k]);
  }
  for (int k = 0; k < cu->num_integrals; ++k) {
    spec.integrals.push_back(str(cu->integral_names[k]));
    spec.integral_orders.push_back(cu->integral_orders[k]);
    if (cu->integral_orders[k] < 2)  // GBSWIntegral.cpp:85-88
      return why = "the order of an integral must be greater or equal to 2", GBX_ERR_INVALID_ARGUMENT;
  }
  for (int k = 0; k < cu->num_values; ++k) {
    spec.value_names.push_back(str(cu->value_names[k]));
    spec.value_expressions.push_back(str(cu->value_expressions[k]));
  }
  for (int k = 0; k < cu->num_terms; ++k) {
    spec.term_expressions.push_back(str(cu->term_expressions[k]));
    if (cu->term_types[k] != GBX_TERM_SINGLE && cu->term_types[k] != GBX_TERM_PAIR &&
        cu->term_types[k] != GBX_TERM_PAIR_NO_EXCLUSIONS)
      return why = "unknown energy term type", GBX_ERR_INVALID_ARGUMENT;
    spec.term_types.push_back(cu->term_types[k]);
  }
  if (cu->num_exclusions < 0 || (cu->num_exclusions > 0 && !cu->exclusions) || cu->num_param_derivs < 0 ||
      (cu->num_param_derivs > 0 && !cu->param_deriv_names))
    return why = "exclusions and parameter derivatives need their arrays", GBX_ERR_INVALID_ARGUMENT;
  for (int k = 0; k < cu->num_exclusions; ++k) {
    spec.exclusions.push_back(cu->exclusions[2 * k]);
    spec.exclusions.push_back(cu->exclusions[2 * k + 1]);
  }
  for (int k = 0; k < cu->num_param_derivs; ++k) {
    spec.param_derivs.push_back(str(cu->param_deriv_names[k]));
    if (std::find(spec.globals.begin(), spec.globals.end(), spec.param_derivs.back()) == spec.globals.end())
      return why = "energy parameter derivative of an unknown global '" + spec.param_derivs.back() + "'",
             GBX_ERR_INVALID_ARGUMENT;
  }
  for (const auto* names : {&spec.params, &spec.globals})
    for (const auto& nm : *names)
      if (nm == "x" || nm == "y" || nm == "z")
        return why = "x, y and z are the particle's coordinates, not parameter names", GBX_ERR_INVALID_ARGUMENT;
  if (cu->num_functions < 0 ||
      (cu->num_functions > 0 &&
       (!cu->function_names || !cu->function_sizes || !cu->function_values || !cu->function_ranges)))
    return why = "tabulated functions need their names, sizes, values and ranges", GBX_ERR_INVALID_ARGUMENT;
  size_t off = 0;
  for (int k = 0; k < cu->num_functions; ++k) {
    gbx::gbx_custom_spec::Function f;
    f.name = str(cu->function_names[k]);
    bool ident = !f.name.empty() && (std::isalpha((unsigned char)f.name[0]) || f.name[0] == '_');
    for (char ch : f.name) ident = ident && (std::isalnum((unsigned char)ch) || ch == '_');
    if (!ident) return why = "tabulated function name '" + f.name + "' is not an identifier", GBX_ERR_INVALID_ARGUMENT;
    const int m = cu->function_sizes[k];
    f.x0 = cu->function_ranges[2 * k];
    f.x1 = cu->function_ranges[2 * k + 1];
    // Continuous1DFunction needs at least two values and max > min
    if (m < 2 || !(f.x1 > f.x0) || !std::isfinite(f.x0) || !std::isfinite(f.x1))
      return why = "tabulated function '" + f.name + "' needs at least 2 values and max > min", GBX_ERR_INVALID_ARGUMENT;
    f.y.assign(cu->function_values + off, cu->function_values + off + m);
    off += (size_t)m;
    for (double v : f.y)
      if (!std::isfinite(v)) return why = "tabulated function '" + f.name + "' has a non-finite value", GBX_ERR_INVALID_ARGUMENT;
    for (const auto& g : spec.functions)
      if (g.name == f.name) return why = "tabulated function '" + f.name + "' defined twice", GBX_ERR_INVALID_ARGUMENT;
    spec.functions.push_back(std::move(f));
  }
  if (std::find(spec.params.begin(), spec.params.end(), std::string("radius")) == spec.params.end())
    return why = "the per-particle parameter 'radius' must be defined", GBX_ERR_INVALID_ARGUMENT;
  return GBX_OK;
}
}  // namespace

extern "C" {

gbx_status gbx_get_custom_param_derivs(gbx_context* handle, double* out, int count) {
  Context* ctx = reinterpret_cast<Context*>(handle);
  if (!ctx || !out || count < 0) return GBX_ERR_INVALID_ARGUMENT;
  if (!ctx->custom) {
    ctx->last_error = "parameter derivatives belong to the compiled-expression path";
    return GBX_ERR_UNSUPPORTED;
  }
  if (!ctx->have_result) return GBX_ERR_NOT_READY;
  return gbx::custom_param_derivs(ctx, out, count);
}

gbx_status gbx_custom_check(const gbx_custom* cu, char* log, size_t len) {
  gbx::gbx_custom_spec spec;
  std::string why;
  gbx_status s = custom_spec_of(cu, spec, why);
  if (s == GBX_OK) s = gbx::custom_compile_only(spec, why);
  if (log && len) {
    strncpy(log, why.c_str(), len - 1);
    log[len - 1] = 0;
  }
  return s;
}

gbx_status gbx_create_custom(const gbx_config* cfg, int num_atoms, const gbx_custom* cu, gbx_context** out) {
  if (!cfg || !cu || !out || num_atoms < 1) return GBX_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  // the integral classes' tables (the standalone GBSW force has fixed expressions)
  if (cfg->table_mode == GBX_TABLE_STANDALONE) return GBX_ERR_UNSUPPORTED;
  gbx::gbx_custom_spec spec;
  std::string why;
  GBX_TRY(custom_spec_of(cu, spec, why));
  gbx_config c = *cfg;
  c.integral_orders[0] = spec.integral_orders[0];
  c.integral_orders[1] = spec.integral_orders.size() > 1 ? spec.integral_orders[1] : spec.integral_orders[0];
  gbx_context* h = nullptr;
  GBX_TRY(gbx_create(&c, num_atoms, &h));
  Context* ctx = reinterpret_cast<Context*>(h);
  gbx_status s = gbx::custom_build(ctx, spec);
  if (s == GBX_OK) {
    ctx->energy_parts = gbx::custom_energy_parts(ctx);
    s = dalloc(ctx, &ctx->d_energy_part, ctx->energy_parts);
  }
  if (s != GBX_OK) {
    fprintf(stderr, "gbx_create_custom: %s\n", ctx->last_error.c_str());
    gbx_destroy(h);
    return s;
  }
  *out = h;
  return GBX_OK;
}

gbx_status gbx_set_custom_parameters(gbx_context* handle, const double* params) {
  Context* ctx = reinterpret_cast<Context*>(handle);
  if (!ctx || !params) return GBX_ERR_INVALID_ARGUMENT;
  if (!ctx->custom) return GBX_ERR_UNSUPPORTED;
  std::vector<double> radius;
  GBX_TRY(gbx::custom_set_parameters(ctx, params, radius));
  std::vector<double> q(ctx->n, 0.0);  // the custom terms read their own parameters
  return gbx_set_particle_parameters(handle, q.data(), radius.data());
}

gbx_status gbx_set_custom_global(gbx_context* handle, const char* name, double value) {
  Context* ctx = reinterpret_cast<Context*>(handle);
  if (!ctx || !name) return GBX_ERR_INVALID_ARGUMENT;
  if (!ctx->custom) return GBX_ERR_UNSUPPORTED;
  GBX_CUDA(cudaStreamSynchronize(ctx->stream));  // the copy must not race a call in flight
  return gbx::custom_set_global(ctx, name, value);
}

gbx_status gbx_execute(gbx_context* handle, const void* posq, unsigned long long* force_fixed, int force_stride,
                       double* energy, int flags, void* stream) {
  Context* ctx = reinterpret_cast<Context*>(handle);
  if (!ctx || !posq) return GBX_ERR_INVALID_ARGUMENT;
  if ((flags & GBX_EXEC_FORCES) && (!force_fixed || force_stride < ctx->n)) return GBX_ERR_INVALID_ARGUMENT;
  if ((flags & GBX_EXEC_ENERGY) && !energy) return GBX_ERR_INVALID_ARGUMENT;
  ctx->stream = stream ? (cudaStream_t)stream : ctx->own_stream;
  const bool forces = (flags & GBX_EXEC_FORCES) != 0, want_e = (flags & GBX_EXEC_ENERGY) != 0;
  const bool count = (flags & GBX_EXEC_COUNT_WORK) != 0;
  const bool permuted = ctx->d_slot_of != nullptr;
  const bool efloat = want_e && (flags & GBX_EXEC_ENERGY_FLOAT);
  // the pipeline's own buffers where the caller's cannot take its output
  // directly: forces not wanted or in another atom order, a float energy
  const bool internal_f = !forces || permuted, internal_e = !want_e || efloat;
  unsigned long long* f = internal_f ? ctx->d_force_fx : force_fixed;
  const int stride = internal_f ? ctx->n : force_stride;
  double* e = internal_e ? ctx->d_energy : energy;
  bool stale = false, nonfinite = false;
  GBX_TRY(poll_status(ctx, &stale, &nonfinite));
  const bool check = (flags & GBX_EXEC_CHECK) || !tables_sized(ctx) || stale;
  auto body = [&]() -> gbx_status {
    ctx->in_double = (flags & GBX_EXEC_POSQ_DOUBLE) != 0;
    ctx->in_permuted = permuted;
    gbx_status st = GBX_OK;
    if (internal_f && cudaMemsetAsync(ctx->d_force_fx, 0, sizeof(unsigned long long) * 3 * ctx->n, ctx->stream))
      st = GBX_ERR_CUDA;
    if (st == GBX_OK && internal_e && cudaMemsetAsync(ctx->d_energy, 0, sizeof(double), ctx->stream))
      st = GBX_ERR_CUDA;
    if (st == GBX_OK) st = run_pipeline(ctx, static_cast<const float4*>(posq), f, stride, e, check, false, count, forces);
    if (st == GBX_OK && ((forces && permuted) || efloat))
      st = gbx::launch_finish_outputs(ctx, forces && permuted ? force_fixed : nullptr, force_stride,
                                      efloat ? reinterpret_cast<float*>(energy) : nullptr);
    ctx->in_double = ctx->in_permuted = false;
    return st;
  };
  auto report = [&](gbx_status st) -> gbx_status {
    if (st != GBX_OK) return st;
    if (stale) {
      ctx->last_error = "an earlier unchecked call's lookup table outgrew its buffers, so that call lacked the "
                        "volume terms; the buffers were grown and this call ran checked";
      return GBX_ERR_STALE_RESULT;
    }
    if (nonfinite) {
      ctx->last_error = "an earlier unchecked call produced a non-finite Born radius";
      return GBX_ERR_NONFINITE;
    }
    return GBX_OK;
  };
  if (check || count || ctx->timing) return report(body());
  // unchecked: one CUDA graph of the whole call, captured on first use
  const Context::GraphKey key{posq, force_fixed, force_stride, energy, flags & ~GBX_EXEC_CHECK, ctx->stream};
  if (!ctx->graph || !(key == ctx->graph_key)) {
    drop_graph(ctx);
    GBX_TRY(fix_chain_records(ctx));
    if (cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
      (void)cudaGetLastError();  // a stream that cannot be captured: launch directly
      return report(body());
    }
    const long long before = ctx->launches;
    gbx_status s = body();
    cudaGraph_t g = nullptr;
    const cudaError_t ce = cudaStreamEndCapture(ctx->stream, &g);
    ctx->graph_kernels = ctx->launches - before;  // captured, not yet run
    ctx->launches = before;
    if (s != GBX_OK || ce != cudaSuccess) {
      if (g) cudaGraphDestroy(g);
      if (s == GBX_OK) {
        ctx->last_error = std::string("graph capture: ") + cudaGetErrorString(ce);
        s = GBX_ERR_CUDA;
      }
      return s;
    }
    const cudaError_t ei = cudaGraphInstantiate(&ctx->graph, g, 0);
    cudaGraphDestroy(g);
    GBX_CUDA(ei);
    ctx->graph_key = key;
  }
  GBX_CUDA(cudaGraphLaunch(ctx->graph, ctx->stream));
  ctx->launches += ctx->graph_kernels;
  ctx->have_result = true;
  return report(GBX_OK);
}

gbx_status gbx_set_atom_order(gbx_context* handle, const int* atom_index) {
  Context* ctx = reinterpret_cast<Context*>(handle);
  if (!ctx) return GBX_ERR_INVALID_ARGUMENT;
  const int n = ctx->n;
  if (!atom_index) {
    if (ctx->d_slot_of) {
      drop_graph(ctx);
      GBX_CUDA(cudaStreamSynchronize(ctx->stream));
      cudaFree(ctx->d_slot_of);
      ctx->d_slot_of = nullptr;
    }
    return GBX_OK;
  }
  std::vector<int> slot_of(n, -1);
  for (int k = 0; k < n; ++k) {
    const int a = atom_index[k];
    if (a < 0 || a >= n || slot_of[a] >= 0) {
      ctx->last_error = "atom_index must be a permutation of 0..n-1";
      return GBX_ERR_INVALID_ARGUMENT;
    }
    slot_of[a] = k;
  }
  if (!ctx->d_slot_of) GBX_TRY(dalloc(ctx, &ctx->d_slot_of, n));  // the captured graphs read the old layout
  // the order is read by the kernels at run time: an update between calls
  // needs no new graph, only the copy ordered after earlier work
  GBX_CUDA(cudaStreamSynchronize(ctx->stream));
  GBX_CUDA(cudaMemcpy(ctx->d_slot_of, slot_of.data(), sizeof(int) * n, cudaMemcpyHostToDevice));
  return GBX_OK;
}

}  // extern "C"

namespace {

// The host-buffer call's two O(N) host loops (positions in, forces out) move
// about 110 bytes per atom through memory; from this many atoms on they are
// split over a few host threads (each element is written by one thread, so
// the results do not depend on the split).
constexpr int kHostParallelAtoms = 16384;
int host_threads() {
  static const int t = std::max(1, std::min(8, omp_get_num_procs()));
  return t;
}

// Host positions -> pinned float4 staging (checked for finite values in the same pass).
gbx_status host_stage(Context* ctx, const double* positions) {
  const int n = ctx->n;
  bool finite = true;
  float4* hp = ctx->h_pos;
  auto stage = [&](int i) {
    const double x = positions[3 * i], y = positions[3 * i + 1], z = positions[3 * i + 2];
    hp[i] = make_float4((float)x, (float)y, (float)z, 0.f);
    return std::isfinite(x) && std::isfinite(y) && std::isfinite(z);
  };
  if (n >= kHostParallelAtoms) {
#pragma omp parallel for reduction(&& : finite) num_threads(host_threads())
    for (int i = 0; i < n; ++i) finite = stage(i) && finite;
  } else {
    for (int i = 0; i < n; ++i) finite = stage(i) && finite;
  }
  if (!finite) {
    ctx->last_error = "non-finite position";
    return GBX_ERR_INVALID_ARGUMENT;
  }
  return GBX_OK;
}

// Upload, evaluation, and the readback of forces (optional), energy and the
// status word, all on the context's own stream.
gbx_status host_enqueue(Context* ctx, bool adjoint, bool count_work, bool check, bool forces) {
  const int n = ctx->n;
  ctx->stream = ctx->own_stream;
  GBX_CUDA(cudaMemcpyAsync(ctx->d_pos, ctx->h_pos, sizeof(float4) * n, cudaMemcpyHostToDevice, ctx->stream));
  GBX_CUDA(cudaMemsetAsync(ctx->d_force_fx, 0, sizeof(unsigned long long) * 3 * n, ctx->stream));
  GBX_CUDA(cudaMemsetAsync(ctx->d_energy, 0, sizeof(double), ctx->stream));
  // d_pos holds the raw copy; staging rewrites it in place with the model parameter
  GBX_TRY(run_pipeline(ctx, ctx->d_pos, ctx->d_force_fx, n, ctx->d_energy, check, adjoint, count_work));
  if (forces)
    GBX_CUDA(cudaMemcpyAsync(ctx->h_force_fx, ctx->d_force_fx, sizeof(unsigned long long) * 3 * n,
                             cudaMemcpyDeviceToHost, ctx->stream));
  GBX_CUDA(cudaMemcpyAsync(ctx->h_energy, ctx->d_energy, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  GBX_CUDA(cudaMemcpyAsync(ctx->h_status, ctx->d_status, sizeof(unsigned), cudaMemcpyDeviceToHost, ctx->stream));
  return GBX_OK;
}

gbx_status host_run(Context* ctx, const double* positions, bool adjoint, bool count_work, bool check = true,
                    bool forces = true) {
  GBX_TRY(host_stage(ctx, positions));
  return host_enqueue(ctx, adjoint, count_work, check, forces);
}

// Waits for the call and writes its results.  With `optimistic` (an
// unchecked run) a table that outgrew its buffers sets *rerun and leaves the
// outputs untouched: the caller runs again checked, which grows the buffers.
gbx_status host_results(Context* ctx, double* forces, double* energy, bool optimistic = false,
                        bool* rerun = nullptr) {
  const int n = ctx->n;
  if (rerun) *rerun = false;
  GBX_CUDA(cudaStreamSynchronize(ctx->stream));
  const unsigned st = *ctx->h_status;
  if (optimistic && (st & (gbx::kStatusTableCells | gbx::kStatusTableEntries | gbx::kStatusSegmentTooLong))) {
    if (rerun) *rerun = true;
    return GBX_OK;
  }
  const double e = *ctx->h_energy;
  if (st & gbx::kStatusNonFinite) {
    ctx->last_error = "non-finite Born radius";
    return GBX_ERR_NONFINITE;
  }
  if (forces) {
    const unsigned long long* hf = ctx->h_force_fx;
    auto add = [&](int i) {
      for (int k = 0; k < 3; ++k) forces[3 * i + k] += gbx::fixed_to_double(hf[(size_t)k * n + i]);
    };
    if (n >= kHostParallelAtoms) {
#pragma omp parallel for num_threads(host_threads())
      for (int i = 0; i < n; ++i) add(i);
    } else {
      for (int i = 0; i < n; ++i) add(i);
    }
  }
  if (energy) *energy = e;
  if (!isfinite(e)) {
    ctx->last_error = "non-finite energy";
    return GBX_ERR_NONFINITE;
  }
  return GBX_OK;
}

// The unchecked host call as one CUDA graph (upload, evaluation, readback
// between the context's pinned buffers), captured on first use.
gbx_status host_graph_launch(Context* ctx, bool forces) {
  ctx->stream = ctx->own_stream;
  if (!ctx->host_graph || ctx->host_graph_forces != (forces ? 1 : 0)) {
    if (ctx->host_graph) cudaGraphExecDestroy(ctx->host_graph);
    ctx->host_graph = nullptr;
    GBX_TRY(fix_chain_records(ctx));
    GBX_CUDA(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    const long long before = ctx->launches;
    gbx_status s = host_enqueue(ctx, false, false, false, forces);
    cudaGraph_t g = nullptr;
    const cudaError_t ce = cudaStreamEndCapture(ctx->stream, &g);
    ctx->host_graph_kernels = ctx->launches - before;  // captured, not yet run
    ctx->launches = before;
    if (s != GBX_OK || ce != cudaSuccess) {
      if (g) cudaGraphDestroy(g);
      if (s == GBX_OK) {
        ctx->last_error = std::string("graph capture: ") + cudaGetErrorString(ce);
        s = GBX_ERR_CUDA;
      }
      return s;
    }
    const cudaError_t ei = cudaGraphInstantiate(&ctx->host_graph, g, 0);
    cudaGraphDestroy(g);
    GBX_CUDA(ei);
    ctx->host_graph_forces = forces ? 1 : 0;
  }
  GBX_CUDA(cudaGraphLaunch(ctx->host_graph, ctx->stream));
  ctx->launches += ctx->host_graph_kernels;
  ctx->have_result = true;
  return GBX_OK;
}

}  // namespace

extern "C" {

gbx_status gbx_execute_host(gbx_context* handle, const double* positions, double* forces, double* energy, int flags) {
  Context* ctx = reinterpret_cast<Context*>(handle);
  if (!ctx || !positions) return GBX_ERR_INVALID_ARGUMENT;
  const bool count = (flags & GBX_EXEC_COUNT_WORK) != 0;
  double* f = (flags & GBX_EXEC_FORCES) ? forces : nullptr;
  const bool optimistic = !count && !(flags & GBX_EXEC_CHECK) && tables_sized(ctx);
  bool rerun = false;
  if (optimistic && !ctx->timing) {  // one graph launch and one synchronisation
    GBX_TRY(host_stage(ctx, positions));
    GBX_TRY(host_graph_launch(ctx, f != nullptr));
    GBX_TRY(host_results(ctx, f, energy, true, &rerun));
    if (!rerun) return GBX_OK;
  } else {
    GBX_TRY(host_run(ctx, positions, false, count, !optimistic, f != nullptr));
    GBX_TRY(host_results(ctx, f, energy, optimistic, &rerun));
    if (!rerun) return GBX_OK;
  }
  GBX_TRY(host_run(ctx, positions, false, count, true, f != nullptr));
  return host_results(ctx, f, energy);
}

gbx_status gbx_adjoint_host(gbx_context* handle, const double* positions, double* energy, double* forces,
                            double* dEdq, double* dEdR, double* dEdalpha) {
  Context* ctx = reinterpret_cast<Context*>(handle);
  if (!ctx || !positions) return GBX_ERR_INVALID_ARGUMENT;
  if (ctx->custom) {
    ctx->last_error = "the adjoint covers the canonical expressions only";
    return GBX_ERR_UNSUPPORTED;
  }
  GBX_TRY(host_run(ctx, positions, true, false));
  const int n = ctx->n;
  std::vector<unsigned long long> q(n), r(n);
  double a[2];
  GBX_CUDA(cudaMemcpyAsync(q.data(), ctx->d_dEdq_fx, sizeof(unsigned long long) * n, cudaMemcpyDeviceToHost,
                           ctx->stream));
  GBX_CUDA(cudaMemcpyAsync(r.data(), ctx->d_dEdR_fx, sizeof(unsigned long long) * n, cudaMemcpyDeviceToHost,
                           ctx->stream));
  GBX_CUDA(cudaMemcpyAsync(a, ctx->d_alpha_grad, sizeof(a), cudaMemcpyDeviceToHost, ctx->stream));
  GBX_TRY(host_results(ctx, forces, energy));
  for (int i = 0; i < n; ++i) {
    if (dEdq) dEdq[i] = gbx::fixed_to_double(q[i]);
    if (dEdR) dEdR[i] = gbx::fixed_to_double(r[i]);
  }
  if (dEdalpha) {
    dEdalpha[0] = a[0];
    dEdalpha[1] = a[1];
  }
  return GBX_OK;
}

gbx_status gbx_adjoint(gbx_context* handle, const void* posq, double* energy, double* forces, double* dEdq,
                       double* dEdR, double* dEdalpha, int flags, void* stream) {
  Context* ctx = reinterpret_cast<Context*>(handle);
  if (!ctx || !posq) return GBX_ERR_INVALID_ARGUMENT;
  if (ctx->custom) {
    ctx->last_error = "the adjoint covers the canonical expressions only";
    return GBX_ERR_UNSUPPORTED;
  }
  ctx->stream = stream ? (cudaStream_t)stream : ctx->own_stream;
  const int n = ctx->n;
  GBX_CUDA(cudaMemsetAsync(ctx->d_force_fx, 0, sizeof(unsigned long long) * 3 * n, ctx->stream));
  GBX_CUDA(cudaMemsetAsync(ctx->d_energy, 0, sizeof(double), ctx->stream));
  const bool check = (flags & GBX_EXEC_CHECK) || (ctx->use_tight ? ctx->tcell_cap == 0 : ctx->cell_cap == 0);
  GBX_TRY(run_pipeline(ctx, reinterpret_cast<const float4*>(posq), ctx->d_force_fx, n, ctx->d_energy, check, true,
                       false));
  return gbx::launch_adjoint_out(ctx, energy, forces, dEdq, dEdR, dEdalpha);
}

gbx_status gbx_get_born_radii(gbx_context* handle, double* born) {
  Context* ctx = reinterpret_cast<Context*>(handle);
  if (!ctx || !born) return GBX_ERR_INVALID_ARGUMENT;
  if (!ctx->have_result) return GBX_ERR_NOT_READY;
  GBX_CUDA(cudaStreamSynchronize(ctx->stream));
  GBX_CUDA(cudaMemcpy(born, ctx->d_born, sizeof(double) * ctx->n, cudaMemcpyDeviceToHost));
  return GBX_OK;
}

gbx_status gbx_get_integrals(gbx_context* handle, double* integrals) {
  Context* ctx = reinterpret_cast<Context*>(handle);
  if (!ctx || !integrals) return GBX_ERR_INVALID_ARGUMENT;
  if (!ctx->have_result) return GBX_ERR_NOT_READY;
  GBX_CUDA(cudaStreamSynchronize(ctx->stream));
  GBX_CUDA(cudaMemcpy(integrals, ctx->d_integrals, sizeof(double) * 2 * ctx->n, cudaMemcpyDeviceToHost));
  return GBX_OK;
}

gbx_status gbx_get_dEdB(gbx_context* handle, double* dEdB) {
  Context* ctx = reinterpret_cast<Context*>(handle);
  if (!ctx || !dEdB) return GBX_ERR_INVALID_ARGUMENT;
  if (!ctx->have_result) return GBX_ERR_NOT_READY;
  std::vector<unsigned long long> v(ctx->n);
  GBX_CUDA(cudaStreamSynchronize(ctx->stream));
  GBX_CUDA(cudaMemcpy(v.data(), ctx->d_dEdB_fx, sizeof(unsigned long long) * ctx->n, cudaMemcpyDeviceToHost));
  for (int i = 0; i < ctx->n; ++i) dEdB[i] = gbx::fixed_to_double(v[i]);
  return GBX_OK;
}

gbx_status gbx_build_lookup_table(gbx_context* handle, const void* posq, void* stream) {
  Context* ctx = reinterpret_cast<Context*>(handle);
  if (!ctx || !posq) return GBX_ERR_INVALID_ARGUMENT;
  ctx->stream = stream ? (cudaStream_t)stream : ctx->own_stream;
  GBX_TRY(gbx::launch_stage_positions(ctx, reinterpret_cast<const float4*>(posq)));
  return build_table_checked(ctx, true);
}

gbx_status gbx_get_lookup_table(gbx_context* handle, int dims[3], double mn[3], double step[3], int64_t* ncell,
                                int32_t* counts, int64_t* total, int32_t* atoms) {
  Context* ctx = reinterpret_cast<Context*>(handle);
  if (!ctx) return GBX_ERR_INVALID_ARGUMENT;
  if (!ctx->table_valid) {
    // the last execute integrated on the exact table: build the reference
    // table from the positions it staged
    if (!ctx->have_result) return GBX_ERR_NOT_READY;
    GBX_TRY(build_table_checked(ctx, true));
  }
  gbx::TableGeom g;
  GBX_CUDA(cudaStreamSynchronize(ctx->stream));
  GBX_CUDA(cudaMemcpy(&g, ctx->d_geom, sizeof(g), cudaMemcpyDeviceToHost));
  for (int k = 0; k < 3; ++k) {
    if (dims) dims[k] = g.dims[k];
    if (mn) mn[k] = g.min[k];
    if (step) step[k] = g.step[k];
  }
  if (ncell) *ncell = g.ncell;
  std::vector<int> cnt(g.ncell), st(g.ncell + 1);
  GBX_CUDA(cudaMemcpy(cnt.data(), ctx->d_cell_count, sizeof(int) * g.ncell, cudaMemcpyDeviceToHost));
  GBX_CUDA(cudaMemcpy(st.data(), ctx->d_cell_start, sizeof(int) * (g.ncell + 1), cudaMemcpyDeviceToHost));
  long long tot = 0;
  for (long long c = 0; c < g.ncell; ++c) tot += cnt[c];
  if (total) *total = tot;
  if (counts) memcpy(counts, cnt.data(), sizeof(int) * g.ncell);
  if (atoms) {
    std::vector<int> all(g.total > 0 ? g.total : 1);
    if (g.total > 0)
      GBX_CUDA(cudaMemcpy(all.data(), ctx->d_entries, sizeof(int) * g.total, cudaMemcpyDeviceToHost));
    long long o = 0;
    for (long long c = 0; c < g.ncell; ++c)
      for (int m = 0; m < cnt[c]; ++m) atoms[o++] = all[st[c] + m];
  }
  return GBX_OK;
}

gbx_status gbx_set_timing(gbx_context* handle, int enable) {
  Context* ctx = reinterpret_cast<Context*>(handle);
  if (!ctx) return GBX_ERR_INVALID_ARGUMENT;
  if (enable && !ctx->ev[0])
    for (int k = 0; k <= Context::kStages; ++k) GBX_CUDA(cudaEventCreate(&ctx->ev[k]));
  ctx->timing = enable != 0;
  return GBX_OK;
}

gbx_status gbx_get_stage_times(gbx_context* handle, double* ms, int max_stages, int* num_stages) {
  Context* ctx = reinterpret_cast<Context*>(handle);
  if (!ctx || !ms) return GBX_ERR_INVALID_ARGUMENT;
  if (!ctx->timing || !ctx->have_result) return GBX_ERR_NOT_READY;
  GBX_CUDA(cudaEventSynchronize(ctx->ev[Context::kStages]));
  const int n = std::min(max_stages, (int)Context::kStages);
  for (int k = 0; k < n; ++k) {
    float t = 0.f;
    GBX_CUDA(cudaEventElapsedTime(&t, ctx->ev[k], ctx->ev[k + 1]));
    ms[k] = t;
  }
  if (num_stages) *num_stages = Context::kStages;
  return GBX_OK;
}

gbx_status gbx_get_work(gbx_context* handle, double* volume_evals, double* shell_evals, double* pairs) {
  Context* ctx = reinterpret_cast<Context*>(handle);
  if (!ctx) return GBX_ERR_INVALID_ARGUMENT;
  unsigned long long w[4];
  GBX_CUDA(cudaStreamSynchronize(ctx->stream));
  GBX_CUDA(cudaMemcpy(w, ctx->d_work, sizeof(w), cudaMemcpyDeviceToHost));
  if (volume_evals) *volume_evals = (double)w[0];
  if (shell_evals) *shell_evals = (double)w[1];
  if (pairs) *pairs = (double)ctx->n * (double)(ctx->n - 1);
  return GBX_OK;
}

gbx_status gbx_set_chain_records(gbx_context* handle, int per_warp) {
  Context* ctx = reinterpret_cast<Context*>(handle);
  if (!ctx) return GBX_ERR_INVALID_ARGUMENT;
  drop_graph(ctx);
  GBX_CUDA(cudaStreamSynchronize(ctx->stream));
  ctx->srec_pending = false;
  ctx->srec_auto = per_warp < 0;
  GBX_TRY(alloc_records(ctx, per_warp > 0 ? per_warp : 0));
  if (per_warp > 0 && ctx->srec_R != per_warp) {
    ctx->last_error = "cannot allocate the chain-record buffer";
    return GBX_ERR_OUT_OF_MEMORY;
  }
  return GBX_OK;
}

gbx_status gbx_get_chain_records(gbx_context* handle, long long* written, int* max_need, int* per_warp,
                                 int* overflowed) {
  Context* ctx = reinterpret_cast<Context*>(handle);
  if (!ctx) return GBX_ERR_INVALID_ARGUMENT;
  GBX_CUDA(cudaStreamSynchronize(ctx->stream));
  long long w = -1;
  int mx = 0, over = 0;
  if (ctx->records) {
    std::vector<int> cnt((size_t)ctx->srec_warps);
    GBX_CUDA(cudaMemcpy(cnt.data(), ctx->d_rcount, sizeof(int) * cnt.size(), cudaMemcpyDeviceToHost));
    w = 0;
    for (int c : cnt) {
      const int need = c >= 0 ? c : -1 - c;
      if (c >= 0) w += c;
      else ++over;
      mx = need > mx ? need : mx;
    }
  }
  if (written) *written = w;
  if (max_need) *max_need = mx;
  if (per_warp) *per_warp = ctx->srec_R;
  if (overflowed) *overflowed = over;
  return GBX_OK;
}

gbx_status gbx_get_launches(gbx_context* handle, long long* launches) {
  Context* ctx = reinterpret_cast<Context*>(handle);
  if (!ctx || !launches) return GBX_ERR_INVALID_ARGUMENT;
  *launches = ctx->launches;
  return GBX_OK;
}

gbx_status gbx_get_chain_work(gbx_context* handle, double* list_evals, double* derivative_evals) {
  Context* ctx = reinterpret_cast<Context*>(handle);
  if (!ctx) return GBX_ERR_INVALID_ARGUMENT;
  unsigned long long w[4];
  GBX_CUDA(cudaStreamSynchronize(ctx->stream));
  GBX_CUDA(cudaMemcpy(w, ctx->d_work, sizeof(w), cudaMemcpyDeviceToHost));
  if (list_evals) *list_evals = (double)w[2];
  if (derivative_evals) *derivative_evals = (double)w[3];
  return GBX_OK;
}

}  // extern "C"
