// Lookup-table build: bins atoms into per-cell lists that are bit-identical
// to the reference's tables.
//
//   geometry  one block reduces the bounding box / centre of geometry and
//             derives the grid exactly as the reference does (FP64);
//   count     one warp per atom enumerates its candidate cells (or samples)
//             and counts members with atomics;
//   scan      exclusive prefix sum of the counts -> CSR offsets;
//   fill      second enumeration writes members at atomic cursors;
//   sort      one warp per cell ranks its entries, restoring the reference's
//             ascending-atom insertion order, then applies the per-cell cap.
//
// Every FP64 operation that decides membership is written with explicit
// round-to-nearest intrinsics so that no multiply-add is contracted: the
// decisions match the reference's separately rounded C++ arithmetic.
#include <math.h>

#include "gbx_internal.cuh"
#include "scan.cuh"

namespace gbx {
namespace {

constexpr int kGeomThreads = 1024;
constexpr int kMaxSamples = 96;  // samples per axis in the periodic branch

__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double ddiv(double a, double b) { return __ddiv_rn(a, b); }

// sqrt(3.0)/2.0 as the reference computes it in double.
__device__ __forceinline__ double half_sqrt3() { return ddiv(__dsqrt_rn(3.0), 2.0); }

// --------------------------------------------------------------------------
// Geometry: CharmmReferenceGBSW.cpp:444-466, CustomGBIntegral.cpp:53-113,163-193
// --------------------------------------------------------------------------
// Per-block partial extents and sums over a fixed range of atoms (FP64 on
// every SM instead of one: the GPU's FP64 rate per SM is low), reduced by
// a fixed-shape tree, so the centre of geometry is the same bits every call.
constexpr int kPartThreads = 256;

struct GeomPart {
  double mn[3], mx[3], sum[3], rmax;
};

__global__ void __launch_bounds__(kPartThreads) table_geom_partial_kernel(const float4* __restrict__ pos,
                                                                          const double* __restrict__ radius, int n,
                                                                          GeomPart* __restrict__ parts) {
  __shared__ double s[10][kPartThreads];
  const int t = threadIdx.x, a = blockIdx.x * kPartThreads + t;
  double v[10];
  if (a < n) {
    const float4 p = pos[a];
    const double c[3] = {(double)p.x, (double)p.y, (double)p.z};
    for (int k = 0; k < 3; ++k) {
      v[k] = c[k];
      v[3 + k] = c[k];
      v[6 + k] = c[k];
    }
    v[9] = radius[a];
  } else {
    const float4 p = pos[blockIdx.x * kPartThreads];  // an atom of this block: neutral for min / max
    for (int k = 0; k < 3; ++k) {
      v[k] = v[3 + k] = (&p.x)[k];
      v[6 + k] = 0.0;
    }
    v[9] = 0.0;
  }
  for (int k = 0; k < 10; ++k) s[k][t] = v[k];
  __syncthreads();
  for (int stride = kPartThreads / 2; stride > 0; stride >>= 1) {
    if (t < stride) {
      for (int k = 0; k < 3; ++k) {
        s[k][t] = fmin(s[k][t], s[k][t + stride]);
        s[3 + k][t] = fmax(s[3 + k][t], s[3 + k][t + stride]);
        s[6 + k][t] = dadd(s[6 + k][t], s[6 + k][t + stride]);
      }
      s[9][t] = fmax(s[9][t], s[9][t + stride]);
    }
    __syncthreads();
  }
  if (t == 0) {
    GeomPart g;
    for (int k = 0; k < 3; ++k) {
      g.mn[k] = s[k][0];
      g.mx[k] = s[3 + k][0];
      g.sum[k] = s[6 + k][0];
    }
    g.rmax = s[9][0];
    parts[blockIdx.x] = g;
  }
}

// CharmmReferenceGBSW.cpp:444-466, CustomGBIntegral.cpp:53-113,163-193: the
// grid from the partial extents (combined in block order).
__global__ void __launch_bounds__(kGeomThreads) table_geom_kernel(const GeomPart* __restrict__ parts, int nparts,
                                                                  int n, int mode, double h, double buffer,
                                                                  double sw, double bx, double by, double bz,
                                                                  TableGeom* __restrict__ g, long long cell_cap,
                                                                  unsigned* __restrict__ status) {
  __shared__ double s[10][kGeomThreads];
  const int t = threadIdx.x;
  double v[10];
  const GeomPart p0 = parts[0];
  for (int k = 0; k < 3; ++k) {
    v[k] = p0.mn[k];
    v[3 + k] = p0.mx[k];
    v[6 + k] = 0.0;
  }
  v[9] = 0.0;
  for (int b = t; b < nparts; b += kGeomThreads) {  // each thread's parts in block order
    const GeomPart p = parts[b];
    for (int k = 0; k < 3; ++k) {
      v[k] = fmin(v[k], p.mn[k]);
      v[3 + k] = fmax(v[3 + k], p.mx[k]);
      v[6 + k] = dadd(v[6 + k], p.sum[k]);
    }
    v[9] = fmax(v[9], p.rmax);
  }
  for (int k = 0; k < 10; ++k) s[k][t] = v[k];
  __syncthreads();
  for (int stride = kGeomThreads / 2; stride > 0; stride >>= 1) {
    if (t < stride) {
      for (int k = 0; k < 3; ++k) {
        s[k][t] = fmin(s[k][t], s[k][t + stride]);
        s[3 + k][t] = fmax(s[3 + k][t], s[3 + k][t + stride]);
        s[6 + k][t] = dadd(s[6 + k][t], s[6 + k][t + stride]);
      }
      s[9][t] = fmax(s[9][t], s[9][t + stride]);
    }
    __syncthreads();
  }
  if (t != 0) return;
  double mn[3], mx[3], sm[3];
  for (int k = 0; k < 3; ++k) {
    mn[k] = s[k][0];
    mx[k] = s[3 + k][0];
    sm[k] = s[6 + k][0];
  }
  const double rmax = s[9][0];
  TableGeom G;
  G.mode = mode;
  G.total = 0;
  G.L = h;
  long long ncell = 1;
  if (mode == GBX_TABLE_STANDALONE || mode == GBX_TABLE_GRID) {
    double pad;
    if (mode == GBX_TABLE_STANDALONE)
      pad = dadd(dadd(dadd(dadd(buffer, rmax), sw), dmul(half_sqrt3(), h)), 1e-6);
    else
      pad = dadd(dadd(0.03, dmul(half_sqrt3(), h)), buffer);
    G.pad = pad;
    for (int k = 0; k < 3; ++k) {
      double lo = dsub(mn[k], pad), hi = dadd(mx[k], pad);
      double length = dsub(hi, lo);
      if (mode == GBX_TABLE_GRID && length > 1000.0) {
        atomicOr(status, kStatusTableCells);
        G.dims[k] = 1;
      } else {
        G.dims[k] = (int)ceil(ddiv(length, h)) + 1;
      }
      G.min[k] = lo;
      G.max[k] = dadd(lo, dmul((double)(G.dims[k] - 1), h));
      G.step[k] = h;
      G.box[k] = k == 0 ? bx : (k == 1 ? by : bz);  // read only by a periodic system's wrapped query
      ncell *= G.dims[k];
    }
  } else {
    double box[3] = {bx, by, bz};
    double cog[3];
    for (int k = 0; k < 3; ++k) cog[k] = ddiv(sm[k], (double)n);
    double L = 0.0;
    for (int k = 0; k < 3; ++k) {
      double d = box[k];
      G.box[k] = d;
      G.min[k] = dsub(cog[k], ddiv(d, 2.0));
      G.max[k] = dadd(cog[k], ddiv(d, 2.0));
      G.dims[k] = (int)ceil(ddiv(d, h)) + 1;
      G.step[k] = ddiv(d, (double)G.dims[k]);
      ncell *= G.dims[k];
    }
    L = fmax(fmax(G.step[0], G.step[1]), G.step[2]);
    G.L = L;
    G.pad = 0.0;
  }
  for (int k = 0; k < 3; ++k) {
    G.inv_step[k] = 1.0 / G.step[k];
    G.inv_box[k] = G.box[k] > 0.0 ? 1.0 / G.box[k] : 0.0;
  }
  G.ncell = ncell;
  if (ncell > cell_cap) atomicOr(status, kStatusTableCells);
  *g = G;
}

// --------------------------------------------------------------------------
// Membership enumeration (count / fill)
// --------------------------------------------------------------------------

struct Emit {
  int* count;
  const int* start;
  int* cursor;
  int* entries;
  long long entry_cap;
  unsigned* status;
  template <bool FILL>
  __device__ __forceinline__ void put(long long idx, int atom, long long ncell) const {
    if (idx < 0 || idx >= ncell) return;
    if (!FILL) {
      atomicAdd(&count[idx], 1);
    } else {
      int slot = atomicAdd(&cursor[idx], 1);
      long long p = (long long)start[idx] + slot;
      if (p < entry_cap) entries[p] = atom;
      else atomicOr(status, kStatusTableEntries);
    }
  }
};

// CharmmReferenceGBSW.cpp:472-496 (STANDALONE) and CustomGBIntegral.cpp:198-227 (GRID).
template <int MODE, bool FILL>
__global__ void table_members_grid_kernel(const float4* __restrict__ pos, const double* __restrict__ radius, int n,
                                          const TableGeom* __restrict__ gp, double h, double buffer, Emit em,
                                          long long cell_cap) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) / kWarp;
  const int lane = threadIdx.x % kWarp;
  const TableGeom& g = *gp;
  if (g.ncell > cell_cap) return;
  const long long ncell = g.ncell;
  for (int a = warp; a < n; a += (gridDim.x * blockDim.x) / kWarp) {
    float4 p = pos[a];
    const double c[3] = {(double)p.x, (double)p.y, (double)p.z};
    double pad;
    if (MODE == GBX_TABLE_STANDALONE) pad = g.pad;
    else pad = dadd(dadd(radius[a], dmul(half_sqrt3(), h)), buffer);
    const double pad2 = dmul(pad, pad);
    int b[3], e[3];
    for (int k = 0; k < 3; ++k) {
      b[k] = (int)floor(ddiv(dsub(dsub(c[k], pad), g.min[k]), h));
      e[k] = (int)ceil(ddiv(dsub(dadd(c[k], pad), g.min[k]), h));
    }
    const int nx = e[0] - b[0] + 1, ny = e[1] - b[1] + 1, nz = e[2] - b[2] + 1;
    // non-finite or absurd inputs: skip the atom instead of looping on garbage bounds
    if (!(nx >= 1 && ny >= 1 && nz >= 1 && nx <= 1024 && ny <= 1024 && nz <= 1024)) {
      if (lane == 0) atomicOr(em.status, kStatusTableCells);
      continue;
    }
    const int total = nx * ny * nz;
    const long long sy = g.dims[2], sx = (long long)g.dims[1] * g.dims[2];
    for (int t = lane; t < total; t += kWarp) {
      const int i = b[0] + t / (ny * nz);
      const int j = b[1] + (t / nz) % ny;
      const int k = b[2] + t % nz;
      const double d0 = dsub(dadd(g.min[0], dmul((double)i, h)), c[0]);
      const double d1 = dsub(dadd(g.min[1], dmul((double)j, h)), c[1]);
      const double d2 = dsub(dadd(g.min[2], dmul((double)k, h)), c[2]);
      const double s = dadd(dadd(dmul(d0, d0), dmul(d1, d1)), dmul(d2, d2));
      bool member;
      if (MODE == GBX_TABLE_STANDALONE) member = __dsqrt_rn(s) < pad;
      else member = s < pad2;
      if (member) em.put<FILL>((long long)i * sx + (long long)j * sy + k, a, ncell);
    }
  }
}

// CustomGBIntegral.cpp:117-159 (PERIODIC): samples at the grid step, accumulated
// by repeated addition exactly as the reference's for-loops do.  The cell
// index of a sample and the membership test are decided in FP32 wherever the
// FP32 value is clear of the decision's boundary by a margin that covers its
// rounding, and in the reference's FP64 operations otherwise (FP64 runs at a
// small fraction of the FP32 rate on this part).
template <bool FILL>
__global__ void table_members_periodic_kernel(const float4* __restrict__ pos, const double* __restrict__ radius,
                                              int n, const TableGeom* __restrict__ gp, double buffer, Emit em,
                                              long long cell_cap, unsigned* __restrict__ status) {
  // per warp and axis: the samples, their cell index (-1 outside) and the
  // squared offset from the atom in FP32 -- each depends on one axis only,
  // so it is computed once per axis value
  __shared__ double s_samp[8][3][kMaxSamples];
  __shared__ float s_sq[8][3][kMaxSamples];
  __shared__ int s_id[8][3][kMaxSamples];
  const int wib = threadIdx.x / kWarp;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) / kWarp;
  const int lane = threadIdx.x % kWarp;
  const TableGeom& g = *gp;
  if (g.ncell > cell_cap) return;
  const long long ncell = g.ncell;
  double (*samp)[kMaxSamples] = s_samp[wib];
  float (*sq)[kMaxSamples] = s_sq[wib];
  int (*idx)[kMaxSamples] = s_id[wib];
  constexpr float kEpsCell = 1e-4f;  // cell units: far above the FP32 rounding of a sample's position
  for (int a = warp; a < n; a += (gridDim.x * blockDim.x) / kWarp) {
    float4 p = pos[a];
    const double c[3] = {(double)p.x, (double)p.y, (double)p.z};
    const double L = g.L;
    const double pad = dadd(dadd(radius[a], dmul(half_sqrt3(), L)), buffer);
    const double pad2 = dmul(pad, pad);
    int cnt0 = 0;
    // lanes 0..2 walk one axis each (samples by repeated addition, as the reference)
    if (lane < 3) {
      const int k = lane;
      double x = dsub(dsub(c[k], pad), L);
      const double end = dadd(dadd(c[k], pad), L);
      int m = 0;
      while (x < end && m <= kMaxSamples) {
        if (m < kMaxSamples) samp[k][m] = x;
        ++m;
        x = dadd(x, g.step[k]);
      }
      if (m > kMaxSamples) atomicOr(status, kStatusTableEntries);
      cnt0 = m;
    }
    int cnt[3];
    for (int k = 0; k < 3; ++k) {
      const int v = __shfl_sync(0xffffffffu, cnt0, k);
      cnt[k] = v < kMaxSamples ? v : kMaxSamples;
    }
    __syncwarp();
    for (int t = lane; t < cnt[0] + cnt[1] + cnt[2]; t += kWarp) {
      const int k = t < cnt[0] ? 0 : (t < cnt[0] + cnt[1] ? 1 : 2);
      const int m = t - (k == 0 ? 0 : (k == 1 ? cnt[0] : cnt[0] + cnt[1]));
      const double xk = samp[k][m];
      // the sample moved into the box by whole box edges, then its cell
      const float rel = (float)(xk - g.min[k]);
      const float tb = rel * (float)g.inv_box[k];
      const float nb = floorf(tb);
      const float u = fmaf(-nb, (float)g.box[k], rel) * (float)g.inv_step[k];
      const float fu = floorf(u);
      int id;
      if (tb - nb > kEpsCell && tb - nb < 1.0f - kEpsCell && u - fu > kEpsCell && u - fu < 1.0f - kEpsCell) {
        id = (int)fu;
      } else {
        const double d = g.box[k];
        const double x0 = dsub(xk, dmul(d, floor(ddiv(dsub(xk, g.min[k]), d))));
        id = (int)floor(ddiv(dsub(x0, g.min[k]), g.step[k]));
      }
      idx[k][m] = (id < 0 || id >= g.dims[k]) ? -1 : id;
      const float e = (float)(xk - c[k]);
      sq[k][m] = e * e;
    }
    __syncwarp();
    const int total = cnt[0] * cnt[1] * cnt[2];
    const long long sy = g.dims[2], sx = (long long)g.dims[1] * g.dims[2];
    // FP32 squared distances carry a relative error below 4 2^-24
    const float in2 = (float)(pad2 * (1.0 - 1e-6)), out2 = (float)(pad2 * (1.0 + 1e-6));
    for (int t = lane; t < total; t += kWarp) {
      const int kx = t / (cnt[1] * cnt[2]);
      const int ky = (t / cnt[2]) % cnt[1];
      const int kz = t % cnt[2];
      const int i0 = idx[0][kx], i1 = idx[1][ky], i2 = idx[2][kz];
      if (i0 < 0 || i1 < 0 || i2 < 0) continue;
      const float sf = (sq[0][kx] + sq[1][ky]) + sq[2][kz];
      bool member = sf < in2;
      if (!member && sf <= out2) {
        // the reference's FP64 test
        const double e0 = dsub(samp[0][kx], c[0]), e1 = dsub(samp[1][ky], c[1]), e2 = dsub(samp[2][kz], c[2]);
        member = dadd(dadd(dmul(e0, e0), dmul(e1, e1)), dmul(e2, e2)) < pad2;
      }
      if (member) em.put<FILL>((long long)i0 * sx + (long long)i1 * sy + i2, a, ncell);
    }
    __syncwarp();
  }
}

// --------------------------------------------------------------------------
// Per-cell rank sort (ascending atom index) and cap.
// --------------------------------------------------------------------------
constexpr int kSortWarps = 4;
constexpr int kSortBuf = 512;  // per-warp shared staging; longer lists rank from global

__global__ void __launch_bounds__(kSortWarps * kWarp) sort_cells_kernel(int* __restrict__ count,
                                                                        const int* __restrict__ start,
                                                                        int* __restrict__ entries,
                                                                        int2* __restrict__ cell,
                                                                        const TableGeom* __restrict__ gp, int cap,
                                                                        long long cell_cap, long long entry_cap,
                                                                        unsigned* __restrict__ status) {
  __shared__ int s_buf[kSortWarps][kSortBuf];
  const int wib = threadIdx.x / kWarp, lane = threadIdx.x % kWarp;
  const long long ncell = gp->ncell <= cell_cap ? gp->ncell : 0;
  if (gp->total > entry_cap) return;
  int* buf = s_buf[wib];
  for (long long c = (long long)blockIdx.x * kSortWarps + wib; c < ncell; c += (long long)gridDim.x * kSortWarps) {
    const int cnt = count[c];
    const int s = start[c];
    if (lane == 0) cell[c] = make_int2(cap > 0 && cnt > cap ? cap : cnt, s);
    if (cnt == 0) continue;
    if (cnt > kSortBuf) {
      if (cnt > kMaxSortSegment && lane == 0) atomicOr(status, kStatusSegmentTooLong);
      if (cnt > kMaxSortSegment) continue;
      // long list: ranks from global memory, results staged per lane
      int vals[kMaxSortSegment / kWarp], ranks[kMaxSortSegment / kWarp];
      int m = 0;
      for (int p = lane; p < cnt; p += kWarp, ++m) {
        const int v = entries[s + p];
        int r = 0;
        for (int q = 0; q < cnt; ++q) {
          const int u = entries[s + q];
          r += (u < v) || (u == v && q < p);
        }
        vals[m] = v;
        ranks[m] = r;
      }
      __syncwarp();
      for (int k = 0; k < m; ++k) entries[s + ranks[k]] = vals[k];
    } else {
      for (int p = lane; p < cnt; p += kWarp) buf[p] = entries[s + p];
      __syncwarp();
      for (int p = lane; p < cnt; p += kWarp) {
        const int v = buf[p];
        int r = 0;
        for (int q = 0; q < cnt; ++q) {
          const int u = buf[q];
          r += (u < v) || (u == v && q < p);
        }
        entries[s + r] = v;
      }
    }
    __syncwarp();
    if (lane == 0 && cap > 0 && cnt > cap) count[c] = cap;
  }
}

// Inline copies of each listed atom's position and parameters, so the
// volume kernels stream a cell's list without a dependent gather.
__global__ void denormalize_kernel(const int* __restrict__ entries, const TableGeom* __restrict__ gp,
                                   const float4* __restrict__ pos, const float2* __restrict__ par,
                                   float4* __restrict__ entry4, float2* __restrict__ entry_par, long long entry_cap) {
  const long long total = gp->total <= entry_cap ? gp->total : 0;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const int j = entries[e];
    entry4[e] = pos[j];
    entry_par[e] = par[j];
  }
}

}  // namespace

// Scratch the geometry pass needs: one GeomPart per 256 atoms, in doubles.
size_t table_geom_scratch_doubles(int n) {
  return ((size_t)(n + kPartThreads - 1) / kPartThreads) * (sizeof(GeomPart) / sizeof(double));
}

namespace {

int grid_for(long long work, int per_block) {
  long long b = (work + per_block - 1) / per_block;
  if (b < 1) b = 1;
  if (b > 1048576) b = 1048576;
  return (int)b;
}

}  // namespace

void launch_standalone_geom(Context* ctx, const float4* pos, TableGeom* out) {
  const gbx_config& c = ctx->cfg;
  cudaStream_t st = ctx->stream;
  const int nparts = (ctx->n + kPartThreads - 1) / kPartThreads;
  GeomPart* parts = reinterpret_cast<GeomPart*>(ctx->d_reduce);
  table_geom_partial_kernel<<<nparts, kPartThreads, 0, st>>>(pos, ctx->d_radius, ctx->n, parts);
  // no cell of this grid is ever allocated or indexed: no capacity to check
  table_geom_kernel<<<1, kGeomThreads, 0, st>>>(parts, nparts, ctx->n, GBX_TABLE_STANDALONE, c.grid_length,
                                                c.table_buffer, c.switch_width, c.box[0], c.box[1], c.box[2], out,
                                                0x7fffffffffffffffLL, ctx->d_status);
  ctx->launches += 2;
}

gbx_status launch_table_build(Context* ctx, const float4* pos) {
  const gbx_config& c = ctx->cfg;
  cudaStream_t st = ctx->stream;
  const int nparts = (ctx->n + kPartThreads - 1) / kPartThreads;
  GeomPart* parts = reinterpret_cast<GeomPart*>(ctx->d_reduce);
  table_geom_partial_kernel<<<nparts, kPartThreads, 0, st>>>(pos, ctx->d_radius, ctx->n, parts);
  table_geom_kernel<<<1, kGeomThreads, 0, st>>>(parts, nparts, ctx->n, c.table_mode, c.grid_length, c.table_buffer,
                                                c.switch_width, c.box[0], c.box[1], c.box[2], ctx->d_geom,
                                                ctx->cell_cap, ctx->d_status);
  ctx->launches += 2;
  const long long cells = ctx->cell_cap;
  if (cells == 0) {
    // sizing call: geometry only; the caller reads it back and allocates
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
      ctx->last_error = std::string("table geometry launch: ") + cudaGetErrorString(e);
      return GBX_ERR_CUDA;
    }
    return GBX_OK;
  }
  cudaMemsetAsync(ctx->d_cell_count, 0, sizeof(int) * cells, st);
  Emit em{ctx->d_cell_count, ctx->d_cell_start, ctx->d_cell_cursor, ctx->d_entries, ctx->entry_cap, ctx->d_status};
  const int threads = 256;
  const int blocks = grid_for((long long)ctx->n * kWarp, threads);
  for (int pass = 0; pass < 2; ++pass) {
    if (pass == 1) {
      launch_scan(ctx->d_cell_count, ctx->d_geom, ctx->d_block_sums, ctx->d_cell_start, ctx->d_cell_cursor, cells,
                  ctx->entry_cap, ctx->d_status, st);
      ctx->launches += 3;  // the scan's three kernels
    }
    const bool fill = pass == 1;
    switch (c.table_mode) {
      case GBX_TABLE_STANDALONE:
        if (fill)
          table_members_grid_kernel<GBX_TABLE_STANDALONE, true><<<blocks, threads, 0, st>>>(
              pos, ctx->d_radius, ctx->n, ctx->d_geom, c.grid_length, c.table_buffer, em, cells);
        else
          table_members_grid_kernel<GBX_TABLE_STANDALONE, false><<<blocks, threads, 0, st>>>(
              pos, ctx->d_radius, ctx->n, ctx->d_geom, c.grid_length, c.table_buffer, em, cells);
        break;
      case GBX_TABLE_GRID:
        if (fill)
          table_members_grid_kernel<GBX_TABLE_GRID, true><<<blocks, threads, 0, st>>>(
              pos, ctx->d_radius, ctx->n, ctx->d_geom, c.grid_length, c.table_buffer, em, cells);
        else
          table_members_grid_kernel<GBX_TABLE_GRID, false><<<blocks, threads, 0, st>>>(
              pos, ctx->d_radius, ctx->n, ctx->d_geom, c.grid_length, c.table_buffer, em, cells);
        break;
      default:
        if (fill)
          table_members_periodic_kernel<true><<<blocks, threads, 0, st>>>(pos, ctx->d_radius, ctx->n, ctx->d_geom,
                                                                          c.table_buffer, em, cells, ctx->d_status);
        else
          table_members_periodic_kernel<false><<<blocks, threads, 0, st>>>(pos, ctx->d_radius, ctx->n, ctx->d_geom,
                                                                           c.table_buffer, em, cells, ctx->d_status);
        break;
    }
    ++ctx->launches;
  }
  sort_cells_kernel<<<grid_for(cells, kSortWarps), kSortWarps * kWarp, 0, st>>>(
      ctx->d_cell_count, ctx->d_cell_start, ctx->d_entries, ctx->d_cell2, ctx->d_geom, c.table_cap, cells, ctx->entry_cap,
      ctx->d_status);
  ++ctx->launches;
  denormalize_kernel<<<grid_for(ctx->entry_cap, 256), 256, 0, st>>>(ctx->d_entries, ctx->d_geom, pos, ctx->d_par,
                                                                    ctx->d_entry4, ctx->d_entry_par, ctx->entry_cap);
  ++ctx->launches;
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    ctx->last_error = std::string("table build launch: ") + cudaGetErrorString(e);
    return GBX_ERR_CUDA;
  }
  return GBX_OK;
}

}  // namespace gbx
