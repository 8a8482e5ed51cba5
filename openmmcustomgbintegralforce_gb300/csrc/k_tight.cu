// Exact GBSW lookup table.
//
// The GBSW volume of a point is V(p) = 0 if some atom buries it
// (|p - x_j| <= R'_j - w), else the product of u_j over the atoms whose
// switching shell holds it (R'_j - w < |p - x_j| < R'_j + w)
// (CharmmReferenceGBSW.cpp:616-639).  The reference's standalone table pads
// every grid point by buffer + maxR + w + (sqrt3/2) h + 1e-6 (:454-455), more
// than any shell reaches from anywhere in the queried cell, so its lists give
// exactly this V.  This table gives the same V with far shorter lists:
//
//   * cell c (edge h, default 0.1 nm) lists atom j when the distance from
//     x_j to the cell's box is below R'_j + w + eps;
//   * a cell whose farthest corner lies within R'_j - w - eps of some x_j is
//     buried: V = 0 for every point in it, no list is read;
//   * the grid spans the atoms' bounding box plus max(R') + w + h, so a
//     point outside it touches no shell (V = 1).
//
// eps (2e-5 nm plus 2 ulp of the largest coordinate) covers the FP32
// rounding of both the build and the point-to-cell assignment, so every
// atom a point needs is in the list of whichever neighbouring cell its FP32
// coordinates select.  Entries are stored inline (x, y, z, R') and sorted by
// the distance from the cell centre to the atom's burying sphere, so a
// buried point usually stops at its first entry.
#include <math.h>

#include "gbx_internal.cuh"
#include "scan.cuh"

namespace gbx {
namespace {

constexpr int kGeomThreads = 1024;
constexpr int kSortWarps = 4;
constexpr int kSortBuf = 256;
constexpr int kSortLanes = 8;                                   // lanes per short list
constexpr int kSortSmall = kSortBuf / (kWarp / kSortLanes);     // longest short list (64)

__global__ void __launch_bounds__(kGeomThreads) tight_geom_kernel(const float4* __restrict__ pos, int n, double h,
                                                                  double w, double extent, TableGeom* __restrict__ g,
                                                                  long long cell_cap, unsigned* __restrict__ status) {
  __shared__ float s_min[3][kGeomThreads / kWarp], s_max[3][kGeomThreads / kWarp], s_r[kGeomThreads / kWarp];
  const int t = threadIdx.x;
  float mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY}, rmax = 0.f;
  for (int a = t; a < n; a += blockDim.x) {
    const float4 p = pos[a];
    mn[0] = fminf(mn[0], p.x);
    mn[1] = fminf(mn[1], p.y);
    mn[2] = fminf(mn[2], p.z);
    mx[0] = fmaxf(mx[0], p.x);
    mx[1] = fmaxf(mx[1], p.y);
    mx[2] = fmaxf(mx[2], p.z);
    rmax = fmaxf(rmax, p.w);
  }
  for (int off = 16; off > 0; off >>= 1) {
    for (int k = 0; k < 3; ++k) {
      mn[k] = fminf(mn[k], __shfl_xor_sync(0xffffffffu, mn[k], off));
      mx[k] = fmaxf(mx[k], __shfl_xor_sync(0xffffffffu, mx[k], off));
    }
    rmax = fmaxf(rmax, __shfl_xor_sync(0xffffffffu, rmax, off));
  }
  if (t % kWarp == 0) {
    for (int k = 0; k < 3; ++k) {
      s_min[k][t / kWarp] = mn[k];
      s_max[k][t / kWarp] = mx[k];
    }
    s_r[t / kWarp] = rmax;
  }
  __syncthreads();
  if (t != 0) return;
  for (int ww = 0; ww < kGeomThreads / kWarp; ++ww) {
    for (int k = 0; k < 3; ++k) {
      mn[k] = fminf(mn[k], s_min[k][ww]);
      mx[k] = fmaxf(mx[k], s_max[k][ww]);
    }
    rmax = fmaxf(rmax, s_r[ww]);
  }
  TableGeom G;
  const double margin = (double)rmax + w + h;
  long long ncell = 1;
  double amax = 0.0;
  for (int k = 0; k < 3; ++k) {
    G.min[k] = (double)mn[k] - margin;
    G.dims[k] = (int)ceil(((double)mx[k] - (double)mn[k] + 2.0 * margin) / h) + 1;
    if (!(G.dims[k] >= 1 && G.dims[k] <= 65536)) {
      atomicOr(status, kStatusTableCells);
      G.dims[k] = 1;
    }
    G.max[k] = G.min[k] + G.dims[k] * h;
    G.step[k] = h;
    G.box[k] = 0.0;
    ncell *= G.dims[k];
    amax = fmax(amax, fmax(fabs((double)mn[k]), fabs((double)mx[k])));
  }
  G.mode = -1;
  G.L = h;
  // membership margin: FP32 rounding of cell coordinates and distances
  // (extent: a periodic system's longest box edge, by which a point may be moved)
  G.pad = 2e-5 + 4.0 * 1.1920929e-7 * (amax + 2.0 * margin + extent);
  G.total = 0;
  for (int k = 0; k < 3; ++k) {
    G.inv_step[k] = 1.0 / h;
    G.inv_box[k] = 0.0;
  }
  G.ncell = ncell;
  if (ncell > cell_cap) atomicOr(status, kStatusTableCells);
  *g = G;
}

struct TightArgs {
  const float4* pos;  // x, y, z, R'
  int n;
  const TableGeom* geom;
  float w;
  int* count;
  const int* start;
  int* cursor;
  int* buried;
  float4* entry;
  int* index;
  long long cell_cap, entry_cap;
  unsigned* status;
};

template <bool FILL>
__global__ void tight_members_kernel(TightArgs a) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) / kWarp;
  const int lane = threadIdx.x % kWarp;
  const TableGeom& g = *a.geom;
  if (g.ncell > a.cell_cap) return;
  const float h = (float)g.step[0];
  const float inv_h = (float)g.inv_step[0];
  const float eps = (float)g.pad;
  const long long sx = (long long)g.dims[1] * g.dims[2], sy = g.dims[2];
  for (int at = warp; at < a.n; at += (gridDim.x * blockDim.x) / kWarp) {
    const float4 p = a.pos[at];
    // coordinates relative to the grid origin, lane k forming axis k in
    // FP64 (the slow FP64 pipe is then busy for one instruction, not three)
    float xk = 0.0f;
    if (lane < 3) xk = (float)((double)(lane == 0 ? p.x : (lane == 1 ? p.y : p.z)) - g.min[lane]);
    const float x[3] = {__shfl_sync(0xffffffffu, xk, 0), __shfl_sync(0xffffffffu, xk, 1),
                        __shfl_sync(0xffffffffu, xk, 2)};
    const float reach = p.w + a.w + eps;
    const float bury = p.w - a.w - eps;
    int b[3], e[3];
    bool ok = true;
    for (int k = 0; k < 3; ++k) {
      b[k] = max(0, (int)floorf((x[k] - reach) * inv_h));
      e[k] = min(g.dims[k] - 1, (int)floorf((x[k] + reach) * inv_h));
      if (!(e[k] >= b[k] && e[k] - b[k] < 256)) ok = false;
    }
    if (!ok) {
      if (lane == 0) atomicOr(a.status, kStatusTableCells);
      continue;
    }
    const int ny = e[1] - b[1] + 1, nz = e[2] - b[2] + 1;
    const int total = (e[0] - b[0] + 1) * ny * nz;
    for (int t = lane; t < total; t += kWarp) {
      const int c[3] = {b[0] + t / (ny * nz), b[1] + (t / nz) % ny, b[2] + t % nz};
      float near2 = 0.f, far2 = 0.f;
      for (int k = 0; k < 3; ++k) {
        const float lo = c[k] * h, hi = lo + h;
        const float dn = fmaxf(fmaxf(lo - x[k], x[k] - hi), 0.f);
        const float df = fmaxf(x[k] - lo, hi - x[k]);
        near2 = fmaf(dn, dn, near2);
        far2 = fmaf(df, df, far2);
      }
      if (!(near2 < reach * reach)) continue;
      const long long cell = c[0] * sx + c[1] * sy + c[2];
      if (!FILL) {
        atomicAdd(&a.count[cell], 1);
        if (bury > 0.f && far2 <= bury * bury) atomicOr(&a.buried[cell], 1);
      } else {
        const int slot = atomicAdd(&a.cursor[cell], 1);
        const long long o = (long long)a.start[cell] + slot;
        if (o < a.entry_cap) {
          a.entry[o] = p;
          a.index[o] = at;
        } else {
          atomicOr(a.status, kStatusTableEntries);
        }
      }
    }
  }
}

// Sort each list by (distance from the cell centre to the atom's burying
// sphere, atom index) -- a deterministic order whatever the fill order was --
// and mark buried cells with count -1.
__global__ void __launch_bounds__(kSortWarps * kWarp) tight_sort_kernel(int* __restrict__ count,
                                                                        const int* __restrict__ start,
                                                                        const int* __restrict__ buried,
                                                                        float4* __restrict__ entry,
                                                                        int* __restrict__ index,
                                                                        int2* __restrict__ cell,
                                                                        TightCell* __restrict__ first,
                                                                        const TableGeom* __restrict__ gp, float w,
                                                                        long long cell_cap, long long entry_cap,
                                                                        unsigned* __restrict__ status) {
  __shared__ float4 s_e[kSortWarps][kSortBuf];
  __shared__ int s_i[kSortWarps][kSortBuf];
  __shared__ float s_k[kSortWarps][kSortBuf];
  const int wib = threadIdx.x / kWarp, lane = threadIdx.x % kWarp;
  const TableGeom& g = *gp;
  if (g.ncell > cell_cap || g.total > entry_cap) return;
  const long long ncell = g.ncell;
  const long long sx = (long long)g.dims[1] * g.dims[2];
  const float cmin[3] = {(float)g.min[0], (float)g.min[1], (float)g.min[2]};
  const float step = (float)g.step[0];
  // lanes classify 32 consecutive cells (coalesced); the warp then sorts the
  // listed, unburied ones one at a time
  for (long long c0 = ((long long)blockIdx.x * kSortWarps + wib) * kWarp; c0 < ncell;
       c0 += (long long)gridDim.x * kSortWarps * kWarp) {
    const long long c = c0 + lane;
    int cnt = 0, s = 0, bur = 0;
    if (c < ncell) {
      cnt = count[c];
      s = start[c];
      bur = cnt > 0 ? buried[c] : 0;
      cell[c] = make_int2(bur ? -1 : cnt, s);
      first[c].cs = make_int2(bur ? -1 : cnt, s);
      if (bur) count[c] = -1;
    }
    // lists of up to kSortSmall entries: four cells at a time, eight lanes
    // per cell, each group in its own quarter of the warp's buffer; longer
    // lists: the whole warp on one cell
    unsigned small = __ballot_sync(0xffffffffu, cnt > 0 && !bur && cnt <= kSortSmall);
    unsigned todo = __ballot_sync(0xffffffffu, cnt > kSortSmall && !bur);
    const int grp = lane / kSortLanes, gl = lane % kSortLanes;
    while (small) {
      unsigned t = small;
      for (int k = 0; k < grp; ++k) t &= t - 1;  // the grp-th listed cell left
      const int src = t ? __ffs(t) - 1 : -1;
      for (int k = 0; k < kWarp / kSortLanes; ++k) small &= small - 1;
      const int ccnt0 = __shfl_sync(0xffffffffu, cnt, src >= 0 ? src : 0);
      const int cs = __shfl_sync(0xffffffffu, s, src >= 0 ? src : 0);
      const int ccnt = src >= 0 ? ccnt0 : 0;
      float4* ge = s_e[wib] + grp * kSortSmall;
      int* gi = s_i[wib] + grp * kSortSmall;
      float* gk = s_k[wib] + grp * kSortSmall;
      if (ccnt > 0) {
        const long long cc = c0 + src;
        const int cx = (int)(cc / sx), cy = (int)((cc / g.dims[2]) % g.dims[1]), cz = (int)(cc % g.dims[2]);
        const float ctr[3] = {cmin[0] + ((float)cx + 0.5f) * step, cmin[1] + ((float)cy + 0.5f) * step,
                              cmin[2] + ((float)cz + 0.5f) * step};
        for (int q = gl; q < ccnt; q += kSortLanes) {
          const float4 e = entry[cs + q];
          ge[q] = e;
          gi[q] = index[cs + q];
          const float dx = e.x - ctr[0], dy = e.y - ctr[1], dz = e.z - ctr[2];
          gk[q] = sqrtf(fmaf(dx, dx, fmaf(dy, dy, dz * dz))) - (e.w - w);
        }
      }
      __syncwarp();
      for (int q = gl; q < ccnt; q += kSortLanes) {
        const float kq = gk[q];
        const int iq = gi[q];
        int r = 0;
        for (int o = 0; o < ccnt; ++o) {
          const float ko = gk[o];
          r += (ko < kq) || (ko == kq && gi[o] < iq);
        }
        entry[cs + r] = ge[q];
        index[cs + r] = iq;
        if (r == 0) first[c0 + src].first = ge[q];
      }
      __syncwarp();
    }
    while (todo) {
      const int src = __ffs(todo) - 1;
      todo &= todo - 1;
      const long long cc = c0 + src;
      const int ccnt = __shfl_sync(0xffffffffu, cnt, src), cs = __shfl_sync(0xffffffffu, s, src);
      if (ccnt > kSortBuf) {
        if (lane == 0) atomicOr(status, kStatusSegmentTooLong);
        continue;
      }
      // key: distance to the cell centre less R' - w (atoms likely to bury
      // the cell's points first); FP32, any fixed order is exact
      const int cx = (int)(cc / sx), cy = (int)((cc / g.dims[2]) % g.dims[1]), cz = (int)(cc % g.dims[2]);
      const float ctr[3] = {cmin[0] + ((float)cx + 0.5f) * step, cmin[1] + ((float)cy + 0.5f) * step,
                            cmin[2] + ((float)cz + 0.5f) * step};
      for (int q = lane; q < ccnt; q += kWarp) {
        const float4 e = entry[cs + q];
        s_e[wib][q] = e;
        s_i[wib][q] = index[cs + q];
        const float dx = e.x - ctr[0], dy = e.y - ctr[1], dz = e.z - ctr[2];
        s_k[wib][q] = sqrtf(fmaf(dx, dx, fmaf(dy, dy, dz * dz))) - (e.w - w);
      }
      __syncwarp();
      for (int q = lane; q < ccnt; q += kWarp) {
        const float kq = s_k[wib][q];
        const int iq = s_i[wib][q];
        int r = 0;
        for (int o = 0; o < ccnt; ++o) {
          const float ko = s_k[wib][o];
          r += (ko < kq) || (ko == kq && s_i[wib][o] < iq);
        }
        entry[cs + r] = s_e[wib][q];
        index[cs + r] = iq;
        if (r == 0) first[cc].first = s_e[wib][q];
      }
      __syncwarp();
    }
  }
}

}  // namespace

gbx_status launch_tight_build(Context* ctx, const float4* pos) {
  cudaStream_t st = ctx->stream;
  const double h = ctx->tight_h;
  const gbx_config& c = ctx->cfg;
  const double extent = c.periodic ? fmax(c.box[0], fmax(c.box[1], c.box[2])) : 0.0;
  if (c.periodic) launch_standalone_geom(ctx, pos, ctx->d_wgeom);
  tight_geom_kernel<<<1, kGeomThreads, 0, st>>>(pos, ctx->n, h, c.switch_width, extent, ctx->d_tgeom, ctx->tcell_cap,
                                                ctx->d_status);
  ++ctx->launches;
  const long long cells = ctx->tcell_cap;
  if (cells > 0) {
    cudaMemsetAsync(ctx->d_tcount, 0, sizeof(int) * cells, st);
    cudaMemsetAsync(ctx->d_tburied, 0, sizeof(int) * cells, st);
    TightArgs a{pos,           ctx->n,          ctx->d_tgeom,   (float)ctx->cfg.switch_width,
                ctx->d_tcount, ctx->d_tstart,   ctx->d_tcursor, ctx->d_tburied,
                ctx->d_tentry, ctx->d_tindex,   cells,          ctx->tentry_cap,
                ctx->d_status};
    const int threads = 256;
    long long blocks = ((long long)ctx->n * kWarp + threads - 1) / threads;
    if (blocks > 65535) blocks = 65535;
    tight_members_kernel<false><<<(int)blocks, threads, 0, st>>>(a);
    ++ctx->launches;
    launch_scan<true>(ctx->d_tcount, ctx->d_tgeom, ctx->d_tblock_sums, ctx->d_tstart, ctx->d_tcursor, cells,
                ctx->tentry_cap, ctx->d_status, st);
    ctx->launches += 3;  // the scan's three kernels
    tight_members_kernel<true><<<(int)blocks, threads, 0, st>>>(a);
    ++ctx->launches;
    long long sb = (cells + kSortWarps * kWarp - 1) / (kSortWarps * kWarp);
    if (sb > (long long)ctx->sms * 64) sb = (long long)ctx->sms * 64;
    tight_sort_kernel<<<(int)sb, kSortWarps * kWarp, 0, st>>>(ctx->d_tcount, ctx->d_tstart, ctx->d_tburied,
                                                               ctx->d_tentry, ctx->d_tindex, ctx->d_tcell, ctx->d_tfirst,
                                                               ctx->d_tgeom,
                                                               (float)ctx->cfg.switch_width, cells, ctx->tentry_cap,
                                                               ctx->d_status);
    ++ctx->launches;
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    ctx->last_error = std::string("tight table launch: ") + cudaGetErrorString(e);
    return GBX_ERR_CUDA;
  }
  return GBX_OK;
}

}  // namespace gbx
