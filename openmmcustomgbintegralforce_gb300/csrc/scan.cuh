// Exclusive prefix sum of per-cell counts into CSR offsets (three phases:
// per-tile sums, a single-block scan of the tile sums, per-tile apply).
// EVEN rounds each cell's allocation up to an even entry count, so every
// list starts at an even entry (a 32-byte boundary for 16-byte entries) and
// a list's entries can be read in aligned pairs without leaving the table.
// Included by the table translation units; internal linkage in each.
#pragma once

#include "gbx_internal.cuh"

namespace gbx {
namespace {

constexpr int kScanThreads = 1024;
constexpr int kScanItems = 8;

__device__ __forceinline__ int block_exclusive_scan(int v, int* s_warp, int* total) {
  const int lane = threadIdx.x % kWarp, w = threadIdx.x / kWarp;
  int x = v;
  for (int off = 1; off < kWarp; off <<= 1) {
    int y = __shfl_up_sync(0xffffffffu, x, off);
    if (lane >= off) x += y;
  }
  if (lane == kWarp - 1) s_warp[w] = x;
  __syncthreads();
  if (w == 0) {
    int s = lane < (int)(blockDim.x / kWarp) ? s_warp[lane] : 0;
    for (int off = 1; off < kWarp; off <<= 1) {
      int y = __shfl_up_sync(0xffffffffu, s, off);
      if (lane >= off) s += y;
    }
    s_warp[lane] = s;
  }
  __syncthreads();
  int base = w > 0 ? s_warp[w - 1] : 0;
  *total = s_warp[blockDim.x / kWarp - 1];
  __syncthreads();
  return base + x - v;
}

template <bool EVEN>
__device__ __forceinline__ int scan_alloc(int count) {
  return EVEN ? (count + 1) & ~1 : count;
}

template <bool EVEN>
__global__ void __launch_bounds__(kScanThreads) scan_tiles_kernel(const int* __restrict__ count,
                                                                  const TableGeom* __restrict__ gp,
                                                                  int* __restrict__ block_sums, long long cell_cap) {
  __shared__ int s_warp[kWarp];
  const long long ncell = gp->ncell <= cell_cap ? gp->ncell : 0;
  // the grid covers the capacity; tiles past this geometry's cells hold nothing
  if ((long long)blockIdx.x * kScanThreads * kScanItems >= ncell && blockIdx.x > 0) {
    if (threadIdx.x == 0) block_sums[blockIdx.x] = 0;
    return;
  }
  const long long base = (long long)blockIdx.x * kScanThreads * kScanItems + (long long)threadIdx.x * kScanItems;
  int v = 0;
  for (int k = 0; k < kScanItems; ++k)
    if (base + k < ncell) v += scan_alloc<EVEN>(count[base + k]);
  int total;
  block_exclusive_scan(v, s_warp, &total);
  if (threadIdx.x == 0) block_sums[blockIdx.x] = total;
}

__global__ void __launch_bounds__(kScanThreads) scan_top_kernel(int* __restrict__ block_sums, int nblocks) {
  __shared__ int s_warp[kWarp];
  __shared__ int s_carry;
  if (threadIdx.x == 0) s_carry = 0;
  __syncthreads();
  for (int b0 = 0; b0 < nblocks; b0 += kScanThreads) {
    int i = b0 + threadIdx.x;
    int v = i < nblocks ? block_sums[i] : 0;
    int total;
    int ex = block_exclusive_scan(v, s_warp, &total);
    if (i < nblocks) block_sums[i] = ex + s_carry;
    __syncthreads();
    if (threadIdx.x == 0) s_carry += total;
    __syncthreads();
  }
}

template <bool EVEN>
__global__ void __launch_bounds__(kScanThreads) scan_apply_kernel(const int* __restrict__ count,
                                                                  TableGeom* __restrict__ gp,
                                                                  const int* __restrict__ block_sums,
                                                                  int* __restrict__ start, int* __restrict__ cursor,
                                                                  long long cell_cap, long long entry_cap,
                                                                  unsigned* __restrict__ status) {
  __shared__ int s_warp[kWarp];
  const long long ncell = gp->ncell <= cell_cap ? gp->ncell : 0;
  if ((long long)blockIdx.x * kScanThreads * kScanItems >= ncell && blockIdx.x > 0) return;  // past the cells
  const long long base = (long long)blockIdx.x * kScanThreads * kScanItems + (long long)threadIdx.x * kScanItems;
  int v[kScanItems];
  int sum = 0;
  for (int k = 0; k < kScanItems; ++k) {
    v[k] = (base + k < ncell) ? scan_alloc<EVEN>(count[base + k]) : 0;
    sum += v[k];
  }
  int total;
  int ex = block_exclusive_scan(sum, s_warp, &total) + block_sums[blockIdx.x];
  for (int k = 0; k < kScanItems; ++k) {
    if (base + k < ncell) {
      start[base + k] = ex;
      if (cursor) cursor[base + k] = 0;
    }
    if (base + k == ncell - 1) {
      start[ncell] = ex + v[k];
      gp->total = (long long)ex + v[k];
      if ((long long)ex + v[k] > entry_cap) atomicOr(status, kStatusTableEntries);
    }
    ex += v[k];
  }
}


// Enqueue the three phases; start[ncell] and geom->total receive the sum.
template <bool EVEN = false>
inline void launch_scan(const int* count, TableGeom* geom, int* block_sums, int* start, int* cursor,
                        long long cell_cap, long long entry_cap, unsigned* status, cudaStream_t st) {
  long long nb = (cell_cap + (long long)kScanThreads * kScanItems - 1) / ((long long)kScanThreads * kScanItems);
  if (nb < 1) nb = 1;
  scan_tiles_kernel<EVEN><<<(int)nb, kScanThreads, 0, st>>>(count, geom, block_sums, cell_cap);
  scan_top_kernel<<<1, kScanThreads, 0, st>>>(block_sums, (int)nb);
  scan_apply_kernel<EVEN><<<(int)nb, kScanThreads, 0, st>>>(count, geom, block_sums, start, cursor, cell_cap, entry_cap,
                                                      status);
}

}  // namespace
}  // namespace gbx
