// Batched evaluation of many independent molecules (uneven atom counts,
// GBSW and GBMV mixed): the batched form of the hot path.
//
// Each molecule keeps its own context (tables, record regions, quadrature),
// so every kernel of the single-molecule path is reused unchanged.  A call
// fans the molecules out over `streams` internal CUDA streams -- largest
// first, each stream taking the next molecule (longest-processing-time
// order) -- forked from and joined back to the caller's stream with events.
// After one checked call has sized every buffer, the whole fan-out is
// captured once in a CUDA graph; later calls replay it with one
// cudaGraphLaunch.  The replay ends with a kernel that ORs every context's
// status word into one, read back with a single 4-byte copy: if any table
// outgrew its capacity the batch re-runs checked (growing the buffers) and
// captures again, so a replay never returns a silently truncated result.
//
// gbx_batch_tune is the autotuner: it times the captured batch for several
// stream counts and quadrature chunkings (quadrature points per warp) and
// keeps the fastest.
#include <omp.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "gbx_internal.cuh"

struct gbx_batch {
  std::vector<gbx::Context*> mols;
  std::vector<long long> off;   // atom offset of each molecule
  std::vector<int> order;       // molecules, largest first
  long long total = 0;
  float4* d_pos = nullptr;                 // [total]
  unsigned long long* d_force = nullptr;   // [3 total]: molecule m at 3 off[m], layout [3][n_m]
  double* d_energy = nullptr;              // [molecules]
  unsigned** d_status_ptr = nullptr;       // [molecules] each context's status word
  unsigned* d_status = nullptr;            // OR of them
  unsigned* h_status = nullptr;            // pinned
  float4* h_pos = nullptr;                 // pinned [total]
  unsigned long long* h_force = nullptr;   // pinned [3 total]
  double* h_energy = nullptr;              // pinned [molecules]
  int n_streams = 8;
  std::vector<cudaStream_t> streams;
  std::vector<cudaEvent_t> joins;
  cudaEvent_t fork = nullptr;
  cudaStream_t own = nullptr;
  cudaGraphExec_t graph = nullptr;
  cudaStream_t graph_stream = nullptr;     // stream the graph was captured for
  std::vector<unsigned long long> epochs;  // each molecule's epoch at capture
  bool sized = false;                      // one checked call has run
  double* d_adj = nullptr;                 // host-form adjoint outputs (allocated on first use)
  double* h_adj = nullptr;                 // pinned copy of them
  std::string last_error;
};

namespace gbx {
namespace {

__global__ void or_status_kernel(unsigned* const* __restrict__ ptrs, int n, unsigned* __restrict__ out) {
  unsigned v = 0;
  for (int k = threadIdx.x; k < n; k += blockDim.x) v |= *ptrs[k];
  for (int off = 16; off > 0; off >>= 1) v |= __shfl_xor_sync(0xffffffffu, v, off);
  __shared__ unsigned s[32];
  if (threadIdx.x % 32 == 0) s[threadIdx.x / 32] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned r = 0;
    for (int w = 0; w < (int)(blockDim.x / 32); ++w) r |= s[w];
    *out = r;
  }
}

#define BTRY(expr)                           \
  do {                                       \
    gbx_status s_ = (expr);                  \
    if (s_ != GBX_OK) return s_;             \
  } while (0)
#define BCUDA(b, expr)                                                        \
  do {                                                                        \
    cudaError_t e_ = (expr);                                                  \
    if (e_ != cudaSuccess) {                                                  \
      (b)->last_error = std::string(#expr) + ": " + cudaGetErrorString(e_);  \
      return e_ == cudaErrorMemoryAllocation ? GBX_ERR_OUT_OF_MEMORY : GBX_ERR_CUDA; \
    }                                                                         \
  } while (0)

gbx_status make_streams(gbx_batch* b, int n) {
  for (auto s : b->streams) cudaStreamDestroy(s);
  for (auto e : b->joins) cudaEventDestroy(e);
  b->streams.assign(n, nullptr);
  b->joins.assign(n, nullptr);
  for (int k = 0; k < n; ++k) {
    BCUDA(b, cudaStreamCreateWithFlags(&b->streams[k], cudaStreamNonBlocking));
    BCUDA(b, cudaEventCreateWithFlags(&b->joins[k], cudaEventDisableTiming));
  }
  b->n_streams = n;
  return GBX_OK;
}

void drop_graph(gbx_batch* b) {
  if (b->graph) cudaGraphExecDestroy(b->graph);
  b->graph = nullptr;
  b->graph_stream = nullptr;
}

// The fan-out: every molecule's pipeline on its stream.  With check each
// context synchronises inside (table sizing) -- never under capture.
gbx_status fan_out(gbx_batch* b, cudaStream_t main, bool check) {
  BCUDA(b, cudaEventRecord(b->fork, main));
  for (auto s : b->streams) BCUDA(b, cudaStreamWaitEvent(s, b->fork, 0));
  for (size_t k = 0; k < b->order.size(); ++k) {
    const int m = b->order[k];
    Context* c = b->mols[m];
    c->stream = b->streams[k % b->streams.size()];
    unsigned long long* f = b->d_force + 3 * b->off[m];
    BCUDA(b, cudaMemsetAsync(f, 0, sizeof(unsigned long long) * 3 * c->n, c->stream));
    BCUDA(b, cudaMemsetAsync(b->d_energy + m, 0, sizeof(double), c->stream));
    const gbx_status s = pipeline(c, b->d_pos + b->off[m], f, c->n, b->d_energy + m, check, false, false, true);
    if (s != GBX_OK) {
      b->last_error = "molecule " + std::to_string(m) + ": " + c->last_error;
      return s;
    }
  }
  for (size_t k = 0; k < b->streams.size(); ++k) {
    BCUDA(b, cudaEventRecord(b->joins[k], b->streams[k]));
    BCUDA(b, cudaStreamWaitEvent(main, b->joins[k], 0));
  }
  or_status_kernel<<<1, 256, 0, main>>>(b->d_status_ptr, (int)b->mols.size(), b->d_status);
  BCUDA(b, cudaGetLastError());
  return GBX_OK;
}

gbx_status capture(gbx_batch* b, cudaStream_t main) {
  drop_graph(b);
  BCUDA(b, cudaStreamBeginCapture(main, cudaStreamCaptureModeThreadLocal));
  const gbx_status s = fan_out(b, main, false);
  cudaGraph_t g = nullptr;
  const cudaError_t e = cudaStreamEndCapture(main, &g);
  if (s != GBX_OK) {
    if (g) cudaGraphDestroy(g);
    return s;
  }
  BCUDA(b, e);
  const cudaError_t ei = cudaGraphInstantiate(&b->graph, g, 0);
  cudaGraphDestroy(g);
  BCUDA(b, ei);
  b->graph_stream = main;
  b->epochs.resize(b->mols.size());
  for (size_t m = 0; m < b->mols.size(); ++m) b->epochs[m] = b->mols[m]->epoch;
  return GBX_OK;
}

// A molecule's parameters or buffers changed since the capture.
bool graph_stale(const gbx_batch* b) {
  for (size_t m = 0; m < b->mols.size(); ++m)
    if (b->epochs[m] != b->mols[m]->epoch) return true;
  return false;
}

// Checked call: sizes every buffer, then freezes the record regions so the
// next call can be captured.
gbx_status run_checked(gbx_batch* b, cudaStream_t main) {
  drop_graph(b);
  BTRY(fan_out(b, main, true));
  BCUDA(b, cudaStreamSynchronize(main));
  for (auto c : b->mols) BTRY(fix_chain_records(c));
  b->sized = true;
  return GBX_OK;
}

gbx_status run(gbx_batch* b, cudaStream_t main, bool force_check) {
  if (force_check || !b->sized) return run_checked(b, main);
  if (!b->graph || b->graph_stream != main || graph_stale(b)) BTRY(capture(b, main));
  BCUDA(b, cudaGraphLaunch(b->graph, main));
  BCUDA(b, cudaMemcpyAsync(b->h_status, b->d_status, sizeof(unsigned), cudaMemcpyDeviceToHost, main));
  BCUDA(b, cudaStreamSynchronize(main));
  const unsigned st = *b->h_status;
  if (st & kStatusNonFinite) {
    b->last_error = "non-finite Born radius in the batch";
    return GBX_ERR_NONFINITE;
  }
  if (st & (kStatusTableCells | kStatusTableEntries | kStatusSegmentTooLong)) return run_checked(b, main);
  return GBX_OK;
}

// Device outputs of the batched adjoint, laid out by the batch's atom
// offsets (any may be null).
struct AdjOut {
  double* energies;  // [molecules]
  double* forces;    // [total][3]
  double* dEdq;      // [total]
  double* dEdR;      // [total]
  double* dEdalpha;  // [molecules][2]
};

// The adjoint fan-out: every molecule's gbx_adjoint on its stream, joined
// back and the status words ORed (as fan_out).  Not captured: each call
// launches the pipelines afresh.
gbx_status adjoint_fan_out(gbx_batch* b, cudaStream_t main, bool check, const AdjOut& o) {
  BCUDA(b, cudaEventRecord(b->fork, main));
  for (auto s : b->streams) BCUDA(b, cudaStreamWaitEvent(s, b->fork, 0));
  for (size_t k = 0; k < b->order.size(); ++k) {
    const int m = b->order[k];
    Context* c = b->mols[m];
    const long long a = b->off[m];
    const gbx_status s =
        gbx_adjoint(reinterpret_cast<gbx_context*>(c), b->d_pos + a, o.energies ? o.energies + m : nullptr,
                    o.forces ? o.forces + 3 * a : nullptr, o.dEdq ? o.dEdq + a : nullptr, o.dEdR ? o.dEdR + a : nullptr,
                    o.dEdalpha ? o.dEdalpha + 2 * m : nullptr, check ? GBX_EXEC_CHECK : 0,
                    b->streams[k % b->streams.size()]);
    if (s != GBX_OK) {
      b->last_error = "molecule " + std::to_string(m) + ": " + c->last_error;
      return s;
    }
  }
  for (size_t k = 0; k < b->streams.size(); ++k) {
    BCUDA(b, cudaEventRecord(b->joins[k], b->streams[k]));
    BCUDA(b, cudaStreamWaitEvent(main, b->joins[k], 0));
  }
  or_status_kernel<<<1, 256, 0, main>>>(b->d_status_ptr, (int)b->mols.size(), b->d_status);
  BCUDA(b, cudaGetLastError());
  return GBX_OK;
}

// Unchecked fan-out, re-run checked when a table outgrew its buffers.
gbx_status run_adjoint(gbx_batch* b, cudaStream_t main, bool force_check, const AdjOut& o) {
  BTRY(adjoint_fan_out(b, main, force_check, o));
  BCUDA(b, cudaMemcpyAsync(b->h_status, b->d_status, sizeof(unsigned), cudaMemcpyDeviceToHost, main));
  BCUDA(b, cudaStreamSynchronize(main));
  unsigned st = *b->h_status;
  if (!force_check && (st & (kStatusTableCells | kStatusTableEntries | kStatusSegmentTooLong))) {
    BTRY(adjoint_fan_out(b, main, true, o));
    BCUDA(b, cudaMemcpyAsync(b->h_status, b->d_status, sizeof(unsigned), cudaMemcpyDeviceToHost, main));
    BCUDA(b, cudaStreamSynchronize(main));
    st = *b->h_status;
  }
  if (st & kStatusNonFinite) {
    b->last_error = "non-finite Born radius in the batch";
    return GBX_ERR_NONFINITE;
  }
  return GBX_OK;
}

}  // namespace
}  // namespace gbx

extern "C" {

gbx_status gbx_batch_create(const gbx_config* configs, const int* n_atoms, int n_molecules, gbx_batch** out) {
  if (!configs || !n_atoms || n_molecules <= 0 || !out) return GBX_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  gbx_batch* b = new gbx_batch();
  gbx_status s = GBX_OK;
  b->mols.assign(n_molecules, nullptr);
  b->off.assign(n_molecules, 0);
  for (int m = 0; m < n_molecules && s == GBX_OK; ++m) {
    if (n_atoms[m] <= 0) s = GBX_ERR_INVALID_ARGUMENT;
    else s = gbx_create(&configs[m], n_atoms[m], reinterpret_cast<gbx_context**>(&b->mols[m]));
    if (s == GBX_OK) {
      b->off[m] = b->total;
      b->total += n_atoms[m];
    }
  }
  auto fail = [&](gbx_status st) {
    gbx_batch_destroy(b);
    return st;
  };
  if (s != GBX_OK) return fail(s);
  b->order.resize(n_molecules);
  std::iota(b->order.begin(), b->order.end(), 0);
  std::stable_sort(b->order.begin(), b->order.end(), [&](int x, int y) { return n_atoms[x] > n_atoms[y]; });
  auto cu = [&](cudaError_t e) { return e == cudaSuccess ? GBX_OK : GBX_ERR_CUDA; };
  if ((s = cu(cudaMalloc((void**)&b->d_pos, sizeof(float4) * b->total))) != GBX_OK ||
      (s = cu(cudaMalloc((void**)&b->d_force, sizeof(unsigned long long) * 3 * b->total))) != GBX_OK ||
      (s = cu(cudaMalloc((void**)&b->d_energy, sizeof(double) * n_molecules))) != GBX_OK ||
      (s = cu(cudaMalloc((void**)&b->d_status_ptr, sizeof(unsigned*) * n_molecules))) != GBX_OK ||
      (s = cu(cudaMalloc((void**)&b->d_status, sizeof(unsigned)))) != GBX_OK ||
      (s = cu(cudaMallocHost((void**)&b->h_status, sizeof(unsigned)))) != GBX_OK ||
      (s = cu(cudaMallocHost((void**)&b->h_pos, sizeof(float4) * b->total))) != GBX_OK ||
      (s = cu(cudaMallocHost((void**)&b->h_force, sizeof(unsigned long long) * 3 * b->total))) != GBX_OK ||
      (s = cu(cudaMallocHost((void**)&b->h_energy, sizeof(double) * n_molecules))) != GBX_OK ||
      (s = cu(cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming))) != GBX_OK ||
      (s = cu(cudaStreamCreateWithFlags(&b->own, cudaStreamNonBlocking))) != GBX_OK)
    return fail(s);
  std::vector<unsigned*> ptrs(n_molecules);
  for (int m = 0; m < n_molecules; ++m) ptrs[m] = b->mols[m]->d_status;
  if ((s = cu(cudaMemcpy(b->d_status_ptr, ptrs.data(), sizeof(unsigned*) * n_molecules, cudaMemcpyHostToDevice))) !=
      GBX_OK)
    return fail(s);
  if ((s = gbx::make_streams(b, std::min(n_molecules, 8))) != GBX_OK) return fail(s);
  *out = b;
  return GBX_OK;
}

gbx_status gbx_batch_destroy(gbx_batch* b) {
  if (!b) return GBX_ERR_INVALID_ARGUMENT;
  cudaDeviceSynchronize();
  gbx::drop_graph(b);
  for (auto c : b->mols)
    if (c) gbx_destroy(reinterpret_cast<gbx_context*>(c));
  for (auto s : b->streams) cudaStreamDestroy(s);
  for (auto e : b->joins) cudaEventDestroy(e);
  if (b->fork) cudaEventDestroy(b->fork);
  if (b->own) cudaStreamDestroy(b->own);
  for (void* p : {(void*)b->d_pos, (void*)b->d_force, (void*)b->d_energy, (void*)b->d_status_ptr, (void*)b->d_status,
                  (void*)b->d_adj})
    if (p) cudaFree(p);
  for (void* p : {(void*)b->h_status, (void*)b->h_pos, (void*)b->h_force, (void*)b->h_energy, (void*)b->h_adj})
    if (p) cudaFreeHost(p);
  delete b;
  return GBX_OK;
}

gbx_status gbx_batch_molecule(gbx_batch* b, int m, gbx_context** ctx, long long* atom_offset) {
  if (!b || m < 0 || m >= (int)b->mols.size()) return GBX_ERR_INVALID_ARGUMENT;
  if (ctx) *ctx = reinterpret_cast<gbx_context*>(b->mols[m]);
  if (atom_offset) *atom_offset = b->off[m];
  return GBX_OK;
}

gbx_status gbx_batch_buffers(gbx_batch* b, void** posq, unsigned long long** forces, double** energies,
                             long long* total_atoms) {
  if (!b) return GBX_ERR_INVALID_ARGUMENT;
  if (posq) *posq = b->d_pos;
  if (forces) *forces = b->d_force;
  if (energies) *energies = b->d_energy;
  if (total_atoms) *total_atoms = b->total;
  return GBX_OK;
}

gbx_status gbx_batch_execute(gbx_batch* b, int flags, void* stream) {
  if (!b) return GBX_ERR_INVALID_ARGUMENT;
  return gbx::run(b, stream ? (cudaStream_t)stream : b->own, (flags & GBX_EXEC_CHECK) != 0);
}

// The host loops over every atom of the batch run on up to 8 host threads
// (each element is written by one thread: the results do not depend on it).
gbx_status gbx_batch_execute_host(gbx_batch* b, const double* positions, double* forces, double* energies) {
  if (!b || !positions) return GBX_ERR_INVALID_ARGUMENT;
  const int threads = std::max(1, std::min(8, omp_get_num_procs()));
  bool finite = true;
  float4* hp = b->h_pos;
#pragma omp parallel for reduction(&& : finite) num_threads(threads)
  for (long long k = 0; k < b->total; ++k) {
    const double x = positions[3 * k], y = positions[3 * k + 1], z = positions[3 * k + 2];
    hp[k] = make_float4((float)x, (float)y, (float)z, 0.f);
    finite = std::isfinite(x) && std::isfinite(y) && std::isfinite(z) && finite;
  }
  if (!finite) {
    b->last_error = "non-finite position";
    return GBX_ERR_INVALID_ARGUMENT;
  }
  BCUDA(b, cudaMemcpyAsync(b->d_pos, b->h_pos, sizeof(float4) * b->total, cudaMemcpyHostToDevice, b->own));
  BTRY(gbx::run(b, b->own, false));
  BCUDA(b, cudaMemcpyAsync(b->h_force, b->d_force, sizeof(unsigned long long) * 3 * b->total, cudaMemcpyDeviceToHost,
                           b->own));
  BCUDA(b, cudaMemcpyAsync(b->h_energy, b->d_energy, sizeof(double) * b->mols.size(), cudaMemcpyDeviceToHost,
                           b->own));
  BCUDA(b, cudaStreamSynchronize(b->own));
  const int nm = (int)b->mols.size();
#pragma omp parallel for schedule(dynamic) num_threads(threads)
  for (int m = 0; m < nm; ++m) {
    const int n = b->mols[m]->n;
    const unsigned long long* f = b->h_force + 3 * b->off[m];
    if (forces)
      for (int i = 0; i < n; ++i)
        for (int k = 0; k < 3; ++k) forces[3 * (b->off[m] + i) + k] = gbx::fixed_to_double(f[(size_t)k * n + i]);
    if (energies) energies[m] = b->h_energy[m];
  }
  return GBX_OK;
}

gbx_status gbx_batch_adjoint(gbx_batch* b, double* energies, double* forces, double* dEdq, double* dEdR,
                             double* dEdalpha, int flags, void* stream) {
  if (!b) return GBX_ERR_INVALID_ARGUMENT;
  return gbx::run_adjoint(b, stream ? (cudaStream_t)stream : b->own, (flags & GBX_EXEC_CHECK) != 0,
                          gbx::AdjOut{energies, forces, dEdq, dEdR, dEdalpha});
}

gbx_status gbx_batch_adjoint_host(gbx_batch* b, const double* positions, double* energies, double* forces,
                                  double* dEdq, double* dEdR, double* dEdalpha) {
  if (!b || !positions) return GBX_ERR_INVALID_ARGUMENT;
  const long long T = b->total, M = (long long)b->mols.size();
  const size_t len = (size_t)(M + 3 * T + T + T + 2 * M);
  if (!b->d_adj) {
    BCUDA(b, cudaMalloc((void**)&b->d_adj, sizeof(double) * len));
    BCUDA(b, cudaMallocHost((void**)&b->h_adj, sizeof(double) * len));
  }
  const int threads = std::max(1, std::min(8, omp_get_num_procs()));
  bool finite = true;
  float4* hp = b->h_pos;
#pragma omp parallel for reduction(&& : finite) num_threads(threads)
  for (long long k = 0; k < T; ++k) {
    const double x = positions[3 * k], y = positions[3 * k + 1], z = positions[3 * k + 2];
    hp[k] = make_float4((float)x, (float)y, (float)z, 0.f);
    finite = std::isfinite(x) && std::isfinite(y) && std::isfinite(z) && finite;
  }
  if (!finite) {
    b->last_error = "non-finite position";
    return GBX_ERR_INVALID_ARGUMENT;
  }
  double* d = b->d_adj;
  const gbx::AdjOut o{d, d + M, d + M + 3 * T, d + M + 4 * T, d + M + 5 * T};
  BCUDA(b, cudaMemcpyAsync(b->d_pos, b->h_pos, sizeof(float4) * T, cudaMemcpyHostToDevice, b->own));
  BTRY(gbx::run_adjoint(b, b->own, false, o));
  BCUDA(b, cudaMemcpyAsync(b->h_adj, b->d_adj, sizeof(double) * len, cudaMemcpyDeviceToHost, b->own));
  BCUDA(b, cudaStreamSynchronize(b->own));
  const double* h = b->h_adj;
  if (energies) std::memcpy(energies, h, sizeof(double) * M);
  if (forces) std::memcpy(forces, h + M, sizeof(double) * 3 * T);
  if (dEdq) std::memcpy(dEdq, h + M + 3 * T, sizeof(double) * T);
  if (dEdR) std::memcpy(dEdR, h + M + 4 * T, sizeof(double) * T);
  if (dEdalpha) std::memcpy(dEdalpha, h + M + 5 * T, sizeof(double) * 2 * M);
  return GBX_OK;
}

gbx_status gbx_batch_tune(gbx_batch* b, int* streams_chosen, int* chunk_scale_chosen, double* ms_best) {
  if (!b) return GBX_ERR_INVALID_ARGUMENT;
  cudaStream_t main = b->own;
  if (!b->sized) BTRY(gbx::run_checked(b, main));
  std::vector<int> base_chunks(b->mols.size());
  for (size_t m = 0; m < b->mols.size(); ++m) base_chunks[m] = b->mols[m]->n_chunks;
  // destroyed on every exit, early error returns included
  struct Events {
    cudaEvent_t a = nullptr, b = nullptr;
    ~Events() {
      if (a) cudaEventDestroy(a);
      if (b) cudaEventDestroy(b);
    }
  } ev;
  BCUDA(b, cudaEventCreate(&ev.a));
  BCUDA(b, cudaEventCreate(&ev.b));
  cudaEvent_t t0 = ev.a, t1 = ev.b;
  double best = 1e30;
  int best_s = b->n_streams, best_div = 1;
  const int nm = (int)b->mols.size();
  for (int div : {1, 2, 4}) {  // quadrature chunks per atom divided by div: more points per warp
    for (size_t m = 0; m < b->mols.size(); ++m)
      BTRY(gbx::set_chunks(b->mols[m], std::max(1, base_chunks[m] / div)));
    BTRY(gbx::run_checked(b, main));
    for (int s : {4, 8, 16, 32}) {
      if (s > nm && s != 4) continue;
      BTRY(gbx::make_streams(b, std::min(s, nm)));
      gbx::drop_graph(b);
      BTRY(gbx::run(b, main, false));  // capture + warm replay
      BCUDA(b, cudaEventRecord(t0, main));
      for (int r = 0; r < 3; ++r) BTRY(gbx::run(b, main, false));
      BCUDA(b, cudaEventRecord(t1, main));
      BCUDA(b, cudaEventSynchronize(t1));
      float ms = 0;
      BCUDA(b, cudaEventElapsedTime(&ms, t0, t1));
      if (ms / 3 < best) {
        best = ms / 3;
        best_s = std::min(s, nm);
        best_div = div;
      }
    }
  }
  for (size_t m = 0; m < b->mols.size(); ++m) BTRY(gbx::set_chunks(b->mols[m], std::max(1, base_chunks[m] / best_div)));
  BTRY(gbx::make_streams(b, best_s));
  BTRY(gbx::run_checked(b, main));
  if (streams_chosen) *streams_chosen = best_s;
  if (chunk_scale_chosen) *chunk_scale_chosen = best_div;
  if (ms_best) *ms_best = best;
  return GBX_OK;
}

gbx_status gbx_batch_last_error(gbx_batch* b, char* buf, size_t len) {
  if (!b || !buf || len == 0) return GBX_ERR_INVALID_ARGUMENT;
  std::strncpy(buf, b->last_error.c_str(), len - 1);
  buf[len - 1] = 0;
  return GBX_OK;
}

}  // extern "C"
