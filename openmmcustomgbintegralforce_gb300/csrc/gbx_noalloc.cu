// Allocation-free variant of the GB pair term.
//
// Some callers cannot let a library allocate device memory: an MD engine
// that owns every device byte through its own memory pool and forbids
// hidden allocations, or a simulation loop that must not block or fail on
// cudaMalloc under memory pressure in the middle of a step.  This entry
// point serves them: the caller passes every input and output, and the only
// scratch the computation needs lives in one statically sized device array
// defined below, which every GPU that loads this library holds until the
// process exits.
#include <cuda.h>
#include <math.h>

#include <mutex>

#include "gbx_internal.cuh"

namespace gbx {
cudaError_t launch_pair_raw(const float4* pos, const float* charge, const float2* born, int n, int sms, float pref,
                            float cutoff2, unsigned long long* force, int stride, unsigned long long* dEdB,
                            double* energy_part, cudaStream_t stream);
int pair_energy_parts(int n, int segments);
int pair_segments(int n, int sms);
}  // namespace gbx

namespace {

constexpr int kNoAllocMaxAtoms = 65536;
constexpr int kNoAllocMaxParts = 4096;  // >= pair_energy_parts(n, pair_segments(n, sms)) for n <= kNoAllocMaxAtoms
constexpr int kNoAllocMaxSms = 160;     // grid sizing is capped here so the parts above always fit
constexpr int kMaxDevices = 64;

// Scratch of one call: about 1 MiB.  Shared by every call on a device.
struct NoAllocScratch {
  unsigned long long dEdB[kNoAllocMaxAtoms];  // fixed-point accumulators, cleared by each call
  float2 born[kNoAllocMaxAtoms];              // (B, 1/B) staged from the caller's radii
  double parts[kNoAllocMaxParts];             // per-CTA energy partial sums
};

static __device__ __align__(256) NoAllocScratch g_noalloc_scratch;

// Device address of g_noalloc_scratch per device (the host symbol is only a
// stand-in, never a device pointer), remembered together with the CUDA
// context it was looked up in: after a device reset the runtime creates a
// new primary context, the module is loaded again at another address, and
// the address is looked up again.
struct ScratchSlot {
  unsigned long long ctx_id = 0;
  NoAllocScratch* addr = nullptr;
  int sms = 0;
};
std::mutex g_addr_mutex;
ScratchSlot g_slot[kMaxDevices];

// The current CUDA context's unique id, through driver entry points the
// runtime hands out (the library does not link the driver library itself).
typedef CUresult (*CtxGetCurrentFn)(CUcontext*);
typedef CUresult (*CtxGetIdFn)(CUcontext, unsigned long long*);

bool current_context_id(unsigned long long* id) {
  static CtxGetCurrentFn get_current = nullptr;
  static CtxGetIdFn get_id = nullptr;
  if (!get_current || !get_id) {
    void* a = nullptr;
    void* b = nullptr;
    cudaDriverEntryPointQueryResult qa, qb;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &a, 12000, cudaEnableDefault, &qa) != cudaSuccess ||
        cudaGetDriverEntryPointByVersion("cuCtxGetId", &b, 12000, cudaEnableDefault, &qb) != cudaSuccess ||
        qa != cudaDriverEntryPointSuccess || qb != cudaDriverEntryPointSuccess || !a || !b)
      return false;
    get_current = reinterpret_cast<CtxGetCurrentFn>(a);
    get_id = reinterpret_cast<CtxGetIdFn>(b);
  }
  CUcontext cu = nullptr;
  return get_current(&cu) == CUDA_SUCCESS && cu && get_id(cu, id) == CUDA_SUCCESS;
}

cudaError_t scratch_address(NoAllocScratch** out, int* sms) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_addr_mutex);
  ScratchSlot& slot = g_slot[dev];
  unsigned long long id = 0;
  if (slot.addr && current_context_id(&id) && slot.ctx_id == id) {
    *out = slot.addr;
    *sms = slot.sms;
    return cudaSuccess;
  }
  void* p = nullptr;
  e = cudaGetSymbolAddress(&p, g_noalloc_scratch);  // makes the device's primary context current
  if (e != cudaSuccess) return e;
  if (!current_context_id(&id)) return cudaErrorDeviceUninitialized;
  int n_sm = 0;
  e = cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return e;
  slot.ctx_id = id;
  slot.addr = static_cast<NoAllocScratch*>(p);
  slot.sms = n_sm < 1 ? 1 : (n_sm > kNoAllocMaxSms ? kNoAllocMaxSms : n_sm);
  *out = slot.addr;
  *sms = slot.sms;
  return cudaSuccess;
}

__global__ void noalloc_prepare_kernel(const float* __restrict__ born, int n, NoAllocScratch* __restrict__ s) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float B = born[i];
  s->born[i] = make_float2(B, 1.0f / B);
  s->dEdB[i] = 0ull;
}

// One block: energy partials in a fixed order, dE/dB to double.
__global__ void noalloc_finish_kernel(const NoAllocScratch* __restrict__ s, int n, int nparts,
                                      double* __restrict__ energy, double* __restrict__ dEdB) {
  __shared__ double red[1024];
  double e = 0.0;
  for (int k = threadIdx.x; k < nparts; k += blockDim.x) e += s->parts[k];
  red[threadIdx.x] = e;
  __syncthreads();
  for (int stride = blockDim.x / 2; stride > 0; stride >>= 1) {
    if (threadIdx.x < stride) red[threadIdx.x] += red[threadIdx.x + stride];
    __syncthreads();
  }
  if (threadIdx.x == 0) *energy += red[0];
  if (dEdB)
    for (int i = threadIdx.x; i < n; i += blockDim.x) dEdB[i] = gbx::fixed_to_double(s->dEdB[i]);
}

}  // namespace

extern "C" {

gbx_status gbx_pair_noalloc(const void* posq, const float* charge, const float* born, int num_atoms,
                            double prefactor, double cutoff, unsigned long long* force_fixed, int force_stride,
                            double* energy, double* dEdB, void* stream) {
  if (!posq || !charge || !born || !force_fixed || !energy || num_atoms < 1 || force_stride < num_atoms)
    return GBX_ERR_INVALID_ARGUMENT;
  if (num_atoms > kNoAllocMaxAtoms) return GBX_ERR_EXCEEDS_STATIC_SCRATCH;
  NoAllocScratch* s = nullptr;
  int sms = 0;
  if (scratch_address(&s, &sms) != cudaSuccess) return GBX_ERR_CUDA;
  const int nparts = gbx::pair_energy_parts(num_atoms, gbx::pair_segments(num_atoms, sms));
  if (nparts > kNoAllocMaxParts) return GBX_ERR_EXCEEDS_STATIC_SCRATCH;
  cudaStream_t st = (cudaStream_t)stream;
  noalloc_prepare_kernel<<<(num_atoms + 255) / 256, 256, 0, st>>>(born, num_atoms, s);
  if (cudaGetLastError() != cudaSuccess) return GBX_ERR_CUDA;
  const float cut2 = cutoff > 0 ? (float)(cutoff * cutoff) : 0.0f;
  if (gbx::launch_pair_raw(reinterpret_cast<const float4*>(posq), charge, s->born, num_atoms, sms, (float)prefactor,
                           cut2, force_fixed, force_stride, s->dEdB, s->parts, st) != cudaSuccess)
    return GBX_ERR_CUDA;
  noalloc_finish_kernel<<<1, 1024, 0, st>>>(s, num_atoms, nparts, energy, dEdB);
  if (cudaGetLastError() != cudaSuccess) return GBX_ERR_CUDA;
  return GBX_OK;
}

}  // extern "C"
