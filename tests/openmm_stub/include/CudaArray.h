// Stand-in for OpenMM's CUDA platform CudaArray (test infrastructure): a
// device buffer known by its address.
#pragma once
#include <cuda.h>

namespace OpenMM {
class CudaArray {
 public:
  explicit CudaArray(CUdeviceptr p = 0) : ptr_(p) {}
  CUdeviceptr& getDevicePointer() { return ptr_; }

 private:
  CUdeviceptr ptr_;
};
}  // namespace OpenMM
