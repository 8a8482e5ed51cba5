// Kernel factory and plugin entry points: OpenMM dlopens the plugin library
// and calls registerKernelFactories(), which puts the GB300 kernels on every
// CUDA platform for the two kernel names of charmmKernels.h -- the entry
// points of the reference plugin's CharmmCudaKernelFactory.cpp:37-69.
#include "CudaPlatform.h"
#include "GB300CharmmKernels.h"
#include "openmm/KernelFactory.h"
#include "openmm/OpenMMException.h"
#include "openmm/internal/ContextImpl.h"

#if defined(_WIN32)
#define GB300_PLUGIN_EXPORT __declspec(dllexport)
#else
#define GB300_PLUGIN_EXPORT __attribute__((visibility("default")))
#endif

namespace GB300 {

class GB300CharmmKernelFactory : public OpenMM::KernelFactory {
 public:
  OpenMM::KernelImpl* createKernelImpl(std::string name, const OpenMM::Platform& platform,
                                       OpenMM::ContextImpl& context) const override {
    auto& data = *static_cast<OpenMM::CudaPlatform::PlatformData*>(context.getPlatformData());
    if (data.contexts.size() != 1)
      throw OpenMM::OpenMMException("GB300 GB kernels run on one GPU per context");
    OpenMM::CudaContext& cu = *data.contexts[0];
    if (name == OpenMM::CalcCharmmGBSWForceKernel::Name())
      return new GB300CalcCharmmGBSWForceKernel(name, platform, cu);
    if (name == OpenMM::CalcCharmmGBMVForceKernel::Name())
      return new GB300CalcCharmmGBMVForceKernel(name, platform, cu);
    throw OpenMM::OpenMMException("Tried to create kernel with illegal kernel name '" + name + "'");
  }
};

}  // namespace GB300

extern "C" GB300_PLUGIN_EXPORT void registerPlatforms() {}

extern "C" GB300_PLUGIN_EXPORT void registerKernelFactories() {
  for (int i = 0; i < OpenMM::Platform::getNumPlatforms(); ++i) {
    OpenMM::Platform& platform = OpenMM::Platform::getPlatform(i);
    if (dynamic_cast<OpenMM::CudaPlatform*>(&platform) != nullptr) {
      auto* factory = new GB300::GB300CharmmKernelFactory();
      platform.registerKernelFactory(OpenMM::CalcCharmmGBSWForceKernel::Name(), factory);
      platform.registerKernelFactory(OpenMM::CalcCharmmGBMVForceKernel::Name(), factory);
    }
  }
}
