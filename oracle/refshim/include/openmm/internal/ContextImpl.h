#ifndef REFSHIM_CONTEXTIMPL_H
#define REFSHIM_CONTEXTIMPL_H
namespace OpenMM {
class ContextImpl {
 public:
  explicit ContextImpl(void* data = 0) : data_(data) {}
  void* getPlatformData() { return data_; }
 private:
  void* data_;
};
}  // namespace OpenMM
#endif
