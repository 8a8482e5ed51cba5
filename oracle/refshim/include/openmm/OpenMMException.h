#ifndef REFSHIM_OPENMMEXCEPTION_H
#define REFSHIM_OPENMMEXCEPTION_H
#include <stdexcept>
#include <string>
namespace OpenMM {
class OpenMMException : public std::runtime_error {
 public:
  explicit OpenMMException(const std::string& m) : std::runtime_error(m) {}
};
}  // namespace OpenMM
#endif
