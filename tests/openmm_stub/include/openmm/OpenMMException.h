// Stand-in for OpenMM's openmm/OpenMMException.h (test infrastructure): just
// enough of the OpenMM surface to compile and exercise the GB300 plugin
// adapter without an OpenMM installation.
#pragma once
#include <exception>
#include <string>

namespace OpenMM {
class OpenMMException : public std::exception {
 public:
  explicit OpenMMException(const std::string& message) : message_(message) {}
  const char* what() const noexcept override { return message_.c_str(); }

 private:
  std::string message_;
};
}  // namespace OpenMM
