// Stand-in for OpenMM's openmm/TabulatedFunction.h (test infrastructure):
// the base class and Continuous1DFunction with the accessor a kernel reads.
#pragma once
#include <vector>

namespace OpenMM {
class TabulatedFunction {
 public:
  virtual ~TabulatedFunction() {}
};

class Continuous1DFunction : public TabulatedFunction {
 public:
  Continuous1DFunction(const std::vector<double>& values, double min, double max)
      : values_(values), min_(min), max_(max) {}
  void getFunctionParameters(std::vector<double>& values, double& min, double& max) const {
    values = values_;
    min = min_;
    max = max_;
  }

 private:
  std::vector<double> values_;
  double min_, max_;
};

class Discrete1DFunction : public TabulatedFunction {
 public:
  explicit Discrete1DFunction(const std::vector<double>& values) : values_(values) {}

 private:
  std::vector<double> values_;
};
}  // namespace OpenMM
