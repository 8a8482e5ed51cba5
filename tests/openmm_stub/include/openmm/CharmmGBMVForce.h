// Stand-in for the plugin's openmm/CharmmGBMVForce.h (test infrastructure):
// the CustomGBForce-style accessors of CharmmGBMVForce (CharmmGBMVForce.h:
// 63-526 in the reference plugin) that a kernel reads.
#pragma once
#include "openmm/TabulatedFunction.h"
#include <memory>
#include <string>
#include <utility>
#include <vector>

namespace OpenMM {
class CharmmGBMVForce {
 public:
  enum NonbondedMethod { NoCutoff = 0, CutoffNonPeriodic = 1, CutoffPeriodic = 2 };
  enum ComputationType { SingleParticle = 0, ParticlePair = 1, ParticlePairNoExclusions = 2 };
  enum GBIntegralType { GBSWIntegral = 0, GBMVIntegralTypeI = 1, GBMVIntegralTypeII = 2, CustomIntegral = 3 };

  int getNumParticles() const { return (int)params_.size(); }
  int getNumPerParticleParameters() const { return (int)pnames_.size(); }
  int getNumGlobalParameters() const { return (int)gnames_.size(); }
  int getNumComputedValues() const { return (int)values_.size(); }
  int getNumGBIntegrals() const { return (int)integrals_.size(); }
  int getNumEnergyTerms() const { return (int)terms_.size(); }
  int getNumExclusions() const { return (int)exclusions_.size(); }
  int getNumEnergyParameterDerivatives() const { return (int)derivs_.size(); }
  int getNumTabulatedFunctions() const { return (int)functions_.size(); }
  NonbondedMethod getNonbondedMethod() const { return method_; }
  void setNonbondedMethod(NonbondedMethod m) { method_ = m; }
  double getCutoffDistance() const { return cutoff_; }
  void setCutoffDistance(double d) { cutoff_ = d; }
  int addPerParticleParameter(const std::string& name) {
    pnames_.push_back(name);
    return (int)pnames_.size() - 1;
  }
  const std::string& getPerParticleParameterName(int index) const { return pnames_[index]; }
  int addGlobalParameter(const std::string& name, double defaultValue) {
    gnames_.push_back(name);
    gdefaults_.push_back(defaultValue);
    return (int)gnames_.size() - 1;
  }
  const std::string& getGlobalParameterName(int index) const { return gnames_[index]; }
  double getGlobalParameterDefaultValue(int index) const { return gdefaults_[index]; }
  int addParticle(const std::vector<double>& parameters) {
    params_.push_back(parameters);
    return (int)params_.size() - 1;
  }
  void getParticleParameters(int index, std::vector<double>& parameters) const { parameters = params_[index]; }
  void setParticleParameters(int index, const std::vector<double>& parameters) { params_[index] = parameters; }
  int addComputedValue(const std::string& name, const std::string& expression, ComputationType type) {
    values_.push_back({name, expression, type});
    return (int)values_.size() - 1;
  }
  void getComputedValueParameters(int index, std::string& name, std::string& expression, ComputationType& type) const {
    name = values_[index].name;
    expression = values_[index].expr;
    type = values_[index].type;
  }
  int addGBIntegral(const std::string& name, const std::vector<int>& parametersInt = std::vector<int>(),
                    const std::vector<double>& parametersReal = std::vector<double>()) {
    integrals_.push_back({name, parametersInt, parametersReal});
    return (int)integrals_.size() - 1;
  }
  void getGBIntegralParameters(int index, std::string& name, std::vector<int>& parametersInt,
                               std::vector<double>& parametersReal) const {
    name = integrals_[index].name;
    parametersInt = integrals_[index].ints;
    parametersReal = integrals_[index].reals;
  }
  void setGBIntegralType(GBIntegralType type) { itype_ = type; }
  GBIntegralType getGBIntegralType() const { return itype_; }
  int addEnergyTerm(const std::string& expression, ComputationType type) {
    terms_.push_back({"", expression, type});
    return (int)terms_.size() - 1;
  }
  void getEnergyTermParameters(int index, std::string& expression, ComputationType& type) const {
    expression = terms_[index].expr;
    type = terms_[index].type;
  }
  int addExclusion(int particle1, int particle2) {
    exclusions_.push_back({particle1, particle2});
    return (int)exclusions_.size() - 1;
  }
  void getExclusionParticles(int index, int& particle1, int& particle2) const {
    particle1 = exclusions_[index].first;
    particle2 = exclusions_[index].second;
  }
  void addEnergyParameterDerivative(const std::string& name) {
    for (size_t k = 0; k < gnames_.size(); ++k)
      if (gnames_[k] == name) derivs_.push_back((int)k);
  }
  const std::string& getEnergyParameterDerivativeName(int index) const { return gnames_[derivs_[index]]; }
  // the force takes ownership of the function (CharmmGBMVForce.h:434-442)
  int addTabulatedFunction(const std::string& name, TabulatedFunction* function) {
    functions_.push_back({name, std::shared_ptr<TabulatedFunction>(function)});
    return (int)functions_.size() - 1;
  }
  const TabulatedFunction& getTabulatedFunction(int index) const { return *functions_[index].second; }
  const std::string& getTabulatedFunctionName(int index) const { return functions_[index].first; }

 private:
  struct Expr {
    std::string name, expr;
    ComputationType type;
  };
  struct Integral {
    std::string name;
    std::vector<int> ints;
    std::vector<double> reals;
  };
  std::vector<std::string> pnames_, gnames_;
  std::vector<double> gdefaults_;
  std::vector<std::vector<double>> params_;
  std::vector<Expr> values_, terms_;
  std::vector<Integral> integrals_;
  std::vector<std::pair<int, int>> exclusions_;
  std::vector<int> derivs_;
  std::vector<std::pair<std::string, std::shared_ptr<TabulatedFunction>>> functions_;
  GBIntegralType itype_ = GBSWIntegral;
  NonbondedMethod method_ = NoCutoff;
  double cutoff_ = 1.0;
};
}  // namespace OpenMM
