// Stand-in for the plugin's openmm/CharmmGBSWForce.h (test infrastructure):
// the accessors of CharmmGBSWForce (CharmmGBSWForce.h:58-203 in the
// reference plugin) that a kernel reads.
#pragma once
#include <vector>

namespace OpenMM {
class CharmmGBSWForce {
 public:
  enum NonbondedMethod { NoCutoff = 0, CutoffNonPeriodic = 1, CutoffPeriodic = 2 };
  int getNumParticles() const { return (int)q_.size(); }
  int addParticle(double charge, double radius, double scalingFactor) {
    q_.push_back(charge);
    r_.push_back(radius);
    s_.push_back(scalingFactor);
    return (int)q_.size() - 1;
  }
  void getParticleParameters(int index, double& charge, double& radius, double& scalingFactor) const {
    charge = q_[index];
    radius = r_[index];
    scalingFactor = s_[index];
  }
  void setParticleParameters(int index, double charge, double radius, double scalingFactor) {
    q_[index] = charge;
    r_[index] = radius;
    s_[index] = scalingFactor;
  }
  double getSolventDielectric() const { return 78.5; }
  double getSoluteDielectric() const { return 1.0; }
  NonbondedMethod getNonbondedMethod() const { return method_; }
  void setNonbondedMethod(NonbondedMethod m) { method_ = m; }
  double getCutoffDistance() const { return cutoff_; }
  void setCutoffDistance(double d) { cutoff_ = d; }

 private:
  std::vector<double> q_, r_, s_;
  NonbondedMethod method_ = NoCutoff;
  double cutoff_ = 1.0;
};
}  // namespace OpenMM
