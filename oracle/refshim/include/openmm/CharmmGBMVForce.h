// Stand-in exposing only what the reference's integral classes read from a
// CharmmGBMVForce (per-particle "radius", integral orders, nonbonded method).
#ifndef REFSHIM_CHARMMGBMVFORCE_H
#define REFSHIM_CHARMMGBMVFORCE_H
#include <map>
#include <string>
#include <vector>
namespace OpenMM {
class CharmmGBMVForce {
 public:
  enum NonbondedMethod { NoCutoff = 0, CutoffNonPeriodic = 1, CutoffPeriodic = 2 };
  enum GBIntegralType { GBSWIntegral = 0, GBMVIntegralTypeI = 1, GBMVIntegralTypeII = 2, CustomIntegral = 3 };
  NonbondedMethod method = NoCutoff;
  std::vector<std::vector<double> > particles;   // one parameter: radius
  std::vector<std::vector<int> > integralOrders;
  NonbondedMethod getNonbondedMethod() const { return method; }
  int getNumGBIntegrals() const { return (int)integralOrders.size(); }
  int getNumPerParticleParameters() const { return 1; }
  std::string getPerParticleParameterName(int) const { return "radius"; }
  void getParticleParameters(int i, std::vector<double>& p) const { p = particles[i]; }
  void getGBIntegralParameters(int i, std::string& name, std::vector<int>& pi, std::vector<double>& pr) const {
    name = "I" + std::to_string(i);
    pi = integralOrders[i];
    pr.clear();
  }
};
}  // namespace OpenMM
#endif
