// Drives the GB300 OpenMM plugin adapter through OpenMM's plugin protocol
// on stand-in OpenMM classes and the recording gbx (test infrastructure).
// Prints the gbx call log per scenario; exits non-zero if an expectation
// fails.
#include <cstdio>
#include <memory>
#include <string>
#include <vector>

#include "CudaPlatform.h"
#include "gbx.h"
#include "openmm/KernelFactory.h"
#include "openmm/OpenMMException.h"
#include "openmm/charmmKernels.h"

extern std::vector<std::string> g_log;
extern gbx_status g_execute_status;
extern "C" void registerKernelFactories();

using namespace OpenMM;

static int failures = 0;
#define EXPECT(cond)                                                       \
  do {                                                                     \
    if (!(cond)) {                                                         \
      std::printf("FAIL %s:%d %s\n", __FILE__, __LINE__, #cond);           \
      ++failures;                                                          \
    }                                                                      \
  } while (0)

static bool logged(const std::string& prefix) {
  for (auto& s : g_log)
    if (s.compare(0, prefix.size(), prefix) == 0) return true;
  return false;
}
static int count(const std::string& prefix) {
  int c = 0;
  for (auto& s : g_log)
    if (s.compare(0, prefix.size(), prefix) == 0) ++c;
  return c;
}
static void dump(const char* scenario) {
  std::printf("== %s\n", scenario);
  for (auto& s : g_log) std::printf("  %s\n", s.c_str());
  g_log.clear();
}

int main() {
  CudaPlatform cuda;
  Platform::registerPlatform(&cuda);
  registerKernelFactories();
  EXPECT(cuda.factories.count("CalcCharmmGBSWForce") == 1);
  EXPECT(cuda.factories.count("CalcCharmmGBMVForce") == 1);
  KernelFactory* factory = cuda.factories["CalcCharmmGBSWForce"];

  const int n = 4;
  System system;
  for (int i = 0; i < n; ++i) system.addParticle(1.0);
  CudaContext cu;
  cu.numAtoms = n;
  cu.paddedNumAtoms = 32;
  cu.atomIndex = {0, 1, 2, 3};
  cu.posq = CudaArray(0x1000);
  cu.force = CudaArray(0x2000);
  cu.energy = CudaArray(0x3000);
  CudaPlatform::PlatformData data;
  data.contexts.push_back(&cu);
  ContextImpl context(system, &data);
  context.setParameter("alpha0", -0.180);
  context.setParameter("alpha1", 1.817);

  // CharmmGBSWForce in single precision
  {
    CharmmGBSWForce force;
    for (int i = 0; i < n; ++i) force.addParticle(0.1 * (i + 1), 0.15, 1.0);
    std::unique_ptr<KernelImpl> k(factory->createKernelImpl("CalcCharmmGBSWForce", cuda, context));
    auto& gbsw = dynamic_cast<CalcCharmmGBSWForceKernel&>(*k);
    gbsw.initialize(system, force);
    EXPECT(logged("preset 0"));
    EXPECT(logged("params q0=0.1 r0=0.15 q3=0.4"));
    EXPECT(gbsw.execute(context, true, true) == 0.0);
    EXPECT(gbsw.execute(context, true, false) == 0.0);
    EXPECT(count("order 0 1 2 3") == 1);  // set once, before the first call
    EXPECT(logged("execute posq=1000 force=2000 stride=32 energy=3000 flags=35"));  // F|E|ENERGY_FLOAT
    EXPECT(logged("execute posq=1000 force=2000 stride=32 energy=3000 flags=33"));  // F|ENERGY_FLOAT
    dump("gbsw single precision");
    // OpenMM reorders the atoms: the new order is handed over, parameters are not re-sent
    cu.atomIndex = {2, 0, 3, 1};
    cu.reordered = true;
    gbsw.execute(context, true, true);
    cu.reordered = false;
    gbsw.execute(context, true, true);
    EXPECT(count("order 2 0 3 1") == 1);
    EXPECT(!logged("params"));
    dump("gbsw reorder");
    // mixed and double precision
    cu.useMixed = true;
    gbsw.execute(context, true, true);
    EXPECT(logged("execute posq=1000 force=2000 stride=32 energy=3000 flags=3 "));
    cu.useMixed = false;
    cu.useDouble = true;
    gbsw.execute(context, true, true);
    EXPECT(logged("execute posq=1000 force=2000 stride=32 energy=3000 flags=19"));  // F|E|POSQ_DOUBLE
    cu.useDouble = false;
    dump("gbsw mixed / double precision");
    // a later call reports an earlier call's overflowed table: an exception, not silence
    g_execute_status = GBX_ERR_STALE_RESULT;
    bool threw = false;
    try {
      gbsw.execute(context, true, true);
    } catch (const OpenMMException& e) {
      threw = std::string(e.what()).find("lacked the volume terms") != std::string::npos;
    }
    g_execute_status = GBX_OK;
    EXPECT(threw);
    force.setParticleParameters(0, -0.5, 0.2, 1.0);
    gbsw.copyParametersToContext(context, force);
    EXPECT(logged("params q0=-0.5 r0=0.2"));
    dump("gbsw stale report, parameter update");
  }
  EXPECT(logged("destroy"));
  g_log.clear();

  // CharmmGBSWForce with CutoffPeriodic: the box follows the context
  {
    CharmmGBSWForce force;
    for (int i = 0; i < n; ++i) force.addParticle(0.1, 0.15, 1.0);
    force.setNonbondedMethod(CharmmGBSWForce::CutoffPeriodic);
    force.setCutoffDistance(0.9);
    system.setDefaultPeriodicBoxVectors(Vec3(3, 0, 0), Vec3(0, 3, 0), Vec3(0, 0, 3));
    cu.box = BoxSize{3.0, 3.0, 3.0, 0.0};
    std::unique_ptr<KernelImpl> k(factory->createKernelImpl("CalcCharmmGBSWForce", cuda, context));
    auto& gbsw = dynamic_cast<CalcCharmmGBSWForceKernel&>(*k);
    gbsw.initialize(system, force);
    EXPECT(logged("create n=4 model=0 table=0 periodic=1 cutoff=0.9 box=3,3,3"));
    gbsw.execute(context, true, true);
    EXPECT(!logged("box"));
    cu.box = BoxSize{3.1, 3.0, 3.2, 0.0};
    gbsw.execute(context, true, true);
    gbsw.execute(context, true, true);
    EXPECT(count("box 3.1 3 3.2") == 1);
    dump("gbsw cutoff periodic");
  }
  g_log.clear();

  // CharmmGBMVForce with the canonical expressions, GBMV-II
  auto canonical = [&](CharmmGBMVForce& f, CharmmGBMVForce::GBIntegralType t) {
    f.addPerParticleParameter("q");
    f.addPerParticleParameter("radius");
    f.addGlobalParameter("alpha0", -0.180);
    f.addGlobalParameter("alpha1", 1.817);
    f.addGBIntegral("I4", {4}, {});
    f.addGBIntegral("I7", {7}, {});
    f.addComputedValue("B", "1/(alpha0*(1/0.05-I4)+alpha1*(1/(4*0.05^4)-I7)^(1/4))", CharmmGBMVForce::SingleParticle);
    f.addEnergyTerm("-0.5*138.935456*(1-1/80)*q^2/B", CharmmGBMVForce::SingleParticle);
    f.addEnergyTerm("-138.935456*(1-1/80)*q1*q2/sqrt(r^2+B1*B2*exp(-r^2/(4*B1*B2)))",
                    CharmmGBMVForce::ParticlePairNoExclusions);
    f.setGBIntegralType(t);
    for (int i = 0; i < n; ++i) f.addParticle({0.2 * (i + 1), 0.17});
  };
  {
    CharmmGBMVForce force;
    canonical(force, CharmmGBMVForce::GBMVIntegralTypeII);
    KernelFactory* gf = cuda.factories["CalcCharmmGBMVForce"];
    std::unique_ptr<KernelImpl> k(gf->createKernelImpl("CalcCharmmGBMVForce", cuda, context));
    auto& gbmv = dynamic_cast<CalcCharmmGBMVForceKernel&>(*k);
    gbmv.initialize(system, force);
    EXPECT(logged("preset 3"));
    EXPECT(logged("create n=4 model=2 table=2 periodic=0 cutoff=0 box=3,3,3"));
    EXPECT(logged("params q0=0.2 r0=0.17 q3=0.8"));
    cu.box = BoxSize{3.0, 3.0, 3.0, 0.0};
    gbmv.execute(context, true, true);
    EXPECT(!logged("globals"));
    context.setParameter("alpha0", -0.2);
    gbmv.execute(context, true, true);
    gbmv.execute(context, true, true);
    EXPECT(count("globals -0.2 1.817") == 1);
    dump("gbmv2 canonical");
  }
  g_log.clear();
  {
    CharmmGBMVForce force;
    canonical(force, CharmmGBMVForce::GBMVIntegralTypeI);
    force.addGlobalParameter("gamma", 0.5);
    force.addEnergyTerm("gamma*radius^2", CharmmGBMVForce::SingleParticle);  // outside the canonical set
    KernelFactory* gf = cuda.factories["CalcCharmmGBMVForce"];
    std::unique_ptr<KernelImpl> k(gf->createKernelImpl("CalcCharmmGBMVForce", cuda, context));
    auto& gbmv = dynamic_cast<CalcCharmmGBMVForceKernel&>(*k);
    gbmv.initialize(system, force);
    EXPECT(logged("create_custom n=4 model=1 params q radius integrals I4:4 I7:7 values B terms 0 2 0"));
    EXPECT(!logged("param_derivs"));
    EXPECT(logged("custom_params p00=0.2 p01=0.17"));
    context.setParameter("gamma", 0.5);
    gbmv.execute(context, true, true);
    EXPECT(!logged("custom_global gamma"));
    EXPECT(count("custom_global alpha0 -0.2") == 1);  // the context's value, changed by the scenario above
    context.setParameter("gamma", 0.75);
    gbmv.execute(context, true, true);
    gbmv.execute(context, true, true);
    EXPECT(count("custom_global gamma 0.75") == 1);
    dump("gbmv expressions outside the canonical set: compiled");
  }
  g_log.clear();
  {
    // exclusions with a ParticlePair term, and energy derivatives by globals
    CharmmGBMVForce force;
    canonical(force, CharmmGBMVForce::GBMVIntegralTypeII);
    force.addGlobalParameter("kr", 2.0);
    force.addEnergyTerm("0.01*q1*q2/r", CharmmGBMVForce::ParticlePair);
    force.addExclusion(0, 1);
    force.addExclusion(2, 3);
    force.addEnergyParameterDerivative("kr");
    force.addEnergyParameterDerivative("alpha1");
    context.setParameter("kr", 2.0);
    KernelFactory* gf = cuda.factories["CalcCharmmGBMVForce"];
    std::unique_ptr<KernelImpl> k(gf->createKernelImpl("CalcCharmmGBMVForce", cuda, context));
    auto& gbmv = dynamic_cast<CalcCharmmGBMVForceKernel&>(*k);
    gbmv.initialize(system, force);
    EXPECT(logged("create_custom n=4 model=2 params q radius integrals I4:4 I7:7 values B terms 0 2 1 "
                  "exclusions 0-1 2-3 param_derivs kr alpha1"));
    EXPECT(cu.paramDerivNames.size() == 2 && cu.paramDerivNames[0] == "kr" && cu.paramDerivNames[1] == "alpha1");
    cu.paramDerivWorkspace.clear();
    gbmv.execute(context, true, true);
    gbmv.execute(context, true, true);
    EXPECT(count("param_derivs 2") == 2);
    EXPECT(cu.paramDerivWorkspace["kr"] == 1.0 && cu.paramDerivWorkspace["alpha1"] == 2.0);  // two steps summed
    dump("gbmv exclusions and energy parameter derivatives");
  }
  g_log.clear();
  {
    // tabulated functions: Continuous1DFunction passes through, another type is refused
    CharmmGBMVForce force;
    canonical(force, CharmmGBMVForce::GBMVIntegralTypeII);
    force.addTabulatedFunction("tail", new OpenMM::Continuous1DFunction({0.5, 0.25, 0.0}, 0.0, 3.0));
    force.addTabulatedFunction("scale", new OpenMM::Continuous1DFunction({1.0, 2.0}, 0.05, 3.0));
    force.addEnergyTerm("q1*q2*tail(r)", CharmmGBMVForce::ParticlePairNoExclusions);
    KernelFactory* gf = cuda.factories["CalcCharmmGBMVForce"];
    std::unique_ptr<KernelImpl> k(gf->createKernelImpl("CalcCharmmGBMVForce", cuda, context));
    dynamic_cast<CalcCharmmGBMVForceKernel&>(*k).initialize(system, force);
    EXPECT(logged("create_custom n=4 model=2 params q radius integrals I4:4 I7:7 values B terms 0 2 2 "
                  "function tail n=3 [0,3] first=0.5 last=0 function scale n=2 [0.05,3] first=1 last=2"));
    CharmmGBMVForce other;
    canonical(other, CharmmGBMVForce::GBMVIntegralTypeII);
    other.addTabulatedFunction("d", new OpenMM::Discrete1DFunction({1.0, 2.0}));
    other.addEnergyTerm("d(q)", CharmmGBMVForce::SingleParticle);
    std::unique_ptr<KernelImpl> k2(gf->createKernelImpl("CalcCharmmGBMVForce", cuda, context));
    bool threw = false;
    try {
      dynamic_cast<CalcCharmmGBMVForceKernel&>(*k2).initialize(system, other);
    } catch (const OpenMMException& e) {
      threw = std::string(e.what()).find("Continuous1DFunction") != std::string::npos;
    }
    EXPECT(threw);
    dump("gbmv tabulated functions");
  }
  {
    CharmmGBMVForce force;
    canonical(force, CharmmGBMVForce::CustomIntegral);
    KernelFactory* gf = cuda.factories["CalcCharmmGBMVForce"];
    std::unique_ptr<KernelImpl> k(gf->createKernelImpl("CalcCharmmGBMVForce", cuda, context));
    bool threw = false;
    try {
      dynamic_cast<CalcCharmmGBMVForceKernel&>(*k).initialize(system, force);
    } catch (const OpenMMException& e) {
      threw = std::string(e.what()).find("CustomIntegral") != std::string::npos;
    }
    EXPECT(threw);
    dump("custom integral refused");
  }
  {
    bool threw = false;
    try {
      delete factory->createKernelImpl("CalcSomethingElse", cuda, context);
    } catch (const OpenMMException&) {
      threw = true;
    }
    EXPECT(threw);
  }
  std::printf(failures ? "FAILED %d\n" : "ALL OK\n", failures);
  return failures ? 1 : 0;
}
