// OpenMM kernels for CharmmGBSWForce / CharmmGBMVForce on the gbx C ABI.
#include "GB300CharmmKernels.h"

#include <algorithm>
#include <cctype>

#include "openmm/OpenMMException.h"
#include "openmm/TabulatedFunction.h"

using OpenMM::CharmmGBMVForce;
using OpenMM::CharmmGBSWForce;
using OpenMM::OpenMMException;

namespace GB300 {

namespace {

std::string squeeze(const std::string& s) {
  std::string out;
  for (char c : s)
    if (!std::isspace(static_cast<unsigned char>(c))) out += c;
  return out;
}

// The canonical CHARMM GB expressions: the Born radius of
// CharmmReferenceGBSW.cpp:591-593 and the pair and self terms of
// CharmmReferenceGBSW.cpp:237-283 with ONE_4PI_EPS0 = 138.935456.
const char* kBorn = "1/(alpha0*(1/0.05-I4)+alpha1*(1/(4*0.05^4)-I7)^(1/4))";
const char* kSelf = "-0.5*138.935456*(1-1/80)*q^2/B";
const char* kPair = "-138.935456*(1-1/80)*q1*q2/sqrt(r^2+B1*B2*exp(-r^2/(4*B1*B2)))";

}  // namespace

GbxForceState::~GbxForceState() {
  if (handle) gbx_destroy(handle);
}

void GbxForceState::check(gbx_status status, const char* what) const {
  if (status == GBX_OK) return;
  std::string detail;
  if (handle) {
    char buf[512];
    if (gbx_last_error(handle, buf, sizeof(buf)) == GBX_OK) detail = buf;
  }
  throw OpenMMException(std::string("GB300 ") + what + ": " + gbx_status_string(status) +
                        (detail.empty() ? "" : " (" + detail + ")"));
}

void GbxForceState::create(const gbx_config& cfg, int n) {
  cu.setAsCurrent();
  numAtoms = n;
  globals[0] = cfg.alpha0;
  globals[1] = cfg.alpha1;
  for (int k = 0; k < 3; ++k) box[k] = cfg.box[k];
  check(gbx_create(&cfg, n, &handle), "gbx_create");
}

void GbxForceState::setParameters(const std::vector<double>& charge, const std::vector<double>& radius) {
  cu.setAsCurrent();
  check(gbx_set_particle_parameters(handle, charge.data(), radius.data()), "gbx_set_particle_parameters");
}

void GbxForceState::setGlobals(double alpha0, double alpha1) {
  if (alpha0 == globals[0] && alpha1 == globals[1]) return;  // a change drops the captured call
  check(gbx_set_global_parameters(handle, alpha0, alpha1), "gbx_set_global_parameters");
  globals[0] = alpha0;
  globals[1] = alpha1;
}

void GbxForceState::createCustom(const gbx_config& cfg, int n, const gbx_custom& custom) {
  cu.setAsCurrent();
  numAtoms = n;
  customGlobals.assign(custom.global_values, custom.global_values + custom.num_globals);
  for (int k = 0; k < 3; ++k) box[k] = cfg.box[k];
  check(gbx_create_custom(&cfg, n, &custom, &handle), "gbx_create_custom (compiling the force's expressions)");
}

void GbxForceState::setCustomParameters(const std::vector<double>& params) {
  cu.setAsCurrent();
  check(gbx_set_custom_parameters(handle, params.data()), "gbx_set_custom_parameters");
}

void GbxForceState::setCustomGlobal(int index, const std::string& name, double value) {
  if (customGlobals[index] == value) return;
  check(gbx_set_custom_global(handle, name.c_str(), value), "gbx_set_custom_global");
  customGlobals[index] = value;
}

void GbxForceState::setBox(double a, double b, double c) {
  if (a == box[0] && b == box[1] && c == box[2]) return;
  const double edges[3] = {a, b, c};
  check(gbx_set_box(handle, edges), "gbx_set_box");
  box[0] = a;
  box[1] = b;
  box[2] = c;
}

double GbxForceState::execute(bool includeForces, bool includeEnergy) {
  cu.setAsCurrent();
  // OpenMM moves atoms between slots for locality; the library keeps atom
  // order internally and reads and writes the slots through this map
  if (!orderSet || cu.getAtomsWereReordered()) {
    check(gbx_set_atom_order(handle, cu.getAtomIndex().data()), "gbx_set_atom_order");
    orderSet = true;
  }
  int flags = (includeForces ? GBX_EXEC_FORCES : 0) | (includeEnergy ? GBX_EXEC_ENERGY : 0);
  if (cu.getUseDoublePrecision()) flags |= GBX_EXEC_POSQ_DOUBLE;   // double4 posq, double energy
  else if (!cu.getUseMixedPrecision()) flags |= GBX_EXEC_ENERGY_FLOAT;  // float4 posq, float energy
  if (!flags) return 0.0;
  const void* posq = reinterpret_cast<const void*>(cu.getPosq().getDevicePointer());
  unsigned long long* force = reinterpret_cast<unsigned long long*>(cu.getForce().getDevicePointer());
  double* energy = reinterpret_cast<double*>(cu.getEnergyBuffer().getDevicePointer());
  check(gbx_execute(handle, posq, force, cu.getPaddedNumAtoms(), energy, flags, cu.getCurrentStream()),
        "gbx_execute");
  return 0.0;
}

// ---------------------------------------------------------------------------
// CharmmGBSWForce
// ---------------------------------------------------------------------------

void GB300CalcCharmmGBSWForceKernel::initialize(const OpenMM::System& system, const CharmmGBSWForce& force) {
  if (force.getNumParticles() != system.getNumParticles())
    throw OpenMMException("CharmmGBSWForce must have exactly as many particles as the System it belongs to.");
  gbx_config cfg;
  state.check(gbx_config_preset(GBX_PRESET_CHARMM_GBSW, &cfg), "gbx_config_preset");
  if (force.getNonbondedMethod() != CharmmGBSWForce::NoCutoff) cfg.cutoff = force.getCutoffDistance();
  if (force.getNonbondedMethod() == CharmmGBSWForce::CutoffPeriodic) {
    // rectangular boxes: minimum-image distances (CharmmReferenceGBSW.cpp:147-159)
    OpenMM::Vec3 a, b, c;
    system.getDefaultPeriodicBoxVectors(a, b, c);
    cfg.periodic = 1;
    cfg.box[0] = a[0];
    cfg.box[1] = b[1];
    cfg.box[2] = c[2];
    periodic = true;
  }
  state.create(cfg, system.getNumParticles());
  copyParameters(force);
}

void GB300CalcCharmmGBSWForceKernel::copyParameters(const CharmmGBSWForce& force) {
  const int n = force.getNumParticles();
  std::vector<double> q(n), r(n);
  for (int i = 0; i < n; ++i) {
    double s;
    force.getParticleParameters(i, q[i], r[i], s);
  }
  state.setParameters(q, r);
}

double GB300CalcCharmmGBSWForceKernel::execute(OpenMM::ContextImpl&, bool includeForces, bool includeEnergy) {
  if (periodic) {  // a barostat may have rescaled the box
    const auto b = state.cu.getPeriodicBoxSize();  // double4: x, y, z edges
    state.setBox(b.x, b.y, b.z);
  }
  return state.execute(includeForces, includeEnergy);
}

void GB300CalcCharmmGBSWForceKernel::copyParametersToContext(OpenMM::ContextImpl&, const CharmmGBSWForce& force) {
  if (force.getNumParticles() != state.numAtoms)
    throw OpenMMException("updateParametersInContext: The number of particles has changed");
  copyParameters(force);
}

// ---------------------------------------------------------------------------
// CharmmGBMVForce
// ---------------------------------------------------------------------------

bool isCanonicalGBMVForce(const CharmmGBMVForce& force, int& chargeIndex, int& radiusIndex) {
  if (force.getGBIntegralType() == CharmmGBMVForce::CustomIntegral)
    throw OpenMMException("GB300: CustomIntegral has no implementation");
  chargeIndex = radiusIndex = -1;
  for (int k = 0; k < force.getNumPerParticleParameters(); ++k) {
    if (force.getPerParticleParameterName(k) == "q") chargeIndex = k;
    if (force.getPerParticleParameterName(k) == "radius") radiusIndex = k;
  }
  // GBSWIntegral.cpp:79-80
  if (radiusIndex < 0) throw OpenMMException("GBSWIntegral: the per perticle parameter 'radius' must be defined");
  for (int k = 0; k < force.getNumGBIntegrals(); ++k) {
    std::string name;
    std::vector<int> pi;
    std::vector<double> pr;
    force.getGBIntegralParameters(k, name, pi, pr);
    if (pi.empty()) throw OpenMMException("GBSWIntegral: the order of integral must be given");
    if (pi[0] < 2) throw OpenMMException("GBSWIntegral: the order of integral must be greater or equal to 2");
  }
  bool ok = chargeIndex >= 0 && force.getNumGBIntegrals() == 2 && force.getNumComputedValues() == 1 &&
            force.getNumEnergyTerms() == 2 && force.getNumTabulatedFunctions() == 0 &&
            force.getNumEnergyParameterDerivatives() == 0;
  const char* integralNames[2] = {"I4", "I7"};
  const int orders[2] = {4, 7};
  for (int k = 0; ok && k < 2; ++k) {
    std::string name;
    std::vector<int> pi;
    std::vector<double> pr;
    force.getGBIntegralParameters(k, name, pi, pr);
    ok = name == integralNames[k] && pi[0] == orders[k];
  }
  if (ok) {
    std::string name, expr;
    CharmmGBMVForce::ComputationType type;
    force.getComputedValueParameters(0, name, expr, type);
    ok = name == "B" && squeeze(expr) == squeeze(kBorn) && type == CharmmGBMVForce::SingleParticle;
  }
  if (ok) {
    std::string expr;
    CharmmGBMVForce::ComputationType type;
    force.getEnergyTermParameters(0, expr, type);
    ok = squeeze(expr) == squeeze(kSelf) && type == CharmmGBMVForce::SingleParticle;
    force.getEnergyTermParameters(1, expr, type);
    ok = ok && squeeze(expr) == squeeze(kPair) && type == CharmmGBMVForce::ParticlePairNoExclusions;
  }
  return ok;
}

void GB300CalcCharmmGBMVForceKernel::initialize(const OpenMM::System& system, const CharmmGBMVForce& force) {
  if (force.getNumParticles() != system.getNumParticles())
    throw OpenMMException("CharmmGBMVForce must have exactly as many particles as the System it belongs to.");
  for (int i = 0; i < force.getNumParticles(); ++i) {
    std::vector<double> p;
    force.getParticleParameters(i, p);
    if ((int)p.size() != force.getNumPerParticleParameters())
      throw OpenMMException("CharmmGBMVForce: Wrong number of parameters for particle " + std::to_string(i));
  }
  custom = !isCanonicalGBMVForce(force, chargeIndex, radiusIndex);
  int preset = GBX_PRESET_GBSW_INTEGRAL;
  if (force.getGBIntegralType() == CharmmGBMVForce::GBMVIntegralTypeI) preset = GBX_PRESET_GBMV1;
  if (force.getGBIntegralType() == CharmmGBMVForce::GBMVIntegralTypeII) preset = GBX_PRESET_GBMV2;
  gbx_config cfg;
  state.check(gbx_config_preset(preset, &cfg), "gbx_config_preset");
  // the integral classes always build their table in the context's box
  // (GBMVIntegralTypeI.cpp:102-105, GBMVIntegralTypeII.cpp:107-110)
  OpenMM::Vec3 a, b, c;
  system.getDefaultPeriodicBoxVectors(a, b, c);
  cfg.box[0] = a[0];
  cfg.box[1] = b[1];
  cfg.box[2] = c[2];
  if (force.getNonbondedMethod() != CharmmGBMVForce::NoCutoff) cfg.cutoff = force.getCutoffDistance();
  if (force.getNonbondedMethod() == CharmmGBMVForce::CutoffPeriodic) {
    // minimum-image integrals (GBSWIntegral on the box-sampled table,
    // GBSWIntegral.cpp:63-68,109) and pair terms (CharmmReferenceGBMV.cpp:294-297)
    cfg.periodic = 1;
    cfg.table_mode = GBX_TABLE_PERIODIC;
  }
  if (!custom) {
    for (int k = 0; k < force.getNumGlobalParameters(); ++k) {
      const std::string& name = force.getGlobalParameterName(k);
      if (name == "alpha0") cfg.alpha0 = force.getGlobalParameterDefaultValue(k);
      if (name == "alpha1") cfg.alpha1 = force.getGlobalParameterDefaultValue(k);
    }
    alphaNames[0] = "alpha0";
    alphaNames[1] = "alpha1";
    state.create(cfg, system.getNumParticles());
  } else {
    // the force's own expressions, compiled for the device
    std::vector<std::string> params, integrals, values, valueExprs, terms, functionNames;
    std::vector<double> globalValues, functionValues, functionRanges;
    std::vector<int> orders, types, exclusions, functionSizes;
    // tabulated functions: Continuous1DFunction (a natural cubic spline, zero outside its range)
    for (int k = 0; k < force.getNumTabulatedFunctions(); ++k) {
      const auto* fn = dynamic_cast<const OpenMM::Continuous1DFunction*>(&force.getTabulatedFunction(k));
      if (!fn) throw OpenMMException("GB300: only Continuous1DFunction tabulated functions are supported");
      std::vector<double> v;
      double lo = 0.0, hi = 0.0;
      fn->getFunctionParameters(v, lo, hi);
      functionNames.push_back(force.getTabulatedFunctionName(k));
      functionSizes.push_back((int)v.size());
      functionValues.insert(functionValues.end(), v.begin(), v.end());
      functionRanges.push_back(lo);
      functionRanges.push_back(hi);
    }
    for (int k = 0; k < force.getNumPerParticleParameters(); ++k)
      params.push_back(force.getPerParticleParameterName(k));
    for (int k = 0; k < force.getNumGlobalParameters(); ++k) {
      globalNames.push_back(force.getGlobalParameterName(k));
      globalValues.push_back(force.getGlobalParameterDefaultValue(k));
    }
    for (int k = 0; k < force.getNumGBIntegrals(); ++k) {
      std::string name;
      std::vector<int> pi;
      std::vector<double> pr;
      force.getGBIntegralParameters(k, name, pi, pr);
      integrals.push_back(name);
      orders.push_back(pi[0]);
    }
    for (int k = 0; k < force.getNumComputedValues(); ++k) {
      std::string name, expr;
      CharmmGBMVForce::ComputationType type;
      force.getComputedValueParameters(k, name, expr, type);
      if (type != CharmmGBMVForce::SingleParticle)
        throw OpenMMException("GB300: computed values must be SingleParticle");
      values.push_back(name);
      valueExprs.push_back(expr);
    }
    for (int k = 0; k < force.getNumEnergyTerms(); ++k) {
      std::string expr;
      CharmmGBMVForce::ComputationType type;
      force.getEnergyTermParameters(k, expr, type);
      terms.push_back(expr);
      types.push_back(type == CharmmGBMVForce::SingleParticle ? GBX_TERM_SINGLE
                      : type == CharmmGBMVForce::ParticlePair ? GBX_TERM_PAIR
                                                              : GBX_TERM_PAIR_NO_EXCLUSIONS);
    }
    for (int k = 0; k < force.getNumExclusions(); ++k) {
      int a = 0, b = 0;
      force.getExclusionParticles(k, a, b);
      exclusions.push_back(a);
      exclusions.push_back(b);
    }
    // the derivatives reach the context through the platform's workspace
    // for derivatives formed outside its own kernels
    for (int k = 0; k < force.getNumEnergyParameterDerivatives(); ++k) {
      paramDerivNames.push_back(force.getEnergyParameterDerivativeName(k));
      state.cu.addEnergyParameterDerivative(paramDerivNames.back());
    }
    auto ptrs = [](const std::vector<std::string>& v) {
      std::vector<const char*> p;
      for (auto& x : v) p.push_back(x.c_str());
      return p;
    };
    const auto pn = ptrs(params), gn = ptrs(globalNames), in = ptrs(integrals), vn = ptrs(values),
               ve = ptrs(valueExprs), te = ptrs(terms), pd = ptrs(paramDerivNames), fnn = ptrs(functionNames);
    gbx_custom cs{};
    cs.num_params = (int)params.size();
    cs.param_names = pn.data();
    cs.num_globals = (int)globalNames.size();
    cs.global_names = gn.data();
    cs.global_values = globalValues.data();
    cs.num_integrals = (int)integrals.size();
    cs.integral_names = in.data();
    cs.integral_orders = orders.data();
    cs.num_values = (int)values.size();
    cs.value_names = vn.data();
    cs.value_expressions = ve.data();
    cs.num_terms = (int)terms.size();
    cs.term_expressions = te.data();
    cs.term_types = types.data();
    cs.num_exclusions = (int)exclusions.size() / 2;
    cs.exclusions = exclusions.data();
    cs.num_param_derivs = (int)paramDerivNames.size();
    cs.param_deriv_names = pd.data();
    cs.num_functions = (int)functionNames.size();
    cs.function_names = fnn.data();
    cs.function_sizes = functionSizes.data();
    cs.function_values = functionValues.data();
    cs.function_ranges = functionRanges.data();
    state.createCustom(cfg, system.getNumParticles(), cs);
  }
  copyParameters(force);
}

void GB300CalcCharmmGBMVForceKernel::copyParameters(const CharmmGBMVForce& force) {
  const int n = force.getNumParticles();
  std::vector<double> p;
  if (custom) {
    const int np = force.getNumPerParticleParameters();
    std::vector<double> all((size_t)n * np);
    for (int i = 0; i < n; ++i) {
      force.getParticleParameters(i, p);
      for (int k = 0; k < np; ++k) all[(size_t)i * np + k] = p[k];
    }
    state.setCustomParameters(all);
    return;
  }
  std::vector<double> q(n), r(n);
  for (int i = 0; i < n; ++i) {
    force.getParticleParameters(i, p);
    q[i] = p[chargeIndex];
    r[i] = p[radiusIndex];
  }
  state.setParameters(q, r);
}

double GB300CalcCharmmGBMVForceKernel::execute(OpenMM::ContextImpl& context, bool includeForces,
                                              bool includeEnergy) {
  if (custom) {
    for (size_t k = 0; k < globalNames.size(); ++k)
      state.setCustomGlobal((int)k, globalNames[k], context.getParameter(globalNames[k]));
  } else {
    state.setGlobals(context.getParameter(alphaNames[0]), context.getParameter(alphaNames[1]));
  }
  const auto b = state.cu.getPeriodicBoxSize();  // double4: x, y, z edges
  state.setBox(b.x, b.y, b.z);
  const double e = state.execute(includeForces, includeEnergy);
  if (!paramDerivNames.empty()) {
    // read back after the step (this waits for the context's stream)
    std::vector<double> d(paramDerivNames.size());
    state.check(gbx_get_custom_param_derivs(state.handle, d.data(), (int)d.size()), "gbx_get_custom_param_derivs");
    auto& workspace = state.cu.getEnergyParamDerivWorkspace();
    for (size_t k = 0; k < d.size(); ++k) workspace[paramDerivNames[k]] += d[k];
  }
  return e;
}

void GB300CalcCharmmGBMVForceKernel::copyParametersToContext(OpenMM::ContextImpl&, const CharmmGBMVForce& force) {
  if (force.getNumParticles() != state.numAtoms)
    throw OpenMMException("updateParametersInContext: The number of particles has changed");
  copyParameters(force);
}

}  // namespace GB300
