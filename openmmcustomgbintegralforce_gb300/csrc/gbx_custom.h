// The custom-expression path of a context (gbx_custom.cu).
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "gbx.h"

namespace gbx {

struct Context;
struct CustomPlan;

// A copy of gbx_custom (include/gbx.h) with owned strings.
struct gbx_custom_spec {
  std::vector<std::string> params, globals, integrals, value_names, value_expressions, term_expressions;
  std::vector<double> global_values;
  std::vector<int> integral_orders, term_types;  // term types: 0 single particle, 1 pair, 2 pair without exclusions
  std::vector<int> exclusions;                   // [pairs][2]
  std::vector<std::string> param_derivs;         // globals whose energy derivative is reported
  struct Function {                              // Continuous1DFunction: natural cubic spline,
    std::string name;                            // zero outside [x0, x1]
    double x0 = 0.0, x1 = 1.0;
    std::vector<double> y;                       // values at evenly spaced points
  };
  std::vector<Function> functions;
};

gbx_status custom_build(Context* ctx, const gbx_custom_spec& spec);
void custom_destroy(Context* ctx);
int custom_energy_parts(const Context* ctx);
gbx_status custom_set_parameters(Context* ctx, const double* params, std::vector<double>& radius);
gbx_status custom_set_global(Context* ctx, const char* name, double value);
gbx_status launch_custom_energy(Context* ctx, const float4* pos, unsigned long long* force, int stride);
gbx_status launch_custom_chain_prep(Context* ctx, unsigned long long* force, int stride);
// dE/dg for the requested globals after the last execute (host sum of the
// per-block partials, in a fixed order).
gbx_status custom_param_derivs(Context* ctx, double* out, int count);
// Parses the expressions and compiles the generated source (no device needed).
gbx_status custom_compile_only(const gbx_custom_spec& spec, std::string& log);

}  // namespace gbx
