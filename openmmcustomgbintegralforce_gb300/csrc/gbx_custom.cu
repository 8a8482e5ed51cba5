// CharmmGBMVForce expressions outside the canonical CHARMM set, compiled
// into device code when the context is created.
//
// The reference evaluates a CharmmGBMVForce's computed values and energy
// terms from user expressions (CharmmReferenceGBMV.cpp:151-444 on the CPU,
// CharmmCudaKernels.cpp:228-827 on CUDA, which splices them into kernel
// source).  Here the Born-radius integrals stay the library's own kernels
// (any two integral orders: the quadrature weights are w / r^(n-2)); the
// expressions and their symbolic derivatives (gbx_expr.cu) are emitted as
// CUDA source, compiled at creation by NVRTC (loaded at run time, so the
// library does not depend on it unless this path is used) and launched from
// the loaded library:
//
//   gbx_values  per atom, FP64: the integrals I_k = S_k - J_k from their
//               complements, the computed values in order and their total
//               derivatives dV/dI (forward mode), the single-particle
//               energy terms with dE/dV and dE/dI
//   gbx_pair    the pair energy terms over every pair i < j: thread per
//               atom over tiles of partners in shared memory, FP32, each
//               pair evaluated by both of its atoms (every thread sums only
//               its own atom's force and derivatives, no atomics per pair);
//               the energy is counted by the lower atom
//   gbx_chain   per atom: dE/dJ_k = -(dE/dI_k + sum_m dE/dV_m dV_m/dI_k),
//               which the library's chain-rule kernels carry through every
//               quadrature point
//
// Derivative sums are 64-bit fixed point (order-free); energies are per-block
// FP64 partials reduced in a fixed order, so results are bit-reproducible.
#include <dlfcn.h>
#include <nvrtc.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <new>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "gbx_custom.h"
#include "gbx_expr.h"
#include "gbx_internal.cuh"

#define GBX_TRY_CUSTOM(expr)     \
  do {                           \
    gbx_status s_ = (expr);      \
    if (s_ != GBX_OK) return s_; \
  } while (0)

namespace gbx {

namespace {

// ---------------------------------------------------------------------------
// NVRTC, resolved at run time
// ---------------------------------------------------------------------------
struct Nvrtc {
  void* lib = nullptr;
  decltype(&nvrtcCreateProgram) create = nullptr;
  decltype(&nvrtcCompileProgram) compile = nullptr;
  decltype(&nvrtcGetProgramLogSize) log_size = nullptr;
  decltype(&nvrtcGetProgramLog) log = nullptr;
  decltype(&nvrtcGetCUBINSize) cubin_size = nullptr;
  decltype(&nvrtcGetCUBIN) cubin = nullptr;
  decltype(&nvrtcDestroyProgram) destroy = nullptr;
  bool ok() const { return lib && create && compile && log_size && log && cubin_size && cubin && destroy; }
};

const Nvrtc& nvrtc() {
  static Nvrtc n;
  static bool tried = false;
  if (tried) return n;
  tried = true;
  const char* names[] = {"libnvrtc.so.13", "libnvrtc.so", "/usr/local/cuda/lib64/libnvrtc.so.13",
                         "/usr/local/cuda/lib64/libnvrtc.so"};
  for (const char* nm : names)
    if ((n.lib = dlopen(nm, RTLD_NOW | RTLD_LOCAL)) != nullptr) break;
  if (!n.lib) return n;
  n.create = reinterpret_cast<decltype(n.create)>(dlsym(n.lib, "nvrtcCreateProgram"));
  n.compile = reinterpret_cast<decltype(n.compile)>(dlsym(n.lib, "nvrtcCompileProgram"));
  n.log_size = reinterpret_cast<decltype(n.log_size)>(dlsym(n.lib, "nvrtcGetProgramLogSize"));
  n.log = reinterpret_cast<decltype(n.log)>(dlsym(n.lib, "nvrtcGetProgramLog"));
  n.cubin_size = reinterpret_cast<decltype(n.cubin_size)>(dlsym(n.lib, "nvrtcGetCUBINSize"));
  n.cubin = reinterpret_cast<decltype(n.cubin)>(dlsym(n.lib, "nvrtcGetCUBIN"));
  n.destroy = reinterpret_cast<decltype(n.destroy)>(dlsym(n.lib, "nvrtcDestroyProgram"));
  return n;
}

// The argument block of every generated kernel (CustomArgs below has the
// same layout on the host).
const char* kArgsDecl = R"(
struct CustomArgs {
  int n, chunks, parts;
  float cutoff2;
  int periodic;
  float L[3], iL[3];
  const double* params;      // [np][n]
  const float* paramsf;      // [np][n]
  const double* S;           // [ni] sum_q w_q / r_q^(n-2)
  const float* J;            // [ni][chunks][n] complement integrals
  const double* globals;     // [ng]
  const float4* pos;         // [n] x, y, z, -
  double* I;                 // [ni][n]
  float* If;                 // [ni][n]
  double* V;                 // [nv][n]
  float* Vf;                 // [nv][n]
  double* dVdI;              // [nv][ni][n]
  unsigned long long* dEdV;  // [nv][n] fixed point 2^-32
  unsigned long long* dEdI;  // [ni][n] fixed point 2^-32
  double* energy_part;       // [parts] per-block energies
  unsigned long long* force; // [3][stride] fixed point, added to
  int stride;
  float2* dEdJ;              // [n] -> the chain-rule kernels
  double* born;              // [n] the first computed value (reported)
  unsigned long long* dEdB;  // [n] dE/d(first computed value), fixed point
  unsigned* status;
  double* dVdX;              // [nv][3][n] total derivatives of the values by the particle's coordinates
  const int* excl_start;     // [n + 1] each particle's excluded partners (CSR, ascending)
  const int* excl;
  double* dVdG;              // [nv][npd][n] total derivatives of the values by the requested globals
  double* pd_part;           // [blocks][npd] per-block energy derivatives by the requested globals
};
)";

const char* kPrelude = R"(
__device__ __forceinline__ double gbx_ipow0(double) { return 1.0; }
__device__ __forceinline__ double gbx_ipow1(double x) { return x; }
__device__ __forceinline__ double gbx_ipow2(double x) { return x * x; }
__device__ __forceinline__ double gbx_ipow3(double x) { return x * x * x; }
__device__ __forceinline__ double gbx_ipow4(double x) { const double y = x * x; return y * y; }
__device__ __forceinline__ double gbx_ipow5(double x) { const double y = x * x; return y * y * x; }
__device__ __forceinline__ double gbx_ipow6(double x) { const double y = x * x * x; return y * y; }
__device__ __forceinline__ double gbx_ipow7(double x) { const double y = x * x * x; return y * y * x; }
__device__ __forceinline__ double gbx_ipow8(double x) { const double y = x * x; const double z = y * y; return z * z; }
__device__ __forceinline__ float gbx_ipow0(float) { return 1.0f; }
__device__ __forceinline__ float gbx_ipow1(float x) { return x; }
__device__ __forceinline__ float gbx_ipow2(float x) { return x * x; }
__device__ __forceinline__ float gbx_ipow3(float x) { return x * x * x; }
__device__ __forceinline__ float gbx_ipow4(float x) { const float y = x * x; return y * y; }
__device__ __forceinline__ float gbx_ipow5(float x) { const float y = x * x; return y * y * x; }
__device__ __forceinline__ float gbx_ipow6(float x) { const float y = x * x * x; return y * y; }
__device__ __forceinline__ float gbx_ipow7(float x) { const float y = x * x * x; return y * y * x; }
__device__ __forceinline__ float gbx_ipow8(float x) { const float y = x * x; const float z = y * y; return z * z; }
__device__ __forceinline__ long long gbx_fixed(double v) { return __double2ll_rn(v * 4294967296.0); }
__device__ __forceinline__ void gbx_add_fixed(unsigned long long* p, double v) {
  const long long q = gbx_fixed(v);
  if (q) atomicAdd(p, (unsigned long long)q);
}
)";

constexpr int kValueThreads = 256;
constexpr int kPairThreads = 128;

}  // namespace

struct CustomPlan {
  gbx_custom_spec spec;
  std::vector<expr::Ptr> values, terms;
  std::vector<int> term_types;
  int radius_index = -1;
  cudaLibrary_t library = nullptr;
  cudaKernel_t k_values = nullptr, k_pair = nullptr, k_chain = nullptr;
  std::vector<double> params;  // host [np][n]
  double* d_params = nullptr;
  float* d_paramsf = nullptr;
  double* d_S = nullptr;
  double* d_globals = nullptr;
  double* d_V = nullptr;
  float* d_Vf = nullptr;
  float* d_If = nullptr;
  double* d_dVdI = nullptr;
  unsigned long long* d_dEdV = nullptr;
  unsigned long long* d_dEdI = nullptr;
  double* d_dVdX = nullptr;
  int* d_excl_start = nullptr;
  int* d_excl = nullptr;
  double* d_dVdG = nullptr;
  double* d_pd_part = nullptr;
  bool coords = false;      // some computed value or single-particle term reads x, y or z
  bool excluding = false;   // exclusions exist and some term honours them
  std::vector<int> pd_index;  // requested globals, as indices into spec.globals
  int value_blocks = 0, pair_blocks = 0;
  std::string source;  // kept for diagnostics
};

namespace {

// Variable names of each kind of expression as the generated code spells them.
struct Names {
  std::map<std::string, std::string> single, pair;
};

Names variable_names(const gbx_custom_spec& s) {
  Names nm;
  for (size_t k = 0; k < s.params.size(); ++k) {
    nm.single[s.params[k]] = "p" + std::to_string(k);
    nm.pair[s.params[k] + "1"] = "pa" + std::to_string(k);
    nm.pair[s.params[k] + "2"] = "pb" + std::to_string(k);
  }
  for (size_t k = 0; k < s.globals.size(); ++k) {
    nm.single[s.globals[k]] = "g" + std::to_string(k);
    nm.pair[s.globals[k]] = "gf" + std::to_string(k);
  }
  for (size_t k = 0; k < s.integrals.size(); ++k) {
    nm.single[s.integrals[k]] = "I" + std::to_string(k);
    nm.pair[s.integrals[k] + "1"] = "Ia" + std::to_string(k);
    nm.pair[s.integrals[k] + "2"] = "Ib" + std::to_string(k);
  }
  for (size_t k = 0; k < s.value_names.size(); ++k) {
    nm.single[s.value_names[k]] = "v" + std::to_string(k);
    nm.pair[s.value_names[k] + "1"] = "va" + std::to_string(k);
    nm.pair[s.value_names[k] + "2"] = "vb" + std::to_string(k);
  }
  nm.single["x"] = "cx";
  nm.single["y"] = "cy";
  nm.single["z"] = "cz";
  nm.pair["r"] = "r";
  return nm;
}

// Per-block reduction of a double held by every thread into out[blockIdx.x * stride + k].
std::string block_sum(const std::string& v, const std::string& out) {
  return "  s_e[threadIdx.x] = " + v + ";\n  __syncthreads();\n"
         "  for (int st = blockDim.x / 2; st > 0; st >>= 1) {\n"
         "    if (threadIdx.x < st) s_e[threadIdx.x] += s_e[threadIdx.x + st];\n    __syncthreads();\n  }\n"
         "  if (threadIdx.x == 0) " + out + " = s_e[0];\n  __syncthreads();\n";
}

std::string generate(const CustomPlan& p) {
  const gbx_custom_spec& s = p.spec;
  const int np = (int)s.params.size(), ng = (int)s.globals.size(), ni = (int)s.integrals.size(),
            nv = (int)s.value_names.size(), npd = (int)p.pd_index.size();
  const Names nm = variable_names(s);
  const char* kCoord[3] = {"x", "y", "z"};
  auto D = [](const expr::Ptr& e, const std::string& v) { return expr::derivative(e, v); };
  std::ostringstream o;
  o << kArgsDecl << kPrelude;

  // ---- per-atom values, their derivatives, single-particle terms (FP64);
  // every expression and derivative shares its common subexpressions
  expr::SharedEmitter ve(nm.single, false, "s", "  ");
  o << "extern \"C\" __global__ void __launch_bounds__(" << kValueThreads << ") gbx_values(CustomArgs a) {\n";
  o << "  __shared__ double s_e[" << kValueThreads << "];\n";
  o << "  const int i = blockIdx.x * blockDim.x + threadIdx.x;\n  double e = 0.0;\n";
  for (int k = 0; k < npd; ++k) o << "  double pd" << k << " = 0.0;\n";
  o << "  if (i < a.n) {\n";
  for (int k = 0; k < np; ++k) o << "  const double p" << k << " = a.params[" << k << " * a.n + i];\n";
  for (int k = 0; k < ng; ++k) o << "  const double g" << k << " = a.globals[" << k << "];\n";
  if (p.coords) o << "  const float4 xp = a.pos[i];\n  const double cx = xp.x, cy = xp.y, cz = xp.z;\n";
  for (int k = 0; k < ni; ++k) {
    o << "  double J" << k << " = 0.0;\n";
    o << "  for (int c = 0; c < a.chunks; ++c) J" << k << " += (double)a.J[(" << k
      << " * a.chunks + c) * a.n + i];\n";
    o << "  const double I" << k << " = a.S[" << k << "] - J" << k << ";\n";
    o << "  a.I[" << k << " * a.n + i] = I" << k << ";\n  a.If[" << k << " * a.n + i] = (float)I" << k << ";\n";
  }
  // total derivative of value m by a variable: its partial plus the chain
  // through the earlier values (forward mode)
  auto total = [&](int m, const std::string& var, const std::string& prefix, const std::string& suffix) {
    std::string t = ve(D(p.values[m], var));
    for (int l = 0; l < m; ++l)
      t += " + " + ve(D(p.values[m], s.value_names[l])) + " * " + prefix + std::to_string(l) + suffix;
    return t;
  };
  for (int m = 0; m < nv; ++m) {
    const std::string vm = ve(p.values[m]);
    std::ostringstream body;
    for (int k = 0; k < ni; ++k)
      body << "  const double dv" << m << "_" << k << " = " << total(m, s.integrals[k], "dv", "_" + std::to_string(k))
           << ";\n  a.dVdI[(" << m << " * " << ni << " + " << k << ") * a.n + i] = dv" << m << "_" << k << ";\n";
    if (p.coords)
      for (int c = 0; c < 3; ++c)
        body << "  const double dx" << m << "_" << c << " = " << total(m, kCoord[c], "dx", "_" + std::to_string(c))
             << ";\n  a.dVdX[(" << m << " * 3 + " << c << ") * a.n + i] = dx" << m << "_" << c << ";\n";
    for (int k = 0; k < npd; ++k)
      body << "  const double dg" << m << "_" << k << " = "
           << total(m, s.globals[p.pd_index[k]], "dg", "_" + std::to_string(k)) << ";\n  a.dVdG[(" << m << " * "
           << npd << " + " << k << ") * a.n + i] = dg" << m << "_" << k << ";\n";
    o << ve.take_decls();
    o << "  const double v" << m << " = " << vm << ";\n";
    o << "  a.V[" << m << " * a.n + i] = v" << m << ";\n  a.Vf[" << m << " * a.n + i] = (float)v" << m << ";\n";
    o << body.str();
  }
  if (nv > 0) o << "  a.born[i] = v0;\n  if (!isfinite(v0)) atomicOr(a.status, 8u);\n";
  for (int m = 0; m < nv; ++m) o << "  double dEdV" << m << " = 0.0;\n";
  for (int k = 0; k < ni; ++k) o << "  double dEdI" << k << " = 0.0;\n";
  if (p.coords) o << "  double tfx = 0.0, tfy = 0.0, tfz = 0.0;\n";
  {
    std::ostringstream acc;
    for (size_t t = 0; t < p.terms.size(); ++t) {
      if (p.term_types[t] != 0) continue;
      acc << "  e += " << ve(p.terms[t]) << ";\n";
      for (int m = 0; m < nv; ++m) acc << "  dEdV" << m << " += " << ve(D(p.terms[t], s.value_names[m])) << ";\n";
      for (int k = 0; k < ni; ++k) acc << "  dEdI" << k << " += " << ve(D(p.terms[t], s.integrals[k])) << ";\n";
      if (p.coords) {
        acc << "  tfx += " << ve(D(p.terms[t], "x")) << ";\n";
        acc << "  tfy += " << ve(D(p.terms[t], "y")) << ";\n";
        acc << "  tfz += " << ve(D(p.terms[t], "z")) << ";\n";
      }
      for (int k = 0; k < npd; ++k) acc << "  pd" << k << " += " << ve(D(p.terms[t], s.globals[p.pd_index[k]])) << ";\n";
    }
    o << ve.take_decls() << acc.str();
  }
  for (int m = 0; m < nv; ++m)
    o << "  a.dEdV[" << m << " * a.n + i] = (unsigned long long)gbx_fixed(dEdV" << m << ");\n";
  for (int k = 0; k < ni; ++k)
    o << "  a.dEdI[" << k << " * a.n + i] = (unsigned long long)gbx_fixed(dEdI" << k << ");\n";
  // a single-particle term's explicit coordinate dependence is a force on the particle
  if (p.coords)
    o << "  gbx_add_fixed(a.force + i, -tfx);\n  gbx_add_fixed(a.force + a.stride + i, -tfy);\n"
         "  gbx_add_fixed(a.force + 2 * a.stride + i, -tfz);\n";
  o << "  }\n" << block_sum("e", "a.energy_part[blockIdx.x]");
  for (int k = 0; k < npd; ++k)
    o << block_sum("pd" + std::to_string(k), "a.pd_part[blockIdx.x * " + std::to_string(npd) + " + " + std::to_string(k) + "]");
  o << "}\n\n";

  // ---- pair terms (FP32, fast math); each thread sums its own particle's
  // side of every pair it is in
  o << "extern \"C\" __global__ void __launch_bounds__(" << kPairThreads << ") gbx_pair(CustomArgs a) {\n";
  o << "  __shared__ float4 s_pos[" << kPairThreads << "];\n";
  if (np) o << "  __shared__ float s_p[" << np << "][" << kPairThreads << "];\n";
  if (nv) o << "  __shared__ float s_v[" << nv << "][" << kPairThreads << "];\n";
  if (ni) o << "  __shared__ float s_I[" << ni << "][" << kPairThreads << "];\n";
  o << "  __shared__ double s_e[" << kPairThreads << "];\n";
  o << "  const int i = blockIdx.x * blockDim.x + threadIdx.x;\n";
  o << "  const bool own = i < a.n;\n  const int ii = own ? i : 0;\n";
  o << "  const float4 xi = a.pos[ii];\n";
  for (int k = 0; k < np; ++k) o << "  const float p" << k << "_i = a.paramsf[" << k << " * a.n + ii];\n";
  for (int k = 0; k < nv; ++k) o << "  const float v" << k << "_i = a.Vf[" << k << " * a.n + ii];\n";
  for (int k = 0; k < ni; ++k) o << "  const float I" << k << "_i = a.If[" << k << " * a.n + ii];\n";
  for (int k = 0; k < ng; ++k) o << "  const float gf" << k << " = (float)a.globals[" << k << "];\n";
  o << "  float fx = 0.f, fy = 0.f, fz = 0.f;\n  double e = 0.0;\n";
  for (int k = 0; k < nv; ++k) o << "  float gV" << k << " = 0.f;\n";
  for (int k = 0; k < ni; ++k) o << "  float gI" << k << " = 0.f;\n";
  for (int k = 0; k < npd; ++k) o << "  float pdp" << k << " = 0.f;\n";
  // the particle's excluded partners, walked in step with j (both ascend)
  if (p.excluding) o << "  int ex = own ? a.excl_start[i] : 0;\n  const int ex_end = own ? a.excl_start[i + 1] : 0;\n";
  o << "  for (int base = 0; base < a.n; base += " << kPairThreads << ") {\n";
  o << "    const int jl = base + threadIdx.x;\n    if (jl < a.n) {\n      s_pos[threadIdx.x] = a.pos[jl];\n";
  for (int k = 0; k < np; ++k) o << "      s_p[" << k << "][threadIdx.x] = a.paramsf[" << k << " * a.n + jl];\n";
  for (int k = 0; k < nv; ++k) o << "      s_v[" << k << "][threadIdx.x] = a.Vf[" << k << " * a.n + jl];\n";
  for (int k = 0; k < ni; ++k) o << "      s_I[" << k << "][threadIdx.x] = a.If[" << k << " * a.n + jl];\n";
  o << "    }\n    __syncthreads();\n";
  o << "    const int jn = min(" << kPairThreads << ", a.n - base);\n";
  o << "    for (int t = 0; t < jn && own; ++t) {\n      const int j = base + t;\n";
  if (p.excluding)
    o << "      while (ex < ex_end && a.excl[ex] < j) ++ex;\n"
         "      const bool excluded = ex < ex_end && a.excl[ex] == j;\n";
  o << "      if (j == i) continue;\n";
  o << "      const float4 xj = s_pos[t];\n";
  o << "      float dx = xi.x - xj.x, dy = xi.y - xj.y, dz = xi.z - xj.z;\n";
  o << "      if (a.periodic) {\n        dx -= a.L[0] * floorf(dx * a.iL[0] + 0.5f);\n        dy -= a.L[1] * "
       "floorf(dy * a.iL[1] + 0.5f);\n        dz -= a.L[2] * floorf(dz * a.iL[2] + 0.5f);\n      }\n";
  o << "      const float r2 = dx * dx + dy * dy + dz * dz;\n";
  o << "      if (a.cutoff2 > 0.f && r2 >= a.cutoff2) continue;\n      const float r = sqrtf(r2);\n";
  // atom 1 is the lower index (CharmmReferenceGBMV.cpp:281-283): this atom is 1 when j > i
  o << "      const bool lo = i < j;\n";
  for (int k = 0; k < np; ++k) {
    const std::string K = std::to_string(k);
    o << "      const float pa" << K << " = lo ? p" << K << "_i : s_p[" << K << "][t];\n";
    o << "      const float pb" << K << " = lo ? s_p[" << K << "][t] : p" << K << "_i;\n";
  }
  for (int k = 0; k < nv; ++k) {
    const std::string K = std::to_string(k);
    o << "      const float va" << K << " = lo ? v" << K << "_i : s_v[" << K << "][t];\n";
    o << "      const float vb" << K << " = lo ? s_v[" << K << "][t] : v" << K << "_i;\n";
  }
  for (int k = 0; k < ni; ++k) {
    const std::string K = std::to_string(k);
    o << "      const float Ia" << K << " = lo ? I" << K << "_i : s_I[" << K << "][t];\n";
    o << "      const float Ib" << K << " = lo ? s_I[" << K << "][t] : I" << K << "_i;\n";
  }
  {
    expr::SharedEmitter pe(nm.pair, true, "u", "      ");
    std::ostringstream acc;
    acc << "      float dEdr = 0.f;\n";
    for (size_t t = 0; t < p.terms.size(); ++t) {
      if (p.term_types[t] == 0) continue;
      // ParticlePair: an excluded pair contributes nothing
      const bool skip = p.excluding && p.term_types[t] == 1;
      auto W = [&](const std::string& x) { return skip ? "(excluded ? 0.f : " + x + ")" : x; };
      acc << "      if (lo) e += (double)" << W(pe(p.terms[t])) << ";\n";
      acc << "      dEdr += " << W(pe(D(p.terms[t], "r"))) << ";\n";
      for (int k = 0; k < nv; ++k) {
        const std::string n1 = s.value_names[k] + "1", n2 = s.value_names[k] + "2";
        acc << "      gV" << k << " += " << W("(lo ? " + pe(D(p.terms[t], n1)) + " : " + pe(D(p.terms[t], n2)) + ")")
            << ";\n";
      }
      for (int k = 0; k < ni; ++k) {
        const std::string n1 = s.integrals[k] + "1", n2 = s.integrals[k] + "2";
        acc << "      gI" << k << " += " << W("(lo ? " + pe(D(p.terms[t], n1)) + " : " + pe(D(p.terms[t], n2)) + ")")
            << ";\n";
      }
      for (int k = 0; k < npd; ++k)
        acc << "      if (lo) pdp" << k << " += " << W(pe(D(p.terms[t], s.globals[p.pd_index[k]]))) << ";\n";
    }
    o << pe.take_decls() << acc.str();
  }
  // F_i = -dE/dx_i = -(dE/dr) (x_i - x_j) / r
  o << "      const float sr = dEdr / r;\n      fx -= sr * dx;\n      fy -= sr * dy;\n      fz -= sr * dz;\n";
  o << "    }\n    __syncthreads();\n  }\n";
  o << "  if (own) {\n";
  o << "    gbx_add_fixed(a.force + i, (double)fx);\n    gbx_add_fixed(a.force + a.stride + i, (double)fy);\n"
       "    gbx_add_fixed(a.force + 2 * a.stride + i, (double)fz);\n";
  for (int k = 0; k < nv; ++k) o << "    gbx_add_fixed(a.dEdV + " << k << " * a.n + i, (double)gV" << k << ");\n";
  for (int k = 0; k < ni; ++k) o << "    gbx_add_fixed(a.dEdI + " << k << " * a.n + i, (double)gI" << k << ");\n";
  o << "  }\n" << block_sum("e", "a.energy_part[blockIdx.x]");
  for (int k = 0; k < npd; ++k)
    o << block_sum("(double)pdp" + std::to_string(k),
                   "a.pd_part[blockIdx.x * " + std::to_string(npd) + " + " + std::to_string(k) + "]");
  o << "}\n\n";

  // ---- the integrals' adjoint for the chain rule; the values' explicit
  // coordinate and global dependence
  o << "extern \"C\" __global__ void __launch_bounds__(" << kValueThreads << ") gbx_chain(CustomArgs a) {\n";
  if (npd) o << "  __shared__ double s_e[" << kValueThreads << "];\n";
  o << "  const int i = blockIdx.x * blockDim.x + threadIdx.x;\n";
  for (int k = 0; k < npd; ++k) o << "  double pd" << k << " = 0.0;\n";
  o << "  if (i < a.n) {\n";
  for (int m = 0; m < nv; ++m)
    o << "  const double ev" << m << " = (double)(long long)a.dEdV[" << m << " * a.n + i] / 4294967296.0;\n";
  for (int k = 0; k < ni; ++k) {
    o << "  double t" << k << " = (double)(long long)a.dEdI[" << k << " * a.n + i] / 4294967296.0;\n";
    for (int m = 0; m < nv; ++m)
      o << "  t" << k << " += ev" << m << " * a.dVdI[(" << m << " * " << ni << " + " << k << ") * a.n + i];\n";
  }
  // I = S - J: dE/dJ = -dE/dI
  o << "  a.dEdJ[i] = make_float2(" << (ni > 0 ? "(float)(-t0)" : "0.f") << ", "
    << (ni > 1 ? "(float)(-t1)" : "0.f") << ");\n";
  if (nv > 0) o << "  a.dEdB[i] = a.dEdV[i];\n";
  if (p.coords && nv > 0) {
    for (int c = 0; c < 3; ++c) {
      o << "  double fc" << c << " = 0.0;\n";
      for (int m = 0; m < nv; ++m)
        o << "  fc" << c << " += ev" << m << " * a.dVdX[(" << m << " * 3 + " << c << ") * a.n + i];\n";
      o << "  gbx_add_fixed(a.force + " << c << " * a.stride + i, -fc" << c << ");\n";
    }
  }
  for (int k = 0; k < npd; ++k)
    for (int m = 0; m < nv; ++m)
      o << "  pd" << k << " += ev" << m << " * a.dVdG[(" << m << " * " << npd << " + " << k << ") * a.n + i];\n";
  o << "  }\n";
  for (int k = 0; k < npd; ++k)
    o << block_sum("pd" + std::to_string(k), "a.pd_part[blockIdx.x * " + std::to_string(npd) + " + " + std::to_string(k) + "]");
  o << "}\n";
  return o.str();
}

gbx_status compile(CustomPlan& p, std::string& err) {
  const Nvrtc& nv = nvrtc();
  if (!nv.ok()) {
    err = "custom expressions need NVRTC (libnvrtc.so.13), which could not be loaded";
    return GBX_ERR_UNSUPPORTED;
  }
  p.source = generate(p);
  nvrtcProgram prog;
  if (nv.create(&prog, p.source.c_str(), "gbx_custom.cu", 0, nullptr, nullptr) != NVRTC_SUCCESS) {
    err = "nvrtcCreateProgram failed";
    return GBX_ERR_CUDA;
  }
  const char* opts[] = {"--gpu-architecture=sm_103a", "--std=c++17", "-default-device", "--use_fast_math",
                        "-diag-suppress=177"};
  const nvrtcResult cr = nv.compile(prog, 5, opts);
  if (cr != NVRTC_SUCCESS) {
    size_t ls = 0;
    nv.log_size(prog, &ls);
    std::string log(ls, '\0');
    nv.log(prog, &log[0]);
    nv.destroy(&prog);
    err = "compiling the expressions failed: " + log;
    return GBX_ERR_INVALID_ARGUMENT;
  }
  size_t n = 0;
  nv.cubin_size(prog, &n);
  std::vector<char> cubin(n);
  nv.cubin(prog, cubin.data());
  nv.destroy(&prog);
  if (cudaLibraryLoadData(&p.library, cubin.data(), nullptr, nullptr, 0, nullptr, nullptr, 0) != cudaSuccess ||
      cudaLibraryGetKernel(&p.k_values, p.library, "gbx_values") != cudaSuccess ||
      cudaLibraryGetKernel(&p.k_pair, p.library, "gbx_pair") != cudaSuccess ||
      cudaLibraryGetKernel(&p.k_chain, p.library, "gbx_chain") != cudaSuccess) {
    err = std::string("loading the compiled expressions failed: ") + cudaGetErrorString(cudaGetLastError());
    return GBX_ERR_CUDA;
  }
  return GBX_OK;
}

// The argument block the generated kernels receive (layout of kArgsDecl).
struct CustomArgs {
  int n, chunks, parts;
  float cutoff2;
  int periodic;
  float L[3], iL[3];
  const double* params;
  const float* paramsf;
  const double* S;
  const float* J;
  const double* globals;
  const float4* pos;
  double* I;
  float* If;
  double* V;
  float* Vf;
  double* dVdI;
  unsigned long long* dEdV;
  unsigned long long* dEdI;
  double* energy_part;
  unsigned long long* force;
  int stride;
  float2* dEdJ;
  double* born;
  unsigned long long* dEdB;
  unsigned* status;
  double* dVdX;
  const int* excl_start;
  const int* excl;
  double* dVdG;
  double* pd_part;
};

template <class T>
gbx_status alloc(Context* ctx, T** p, size_t count) {
  if (*p) cudaFree(*p);
  *p = nullptr;
  if (count == 0) count = 1;
  if (cudaMalloc((void**)p, sizeof(T) * count) != cudaSuccess) {
    ctx->last_error = "out of device memory (custom expressions)";
    return GBX_ERR_OUT_OF_MEMORY;
  }
  return GBX_OK;
}

}  // namespace

gbx_status custom_build(Context* ctx, const gbx_custom_spec& spec) {
  auto plan = new (std::nothrow) CustomPlan();
  if (!plan) return GBX_ERR_OUT_OF_MEMORY;
  ctx->custom = plan;
  plan->spec = spec;
  try {
    for (auto& e : spec.value_expressions) plan->values.push_back(expr::parse(e));
    for (auto& e : spec.term_expressions) plan->terms.push_back(expr::parse(e));
  } catch (const std::exception& e) {
    ctx->last_error = std::string("expression: ") + e.what();
    return GBX_ERR_INVALID_ARGUMENT;
  }
  plan->term_types = spec.term_types;
  for (size_t k = 0; k < spec.params.size(); ++k)
    if (spec.params[k] == "radius") plan->radius_index = (int)k;
  // every variable must be known to its kind of expression, and a computed
  // value may read only the values before it
  const Names nm = variable_names(spec);
  auto check = [&](const expr::Ptr& e, const std::map<std::string, std::string>& known, const char* what,
                   size_t defined_values) -> bool {
    std::vector<std::string> vars;
    expr::variables(e, vars);
    for (auto& v : vars) {
      if (!known.count(v)) {
        ctx->last_error = std::string(what) + ": unknown variable '" + v + "'";
        return false;
      }
      for (size_t m = defined_values; m < spec.value_names.size(); ++m)
        if (v == spec.value_names[m]) {
          ctx->last_error = std::string(what) + ": computed value '" + v + "' used before it is defined";
          return false;
        }
    }
    return true;
  };
  for (size_t m = 0; m < plan->values.size(); ++m)
    if (!check(plan->values[m], nm.single, "computed value", m)) return GBX_ERR_INVALID_ARGUMENT;
  for (size_t t = 0; t < plan->terms.size(); ++t)
    if (!check(plan->terms[t], plan->term_types[t] == 0 ? nm.single : nm.pair, "energy term",
               spec.value_names.size()))
      return GBX_ERR_INVALID_ARGUMENT;
  // coordinates read by a computed value or a single-particle term
  auto reads_coords = [](const expr::Ptr& e) {
    std::vector<std::string> vars;
    expr::variables(e, vars);
    for (auto& v : vars)
      if (v == "x" || v == "y" || v == "z") return true;
    return false;
  };
  for (auto& e : plan->values) plan->coords = plan->coords || reads_coords(e);
  for (size_t t = 0; t < plan->terms.size(); ++t)
    if (plan->term_types[t] == 0) plan->coords = plan->coords || reads_coords(plan->terms[t]);
  for (auto& g : spec.param_derivs)
    plan->pd_index.push_back((int)(std::find(spec.globals.begin(), spec.globals.end(), g) - spec.globals.begin()));
  bool pair_with_exclusions = false;
  for (int t : plan->term_types) pair_with_exclusions = pair_with_exclusions || t == 1;
  plan->excluding = !spec.exclusions.empty() && pair_with_exclusions;
  // each particle's excluded partners, both directions, ascending
  std::vector<int> excl_start, excl;
  if (plan->excluding) {
    const int n = ctx->n;
    std::vector<std::vector<int>> per(n);
    for (size_t k = 0; k + 1 < spec.exclusions.size(); k += 2) {
      const int a = spec.exclusions[k], b = spec.exclusions[k + 1];
      if (a < 0 || b < 0 || a >= n || b >= n || a == b) {
        ctx->last_error = "exclusion of particles " + std::to_string(a) + " and " + std::to_string(b) +
                          " is out of range";
        return GBX_ERR_INVALID_ARGUMENT;
      }
      per[a].push_back(b);
      per[b].push_back(a);
    }
    excl_start.push_back(0);
    for (auto& v : per) {
      std::sort(v.begin(), v.end());
      v.erase(std::unique(v.begin(), v.end()), v.end());
      excl.insert(excl.end(), v.begin(), v.end());
      excl_start.push_back((int)excl.size());
    }
  }
  std::string err;
  try {
    const gbx_status s = compile(*plan, err);
    if (s != GBX_OK) {
      ctx->last_error = err;
      return s;
    }
  } catch (const std::exception& e) {
    ctx->last_error = std::string("expression: ") + e.what();
    return GBX_ERR_INVALID_ARGUMENT;
  }
  const int n = ctx->n, np = (int)spec.params.size(), ni = (int)spec.integrals.size(),
            nv = (int)spec.value_names.size();
  plan->value_blocks = (n + kValueThreads - 1) / kValueThreads;
  plan->pair_blocks = (n + kPairThreads - 1) / kPairThreads;
  GBX_TRY_CUSTOM(alloc(ctx, &plan->d_params, (size_t)np * n));
  GBX_TRY_CUSTOM(alloc(ctx, &plan->d_paramsf, (size_t)np * n));
  GBX_TRY_CUSTOM(alloc(ctx, &plan->d_S, (size_t)ni));
  GBX_TRY_CUSTOM(alloc(ctx, &plan->d_globals, spec.globals.size()));
  GBX_TRY_CUSTOM(alloc(ctx, &plan->d_V, (size_t)nv * n));
  GBX_TRY_CUSTOM(alloc(ctx, &plan->d_Vf, (size_t)nv * n));
  GBX_TRY_CUSTOM(alloc(ctx, &plan->d_If, (size_t)ni * n));
  GBX_TRY_CUSTOM(alloc(ctx, &plan->d_dVdI, (size_t)nv * ni * n));
  GBX_TRY_CUSTOM(alloc(ctx, &plan->d_dEdV, (size_t)nv * n));
  GBX_TRY_CUSTOM(alloc(ctx, &plan->d_dEdI, (size_t)ni * n));
  const int npd = (int)plan->pd_index.size();
  if (plan->coords) GBX_TRY_CUSTOM(alloc(ctx, &plan->d_dVdX, (size_t)nv * 3 * n));
  if (npd) {
    GBX_TRY_CUSTOM(alloc(ctx, &plan->d_dVdG, (size_t)nv * npd * n));
    GBX_TRY_CUSTOM(alloc(ctx, &plan->d_pd_part, (size_t)(2 * plan->value_blocks + plan->pair_blocks) * npd));
  }
  if (plan->excluding) {
    GBX_TRY_CUSTOM(alloc(ctx, &plan->d_excl_start, excl_start.size()));
    GBX_TRY_CUSTOM(alloc(ctx, &plan->d_excl, excl.size()));
    if (cudaMemcpy(plan->d_excl_start, excl_start.data(), sizeof(int) * excl_start.size(), cudaMemcpyHostToDevice) !=
            cudaSuccess ||
        (!excl.empty() &&
         cudaMemcpy(plan->d_excl, excl.data(), sizeof(int) * excl.size(), cudaMemcpyHostToDevice) != cudaSuccess))
      return GBX_ERR_CUDA;
  }
  const double S[2] = {ctx->S4, ctx->S7};  // the sums of the two integrals' weights
  if (cudaMemcpy(plan->d_S, S, sizeof(double) * ni, cudaMemcpyHostToDevice) != cudaSuccess ||
      (!spec.globals.empty() && cudaMemcpy(plan->d_globals, spec.global_values.data(),
                                           sizeof(double) * spec.globals.size(), cudaMemcpyHostToDevice) !=
                                    cudaSuccess))
    return GBX_ERR_CUDA;
  return GBX_OK;
}

void custom_destroy(Context* ctx) {
  CustomPlan* p = ctx->custom;
  if (!p) return;
  for (void* q : {(void*)p->d_params, (void*)p->d_paramsf, (void*)p->d_S, (void*)p->d_globals, (void*)p->d_V,
                  (void*)p->d_Vf, (void*)p->d_If, (void*)p->d_dVdI, (void*)p->d_dEdV, (void*)p->d_dEdI,
                  (void*)p->d_dVdX, (void*)p->d_excl_start, (void*)p->d_excl, (void*)p->d_dVdG,
                  (void*)p->d_pd_part})
    if (q) cudaFree(q);
  if (p->library) cudaLibraryUnload(p->library);
  delete p;
  ctx->custom = nullptr;
}

int custom_energy_parts(const Context* ctx) {
  return ctx->custom ? ctx->custom->value_blocks + ctx->custom->pair_blocks : 0;
}

gbx_status custom_set_parameters(Context* ctx, const double* params, std::vector<double>& radius) {
  CustomPlan* p = ctx->custom;
  const int n = ctx->n, np = (int)p->spec.params.size();
  p->params.assign((size_t)np * n, 0.0);
  std::vector<float> pf((size_t)np * n);
  radius.assign(n, 0.0);
  for (int i = 0; i < n; ++i)
    for (int k = 0; k < np; ++k) {
      const double v = params[(size_t)i * np + k];
      if (!std::isfinite(v)) {
        ctx->last_error = "custom parameters must be finite (particle " + std::to_string(i) + ")";
        return GBX_ERR_INVALID_ARGUMENT;
      }
      p->params[(size_t)k * n + i] = v;
      pf[(size_t)k * n + i] = (float)v;
    }
  for (int i = 0; i < n; ++i) radius[i] = p->params[(size_t)p->radius_index * n + i];
  if (cudaMemcpy(p->d_params, p->params.data(), sizeof(double) * p->params.size(), cudaMemcpyHostToDevice) !=
          cudaSuccess ||
      cudaMemcpy(p->d_paramsf, pf.data(), sizeof(float) * pf.size(), cudaMemcpyHostToDevice) != cudaSuccess)
    return GBX_ERR_CUDA;
  return GBX_OK;
}

gbx_status custom_set_global(Context* ctx, const char* name, double value) {
  CustomPlan* p = ctx->custom;
  for (size_t k = 0; k < p->spec.globals.size(); ++k)
    if (p->spec.globals[k] == name) {
      p->spec.global_values[k] = value;
      if (cudaMemcpy(p->d_globals + k, &value, sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess)
        return GBX_ERR_CUDA;
      return GBX_OK;
    }
  ctx->last_error = std::string("no global parameter named ") + name;
  return GBX_ERR_INVALID_ARGUMENT;
}

namespace {
CustomArgs args_of(Context* ctx, const float4* pos, unsigned long long* force, int stride) {
  CustomPlan* p = ctx->custom;
  CustomArgs a{};
  a.n = ctx->n;
  a.chunks = ctx->n_chunks;
  a.parts = custom_energy_parts(ctx);
  a.cutoff2 = ctx->cfg.cutoff > 0 ? (float)(ctx->cfg.cutoff * ctx->cfg.cutoff) : 0.0f;
  a.periodic = ctx->cfg.periodic;
  for (int k = 0; k < 3; ++k) {
    a.L[k] = (float)ctx->cfg.box[k];
    a.iL[k] = ctx->cfg.box[k] > 0 ? (float)(1.0 / ctx->cfg.box[k]) : 0.0f;
  }
  a.params = p->d_params;
  a.paramsf = p->d_paramsf;
  a.S = p->d_S;
  a.J = ctx->d_J;
  a.globals = p->d_globals;
  a.pos = pos;
  a.I = ctx->d_integrals;
  a.If = p->d_If;
  a.V = p->d_V;
  a.Vf = p->d_Vf;
  a.dVdI = p->d_dVdI;
  a.dEdV = p->d_dEdV;
  a.dEdI = p->d_dEdI;
  a.energy_part = ctx->d_energy_part;
  a.force = force;
  a.stride = stride;
  a.dEdJ = ctx->d_dEdJ;
  a.born = ctx->d_born;
  a.dEdB = ctx->d_dEdB_fx;
  a.status = ctx->d_status;
  a.dVdX = p->d_dVdX;
  a.excl_start = p->d_excl_start;
  a.excl = p->d_excl;
  a.dVdG = p->d_dVdG;
  a.pd_part = p->d_pd_part;
  return a;
}
}  // namespace

gbx_status launch_custom_energy(Context* ctx, const float4* pos, unsigned long long* force, int stride) {
  CustomPlan* p = ctx->custom;
  CustomArgs a = args_of(ctx, pos, force, stride);
  void* args[] = {&a};
  cudaStream_t st = ctx->stream;
  cudaError_t e = cudaLaunchKernel((const void*)p->k_values, dim3(p->value_blocks), dim3(kValueThreads), args, 0, st);
  if (e == cudaSuccess) {
    CustomArgs b = a;
    b.energy_part = ctx->d_energy_part + p->value_blocks;
    if (b.pd_part) b.pd_part += (size_t)p->value_blocks * p->pd_index.size();
    void* bargs[] = {&b};
    e = cudaLaunchKernel((const void*)p->k_pair, dim3(p->pair_blocks), dim3(kPairThreads), bargs, 0, st);
  }
  if (e == cudaSuccess) e = cudaMemsetAsync(ctx->d_energy_fx, 0, sizeof(unsigned long long), st);
  ctx->launches += 2;
  if (e != cudaSuccess) {
    ctx->last_error = std::string("custom energy launch: ") + cudaGetErrorString(e);
    return GBX_ERR_CUDA;
  }
  return GBX_OK;
}

gbx_status launch_custom_chain_prep(Context* ctx, unsigned long long* force, int stride) {
  CustomPlan* p = ctx->custom;
  CustomArgs a = args_of(ctx, ctx->d_pos, force, stride);
  if (a.pd_part) a.pd_part += (size_t)(p->value_blocks + p->pair_blocks) * p->pd_index.size();
  void* args[] = {&a};
  const cudaError_t e = cudaLaunchKernel((const void*)p->k_chain, dim3(p->value_blocks), dim3(kValueThreads), args,
                                         0, ctx->stream);
  ++ctx->launches;
  if (e != cudaSuccess) {
    ctx->last_error = std::string("custom chain launch: ") + cudaGetErrorString(e);
    return GBX_ERR_CUDA;
  }
  return GBX_OK;
}

gbx_status custom_param_derivs(Context* ctx, double* out, int count) {
  CustomPlan* p = ctx->custom;
  const int npd = (int)p->pd_index.size();
  if (count > npd) {
    ctx->last_error = "more parameter derivatives asked for than were requested at creation";
    return GBX_ERR_INVALID_ARGUMENT;
  }
  if (npd == 0) return GBX_OK;
  const size_t parts = (size_t)(2 * p->value_blocks + p->pair_blocks);
  std::vector<double> h(parts * npd);
  if (cudaStreamSynchronize(ctx->stream) != cudaSuccess ||
      cudaMemcpy(h.data(), p->d_pd_part, sizeof(double) * h.size(), cudaMemcpyDeviceToHost) != cudaSuccess)
    return GBX_ERR_CUDA;
  for (int k = 0; k < count; ++k) {
    double v = 0.0;
    for (size_t b = 0; b < parts; ++b) v += h[b * npd + k];  // fixed order: values, pairs, chain blocks
    out[k] = v;
  }
  return GBX_OK;
}

// For tests without a GPU: the generated CUDA source of an expression set,
// compiled by NVRTC (no device needed).  Writes the NVRTC log on failure.
gbx_status custom_compile_only(const gbx_custom_spec& spec, std::string& log) {
  CustomPlan p;
  p.spec = spec;
  try {
    for (auto& e : spec.value_expressions) p.values.push_back(expr::parse(e));
    for (auto& e : spec.term_expressions) p.terms.push_back(expr::parse(e));
    p.term_types = spec.term_types;
    auto reads_coords = [](const expr::Ptr& e) {
      std::vector<std::string> vars;
      expr::variables(e, vars);
      for (auto& v : vars)
        if (v == "x" || v == "y" || v == "z") return true;
      return false;
    };
    for (auto& e : p.values) p.coords = p.coords || reads_coords(e);
    for (size_t t = 0; t < p.terms.size(); ++t)
      if (p.term_types[t] == 0) p.coords = p.coords || reads_coords(p.terms[t]);
    for (auto& g : spec.param_derivs)
      p.pd_index.push_back((int)(std::find(spec.globals.begin(), spec.globals.end(), g) - spec.globals.begin()));
    for (int t : p.term_types) p.excluding = p.excluding || (t == 1 && !spec.exclusions.empty());
    const Nvrtc& nv = nvrtc();
    if (!nv.ok()) {
      log = "NVRTC could not be loaded";
      return GBX_ERR_UNSUPPORTED;
    }
    p.source = generate(p);
    nvrtcProgram prog;
    if (nv.create(&prog, p.source.c_str(), "gbx_custom.cu", 0, nullptr, nullptr) != NVRTC_SUCCESS)
      return GBX_ERR_CUDA;
    const char* opts[] = {"--gpu-architecture=sm_103a", "--std=c++17", "-default-device", "--use_fast_math",
                          "-diag-suppress=177"};
    const nvrtcResult cr = nv.compile(prog, 5, opts);
    size_t ls = 0;
    nv.log_size(prog, &ls);
    log.assign(ls, '\0');
    nv.log(prog, &log[0]);
    nv.destroy(&prog);
    return cr == NVRTC_SUCCESS ? GBX_OK : GBX_ERR_INVALID_ARGUMENT;
  } catch (const std::exception& e) {
    log = e.what();
    return GBX_ERR_INVALID_ARGUMENT;
  }
}

}  // namespace gbx
