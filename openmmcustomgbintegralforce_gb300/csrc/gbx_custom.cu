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
#include <cstdio>
#include <cmath>
#include <cstring>
#include <map>
#include <set>
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
  const int* excl_row;       // [tiles + 1] each 32-particle tile's entries in excl_tile
  const int* excl_tile;      // the partner tile J >= I of each entry
  const unsigned* excl_mask; // [entries][32] bit b of word l: particles l of I and b of J are excluded
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
// FP32 sums to fixed point without the FP64 pipe: floor(v) 2^32 plus the
// fraction's 2^32 multiple, two 32-bit conversions (|v| < 2^31; within
// 2^-25 of round(v 2^32))
__device__ __forceinline__ long long gbx_fixed_f(float v) {
  const float hf = floorf(v);
  const unsigned lo = __float2uint_rn((v - hf) * 4294967296.0f);
  return (long long)(((unsigned long long)(long long)__float2int_rz(hf) << 32) + lo);
}
__device__ __forceinline__ void gbx_add_fixed_f(unsigned long long* p, float v) {
  const long long q = gbx_fixed_f(v);
  if (q) atomicAdd(p, (unsigned long long)q);
}
// A tabulated function (natural cubic spline, zero outside [x0, x1]) and its
// first and second derivatives: interval i holds c0 + u (c1 + u (c2 + u c3))
// in u = (x - x_i) / h
template <class T, int D>
__device__ __forceinline__ T gbx_spline(const T* __restrict__ c, int intervals, T x0, T x1, T ih, T x) {
  if (!(x >= x0 && x <= x1)) return T(0);
  const T s = (x - x0) * ih;
  int i = (int)s;
  i = i < intervals - 1 ? i : intervals - 1;
  const T u = s - (T)i;
  const T* k = c + 4 * i;
  if (D == 0) return k[0] + u * (k[1] + u * (k[2] + u * k[3]));
  if (D == 1) return (k[1] + u * ((T)2 * k[2] + (T)3 * u * k[3])) * ih;
  return ((T)2 * k[2] + (T)6 * u * k[3]) * ih * ih;
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
  int* d_excl_row = nullptr;
  int* d_excl_tile = nullptr;
  unsigned* d_excl_mask = nullptr;
  double* d_dVdG = nullptr;
  double* d_pd_part = nullptr;
  bool coords = false;      // some computed value or single-particle term reads x, y or z
  bool excluding = false;   // exclusions exist and some term honours them
  bool cutoff = false;      // pair terms only within the cutoff (fixed at creation)
  bool periodic = false;    // pair distances by minimum image (fixed at creation)
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

// Natural cubic spline through evenly spaced values (second derivatives M
// from the tridiagonal system M[i-1] + 4 M[i] + M[i+1] = 6 (y[i+1] - 2 y[i]
// + y[i-1]) / h^2 with M = 0 at both ends, the standard construction OpenMM
// documents for Continuous1DFunction), as four power-form coefficients per
// interval in u = (x - x_i) / h.
std::vector<double> spline_coefficients(const gbx_custom_spec::Function& f) {
  const int n = (int)f.y.size();
  const double h = (f.x1 - f.x0) / (n - 1);
  std::vector<double> M(n, 0.0), cp(n, 0.0), dp(n, 0.0);
  for (int i = 1; i < n - 1; ++i) {
    const double rhs = 6.0 * (f.y[i + 1] - 2.0 * f.y[i] + f.y[i - 1]) / (h * h);
    const double den = 4.0 - cp[i - 1];
    cp[i] = 1.0 / den;
    dp[i] = (rhs - dp[i - 1]) / den;
  }
  for (int i = n - 2; i >= 1; --i) M[i] = dp[i] - cp[i] * M[i + 1];
  std::vector<double> c;
  const double h6 = h * h / 6.0;
  for (int i = 0; i + 1 < n; ++i) {
    c.push_back(f.y[i]);
    c.push_back((f.y[i + 1] - f.y[i]) - h6 * (2.0 * M[i] + M[i + 1]));
    c.push_back(3.0 * h6 * M[i]);
    c.push_back(h6 * (M[i + 1] - M[i]));
  }
  return c;
}

// Each tabulated function's coefficients (FP64 and FP32 copies) and
// gbx_tab_<name>_<derivative>(x) in both precisions.
std::string tabulated_source(const gbx_custom_spec& s) {
  std::ostringstream o;
  char buf[64];
  auto d = [&](double v) {
    std::snprintf(buf, sizeof(buf), "%.17g", v);
    return std::string(buf);
  };
  auto f = [&](double v) {
    std::snprintf(buf, sizeof(buf), "%.9ef", (double)(float)v);
    return std::string(buf);
  };
  for (size_t k = 0; k < s.functions.size(); ++k) {
    const auto& fn = s.functions[k];
    const std::vector<double> c = spline_coefficients(fn);
    const int intervals = (int)fn.y.size() - 1;
    const double ih = intervals / (fn.x1 - fn.x0);
    const std::string K = std::to_string(k);
    o << "__device__ const double gbx_tcd_" << K << "[" << c.size() << "] = {";
    for (size_t q = 0; q < c.size(); ++q) o << (q ? ", " : "") << d(c[q]);
    o << "};\n__device__ const float gbx_tcf_" << K << "[" << c.size() << "] = {";
    for (size_t q = 0; q < c.size(); ++q) o << (q ? ", " : "") << f(c[q]);
    o << "};\n";
    for (int D = 0; D < 3; ++D) {
      o << "__device__ __forceinline__ double gbx_tab_" << fn.name << "_" << D << "(double x) { return gbx_spline<double, "
        << D << ">(gbx_tcd_" << K << ", " << intervals << ", " << d(fn.x0) << ", " << d(fn.x1) << ", " << d(ih)
        << ", x); }\n";
      o << "__device__ __forceinline__ float gbx_tab_" << fn.name << "_" << D << "(float x) { return gbx_spline<float, "
        << D << ">(gbx_tcf_" << K << ", " << intervals << ", " << f(fn.x0) << ", " << f(fn.x1) << ", " << f(ih)
        << ", x); }\n";
    }
  }
  return o.str();
}

std::string generate(const CustomPlan& p) {
  const gbx_custom_spec& s = p.spec;
  const int np = (int)s.params.size(), ng = (int)s.globals.size(), ni = (int)s.integrals.size(),
            nv = (int)s.value_names.size(), npd = (int)p.pd_index.size();
  const Names nm = variable_names(s);
  const char* kCoord[3] = {"x", "y", "z"};
  auto D = [](const expr::Ptr& e, const std::string& v) { return expr::derivative(e, v); };
  std::ostringstream o;
  o << kArgsDecl << kPrelude << tabulated_source(s);

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

  // ---- pair terms (FP32, fast math).  Each unordered pair once: tiles of
  // 32 particles, tile pairs (I, J) with I <= J numbered row by row and
  // split into contiguous runs, one run per warp.  A lane holds particle i
  // of tile I; tile J's particles and their sums rotate through the warp
  // by one lane a step, so at step k lane l meets particle (l + k) mod 32
  // of tile J.  On a diagonal tile steps 1..15, and step 16 for the lower
  // half of the lanes, meet every pair once.
  {
    // what the pair terms read: per-particle inputs rotated with j, and the
    // derivatives summed for each particle
    std::set<std::string> used;
    for (size_t t = 0; t < p.terms.size(); ++t) {
      if (p.term_types[t] == 0) continue;
      std::vector<std::string> vars;
      expr::variables(p.terms[t], vars);
      used.insert(vars.begin(), vars.end());
    }
    auto uses = [&](const std::string& name) { return used.count(name + "1") || used.count(name + "2"); };
    std::vector<int> up, uv, ui;
    for (int k = 0; k < np; ++k)
      if (uses(s.params[k])) up.push_back(k);
    for (int k = 0; k < nv; ++k)
      if (uses(s.value_names[k])) uv.push_back(k);
    for (int k = 0; k < ni; ++k)
      if (uses(s.integrals[k])) ui.push_back(k);
    std::vector<std::string> inputs;  // "p0", "v1", "I0": arrays a.paramsf / a.Vf / a.If
    auto array_of = [](const std::string& in) {
      return in[0] == 'p' ? std::string("a.paramsf") : in[0] == 'v' ? std::string("a.Vf") : std::string("a.If");
    };
    for (int k : up) inputs.push_back("p" + std::to_string(k));
    for (int k : uv) inputs.push_back("v" + std::to_string(k));
    for (int k : ui) inputs.push_back("I" + std::to_string(k));
    std::vector<std::string> sums = {"fx", "fy", "fz"};  // per-particle sums
    for (int k : uv) sums.push_back("gV" + std::to_string(k));
    for (int k : ui) sums.push_back("gI" + std::to_string(k));
    // the rotation: every lane takes the j data and sums of the next lane
    std::string rot;
    auto shfl = [&](const std::string& v) {
      rot += "        " + v + " = __shfl_sync(0xffffffffu, " + v + ", (lane + 1) & 31);\n";
    };
    for (const char* c : {"xj.x", "xj.y", "xj.z"}) shfl(c);
    for (auto& in : inputs) shfl(in + "_j");
    for (auto& sm : sums) shfl(sm + "_j");
    auto sum_target = [](const std::string& sname, const std::string& idx) {
      if (sname == "fx") return "a.force + " + idx;
      if (sname == "fy") return "a.force + a.stride + " + idx;
      if (sname == "fz") return "a.force + 2 * a.stride + " + idx;
      if (sname[1] == 'V') return "a.dEdV + " + sname.substr(2) + " * a.n + " + idx;
      return "a.dEdI + " + sname.substr(2) + " * a.n + " + idx;
    };

    o << "extern \"C\" __global__ void __launch_bounds__(" << kPairThreads << ") gbx_pair(CustomArgs a) {\n";
    o << "  __shared__ double s_e[" << kPairThreads << "];\n";
    o << "  const int lane = threadIdx.x & 31;\n";
    o << "  const int nt = (a.n + 31) >> 5;\n";
    o << "  const long long T = (long long)nt * (nt + 1) / 2;\n";
    o << "  const long long W = (long long)gridDim.x * (blockDim.x >> 5);\n";
    o << "  const long long w = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);\n";
    o << "  long long t = w * T / W;\n  const long long t_end = (w + 1) * T / W;\n";
    // the row of tile t: the largest I with I * nt - I * (I - 1) / 2 <= t
    o << "  auto row_start = [nt](long long r) { return r * nt - r * (r - 1) / 2; };\n";
    o << "  const double b2 = 2.0 * nt + 1.0;\n";
    o << "  int I = (int)((b2 - sqrt(fmax(b2 * b2 - 8.0 * (double)t, 0.0))) * 0.5);\n";
    o << "  I = max(0, min(I, nt - 1));\n";
    o << "  while (I > 0 && row_start(I) > t) --I;\n  while (I + 1 < nt && row_start(I + 1) <= t) ++I;\n";
    o << "  int J = I + (int)(t - row_start(I));\n";
    o << "  double e = 0.0;\n";
    for (int k = 0; k < npd; ++k) o << "  double pdp" << k << " = 0.0;\n";
    for (int k = 0; k < ng; ++k) o << "  const float gf" << k << " = (float)a.globals[" << k << "];\n";
    o << "  int cur = -1, i = 0;\n  bool iok = false;\n  float4 xi = make_float4(0.f, 0.f, 0.f, 0.f);\n";
    for (auto& in : inputs) o << "  float " << in << "_i = 0.f;\n";
    for (auto& sm : sums) o << "  float " << sm << "_i = 0.f;\n";
    o << "  for (; t < t_end; ++t) {\n";
    o << "    if (I != cur) {\n";
    o << "      if (iok) {\n";
    for (auto& sm : sums) o << "        gbx_add_fixed_f(" << sum_target(sm, "i") << ", " << sm << "_i);\n";
    o << "      }\n";
    o << "      cur = I;\n      i = I * 32 + lane;\n      iok = i < a.n;\n      const int ii = iok ? i : 0;\n";
    o << "      xi = a.pos[ii];\n";
    for (auto& in : inputs)
      o << "      " << in << "_i = " << array_of(in) << "[" << in.substr(1) << " * a.n + ii];\n";
    for (auto& sm : sums) o << "      " << sm << "_i = 0.f;\n";
    o << "    }\n";
    o << "    const bool diag = I == J;\n";
    o << "    const int j0 = J * 32 + lane;\n    const int jj = j0 < a.n ? j0 : 0;\n";
    o << "    float4 xj = a.pos[jj];\n";
    for (auto& in : inputs) o << "    float " << in << "_j = " << array_of(in) << "[" << in.substr(1) << " * a.n + jj];\n";
    for (auto& sm : sums) o << "    float " << sm << "_j = 0.f;\n";
    if (p.excluding) {
      // the tile's exclusion mask: bit b of lane l's word excludes particle
      // b of tile J for particle l of tile I
      o << "    unsigned xmask = 0u;\n";
      o << "    for (int q = a.excl_row[I]; q < a.excl_row[I + 1]; ++q)\n";
      o << "      if (a.excl_tile[q] == J) { xmask = a.excl_mask[q * 32 + lane]; break; }\n";
    }
    o << "    float et = 0.f;\n";
    for (int k = 0; k < npd; ++k) o << "    float pdt" << k << " = 0.f;\n";
    // one pair: `full` for a whole off-diagonal tile (i < j always, every
    // particle present), else the general case with the ordering selects
    auto pair_body = [&](bool full, const std::string& ind) {
      std::ostringstream b;
      b << ind << "float dx = xi.x - xj.x, dy = xi.y - xj.y, dz = xi.z - xj.z;\n";
      if (p.periodic)
        b << ind << "dx -= a.L[0] * floorf(dx * a.iL[0] + 0.5f);\n" << ind
          << "dy -= a.L[1] * floorf(dy * a.iL[1] + 0.5f);\n" << ind << "dz -= a.L[2] * floorf(dz * a.iL[2] + 0.5f);\n";
      b << ind << "const float r2 = dx * dx + dy * dy + dz * dz;\n";
      std::string in2 = ind;
      if (p.cutoff) {
        b << ind << "if (r2 < a.cutoff2) {\n";
        in2 += "  ";
      }
      b << in2 << "const float r = sqrtf(r2);\n";
      if (p.excluding) b << in2 << "const bool excluded = (xmask >> jl) & 1u;\n";
      // atom 1 is the lower index (CharmmReferenceGBMV.cpp:281-283)
      if (!full) b << in2 << "const bool lo = i < j;\n";
      auto side = [&](const std::string& a_name, const std::string& b_name, const std::string& in) {
        if (full) {
          b << in2 << "const float " << a_name << " = " << in << "_i, " << b_name << " = " << in << "_j;\n";
        } else {
          b << in2 << "const float " << a_name << " = lo ? " << in << "_i : " << in << "_j;\n";
          b << in2 << "const float " << b_name << " = lo ? " << in << "_j : " << in << "_i;\n";
        }
      };
      for (int k : up) side("pa" + std::to_string(k), "pb" + std::to_string(k), "p" + std::to_string(k));
      for (int k : uv) side("va" + std::to_string(k), "vb" + std::to_string(k), "v" + std::to_string(k));
      for (int k : ui) side("Ia" + std::to_string(k), "Ib" + std::to_string(k), "I" + std::to_string(k));
      expr::SharedEmitter pe(nm.pair, true, "u", in2);
      std::ostringstream acc;
      acc << in2 << "float dEdr = 0.f;\n";
      for (size_t t = 0; t < p.terms.size(); ++t) {
        if (p.term_types[t] == 0) continue;
        // ParticlePair: an excluded pair contributes nothing
        const bool skip = p.excluding && p.term_types[t] == 1;
        auto W = [&](const std::string& x) { return skip ? "(excluded ? 0.f : " + x + ")" : x; };
        acc << in2 << "et += " << W(pe(p.terms[t])) << ";\n";
        acc << in2 << "dEdr += " << W(pe(D(p.terms[t], "r"))) << ";\n";
        auto both = [&](const std::string& sname, const std::string& base) {
          const std::string d1 = W(pe(D(p.terms[t], base + "1"))), d2 = W(pe(D(p.terms[t], base + "2")));
          if (full) {
            acc << in2 << sname << "_i += " << d1 << ";\n" << in2 << sname << "_j += " << d2 << ";\n";
          } else {
            acc << in2 << sname << "_i += lo ? " << d1 << " : " << d2 << ";\n";
            acc << in2 << sname << "_j += lo ? " << d2 << " : " << d1 << ";\n";
          }
        };
        for (int k : uv) both("gV" + std::to_string(k), s.value_names[k]);
        for (int k : ui) both("gI" + std::to_string(k), s.integrals[k]);
        for (int k = 0; k < npd; ++k)
          acc << in2 << "pdt" << k << " += " << W(pe(D(p.terms[t], s.globals[p.pd_index[k]]))) << ";\n";
      }
      b << pe.take_decls() << acc.str();
      // F_i = -dE/dx_i = -(dE/dr) (x_i - x_j) / r, and F_j the opposite
      b << in2 << "const float sr = dEdr / r;\n";
      b << in2 << "fx_i -= sr * dx;\n" << in2 << "fy_i -= sr * dy;\n" << in2 << "fz_i -= sr * dz;\n";
      b << in2 << "fx_j += sr * dx;\n" << in2 << "fy_j += sr * dy;\n" << in2 << "fz_j += sr * dz;\n";
      if (p.cutoff) b << ind << "}\n";
      return b.str();
    };
    o << "    if (!diag && J * 32 + 32 <= a.n) {\n";
    o << "      for (int k = 0; k < 32; ++k) {\n";
    if (p.excluding) o << "        const int jl = (lane + k) & 31;\n";
    o << pair_body(true, "        ");
    o << rot;
    o << "      }\n";
    o << "    } else {\n";
    o << "      for (int k = 0; k < 32; ++k) {\n";
    o << "        const int jl = (lane + k) & 31;\n        const int j = J * 32 + jl;\n";
    o << "        if (iok && j < a.n && (!diag || (k >= 1 && (k < 16 || lane < 16)))) {\n";
    o << pair_body(false, "          ");
    o << "        }\n";
    o << "        if (diag && k == 16) break;\n";
    o << rot;
    o << "      }\n";
    o << "    }\n";
    o << "    e += (double)et;\n";
    for (int k = 0; k < npd; ++k) o << "    pdp" << k << " += (double)pdt" << k << ";\n";
    // the j data's particle after the rotations: 32 steps bring it back, a
    // diagonal tile stops after 16
    o << "    const int jn = J * 32 + ((lane + (diag ? 16 : 0)) & 31);\n";
    o << "    if (jn < a.n) {\n";
    for (auto& sm : sums) o << "      gbx_add_fixed_f(" << sum_target(sm, "jn") << ", " << sm << "_j);\n";
    o << "    }\n";
    o << "    if (++J == nt) { ++I; J = I; }\n";
    o << "  }\n";
    o << "  if (iok) {\n";
    for (auto& sm : sums) o << "    gbx_add_fixed_f(" << sum_target(sm, "i") << ", " << sm << "_i);\n";
    o << "  }\n";
    o << block_sum("e", "a.energy_part[blockIdx.x]");
    for (int k = 0; k < npd; ++k)
      o << block_sum("pdp" + std::to_string(k),
                     "a.pd_part[blockIdx.x * " + std::to_string(npd) + " + " + std::to_string(k) + "]");
    o << "}\n\n";
  }

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
  const int* excl_row;
  const int* excl_tile;
  const unsigned* excl_mask;
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
    std::set<std::string> fnames;
    for (auto& f : spec.functions) fnames.insert(f.name);
    for (auto& e : spec.value_expressions) plan->values.push_back(expr::parse(e, fnames));
    for (auto& e : spec.term_expressions) plan->terms.push_back(expr::parse(e, fnames));
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
  plan->cutoff = ctx->cfg.cutoff > 0;
  plan->periodic = ctx->cfg.periodic != 0;
  // exclusions as 32 x 32 bit masks of the tile pairs (I <= J) that hold
  // any: bit b of word l excludes particle l of tile I with particle b of
  // tile J (on a diagonal tile both ways)
  std::vector<int> excl_row, excl_tile;
  std::vector<unsigned> excl_mask;
  if (plan->excluding) {
    const int n = ctx->n, nt = (n + 31) / 32;
    std::vector<std::map<int, std::vector<unsigned>>> rows(nt);
    for (size_t k = 0; k + 1 < spec.exclusions.size(); k += 2) {
      const int a = spec.exclusions[k], b = spec.exclusions[k + 1];
      if (a < 0 || b < 0 || a >= n || b >= n || a == b) {
        ctx->last_error = "exclusion of particles " + std::to_string(a) + " and " + std::to_string(b) +
                          " is out of range";
        return GBX_ERR_INVALID_ARGUMENT;
      }
      const int lo = std::min(a, b), hi = std::max(a, b);
      auto& m = rows[lo / 32][hi / 32];
      m.resize(32, 0u);
      m[lo % 32] |= 1u << (hi % 32);
      if (lo / 32 == hi / 32) m[hi % 32] |= 1u << (lo % 32);
    }
    excl_row.push_back(0);
    for (auto& row : rows) {
      for (auto& [J, m] : row) {
        excl_tile.push_back(J);
        excl_mask.insert(excl_mask.end(), m.begin(), m.end());
      }
      excl_row.push_back((int)excl_tile.size());
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
  {
    // tile pairs over warps: up to 32 warps per multiprocessor
    const long long nt = (n + 31) / 32, tiles = nt * (nt + 1) / 2;
    const long long warps = std::min<long long>(tiles, 32LL * std::max(ctx->sms, 1));
    plan->pair_blocks = (int)((warps + kPairThreads / 32 - 1) / (kPairThreads / 32));
  }
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
    GBX_TRY_CUSTOM(alloc(ctx, &plan->d_excl_row, excl_row.size()));
    GBX_TRY_CUSTOM(alloc(ctx, &plan->d_excl_tile, excl_tile.size()));
    GBX_TRY_CUSTOM(alloc(ctx, &plan->d_excl_mask, excl_mask.size()));
    if (cudaMemcpy(plan->d_excl_row, excl_row.data(), sizeof(int) * excl_row.size(), cudaMemcpyHostToDevice) !=
            cudaSuccess ||
        (!excl_tile.empty() &&
         (cudaMemcpy(plan->d_excl_tile, excl_tile.data(), sizeof(int) * excl_tile.size(), cudaMemcpyHostToDevice) !=
              cudaSuccess ||
          cudaMemcpy(plan->d_excl_mask, excl_mask.data(), sizeof(unsigned) * excl_mask.size(),
                     cudaMemcpyHostToDevice) != cudaSuccess)))
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
                  (void*)p->d_dVdX, (void*)p->d_excl_row, (void*)p->d_excl_tile, (void*)p->d_excl_mask,
                  (void*)p->d_dVdG, (void*)p->d_pd_part})
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
  a.excl_row = p->d_excl_row;
  a.excl_tile = p->d_excl_tile;
  a.excl_mask = p->d_excl_mask;
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
    std::set<std::string> fnames;
    for (auto& f : spec.functions) fnames.insert(f.name);
    for (auto& e : spec.value_expressions) p.values.push_back(expr::parse(e, fnames));
    for (auto& e : spec.term_expressions) p.terms.push_back(expr::parse(e, fnames));
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
