/*
 * gbx -- GB300-native CHARMM GBSW / GBMV implicit-solvent energy and forces.
 *
 * Plain C ABI over the CUDA implementation (sm_103a).  No C++ or torch types
 * cross this boundary: handles are opaque, arrays are raw pointers with
 * explicit sizes, every call returns a gbx_status and never throws.
 *
 * One gbx_context plays the role of one instance of the reference's kernel
 * objects: it is what CalcCharmmGBSWForceKernel / CalcCharmmGBMVForceKernel
 * (openmmapi/include/openmm/charmmKernels.h:49-129) hold between
 * initialize(), execute() and copyParametersToContext().  An OpenMM plugin
 * adapter is a thin C++ layer that forwards those three virtuals to the
 * calls below.
 *
 * Units: nm, e, kJ/mol.  Device buffers follow OpenMM's CUDA conventions:
 * positions as float4 (x, y, z, unused), forces as 64-bit fixed point
 * (value * 2^32, two's complement) laid out [x(stride) | y(stride) | z(stride)].
 */
#ifndef GBX_H
#define GBX_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(_WIN32)
#define GBX_API __declspec(dllexport)
#else
#define GBX_API __attribute__((visibility("default")))
#endif

typedef struct gbx_context gbx_context;
typedef struct gbx_batch gbx_batch;

typedef enum {
  GBX_OK = 0,
  GBX_ERR_INVALID_ARGUMENT = 1,
  GBX_ERR_CUDA = 2,
  GBX_ERR_OUT_OF_MEMORY = 3,
  GBX_ERR_UNSUPPORTED = 4,
  GBX_ERR_NONFINITE = 5,      /* a Born radius or the energy came out NaN/Inf */
  GBX_ERR_TABLE_TOO_LARGE = 6, /* lookup grid would exceed its limits (reference: length > 1000 nm) */
  GBX_ERR_NOT_READY = 7,      /* result queried before an execute */
  GBX_ERR_TIMEOUT = 8,        /* reserved for a device-side wait that gives up; no kernel of this
                                 library waits on another (no spin, no grid barrier), so no
                                 entry point returns it */
  GBX_ERR_EXCEEDS_STATIC_SCRATCH = 9, /* gbx_pair_noalloc: more atoms than its static scratch holds */
  GBX_ERR_STALE_RESULT = 10   /* gbx_execute: an earlier unchecked call's lookup table outgrew its
                                 buffers, so that call's results lacked the volume terms; the
                                 buffers were grown and the reporting call's results are complete */
} gbx_status;

/* Volume models: CharmmGBMVForce::GBIntegralType (CharmmGBMVForce.h:99-104). */
enum { GBX_MODEL_GBSW = 0, GBX_MODEL_GBMV1 = 1, GBX_MODEL_GBMV2 = 2 };

/* Lookup-table semantics. */
enum {
  GBX_TABLE_STANDALONE = 0, /* CharmmReferenceGBSW.cpp:440-552: grid points, uniform pad, uncapped */
  GBX_TABLE_GRID = 1,       /* CustomGBIntegral.cpp:162-228,310-324: grid points, per-atom pad, capped */
  GBX_TABLE_PERIODIC = 2    /* CustomGBIntegral.cpp:45-160,284-309: box grid, sampled membership, capped */
};

/* Presets reproducing the reference's native settings. */
enum {
  GBX_PRESET_CHARMM_GBSW = 0,   /* CharmmGBSWForce, Reference platform */
  GBX_PRESET_GBSW_INTEGRAL = 1, /* CharmmGBMVForce + GBSWIntegral */
  GBX_PRESET_GBMV1 = 2,         /* CharmmGBMVForce + GBMVIntegralTypeI */
  GBX_PRESET_GBMV2 = 3          /* CharmmGBMVForce + GBMVIntegralTypeII */
};

/* Execute flags. */
enum {
  GBX_EXEC_FORCES = 1,  /* includeForces  */
  GBX_EXEC_ENERGY = 2,  /* includeEnergy  */
  GBX_EXEC_CHECK = 4,   /* synchronise the stream and report device status (table
                           capacity, non-finite values); grows buffers and
                           re-runs once if a capacity limit was hit */
  GBX_EXEC_COUNT_WORK = 8, /* count (point, listed atom) evaluations (gbx_get_work) */
  GBX_EXEC_POSQ_DOUBLE = 16, /* gbx_execute: posq is double4 (OpenMM's double precision mode) */
  GBX_EXEC_ENERGY_FLOAT = 32 /* gbx_execute: energy points to one float, added to (OpenMM's
                                single precision energy buffer) */
};

typedef struct {
  int model;            /* GBX_MODEL_* */
  int n_radial;         /* Gauss-Legendre points on [r0, r1] */
  int lebedev_order;    /* 6, 14, 26, 38, 50, 74, 86 or 110 */
  double r0, r1;        /* radial integration range (nm) */
  int table_mode;       /* GBX_TABLE_* */
  int table_cap;        /* per-cell cap (<= 0: uncapped) */
  double grid_length;   /* lookup grid spacing h (nm) */
  double table_buffer;  /* buffer length (nm) */
  double box[3];        /* periodic box edge lengths (GBX_TABLE_PERIODIC) */
  double switch_width;  /* GBSW half-width w (nm) */
  double gamma0, beta, lambda, p1, p2, s0; /* GBMV constants */
  double alpha0, alpha1; /* Born-radius coefficients (global parameters) */
  double prefactor;     /* pair prefactor, -ONE_4PI_EPS0 (1 - 1/80) by default */
  double cutoff;        /* <= 0: full N^2 pair term */
  int cutoff_chain_quirk; /* drop chain terms beyond the cutoff (CharmmReferenceGBSW.cpp:291-292) */
  int skip_empty;       /* GBSW: an empty list means V = 1 */
  int table_policy;     /* GBX_TABLE_POLICY_* */
  int periodic;         /* CutoffPeriodic (GBSW, standalone table): minimum-image distances in the
                           rectangular box[3] (edges >= 2 cutoff), the table query wrapped once per
                           axis (CharmmReferenceGBSW.cpp:242-243,287-288,522-535,620-621,647-648) */
  double tight_grid_length; /* cell edge of the exact GBSW table (nm); <= 0: 0.1 */
  int integral_orders[2];   /* orders n of the two GB integrals (weights w / r^(n-2),
                               GBSWIntegral.cpp:96,144); 0: 4 and 7 */
  int reserved[2];
} gbx_config;

/* Which table the integrals read.  The reference's standalone GBSW table
 * (GBX_TABLE_STANDALONE) pads every cell by more than any switching shell
 * can reach, so the volume it yields is the exact product over all atoms.
 * AUTO then evaluates the integrals on a tighter table that provably holds
 * the same atoms for every point (sphere-box membership with a safety
 * margin, fully buried cells marked), which gives the same volumes with a
 * fraction of the list work; the reference table is still built on request
 * (gbx_build_lookup_table).  For the other table modes the list contents
 * define the result, so the reference table is always used. */
enum { GBX_TABLE_POLICY_AUTO = 0, GBX_TABLE_POLICY_REFERENCE = 1 };

/* Library / error helpers. */
GBX_API const char* gbx_status_string(gbx_status s);
GBX_API int gbx_version(void);

/* Fill *cfg with a preset (reference constants: CharmmReferenceGBSW.cpp:20-52,
 * GBSWIntegral.cpp:24-61, GBMVIntegralTypeI.cpp:18-57, GBMVIntegralTypeII.cpp:19-62). */
GBX_API gbx_status gbx_config_preset(int preset, gbx_config* cfg);

/* Create a context for num_atoms particles on the current CUDA device.
 * Replaces CalcCharmmGBSWForceKernel::initialize / CalcCharmmGBMVForceKernel::initialize
 * (charmmKernels.h:71,111; CharmmCudaKernels.cpp:136-843). */
GBX_API gbx_status gbx_create(const gbx_config* cfg, int num_atoms, gbx_context** out);
GBX_API gbx_status gbx_destroy(gbx_context* ctx);
GBX_API gbx_status gbx_last_error(const gbx_context* ctx, char* buf, size_t len);

/* Per-particle charge (e) and input radius (nm).  Replaces
 * copyParametersToContext (charmmKernels.h:88,128; CharmmReferenceKernels.cpp:439-458). */
GBX_API gbx_status gbx_set_particle_parameters(gbx_context* ctx, const double* charge, const double* radius);
/* ------------------------------------------------------------------------
 * A CharmmGBMVForce with expressions outside the canonical CHARMM set
 * (CharmmGBMVForce.h:294-391: computed values and energy terms).  Replaces
 * the reference's runtime-generated kernels (CharmmCudaKernels.cpp:228-827;
 * CharmmReferenceGBMV.cpp:151-444 on the CPU): the expressions and their
 * derivatives are compiled for the device when the context is created (NVRTC,
 * loaded at run time).  Variables: per-particle parameters, globals, the GB
 * integrals and earlier computed values by name, and in computed values and
 * single-particle terms the particle's coordinates x, y, z (their gradients
 * become forces, CharmmReferenceGBMV.cpp:232-262,409-435); pair terms read r
 * and every per-particle quantity with the suffix 1 or 2 (atom 1 is the
 * lower index).  GBX_TERM_PAIR terms skip the excluded pairs,
 * GBX_TERM_PAIR_NO_EXCLUSIONS terms do not (CharmmReferenceGBMV.cpp:196-200).
 * Tabulated functions of one variable (Continuous1DFunction) may appear in
 * any expression.  One or two integrals; computed values are SingleParticle.  Per-particle
 * parameters must include "radius" (GBSWIntegral.cpp:79-80); x, y and z name
 * no parameter or global.  gbx_adjoint is not available here.  Zero-fill
 * the struct before setting it: fields added later default to none.
 * ------------------------------------------------------------------------ */
enum { GBX_TERM_SINGLE = 0, GBX_TERM_PAIR = 1, GBX_TERM_PAIR_NO_EXCLUSIONS = 2 };
typedef struct {
  int num_params;
  const char* const* param_names;
  int num_globals;
  const char* const* global_names;
  const double* global_values;
  int num_integrals;
  const char* const* integral_names;
  const int* integral_orders;
  int num_values;
  const char* const* value_names;
  const char* const* value_expressions;
  int num_terms;
  const char* const* term_expressions;
  const int* term_types; /* GBX_TERM_* */
  int num_exclusions;    /* addExclusion (CharmmGBMVForce.h:416) */
  const int* exclusions; /* [num_exclusions][2] particle pairs */
  int num_param_derivs;  /* addEnergyParameterDerivative (CharmmGBMVForce.h:258): globals whose */
  const char* const* param_deriv_names; /* energy derivative gbx_get_custom_param_derivs reports */
  /* addTabulatedFunction (CharmmGBMVForce.h:442) with OpenMM's Continuous1DFunction: a natural
   * cubic spline through function_sizes[k] (>= 2) values at evenly spaced points from
   * function_ranges[2k] to function_ranges[2k+1], zero outside that range; called by name with
   * one argument in any expression.  Values of all functions concatenated. */
  int num_functions;
  const char* const* function_names;
  const int* function_sizes;
  const double* function_values;
  const double* function_ranges;
} gbx_custom;

GBX_API gbx_status gbx_create_custom(const gbx_config* cfg, int num_atoms, const gbx_custom* custom,
                                     gbx_context** out);
/* Per-particle parameters [num_atoms][num_params] (the radius among them). */
GBX_API gbx_status gbx_set_custom_parameters(gbx_context* ctx, const double* params);
GBX_API gbx_status gbx_set_custom_global(gbx_context* ctx, const char* name, double value);
/* dE/dg of the last execute for each global named in param_deriv_names, in
 * that order (synchronises the context's stream). */
GBX_API gbx_status gbx_get_custom_param_derivs(gbx_context* ctx, double* out, int count);
/* Checks an expression set without a device: parses it, checks every
 * variable and compiles the generated code.  On failure `log` (may be NULL)
 * receives the reason. */
GBX_API gbx_status gbx_custom_check(const gbx_custom* custom, char* log, size_t len);

/* Global parameters alpha0, alpha1 (the GBMV force's computed-value globals). */
GBX_API gbx_status gbx_set_global_parameters(gbx_context* ctx, double alpha0, double alpha1);
/* Periodic box edges (nm) for GBX_TABLE_PERIODIC. */
GBX_API gbx_status gbx_set_box(gbx_context* ctx, const double box[3]);

/* Energy and forces on device buffers.  Replaces CalcCharmmGB*ForceKernel::execute
 * (charmmKernels.h:81,121; CharmmCudaKernels.cpp:845-993).  posq: float4[num_atoms]
 * on the device.  force_fixed: fixed-point buffer, ADDED to, components at
 * [0, stride), [stride, 2 stride), [2 stride, 3 stride).  energy: one double on
 * the device, ADDED to.  Either may be NULL when not requested by flags.
 * GBX_EXEC_POSQ_DOUBLE: posq is double4; GBX_EXEC_ENERGY_FLOAT: energy is a
 * float (OpenMM's precision modes).
 *
 * Without GBX_EXEC_CHECK the call neither synchronises nor is silently
 * wrong: every call's last kernel publishes the table's size and status to
 * mapped host memory, which the next calls read without waiting.  Buffers
 * grow ahead of need once the largest table seen reaches 90 % of them; if
 * the atoms nevertheless outgrew the table within one call, that call lacks
 * the volume terms (the oversized table is never indexed) and a later call
 * (the next one once the GPU has finished it) grows the buffers, runs
 * checked and returns GBX_ERR_STALE_RESULT; a non-finite Born radius is
 * reported the same way as GBX_ERR_NONFINITE.  GBX_EXEC_CHECK synchronises
 * and reports the call's own status. */
GBX_API gbx_status gbx_execute(gbx_context* ctx, const void* posq, unsigned long long* force_fixed,
                               int force_stride, double* energy, int flags, void* stream);

/* The caller's atom order (OpenMM reorders atoms for locality): slot k of
 * posq and of the force buffer holds atom atom_index[k] (a permutation of
 * 0..n-1; host array, copied; NULL: identity).  Parameters stay in atom
 * order and the lookup-table lists keep ascending atom order, as the
 * reference CPU classes (CharmmReferenceGBSW.cpp:440-514) -- so a reorder
 * changes no result.  Replaces the parameter re-upload the reference's
 * CUDA kernel does on a reorder.  Call it whenever the order changes. */
GBX_API gbx_status gbx_set_atom_order(gbx_context* ctx, const int* atom_index);

/* Same computation on host arrays (Reference-platform style): positions
 * double[3n]; forces double[3n] ADDED to; *energy set.  Copies inside.  Once
 * the lookup table's buffers are sized the call synchronises once, at the
 * end; a table that outgrew them is detected there and the call runs again
 * checked (the outputs are written once). */
GBX_API gbx_status gbx_execute_host(gbx_context* ctx, const double* positions, double* forces, double* energy,
                                    int flags);

/* Results of the last execute, copied to host: Born radii (nm), integrals
 * I4/I7 [2n], dE/dB [n]. */
GBX_API gbx_status gbx_get_born_radii(gbx_context* ctx, double* born);
GBX_API gbx_status gbx_get_integrals(gbx_context* ctx, double* integrals);
GBX_API gbx_status gbx_get_dEdB(gbx_context* ctx, double* dEdB);

/* Lookup table of the last execute (or built by gbx_build_lookup_table):
 * dims, min corner, steps and the per-cell lists in ascending atom order.
 * Pass NULL arrays to query sizes first. */
GBX_API gbx_status gbx_build_lookup_table(gbx_context* ctx, const void* posq, void* stream);
GBX_API gbx_status gbx_get_lookup_table(gbx_context* ctx, int dims[3], double min[3], double step[3],
                                        int64_t* ncell, int32_t* counts, int64_t* total, int32_t* atoms);

/* Adjoint: dE/dx (as forces), dE/dq [n], dE/dR_in [n], dE/dalpha [2].  The
 * per-point volumes are recomputed, not stored.  No counterpart in the
 * reference, which only returns forces; it carries the same chain rule
 * (CharmmReferenceGBSW.cpp:597-674) to the parameters.  Host arrays. */
GBX_API gbx_status gbx_adjoint_host(gbx_context* ctx, const double* positions, double* energy, double* forces,
                                    double* dEdq, double* dEdR, double* dEdalpha);

/* Device form of gbx_adjoint_host for differentiable callers (a
 * torch.autograd.Function): posq = device float4 [n] (x, y, z, unused) in nm;
 * outputs are device FP64 arrays, any of them may be NULL: energy [1],
 * forces [n][3] (-dE/dx), dEdq [n], dEdR [n], dEdalpha [2].  Runs on `stream`
 * (NULL: the context's own); flags may hold GBX_EXEC_CHECK. */
GBX_API gbx_status gbx_adjoint(gbx_context* ctx, const void* posq, double* energy, double* forces, double* dEdq,
                               double* dEdR, double* dEdalpha, int flags, void* stream);

/* ------------------------------------------------------------------------
 * Batched evaluation: many independent molecules (uneven sizes, any mix of
 * presets) per call.  One context per molecule; positions, forces and
 * energies live in batch-owned device buffers:
 *   posq     float4 [total atoms], molecule m from atom_offset(m) on (nm)
 *   forces   u64 fixed point (2^-32) [3 * total], molecule m's block at
 *            3 * atom_offset(m), layout [3][n_m]
 *   energies double [molecules] (kJ/mol)
 * The first call (or one with GBX_EXEC_CHECK) sizes every buffer; later
 * calls replay one CUDA graph of the whole batch and re-run checked when a
 * device status word reports that a table outgrew its capacity.  No
 * counterpart in the reference (which loops one Context per molecule).
 * ------------------------------------------------------------------------ */
typedef struct gbx_batch gbx_batch;
GBX_API gbx_status gbx_batch_create(const gbx_config* configs, const int* n_atoms, int n_molecules, gbx_batch** out);
GBX_API gbx_status gbx_batch_destroy(gbx_batch* batch);
/* Molecule m's context (for gbx_set_particle_parameters / _global_ / _box)
 * and its first atom in the batch buffers. */
GBX_API gbx_status gbx_batch_molecule(gbx_batch* batch, int m, gbx_context** ctx, long long* atom_offset);
GBX_API gbx_status gbx_batch_buffers(gbx_batch* batch, void** posq, unsigned long long** forces, double** energies,
                                     long long* total_atoms);
/* Device-resident call on `stream` (NULL: the batch's own); returns after
 * the replay's status check (one 4-byte read-back). */
GBX_API gbx_status gbx_batch_execute(gbx_batch* batch, int flags, void* stream);
/* Host arrays: positions / forces [total][3] (nm, kJ/mol/nm), energies [molecules]. */
GBX_API gbx_status gbx_batch_execute_host(gbx_batch* batch, const double* positions, double* forces,
                                          double* energies);
/* Batched adjoint (the differentiable form over many molecules): gbx_adjoint
 * of every molecule on the batch's positions (posq buffer), fanned out over
 * the batch's streams.  Device FP64 outputs laid out by the atom offsets,
 * any may be NULL: energies [molecules], forces [total][3] (-dE/dx),
 * dEdq [total], dEdR [total], dEdalpha [molecules][2].  Unchecked calls
 * re-run checked when a table outgrew its buffers; flags may hold
 * GBX_EXEC_CHECK.  Molecules built on compiled expressions are refused
 * (GBX_ERR_UNSUPPORTED), as by gbx_adjoint. */
GBX_API gbx_status gbx_batch_adjoint(gbx_batch* batch, double* energies, double* forces, double* dEdq, double* dEdR,
                                     double* dEdalpha, int flags, void* stream);
/* Host arrays: positions [total][3] in, the same outputs on the host. */
GBX_API gbx_status gbx_batch_adjoint_host(gbx_batch* batch, const double* positions, double* energies,
                                          double* forces, double* dEdq, double* dEdR, double* dEdalpha);
/* Autotuner: times the captured batch over stream counts {4, 8, 16, 32} and
 * quadrature chunkings (default chunks per atom / {1, 2, 4}) and keeps the
 * fastest.  Outputs may be NULL. */
GBX_API gbx_status gbx_batch_tune(gbx_batch* batch, int* streams, int* chunk_divisor, double* ms_per_call);
GBX_API gbx_status gbx_batch_last_error(gbx_batch* batch, char* buf, size_t len);

/* Work counters of the last execute run with GBX_EXEC_COUNT_WORK: (point,
 * listed atom) evaluations, of which inside a GBSW switching shell, and
 * ordered pairs.  Diagnostics for roofline accounting; no counterpart in the
 * reference. */
GBX_API gbx_status gbx_get_work(gbx_context* ctx, double* volume_evals, double* shell_evals, double* pairs);

/* Chain-rule work of the same run: every listed atom of every quadrature
 * point (the reference chain kernel walks whole lists,
 * platforms/cuda/src/kernels/reduceIntegralForce.cu:45-65), and of those the
 * ones inside a GBSW switching shell (all of them for GBMV).  Diagnostics for
 * roofline accounting; no counterpart in the reference. */
GBX_API gbx_status gbx_get_chain_work(gbx_context* ctx, double* list_evals, double* derivative_evals);

/* Kernels this context has launched so far (all entry points).  No
 * counterpart in the reference. */
GBX_API gbx_status gbx_get_launches(gbx_context* ctx, long long* launches);

/* GBSW forces: the integral pass writes one 16-byte record (q, V, mask of
 * the shaping list entries) per quadrature point that an atom other than its
 * own shapes, so that the chain rule visits only those entries instead of
 * re-walking every point's cell list.  Each warp (atom x quadrature chunk) owns per_warp records.  per_warp < 0: automatic (the default; first half a warp's points,
 * then 1.125x the largest need seen), 0: no records (the chain rule walks the
 * lists), > 0: that fixed size.  A warp whose records do not fit walks its
 * lists instead, with bit-identical results, so the size only affects speed.
 * No counterpart in the reference. */
GBX_API gbx_status gbx_set_chain_records(gbx_context* ctx, int per_warp);

/* Records of the last execute: written (-1 if it kept none), the largest
 * per-warp need, the per-warp size and the warps that did not fit.
 * Synchronises the context's stream. */
GBX_API gbx_status gbx_get_chain_records(gbx_context* ctx, long long* written, int* max_need, int* per_warp,
                                         int* overflowed);

/* Per-stage device times (ms) of the last execute, from CUDA events recorded
 * on the execute stream when timing is enabled.  Stages: 0 position staging,
 * 1 lookup table, 2 integrals, 3 Born radii, 4 pair term, 5 chain prep,
 * 6 chain rule, 7 energy reduction.  Diagnostics; no counterpart in the
 * reference. */
GBX_API gbx_status gbx_set_timing(gbx_context* ctx, int enable);
GBX_API gbx_status gbx_get_stage_times(gbx_context* ctx, double* ms, int max_stages, int* num_stages);

/* Allocation-free GB pair term, for callers that cannot let a library
 * allocate device memory (an engine that owns all device memory through its
 * own pool, or a step loop that must not block or fail in cudaMalloc).  No
 * counterpart in the reference.  It computes the same pair energy (including
 * the 1/2 pref q^2/B self terms), pair forces and dE/dB as gbx_execute's pair
 * stage, from caller-supplied device arrays: posq float4[n] (x, y, z, -),
 * charge float[n], born float[n] (Born radii, nm).  force_fixed (fixed point,
 * stride as in gbx_execute) and *energy are ADDED to; dEdB double[n] is
 * written when not NULL.  cutoff <= 0: all pairs.  Distances are plain
 * differences (no minimum image): non-periodic systems only.
 *
 * Nothing is allocated: the scratch is one static device array of about
 * 1 MiB that every GPU loading the library holds until exit, which limits
 * num_atoms to 65536 (larger sizes return GBX_ERR_EXCEEDS_STATIC_SCRATCH).
 * All calls on a device share that array, so calls whose kernels overlap on
 * the GPU (different streams, host threads) race: serialise them.  The first
 * call on each device looks the array's device address up
 * (cudaGetSymbolAddress); make that first call before any stream capture.
 * The address is remembered per CUDA context, so a call after a device
 * reset looks it up again in the new context. */
GBX_API gbx_status gbx_pair_noalloc(const void* posq, const float* charge, const float* born, int num_atoms,
                                    double prefactor, double cutoff, unsigned long long* force_fixed,
                                    int force_stride, double* energy, double* dEdB, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* GBX_H */
