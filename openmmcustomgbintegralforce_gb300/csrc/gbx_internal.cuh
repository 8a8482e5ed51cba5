// Internal types shared by the gbx CUDA translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "gbx.h"
#include "gbx_custom.h"

namespace gbx {

constexpr int kWarp = 32;
constexpr double kFixedScale = 4294967296.0;  // 2^32, OpenMM's force fixed-point scale
constexpr int kMaxSortSegment = 2048;         // longest cell list the sort handles
constexpr int kMaxSortCells = 1 << 17;        // cells of the cutoff pair term's spatial order

// Device status bits (context->d_status).
enum : unsigned {
  kStatusTableCells = 1u,     // grid has more cells than allocated
  kStatusTableEntries = 2u,   // more list entries than allocated
  kStatusSegmentTooLong = 4u, // a cell list exceeded kMaxSortSegment
  kStatusNonFinite = 8u,      // NaN/Inf Born radius
  kStatusTimeout = 16u,       // bounded device wait expired
};

// Status of the device calls, published by the last kernel of every call
// into mapped host memory (monotone counters; seq written last).
struct StatusRecord {
  unsigned long long seq;          // calls published
  unsigned long long overflows;    // calls whose lookup table outgrew its buffers
  unsigned long long nonfinite;    // calls with a non-finite Born radius
  unsigned long long max_cells;    // largest table geometry seen (cells)
  unsigned long long max_entries;  // largest list-entry total seen
};

// Lookup-table geometry, computed on the device each step.
struct TableGeom {
  double min[3];
  double max[3];
  double step[3];
  double box[3];
  double inv_step[3];  // 1 / step and 1 / box (0 without a box), for the FP32
  double inv_box[3];   // queries: formed once here, not per lane in FP64
  double pad;       // standalone uniform pad
  double L;         // periodic: max(step)
  int dims[3];
  int mode;
  long long ncell;
  long long total;  // list entries before capping
};

// Exact GBSW table, per cell: the list's first (sorted) entry and the cell's
// (count or -1 if buried, start) record, read together by one 32-byte load.
struct __align__(32) TightCell {
  float4 first;
  int2 cs;
  int2 pad;
};

// Two consecutive 16-byte entries at a 32-byte aligned address in one
// 256-bit non-coherent load (sm_100 and later).
struct __align__(32) Float4x2 {
  float4 a, b;
};
__device__ __forceinline__ Float4x2 ldg_pair(const void* p) {
  Float4x2 r;
  asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
      : "=f"(r.a.x), "=f"(r.a.y), "=f"(r.a.z), "=f"(r.a.w), "=f"(r.b.x), "=f"(r.b.y), "=f"(r.b.z), "=f"(r.b.w)
      : "l"(p));
  return r;
}

// Per-model constants used inside the kernels (FP32 hot path + FP64 exact paths).
struct ModelConst {
  int model;
  int table_mode;
  int cap;
  int skip_empty;
  int nq;
  int nshell;                // points per radial shell (index = radial * nshell + angular)
  int cutoff_chain_quirk;
  float sw, c1, c3;          // GBSW: u = 1/2 + c1 dr - c3 dr^3, c1 = 3/(4w), c3 = 1/(4w^3)
  float gamma0_lnlambda;     // GBMV-I gamma_j = gamma0 ln(lambda) / R^4
  float beta, lambda, s0;    // GBMV
  float p1, p2;              // GBMV-II
  float cutoff2;             // pair cutoff squared (<= 0: none)
  float pref;                // pair prefactor
  double h, buffer, cutoff;
};

// One evaluation context (one force instance).
struct Context {
  gbx_config cfg{};
  int n = 0;
  int device = 0;
  int sms = 0;  // multiprocessors of `device` (grid sizing), read once at creation
  std::string last_error;

  // quadrature (host, FP64) and device copies
  std::vector<double> q_off, q_rad, q_w;  // [Q*3], [Q], [Q]
  double S4 = 0, S7 = 0;                  // sum_q w/r^2, sum_q w/r^5 (FP64)
  double C4 = 0, C7 = 0;                  // 1/r0 - S4, 1/(4 r0^4) - S7
  float4* d_qv = nullptr;                 // (vx, vy, vz, r) FP32
  float2* d_qw = nullptr;                 // (w/r^2, w/r^5) FP32
  double* d_qoff = nullptr;               // FP64 offsets for the exact cell query

  // particle data
  std::vector<double> charge, radius;
  double* d_radius = nullptr;  // FP64 radii (table geometry)
  float* d_charge = nullptr;
  float2* d_par = nullptr;     // secondary model parameters per atom
  float* d_wpar = nullptr;     // main model parameter (staged into pos.w)
  float alpha0 = 0, alpha1 = 0;

  // table
  TableGeom* d_geom = nullptr;
  long long cell_cap = 0, entry_cap = 0;
  int* d_cell_count = nullptr;   // uncapped count -> final (capped) count
  int* d_cell_start = nullptr;   // [cell_cap+1]
  int* d_cell_cursor = nullptr;
  int2* d_cell2 = nullptr;       // [cell_cap] (capped count, start) for the volume kernels
  int* d_entries = nullptr;      // [entry_cap] atom indices, ascending per cell
  float4* d_entry4 = nullptr;    // [entry_cap] inline copies (x, y, z, main parameter)
  float2* d_entry_par = nullptr; // [entry_cap] inline secondary parameters
  int* d_block_sums = nullptr;
  double* d_reduce = nullptr;    // geometry reduction scratch
  bool table_valid = false;

  // exact GBSW table (GBX_TABLE_POLICY_AUTO on a standalone table):
  // count[c] = -1 marks a cell every point of which is buried
  bool use_tight = false;
  bool tight_eligible = false;   // GBSW on a standalone table with the AUTO policy
  double tight_h = 0.1;
  TableGeom* d_tgeom = nullptr;
  TableGeom* d_wgeom = nullptr;  // periodic: the reference's standalone grid (its edges decide the move)
  long long tcell_cap = 0, tentry_cap = 0;
  int* d_tcount = nullptr;
  int* d_tstart = nullptr;
  int* d_tcursor = nullptr;
  int* d_tburied = nullptr;
  int2* d_tcell = nullptr;       // (count or -1 if buried, start)
  TightCell* d_tfirst = nullptr; // per cell: first entry and (count, start)
  int* d_tblock_sums = nullptr;
  float4* d_tentry = nullptr;    // (x, y, z, R') per list entry; lists start at even entries
  int* d_tindex = nullptr;       // atom index per list entry
  bool tight_valid = false;

  // per-step state
  float4* d_pos = nullptr;       // internal positions (x, y, z, 0)
  int n_chunks = 0;              // quadrature chunks per atom
  float* d_J = nullptr;          // [2][n_chunks][n] FP32 partial integrals
  double* d_born = nullptr;      // [n]
  float* d_bornf = nullptr;      // [n] (B, 1/B interleaved as float2)
  double* d_dBdJ = nullptr;      // [6n]: dB/dJ [2n], dB/dalpha [2n], adjoint alpha terms [2n]
  double* d_integrals = nullptr; // [2n]  I4, I7
  unsigned long long* d_dEdB_fx = nullptr;  // [n] fixed point
  float2* d_dEdJ = nullptr;      // [n]
  double* d_energy_part = nullptr;  // [energy_parts] per-CTA energy partials
  int energy_parts = 0;
  unsigned long long* d_energy_fx = nullptr;  // pair energy, fixed point (2^-32)
  float4* d_tile_box = nullptr;               // cutoff: bounding box of each 32-atom tile
  int* d_perm = nullptr;                      // cutoff: atoms in spatial order [n]
  int* d_perm_tmp = nullptr;                  // cutoff: the same before the per-cell sort [n]
  int* d_cell_of = nullptr;                   // cutoff: spatial cell of each atom [n]
  int* d_scount = nullptr;                    // cutoff: atoms per spatial cell [kMaxSortCells]
  int* d_sstart = nullptr;
  int* d_scursor = nullptr;
  int4* d_sgeom = nullptr;                    // cutoff: spatial grid geometry
  float* d_pstate = nullptr;                  // GBMV: per-point sums kept for the chain rule
  // GBMV points binned by lookup-table cell (k_gbmv.cu)
  int* d_pcell = nullptr;                     // [n Q] the point's cell or -1
  int* d_prank = nullptr;                     // [n Q] slot within the cell
  int* d_porder = nullptr;                    // [n Q] point id per slot
  float* d_sval = nullptr;                    // [n Q] solvent fraction by point id
  int* d_pcount = nullptr;                    // [cell_cap] points per cell
  int* d_pstart = nullptr;                    // [cell_cap + 1] first slot per cell
  int* d_pblock_sums = nullptr;               // scan scratch
  TableGeom* d_pgeom = nullptr;               // the point scan's cell count and total
  bool gbmv_cells = false;                    // this call's GBMV passes run by cell
  CustomPlan* custom = nullptr;               // expressions outside the canonical set (gbx_custom.cu)
  unsigned long long* d_force_fx = nullptr;  // internal force buffer [3n] (host path)
  double* d_energy = nullptr;     // internal energy (host path)
  unsigned long long* d_dEdR_fx = nullptr;  // adjoint [n]
  unsigned long long* d_dEdq_fx = nullptr;  // adjoint [n]
  double* d_alpha_grad = nullptr; // adjoint [2]
  unsigned* d_status = nullptr;
  unsigned long long* d_work = nullptr;  // [4] evaluation counters

  // GBSW chain-rule records (q, V, shaping-entry mask) of the points an atom
  // other than i shapes, written by the integral pass: warp w (atom,
  // quadrature chunk) owns records [w R, (w + 1) R)
  bool records = false;          // this call writes and reads records
  bool srec_auto = true;         // size R from the largest need seen
  int4* d_srec = nullptr;
  int* d_srec_st = nullptr;      // the recorded point's list start, beside each record
  int srec_R = 0;                // records per warp (0: no buffer)
  long long srec_warps = 0;      // warps the buffer was sized for
  int* d_rcount = nullptr;       // [warps] records written, or -1 - needed
  unsigned* d_rmax = nullptr;    // largest per-warp need of the call
  unsigned* d_next_item = nullptr;  // the GBSW integral pass's (atom, chunk) work counter
  int integral_grid = 0;            // its persistent grid: resident blocks on all SMs
  unsigned* h_rmax = nullptr;    // pinned copy of the last d_rmax
  unsigned* h_status = nullptr;  // pinned: status word of the last host-path call
  double* h_energy = nullptr;    // pinned: energy of the last host-path call
  cudaEvent_t srec_ev = nullptr;
  bool srec_pending = false;     // srec_ev recorded and not yet read
  bool have_result = false;

  long long launches = 0;  // kernels this context has launched

  // CUDA graph of the unchecked device call, replayed while its arguments
  // (buffers, flags, stream) stay the same; dropped by every setter and
  // every reallocation
  cudaGraphExec_t graph = nullptr;
  long long graph_kernels = 0;  // kernels one replay launches
  cudaGraphExec_t host_graph = nullptr;  // the host-buffer call: upload, evaluation, readback
  long long host_graph_kernels = 0;
  int host_graph_forces = -1;            // whether the captured call reads forces back
  unsigned long long epoch = 0; // bumped whenever captured arguments may change
                                // (setters, reallocation): graphs that hold this
                                // context's launches (its own, a batch's) are stale
  struct GraphKey {
    const void* posq = nullptr;
    const void* force = nullptr;
    int stride = 0;
    const void* energy = nullptr;
    int flags = 0;
    cudaStream_t stream = nullptr;
    bool operator==(const GraphKey& o) const {
      return posq == o.posq && force == o.force && stride == o.stride && energy == o.energy && flags == o.flags &&
             stream == o.stream;
    }
  } graph_key;

  // optional per-stage timing (CUDA events on the execute stream)
  bool timing = false;
  static constexpr int kStages = 9;
  cudaEvent_t ev[kStages + 1] = {};

  // caller-facing layout of the device call
  int* d_slot_of = nullptr;       // internal atom i -> the caller's slot (gbx_set_atom_order)
  bool in_permuted = false;       // this call reads and writes through d_slot_of
  bool in_double = false;         // this call's positions are double4

  // status of unchecked device calls, read without synchronising
  unsigned long long* d_pub = nullptr;  // [5] device-side counters of StatusRecord
  StatusRecord* h_pub = nullptr;        // mapped pinned record
  StatusRecord* h_pub_dev = nullptr;    // its device address
  unsigned long long pub_seen_overflows = 0, pub_seen_nonfinite = 0;

  // host staging
  float4* h_pos = nullptr;                 // pinned
  unsigned long long* h_force_fx = nullptr; // pinned
  cudaStream_t own_stream = nullptr;  // created and destroyed by the context
  cudaStream_t stream = nullptr;      // stream of the current call (the caller's or own_stream)
};

// --------------------------------------------------------------------------
// Device helpers
// --------------------------------------------------------------------------

// round(v * 2^32) as a 64-bit integer.  Scaling by a power of two is exact
// in FP32, so converting the float directly gives the same integer as the
// FP64 route without touching the (slow) FP64 pipe.
__device__ __forceinline__ long long float_to_fixed(float v) { return __float2ll_rn(v * 4294967296.0f); }

// Fixed point from two 32-bit conversions (|v| < 2^31): floor(v) 2^32 +
// round((v - floor(v)) 2^32), the fraction formed in FP32.  For v >= 0 and
// v <= -1/2 the fraction is exact and the result is round(v 2^32), the
// integer float_to_fixed gives; for -1/2 < v < 0 the fraction 1 + v is first
// rounded to FP32 (a multiple of 2^-24), so the result can differ from
// round(v 2^32) by up to 2^7 units: an absolute error of at most 2^-25
// (3e-8 in force units) per contribution.  Deterministic; cheaper where
// conversions dominate (the chain rule's force pushes: an exact form on |v|
// measured 13 % slower in the GBMV chain).
__device__ __forceinline__ long long float_to_fixed_split(float v) {
  const float hf = floorf(v);
  const unsigned lo = __float2uint_rn((v - hf) * 4294967296.0f);
  return (long long)(((unsigned long long)(long long)__float2int_rz(hf) << 32) + lo);
}

__device__ __forceinline__ void red_add_fixed(unsigned long long* addr, float v) {
  atomicAdd(addr, (unsigned long long)float_to_fixed(v));
}

__device__ __forceinline__ void red_add_fixed_d(unsigned long long* addr, double v) {
  long long q = __double2ll_rn(v * kFixedScale);
  atomicAdd(addr, (unsigned long long)q);
}

__host__ __device__ __forceinline__ double fixed_to_double(unsigned long long v) {
  return (double)(long long)v / kFixedScale;
}

// --------------------------------------------------------------------------
// Launchers (implemented in the k_*.cu files); all enqueue on ctx->stream.
// --------------------------------------------------------------------------

// Whole evaluation on ctx->stream (gbx_api.cu); used by the batch.
gbx_status pipeline(Context* ctx, const float4* posq, unsigned long long* force, int stride, double* energy, bool check,
                    bool adjoint, bool count_work, bool forces);
gbx_status set_chunks(Context* ctx, int chunks);
gbx_status fix_chain_records(Context* ctx);
// Whether the exact GBSW table serves this context's configuration and
// parameters (a periodic one needs the standalone grid's reach below half
// the shortest box edge); switching drops graphs and tables.
void choose_table(Context* ctx);

gbx_status launch_stage_positions(Context* ctx, const void* posq);
gbx_status launch_finish_outputs(Context* ctx, unsigned long long* force, int stride, float* energy_float);
gbx_status launch_publish_status(Context* ctx);
gbx_status launch_table_build(Context* ctx, const float4* pos);
size_t table_geom_scratch_doubles(int n);
gbx_status launch_tight_build(Context* ctx, const float4* pos);
// The standalone (reference) table's grid geometry alone, into out.
void launch_standalone_geom(Context* ctx, const float4* pos, TableGeom* out);
// GBMV on a table the cell passes serve: bins the quadrature points by
// cell (the cell passes' data layout); nothing otherwise.
gbx_status launch_binning(Context* ctx, const float4* pos, bool count_work);
gbx_status launch_integrals(Context* ctx, const float4* pos, bool count_work);
gbx_status launch_born(Context* ctx);
gbx_status launch_pair(Context* ctx, const float4* pos, unsigned long long* force, int stride, bool adjoint);
int pair_energy_parts(int n, int segments);
int pair_segments(int n, int sms);
ModelConst make_model_const(const Context* ctx);
gbx_status launch_chain_prep(Context* ctx, bool adjoint);
gbx_status launch_chain(Context* ctx, const float4* pos, unsigned long long* force, int stride, bool adjoint);
bool gbmv_cells_apply(const Context* ctx);
gbx_status launch_gbmv_cells_bin(Context* ctx, const float4* pos, const ModelConst& m);
gbx_status launch_gbmv_cells_integral(Context* ctx, const float4* pos, const ModelConst& m);
gbx_status launch_gbmv_cells_chain(Context* ctx, const float4* pos, const ModelConst& m, unsigned long long* force,
                                   int stride, bool adjoint);
gbx_status launch_energy_reduce(Context* ctx, double* energy, bool adjoint);
gbx_status launch_adjoint_out(Context* ctx, double* energy, double* forces, double* dEdq, double* dEdR,
                              double* dEdalpha);

}  // namespace gbx
