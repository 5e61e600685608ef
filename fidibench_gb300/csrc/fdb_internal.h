// fdb_internal.h -- shared declarations of libfdb_upwind (not installed).
#pragma once

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>
#include <stdint.h>

#include <string>
#include <utility>
#include <vector>

#include "fdb_upwind.h"

namespace fdb {

// Thread-local error message behind fdb_last_error().
void set_error(const std::string& msg);
int fail(int code, const std::string& msg);
int cuda_fail(cudaError_t e, const char* what);

#define FDB_CUDA_TRY(expr)                               \
  do {                                                   \
    cudaError_t _e = (expr);                             \
    if (_e != cudaSuccess) return ::fdb::cuda_fail(_e, #expr); \
  } while (0)

#define FDB_TRY(expr)            \
  do {                           \
    int _rc = (expr);            \
    if (_rc != FDB_OK) return _rc; \
  } while (0)

// Host-side fault injection (env FDB_FAULT=alloc|launch|timeout|nan): lets the
// failure paths be exercised without faulting a GPU.
bool fault_injected(const char* kind);

// Launch accounting behind fdb_launch_count(): every launch wrapper adds the
// number of kernels it enqueued.
void note_launch(uint64_t n = 1);

// NVTX range for the lifetime of a scope (names the library's phases in
// profiler timelines and lets ncu filter captures by phase, e.g.
// `ncu --nvtx --nvtx-include "fdb.adjoint.transposed/"`; no cost without a tool).
struct NvtxScope {
  explicit NvtxScope(const char* name) { nvtxRangePushA(name); }
  ~NvtxScope() { nvtxRangePop(); }
  NvtxScope(const NvtxScope&) = delete;
  NvtxScope& operator=(const NvtxScope&) = delete;
};

// Timing events of one call: every event the call creates comes from here and
// is destroyed when the pool goes out of scope, on every return path.
struct EventPool {
  std::vector<cudaEvent_t> all;
  EventPool() = default;
  EventPool(const EventPool&) = delete;
  EventPool& operator=(const EventPool&) = delete;
  ~EventPool() {
    for (cudaEvent_t e : all) cudaEventDestroy(e);
  }
  // null when creation fails (the timings then read as 0)
  cudaEvent_t make() {
    cudaEvent_t e = nullptr;
    if (cudaEventCreate(&e) != cudaSuccess) {
      cudaGetLastError();
      return nullptr;
    }
    all.push_back(e);
    return e;
  }
  static void record(cudaEvent_t e, cudaStream_t s) {
    if (e) cudaEventRecord(e, s);
  }
};

// Geometry of one problem, normalised to 3 internal axes (z, y, x) = reference
// axes (ndims-3, ndims-2, ndims-1); missing leading axes have extent 1 and
// zero velocity.  Problems with more than 3 axes use the generic kernels.
struct Geom {
  int ndims = 0;
  uint64_t n[FDB_MAX_DIMS] = {0};
  double v[FDB_MAX_DIMS] = {0};
  double L[FDB_MAX_DIMS] = {0};
  double dx[FDB_MAX_DIMS] = {0};
  int up[FDB_MAX_DIMS] = {0};
  uint64_t dimProd[FDB_MAX_DIMS] = {0};
  uint64_t nsp[FDB_MAX_DIMS] = {0};  // the grid the spacings come from (n, or a slab's global grid)
  uint64_t ntot = 0;
  // 3-D view (valid when ndims <= 3)
  int64_t nz = 1, ny = 1, nx = 1;
  int upz = -1, upy = -1, upx = -1;
  int jz = -1, jy = -1, jx = -1;  // reference axis of each internal axis (-1: padded)
  int coeff_form = FDB_COEFF_CXX;  // how ref_coeff rounds c_j (FDB_COEFF_*)
  // a slab's own planes [own0, own0 + own_n) of axis 0 (own_n = 0: all): the
  // fixed-point scale is measured over them only, so that every slab of a
  // distributed grid can agree on the global one
  uint64_t own0 = 0, own_n = 0;
};

int make_geom(int ndims, const double* v, const double* L, const uint64_t* n, Geom* g);
// As make_geom, with the spacings dx_j = L_j / n_spacing[j] of another grid
// (a slab of a larger grid keeps the global grid's spacings).
int make_geom_spacing(int ndims, const double* v, const double* L, const uint64_t* n,
                      const uint64_t* n_spacing, Geom* g);

// The reference coefficient of axis j: ((dt * v_j) * up_j) / dx_j (upwind.cxx:72),
// or dt * ((v_j * up_j) / dx_j) under FDB_COEFF_PRODUCT (upwindAcc.cxx:45,79).
double ref_coeff(const Geom& g, int j, double dt);

// The geometry of the transposed step: every upwind direction reversed
// (with the coefficients of g, the step on it is A^T).
Geom transposed_geom(const Geom& g);

// Step coefficients in the 3-D view.  c* are the reference coefficients
// (c <= 0); a* = -c* are the Courant numbers; w = ((1 - a_z) - a_y) - a_x.
struct Coeffs3 {
  double cz, cy, cx;
  double az, ay, ax;
  double w;
};
Coeffs3 coeffs3(const Geom& g, double dt);

// ---- kernels (launch wrappers return FDB_OK or an error code) -------------
int launch_step_f64(const Geom& g, const Coeffs3& c, int arith, const double* in,
                    double* out, cudaStream_t s);
int launch_step_generic(const Geom& g, double dt, const double* in, double* out,
                        cudaStream_t s);

// Temporally blocked block-fixed-point kernel: advances `steps` steps (a
// multiple of nothing in particular; the wrapper splits into blocks of
// `depth`).  Returns FDB_ERR_UNSUPPORTED when the geometry or coefficients
// are outside what it serves (the caller then uses the FP64 kernel).
int fixed_supported(const Geom& g, const Coeffs3& c, int depth);
bool fixed_preferred(const Geom& g);
// number of CTA shapes the fixed kernel is compiled for (FDB_TUNE_SHAPE range)
int fx_num_shapes();
// steps per launch the fixed kernel picks for g when none is asked for
int default_depth(const Geom& g);
size_t fixed_scratch_bytes();
// Device error word inside the fixed kernel's scratch (non-zero: non-finite input).
int* fixed_error_word(double* d_scratch);
// Launch-shape knobs of the fixed kernel (0 / -1 = automatic).
struct FixedTuning {
  int depth = 0;   // temporal depth K (steps per launch), 1..4
  int shape = -1;  // 0 = 8x8, 1 = 4x16 (history in registers), 2 = 8x8, 3 = 4x16, 4 = 4x8
                   // (in smem), 5 = 4x8, 6 = 6x8 (in smem, register loads, x-1 from smem)
  int tz = 0;      // output planes per CTA along z
};

int launch_advect_fixed(const Geom& g, const Coeffs3& c, int steps, int depth,
                        double** buf, int* cur, double* d_scratch, size_t scratch_bytes,
                        cudaStream_t s);
// The scale pre-pass: slot ring reset, slot 0 = max|f| (FP64 bits) of the
// geometry's own planes of f.
int launch_scale_prepass(const Geom& g, const double* f, double* d_scratch, cudaStream_t s);
// As above; *scale_slot (in/out, may be null) names the scratch slot that
// holds max|f| of the current field (-1: unknown, a pre-pass measures it).
int launch_advect_fixed_ex(const Geom& g, const Coeffs3& c, int steps, const FixedTuning& tune,
                           double** buf, int* cur, double* d_scratch, size_t scratch_bytes,
                           int* scale_slot, cudaStream_t s);

// One launch of a block chain (fdb_upwind_advect_block): k <= guard_K steps
// at ring position i, FP64 in/out as asked, int64 otherwise; flips *cur.
// The launches of a chain are those launch_advect_fixed_ex makes for the
// same steps, so the field is the same bit for bit.
int launch_fixed_block(const Geom& g, const Coeffs3& c, int k, const FixedTuning& tune,
                       int guard_K, double** buf, int* cur, bool in_f64, bool out_f64,
                       double* d_scratch, int i, cudaStream_t s);
// The 64-bit word of ring slot i that the launch at position i reads to set
// its scale (FP64 bits of max|f| after a pre-pass, else an OR of |F|).
uint64_t* scale_word(double* d_scratch, int i);

// Deterministic reductions.  `part` holds at least reduce_partials(n) doubles.
uint32_t reduce_partials(uint64_t n);
int launch_sum(const double* f, uint64_t n, double* part, double* d_out, cudaStream_t s);
int launch_std(const double* f, uint64_t n, double* part, double* d_tmp2, double* d_out,
               cudaStream_t s);

int launch_fill_corner(double* f, uint64_t n, cudaStream_t s);
int launch_sphere_noise(const Geom& g, const double* center, double radius, double amp,
                        uint64_t seed, double* f, cudaStream_t s);

// Adjoint step (3-D view): lam_out = A^T lam_in; dpart[3*G] accumulates the
// per-block velocity-coefficient partials -<lam_in, S_j f - f>.
uint32_t adjoint_blocks();
int launch_adjoint_step(const Geom& g, const Coeffs3& c, const double* f,
                        const double* lam_in, double* lam_out, double* dpart,
                        cudaStream_t s);
int launch_adjoint_finish(const double* dpart, double* d_out3, cudaStream_t s);

// Device memory that grows on demand and is freed by its owner.
struct DeviceScratch {
  void* ptr = nullptr;
  size_t bytes = 0;
  int reserve(size_t need);
  void release();
};

// The velocity contraction of the closed-form adjoint (adjoint.cu): for each
// instance i (geometry geoms[i], cells at offsets[i] of f and lam),
// d_out[3 i + k] = sum_c lam[c] (f[c + up_k e_k] - f[c]) over the internal
// axes k = z, y, x.  Deterministic; two launches.
int launch_vel_contract(int count, const Geom* geoms, const int64_t* offsets, const double* f,
                        const double* lam, double* d_out, DeviceScratch& scratch,
                        cudaStream_t s);

// Fixed-point adjoint of a whole advect (adjoint_fixed.cu).  The forward
// checkpoints ckpt[0..nseg) (FP64, every K steps) must already exist.
struct AdjointFixedIO {
  const Geom* g;
  const Coeffs3* c;
  int S;      // steps
  int K;      // checkpoint interval
  int nseg;   // ceil(S / K)
  double* const* ckpt;
  // recomputed segment: its states march through two int64 buffers; the
  // contraction reads each state in 2^29 units, kept as int32 (K arrays of
  // ntot)
  int64_t* chain[2];
  int32_t* const* state_hi;
  int64_t* lam[2];         // adjoint ping-pong (int64)
  const double* lam_T;     // device, FP64
  double* grad_f0;         // device, FP64
  double* dpart;           // 3 doubles per adjoint CTA
  int dpart_cap;           // CTAs the buffer holds
  double* dda3;            // device [3]: dL/da for the internal (z, y, x) axes
  void* scratch;           // adjoint_fixed_scratch_bytes(K) bytes
  // nullable: event pairs bracketing each recompute / transposed-step block,
  // for the caller to read after it synchronises; the events come from (and
  // are owned by) `events`, which must be set when either list is
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>>* recompute_ev = nullptr;
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>>* adjoint_ev = nullptr;
  EventPool* events = nullptr;
};
size_t adjoint_fixed_scratch_bytes(int seg_len);
// ntot-double buffers the fixed-point adjoint needs for a segment of K steps:
// the two int64 chain buffers and K int32 arrays (two per buffer)
inline int adjoint_fixed_segment_buffers(int K) { return 2 + (K + 1) / 2; }
int adjoint_fixed_ctas(const Geom& g, const Coeffs3& c);
int adjoint_fixed_run(const AdjointFixedIO& io, cudaStream_t st);

// The same for many instances stepping together (adjoint_fixed.cu): every
// launch covers all instances; buffers hold the instances at `offsets`.
struct BatchAdjointIO {
  int count;
  const Geom* geoms;        // geometry of each instance as stored (host)
  const Coeffs3* coeffs;    // host
  const int64_t* offsets;   // host, cells
  const int64_t* d_offs;    // device copies of offsets and sizes
  const uint64_t* d_sizes;
  int S, K, nseg;
  double* const* ckpt;       // nseg FP64 buffers: the instances at step s K
  int64_t* chain[2];         // recompute chain (int64)
  int32_t* const* state_hi;  // K int32 buffers: the segment's states in 2^29 units
  int64_t* lam[2];           // adjoint ping-pong (int64)
  const double* lam_T;       // device, FP64
  double* grad_f0;           // device, FP64
  double* dda3;              // device [3 * count]: dL/da per stored axis (z, y, x)
  int* err;                  // device error word (bit 0: non-finite input)
  void* scratch;             // batch_adjoint_scratch_bytes(count, K, grid) bytes
};
// CTAs of one batched launch
int batch_adjoint_grid(int count, const Geom* geoms);
size_t batch_adjoint_scratch_bytes(int count, int K, int grid);
int batch_adjoint_run(const BatchAdjointIO& io, cudaStream_t st);

}  // namespace fdb
