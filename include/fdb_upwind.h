/*
 * fdb_upwind.h -- C-ABI of the GB300-native upwind advection library
 * (libfdb_upwind.so).  Plain C types only: pointers, sizes and status codes.
 *
 * The reference has no FFI of its own: its interface is the class template
 * Upwind<NDIMS> defined inside the driver translation unit
 * upwind/cxx/upwind.cxx:19-135.  Each entry point below names the member it
 * replaces.  include/fidibench_gb/Upwind.h rebuilds that class on top of
 * these calls with the reference's exact signatures, and
 * fidibench_gb300/upwind.py mirrors the Python class of
 * upwind/python/upwind.py:8-86.
 *
 * Conventions
 *  - Every call returns FDB_OK (0) or a positive FDB_ERR_* code;
 *    fdb_last_error() returns a thread-local message for the last failure.
 *  - Fields are FP64, row-major with the LAST index varying fastest
 *    (upwind.cxx:39-44).  Axis j uses the upwind neighbour i_j + up_j with
 *    up_j = -1 for v_j >= 0 and +1 for v_j < 0 (upwind.cxx:34-35), periodic.
 *  - A handle owns its device buffers and one CUDA stream.  Handles are not
 *    thread-safe; distinct handles are independent.
 *  - `is_device` = 1 means the pointer is device memory of the handle's GPU
 *    (e.g. a torch CUDA tensor's data_ptr()); 0 means host memory.
 *  - Calls that return data to the host synchronise the handle's stream.
 */
#ifndef FDB_UPWIND_H
#define FDB_UPWIND_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FDB_OK 0
#define FDB_ERR_INVALID 1      /* bad argument (sizes, dims, null pointers)    */
#define FDB_ERR_CUDA 2         /* a CUDA runtime call or kernel launch failed  */
#define FDB_ERR_ALLOC 3        /* device or pinned allocation failed           */
#define FDB_ERR_UNSUPPORTED 4  /* valid request that this library does not serve */
#define FDB_ERR_TIMEOUT 5      /* a bounded device-side wait gave up           */
#define FDB_ERR_NONFINITE 6    /* finiteness check found a NaN/Inf             */
#define FDB_ERR_INJECTED 7     /* host-side fault injection (FDB_FAULT)        */

#define FDB_MAX_DIMS 8

/* Arithmetic of the step kernel (fdb_upwind_set_arith).
 *  FDB_ARITH_EXACT : the reference's operation order with every FP64
 *                    operation separately rounded (upwind.cxx:72,80): the
 *                    field is bit-identical to the reference built without
 *                    FMA contraction.
 *  FDB_ARITH_FMA   : FP64 in the minimal form w*f + sum_j a_j*f_up_j
 *                    (1 DMUL + 3 DFMA per cell-update).
 *  FDB_ARITH_FIXED : temporally blocked kernel that carries the field in
 *                    64-bit block-fixed-point between one FP64 load and one
 *                    FP64 store per block of steps (integer pipes instead of
 *                    the FP64 pipe).
 *  FDB_ARITH_AUTO  : FIXED where the geometry allows it, else FMA (default). */
#define FDB_ARITH_AUTO 0
#define FDB_ARITH_EXACT 1
#define FDB_ARITH_FMA 2
#define FDB_ARITH_FIXED 3

typedef struct fdb_upwind fdb_upwind;

/* Replaces Upwind(velocity, lengths, numCells)  -- upwind/cxx/upwind.cxx:23-49.
 * Allocates the field on the current CUDA device and sets f = 0, f[0] = 1
 * like the reference constructor (:45-48).  ndims in [1, FDB_MAX_DIMS]. */
int fdb_upwind_create(int ndims, const double* velocity, const double* lengths,
                      const uint64_t* num_cells, fdb_upwind** out);

/* Replaces ~Upwind (implicit; std::vector members freed). */
int fdb_upwind_destroy(fdb_upwind* h);

/* setInitialCondition: overwrite f with ntot values (upwind.cxx:45-48 is the
 * reference's hard-coded initial condition; this replaces it). */
int fdb_upwind_set_field(fdb_upwind* h, const double* src, int is_device);

/* Copy f out (the reference exposes f only through print()/saveVTK(),
 * upwind.cxx:105-109 and saveVTK.h:1-60). */
int fdb_upwind_get_field(fdb_upwind* h, double* dst, int is_device);

/* Device address of the current field (valid until the next advect/set). */
int fdb_upwind_field_ptr(fdb_upwind* h, double** out);

/* Replaces advect(int numTimeSteps, double deltaTime) -- upwind.cxx:51-86.
 * Enqueued on the handle's stream; does not synchronise. */
int fdb_upwind_advect(fdb_upwind* h, int num_steps, double dt);

/* Replaces checksum() -- upwind.cxx:91-93 (sum of f, no cell volume).
 * Deterministic fixed-order tree sum on the device; synchronises. */
int fdb_upwind_checksum(fdb_upwind* h, double* out);

/* The driver's cycle (upwind/cxx/upwind.cxx:194-199: construct with the
 * initial field, advect(numTimeSteps, dt), print checksum()) over `count`
 * independent initial fields held in HOST memory: field k is read from in[k]
 * (ntot doubles), advected with the same kernels, launch blocking and
 * arithmetic as fdb_upwind_advect, written back to out[k], and its checksum (as
 * fdb_upwind_checksum) stored in checksums[k] (checksums may be NULL).
 * The upload of field k+1 and the download of field k-1 run on two copy
 * streams while field k advects, so with pinned host buffers (cudaHostAlloc /
 * cudaHostRegister) the host link is hidden behind the kernels; pageable
 * buffers give the same results without the overlap.  out[k] may be in[k]
 * and several in[k] (or several out[k]: the last field written wins) may
 * share a buffer, but out[k] must not overlap any other in[j].  Needs one
 * more field-sized device buffer (allocated on first use, freed with the
 * handle).  On return the handle's field is the last result; synchronises.
 * FDB_ERR_NONFINITE when any field held NaN/Inf on the fixed-point path. */
int fdb_upwind_advect_host_stream(fdb_upwind* h, int count, const double* const* in,
                                  double* const* out, int num_steps, double dt,
                                  double* checksums);

/* ---------------------------------------------------------------------------
 * Slabs of a distributed grid.  The reference distributes its upwind run with
 * the MPI Filter (upwind/cxx/upwindMpi.cxx:30-165): each rank owns a
 * sub-domain of CubeDecomp (cxx/CubeDecomp.cpp, Filter.cpp:26-56), fetches the
 * neighbour's halo window with MPI_Get (Filter.cpp:114-129) before each
 * stencil term (:212-221) and reduces the checksum with MPI_Reduce (:465-485).
 * Here a rank owns a slab of consecutive planes of axis 0 (the slowest axis,
 * so every plane range is one contiguous block), and the halo is the K
 * planes on the upwind side, exchanged once every K steps
 * (fidibench_gb300/distributed.py).
 *
 * fdb_upwind_create_slab: a handle over slab_planes consecutive planes of
 * axis 0 of the global grid num_cells_global (other axes whole).  The step
 * uses the global grid's spacings dx_j = L_j / num_cells_global[j], so its
 * coefficients are the global problem's bit for bit.  Axis 0 of the slab is
 * treated as periodic: after k steps the k planes nearest the slab's upwind
 * end are stale (they read the far end), every other plane is exact.  The
 * constructor's field is f = 0, f[0] = 1, as for fdb_upwind_create. */
int fdb_upwind_create_slab(int ndims, const double* velocity, const double* lengths,
                           const uint64_t* num_cells_global, uint64_t slab_planes,
                           fdb_upwind** out);

/* Copy planes [first, first + count) of axis 0 of the field out of / into
 * dst / src.  With is_device = 1 the copy is enqueued on the handle's stream
 * and not synchronised (order other streams' use of the buffer with events or
 * by sharing the stream); with host memory the call synchronises.  Works on
 * any handle; for a slab these are its halo and boundary planes. */
int fdb_upwind_get_planes(fdb_upwind* h, uint64_t first, uint64_t count, double* dst,
                          int is_device);
int fdb_upwind_set_planes(fdb_upwind* h, uint64_t first, uint64_t count, const double* src,
                          int is_device);

/* The planes [first, first + count) of axis 0 that this handle owns (a slab's
 * planes without its halo; default: all).  The fixed-point arithmetic measures
 * its scale over them only, so that the slabs of a distributed grid can agree
 * on the scale of the whole grid (fdb_upwind_get/set_scale_word).  The
 * restriction applies when axis 0 is the handle's third-from-last axis (3-D
 * grids); other grids measure every plane. */
int fdb_upwind_set_own_planes(fdb_upwind* h, uint64_t first, uint64_t count);

/* Block-wise advance for a caller that exchanges halo planes between blocks
 * of steps (the distributed form: upwindMpi.cxx advances one step between
 * two halo fetches, Filter.cpp:212-221; here a block is up to the halo depth
 * of steps).  fdb_upwind_block_begin(h, dt, &fixed) opens a chain with the
 * arithmetic advect(dt) would use (fixed = 1 for the block-fixed-point one);
 * each fdb_upwind_advect_block(h, steps, dt, last) then advances `steps`
 * steps, `last` = 1 closing the chain.  Under the fixed-point arithmetic the
 * field stays int64 between blocks (FP64 before the first and after the
 * last), each block is one launch of at most the handle's temporal depth of
 * steps, and a chain of blocks of that depth (the last one shorter) gives
 * the field advect(total steps) gives, bit for bit.  Between blocks a caller
 * may move planes with fdb_upwind_get/set_planes (raw 8-byte copies) and must
 * make every slab's scale word equal to the maximum over the slabs
 * (fdb_upwind_get/set_scale_word, device pointers, stream-ordered): then the
 * slabs of a grid advance with one scale, exactly as the whole grid would.
 * While a chain is open the calls that read or write the field as FP64
 * return FDB_ERR_INVALID.  No reference counterpart. */
int fdb_upwind_block_begin(fdb_upwind* h, double dt, int* fixed);
int fdb_upwind_advect_block(fdb_upwind* h, int steps, double dt, int last);
int fdb_upwind_get_scale_word(fdb_upwind* h, uint64_t* dst, int is_device);
int fdb_upwind_set_scale_word(fdb_upwind* h, const uint64_t* src, int is_device);

/* checksum() of planes [first, first + count) of axis 0 only (a slab's own
 * planes, without its halo): the local sum of Filter::computeCheckSum
 * (Filter.cpp:465-482); the caller reduces over ranks.  Synchronises. */
int fdb_upwind_checksum_planes(fdb_upwind* h, uint64_t first, uint64_t count, double* out);

/* Replaces std() -- upwind.cxx:95-103 (population standard deviation). */
int fdb_upwind_std(fdb_upwind* h, double* out);

/* Replace the velocity (ndims values) of an existing problem, re-deriving the
 * upwind directions as the constructor does (upwind.cxx:34-35); the field is
 * kept.  Lets optimisation loops reuse one handle. */
int fdb_upwind_set_velocity(fdb_upwind* h, const double* velocity);

/* How the per-axis coefficient c_j of the update f -= c_j (f_up - f) is
 * rounded from dt, v_j, up_j and dx_j.  The reference's variants differ:
 *  FDB_COEFF_CXX     : c_j = ((dt * v_j) * up_j) / dx_j, evaluated per step
 *                      (upwind/cxx/upwind.cxx:72; the default).
 *  FDB_COEFF_PRODUCT : c_j = dt * ((v_j * up_j) / dx_j), with the bracket
 *                      precomputed in the constructor (upwindAcc.cxx:45,79,
 *                      upwindAcc2.cxx:48,85, upwindOMP5.cxx:46,86 and the
 *                      Python class, upwind/python/upwind.py:32,64).
 * Under FDB_ARITH_EXACT each form is bit-identical to the variant that uses
 * it; the two differ by rounding only.  Applies to this handle's advect,
 * adjoint and transposed runs. */
#define FDB_COEFF_CXX 0
#define FDB_COEFF_PRODUCT 1
int fdb_upwind_set_coeff_form(fdb_upwind* h, int form);

/* Stream to enqueue on (a cudaStream_t; NULL restores the handle's own). */
int fdb_upwind_set_stream(fdb_upwind* h, void* cuda_stream);

/* Select the step arithmetic (FDB_ARITH_*) and the temporal block depth of
 * the FIXED kernel (0 = autotuned/default). */
int fdb_upwind_set_arith(fdb_upwind* h, int arith, int temporal_depth);

/* Launch-shape tuning of the FIXED kernel (the autotuner's knobs).
 *  FDB_TUNE_TILE_Z : single field: most output planes one CTA takes along
 *                    the slowest axis (0 = auto: a quarter of the planes per
 *                    resident CTA, at least 32; the last z-slabs shrink so
 *                    that the last wave is short); batches: output planes
 *                    per work item (0 = auto).
 *  FDB_TUNE_SHAPE  : rows per thread x warps per CTA and where the plane
 *                    history lives: 0 = 8x8 registers, 1 = 4x16 registers,
 *                    2 = 8x8 shared memory, 3 = 4x16 shared memory,
 *                    4 = 4x8 shared memory (-1 = auto). */
#define FDB_TUNE_TILE_Z 1
#define FDB_TUNE_SHAPE 2
#define FDB_TUNE_DEPTH 3 /* batches only: steps per time block (0 = auto, 2..4) */
/* FDB_TUNE_ADJOINT (single fields and batches): how fdb_*_adjoint computes
 * dL/dv.  0 (default) = in closed form: the step is A = I + sum_j a_j D_j
 * with D_j a periodic shift minus the identity, so A, A^T and every D_j
 * commute and dL/da_j = S <lam^1, D_j f0> with lam^1 = (A^T)^(S-1) lam_T:
 * one transposed run, one contraction and the forward advect, no
 * checkpoints.  1 = step by step with checkpoints and recompute
 * (checkpoint_every applies), one contraction per transposed step.  2 = the
 * closed form with the field(s) left at f0 instead of f_T, for callers that
 * already hold f_T (a reverse-mode framework's backward pass): one transposed
 * run and one contraction.  All compute the same gradient of the discrete
 * scheme, to rounding. */
#define FDB_TUNE_ADJOINT 4
int fdb_upwind_set_tuning(fdb_upwind* h, int key, int value);

/* Number of cells, and the arithmetic the last advect actually used. */
int fdb_upwind_info(fdb_upwind* h, uint64_t* ntot, int* arith_used);

/* Synthetic initial condition on the device: 1 inside the sphere of the given
 * centre/radius (cell centres (i+0.5)*dx), 0 outside, plus noise_amp*U[0,1)
 * from a counter-based SplitMix64 stream keyed by (seed, flat index).  The
 * reference has no such call (its IC is hard-coded, upwind.cxx:48). */
int fdb_upwind_init_sphere(fdb_upwind* h, const double* center, double radius,
                           double noise_amp, uint64_t seed);

/* ---------------------------------------------------------------------------
 * Adjoint (no reference counterpart; the transpose of advect()).
 * Gradients of a loss L(f_T), f_T = advect(num_steps, dt) of the handle's
 * current field f0, given lambda_T = dL/df_T: writes grad_f0 = dL/df0 (ntot
 * values) and grad_v = dL/dv (ndims values, host memory), and leaves the
 * field at f_T (as after advect).  Pointers are device memory when
 * is_device = 1.  dL/df0 = (A^T)^S lambda_T is the forward kernels run on the
 * problem with every upwind direction reversed (the transpose of the step).
 * dL/dv, by default (FDB_TUNE_ADJOINT 0), in closed form: S <lam^1, D_j f0>
 * with lam^1 = (A^T)^(S-1) lambda_T, one contraction -- the whole call costs
 * about two advects.  With FDB_TUNE_ADJOINT 1 it is summed step by step: a
 * forward pass storing a checkpoint every `checkpoint_every` steps
 * (0 = sqrt(num_steps)), then the transposed steps backward, each segment
 * recomputed from its checkpoint, one contraction per step.  With
 * grad_v = NULL only dL/df0 is computed.  The forms agree to rounding.
 * ------------------------------------------------------------------------- */
int fdb_upwind_adjoint(fdb_upwind* h, int num_steps, double dt,
                       const double* lambda_T, double* grad_f0, double* grad_v,
                       int checkpoint_every, int is_device);

/* The transpose of advect() alone: out = (A^T)^num_steps in, by the forward
 * kernels (the handle's arithmetic) on the problem with every upwind direction
 * reversed -- the dL/df0 part of fdb_upwind_adjoint (bit-identical to its
 * grad_v = NULL result) without advancing the field: the field, and what the
 * next advect continues from, are untouched.  For callers that already hold
 * f_T (a reverse-mode framework's backward pass).  ntot values each; device
 * pointers when is_device = 1; in == out allowed.  ndims <= 3.  Synchronises;
 * FDB_ERR_NONFINITE when `in` holds NaN/Inf on the fixed-point path. */
int fdb_upwind_advect_transposed(fdb_upwind* h, int num_steps, double dt, const double* in,
                                 double* out, int is_device);

/* Device time (ms) of the last fdb_upwind_adjoint call, by phase: ms3[0] =
 * forward pass (with checkpoints in the step-by-step form), ms3[1] =
 * recompute of the segment states (step-by-step fixed-point path only),
 * ms3[2] = transposed steps (with the closed form's contraction; in the
 * step-by-step FP64 path: recompute + transposed steps). */
int fdb_upwind_adjoint_timings(fdb_upwind* h, double* ms3);

/* One transposed step on caller buffers (device pointers):
 * lam_out = A^T lam_in, and dcoef[j] += -<lam_in, S_j f - f> (host array).
 * Used by tests and by callers that manage their own checkpoints. */
int fdb_upwind_adjoint_step(fdb_upwind* h, double dt, const double* f_dev,
                            const double* lam_in_dev, double* lam_out_dev,
                            double* dcoef_host);

/* ---------------------------------------------------------------------------
 * Batches (no reference counterpart): many independent Upwind problems of
 * uneven sizes and velocities, each one the reference's Upwind<ndims>
 * (upwind.cxx:23-49) with ndims <= 3, advanced together.
 * fdb_batch_advect runs one persistent launch per call (all instances, all
 * time blocks, per-instance dependency tracking with bounded waits; replayed
 * from a CUDA graph when called again with the same steps, dt and tuning).
 * fdb_batch_advect_looped is the comparator: the single-field kernel looped
 * over the instances, with the depth set by FDB_TUNE_DEPTH (equal depths
 * give bit-identical fields) or, without one, each instance's single-field
 * default (what fdb_upwind_advect picks).  dt holds one time step per
 * instance.
 * ------------------------------------------------------------------------- */
typedef struct {
  int ndims;              /* 1..3 */
  uint64_t num_cells[3];  /* first ndims entries used */
  double velocity[3];
  double lengths[3];
} fdb_instance_desc;

typedef struct fdb_batch fdb_batch;

/* Each instance starts with f = 0, f[0] = 1 (upwind.cxx:45-48). */
int fdb_batch_create(int count, const fdb_instance_desc* descs, fdb_batch** out);
int fdb_batch_destroy(fdb_batch* b);
int fdb_batch_count(fdb_batch* b, int* count, uint64_t* total_cells);
/* Stored axis order of instance `index`: stored axis k (z, y, x) is axis
 * order3[k] of the instance's 3-D view (missing leading axes count as extent
 * 1).  The batch picks the order with the fewest computed cells; fields go in
 * and out in the caller's order regardless. */
int fdb_batch_storage_order(fdb_batch* b, int index, int* order3);
int fdb_batch_set_field(fdb_batch* b, int index, const double* src, int is_device);
int fdb_batch_get_field(fdb_batch* b, int index, double* dst, int is_device);
int fdb_batch_init_sphere(fdb_batch* b, int index, const double* center, double radius,
                          double noise_amp, uint64_t seed);
int fdb_batch_set_stream(fdb_batch* b, void* cuda_stream);
/* New velocity of one instance (ndims values); the field is kept. */
int fdb_batch_set_velocity(fdb_batch* b, int index, const double* velocity);
/* keys FDB_TUNE_DEPTH, FDB_TUNE_SHAPE (2, 3 or 4), FDB_TUNE_TILE_Z, FDB_TUNE_ADJOINT */
int fdb_batch_set_tuning(fdb_batch* b, int key, int value);
int fdb_batch_advect(fdb_batch* b, int num_steps, const double* dt);
int fdb_batch_advect_looped(fdb_batch* b, int num_steps, const double* dt);
/* Batched adjoint: fdb_upwind_adjoint for every instance at once (the
 * fixed-point kernels; FDB_ERR_UNSUPPORTED when an instance is outside the
 * fixed kernel's domain).  By default (FDB_TUNE_ADJOINT 0) dL/dv is in
 * closed form: the transposed persistent launch, one contraction launch over
 * all instances, then the forward persistent launch.  Step by step
 * (FDB_TUNE_ADJOINT 1): the forward pass with checkpoints runs the
 * persistent launch; every recompute and transposed step is one launch over
 * all instances.  lambda_T and grad_f0 hold the instances' fields one after
 * another in the caller's order (instance i starts at the sum of the sizes of
 * instances 0..i-1); grad_v receives 3 values per instance (dL/dv per
 * reference axis, 0 for missing axes; host memory); dt holds one time step
 * per instance; checkpoint_every as in fdb_upwind_adjoint.  The batch's fields
 * are left at f_T.  Field pointers are device memory when is_device = 1.
 * With grad_v = NULL only dL/df0 is computed: the persistent launch on the
 * problems with every upwind direction reversed (as in fdb_upwind_adjoint). */
int fdb_batch_adjoint(fdb_batch* b, int num_steps, const double* dt, const double* lambda_T,
                      double* grad_f0, double* grad_v, int checkpoint_every, int is_device);
/* The transpose of fdb_batch_advect alone for every instance: out = (A^T)^S
 * in (the persistent launch on the problems with every upwind direction
 * reversed), the batch's fields untouched; bit-identical to the grad_f0 of
 * fdb_batch_adjoint with grad_v = NULL.  in and out hold the instances one
 * after another in the caller's order; in == out allowed. */
int fdb_batch_advect_transposed(fdb_batch* b, int num_steps, const double* dt, const double* in,
                                double* out, int is_device);
/* checksum() of every instance (upwind.cxx:91-93) into out[count]; synchronises. */
int fdb_batch_checksums(fdb_batch* b, double* out);
/* Times the compiled (depth, shape, tile_z) choices on a copy of the fields
 * and keeps the fastest; with cache_path, reuses/stores the choice per problem
 * class.  chosen (nullable) receives {depth, shape, tile_z}. */
int fdb_batch_autotune(fdb_batch* b, int num_steps, const double* dt, const char* cache_path,
                       int* chosen);

/* ---------------------------------------------------------------------------
 * Checksum without any allocation.  No counterpart in the reference: it exists
 * for callers that may not allocate GPU memory while they run (a memory pool
 * or arena that owns all device memory, a host that forbids allocation after
 * start-up, a callback where cudaMalloc would synchronise or fail).
 *
 * Sums n FP64 values at d_field into *d_sum, enqueued on cuda_stream (a
 * cudaStream_t; NULL = legacy default stream) and not synchronised.  Both
 * pointers must be device (or managed) memory of the current device; host
 * memory or another GPU's memory returns FDB_ERR_INVALID.  Same kernels and chunking as fdb_upwind_checksum, so the
 * same result.  Scratch is a 2048-double (16 KB) static device array that the
 * library keeps on every GPU it is loaded on until the process exits; nothing
 * in it needs clearing between calls.  Calls that overlap on the GPU share the
 * array and race: serialise them.  The first call on each device looks up the
 * array's device address; make that first call before any stream capture.
 * n must be in [1, FDB_NOALLOC_MAX_VALUES]; other sizes return
 * FDB_ERR_INVALID.
 * ------------------------------------------------------------------------- */
#define FDB_NOALLOC_MAX_VALUES (1ull << 34)
int fdb_checksum_noalloc(const double* d_field, uint64_t n, double* d_sum, void* cuda_stream);

/* Number of kernels this library has launched in this process (all handles,
 * all threads).  A diagnostic for benchmarks; no reference counterpart. */
uint64_t fdb_launch_count(void);

/* Thread-local message for the last non-zero status. */
const char* fdb_last_error(void);

/* Library version string. */
const char* fdb_version(void);

#ifdef __cplusplus
}
#endif
#endif /* FDB_UPWIND_H */
