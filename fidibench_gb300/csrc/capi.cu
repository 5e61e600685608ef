// capi.cu -- the C-ABI of libfdb_upwind (declared in include/fdb_upwind.h).
//
// One handle = one problem on the current CUDA device: two FP64 fields used
// as a ping-pong pair (the reference keeps f plus an oldF copy and copies
// every step, upwind/cxx/upwind.cxx:53-62; here the step reads one buffer and
// writes the other), small reduction scratch, and lazily allocated adjoint
// checkpoint storage.
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <string>
#include <vector>

#include "fdb_internal.h"

struct fdb_upwind {
  fdb::Geom g;
  double* buf[2] = {nullptr, nullptr};
  int cur = 0;
  double* part = nullptr;     // reduction partials (reduce_partials(ntot))
  double* dscal = nullptr;    // device scalars [8]
  double* dpart = nullptr;    // adjoint per-CTA coefficient partials [3 * adjoint_blocks()]
  double* hscal = nullptr;    // pinned host scalars [8]
  double* scratch = nullptr;  // fixed-point path: max|f| slots + error word
  size_t scratch_bytes = 0;
  int scale_slot = -1;        // scratch slot holding max|f| of the current field (-1: unknown)
  fdb::FixedTuning tune;      // fixed kernel launch shape (depth mirrors `depth`)
  cudaStream_t own = nullptr;
  cudaStream_t stream = nullptr;
  int device = 0;
  int arith = FDB_ARITH_AUTO;
  int depth = 0;
  int arith_used = 0;
  // adjoint storage
  std::vector<double*> ckpt;
  std::vector<double*> seg;
  double* lam[2] = {nullptr, nullptr};
  double* adj_dpart = nullptr;  // fixed-point adjoint: per-CTA contraction slots
  int adj_dpart_cap = 0;
  double* adj_scratch = nullptr;
  size_t adj_scratch_bytes = 0;
  double adj_ms[3] = {0.0, 0.0, 0.0};  // last adjoint: forward, recompute, transposed steps
  // fdb_upwind_advect_host_stream: a third field buffer (the three rotate
  // between upload, advect pair and download), the upload and download
  // streams and their events (two of each kind, alternating by field parity)
  double* extra = nullptr;
  // the transposed problem's own max|f| slots and error word, so that a
  // transposed run leaves the field's scale slot valid
  double* tscratch = nullptr;
  // adjoint form: 0 = dL/dv in closed form, 1 = step by step with checkpoints
  int adj_mode = 0;
  fdb::DeviceScratch contract;  // the closed form's contraction tables and partials
  cudaStream_t io_stream[2] = {nullptr, nullptr};
  cudaEvent_t io_ev[7] = {};
  // an open block chain (fdb_upwind_block_begin .. the last
  // fdb_upwind_advect_block): arithmetic, ring position of the next launch,
  // whether it reads FP64, and the depth its guard bits are sized for
  int chain = 0;
  int chain_arith = 0;
  int chain_i = 0;
  int chain_first = 0;
  int chain_K = 0;
};

namespace fdb {

static thread_local std::string g_err;

void set_error(const std::string& msg) { g_err = msg; }

int fail(int code, const std::string& msg) {
  g_err = msg;
  return code;
}

int cuda_fail(cudaError_t e, const char* what) {
  g_err = std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")";
  return FDB_ERR_CUDA;
}

static std::atomic<uint64_t> g_launches{0};

void note_launch(uint64_t n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

bool fault_injected(const char* kind) {
  const char* f = getenv("FDB_FAULT");
  return f && strcmp(f, kind) == 0;
}

int make_geom(int ndims, const double* v, const double* L, const uint64_t* n, Geom* g) {
  return make_geom_spacing(ndims, v, L, n, n, g);
}

int make_geom_spacing(int ndims, const double* v, const double* L, const uint64_t* n,
                      const uint64_t* n_spacing, Geom* g) {
  if (ndims < 1 || ndims > FDB_MAX_DIMS) return fail(FDB_ERR_INVALID, "ndims must be in [1, 8]");
  if (!v || !L || !n || !n_spacing) return fail(FDB_ERR_INVALID, "null velocity/lengths/num_cells");
  Geom r;
  r.ndims = ndims;
  r.ntot = 1;
  for (int j = 0; j < ndims; ++j) {
    if (n[j] == 0 || n_spacing[j] == 0)
      return fail(FDB_ERR_INVALID, "num_cells must be positive on every axis");
    if (!(L[j] > 0.0) || !isfinite(L[j])) return fail(FDB_ERR_INVALID, "lengths must be finite and > 0");
    if (!isfinite(v[j])) return fail(FDB_ERR_INVALID, "velocity must be finite");
    if (r.ntot > (UINT64_MAX / 16) / n[j]) return fail(FDB_ERR_INVALID, "grid too large");
    r.n[j] = n[j];
    r.v[j] = v[j];
    r.L[j] = L[j];
    // upwind.cxx:34-36
    r.up[j] = (v[j] < 0.) ? +1 : -1;
    r.dx[j] = L[j] / (double)n_spacing[j];
    r.nsp[j] = n_spacing[j];
    r.ntot *= n[j];
  }
  r.dimProd[ndims - 1] = 1;
  for (int i = ndims - 2; i >= 0; --i) r.dimProd[i] = r.dimProd[i + 1] * r.n[i + 1];
  if (ndims <= 3) {
    const int pad = 3 - ndims;
    int64_t nn[3] = {1, 1, 1};
    int uu[3] = {-1, -1, -1};
    int jj[3] = {-1, -1, -1};
    for (int j = 0; j < ndims; ++j) {
      nn[pad + j] = (int64_t)r.n[j];
      uu[pad + j] = r.up[j];
      jj[pad + j] = j;
    }
    r.nz = nn[0]; r.ny = nn[1]; r.nx = nn[2];
    r.upz = uu[0]; r.upy = uu[1]; r.upx = uu[2];
    r.jz = jj[0]; r.jy = jj[1]; r.jx = jj[2];
  }
  *g = r;
  return FDB_OK;
}

double ref_coeff(const Geom& g, int j, double dt) {
  if (g.coeff_form == FDB_COEFF_PRODUCT) {
    // coeff[j] = v[j] * upDirection[j] / deltas[j] in the constructor, then
    // deltaTime * coeff[j] per update (upwindAcc.cxx:45,79; upwind.py:32,64)
    const double k = g.v[j] * (double)g.up[j] / g.dx[j];
    return dt * k;
  }
  // deltaTime * this->v[j] * this->upDirection[j] / this->deltas[j]
  return dt * g.v[j] * (double)g.up[j] / g.dx[j];
}

Coeffs3 coeffs3(const Geom& g, double dt) {
  Coeffs3 c{};
  c.cz = g.jz >= 0 ? ref_coeff(g, g.jz, dt) : 0.0;
  c.cy = g.jy >= 0 ? ref_coeff(g, g.jy, dt) : 0.0;
  c.cx = g.jx >= 0 ? ref_coeff(g, g.jx, dt) : 0.0;
  c.az = -c.cz;
  c.ay = -c.cy;
  c.ax = -c.cx;
  c.w = ((1.0 - c.az) - c.ay) - c.ax;
  return c;
}

}  // namespace fdb

using namespace fdb;

namespace {

int check_handle(fdb_upwind* h) {
  if (!h) return fail(FDB_ERR_INVALID, "null handle");
  return FDB_OK;
}

// Calls that read, write or advance the field as FP64 need it closed: between
// fdb_upwind_block_begin and the last block the buffers may hold int64.
int check_no_chain(fdb_upwind* h) {
  FDB_TRY(check_handle(h));
  if (h->chain)
    return fail(FDB_ERR_INVALID, "a block chain is open (finish it with a last "
                                 "fdb_upwind_advect_block first)");
  return FDB_OK;
}

// Report (and clear) the error word that the fixed-point kernels set in a
// scratch block when they meet a non-finite input.  The stream must be
// synchronised.
int check_error_word(double* scratch, const char* what) {
  int* err = fixed_error_word(scratch);
  int herr = 0;
  FDB_CUDA_TRY(cudaMemcpy(&herr, err, sizeof(int), cudaMemcpyDeviceToHost));
  if (herr) {
    FDB_CUDA_TRY(cudaMemset(err, 0, sizeof(int)));
    return fail(FDB_ERR_NONFINITE, std::string(what) +
                                       " holds NaN or Inf values (the fixed-point kernel needs "
                                       "finite input)");
  }
  return FDB_OK;
}

// Synchronise the handle's stream and report a non-finite field.
int sync(fdb_upwind* h) {
  FDB_CUDA_TRY(cudaStreamSynchronize(h->stream));
  FDB_TRY(check_error_word(h->scratch, "the field"));
  if (h->tscratch) FDB_TRY(check_error_word(h->tscratch, "the transposed input"));
  return FDB_OK;
}

void free_adjoint(fdb_upwind* h) {
  for (double* p : h->ckpt) cudaFree(p);
  for (double* p : h->seg) cudaFree(p);
  h->ckpt.clear();
  h->seg.clear();
  for (int k = 0; k < 2; ++k) {
    if (h->lam[k]) cudaFree(h->lam[k]);
    h->lam[k] = nullptr;
  }
  if (h->adj_dpart) cudaFree(h->adj_dpart);
  if (h->adj_scratch) cudaFree(h->adj_scratch);
  h->adj_dpart = nullptr;
  h->adj_scratch = nullptr;
  h->adj_dpart_cap = 0;
  h->adj_scratch_bytes = 0;
}

int dalloc(double** p, size_t count) {
  if (fault_injected("alloc")) return fail(FDB_ERR_INJECTED, "injected allocation failure");
  cudaError_t e = cudaMalloc((void**)p, count * sizeof(double));
  if (e != cudaSuccess) {
    *p = nullptr;
    cudaGetLastError();
    return fail(FDB_ERR_ALLOC, std::string("cudaMalloc of ") + std::to_string(count * 8) +
                                   " bytes failed: " + cudaGetErrorString(e));
  }
  return FDB_OK;
}

int resolve_arith(fdb_upwind* h, const Coeffs3& c) {
  const Geom& g = h->g;
  if (g.ndims > 3) return FDB_ARITH_EXACT;  // generic kernel
  if (h->arith == FDB_ARITH_EXACT || h->arith == FDB_ARITH_FMA) return h->arith;
  const bool ok = fixed_supported(g, c, h->depth) == FDB_OK;
  if (h->arith == FDB_ARITH_FIXED) return ok ? FDB_ARITH_FIXED : -1;
  return (ok && fixed_preferred(g)) ? FDB_ARITH_FIXED : FDB_ARITH_FMA;
}

// The arithmetic an advect by dt uses (FDB_ERR_UNSUPPORTED when FIXED was
// forced outside its domain).
int pick_arith(fdb_upwind* h, double dt, int* arith) {
  *arith = FDB_ARITH_EXACT;
  if (h->g.ndims > 3) return FDB_OK;  // generic kernel
  *arith = resolve_arith(h, coeffs3(h->g, dt));
  if (*arith < 0)
    return fail(FDB_ERR_UNSUPPORTED,
                "FDB_ARITH_FIXED requested but the geometry/coefficients are outside its "
                "domain (see fdb_upwind_set_arith)");
  return FDB_OK;
}

// Advance the handle's field by `steps` steps with the given arithmetic.
int advance(fdb_upwind* h, int steps, double dt, int arith) {
  const Geom& g = h->g;
  if (g.ndims > 3) {
    for (int s = 0; s < steps; ++s) {
      FDB_TRY(launch_step_generic(g, dt, h->buf[h->cur], h->buf[h->cur ^ 1], h->stream));
      h->cur ^= 1;
    }
    return FDB_OK;
  }
  const Coeffs3 c = coeffs3(g, dt);
  if (arith == FDB_ARITH_FIXED) {
    h->tune.depth = h->depth;
    const int rc = launch_advect_fixed_ex(g, c, steps, h->tune, h->buf, &h->cur, h->scratch,
                                          h->scratch_bytes, &h->scale_slot, h->stream);
    if (rc) h->scale_slot = -1;
    return rc;
  }
  h->scale_slot = -1;
  for (int s = 0; s < steps; ++s) {
    FDB_TRY(launch_step_f64(g, c, arith, h->buf[h->cur], h->buf[h->cur ^ 1], h->stream));
    h->cur ^= 1;
  }
  return FDB_OK;
}

// A CUDA event that lives as long as its scope.
struct ScopedEvent {
  cudaEvent_t e = nullptr;
  ScopedEvent() { cudaEventCreate(&e); }
  ~ScopedEvent() {
    if (e) cudaEventDestroy(e);
  }
  ScopedEvent(const ScopedEvent&) = delete;
  ScopedEvent& operator=(const ScopedEvent&) = delete;
};

// The arithmetic of the adjoint and of transposed runs: the fixed-point
// kernels where the handle's settings allow them and the coefficients are in
// their domain, else the FP64 kernel the handle asks for.
int adjoint_arith(fdb_upwind* h, const Coeffs3& c) {
  const bool fixed = (h->arith == FDB_ARITH_AUTO || h->arith == FDB_ARITH_FIXED) &&
                     fixed_supported(h->g, c, 1) == FDB_OK &&
                     fixed_supported(h->g, c, h->depth) == FDB_OK;
  return fixed ? FDB_ARITH_FIXED
               : ((h->arith == FDB_ARITH_EXACT) ? FDB_ARITH_EXACT : FDB_ARITH_FMA);
}

// The transposed problem runs through the handle's adjoint buffers lam[0..1]
// with its own scale scratch, so the field, its buffers and its scale slot are
// untouched.  A^T is the upwind step with every direction reversed and the
// same Courant numbers, so the forward kernels on the transposed geometry
// (with the coefficients of g) apply it.
//
// lam[0] = in (allocating the buffers on first use).
int transposed_load(fdb_upwind* h, const double* in, int is_device) {
  const Geom& g = h->g;
  if (!h->lam[0]) {
    int rc = dalloc(&h->lam[0], g.ntot);
    if (!rc) rc = dalloc(&h->lam[1], g.ntot);
    if (rc) {
      free_adjoint(h);
      return rc;
    }
  }
  if (!h->tscratch) {
    FDB_TRY(dalloc(&h->tscratch, (fixed_scratch_bytes() + 7) / 8));
    FDB_CUDA_TRY(cudaMemsetAsync(h->tscratch, 0, h->scratch_bytes, h->stream));
  }
  FDB_CUDA_TRY(cudaMemcpyAsync(h->lam[0], in, g.ntot * sizeof(double),
                               is_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                               h->stream));
  return FDB_OK;
}

// Advance the adjoint buffers by S transposed steps: *lc (in/out) names the
// buffer that holds the state, *slot (in/out, fixed path; -1: unknown) the
// transposed scratch slot that describes it.  The state is FP64 on return.
int transposed_steps(fdb_upwind* h, int S, double dt, int arith, int* lc, int* slot) {
  if (S <= 0) return FDB_OK;
  const Geom gT = transposed_geom(h->g);
  const Coeffs3 c = coeffs3(h->g, dt);
  if (arith == FDB_ARITH_FIXED) {
    FixedTuning t = h->tune;
    t.depth = h->depth;
    return launch_advect_fixed_ex(gT, c, S, t, h->lam, lc, h->tscratch, h->scratch_bytes, slot,
                                  h->stream);
  }
  *slot = -1;
  for (int k = 0; k < S; ++k) {
    FDB_TRY(launch_step_f64(gT, c, arith, h->lam[*lc], h->lam[*lc ^ 1], h->stream));
    *lc ^= 1;
  }
  return FDB_OK;
}

// out = (A^T)^S in.  t_done (nullable) is recorded after the last step.
int transposed_run(fdb_upwind* h, int S, double dt, const double* in, double* out,
                   int is_device, cudaEvent_t t_done) {
  const int arith = adjoint_arith(h, coeffs3(h->g, dt));
  FDB_TRY(transposed_load(h, in, is_device));
  int lc = 0, slot = -1;
  FDB_TRY(transposed_steps(h, S, dt, arith, &lc, &slot));
  if (t_done) FDB_CUDA_TRY(cudaEventRecord(t_done, h->stream));
  FDB_CUDA_TRY(cudaMemcpyAsync(out, h->lam[lc], h->g.ntot * sizeof(double),
                               is_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                               h->stream));
  return FDB_OK;
}

// The full gradient in closed form.  The step is A = I + sum_j a_j D_j with
// D_j = S_j - I, S_j the periodic shift by up_j along axis j: constant
// coefficients on a periodic grid, so A, A^T and every D_j commute, and
//   dL/da_j = sum_n <lam^{n+1}, D_j f^n>
//           = sum_n <lam_T, A^{S-1-n} D_j A^n f0> = S <lam^1, D_j f0>,
// lam^1 = (A^T)^{S-1} lam_T.  So: S - 1 transposed steps, one contraction with
// the field (still f0), the last transposed step (dL/df0 = (A^T)^S lam_T),
// then advect(S) leaves the field at f_T exactly as advect() does.  No
// checkpoints and no recompute; the identity is exact for the discrete
// scheme, so it agrees with the step-by-step form to rounding.
int adjoint_closed_form(fdb_upwind* h, int S, double dt, int arith, const double* lambda_T,
                        double* grad_f0, int is_device, bool advance_field, double dda[3]) {
  ScopedEvent t0, t1, t2;
  cudaEventRecord(t0.e, h->stream);
  FDB_TRY(transposed_load(h, lambda_T, is_device));
  int lc = 0, slot = -1;
  FDB_TRY(transposed_steps(h, S - 1, dt, arith, &lc, &slot));
  const int64_t zero = 0;
  FDB_TRY(launch_vel_contract(1, &h->g, &zero, h->buf[h->cur], h->lam[lc], h->dscal, h->contract,
                              h->stream));
  // the last step measures max|lam^1| afresh, as the batched form does, so
  // that dL/df0 is the same bit for bit in both
  slot = -1;
  FDB_TRY(transposed_steps(h, 1, dt, arith, &lc, &slot));
  cudaEventRecord(t1.e, h->stream);
  FDB_CUDA_TRY(cudaMemcpyAsync(grad_f0, h->lam[lc], h->g.ntot * sizeof(double),
                               is_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                               h->stream));
  if (advance_field) FDB_TRY(advance(h, S, dt, arith));
  cudaEventRecord(t2.e, h->stream);
  FDB_CUDA_TRY(cudaMemcpyAsync(h->hscal, h->dscal, 3 * sizeof(double), cudaMemcpyDeviceToHost,
                               h->stream));
  FDB_TRY(sync(h));
  float ms = 0.f;
  h->adj_ms[0] = h->adj_ms[1] = h->adj_ms[2] = 0.0;
  if (cudaEventElapsedTime(&ms, t1.e, t2.e) == cudaSuccess) h->adj_ms[0] = ms;
  if (cudaEventElapsedTime(&ms, t0.e, t1.e) == cudaSuccess) h->adj_ms[2] = ms;
  cudaGetLastError();
  for (int k = 0; k < 3; ++k) dda[k] = (double)S * h->hscal[k];
  return FDB_OK;
}

// dL/dv from dL/da of the internal axes (z, y, x):
// a_j = -c_j = -dt v_j up_j / dx_j  =>  dL/dv_j = dL/da_j * (-dt up_j / dx_j).
void velocity_grad(const Geom& g, double dt, const double dda[3], double* grad_v) {
  const int jj[3] = {g.jz, g.jy, g.jx};
  for (int j = 0; j < g.ndims; ++j) grad_v[j] = 0.0;
  for (int k = 0; k < 3; ++k)
    if (jj[k] >= 0) grad_v[jj[k]] = dda[k] * (-dt * (double)g.up[jj[k]] / g.dx[jj[k]]);
}

// Buffers and streams of fdb_upwind_advect_host_stream, created on first use.
int ensure_host_stream(fdb_upwind* h) {
  if (!h->extra) FDB_TRY(dalloc(&h->extra, h->g.ntot));
  for (cudaStream_t& s : h->io_stream)
    if (!s) FDB_CUDA_TRY(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  for (cudaEvent_t& e : h->io_ev)
    if (!e) FDB_CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  return FDB_OK;
}

// The three field buffers of the host stream and the role each plays now:
// `in` holds the field about to advect, `other` is its ping-pong partner and
// `third` receives the next upload (it held the previous result, whose
// download must end first).  The roles rotate after every field; the three
// pointers never change.
struct FieldRing {
  double* d[3];
  int in, other, third;
};

// Enqueue the whole host stream.  Event slots: 0 = start, 1 + p = field
// uploaded, 3 + p = field advected and summed, 5 + p = field downloaded, with
// p the parity of the field (a wait binds to the record made before it, so
// two slots per kind suffice).
int host_stream_enqueue(fdb_upwind* h, int count, const double* const* in, double* const* out,
                        int num_steps, double dt, int arith, double* dsum, FieldRing& r) {
  const size_t bytes = h->g.ntot * sizeof(double);
  cudaStream_t cs = h->stream, up = h->io_stream[0], down = h->io_stream[1];
  cudaEvent_t* ev = h->io_ev;
  // the copy streams start after the work already on the handle's stream
  FDB_CUDA_TRY(cudaEventRecord(ev[0], cs));
  FDB_CUDA_TRY(cudaStreamWaitEvent(up, ev[0], 0));
  FDB_CUDA_TRY(cudaStreamWaitEvent(down, ev[0], 0));
  FDB_CUDA_TRY(cudaMemcpyAsync(r.d[r.in], in[0], bytes, cudaMemcpyHostToDevice, up));
  FDB_CUDA_TRY(cudaEventRecord(ev[1], up));
  for (int k = 0; k < count; ++k) {
    const int p = k & 1;
    if (k + 1 < count) {
      if (k >= 1) FDB_CUDA_TRY(cudaStreamWaitEvent(up, ev[5 + (p ^ 1)], 0));
      FDB_CUDA_TRY(cudaMemcpyAsync(r.d[r.third], in[k + 1], bytes, cudaMemcpyHostToDevice, up));
      FDB_CUDA_TRY(cudaEventRecord(ev[1 + (p ^ 1)], up));
    }
    FDB_CUDA_TRY(cudaStreamWaitEvent(cs, ev[1 + p], 0));
    h->buf[0] = r.d[r.in];
    h->buf[1] = r.d[r.other];
    h->cur = 0;
    h->scale_slot = -1;  // a new field: the fixed path measures max|f| again
    if (num_steps > 0) FDB_TRY(advance(h, num_steps, dt, arith));
    const int res = h->cur == 0 ? r.in : r.other;
    const int spare = h->cur == 0 ? r.other : r.in;
    FDB_TRY(launch_sum(r.d[res], h->g.ntot, h->part, dsum + k, cs));
    FDB_CUDA_TRY(cudaEventRecord(ev[3 + p], cs));
    FDB_CUDA_TRY(cudaStreamWaitEvent(down, ev[3 + p], 0));
    FDB_CUDA_TRY(cudaMemcpyAsync(out[k], r.d[res], bytes, cudaMemcpyDeviceToHost, down));
    FDB_CUDA_TRY(cudaEventRecord(ev[5 + p], down));
    r.in = r.third;  // uploaded while this field advected
    r.other = spare;
    r.third = res;   // free again once its download ends
  }
  return FDB_OK;
}

}  // namespace

extern "C" {

const char* fdb_last_error(void) { return g_err.c_str(); }

const char* fdb_version(void) { return "fidibench_gb300 0.1.0 (sm_103a)"; }

uint64_t fdb_launch_count(void) { return g_launches.load(std::memory_order_relaxed); }

}  // extern "C"

namespace {

int create_handle(int ndims, const double* velocity, const double* lengths,
                  const uint64_t* num_cells, const uint64_t* n_spacing, fdb_upwind** out) {
  if (!out) return fail(FDB_ERR_INVALID, "null output handle pointer");
  *out = nullptr;
  Geom g;
  FDB_TRY(make_geom_spacing(ndims, velocity, lengths, num_cells, n_spacing, &g));
  fdb_upwind* h = new fdb_upwind();
  h->g = g;
  int rc = FDB_OK;
  cudaError_t e = cudaGetDevice(&h->device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&h->own, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    rc = cuda_fail(e, "cudaStreamCreate");
    delete h;
    return rc;
  }
  h->stream = h->own;
  if ((rc = dalloc(&h->buf[0], g.ntot)) || (rc = dalloc(&h->buf[1], g.ntot)) ||
      (rc = dalloc(&h->part, reduce_partials(g.ntot))) || (rc = dalloc(&h->dscal, 8)) ||
      (rc = dalloc(&h->dpart, 3 * (size_t)adjoint_blocks())) ||
      (rc = dalloc(&h->scratch, (fixed_scratch_bytes() + 7) / 8))) {
    fdb_upwind_destroy(h);
    return rc;
  }
  h->scratch_bytes = (fixed_scratch_bytes() + 7) / 8 * 8;
  e = cudaMemsetAsync(h->scratch, 0, h->scratch_bytes, h->stream);
  if (e == cudaSuccess) e = cudaMallocHost((void**)&h->hscal, 8 * sizeof(double));
  if (e != cudaSuccess) {
    fdb_upwind_destroy(h);
    return cuda_fail(e, "cudaMallocHost");
  }
  // f = 0, f[0] = 1 (upwind.cxx:45-48)
  rc = launch_fill_corner(h->buf[0], g.ntot, h->stream);
  if (!rc) rc = sync(h);
  if (rc) {
    fdb_upwind_destroy(h);
    return rc;
  }
  *out = h;
  return FDB_OK;
}

// A plane range [first, first + count) of axis 0, as offsets in values.
int plane_range(fdb_upwind* h, uint64_t first, uint64_t count, uint64_t* off, uint64_t* len) {
  const uint64_t plane = h->g.ntot / h->g.n[0];
  if (first > h->g.n[0] || count > h->g.n[0] - first)
    return fail(FDB_ERR_INVALID, "plane range outside the field");
  *off = first * plane;
  *len = count * plane;
  return FDB_OK;
}

}  // namespace

extern "C" {

int fdb_upwind_create(int ndims, const double* velocity, const double* lengths,
                      const uint64_t* num_cells, fdb_upwind** out) {
  return create_handle(ndims, velocity, lengths, num_cells, num_cells, out);
}

int fdb_upwind_create_slab(int ndims, const double* velocity, const double* lengths,
                           const uint64_t* num_cells_global, uint64_t slab_planes,
                           fdb_upwind** out) {
  if (!num_cells_global) return fail(FDB_ERR_INVALID, "null num_cells_global");
  if (ndims < 1 || ndims > FDB_MAX_DIMS) return fail(FDB_ERR_INVALID, "ndims must be in [1, 8]");
  if (slab_planes == 0) return fail(FDB_ERR_INVALID, "slab_planes must be positive");
  uint64_t n[FDB_MAX_DIMS];
  for (int j = 0; j < ndims; ++j) n[j] = num_cells_global[j];
  n[0] = slab_planes;
  return create_handle(ndims, velocity, lengths, n, num_cells_global, out);
}

int fdb_upwind_get_planes(fdb_upwind* h, uint64_t first, uint64_t count, double* dst,
                          int is_device) {
  FDB_TRY(check_handle(h));
  if (!dst) return fail(FDB_ERR_INVALID, "null destination");
  uint64_t off = 0, len = 0;
  FDB_TRY(plane_range(h, first, count, &off, &len));
  if (len == 0) return FDB_OK;
  FDB_CUDA_TRY(cudaMemcpyAsync(dst, h->buf[h->cur] + off, len * sizeof(double),
                               is_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                               h->stream));
  return is_device ? FDB_OK : sync(h);
}

int fdb_upwind_set_planes(fdb_upwind* h, uint64_t first, uint64_t count, const double* src,
                          int is_device) {
  FDB_TRY(check_handle(h));
  if (!src) return fail(FDB_ERR_INVALID, "null source");
  uint64_t off = 0, len = 0;
  FDB_TRY(plane_range(h, first, count, &off, &len));
  // new values: the fixed path measures max|f| again (inside a block chain
  // the caller agrees the scale word instead)
  if (!h->chain) h->scale_slot = -1;
  if (len == 0) return FDB_OK;
  FDB_CUDA_TRY(cudaMemcpyAsync(h->buf[h->cur] + off, src, len * sizeof(double),
                               is_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                               h->stream));
  return is_device ? FDB_OK : sync(h);
}

int fdb_upwind_set_own_planes(fdb_upwind* h, uint64_t first, uint64_t count) {
  FDB_TRY(check_no_chain(h));
  if (count == 0 || first > h->g.n[0] || count > h->g.n[0] - first)
    return fail(FDB_ERR_INVALID, "own planes outside the field");
  h->g.own0 = first;
  h->g.own_n = count == h->g.n[0] ? 0 : count;
  h->scale_slot = -1;
  return FDB_OK;
}

int fdb_upwind_block_begin(fdb_upwind* h, double dt, int* fixed) {
  FDB_TRY(check_no_chain(h));
  if (!isfinite(dt)) return fail(FDB_ERR_INVALID, "dt must be finite");
  int arith = 0;
  FDB_TRY(pick_arith(h, dt, &arith));
  h->arith_used = arith;
  h->chain_arith = arith;
  h->chain_first = 1;
  if (arith == FDB_ARITH_FIXED) {
    h->chain_K = h->depth > 0 ? h->depth : default_depth(h->g);
    if (h->scale_slot < 0) {
      FDB_TRY(launch_scale_prepass(h->g, h->buf[h->cur], h->scratch, h->stream));
      h->scale_slot = 0;
    }
    h->chain_i = h->scale_slot;
  }
  h->chain = 1;
  if (fixed) *fixed = arith == FDB_ARITH_FIXED;
  return FDB_OK;
}

int fdb_upwind_advect_block(fdb_upwind* h, int steps, double dt, int last) {
  NvtxScope nvtx_("fdb.advect_block");
  FDB_TRY(check_handle(h));
  if (!h->chain) return fail(FDB_ERR_INVALID, "no block chain is open (fdb_upwind_block_begin)");
  if (steps < 1) return fail(FDB_ERR_INVALID, "a block advances at least one step");
  if (!isfinite(dt)) return fail(FDB_ERR_INVALID, "dt must be finite");
  const Coeffs3 c = coeffs3(h->g, dt);
  int rc = FDB_OK;
  if (h->chain_arith == FDB_ARITH_FIXED) {
    if (steps > h->chain_K)
      return fail(FDB_ERR_INVALID, "a fixed-point block advances at most its depth of steps");
    rc = launch_fixed_block(h->g, c, steps, h->tune, h->chain_K, h->buf, &h->cur,
                            h->chain_first != 0, last != 0, h->scratch, h->chain_i, h->stream);
    if (!rc) {
      ++h->chain_i;
      h->chain_first = 0;
      if (last) h->scale_slot = h->chain_i % 3;
    }
  } else {
    rc = advance(h, steps, dt, h->chain_arith);
  }
  if (rc) {
    h->chain = 0;  // the field is no longer defined: measure afresh next time
    h->scale_slot = -1;
    return rc;
  }
  if (last) h->chain = 0;
  return FDB_OK;
}

int fdb_upwind_get_scale_word(fdb_upwind* h, uint64_t* dst, int is_device) {
  FDB_TRY(check_handle(h));
  if (!dst) return fail(FDB_ERR_INVALID, "null destination");
  if (!h->chain || h->chain_arith != FDB_ARITH_FIXED)
    return fail(FDB_ERR_INVALID, "no fixed-point block chain is open");
  FDB_CUDA_TRY(cudaMemcpyAsync(dst, scale_word(h->scratch, h->chain_i), sizeof(uint64_t),
                               is_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                               h->stream));
  return is_device ? FDB_OK : sync(h);
}

int fdb_upwind_set_scale_word(fdb_upwind* h, const uint64_t* src, int is_device) {
  FDB_TRY(check_handle(h));
  if (!src) return fail(FDB_ERR_INVALID, "null source");
  if (!h->chain || h->chain_arith != FDB_ARITH_FIXED)
    return fail(FDB_ERR_INVALID, "no fixed-point block chain is open");
  FDB_CUDA_TRY(cudaMemcpyAsync(scale_word(h->scratch, h->chain_i), src, sizeof(uint64_t),
                               is_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                               h->stream));
  return is_device ? FDB_OK : sync(h);
}

int fdb_upwind_checksum_planes(fdb_upwind* h, uint64_t first, uint64_t count, double* out) {
  FDB_TRY(check_no_chain(h));
  if (!out) return fail(FDB_ERR_INVALID, "null output");
  uint64_t off = 0, len = 0;
  FDB_TRY(plane_range(h, first, count, &off, &len));
  if (len == 0) {
    *out = 0.0;
    return FDB_OK;
  }
  FDB_TRY(launch_sum(h->buf[h->cur] + off, len, h->part, h->dscal, h->stream));
  FDB_CUDA_TRY(cudaMemcpyAsync(h->hscal, h->dscal, sizeof(double), cudaMemcpyDeviceToHost,
                               h->stream));
  FDB_TRY(sync(h));
  *out = h->hscal[0];
  return FDB_OK;
}

int fdb_upwind_destroy(fdb_upwind* h) {
  if (!h) return FDB_OK;
  if (h->stream) cudaStreamSynchronize(h->stream);
  free_adjoint(h);
  for (int k = 0; k < 2; ++k)
    if (h->buf[k]) cudaFree(h->buf[k]);
  if (h->part) cudaFree(h->part);
  if (h->dscal) cudaFree(h->dscal);
  if (h->dpart) cudaFree(h->dpart);
  if (h->scratch) cudaFree(h->scratch);
  if (h->hscal) cudaFreeHost(h->hscal);
  if (h->extra) cudaFree(h->extra);
  if (h->tscratch) cudaFree(h->tscratch);
  h->contract.release();
  for (cudaStream_t s : h->io_stream)
    if (s) cudaStreamDestroy(s);
  for (cudaEvent_t e : h->io_ev)
    if (e) cudaEventDestroy(e);
  if (h->own) cudaStreamDestroy(h->own);
  delete h;
  return FDB_OK;
}

int fdb_upwind_set_field(fdb_upwind* h, const double* src, int is_device) {
  FDB_TRY(check_no_chain(h));
  if (!src) return fail(FDB_ERR_INVALID, "null source field");
  h->scale_slot = -1;
  FDB_CUDA_TRY(cudaMemcpyAsync(h->buf[h->cur], src, h->g.ntot * sizeof(double),
                               is_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                               h->stream));
  return sync(h);
}

int fdb_upwind_get_field(fdb_upwind* h, double* dst, int is_device) {
  FDB_TRY(check_no_chain(h));
  if (!dst) return fail(FDB_ERR_INVALID, "null destination field");
  FDB_CUDA_TRY(cudaMemcpyAsync(dst, h->buf[h->cur], h->g.ntot * sizeof(double),
                               is_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                               h->stream));
  return sync(h);
}

int fdb_upwind_field_ptr(fdb_upwind* h, double** out) {
  FDB_TRY(check_handle(h));
  if (!out) return fail(FDB_ERR_INVALID, "null output pointer");
  *out = h->buf[h->cur];
  h->scale_slot = -1;  // the caller may write through the pointer
  return FDB_OK;
}

int fdb_upwind_advect(fdb_upwind* h, int num_steps, double dt) {
  NvtxScope nvtx_("fdb.advect");
  FDB_TRY(check_no_chain(h));
  if (num_steps < 0) return fail(FDB_ERR_INVALID, "num_steps must be >= 0");
  if (!isfinite(dt)) return fail(FDB_ERR_INVALID, "dt must be finite");
  if (num_steps == 0) return FDB_OK;
  int arith = 0;
  FDB_TRY(pick_arith(h, dt, &arith));
  h->arith_used = arith;
  return advance(h, num_steps, dt, arith);
}

int fdb_upwind_checksum(fdb_upwind* h, double* out) {
  FDB_TRY(check_no_chain(h));
  if (!out) return fail(FDB_ERR_INVALID, "null output");
  FDB_TRY(launch_sum(h->buf[h->cur], h->g.ntot, h->part, h->dscal, h->stream));
  FDB_CUDA_TRY(cudaMemcpyAsync(h->hscal, h->dscal, sizeof(double), cudaMemcpyDeviceToHost,
                               h->stream));
  FDB_TRY(sync(h));
  *out = h->hscal[0];
  return FDB_OK;
}

int fdb_upwind_advect_host_stream(fdb_upwind* h, int count, const double* const* in,
                                  double* const* out, int num_steps, double dt,
                                  double* checksums) {
  NvtxScope nvtx_("fdb.advect_host_stream");
  FDB_TRY(check_no_chain(h));
  if (count < 0) return fail(FDB_ERR_INVALID, "count must be >= 0");
  if (num_steps < 0) return fail(FDB_ERR_INVALID, "num_steps must be >= 0");
  if (!isfinite(dt)) return fail(FDB_ERR_INVALID, "dt must be finite");
  if (count == 0) return FDB_OK;
  if (!in || !out) return fail(FDB_ERR_INVALID, "null field array");
  for (int k = 0; k < count; ++k)
    if (!in[k] || !out[k]) return fail(FDB_ERR_INVALID, "null host field");
  int arith = h->arith_used;
  if (num_steps > 0) FDB_TRY(pick_arith(h, dt, &arith));
  FDB_TRY(ensure_host_stream(h));
  double* dsum = nullptr;
  FDB_TRY(dalloc(&dsum, (size_t)count));
  FieldRing r{{h->buf[h->cur], h->buf[h->cur ^ 1], h->extra}, 0, 1, 2};
  int rc = host_stream_enqueue(h, count, in, out, num_steps, dt, arith, dsum, r);
  // drain the copy streams before the buffers change hands
  cudaError_t e0 = cudaStreamSynchronize(h->io_stream[0]);
  cudaError_t e1 = cudaStreamSynchronize(h->io_stream[1]);
  if (rc == FDB_OK) {
    h->buf[0] = r.d[r.third];  // the last result
    h->buf[1] = r.d[r.other];
    h->extra = r.d[r.in];
    h->arith_used = arith;
    rc = sync(h);
    if (rc == FDB_OK && e0 != cudaSuccess) rc = cuda_fail(e0, "upload stream");
    if (rc == FDB_OK && e1 != cudaSuccess) rc = cuda_fail(e1, "download stream");
  } else {
    cudaStreamSynchronize(h->stream);
    h->buf[0] = r.d[0];
    h->buf[1] = r.d[1];
    h->extra = r.d[2];
    h->scale_slot = -1;
  }
  h->cur = 0;
  if (rc == FDB_OK && checksums) {
    cudaError_t e = cudaMemcpy(checksums, dsum, (size_t)count * sizeof(double),
                               cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) rc = cuda_fail(e, "checksum copy");
  }
  cudaFree(dsum);
  return rc;
}

int fdb_upwind_advect_transposed(fdb_upwind* h, int num_steps, double dt, const double* in,
                                 double* out, int is_device) {
  NvtxScope nvtx_("fdb.advect_transposed");
  FDB_TRY(check_no_chain(h));
  if (h->g.ndims > 3) return fail(FDB_ERR_UNSUPPORTED, "the transposed advect serves ndims <= 3");
  if (num_steps < 0) return fail(FDB_ERR_INVALID, "num_steps must be >= 0");
  if (!isfinite(dt)) return fail(FDB_ERR_INVALID, "dt must be finite");
  if (!in || !out) return fail(FDB_ERR_INVALID, "null input or output");
  FDB_TRY(transposed_run(h, num_steps, dt, in, out, is_device, nullptr));
  return sync(h);
}

int fdb_upwind_std(fdb_upwind* h, double* out) {
  FDB_TRY(check_no_chain(h));
  if (!out) return fail(FDB_ERR_INVALID, "null output");
  FDB_TRY(launch_std(h->buf[h->cur], h->g.ntot, h->part, h->dscal + 1, h->dscal, h->stream));
  FDB_CUDA_TRY(cudaMemcpyAsync(h->hscal, h->dscal, sizeof(double), cudaMemcpyDeviceToHost,
                               h->stream));
  FDB_TRY(sync(h));
  *out = h->hscal[0];
  return FDB_OK;
}

int fdb_upwind_set_velocity(fdb_upwind* h, const double* velocity) {
  FDB_TRY(check_handle(h));
  if (!velocity) return fail(FDB_ERR_INVALID, "null velocity");
  Geom g;
  FDB_TRY(make_geom_spacing(h->g.ndims, velocity, h->g.L, h->g.n, h->g.nsp, &g));
  g.coeff_form = h->g.coeff_form;
  h->g = g;
  return FDB_OK;
}

int fdb_upwind_set_coeff_form(fdb_upwind* h, int form) {
  FDB_TRY(check_handle(h));
  if (form != FDB_COEFF_CXX && form != FDB_COEFF_PRODUCT)
    return fail(FDB_ERR_INVALID, "coefficient form must be FDB_COEFF_CXX or FDB_COEFF_PRODUCT");
  h->g.coeff_form = form;
  return FDB_OK;
}

int fdb_upwind_set_stream(fdb_upwind* h, void* cuda_stream) {
  FDB_TRY(check_handle(h));
  FDB_TRY(sync(h));
  h->stream = cuda_stream ? (cudaStream_t)cuda_stream : h->own;
  return FDB_OK;
}

int fdb_upwind_set_arith(fdb_upwind* h, int arith, int temporal_depth) {
  FDB_TRY(check_handle(h));
  if (arith < FDB_ARITH_AUTO || arith > FDB_ARITH_FIXED)
    return fail(FDB_ERR_INVALID, "unknown arithmetic");
  if (temporal_depth < 0 || temporal_depth > 16)
    return fail(FDB_ERR_INVALID, "temporal_depth must be in [0, 16]");
  h->arith = arith;
  h->depth = temporal_depth;
  return FDB_OK;
}

int fdb_upwind_set_tuning(fdb_upwind* h, int key, int value) {
  FDB_TRY(check_handle(h));
  if (key == FDB_TUNE_TILE_Z) {
    if (value < 0) return fail(FDB_ERR_INVALID, "tile_z must be >= 0");
    h->tune.tz = value;
    return FDB_OK;
  }
  if (key == FDB_TUNE_SHAPE) {
    if (value < -1 || value >= fx_num_shapes())
      return fail(FDB_ERR_INVALID, "shape must be in [-1, 6]");
    h->tune.shape = value;
    return FDB_OK;
  }
  if (key == FDB_TUNE_ADJOINT) {
    if (value < 0 || value > 2) return fail(FDB_ERR_INVALID, "adjoint form must be 0, 1 or 2");
    h->adj_mode = value;
    return FDB_OK;
  }
  return fail(FDB_ERR_INVALID, "unknown tuning key");
}

int fdb_upwind_info(fdb_upwind* h, uint64_t* ntot, int* arith_used) {
  FDB_TRY(check_handle(h));
  if (ntot) *ntot = h->g.ntot;
  if (arith_used) *arith_used = h->arith_used;
  return FDB_OK;
}

int fdb_upwind_init_sphere(fdb_upwind* h, const double* center, double radius, double noise_amp,
                           uint64_t seed) {
  FDB_TRY(check_no_chain(h));
  if (!center) return fail(FDB_ERR_INVALID, "null centre");
  h->scale_slot = -1;
  FDB_TRY(launch_sphere_noise(h->g, center, radius, noise_amp, seed, h->buf[h->cur], h->stream));
  return sync(h);
}

int fdb_upwind_adjoint_timings(fdb_upwind* h, double* ms3) {
  FDB_TRY(check_handle(h));
  if (!ms3) return fail(FDB_ERR_INVALID, "null output");
  for (int k = 0; k < 3; ++k) ms3[k] = h->adj_ms[k];
  return FDB_OK;
}

int fdb_upwind_adjoint_step(fdb_upwind* h, double dt, const double* f_dev,
                            const double* lam_in_dev, double* lam_out_dev, double* dcoef_host) {
  FDB_TRY(check_handle(h));
  if (h->g.ndims > 3) return fail(FDB_ERR_UNSUPPORTED, "adjoint serves ndims <= 3");
  if (!f_dev || !lam_in_dev || !lam_out_dev) return fail(FDB_ERR_INVALID, "null buffer");
  const Geom& g = h->g;
  const Coeffs3 c = coeffs3(g, dt);
  FDB_CUDA_TRY(cudaMemsetAsync(h->dpart, 0, 3 * adjoint_blocks() * sizeof(double), h->stream));
  FDB_TRY(launch_adjoint_step(g, c, f_dev, lam_in_dev, lam_out_dev, h->dpart, h->stream));
  FDB_TRY(launch_adjoint_finish(h->dpart, h->dscal, h->stream));
  FDB_CUDA_TRY(cudaMemcpyAsync(h->hscal, h->dscal, 3 * sizeof(double), cudaMemcpyDeviceToHost,
                               h->stream));
  FDB_TRY(sync(h));
  if (dcoef_host) {
    const int jj[3] = {g.jz, g.jy, g.jx};
    for (int k = 0; k < 3; ++k)
      if (jj[k] >= 0) dcoef_host[jj[k]] += h->hscal[k];
  }
  return FDB_OK;
}

int fdb_upwind_adjoint(fdb_upwind* h, int num_steps, double dt, const double* lambda_T,
                       double* grad_f0, double* grad_v, int checkpoint_every, int is_device) {
  NvtxScope nvtx_("fdb.adjoint");
  FDB_TRY(check_no_chain(h));
  const Geom& g = h->g;
  if (g.ndims > 3) return fail(FDB_ERR_UNSUPPORTED, "adjoint serves ndims <= 3");
  if (num_steps < 0) return fail(FDB_ERR_INVALID, "num_steps must be >= 0");
  if (!lambda_T || !grad_f0) return fail(FDB_ERR_INVALID, "null lambda_T or grad_f0");
  if (checkpoint_every < 0) return fail(FDB_ERR_INVALID, "checkpoint_every must be >= 0");
  const int S = num_steps;
  int K = checkpoint_every;
  if (K == 0) K = std::max(1, (int)ceil(sqrt((double)std::max(S, 1))));
  if (K > std::max(S, 1)) K = std::max(S, 1);
  const int nseg = (S + K - 1) / K;
  const size_t bytes = g.ntot * sizeof(double);
  const Coeffs3 c = coeffs3(g, dt);
  // Default: the fixed-point adjoint (forward and recompute on the integer
  // pipes).  EXACT/FMA requests, or coefficients outside the fixed kernel's
  // domain, use the FP64 adjoint with FP64 recompute.
  const int arith = adjoint_arith(h, c);
  const bool fixed = arith == FDB_ARITH_FIXED;

  if (!grad_v) {
    // dL/df0 only: grad_f0 = (A^T)^S lambda_T by the forward kernels on the
    // transposed geometry (transposed_run): no checkpoints, no recompute, no
    // contraction.  The field is advanced to f_T as in the full path (kept
    // at f0 in form 2).
    ScopedEvent t0, t1, t2;
    cudaEventRecord(t0.e, h->stream);
    if (h->adj_mode != 2) FDB_TRY(advance(h, S, dt, arith));
    cudaEventRecord(t1.e, h->stream);
    FDB_TRY(transposed_run(h, S, dt, lambda_T, grad_f0, is_device, t2.e));
    const int rc = sync(h);
    float ms = 0.f;
    h->adj_ms[0] = h->adj_ms[1] = h->adj_ms[2] = 0.0;
    if (cudaEventElapsedTime(&ms, t0.e, t1.e) == cudaSuccess) h->adj_ms[0] = ms;
    if (cudaEventElapsedTime(&ms, t1.e, t2.e) == cudaSuccess) h->adj_ms[2] = ms;
    cudaGetLastError();
    return rc;
  }

  if (h->adj_mode != 1) {
    double dda[3] = {0.0, 0.0, 0.0};
    if (S == 0) {
      FDB_TRY(sync(h));
      FDB_CUDA_TRY(cudaMemcpy(grad_f0, lambda_T, bytes,
                              is_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToHost));
      h->adj_ms[0] = h->adj_ms[1] = h->adj_ms[2] = 0.0;
    } else {
      NvtxScope nvtx_c("fdb.adjoint.closed_form");
      FDB_TRY(adjoint_closed_form(h, S, dt, arith, lambda_T, grad_f0, is_device,
                                  h->adj_mode == 0, dda));
    }
    velocity_grad(g, dt, dda, grad_v);
    return FDB_OK;
  }

  // storage: nseg checkpoints, the segment's states (FP64: K - 1 buffers;
  // fixed point: two int64 chain buffers and K int32 arrays), two adjoint
  // buffers
  const int nsegbuf = std::max(K, adjoint_fixed_segment_buffers(K));
  if ((int)h->ckpt.size() < nseg || (int)h->seg.size() < nsegbuf || !h->lam[0]) {
    free_adjoint(h);
    h->ckpt.assign(nseg, nullptr);
    h->seg.assign(nsegbuf, nullptr);
    int rc = FDB_OK;
    for (auto& p : h->ckpt)
      if (!rc) rc = dalloc(&p, g.ntot);
    for (auto& p : h->seg)
      if (!rc) rc = dalloc(&p, g.ntot);
    if (!rc) rc = dalloc(&h->lam[0], g.ntot);
    if (!rc) rc = dalloc(&h->lam[1], g.ntot);
    if (rc) {
      free_adjoint(h);
      return rc;
    }
  }
  // forward with checkpoints: ckpt[s] = f^{sK}.  Every timing event of the
  // call lives in `events` and is destroyed on every return path.
  EventPool events;
  cudaEvent_t fe0 = events.make(), fe1 = events.make();
  EventPool::record(fe0, h->stream);
  {
    NvtxScope nvtx_f("fdb.adjoint.forward");
    for (int s = 0; s < nseg; ++s) {
      FDB_CUDA_TRY(cudaMemcpyAsync(h->ckpt[s], h->buf[h->cur], bytes, cudaMemcpyDeviceToDevice,
                                   h->stream));
      const int len = std::min(K, S - s * K);
      FDB_TRY(advance(h, len, dt, arith));
    }
  }
  EventPool::record(fe1, h->stream);
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> rec_ev, adj_ev;
  auto collect_times = [&]() {
    float ms = 0.f;
    h->adj_ms[0] = h->adj_ms[1] = h->adj_ms[2] = 0.0;
    if (fe0 && fe1 && cudaEventElapsedTime(&ms, fe0, fe1) == cudaSuccess) h->adj_ms[0] = ms;
    for (auto& e : rec_ev) {
      if (cudaEventElapsedTime(&ms, e.first, e.second) == cudaSuccess) h->adj_ms[1] += ms;
    }
    for (auto& e : adj_ev) {
      if (cudaEventElapsedTime(&ms, e.first, e.second) == cudaSuccess) h->adj_ms[2] += ms;
    }
    cudaGetLastError();
  };
  double dda[3] = {0.0, 0.0, 0.0};  // dL/da (internal axes z, y, x)

  if (fixed) {
    const int ctas = adjoint_fixed_ctas(g, c);
    const size_t sb = adjoint_fixed_scratch_bytes(K);
    if (h->adj_dpart_cap < ctas || h->adj_scratch_bytes < sb) {
      if (h->adj_dpart) cudaFree(h->adj_dpart);
      if (h->adj_scratch) cudaFree(h->adj_scratch);
      h->adj_dpart = nullptr;
      h->adj_scratch = nullptr;
      h->adj_dpart_cap = 0;
      h->adj_scratch_bytes = 0;
      FDB_TRY(dalloc(&h->adj_dpart, 3 * (size_t)ctas));
      FDB_TRY(dalloc(&h->adj_scratch, (sb + 7) / 8));
      h->adj_dpart_cap = ctas;
      h->adj_scratch_bytes = (sb + 7) / 8 * 8;
      FDB_CUDA_TRY(cudaMemsetAsync(h->adj_scratch, 0, h->adj_scratch_bytes, h->stream));
    }
    // the field's partner buffer is free after the forward pass: it holds
    // lam_T (host input) and then dL/df0 (host output)
    double* tmp = h->buf[h->cur ^ 1];
    const double* lamT = lambda_T;
    if (!is_device) {
      FDB_CUDA_TRY(cudaMemcpyAsync(tmp, lambda_T, bytes, cudaMemcpyHostToDevice, h->stream));
      lamT = tmp;
    }
    AdjointFixedIO io;
    io.g = &g;
    io.c = &c;
    io.S = S;
    io.K = K;
    io.nseg = nseg;
    io.ckpt = h->ckpt.data();
    io.chain[0] = (int64_t*)h->seg[0];
    io.chain[1] = (int64_t*)h->seg[1];
    std::vector<int32_t*> hi(K);
    for (int k = 0; k < K; ++k) hi[k] = (int32_t*)h->seg[2 + k / 2] + (k & 1) * g.ntot;
    io.state_hi = hi.data();
    io.lam[0] = (int64_t*)h->lam[0];
    io.lam[1] = (int64_t*)h->lam[1];
    io.lam_T = lamT;
    io.grad_f0 = is_device ? grad_f0 : tmp;
    io.dpart = h->adj_dpart;
    io.dpart_cap = h->adj_dpart_cap;
    io.dda3 = h->dscal;
    io.scratch = h->adj_scratch;
    io.recompute_ev = &rec_ev;
    io.adjoint_ev = &adj_ev;
    io.events = &events;
    FDB_TRY(adjoint_fixed_run(io, h->stream));
    if (!is_device)
      FDB_CUDA_TRY(cudaMemcpyAsync(grad_f0, tmp, bytes, cudaMemcpyDeviceToHost, h->stream));
    FDB_CUDA_TRY(cudaMemcpyAsync(h->hscal, h->dscal, 3 * sizeof(double), cudaMemcpyDeviceToHost,
                                 h->stream));
    FDB_TRY(sync(h));
    collect_times();
    int herr = 0;
    FDB_CUDA_TRY(cudaMemcpy(&herr, (char*)h->adj_scratch + 6 * 16, sizeof(int),
                            cudaMemcpyDeviceToHost));
    if (herr) {
      cudaMemset((char*)h->adj_scratch + 6 * 16, 0, sizeof(int));
      return fail(FDB_ERR_NONFINITE, "adjoint: lambda_T or the field holds NaN or Inf");
    }
    for (int k = 0; k < 3; ++k) dda[k] = h->hscal[k];
  } else {
    // backward in FP64; the recompute repeats the forward's per-step arithmetic
    int lc = 0;
    FDB_CUDA_TRY(cudaMemcpyAsync(h->lam[lc], lambda_T, bytes,
                                 is_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                                 h->stream));
    FDB_CUDA_TRY(cudaMemsetAsync(h->dpart, 0, 3 * adjoint_blocks() * sizeof(double), h->stream));
    cudaEvent_t be0 = events.make(), be1 = events.make();
    EventPool::record(be0, h->stream);
    if (be0 && be1) adj_ev.push_back({be0, be1});
    rec_ev.clear();
    for (int s = nseg - 1; s >= 0; --s) {
      const int len = std::min(K, S - s * K);
      // states f^{sK+1} .. f^{sK+len-1} into seg[0 .. len-2]
      const double* prev = h->ckpt[s];
      for (int k = 1; k < len; ++k) {
        FDB_TRY(launch_step_f64(g, c, arith, prev, h->seg[k - 1], h->stream));
        prev = h->seg[k - 1];
      }
      for (int k = len - 1; k >= 0; --k) {
        const double* fk = (k == 0) ? h->ckpt[s] : h->seg[k - 1];
        FDB_TRY(launch_adjoint_step(g, c, fk, h->lam[lc], h->lam[lc ^ 1], h->dpart, h->stream));
        lc ^= 1;
      }
    }
    EventPool::record(be1, h->stream);
    FDB_CUDA_TRY(cudaMemcpyAsync(grad_f0, h->lam[lc], bytes,
                                 is_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                                 h->stream));
    FDB_TRY(launch_adjoint_finish(h->dpart, h->dscal, h->stream));
    FDB_CUDA_TRY(cudaMemcpyAsync(h->hscal, h->dscal, 3 * sizeof(double), cudaMemcpyDeviceToHost,
                                 h->stream));
    FDB_TRY(sync(h));
    collect_times();
    // the FP64 kernel accumulates dL/dc = -dL/da
    for (int k = 0; k < 3; ++k) dda[k] = -h->hscal[k];
  }
  velocity_grad(g, dt, dda, grad_v);
  return FDB_OK;
}

}  // extern "C"
