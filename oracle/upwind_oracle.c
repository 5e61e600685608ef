/*
 * upwind_oracle.c -- CPU restatement of FiDiBench's upwind advection hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the parity oracle and the timed CPU
 * baseline.  Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
 * and reference legs may load it; the product path (fidibench_gb300) never
 * links, imports or calls it and fails loudly when its CUDA library is absent.
 *
 * Every function restates the reference algorithm in plain C with the same
 * loop structure and the same floating-point operation order, so that a build
 * without FMA contraction (-ffp-contract=off, which the Makefile sets on every
 * host) gives results bit-identical to the reference's own advect():
 *
 *   fdbo_geometry   <- upwind/cxx/upwind.cxx:27-44   (Upwind ctor: upDirection,
 *                      deltas, ntot, dimProd with the last index fastest)
 *   fdbo_advect     <- upwind/cxx/upwind.cxx:51-86   (copy loop :59-62, update
 *                      loop :64-84, coeff :72, periodic wrap :75-76,
 *                      getIndexSet :122-129, getFlatIndex :131-134)
 *   fdbo_checksum   <- upwind/cxx/upwind.cxx:91-93   (sequential accumulate)
 *   fdbo_std        <- upwind/cxx/upwind.cxx:95-103
 *
 * Pinning: the restatement is checked bit-for-bit against the reference's own
 * upwind.cxx compiled by oracle/Makefile (target `ref`), and against the golden
 * fixtures in tests/golden/ that tests/golden/make_golden.py generated from it.
 *
 * The adjoint and the synthetic-input helpers below have no counterpart in
 * the reference: the adjoint is the exact transpose of fdbo_advect's step (its
 * own correctness is pinned by the dot-product identity against the pinned
 * forward), and the sphere/noise generator is the CPU twin of the device
 * initial-condition kernel.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define FDBO_MAXD 8

typedef struct {
  int ndims;
  uint64_t n[FDBO_MAXD];
  uint64_t dimProd[FDBO_MAXD];
  int up[FDBO_MAXD];
  double deltas[FDBO_MAXD];
  double v[FDBO_MAXD];
  uint64_t ntot;
} fdbo_geom;

/* upwind.cxx:27-44; the spacings come from the grid n_spacing (n itself,
 * or the global grid of which n is a slab). */
static int fdbo_geometry_spacing(int ndims, const uint64_t *n, const double *v,
                                 const double *L, const uint64_t *n_spacing, fdbo_geom *g);

static int fdbo_geometry(int ndims, const uint64_t *n, const double *v,
                         const double *L, fdbo_geom *g) {
  return fdbo_geometry_spacing(ndims, n, v, L, n, g);
}

static int fdbo_geometry_spacing(int ndims, const uint64_t *n, const double *v,
                                 const double *L, const uint64_t *n_spacing, fdbo_geom *g) {
  if (ndims < 1 || ndims > FDBO_MAXD) return 1;
  g->ndims = ndims;
  g->ntot = 1;
  for (int j = 0; j < ndims; ++j) {
    if (n[j] == 0) return 1;
    g->n[j] = n[j];
    g->v[j] = v[j];
    g->up[j] = -1;
    if (v[j] < 0.) g->up[j] = +1;
    if (n_spacing[j] == 0) return 1;
    g->deltas[j] = L[j] / (double)n_spacing[j];
    g->ntot *= n[j];
  }
  g->dimProd[ndims - 1] = 1;
  for (int i = ndims - 2; i >= 0; --i) g->dimProd[i] = g->dimProd[i + 1] * g->n[i + 1];
  return 0;
}

/* The per-axis coefficient exactly as upwind.cxx:72 evaluates it:
 * ((deltaTime * v[j]) * upDirection[j]) / deltas[j]. */
double fdbo_coeff(double dt, double v, int up, double delta) {
  return dt * v * (double)up / delta;
}

uint64_t fdbo_ntot(int ndims, const uint64_t *n) {
  uint64_t t = 1;
  for (int j = 0; j < ndims; ++j) t *= n[j];
  return t;
}

/* The coefficient as the OpenACC/OpenMP-offload variants and the Python
 * class round it: coeff[j] = v[j] * upDirection[j] / deltas[j] once in the
 * constructor (upwindAcc.cxx:45, upwindAcc2.cxx:48, upwind.py:32), then
 * deltaTime * coeff[j] in each update (upwindAcc.cxx:79, upwindAcc2.cxx:85,
 * upwind.py:64). */
double fdbo_coeff_product(double dt, double v, int up, double delta) {
  const double k = v * (double)up / delta;
  return dt * k;
}

/* advect with a choice of coefficient rounding: form 0 = upwind.cxx:72,
 * form 1 = fdbo_coeff_product.  The update itself, f[i] -= c_j * (oldF[upI] -
 * oldF[i]) axis by axis in order j = 0..ndims-1, is the same in every
 * variant (upwind.cxx:80, upwindAcc.cxx:79-87, upwindAcc2.cxx:85-91,
 * upwind.py:55-67). */
int fdbo_advect_form(int ndims, const uint64_t *n, const double *v, const double *L,
                     double *f, double *oldF, int numTimeSteps, double deltaTime,
                     int nthreads, int form);

/* One full advect(numTimeSteps, deltaTime) -- upwind.cxx:51-86.
 * f is updated in place; oldF is caller-provided scratch of ntot doubles.
 * nthreads <= 0 keeps the OpenMP default. Returns 0 on success. */
int fdbo_advect(int ndims, const uint64_t *n, const double *v, const double *L,
                double *f, double *oldF, int numTimeSteps, double deltaTime,
                int nthreads) {
  return fdbo_advect_form(ndims, n, v, L, f, oldF, numTimeSteps, deltaTime, nthreads, 0);
}

static int fdbo_advect_geom(const fdbo_geom *gp, double *f, double *oldF, int numTimeSteps,
                            double deltaTime, int nthreads, int form);

int fdbo_advect_form(int ndims, const uint64_t *n, const double *v, const double *L,
                     double *f, double *oldF, int numTimeSteps, double deltaTime,
                     int nthreads, int form) {
  fdbo_geom g;
  if (fdbo_geometry(ndims, n, v, L, &g)) return 1;
  return fdbo_advect_geom(&g, f, oldF, numTimeSteps, deltaTime, nthreads, form);
}

/* advect on a grid n whose spacings are those of the grid n_spacing (a slab
 * of planes of axis 0 of a larger periodic grid, treated as periodic itself:
 * the test harness of the distributed form). */
int fdbo_advect_spacing(int ndims, const uint64_t *n, const double *v, const double *L,
                        const uint64_t *n_spacing, double *f, double *oldF, int numTimeSteps,
                        double deltaTime, int nthreads, int form) {
  fdbo_geom g;
  if (fdbo_geometry_spacing(ndims, n, v, L, n_spacing, &g)) return 1;
  return fdbo_advect_geom(&g, f, oldF, numTimeSteps, deltaTime, nthreads, form);
}

static int fdbo_advect_geom(const fdbo_geom *gp, double *f, double *oldF, int numTimeSteps,
                            double deltaTime, int nthreads, int form) {
  const fdbo_geom g = *gp;
  const int64_t ntot = (int64_t)g.ntot;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#else
  (void)nthreads;
#endif

#pragma omp parallel
  for (int istep = 0; istep < numTimeSteps; ++istep) {

#pragma omp for
    for (int64_t i = 0; i < ntot; ++i) oldF[i] = f[i];

#pragma omp for
    for (int64_t i = 0; i < ntot; ++i) {
      int64_t inds[FDBO_MAXD];
      /* getIndexSet: upwind.cxx:122-129 */
      for (int d = 0; d < g.ndims; ++d)
        inds[d] = (int64_t)(((uint64_t)i / g.dimProd[d]) % g.n[d]);
      for (int j = 0; j < g.ndims; ++j) {
        int64_t oldIndex = inds[j];
        const double coeff =
            form == 1 ? fdbo_coeff_product(deltaTime, g.v[j], g.up[j], g.deltas[j])
                      : deltaTime * g.v[j] * (double)g.up[j] / g.deltas[j];
        /* periodic BCs: upwind.cxx:75-76 */
        inds[j] = (inds[j] + g.up[j] + (int64_t)g.n[j]) % (int64_t)g.n[j];
        /* getFlatIndex: upwind.cxx:131-134 */
        uint64_t upI = 0;
        for (int d = 0; d < g.ndims; ++d) upI += g.dimProd[d] * (uint64_t)inds[d];
        f[i] -= coeff * (oldF[upI] - oldF[i]);
        inds[j] = oldIndex;
      }
    }
  }
  return 0;
}

/* checksum(): upwind.cxx:91-93, a sequential left-to-right sum. */
double fdbo_checksum(const double *f, uint64_t ntot) {
  double s = 0.0;
  for (uint64_t i = 0; i < ntot; ++i) s = s + f[i];
  return s;
}

/* std(): upwind.cxx:95-103. */
double fdbo_std(const double *f, uint64_t ntot) {
  double mean = fdbo_checksum(f, ntot) / (double)ntot;
  double res = 0;
  for (uint64_t i = 0; i < ntot; ++i) {
    double d = f[i] - mean;
    res += d * d;
  }
  return sqrt(res / (double)ntot);
}

/* ------------------------------------------------------------------------
 * Adjoint of one advect step (no reference counterpart).
 *
 * The forward step is f' = f - sum_j c_j (S_j f - f) with (S_j f)[i] =
 * f[i + up_j e_j] (periodic).  Its transpose is
 *     lam[i] = lam'[i] - sum_j c_j (lam'[i - up_j e_j] - lam'[i]).
 * The velocity gradient of <lam', f'> is accumulated into dcoef[j] as
 *     dcoef[j] += -sum_i lam'[i] (f[i + up_j e_j] - f[i]),
 * the derivative with respect to c_j; the caller applies dc_j/dv_j.
 * lam_in is lam' (after the step), lam_out receives lam (before it), f is the
 * forward state before the step.  Serial and plain: it is only a checker.
 * ------------------------------------------------------------------------ */
int fdbo_adjoint_step(int ndims, const uint64_t *n, const double *v,
                      const double *L, double dt, const double *f,
                      const double *lam_in, double *lam_out, double *dcoef) {
  fdbo_geom g;
  if (fdbo_geometry(ndims, n, v, L, &g)) return 1;
  const int64_t ntot = (int64_t)g.ntot;
  for (int64_t i = 0; i < ntot; ++i) {
    int64_t inds[FDBO_MAXD];
    for (int d = 0; d < g.ndims; ++d)
      inds[d] = (int64_t)(((uint64_t)i / g.dimProd[d]) % g.n[d]);
    double acc = lam_in[i];
    for (int j = 0; j < g.ndims; ++j) {
      const double c = dt * g.v[j] * (double)g.up[j] / g.deltas[j];
      int64_t old = inds[j];
      int64_t nj = (int64_t)g.n[j];
      /* downstream neighbour (i - up_j e_j) for the transposed shift */
      inds[j] = (old - g.up[j] + nj) % nj;
      uint64_t dn = 0;
      for (int d = 0; d < g.ndims; ++d) dn += g.dimProd[d] * (uint64_t)inds[d];
      /* upstream neighbour (i + up_j e_j) for the velocity gradient */
      inds[j] = (old + g.up[j] + nj) % nj;
      uint64_t upI = 0;
      for (int d = 0; d < g.ndims; ++d) upI += g.dimProd[d] * (uint64_t)inds[d];
      inds[j] = old;
      acc -= c * (lam_in[dn] - lam_in[i]);
      dcoef[j] -= lam_in[i] * (f[upI] - f[i]);
    }
    lam_out[i] = acc;
  }
  return 0;
}

/* ------------------------------------------------------------------------
 * Synthetic inputs (no reference counterpart): CPU twin of the device
 * initial-condition kernel.  Uniform deviates come from SplitMix64
 * (Steele, Lea & Flood, OOPSLA 2014) applied to seed + (i+1)*golden-gamma,
 * mapped to [0,1) with the top 53 bits.  The sphere test uses cell centres
 * (i_d + 0.5) * dx_d and sum_d (x_d - c_d)^2 < r^2 evaluated in axis order.
 * ------------------------------------------------------------------------ */
static uint64_t fdbo_splitmix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

double fdbo_uniform(uint64_t seed, uint64_t i) {
  uint64_t h = fdbo_splitmix64(seed + (i + 1) * 0x9E3779B97F4A7C15ull);
  return (double)(h >> 11) * (1.0 / 9007199254740992.0);
}

int fdbo_fill_sphere_noise(int ndims, const uint64_t *n, const double *L,
                           const double *center, double radius,
                           double noise_amp, uint64_t seed, double *f) {
  fdbo_geom g;
  double vzero[FDBO_MAXD] = {0};
  if (fdbo_geometry(ndims, n, vzero, L, &g)) return 1;
  const double r2 = radius * radius;
  const int64_t ntot = (int64_t)g.ntot;
#pragma omp parallel for
  for (int64_t i = 0; i < ntot; ++i) {
    double s = 0.0;
    for (int d = 0; d < g.ndims; ++d) {
      uint64_t id = ((uint64_t)i / g.dimProd[d]) % g.n[d];
      double x = ((double)id + 0.5) * g.deltas[d];
      double e = x - center[d];
      s = s + e * e;
    }
    double val = (s < r2) ? 1.0 : 0.0;
    if (noise_amp != 0.0) val = val + noise_amp * fdbo_uniform(seed, (uint64_t)i);
    f[i] = val;
  }
  return 0;
}

int fdbo_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
