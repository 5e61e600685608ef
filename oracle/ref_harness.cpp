// ref_harness.cpp -- wraps the reference's own Upwind<NDIMS> class
// (upwind/cxx/upwind.cxx:19-135), compiled from the reference source tree by
// oracle/Makefile (target `ref`).  TEST INFRASTRUCTURE ONLY: it pins the C
// restatement in upwind_oracle.c and generates the golden fixtures under
// tests/golden/.  Nothing from the reference is copied here: the reference
// file is #included by path at build time (REFDIR), with `main` renamed and
// `private` opened so that the harness can read and write the field `f`.
//
// Exported C entry points (all fields row-major, last index fastest):
//   fdbr_advect(ndims, n, v, L, f_in, f_out, steps, dt, seconds)
//       builds Upwind<ndims>(v, L, n) (upwind.cxx:23-49), overwrites f with
//       f_in (the reference hard-codes f[0]=1 at :48; the harness replaces it),
//       calls advect(steps, dt) (:51-86) and copies f to f_out.
//   fdbr_checksum / fdbr_std: Upwind::checksum() (:91-93) / std() (:95-103)
//       on a given field.
//   fdbr_default_field(ndims, n, out): the constructor's own initial field.
#include <vector>
#include <array>
#include <functional>
#include <algorithm>
#include <numeric>
#include <string>
#include <fstream>
#include <limits>
#include <iostream>
#include <sstream>
#include <cstring>
#include <cmath>
#include <map>
#include <chrono>
#include <cstdint>
#include <cstdlib>
#ifdef HAVE_OPENMP
#include <omp.h>
#endif
#include "CmdLineArgParser.h"

#define main upwind_ref_main
#define private public
#include "upwind/cxx/upwind.cxx"
#undef private
#undef main

namespace {

double wall_seconds() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch())
      .count();
}

template <size_t D>
int run_advect(const uint64_t* n, const double* v, const double* L,
               const double* f_in, double* f_out, int steps, double dt, double* seconds) {
  std::vector<double> vel(v, v + D), len(L, L + D);
  std::vector<size_t> nc(n, n + D);
  Upwind<D> up(vel, len, nc);
  if (f_in) std::copy(f_in, f_in + up.ntot, up.f.begin());
  const double t0 = wall_seconds();
  up.advect(steps, dt);
  if (seconds) *seconds = wall_seconds() - t0;
  std::copy(up.f.begin(), up.f.end(), f_out);
  return 0;
}

template <size_t D>
double run_reduce(const uint64_t* n, const double* f, int which) {
  std::vector<double> vel(D, 1.0), len(D, 1.0);
  std::vector<size_t> nc(n, n + D);
  Upwind<D> up(vel, len, nc);
  std::copy(f, f + up.ntot, up.f.begin());
  return which == 0 ? up.checksum() : up.std();
}

}  // namespace

extern "C" {

// `seconds` (nullable) receives the wall time of the advect() call alone.
int fdbr_advect(int ndims, const uint64_t* n, const double* v, const double* L,
                const double* f_in, double* f_out, int steps, double dt, double* seconds) {
  switch (ndims) {
    case 1: return run_advect<1>(n, v, L, f_in, f_out, steps, dt, seconds);
    case 2: return run_advect<2>(n, v, L, f_in, f_out, steps, dt, seconds);
    case 3: return run_advect<3>(n, v, L, f_in, f_out, steps, dt, seconds);
    case 4: return run_advect<4>(n, v, L, f_in, f_out, steps, dt, seconds);
    default: return 1;
  }
}

int fdbr_default_field(int ndims, const uint64_t* n, double* out) {
  double v[4] = {1, 1, 1, 1}, L[4] = {1, 1, 1, 1};
  return fdbr_advect(ndims, n, v, L, nullptr, out, 0, 0.0, nullptr);
}

double fdbr_checksum(int ndims, const uint64_t* n, const double* f) {
  switch (ndims) {
    case 1: return run_reduce<1>(n, f, 0);
    case 2: return run_reduce<2>(n, f, 0);
    case 3: return run_reduce<3>(n, f, 0);
    case 4: return run_reduce<4>(n, f, 0);
    default: return std::nan("");
  }
}

double fdbr_std(int ndims, const uint64_t* n, const double* f) {
  switch (ndims) {
    case 1: return run_reduce<1>(n, f, 1);
    case 2: return run_reduce<2>(n, f, 1);
    case 3: return run_reduce<3>(n, f, 1);
    case 4: return run_reduce<4>(n, f, 1);
    default: return std::nan("");
  }
}

int fdbr_max_threads(void) {
#ifdef HAVE_OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

}  // extern "C"
