// ref_acc_harness.cpp -- wraps the reference's OpenACC variants of the upwind
// class, upwind/cxx/upwindAcc.cxx (one-step advect(double), :49-90) and
// upwind/cxx/upwindAcc2.cxx (advect(int, double), :52-99), compiled from the
// reference source tree by oracle/Makefile (target `ref`) with g++, which
// ignores the `#pragma acc` directives and runs the loops serially.  TEST
// INFRASTRUCTURE ONLY: it generates golden fixtures for the product
// coefficient form (deltaTime * (v * up / dx)) that these variants use.
// Nothing from the reference is copied: each file is #included by path at
// build time inside its own namespace (both define `Upwind<NDIMS>`), with
// `main` renamed and `private` opened so that the harness can set the field.
//
// Exported C entry point (3-D only: the variants' index headers assume 3 axes):
//   fdbr_acc_advect(variant, n[3], v[3], L[3], f_in, f_out, steps, dt)
//       variant 1: Upwind(v, L, std::vector<int> n) of upwindAcc.cxx, then
//                  `steps` calls of advect(dt);
//       variant 2: the same class of upwindAcc2.cxx, then advect(steps, dt).
//       f_in (nullable) replaces the constructor's f = 0, f[0] = 1.
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
#include <cstdint>
#include "CmdLineArgParser.h"

#define private public
#define main upwind_acc1_main
namespace acc1 {
#include "upwind/cxx/upwindAcc.cxx"
}
#undef main
#define main upwind_acc2_main
namespace acc2 {
#include "upwind/cxx/upwindAcc2.cxx"
}
#undef main
#undef private

namespace {

template <class U>
U make(const uint64_t* n, const double* v, const double* L, const double* f_in) {
  std::vector<double> vel(v, v + 3), len(L, L + 3);
  std::vector<int> nc(n, n + 3);
  U up(vel, len, nc);
  if (f_in) std::copy(f_in, f_in + up.ntot, up.f.begin());
  return up;
}

}  // namespace

extern "C" int fdbr_acc_advect(int variant, const uint64_t* n, const double* v, const double* L,
                               const double* f_in, double* f_out, int steps, double dt) {
  if (variant == 1) {
    acc1::Upwind<3> up = make<acc1::Upwind<3>>(n, v, L, f_in);
    for (int s = 0; s < steps; ++s) up.advect(dt);
    std::copy(up.f.begin(), up.f.end(), f_out);
    return 0;
  }
  if (variant == 2) {
    acc2::Upwind<3> up = make<acc2::Upwind<3>>(n, v, L, f_in);
    up.advect(steps, dt);
    std::copy(up.f.begin(), up.f.end(), f_out);
    return 0;
  }
  return 1;
}
