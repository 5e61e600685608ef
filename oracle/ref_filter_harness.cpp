// ref_filter_harness.cpp -- wraps the reference's stencil Filter
// (cxx/Filter.cpp with CubeDecomp.cpp, MultiArrayIter.cpp and writeVTK.cpp),
// compiled from the reference source tree by oracle/Makefile (target `ref`)
// against the single-rank MPI stand-in in oracle/mpi_stub/.  TEST
// INFRASTRUCTURE ONLY: it pins the Filter restatement in filter_oracle.c and
// generates the golden fixtures tests/golden/filter_*.npz.  Nothing is copied:
// the four reference files are #included by path into this one translation
// unit (so that `private` can be opened consistently) after every standard
// header they use.
//
// Exported C entry point:
//   fdbr_filter_run(ndims, dims, nterms, offsets[nterms*ndims], weights,
//                   in, out, iterations, sums[2])
//       Filter(dims, xmins = 0, xmaxs = 1, stencil) with the terms inserted
//       into the std::map in the given order (a repeated offset keeps its
//       first weight, as std::map::insert does); in (column-major, axis 0
//       fastest: the Filter's own order) is set through setInDataByIndices;
//       then `iterations` x (applyFilter; copyOutToIn), except that the last
//       iteration skips copyOutToIn; out = outData; sums = computeCheckSum of
//       "input" and "output" at the end.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <functional>
#include <iostream>
#include <limits>
#include <map>
#include <numeric>
#include <ostream>
#include <string>
#include <vector>

#include "mpi.h"

#define private public
#include "cxx/MultiArrayIter.cpp"
#include "cxx/CubeDecomp.cpp"
#include "cxx/writeVTK.cpp"
#include "cxx/Filter.cpp"
#undef private

namespace {

const double* g_in = nullptr;
std::vector<size_t> g_dims;

// the input value of a cell from its global indices (column-major)
double input_at(const std::vector<size_t>& inds) {
  size_t big = 0, stride = 1;
  for (size_t d = 0; d < g_dims.size(); ++d) {
    big += inds[d] * stride;
    stride *= g_dims[d];
  }
  return g_in[big];
}

}  // namespace

extern "C" int fdbr_filter_run(int ndims, const uint64_t* dims, int nterms, const int* offsets,
                               const double* weights, const double* in, double* out,
                               int iterations, double* sums) {
  if (ndims < 1 || nterms < 1 || iterations < 1) return 1;
  std::vector<size_t> globalDims(dims, dims + ndims);
  std::map<std::vector<int>, double> stencil;
  for (int t = 0; t < nterms; ++t) {
    std::vector<int> off(offsets + t * ndims, offsets + (t + 1) * ndims);
    stencil.insert(std::pair<std::vector<int>, double>(off, weights[t]));
  }
  std::vector<double> xmins(ndims, 0.0), xmaxs(ndims, 1.0);
  Filter fltr(globalDims, xmins, xmaxs, stencil);
  if (!fltr.isDecompValid()) return 2;
  g_in = in;
  g_dims = globalDims;
  fltr.setInDataByIndices(input_at);
  for (int it = 0; it < iterations; ++it) {
    fltr.applyFilter();
    if (it + 1 < iterations) fltr.copyOutToIn();
  }
  std::copy(fltr.outData.begin(), fltr.outData.end(), out);
  sums[0] = fltr.computeCheckSum("input");
  sums[1] = fltr.computeCheckSum("output");
  return 0;
}
