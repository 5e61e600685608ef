/*
 * filter_oracle.c -- CPU restatement of the reference's stencil Filter on one
 * process (TEST INFRASTRUCTURE ONLY: tests/, smoke() and bench.py's CPU legs
 * call it as the checker; the product never does).
 *
 * Follows cxx/Filter.cpp and cxx/MultiArrayIter.{h,cpp} of the reference:
 *  - data are column-major: the big index runs over axis 0 fastest
 *    (MultiArrayIter built with rowMajor = false, Filter.cpp:50,
 *    MultiArrayIter.cpp:43-47);
 *  - the stencil is a std::map<std::vector<int>, double>: its terms are
 *    visited in lexicographic order of the offset vectors, and a repeated
 *    offset keeps its first weight (std::map::insert) -- fdbo_stencil_order;
 *  - applyFilter (Filter.cpp:192-260): out = 0, then for each term and each
 *    cell, out[i] += w * in[neighbour], every product and sum separately
 *    rounded;
 *  - the neighbour index along axis j is (int)inds[j] + offset[j] reduced with
 *    `%= globalDims[j]` (Filter.cpp:238-240): the int is converted to size_t
 *    first, so a negative index -m becomes (2^64 - m) mod N.  This equals the
 *    periodic N - m only when N divides 2^64 (powers of two); mode
 *    FDBO_WRAP_REFERENCE reproduces it, FDBO_WRAP_PERIODIC is the periodic
 *    wrap;
 *  - computeCheckSum (Filter.cpp:466-485): sequential sum in big-index order;
 *  - setInData (Filter.cpp:132-141) with cell centres xmin + (i + 0.5) dx
 *    (Filter.cpp:104-112).
 *
 * Parity of this row is anchored on these reads of the source and on known
 * answers (the reference Filter needs MPI, which this image does not have, so
 * it is not compiled here): the discrete Laplacian of prod_j sin(2 pi x_j) on
 * a power-of-two periodic grid, and the reference's testStencil2d case.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifndef M_PI
#define M_PI 3.14159265358979323846 /* the value <cmath> gives the reference */
#endif

#define FDBO_WRAP_REFERENCE 0
#define FDBO_WRAP_PERIODIC 1

/* Lexicographic comparison of two offset vectors (std::vector<int>::operator<). */
static int lex_less(const int* a, const int* b, int nd) {
  for (int j = 0; j < nd; ++j) {
    if (a[j] < b[j]) return 1;
    if (b[j] < a[j]) return 0;
  }
  return 0;
}

/* order[0..*nuniq) = the term indices in std::map order, a repeated offset
 * keeping its first insertion.  Insertion sort: stencils are small. */
int fdbo_stencil_order(int ndims, int nterms, const int* offsets, int* order, int* nuniq) {
  int n = 0;
  for (int t = 0; t < nterms; ++t) {
    const int* o = offsets + (size_t)t * ndims;
    int dup = 0;
    for (int k = 0; k < n && !dup; ++k)
      if (memcmp(offsets + (size_t)order[k] * ndims, o, sizeof(int) * (size_t)ndims) == 0) dup = 1;
    if (dup) continue;
    int k = n;
    while (k > 0 && lex_less(o, offsets + (size_t)order[k - 1] * ndims, ndims)) {
      order[k] = order[k - 1];
      --k;
    }
    order[k] = t;
    ++n;
  }
  *nuniq = n;
  return 0;
}

static int64_t wrap_index(int64_t t, uint64_t N, int mode) {
  if (mode == FDBO_WRAP_PERIODIC) {
    int64_t r = t % (int64_t)N;
    return r < 0 ? r + (int64_t)N : r;
  }
  /* (int)inds + offset, then `%= size_t` (Filter.cpp:238-240) */
  const int32_t as_int = (int32_t)t;
  return (int64_t)((uint64_t)(int64_t)as_int % N);
}

int fdbo_filter_apply(int ndims, const uint64_t* dims, int nterms, const int* offsets,
                      const double* weights, const double* in, double* out, int mode) {
  if (ndims < 1 || ndims > 8 || nterms < 0) return 1;
  int* order = (int*)malloc(sizeof(int) * (size_t)(nterms > 0 ? nterms : 1));
  int nu = 0;
  fdbo_stencil_order(ndims, nterms, offsets, order, &nu);
  uint64_t ntot = 1, prod[8];
  for (int j = 0; j < ndims; ++j) {
    prod[j] = ntot; /* column-major strides */
    ntot *= dims[j];
  }
  for (uint64_t i = 0; i < ntot; ++i) out[i] = 0.0;
  for (int k = 0; k < nu; ++k) {
    const int* o = offsets + (size_t)order[k] * ndims;
    const double w = weights[order[k]];
#pragma omp parallel for schedule(static)
    for (int64_t ii = 0; ii < (int64_t)ntot; ++ii) {
      const uint64_t i = (uint64_t)ii;
      uint64_t bi = 0;
      for (int j = 0; j < ndims; ++j) {
        const int64_t ind = (int64_t)(i / prod[j] % dims[j]);
        bi += prod[j] * (uint64_t)wrap_index(ind + o[j], dims[j], mode);
      }
      const double p = w * in[bi];
      out[i] = out[i] + p;
    }
  }
  free(order);
  return 0;
}

double fdbo_filter_checksum(const double* f, uint64_t n) {
  double s = 0.0;
  for (uint64_t i = 0; i < n; ++i) s += f[i];
  return s;
}

/* setInData with the laplacian driver's input, prod_j sin(2 pi x_j) at the
 * cell centres (laplacian/cxx/laplacian.cxx:22-28, Filter.cpp:104-112). */
int fdbo_filter_sin_input(int ndims, const uint64_t* dims, const double* xmins,
                          const double* xmaxs, double* f) {
  uint64_t ntot = 1, prod[8];
  for (int j = 0; j < ndims; ++j) {
    prod[j] = ntot;
    ntot *= dims[j];
  }
  for (uint64_t i = 0; i < ntot; ++i) {
    double res = 1.0;
    for (int j = 0; j < ndims; ++j) {
      const uint64_t ind = i / prod[j] % dims[j];
      const double delta = (xmaxs[j] - xmins[j]) / (double)dims[j];
      const double pos = xmins[j] + ((double)ind + 0.5) * delta;
      res *= sin(2.0 * M_PI * pos);
    }
    f[i] = res;
  }
  return 0;
}
