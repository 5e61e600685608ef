/*
 * fdb_filter.h -- C-ABI of the constant-coefficient stencil Filter of
 * libfdb_upwind.so (plain C types; status codes and fdb_last_error() as in
 * fdb_upwind.h).
 *
 * Replaces the reference's class Filter (cxx/Filter.h:25-230,
 * cxx/Filter.cpp) on one process: the whole grid lives on one GPU, so there
 * are no MPI windows, fetches or domain decomposition (one process gives the
 * decomposition 1 x ... x 1, CubeDecomp.cpp:12-30).  The field is stored as
 * the reference stores it: column-major, axis 0 varying fastest
 * (MultiArrayIter built with rowMajor = false, Filter.cpp:50).
 * include/fidibench_gb/Filter.h rebuilds the class with the reference's
 * signatures on top of these calls.
 */
#ifndef FDB_FILTER_H
#define FDB_FILTER_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct fdb_filter fdb_filter;

/* Index wrap of a neighbour outside the grid (fdb_filter_set_wrap).
 *  FDB_WRAP_REFERENCE : the reference's `(int)i + offset` reduced with
 *                       `%= size_t(N)` (Filter.cpp:238-240): a negative index
 *                       -m becomes (2^64 - m) mod N, which is the periodic
 *                       N - m only when N is a power of two (default, for
 *                       identical results).
 *  FDB_WRAP_PERIODIC  : periodic wrap for every N. */
#define FDB_WRAP_REFERENCE 0
#define FDB_WRAP_PERIODIC 1

/* Replaces Filter(globalDims, xmins, xmaxs, stencil) -- Filter.h:34-38,
 * Filter.cpp:11-75.  offsets: nterms x ndims ints (term t at offsets[t*ndims]),
 * weights: nterms.  Terms are applied in the order of the reference's
 * std::map<std::vector<int>, double> (lexicographic offsets; a repeated
 * offset keeps its first weight, as std::map::insert does).  ndims in
 * [1, 8], nterms in [1, 256]. */
int fdb_filter_create(int ndims, const uint64_t* dims, const double* xmins, const double* xmaxs,
                      int nterms, const int* offsets, const double* weights, fdb_filter** out);

/* Replaces ~Filter (Filter.cpp:77-84). */
int fdb_filter_destroy(fdb_filter* f);

/* setInData / setInDataByIndices (Filter.h:70-79, Filter.cpp:132-190): the
 * input field, ntot values in column-major order (the facade evaluates the
 * user's function on the host, as the reference does, and uploads it). */
int fdb_filter_set_in_data(fdb_filter* f, const double* src, int is_device);

/* The input (which = 0) or output (which = 1) field, column-major (the
 * reference exposes them through printInData/printOutData/saveVTK). */
int fdb_filter_get_data(fdb_filter* f, int which, double* dst, int is_device);

/* applyFilter (Filter.h:84, Filter.cpp:192-260): out = sum over the terms, in
 * map order, of weight * in[neighbour], every product and sum separately
 * rounded as in the reference (bit-identical output).  Enqueued on the
 * filter's stream. */
int fdb_filter_apply(fdb_filter* f);

/* copyOutToIn (Filter.h:150, Filter.cpp:441-463). */
int fdb_filter_copy_out_to_in(fdb_filter* f);

/* `iterations` x (applyFilter; copyOutToIn): the laplacian driver's timing
 * loop (laplacian/cxx/laplacian.cxx:85-90) in one call (the copy is a buffer
 * swap, so input and output hold the same field afterwards). */
int fdb_filter_iterate(fdb_filter* f, int iterations);

/* computeCheckSum("input" | "output") (Filter.h:157, Filter.cpp:466-485):
 * which = 0 input, 1 output.  A deterministic fixed-order tree sum on the
 * device (the reference sums sequentially); synchronises. */
int fdb_filter_checksum(fdb_filter* f, int which, double* out);

/* FDB_WRAP_REFERENCE (default) or FDB_WRAP_PERIODIC. */
int fdb_filter_set_wrap(fdb_filter* f, int mode);

/* Stream to enqueue on (a cudaStream_t; NULL restores the filter's own). */
int fdb_filter_set_stream(fdb_filter* f, void* cuda_stream);

/* Number of cells and of distinct stencil terms. */
int fdb_filter_info(fdb_filter* f, uint64_t* ntot, int* nterms);

/* Wait for the work enqueued on the filter's stream (the reference's calls
 * are synchronous; timing loops call this before reading a clock). */
int fdb_filter_synchronize(fdb_filter* f);

#ifdef __cplusplus
}
#endif

#endif /* FDB_FILTER_H */
