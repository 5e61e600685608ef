// filter.cu -- the constant-coefficient stencil Filter (include/fdb_filter.h),
// the GPU form of the reference's cxx/Filter.cpp on one process.
//
// out[i] = sum over the terms (std::map order of the offsets) of
// w_t * in[neighbour_t(i)], each product and each sum separately rounded and
// accumulated from +0 as in Filter.cpp:192-260, so the output is
// bit-identical to the reference.  Weights of exactly +1 or -1 skip the FP64
// multiply (x * 1 = x and x * -1 = -x exactly for every x but a signalling
// NaN, which stays signalling instead of being quietened); the first term
// replaces `0 + p` by p with -0 turned into +0 (the only case in which the
// sum differs from p).  GB300's FP64 pipe (about 2 operations per clock per
// SM) bounds the kernel: the 7-point Laplacian costs 6 DADD + 1 DMUL per cell.
//
// Layout: column-major like the reference (axis 0 fastest).  Up to 3 axes use
// a 3-D grid over (x = axis 0, y = axis 1, z = axis 2) with one thread per
// cell; cells whose every neighbour is inside the grid use precomputed linear
// offsets, the others wrap each axis (FDB_WRAP_REFERENCE reproduces the
// reference's `%= size_t` of a negative int, see fdb_filter.h).  More axes
// use a generic kernel that decodes every index.
#include <algorithm>
#include <cstring>
#include <vector>

#include "fdb_filter.h"
#include "fdb_internal.h"

namespace {

constexpr int kMaxFastTerms = 32;
constexpr int kMaxTerms = 256;

struct FTerm {
  int o[3];
  int kind;  // 0: w * x, 1: x, 2: -x
  long long lin;
  double w;
};

struct FArgs3 {
  long long n[3];
  long long r[3];  // 2^64 mod n (reference wrap) or 0 (periodic)
  int lo[3], hi[3];  // neighbours stay inside for i in [lo, n - hi)
  int nterms;
  FTerm t[kMaxFastTerms];
};

// (2^64 + v) mod n for v < 0 (reference) or the periodic wrap (r = 0), and v
// mod n for v >= 0
__device__ __forceinline__ long long wrap_axis(long long v, long long n, long long r) {
  long long u = (v >= 0 ? v : v + r) % n;
  return u < 0 ? u + n : u;
}

__device__ __forceinline__ double term_value(const FTerm& t, double x) {
  if (t.kind == 1) return x;
  if (t.kind == 2) return __longlong_as_double(__double_as_longlong(x) ^ (long long)0x8000000000000000ull);
  return __dmul_rn(t.w, x);
}

// first term: 0 + p, i.e. p with -0 -> +0
__device__ __forceinline__ double first_sum(double p) {
  const long long b = __double_as_longlong(p);
  return b == (long long)0x8000000000000000ull ? 0.0 : p;
}

__global__ void __launch_bounds__(128)
k_filter3(const double* __restrict__ in, double* __restrict__ out, const FArgs3 a) {
  const long long x = (long long)blockIdx.x * 128 + threadIdx.x;
  if (x >= a.n[0]) return;
  for (long long z = blockIdx.z; z < a.n[2]; z += gridDim.z) {
    for (long long y = blockIdx.y; y < a.n[1]; y += gridDim.y) {
      const long long i = x + a.n[0] * (y + a.n[1] * z);
      const bool inside = x >= a.lo[0] && x < a.n[0] - a.hi[0] && y >= a.lo[1] &&
                          y < a.n[1] - a.hi[1] && z >= a.lo[2] && z < a.n[2] - a.hi[2];
      double acc = 0.0;
      for (int k = 0; k < a.nterms; ++k) {
        const FTerm& t = a.t[k];
        long long j;
        if (inside) {
          j = i + t.lin;
        } else {
          const long long jx = wrap_axis(x + t.o[0], a.n[0], a.r[0]);
          const long long jy = wrap_axis(y + t.o[1], a.n[1], a.r[1]);
          const long long jz = wrap_axis(z + t.o[2], a.n[2], a.r[2]);
          j = jx + a.n[0] * (jy + a.n[1] * jz);
        }
        const double p = term_value(t, __ldg(in + j));
        acc = (k == 0) ? first_sum(p) : __dadd_rn(acc, p);
      }
      out[i] = acc;
    }
  }
}

struct FArgsN {
  int ndims;
  int nterms;
  unsigned long long n[FDB_MAX_DIMS];
  unsigned long long prod[FDB_MAX_DIMS];
  long long r[FDB_MAX_DIMS];
  unsigned long long ntot;
};

// generic: any number of axes, terms in global memory (offsets [t][ndims])
__global__ void __launch_bounds__(256)
k_filter_nd(const double* __restrict__ in, double* __restrict__ out, const FArgsN a,
            const int* __restrict__ offs, const int* __restrict__ kinds,
            const double* __restrict__ w) {
  for (unsigned long long i = blockIdx.x * 256ull + threadIdx.x; i < a.ntot;
       i += (unsigned long long)gridDim.x * 256ull) {
    double acc = 0.0;
    for (int k = 0; k < a.nterms; ++k) {
      unsigned long long j = 0;
      for (int d = 0; d < a.ndims; ++d) {
        const long long ind = (long long)(i / a.prod[d] % a.n[d]);
        j += a.prod[d] *
             (unsigned long long)wrap_axis(ind + offs[k * a.ndims + d], (long long)a.n[d], a.r[d]);
      }
      FTerm t;
      t.kind = kinds[k];
      t.w = w[k];
      const double p = term_value(t, __ldg(in + j));
      acc = (k == 0) ? first_sum(p) : __dadd_rn(acc, p);
    }
    out[i] = acc;
  }
}

}  // namespace

struct fdb_filter {
  int ndims = 0;
  uint64_t n[FDB_MAX_DIMS] = {0};
  double xmins[FDB_MAX_DIMS] = {0};
  double xmaxs[FDB_MAX_DIMS] = {0};
  uint64_t ntot = 0;
  std::vector<int> offs;  // [nterms][ndims], map order
  std::vector<double> w;
  std::vector<int> kind;
  int wrap = FDB_WRAP_REFERENCE;
  double* buf[2] = {nullptr, nullptr};  // in = buf[cur], out = buf[cur ^ 1]
  int cur = 0;
  double* part = nullptr;
  double* dsum = nullptr;
  double* hsum = nullptr;
  int* d_offs = nullptr;
  int* d_kind = nullptr;
  double* d_w = nullptr;
  cudaStream_t own = nullptr;
  cudaStream_t stream = nullptr;
};

namespace {

using fdb::fail;

int falloc(void** p, size_t bytes) {
  if (fdb::fault_injected("alloc")) return fail(FDB_ERR_INJECTED, "injected allocation failure");
  cudaError_t e = cudaMalloc(p, bytes);
  if (e != cudaSuccess) {
    *p = nullptr;
    cudaGetLastError();
    return fail(FDB_ERR_ALLOC, std::string("cudaMalloc of ") + std::to_string(bytes) +
                                   " bytes failed: " + cudaGetErrorString(e));
  }
  return FDB_OK;
}

int check(fdb_filter* f) { return f ? FDB_OK : fail(FDB_ERR_INVALID, "null filter handle"); }

bool lex_less(const int* a, const int* b, int nd) {
  return std::lexicographical_compare(a, a + nd, b, b + nd);
}

// 2^64 mod n
long long pow2_64_mod(uint64_t n) { return (long long)((~0ull % n + 1) % n); }

int launch_apply(fdb_filter* f) {
  if (fdb::fault_injected("launch")) return fail(FDB_ERR_INJECTED, "injected launch failure");
  const double* in = f->buf[f->cur];
  double* out = f->buf[f->cur ^ 1];
  const int nt = (int)f->w.size();
  if (f->ndims <= 3 && nt <= kMaxFastTerms) {
    FArgs3 a{};
    for (int d = 0; d < 3; ++d) {
      a.n[d] = d < f->ndims ? (long long)f->n[d] : 1;
      a.r[d] = f->wrap == FDB_WRAP_REFERENCE ? pow2_64_mod((uint64_t)a.n[d]) : 0;
      a.lo[d] = 0;
      a.hi[d] = 0;
    }
    a.nterms = nt;
    for (int k = 0; k < nt; ++k) {
      FTerm& t = a.t[k];
      long long lin = 0, stride = 1;
      for (int d = 0; d < 3; ++d) {
        t.o[d] = d < f->ndims ? f->offs[(size_t)k * f->ndims + d] : 0;
        lin += stride * t.o[d];
        stride *= a.n[d];
        a.lo[d] = std::max(a.lo[d], -t.o[d]);
        a.hi[d] = std::max(a.hi[d], t.o[d]);
      }
      t.lin = lin;
      t.kind = f->kind[k];
      t.w = f->w[k];
    }
    dim3 grid((unsigned)((a.n[0] + 127) / 128), (unsigned)std::min<long long>(a.n[1], 65535),
              (unsigned)std::min<long long>(a.n[2], 65535));
    k_filter3<<<grid, 128, 0, f->stream>>>(in, out, a);
  } else {
    FArgsN a{};
    a.ndims = f->ndims;
    a.nterms = nt;
    unsigned long long p = 1;
    for (int d = 0; d < f->ndims; ++d) {
      a.n[d] = f->n[d];
      a.prod[d] = p;
      p *= f->n[d];
      a.r[d] = f->wrap == FDB_WRAP_REFERENCE ? pow2_64_mod(f->n[d]) : 0;
    }
    a.ntot = f->ntot;
    uint64_t blocks = (f->ntot + 255) / 256;
    if (blocks > 152 * 16) blocks = 152 * 16;
    k_filter_nd<<<(unsigned)blocks, 256, 0, f->stream>>>(in, out, a, f->d_offs, f->d_kind,
                                                         f->d_w);
  }
  fdb::note_launch();
  FDB_CUDA_TRY(cudaGetLastError());
  return FDB_OK;
}

}  // namespace

extern "C" {

int fdb_filter_create(int ndims, const uint64_t* dims, const double* xmins, const double* xmaxs,
                      int nterms, const int* offsets, const double* weights, fdb_filter** out) {
  if (!out) return fail(FDB_ERR_INVALID, "null output pointer");
  *out = nullptr;
  if (ndims < 1 || ndims > FDB_MAX_DIMS) return fail(FDB_ERR_INVALID, "ndims must be in [1, 8]");
  if (nterms < 1 || nterms > kMaxTerms) return fail(FDB_ERR_INVALID, "nterms must be in [1, 256]");
  if (!dims || !xmins || !xmaxs || !offsets || !weights)
    return fail(FDB_ERR_INVALID, "null argument");
  fdb_filter* f = new fdb_filter();
  f->ndims = ndims;
  f->ntot = 1;
  for (int d = 0; d < ndims; ++d) {
    if (dims[d] == 0 || dims[d] >= (1ull << 31)) {
      delete f;
      return fail(FDB_ERR_INVALID, "each dimension must be in [1, 2^31)");
    }
    f->n[d] = dims[d];
    f->xmins[d] = xmins[d];
    f->xmaxs[d] = xmaxs[d];
    f->ntot *= dims[d];
  }
  // std::map order: sorted offsets, the first weight of a repeated offset
  std::vector<int> order;
  for (int t = 0; t < nterms; ++t) {
    const int* o = offsets + (size_t)t * ndims;
    bool dup = false;
    for (int k : order)
      if (std::memcmp(offsets + (size_t)k * ndims, o, sizeof(int) * ndims) == 0) dup = true;
    if (dup) continue;
    for (int d = 0; d < ndims; ++d)
      if (o[d] <= -(1 << 30) || o[d] >= (1 << 30)) {
        delete f;
        return fail(FDB_ERR_INVALID, "stencil offsets must be below 2^30 in magnitude");
      }
    order.insert(std::upper_bound(order.begin(), order.end(), t,
                                  [&](int a, int b) {
                                    return lex_less(offsets + (size_t)a * ndims,
                                                    offsets + (size_t)b * ndims, ndims);
                                  }),
                 t);
  }
  for (int t : order) {
    for (int d = 0; d < ndims; ++d) f->offs.push_back(offsets[(size_t)t * ndims + d]);
    const double w = weights[t];
    f->w.push_back(w);
    f->kind.push_back(w == 1.0 ? 1 : (w == -1.0 ? 2 : 0));
  }
  cudaError_t e = cudaStreamCreateWithFlags(&f->own, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete f;
    return fdb::cuda_fail(e, "cudaStreamCreate");
  }
  f->stream = f->own;
  int rc = falloc((void**)&f->buf[0], f->ntot * sizeof(double));
  if (rc == FDB_OK) rc = falloc((void**)&f->buf[1], f->ntot * sizeof(double));
  if (rc == FDB_OK) rc = falloc((void**)&f->part, fdb::reduce_partials(f->ntot) * sizeof(double));
  if (rc == FDB_OK) rc = falloc((void**)&f->dsum, sizeof(double));
  if (rc == FDB_OK) rc = falloc((void**)&f->d_offs, f->offs.size() * sizeof(int));
  if (rc == FDB_OK) rc = falloc((void**)&f->d_kind, f->kind.size() * sizeof(int));
  if (rc == FDB_OK) rc = falloc((void**)&f->d_w, f->w.size() * sizeof(double));
  if (rc == FDB_OK && cudaMallocHost((void**)&f->hsum, sizeof(double)) != cudaSuccess)
    rc = fail(FDB_ERR_ALLOC, "cudaMallocHost failed");
  if (rc == FDB_OK) {
    e = cudaMemcpyAsync(f->d_offs, f->offs.data(), f->offs.size() * sizeof(int),
                        cudaMemcpyHostToDevice, f->stream);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(f->d_kind, f->kind.data(), f->kind.size() * sizeof(int),
                          cudaMemcpyHostToDevice, f->stream);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(f->d_w, f->w.data(), f->w.size() * sizeof(double),
                          cudaMemcpyHostToDevice, f->stream);
    // inData and outData start at zero (std::vector::resize, Filter.cpp:54-55)
    if (e == cudaSuccess) e = cudaMemsetAsync(f->buf[0], 0, f->ntot * sizeof(double), f->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(f->buf[1], 0, f->ntot * sizeof(double), f->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(f->stream);
    if (e != cudaSuccess) rc = fdb::cuda_fail(e, "filter set-up copies");
  }
  if (rc != FDB_OK) {
    fdb_filter_destroy(f);
    return rc;
  }
  *out = f;
  return FDB_OK;
}

int fdb_filter_destroy(fdb_filter* f) {
  if (!f) return FDB_OK;
  if (f->own) cudaStreamSynchronize(f->own);
  if (f->stream && f->stream != f->own) cudaStreamSynchronize(f->stream);
  cudaFree(f->buf[0]);
  cudaFree(f->buf[1]);
  cudaFree(f->part);
  cudaFree(f->dsum);
  cudaFree(f->d_offs);
  cudaFree(f->d_kind);
  cudaFree(f->d_w);
  if (f->hsum) cudaFreeHost(f->hsum);
  if (f->own) cudaStreamDestroy(f->own);
  delete f;
  return FDB_OK;
}

int fdb_filter_set_in_data(fdb_filter* f, const double* src, int is_device) {
  FDB_TRY(check(f));
  if (!src) return fail(FDB_ERR_INVALID, "null source");
  FDB_CUDA_TRY(cudaMemcpyAsync(f->buf[f->cur], src, f->ntot * sizeof(double),
                               is_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                               f->stream));
  if (!is_device) FDB_CUDA_TRY(cudaStreamSynchronize(f->stream));
  return FDB_OK;
}

int fdb_filter_get_data(fdb_filter* f, int which, double* dst, int is_device) {
  FDB_TRY(check(f));
  if (!dst || (which != 0 && which != 1)) return fail(FDB_ERR_INVALID, "bad destination");
  const double* src = f->buf[which == 0 ? f->cur : (f->cur ^ 1)];
  FDB_CUDA_TRY(cudaMemcpyAsync(dst, src, f->ntot * sizeof(double),
                               is_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                               f->stream));
  FDB_CUDA_TRY(cudaStreamSynchronize(f->stream));
  return FDB_OK;
}

int fdb_filter_apply(fdb_filter* f) {
  fdb::NvtxScope nvtx_("fdb.filter.apply");
  FDB_TRY(check(f));
  return launch_apply(f);
}

int fdb_filter_copy_out_to_in(fdb_filter* f) {
  FDB_TRY(check(f));
  FDB_CUDA_TRY(cudaMemcpyAsync(f->buf[f->cur], f->buf[f->cur ^ 1], f->ntot * sizeof(double),
                               cudaMemcpyDeviceToDevice, f->stream));
  return FDB_OK;
}

int fdb_filter_iterate(fdb_filter* f, int iterations) {
  fdb::NvtxScope nvtx_("fdb.filter.iterate");
  FDB_TRY(check(f));
  if (iterations < 0) return fail(FDB_ERR_INVALID, "iterations must be >= 0");
  for (int k = 0; k < iterations; ++k) {
    FDB_TRY(launch_apply(f));
    f->cur ^= 1;  // the output becomes the input ...
  }
  if (iterations > 0) {
    // ... and, as after copyOutToIn, the output holds the same field
    FDB_CUDA_TRY(cudaMemcpyAsync(f->buf[f->cur ^ 1], f->buf[f->cur], f->ntot * sizeof(double),
                                 cudaMemcpyDeviceToDevice, f->stream));
  }
  return FDB_OK;
}

int fdb_filter_checksum(fdb_filter* f, int which, double* out) {
  FDB_TRY(check(f));
  if (!out || (which != 0 && which != 1)) return fail(FDB_ERR_INVALID, "bad checksum request");
  FDB_TRY(fdb::launch_sum(f->buf[which == 0 ? f->cur : (f->cur ^ 1)], f->ntot, f->part, f->dsum,
                          f->stream));
  FDB_CUDA_TRY(cudaMemcpyAsync(f->hsum, f->dsum, sizeof(double), cudaMemcpyDeviceToHost,
                               f->stream));
  FDB_CUDA_TRY(cudaStreamSynchronize(f->stream));
  *out = *f->hsum;
  return FDB_OK;
}

int fdb_filter_set_wrap(fdb_filter* f, int mode) {
  FDB_TRY(check(f));
  if (mode != FDB_WRAP_REFERENCE && mode != FDB_WRAP_PERIODIC)
    return fail(FDB_ERR_INVALID, "unknown wrap mode");
  f->wrap = mode;
  return FDB_OK;
}

int fdb_filter_set_stream(fdb_filter* f, void* cuda_stream) {
  FDB_TRY(check(f));
  FDB_CUDA_TRY(cudaStreamSynchronize(f->stream));
  f->stream = cuda_stream ? (cudaStream_t)cuda_stream : f->own;
  return FDB_OK;
}

int fdb_filter_info(fdb_filter* f, uint64_t* ntot, int* nterms) {
  FDB_TRY(check(f));
  if (ntot) *ntot = f->ntot;
  if (nterms) *nterms = (int)f->w.size();
  return FDB_OK;
}

int fdb_filter_synchronize(fdb_filter* f) {
  FDB_TRY(check(f));
  FDB_CUDA_TRY(cudaStreamSynchronize(f->stream));
  return FDB_OK;
}

}  // extern "C"
