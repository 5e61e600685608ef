// reduce.cu -- checksum() and std() of the field (upwind/cxx/upwind.cxx:91-103)
// as deterministic two-level tree sums.
//
// The reference sums sequentially (std::accumulate).  Here the field is cut
// into G = reduce_partials(n) contiguous chunks that depend on n only (not on
// the GPU), each CTA sums its chunk with four interleaved per-thread
// accumulators and a fixed shared-memory tree, and one CTA sums the G
// partials in a fixed order.  The result is bit-reproducible run to run and
// GPU to GPU, and its rounding error (~(n/G/1024 + log2 n) ulp) is far below
// the sequential sum's worst case, so it agrees with the reference to ~1e-15
// relative on fields of mixed sign and much better on non-negative ones.
#include <math.h>

#include "fdb_internal.h"

namespace fdb {
namespace {

constexpr int kThreads = 256;
constexpr uint32_t kMaxPartials = 2048;

__device__ __forceinline__ double block_sum(double v, double* sh) {
  sh[threadIdx.x] = v;
  __syncthreads();
#pragma unroll
  for (int s = kThreads / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) sh[threadIdx.x] = sh[threadIdx.x] + sh[threadIdx.x + s];
    __syncthreads();
  }
  return sh[0];
}

// MODE 0: sum f.  MODE 1: sum (f - mean)^2 with mean = d_mean[0].
template <int MODE>
__global__ void __launch_bounds__(kThreads)
k_partial(const double* __restrict__ f, uint64_t n, uint64_t chunk,
          const double* __restrict__ d_mean, double* __restrict__ part) {
  __shared__ double sh[kThreads];
  const uint64_t lo = (uint64_t)blockIdx.x * chunk;
  uint64_t hi = lo + chunk;
  if (hi > n) hi = n;
  const double mean = (MODE == 1) ? d_mean[0] : 0.0;
  double acc[4] = {0.0, 0.0, 0.0, 0.0};
  uint64_t i = lo + threadIdx.x;
  for (; i + 3 * kThreads < hi; i += 4 * kThreads) {
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      double x = __ldg(f + i + k * kThreads);
      if (MODE == 1) {
        x = x - mean;
        x = x * x;
      }
      acc[k] = acc[k] + x;
    }
  }
  for (int k = 0; i < hi; i += kThreads, ++k) {
    double x = __ldg(f + i);
    if (MODE == 1) {
      x = x - mean;
      x = x * x;
    }
    acc[k & 3] = acc[k & 3] + x;
  }
  const double t = block_sum((acc[0] + acc[1]) + (acc[2] + acc[3]), sh);
  if (threadIdx.x == 0) part[blockIdx.x] = t;
}

// MODE 0: out = sum.  MODE 1: out = sum / n (the mean).  MODE 2: out = sqrt(sum / n).
template <int MODE>
__global__ void __launch_bounds__(kThreads)
k_final(const double* __restrict__ part, uint32_t g, uint64_t n, double* __restrict__ out) {
  __shared__ double sh[kThreads];
  double acc = 0.0;
  for (uint32_t i = threadIdx.x; i < g; i += kThreads) acc = acc + part[i];
  const double t = block_sum(acc, sh);
  if (threadIdx.x == 0) {
    if (MODE == 0) out[0] = t;
    else if (MODE == 1) out[0] = t / (double)n;
    else out[0] = sqrt(t / (double)n);
  }
}

}  // namespace

uint32_t reduce_partials(uint64_t n) {
  uint64_t g = (n + 8191) / 8192;
  if (g < 1) g = 1;
  if (g > kMaxPartials) g = kMaxPartials;
  return (uint32_t)g;
}

static uint64_t chunk_of(uint64_t n, uint32_t g) { return (n + g - 1) / g; }

int launch_sum(const double* f, uint64_t n, double* part, double* d_out, cudaStream_t s) {
  const uint32_t g = reduce_partials(n);
  k_partial<0><<<g, kThreads, 0, s>>>(f, n, chunk_of(n, g), nullptr, part);
  k_final<0><<<1, kThreads, 0, s>>>(part, g, n, d_out);
  note_launch(2);
  FDB_CUDA_TRY(cudaGetLastError());
  return FDB_OK;
}

// std(): mean = sum/n (upwind.cxx:96), then sqrt(sum (f-mean)^2 / n) (:97-102).
int launch_std(const double* f, uint64_t n, double* part, double* d_tmp, double* d_out,
               cudaStream_t s) {
  const uint32_t g = reduce_partials(n);
  k_partial<0><<<g, kThreads, 0, s>>>(f, n, chunk_of(n, g), nullptr, part);
  k_final<1><<<1, kThreads, 0, s>>>(part, g, n, d_tmp);
  k_partial<1><<<g, kThreads, 0, s>>>(f, n, chunk_of(n, g), d_tmp, part);
  k_final<2><<<1, kThreads, 0, s>>>(part, g, n, d_out);
  note_launch(4);
  FDB_CUDA_TRY(cudaGetLastError());
  return FDB_OK;
}

}  // namespace fdb

// ---------------------------------------------------------------------------
// fdb_checksum_noalloc: the checksum reduction for callers that cannot
// allocate device memory.
//
// Some callers must not allocate GPU memory while they run: code that runs
// inside a memory pool or arena that owns all device memory, real-time or
// embedded hosts that forbid allocation after start-up, and callbacks that
// run where cudaMalloc would synchronise the device or fail.  This entry point
// runs the same two kernels as fdb_upwind_checksum (same chunking, so the same
// result bit for bit), but keeps the per-CTA partial sums in the file-scope
// array below instead of memory that a handle allocated.
//
// Limits and sharing: the array holds kNoAllocPartials (2048) doubles, 16 KB,
// which every GPU that loads this library keeps until the process exits.  The
// reduction never needs more than 2048 partials; fields are accepted up to
// FDB_NOALLOC_MAX_VALUES values.  Every call writes every partial it later
// reads, so nothing has to be cleared between calls, but all calls share the
// one array: calls whose kernels overlap on the GPU (on different streams, or
// from different host threads) race and must be serialised by the caller.
// ---------------------------------------------------------------------------
#include <mutex>
#include <string>

namespace {

constexpr uint32_t kNoAllocPartials = 2048;
static_assert(kNoAllocPartials >= fdb::kMaxPartials, "scratch must hold every partial");

static __device__ __align__(256) double g_noalloc_partials[kNoAllocPartials];

constexpr int kNoAllocMaxDevices = 64;
std::mutex g_noalloc_mutex;
double* g_noalloc_ptr[kNoAllocMaxDevices] = {nullptr};

// Device address of g_noalloc_partials on the current device (looked up once
// per device; the host-side symbol is not a device address).
int noalloc_scratch(double** out) {
  int dev = 0;
  FDB_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kNoAllocMaxDevices)
    return fdb::fail(FDB_ERR_UNSUPPORTED, "device ordinal beyond the no-allocation table");
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (!g_noalloc_ptr[dev]) {
    void* p = nullptr;
    FDB_CUDA_TRY(cudaGetSymbolAddress(&p, g_noalloc_partials));
    g_noalloc_ptr[dev] = (double*)p;
  }
  *out = g_noalloc_ptr[dev];
  return FDB_OK;
}

// The kernels dereference d_field and d_sum on the current device: a host
// pointer, or memory of another GPU, would fault there instead of failing
// here.  cudaPointerGetAttributes only reads the driver's records (it
// allocates nothing).
int check_on_current_device(const void* p, const char* what) {
  int dev = 0;
  FDB_CUDA_TRY(cudaGetDevice(&dev));
  cudaPointerAttributes at{};
  const cudaError_t e = cudaPointerGetAttributes(&at, p);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fdb::fail(FDB_ERR_INVALID, std::string("fdb_checksum_noalloc: ") + what +
                                          " is not a pointer the CUDA runtime knows");
  }
  const bool on_device = at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
  if (!on_device || at.device != dev)
    return fdb::fail(FDB_ERR_INVALID, std::string("fdb_checksum_noalloc: ") + what +
                                          " must be device (or managed) memory of the current "
                                          "device");
  return FDB_OK;
}

}  // namespace

extern "C" int fdb_checksum_noalloc(const double* d_field, uint64_t n, double* d_sum,
                                    void* cuda_stream) {
  if (!d_field || !d_sum) return fdb::fail(FDB_ERR_INVALID, "null field or result pointer");
  if (n == 0 || n > FDB_NOALLOC_MAX_VALUES)
    return fdb::fail(FDB_ERR_INVALID,
                     "fdb_checksum_noalloc: n must be in [1, FDB_NOALLOC_MAX_VALUES = 2^34]");
  const uint32_t g = fdb::reduce_partials(n);
  if (g > kNoAllocPartials)
    return fdb::fail(FDB_ERR_INVALID, "fdb_checksum_noalloc: field needs more partial sums "
                                      "than the 2048-entry static scratch holds");
  double* part = nullptr;
  FDB_TRY(noalloc_scratch(&part));
  FDB_TRY(check_on_current_device(d_field, "d_field"));
  FDB_TRY(check_on_current_device(d_sum, "d_sum"));
  return fdb::launch_sum(d_field, n, part, d_sum, (cudaStream_t)cuda_stream);
}
