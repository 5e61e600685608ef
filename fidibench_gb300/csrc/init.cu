// init.cu -- initial fields on the device.
//
//  * corner: f = 0, f[0] = 1, the reference constructor's field
//    (upwind/cxx/upwind.cxx:45-48).
//  * sphere + noise: the synthetic workloads' field (no reference
//    counterpart).  Cell centres x_d = (i_d + 0.5) dx_d, inside when
//    sum_d (x_d - c_d)^2 < r^2 summed in axis order, plus amp * U[0,1) with
//    U from SplitMix64 (Steele, Lea & Flood 2014) at seed + (i+1)*0x9E37...;
//    every operation separately rounded so the field is bit-identical to the
//    host generator.
#include "fdb_internal.h"

namespace fdb {
namespace {

__global__ void k_corner(double* __restrict__ f, uint64_t n) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x)
    f[i] = (i == 0) ? 1.0 : 0.0;
}

struct SphereArgs {
  int ndims;
  uint64_t n[FDB_MAX_DIMS];
  uint64_t dimProd[FDB_MAX_DIMS];
  double dx[FDB_MAX_DIMS];
  double c[FDB_MAX_DIMS];
  double r2;
  double amp;
  uint64_t seed;
};

__device__ __forceinline__ uint64_t splitmix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

__global__ void k_sphere(double* __restrict__ f, uint64_t n, SphereArgs a) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int d = 0; d < a.ndims; ++d) {
      const uint64_t id = (i / a.dimProd[d]) % a.n[d];
      const double x = __dmul_rn(__dadd_rn((double)id, 0.5), a.dx[d]);
      const double e = __dsub_rn(x, a.c[d]);
      s = __dadd_rn(s, __dmul_rn(e, e));
    }
    double val = (s < a.r2) ? 1.0 : 0.0;
    if (a.amp != 0.0) {
      const uint64_t h = splitmix64(a.seed + (i + 1) * 0x9E3779B97F4A7C15ull);
      const double u = __dmul_rn((double)(h >> 11), 1.0 / 9007199254740992.0);
      val = __dadd_rn(val, __dmul_rn(a.amp, u));
    }
    f[i] = val;
  }
}

unsigned blocks_for(uint64_t n) {
  uint64_t b = (n + 255) / 256;
  if (b > 152 * 64) b = 152 * 64;
  if (b < 1) b = 1;
  return (unsigned)b;
}

}  // namespace

int launch_fill_corner(double* f, uint64_t n, cudaStream_t s) {
  k_corner<<<blocks_for(n), 256, 0, s>>>(f, n);
  note_launch();
  FDB_CUDA_TRY(cudaGetLastError());
  return FDB_OK;
}

int launch_sphere_noise(const Geom& g, const double* center, double radius, double amp,
                        uint64_t seed, double* f, cudaStream_t s) {
  SphereArgs a{};
  a.ndims = g.ndims;
  for (int d = 0; d < g.ndims; ++d) {
    a.n[d] = g.n[d];
    a.dimProd[d] = g.dimProd[d];
    a.dx[d] = g.dx[d];
    a.c[d] = center[d];
  }
  a.r2 = radius * radius;
  a.amp = amp;
  a.seed = seed;
  k_sphere<<<blocks_for(g.ntot), 256, 0, s>>>(f, g.ntot, a);
  note_launch();
  FDB_CUDA_TRY(cudaGetLastError());
  return FDB_OK;
}

}  // namespace fdb
