// adjoint.cu -- transposed upwind step (no reference counterpart; it is the
// exact transpose of the step in upwind/cxx/upwind.cxx:64-84).
//
// Forward:  f' = f - sum_j c_j (S_j f - f),  (S_j f)[i] = f[i + up_j e_j].
// Adjoint:  lam[i] = lam'[i] - sum_j c_j (lam'[i - up_j e_j] - lam'[i]).
// Velocity coefficients: dL/dc_j = -<lam', S_j f - f> = -sum_i D_j[i] f[i],
// with D_j[i] = lam'[i - up_j e_j] - lam'[i] (periodic shift invariance), so
// the kernel reuses the differences of the lam update and reads f only at i:
// 24 B per cell (read lam', read f, write lam).
//
// The three partial dot products are reduced per CTA and added to that CTA's
// own slot dpart[3*b + j] every step; CTAs own a fixed set of rows (fixed
// grid of kAdjBlocks), so the accumulation order, and hence the result, is
// deterministic.  launch_adjoint_finish sums the slots in a fixed order.
#include "fdb_internal.h"

namespace fdb {
namespace {

constexpr int kThreads = 256;
constexpr uint32_t kAdjBlocks = 1024;

__device__ __forceinline__ int64_t wrap_dn(int64_t i, int up, int64_t n) {
  int64_t j = i - up;
  if (j < 0) j += n;
  else if (j >= n) j -= n;
  return j;
}

__device__ __forceinline__ double block_sum(double v, double* sh) {
  sh[threadIdx.x] = v;
  __syncthreads();
#pragma unroll
  for (int s = kThreads / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) sh[threadIdx.x] = sh[threadIdx.x] + sh[threadIdx.x + s];
    __syncthreads();
  }
  const double r = sh[0];
  __syncthreads();
  return r;
}

__global__ void __launch_bounds__(kThreads)
k_adjoint3(const double* __restrict__ f, const double* __restrict__ lam,
           double* __restrict__ out, int64_t nz, int64_t ny, int64_t nx, int upz, int upy,
           int upx, Coeffs3 c, double* __restrict__ dpart) {
  __shared__ double sh[kThreads];
  const int64_t nrows = nz * ny;
  double gz = 0.0, gy = 0.0, gx = 0.0;
  for (int64_t row = blockIdx.x; row < nrows; row += gridDim.x) {
    const int64_t z = row / ny;
    const int64_t y = row - z * ny;
    const int64_t zd = wrap_dn(z, upz, nz);
    const int64_t yd = wrap_dn(y, upy, ny);
    const double* __restrict__ lc = lam + row * nx;
    const double* __restrict__ lz = lam + (zd * ny + y) * nx;
    const double* __restrict__ ly = lam + (z * ny + yd) * nx;
    const double* __restrict__ fc = f + row * nx;
    double* __restrict__ lo = out + row * nx;
    for (int64_t x = threadIdx.x; x < nx; x += kThreads) {
      const int64_t xd = wrap_dn(x, upx, nx);
      const double l0 = __ldg(lc + x);
      const double dz = __ldg(lz + x) - l0;
      const double dy = __ldg(ly + x) - l0;
      const double dx = __ldg(lc + xd) - l0;
      const double fv = __ldg(fc + x);
      double t = l0;
      t = t - c.cz * dz;
      t = t - c.cy * dy;
      t = t - c.cx * dx;
      lo[x] = t;
      gz = fma(dz, fv, gz);
      gy = fma(dy, fv, gy);
      gx = fma(dx, fv, gx);
    }
  }
  const double sz = block_sum(gz, sh);
  const double sy = block_sum(gy, sh);
  const double sx = block_sum(gx, sh);
  if (threadIdx.x == 0) {
    dpart[3 * blockIdx.x + 0] -= sz;
    dpart[3 * blockIdx.x + 1] -= sy;
    dpart[3 * blockIdx.x + 2] -= sx;
  }
}

__global__ void __launch_bounds__(kThreads)
k_adjoint_finish(const double* __restrict__ dpart, double* __restrict__ out3) {
  __shared__ double sh[kThreads];
  for (int j = 0; j < 3; ++j) {
    double acc = 0.0;
    for (uint32_t b = threadIdx.x; b < kAdjBlocks; b += kThreads) acc = acc + dpart[3 * b + j];
    const double t = block_sum(acc, sh);
    if (threadIdx.x == 0) out3[j] = t;
  }
}

}  // namespace

uint32_t adjoint_blocks() { return kAdjBlocks; }

int launch_adjoint_step(const Geom& g, const Coeffs3& c, const double* f, const double* lam_in,
                        double* lam_out, double* dpart, cudaStream_t s) {
  if (fault_injected("launch")) return fail(FDB_ERR_INJECTED, "injected launch failure");
  k_adjoint3<<<kAdjBlocks, kThreads, 0, s>>>(f, lam_in, lam_out, g.nz, g.ny, g.nx, g.upz, g.upy,
                                             g.upx, c, dpart);
  note_launch();
  FDB_CUDA_TRY(cudaGetLastError());
  return FDB_OK;
}

int launch_adjoint_finish(const double* dpart, double* d_out3, cudaStream_t s) {
  k_adjoint_finish<<<1, kThreads, 0, s>>>(dpart, d_out3);
  note_launch();
  FDB_CUDA_TRY(cudaGetLastError());
  return FDB_OK;
}

}  // namespace fdb
