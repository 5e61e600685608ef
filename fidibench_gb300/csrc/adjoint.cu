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
// This per-step contraction serves the step-by-step adjoint.  The default
// (closed) form needs one contraction in all: the step's operators commute on
// the periodic grid, so dL/da_j = S <lam^1, D_j f0> (k_vel_contract below).
//
// The three partial dot products are reduced per CTA and added to that CTA's
// own slot dpart[3*b + j] every step; CTAs own a fixed set of rows (fixed
// grid of kAdjBlocks), so the accumulation order, and hence the result, is
// deterministic.  launch_adjoint_finish sums the slots in a fixed order.
#include <string>
#include <vector>

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

__device__ __forceinline__ int64_t wrap_up(int64_t i, int up, int64_t n) {
  int64_t j = i + up;
  if (j < 0) j += n;
  else if (j >= n) j -= n;
  return j;
}

// The closed-form velocity contraction: part[3 b + k] = the sum over block
// b's rows of lam[i] (f[i + up_k e_k] - f[i]) for the internal axes k = z, y,
// x of block b's instance.  Each instance's rows are dealt round-robin to its
// own blocks; one FMA chain per thread and a fixed-order tree per block, so
// the partials, and their fixed-order sums, do not depend on timing.
struct ContractDev {
  int64_t offset;
  int64_t nz, ny, nx;
  int upz, upy, upx;
  int block0, nblocks;
};

__global__ void __launch_bounds__(kThreads)
k_vel_contract(const double* __restrict__ f, const double* __restrict__ lam,
               const ContractDev* __restrict__ insts, const int* __restrict__ block_inst,
               double* __restrict__ part) {
  __shared__ double sh[kThreads];
  const ContractDev I = insts[block_inst[blockIdx.x]];
  const double* __restrict__ fb = f + I.offset;
  const double* __restrict__ lb = lam + I.offset;
  const int64_t nrows = I.nz * I.ny;
  double gz = 0.0, gy = 0.0, gx = 0.0;
  for (int64_t row = (int64_t)blockIdx.x - I.block0; row < nrows; row += I.nblocks) {
    const int64_t z = row / I.ny;
    const int64_t y = row - z * I.ny;
    const double* __restrict__ fc = fb + row * I.nx;
    const double* __restrict__ fz = fb + (wrap_up(z, I.upz, I.nz) * I.ny + y) * I.nx;
    const double* __restrict__ fy = fb + (z * I.ny + wrap_up(y, I.upy, I.ny)) * I.nx;
    const double* __restrict__ lc = lb + row * I.nx;
    for (int64_t x = threadIdx.x; x < I.nx; x += kThreads) {
      const double f0 = __ldg(fc + x);
      const double l = __ldg(lc + x);
      gz = fma(l, __ldg(fz + x) - f0, gz);
      gy = fma(l, __ldg(fy + x) - f0, gy);
      gx = fma(l, __ldg(fc + wrap_up(x, I.upx, I.nx)) - f0, gx);
    }
  }
  const double sz = block_sum(gz, sh);
  const double sy = block_sum(gy, sh);
  const double sx = block_sum(gx, sh);
  if (threadIdx.x == 0) {
    part[3 * blockIdx.x + 0] = sz;
    part[3 * blockIdx.x + 1] = sy;
    part[3 * blockIdx.x + 2] = sx;
  }
}

// out[3 i + k] = the sum of instance i's block partials of axis k: one CTA
// per (instance, axis), each thread a fixed stride of the blocks, then the
// fixed-order tree of block_sum
__global__ void __launch_bounds__(kThreads)
k_vel_contract_finish(const double* __restrict__ part, const ContractDev* __restrict__ insts,
                      double* __restrict__ out) {
  __shared__ double sh[kThreads];
  const int i = blockIdx.x / 3;
  const int k = blockIdx.x - 3 * i;
  const ContractDev I = insts[i];
  double acc = 0.0;
  for (int b = threadIdx.x; b < I.nblocks; b += kThreads) acc = acc + part[3 * (I.block0 + b) + k];
  const double t = block_sum(acc, sh);
  if (threadIdx.x == 0) out[blockIdx.x] = t;
}

}  // namespace

int launch_vel_contract(int count, const Geom* geoms, const int64_t* offsets, const double* f,
                        const double* lam, double* d_out, DeviceScratch& scratch,
                        cudaStream_t s) {
  if (count <= 0) return FDB_OK;
  std::vector<ContractDev> insts(count);
  std::vector<int> block_inst;
  int total = 0;
  for (int i = 0; i < count; ++i) {
    const Geom& g = geoms[i];
    ContractDev& I = insts[i];
    I.offset = offsets[i];
    I.nz = g.nz;
    I.ny = g.ny;
    I.nx = g.nx;
    I.upz = g.upz;
    I.upy = g.upy;
    I.upx = g.upx;
    // about 16 K cells per block, at least one row each
    const int64_t rows = g.nz * g.ny;
    int64_t nb = ((int64_t)g.ntot + 16383) / 16384;
    if (nb > rows) nb = rows;
    if (nb > 65536) nb = 65536;
    if (nb < 1) nb = 1;
    if ((int64_t)total + nb > 0x7FFFFFFF / 4)
      return fail(FDB_ERR_UNSUPPORTED, "velocity contraction: too many blocks");
    I.block0 = total;
    I.nblocks = (int)nb;
    block_inst.insert(block_inst.end(), (size_t)nb, i);
    total += (int)nb;
  }
  const size_t b_insts = ((count * sizeof(ContractDev)) + 255) / 256 * 256;
  const size_t b_table = ((total * sizeof(int)) + 255) / 256 * 256;
  const size_t need = b_insts + b_table + 3 * (size_t)total * sizeof(double);
  FDB_TRY(scratch.reserve(need));
  char* base = (char*)scratch.ptr;
  ContractDev* d_insts = (ContractDev*)base;
  int* d_table = (int*)(base + b_insts);
  double* d_part = (double*)(base + b_insts + b_table);
  // pageable sources: the copies are staged before cudaMemcpyAsync returns
  FDB_CUDA_TRY(cudaMemcpyAsync(d_insts, insts.data(), count * sizeof(ContractDev),
                               cudaMemcpyHostToDevice, s));
  FDB_CUDA_TRY(cudaMemcpyAsync(d_table, block_inst.data(), total * sizeof(int),
                               cudaMemcpyHostToDevice, s));
  k_vel_contract<<<total, kThreads, 0, s>>>(f, lam, d_insts, d_table, d_part);
  k_vel_contract_finish<<<3 * count, kThreads, 0, s>>>(d_part, d_insts, d_out);
  note_launch(2);
  FDB_CUDA_TRY(cudaGetLastError());
  return FDB_OK;
}

int DeviceScratch::reserve(size_t need) {
  if (need <= bytes) return FDB_OK;
  release();
  if (fault_injected("alloc")) return fail(FDB_ERR_INJECTED, "injected allocation failure");
  cudaError_t e = cudaMalloc(&ptr, need);
  if (e != cudaSuccess) {
    ptr = nullptr;
    cudaGetLastError();
    return fail(FDB_ERR_ALLOC, std::string("cudaMalloc failed: ") + cudaGetErrorString(e));
  }
  bytes = need;
  return FDB_OK;
}

void DeviceScratch::release() {
  if (ptr) cudaFree(ptr);
  ptr = nullptr;
  bytes = 0;
}

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
