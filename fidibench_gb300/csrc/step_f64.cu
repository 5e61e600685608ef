// step_f64.cu -- one upwind time step in FP64 (the reference's advect() body,
// upwind/cxx/upwind.cxx:64-84), ping-pong between two device fields instead
// of the reference's copy pass (:59-62).
//
// Two arithmetics share one memory pattern:
//   EXACT  f' = ((f - c_z (f_zu - f)) - c_y (f_yu - f)) - c_x (f_xu - f), every
//          operation separately rounded (__dsub_rn/__dmul_rn, no contraction)
//          in the reference's axis order j = 0..ndims-1: bit-identical to the
//          reference compiled without FMA.  9 FP64 instructions per cell.
//   FMA    f' = w f + a_z f_zu + a_y f_yu + a_x f_xu (a_j = -c_j,
//          w = ((1 - a_z) - a_y) - a_x): 1 DMUL + 3 DFMA per cell.
// On GB300 both are FP64-pipe bound, not HBM bound; the block-fixed-point
// kernel in step_fixed.cu is the bandwidth-class path.
//
// Layout: row-major, x (last reference axis) contiguous.  One CTA walks whole
// x-rows (coalesced), rows are distributed grid-stride; the upstream rows in
// y and z are read through L1/L2 (each row is re-read by two other rows'
// CTAs, which hit L2 because rows are processed in order).
#include "fdb_internal.h"

namespace fdb {
namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ int64_t wrap_up(int64_t i, int up, int64_t n) {
  int64_t j = i + up;
  if (j < 0) j += n;
  else if (j >= n) j -= n;
  return j;
}

template <int ARITH>
__global__ void __launch_bounds__(kThreads)
k_step3(const double* __restrict__ in, double* __restrict__ out, int64_t nz, int64_t ny,
        int64_t nx, int upz, int upy, int upx, Coeffs3 c) {
  const int64_t nrows = nz * ny;
  for (int64_t row = blockIdx.x; row < nrows; row += gridDim.x) {
    const int64_t z = row / ny;
    const int64_t y = row - z * ny;
    const int64_t zu = wrap_up(z, upz, nz);
    const int64_t yu = wrap_up(y, upy, ny);
    const double* __restrict__ rc = in + row * nx;
    const double* __restrict__ rz = in + (zu * ny + y) * nx;
    const double* __restrict__ ry = in + (z * ny + yu) * nx;
    double* __restrict__ ro = out + row * nx;
    for (int64_t x = threadIdx.x; x < nx; x += kThreads) {
      const int64_t xu = wrap_up(x, upx, nx);
      const double o = __ldg(rc + x);
      const double uz = __ldg(rz + x);
      const double uy = __ldg(ry + x);
      const double ux = __ldg(rc + xu);
      double t;
      if (ARITH == FDB_ARITH_EXACT) {
        t = o;
        t = __dsub_rn(t, __dmul_rn(c.cz, __dsub_rn(uz, o)));
        t = __dsub_rn(t, __dmul_rn(c.cy, __dsub_rn(uy, o)));
        t = __dsub_rn(t, __dmul_rn(c.cx, __dsub_rn(ux, o)));
      } else {
        t = fma(c.ax, ux, fma(c.ay, uy, fma(c.az, uz, c.w * o)));
      }
      ro[x] = t;
    }
  }
}

struct GenericArgs {
  int ndims;
  uint64_t n[FDB_MAX_DIMS];
  uint64_t dimProd[FDB_MAX_DIMS];
  int up[FDB_MAX_DIMS];
  double coeff[FDB_MAX_DIMS];
};

// Any number of axes (up to FDB_MAX_DIMS), the reference's own per-cell index
// reconstruction (getIndexSet/getFlatIndex, upwind.cxx:122-134) and EXACT
// arithmetic.  Used for ndims > 3 only.
__global__ void k_step_generic(const double* __restrict__ in, double* __restrict__ out,
                               uint64_t ntot, GenericArgs a) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < ntot;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const double o = in[i];
    double t = o;
    for (int j = 0; j < a.ndims; ++j) {
      const uint64_t ij = (i / a.dimProd[j]) % a.n[j];
      uint64_t iu = ij;
      if (a.up[j] < 0) iu = (ij == 0) ? a.n[j] - 1 : ij - 1;
      else iu = (ij + 1 == a.n[j]) ? 0 : ij + 1;
      const uint64_t upI = i - ij * a.dimProd[j] + iu * a.dimProd[j];
      t = __dsub_rn(t, __dmul_rn(a.coeff[j], __dsub_rn(in[upI], o)));
    }
    out[i] = t;
  }
}

int grid_for_rows(int64_t nrows) {
  const int64_t cap = 152 * 16;
  return (int)(nrows < cap ? nrows : cap);
}

}  // namespace

int launch_step_f64(const Geom& g, const Coeffs3& c, int arith, const double* in, double* out,
                    cudaStream_t s) {
  if (fault_injected("launch")) return fail(FDB_ERR_INJECTED, "injected launch failure");
  const int grid = grid_for_rows(g.nz * g.ny);
  if (arith == FDB_ARITH_EXACT)
    k_step3<FDB_ARITH_EXACT><<<grid, kThreads, 0, s>>>(in, out, g.nz, g.ny, g.nx, g.upz, g.upy,
                                                      g.upx, c);
  else
    k_step3<FDB_ARITH_FMA><<<grid, kThreads, 0, s>>>(in, out, g.nz, g.ny, g.nx, g.upz, g.upy,
                                                    g.upx, c);
  note_launch();
  FDB_CUDA_TRY(cudaGetLastError());
  return FDB_OK;
}

int launch_step_generic(const Geom& g, double dt, const double* in, double* out,
                        cudaStream_t s) {
  if (fault_injected("launch")) return fail(FDB_ERR_INJECTED, "injected launch failure");
  GenericArgs a{};
  a.ndims = g.ndims;
  for (int j = 0; j < g.ndims; ++j) {
    a.n[j] = g.n[j];
    a.dimProd[j] = g.dimProd[j];
    a.up[j] = g.up[j];
    a.coeff[j] = ref_coeff(g, j, dt);
  }
  uint64_t blocks = (g.ntot + 255) / 256;
  if (blocks > 152 * 32) blocks = 152 * 32;
  k_step_generic<<<(unsigned)blocks, 256, 0, s>>>(in, out, g.ntot, a);
  note_launch();
  FDB_CUDA_TRY(cudaGetLastError());
  return FDB_OK;
}

}  // namespace fdb
