// adjoint_fixed.cu -- the transposed upwind step in 64-bit block-fixed-point
// (no reference counterpart; the transpose of upwind/cxx/upwind.cxx:64-84).
//
// Adjoint step n (lam' = lam^{n+1} -> lam = lam^n, f = f^n):
//   lam[i] = lam'[i] + sum_j a_j (lam'[i - up_j e_j] - lam'[i])
//   dL/da_j += sum_i D_j[i] f[i],   D_j = lam'[i - up_j e_j] - lam'[i]
// (a_j = -c_j are the Courant numbers; the second line follows from
// <lam', S_j f - f> and the periodic shift invariance, so f is read only at
// i).  The lam update is the forward fixed-point update with every axis
// flipped, so the kernel reuses its tile geometry, update and scale ring
// (step_fixed.cuh) with one step per launch: 24 B of HBM per cell-step
// (lam in and out, f^n in).  The contraction D_j * F^n is an exact 64x64
// product rounded to 2^64 units (three IMAD.WIDE on balanced 32-bit halves),
// summed per thread in int64 per plane and in FP64 across planes; each CTA
// adds its three sums into its own slot of a per-call array (fixed
// CTA -> tile map, so the result is deterministic).
//
// Forward states f^n of a checkpoint segment are recomputed by the forward
// fixed kernel with one step per launch into int64 buffers; each launch logs
// its output scale on the device, which the adjoint launch for that step
// reads.  Elementwise kernels convert FP64 <-> int64 at the ends.
#include <math.h>

#include <algorithm>
#include <vector>

#include "step_fixed.cuh"

namespace fdb {

using fx::FixedArgs;
using fx::ScaleSlot;

namespace {

constexpr int kAR = 4;  // rows per thread
constexpr int kAW = 8;  // warps per CTA

__device__ __forceinline__ void split_balanced(int64_t v, int32_t* hi, int32_t* lo) {
  const int32_t l = (int32_t)(uint32_t)v;
  *lo = l;
  *hi = (int32_t)((v - (int64_t)l) >> 32);
}

// round(D * F / 2^64) from balanced halves (|D| < 2^62, |F| < 2^61)
__device__ __forceinline__ int64_t prod64(int64_t D, int32_t g1, int32_t g0) {
  int32_t d1, d0;
  split_balanced(D, &d1, &d0);
  int64_t t = fx::mad_s(d1, g0, 0x80000000ll);
  t = fx::mad_s(d0, g1, t);
  return fx::mad_s(d1, g1, t >> 32);
}

// 128-bit accumulator of signed int64 terms
struct Acc128 {
  unsigned long long lo = 0ull;
  long long hi = 0ll;
  __device__ __forceinline__ void add(int64_t v) {
    const unsigned long long nlo = lo + (unsigned long long)v;
    hi += (long long)(nlo < lo) + (v >> 63);
    lo = nlo;
  }
  __device__ __forceinline__ double to_double() const {
    return fma((double)hi, 18446744073709551616.0, (double)lo);
  }
};

// One step per launch.  Every warp is independent: it owns 32 columns x R
// rows of the logical (x, y) plane and marches along z; it loads its own
// y-1 halo row and lane 0 loads the x-1 column, so no barrier is needed and
// every lane computes an output.  The plane z-1 value of each cell is the
// thread's previous-plane register.  Loads of the next plane are issued
// into registers while the current plane is computed.
// DOTS = false gives the plain forward step with the same structure (used to
// recompute the forward states of a segment, one step per launch).
template <int R, int W, bool DOTS>
__global__ void __launch_bounds__(32 * W, 2)
k_adjoint_fixed(const int64_t* __restrict__ in, int64_t* __restrict__ out,
                const int64_t* __restrict__ fstate, const int* __restrict__ fscale,
                const FixedArgs a, double* __restrict__ dpart) {
  __shared__ unsigned long long s_or[W];
  __shared__ double s_red[3][W];

  const int tid = threadIdx.x;
  const int lane = tid & 31;
  const int warp = tid >> 5;
  int bid = blockIdx.x;
  const int tile_x = bid % a.tiles_x;
  bid /= a.tiles_x;
  const int tile_y = bid % a.tiles_y;
  const int tile_z = bid / a.tiles_y;

  int s, d;
  if (!fx::scale_from_slot(a.slot_in, a.guard, &s, &d) && tid == 0) atomicOr(a.err, 1);
  if (blockIdx.x == 0 && tid == 0) {
    a.slot_reset->m = 0ull;
    a.slot_reset->kind = 1;
    a.slot_out->s = s;
    a.slot_out->kind = 1;
    if (a.scale_log) *a.scale_log = s;
  }
  const int sf = DOTS ? *fscale : 0;

  // logical coordinates of this thread's column and rows
  const int gx = tile_x * 32 + lane;
  const bool in_x = gx < a.nx;
  const int lx = gx < a.nx ? gx : a.nx - 1;  // clamp idle lanes onto a valid column
  const int lxm = fx::wrap_mod(lx - 1, a.nx);
  const int px = a.fx ? a.nx - 1 - lx : lx;
  const int pxm = a.fx ? a.nx - 1 - lxm : lxm;
  const int Y0 = tile_y * (R * W) + warp * R;
  auto prow = [&](int ly) {  // physical row offset of logical row ly (wrapped)
    const int w = fx::wrap_mod(ly, a.ny);
    return (a.fy ? a.ny - 1 - w : w) * a.nx;
  };
  int roff[R];
  unsigned row_mask = 0u;
#pragma unroll
  for (int r = 0; r < R; ++r) {
    roff[r] = prow(Y0 + r);
    if (in_x && Y0 + r < a.ny) row_mask |= 1u << r;
  }
  const int rhalo = prow(Y0 - 1);
  const int64_t plane_sz = (int64_t)a.ny * a.nx;
  const int Z0 = tile_z * a.tz;
  const int nz_tile = min(a.tz, a.nz - Z0);
  auto plane_off = [&](int lz) -> int64_t {
    return (int64_t)(a.fz ? a.nz - 1 - lz : lz) * plane_sz;
  };

  // plane values: lam rows, the y-1 halo row, lane 0's x-1 column, f rows
  int64_t cur[R], hist[R], nx_cur[R], nx_f[R], nx_xl[R], fv[R], xl[R];
  int64_t yh, nx_yh;
  int lz = fx::wrap_mod(Z0 - 1, a.nz);
  {
    const int64_t po = plane_off(lz);
#pragma unroll
    for (int r = 0; r < R; ++r) hist[r] = __ldg(in + po + roff[r] + px);
  }
  lz = (lz + 1 == a.nz) ? 0 : lz + 1;
  auto load_plane = [&](int z) {
    const int64_t po = plane_off(z);
#pragma unroll
    for (int r = 0; r < R; ++r) {
      nx_cur[r] = __ldg(in + po + roff[r] + px);
      nx_f[r] = DOTS ? __ldg(fstate + po + roff[r] + px) : 0;
      nx_xl[r] = (lane == 0) ? __ldg(in + po + roff[r] + pxm) : 0;
    }
    nx_yh = __ldg(in + po + rhalo + px);
  };
  if (nz_tile > 0) load_plane(lz);
  if (d != 0) {
#pragma unroll
    for (int r = 0; r < R; ++r) hist[r] = d > 0 ? (hist[r] << d) : (hist[r] >> (-d));
  }

  Acc128 acc[3];
  unsigned long long my_or = 0ull;
  for (int p = 0; p < nz_tile; ++p) {
#pragma unroll
    for (int r = 0; r < R; ++r) {
      cur[r] = nx_cur[r];
      fv[r] = nx_f[r];
      xl[r] = nx_xl[r];
    }
    yh = nx_yh;
    const int lz_next = (lz + 1 == a.nz) ? 0 : lz + 1;
    if (p + 1 < nz_tile) load_plane(lz_next);
    if (d != 0) {
#pragma unroll
      for (int r = 0; r < R; ++r) {
        cur[r] = d > 0 ? (cur[r] << d) : (cur[r] >> (-d));
        xl[r] = d > 0 ? (xl[r] << d) : (xl[r] >> (-d));
      }
      yh = d > 0 ? (yh << d) : (yh >> (-d));
    }
    int64_t pz = 0, py = 0, pxx = 0;
    int64_t* dst = out + plane_off(lz);
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const int64_t c = cur[r];
      int64_t left = __shfl_up_sync(0xffffffffu, c, 1);
      if (lane == 0) left = xl[r];
      const int64_t upv = (r > 0) ? cur[r - 1] : yh;
      const int64_t nv = fx::update(c, hist[r], upv, left, a);
      if (row_mask & (1u << r)) {
        if (DOTS) {
          int32_t g1, g0;
          split_balanced(fv[r], &g1, &g0);
          pz += prod64(hist[r] - c, g1, g0);
          py += prod64(upv - c, g1, g0);
          pxx += prod64(left - c, g1, g0);
        }
        my_or |= (unsigned long long)(nv ^ (nv >> 63));
        dst[roff[r] + px] = nv;
      }
      hist[r] = c;
    }
    acc[0].add(pz);
    acc[1].add(py);
    acc[2].add(pxx);
    lz = lz_next;
  }

  // CTA sums of the three contractions, in units of 2^(64 - s - sf)
  if (DOTS) {
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      double v = acc[j].to_double();
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
      if (lane == 0) s_red[j][warp] = v;
    }
  }
  fx::cta_or<W>(my_or, s_or, &a.slot_out->m);  // contains __syncthreads
  if (DOTS && tid == 0) {
    const double unit = ldexp(1.0, 64 - s - sf);
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      double t = 0.0;
      for (int w = 0; w < W; ++w) t += s_red[j][w];
      dpart[3 * blockIdx.x + j] += t * unit;
    }
  }
}

// f (FP64) -> F (int64) with the scale of a kind-0 slot (max|f| pre-pass);
// writes the output slot (OR of |F|, scale, kind 1), clears the next one and
// logs the scale.
__global__ void __launch_bounds__(256)
k_to_fixed(const double* __restrict__ f, int64_t* __restrict__ F, uint64_t n,
           const ScaleSlot* slot_in, ScaleSlot* slot_out, ScaleSlot* slot_reset, int guard,
           int* scale_log, int* err) {
  __shared__ unsigned long long s_or[8];
  int s, d;
  if (!fx::scale_from_slot(slot_in, guard, &s, &d) && threadIdx.x == 0) atomicOr(err, 1);
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    slot_reset->m = 0ull;
    slot_reset->kind = 1;
    slot_out->s = s;
    slot_out->kind = 1;
    if (scale_log) *scale_log = s;
  }
  unsigned long long my_or = 0ull;
  for (uint64_t i = blockIdx.x * 256ull + threadIdx.x; i < n; i += (uint64_t)gridDim.x * 256ull) {
    const int64_t v = to_fixed(__ldg(f + i), s);
    F[i] = v;
    my_or |= (unsigned long long)(v ^ (v >> 63));
  }
  fx::cta_or<8>(my_or, s_or, &slot_out->m);
}

// F (int64, scale from a kind-1 slot) -> f (FP64)
__global__ void __launch_bounds__(256)
k_to_double(const int64_t* __restrict__ F, double* __restrict__ f, uint64_t n,
            const ScaleSlot* slot) {
  const int s = __ldcg(&slot->s);
  for (uint64_t i = blockIdx.x * 256ull + threadIdx.x; i < n; i += (uint64_t)gridDim.x * 256ull)
    f[i] = to_double(__ldg(F + i), s);
}

// max|f| bit patterns -> slot m (kind 0), other slots cleared
__global__ void __launch_bounds__(256)
k_absmax_slot(const double* __restrict__ f, uint64_t n, ScaleSlot* slots) {
  __shared__ unsigned long long sh[8];
  unsigned long long m = 0ull;
  for (uint64_t i = blockIdx.x * 256ull + threadIdx.x; i < n; i += (uint64_t)gridDim.x * 256ull) {
    const unsigned long long b =
        (unsigned long long)__double_as_longlong(__ldg(f + i)) & 0x7FFFFFFFFFFFFFFFull;
    m = b > m ? b : m;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long v = __shfl_xor_sync(0xffffffffu, m, o);
    m = v > m ? v : m;
  }
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < 8; ++w) m = sh[w] > m ? sh[w] : m;
    atomicMax(&slots[0].m, m);
  }
}

__global__ void k_ring_init(ScaleSlot* slots) {
  if (threadIdx.x < 3) {
    slots[threadIdx.x].m = 0ull;
    slots[threadIdx.x].s = 0;
    slots[threadIdx.x].kind = threadIdx.x == 0 ? 0 : 1;
  }
}

__global__ void __launch_bounds__(256)
k_sum3(const double* __restrict__ dpart, int nblocks, double* __restrict__ out3) {
  __shared__ double sh[256];
  for (int j = 0; j < 3; ++j) {
    double acc = 0.0;
    for (int b = threadIdx.x; b < nblocks; b += 256) acc += dpart[3 * b + j];
    sh[threadIdx.x] = acc;
    __syncthreads();
    for (int st = 128; st > 0; st >>= 1) {
      if (threadIdx.x < st) sh[threadIdx.x] += sh[threadIdx.x + st];
      __syncthreads();
    }
    if (threadIdx.x == 0) out3[j] = sh[0];
    __syncthreads();
  }
}

unsigned grid_for(uint64_t n) {
  uint64_t b = (n + 255) / 256;
  if (b > 152 * 16) b = 152 * 16;
  return (unsigned)std::max<uint64_t>(b, 1);
}

}  // namespace

// Geometry of the transposed step: every upwind direction reversed.
static Geom transposed(const Geom& g) {
  Geom t = g;
  t.upz = -g.upz;
  t.upy = -g.upy;
  t.upx = -g.upx;
  return t;
}

size_t adjoint_fixed_scratch_bytes(int seg_len) {
  return 6 * sizeof(ScaleSlot) + 4 * sizeof(int) + (size_t)(seg_len + 1) * sizeof(int);
}

// Tiling of the warp-independent one-step kernel: 32 columns x (kAR*kAW)
// rows per CTA, tz planes chosen for about four waves of two CTAs per SM.
// transpose = true: the adjoint (every upwind direction reversed).
static FixedArgs step1_args(const Geom& g, const Coeffs3& c, bool transpose) {
  FixedArgs a = make_fixed_args(transpose ? transposed(g) : g, c, fx::kR4W8S, 1, 0,
                                (int64_t)2 * 152);
  a.tx = 32;
  a.ty = kAR * kAW;
  a.tiles_x = (a.nx + a.tx - 1) / a.tx;
  a.tiles_y = (a.ny + a.ty - 1) / a.ty;
  const int64_t txy = (int64_t)a.tiles_x * a.tiles_y;
  const int64_t want = 4 * 2 * 152;
  int64_t cz = (want + txy - 1) / txy;
  if (cz < 1) cz = 1;
  int tz = (int)((a.nz + cz - 1) / cz);
  if (tz < 4) tz = 4;
  if (tz > a.nz) tz = a.nz;
  a.tz = tz;
  a.tiles_z = (a.nz + tz - 1) / tz;
  a.guard = guard_bits(c, 1);
  a.scale_log = nullptr;
  return a;
}

int adjoint_fixed_ctas(const Geom& g, const Coeffs3& c) {
  const FixedArgs a = step1_args(g, c, true);
  return a.tiles_x * a.tiles_y * a.tiles_z;
}

int adjoint_fixed_run(const AdjointFixedIO& io, cudaStream_t st) {
  const Geom& g = *io.g;
  const Coeffs3& c = *io.c;
  const uint64_t n = g.ntot;
  ScaleSlot* fr = (ScaleSlot*)io.scratch;  // forward-recompute ring
  ScaleSlot* lr = fr + 3;                  // adjoint ring
  int* err = (int*)(fr + 6);
  int* logs = err + 4;                      // scale of each recomputed state
  const int gK = guard_bits(c, 1);
  FixedArgs aT = step1_args(g, c, true);
  aT.err = err;
  FixedArgs aF = step1_args(g, c, false);
  aF.err = err;
  const int nblk = aT.tiles_x * aT.tiles_y * aT.tiles_z;
  if (nblk > io.dpart_cap) return fail(FDB_ERR_INVALID, "adjoint partial-sum buffer too small");

  // lam_T -> int64 (adjoint ring, launch index 0)
  FDB_CUDA_TRY(cudaMemsetAsync(io.dpart, 0, 3 * sizeof(double) * nblk, st));
  k_ring_init<<<1, 32, 0, st>>>(lr);
  k_absmax_slot<<<grid_for(n), 256, 0, st>>>(io.lam_T, n, lr);
  k_to_fixed<<<grid_for(n), 256, 0, st>>>(io.lam_T, io.lam[0], n, lr, lr + 1, lr + 2, gK, nullptr,
                                         err);
  note_launch(3);
  int li = 1;  // adjoint ring position of the next launch
  int lc = 0;
  for (int sgi = io.nseg - 1; sgi >= 0; --sgi) {
    const int len = std::min(io.K, io.S - sgi * io.K);
    cudaEvent_t e0 = nullptr, e1 = nullptr, e2 = nullptr;
    if (io.recompute_ev) {
      cudaEventCreate(&e0);
      cudaEventCreate(&e1);
      cudaEventCreate(&e2);
      cudaEventRecord(e0, st);
    }
    // states f^{sK} .. f^{sK+len-1} in int64 (forward ring, launch index 0..len-1)
    k_ring_init<<<1, 32, 0, st>>>(fr);
    k_absmax_slot<<<grid_for(n), 256, 0, st>>>(io.ckpt[sgi], n, fr);
    k_to_fixed<<<grid_for(n), 256, 0, st>>>(io.ckpt[sgi], io.states[0], n, fr, fr + 1, fr + 2, gK,
                                           logs + 0, err);
    note_launch(3);
    for (int k = 1; k < len; ++k) {
      aF.slot_in = fr + (k % 3);
      aF.slot_out = fr + ((k + 1) % 3);
      aF.slot_reset = fr + ((k + 2) % 3);
      aF.scale_log = logs + k;
      k_adjoint_fixed<kAR, kAW, false><<<nblk, 32 * kAW, 0, st>>>(
          io.states[k - 1], io.states[k], nullptr, nullptr, aF, nullptr);
      note_launch();
    }
    FDB_CUDA_TRY(cudaGetLastError());
    if (io.recompute_ev) {
      cudaEventRecord(e1, st);
      io.recompute_ev->push_back({e0, e1});
    }
    // adjoint steps n = sK+len-1 .. sK
    for (int k = len - 1; k >= 0; --k) {
      aT.slot_in = lr + (li % 3);
      aT.slot_out = lr + ((li + 1) % 3);
      aT.slot_reset = lr + ((li + 2) % 3);
      k_adjoint_fixed<kAR, kAW, true><<<nblk, 32 * kAW, 0, st>>>(io.lam[lc], io.lam[lc ^ 1],
                                                               io.states[k], logs + k, aT,
                                                               io.dpart);
      note_launch();
      FDB_CUDA_TRY(cudaGetLastError());
      lc ^= 1;
      ++li;
    }
    if (io.adjoint_ev) {
      cudaEventRecord(e2, st);
      io.adjoint_ev->push_back({e1, e2});
    }
  }
  k_to_double<<<grid_for(n), 256, 0, st>>>(io.lam[lc], io.grad_f0, n, lr + (li % 3));
  k_sum3<<<1, 256, 0, st>>>(io.dpart, nblk, io.dda3);
  note_launch(2);
  FDB_CUDA_TRY(cudaGetLastError());
  return FDB_OK;
}

}  // namespace fdb
