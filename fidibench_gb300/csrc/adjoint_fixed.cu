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

constexpr int kAR = 4;   // rows per thread
constexpr int kAW = 16;  // warps per CTA

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

template <int R, int W>
__global__ void __launch_bounds__(32 * W, 2)
k_adjoint_fixed(const int64_t* __restrict__ in, int64_t* __restrict__ out,
                const int64_t* __restrict__ fstate, const int* __restrict__ fscale,
                const FixedArgs a, double* __restrict__ dpart) {
  constexpr int K = 1;
  constexpr int kThreads = 32 * W;
  extern __shared__ __align__(16) int64_t s_dyn[];  // [2 buffers][lam, f][R][threads]
  int64_t(*s_pre)[2][R][kThreads] = reinterpret_cast<int64_t(*)[2][R][kThreads]>(s_dyn);
  __shared__ int64_t s_row[2][W][32];
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
  }
  const int sf = *fscale;

  const int X0 = tile_x * a.tx;
  const int Y0 = tile_y * a.ty;
  const int Z0 = tile_z * a.tz;
  const int lx = fx::wrap_mod(X0 - K + lane, a.nx);
  const int px = a.fx ? a.nx - 1 - lx : lx;
  const bool out_x = (lane >= K) && (X0 + lane - K < a.nx);
  const int ly0 = Y0 - K + warp * R;
  const bool rows_linear = (ly0 >= 0) && (ly0 + R - 1 < a.ny);
  const int rstep = a.fy ? -a.nx : a.nx;
  const int roff0 =
      (a.fy ? a.ny - 1 - fx::wrap_mod(ly0, a.ny) : fx::wrap_mod(ly0, a.ny)) * a.nx + px;
  auto row_off = [&](int r) -> int {
    if (rows_linear) return roff0 + r * rstep;
    const int ly = fx::wrap_mod(ly0 + r, a.ny);
    return (a.fy ? a.ny - 1 - ly : ly) * a.nx + px;
  };
  const int64_t plane_sz = (int64_t)a.ny * a.nx;
  const int nplanes = a.tz + K;
  auto plane_off = [&](int lz) -> int64_t {
    return (int64_t)(a.fz ? a.nz - 1 - lz : lz) * plane_sz;
  };
  unsigned row_mask = 0u;
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const int ry = warp * R + r;
    if (out_x && ry >= K && Y0 + ry - K < a.ny) row_mask |= 1u << r;
  }

  int64_t hist[R];
  int64_t cur[R];
#pragma unroll
  for (int r = 0; r < R; ++r) hist[r] = 0;
  double dacc[3] = {0.0, 0.0, 0.0};
  unsigned long long my_or = 0ull;

  int lz = fx::wrap_mod(Z0 - K, a.nz);
  {
    const int64_t po = plane_off(lz);
#pragma unroll
    for (int r = 0; r < R; ++r) {
      fx::cp_async8(&s_pre[0][0][r][tid], in + po + row_off(r));
      fx::cp_async8(&s_pre[0][1][r][tid], fstate + po + row_off(r));
    }
    fx::cp_async_commit();
  }
  int parity = 0;
  for (int p = 0; p < nplanes; ++p) {
    const int lz_next = (lz + 1 == a.nz) ? 0 : lz + 1;
    if (p + 1 < nplanes) {
      const int64_t po = plane_off(lz_next);
#pragma unroll
      for (int r = 0; r < R; ++r) {
        fx::cp_async8(&s_pre[(p + 1) & 1][0][r][tid], in + po + row_off(r));
        fx::cp_async8(&s_pre[(p + 1) & 1][1][r][tid], fstate + po + row_off(r));
      }
    }
    fx::cp_async_commit();
    fx::cp_async_wait<1>();
#pragma unroll
    for (int r = 0; r < R; ++r) cur[r] = s_pre[p & 1][0][r][tid];
    if (d != 0) {
#pragma unroll
      for (int r = 0; r < R; ++r) cur[r] = d > 0 ? (cur[r] << d) : (cur[r] >> (-d));
    }
    const bool store = (p >= K) && (Z0 + p - K < a.nz);
    s_row[parity][warp][lane] = cur[R - 1];
    __syncthreads();
    const int64_t up0 = (warp > 0) ? s_row[parity][warp - 1][lane] : cur[0];
    parity ^= 1;
    int64_t left[R];
#pragma unroll
    for (int r = 0; r < R; ++r) left[r] = __shfl_up_sync(0xffffffffu, cur[r], 1);
    int64_t pz = 0, py = 0, pxx = 0;
#pragma unroll
    for (int r = R - 1; r >= 0; --r) {
      const int64_t c = cur[r];
      const int64_t upv = (r > 0) ? cur[r - 1] : up0;
      const int64_t Dz = hist[r] - c, Dy = upv - c, Dx = left[r] - c;
      const int64_t nv = fx::update(c, hist[r], upv, left[r], a);
      if (store && (row_mask & (1u << r))) {
        int32_t g1, g0;
        split_balanced(s_pre[p & 1][1][r][tid], &g1, &g0);
        pz += prod64(Dz, g1, g0);
        py += prod64(Dy, g1, g0);
        pxx += prod64(Dx, g1, g0);
      }
      hist[r] = c;
      cur[r] = nv;
    }
    if (store) {
      dacc[0] += (double)pz;
      dacc[1] += (double)py;
      dacc[2] += (double)pxx;
      int64_t* dst = out + plane_off(lz);
#pragma unroll
      for (int r = 0; r < R; ++r) {
        if (row_mask & (1u << r)) {
          const int64_t v = cur[r];
          my_or |= (unsigned long long)(v ^ (v >> 63));
          dst[row_off(r)] = v;
        }
      }
    }
    lz = lz_next;
  }
  fx::cp_async_wait<0>();

  // CTA sums of the three contractions, in units of 2^(64 - s - sf)
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    double v = dacc[j];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) s_red[j][warp] = v;
  }
  fx::cta_or<W>(my_or, s_or, &a.slot_out->m);  // contains __syncthreads
  if (tid == 0) {
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

int adjoint_fixed_ctas(const Geom& g, const Coeffs3& c) {
  const FixedArgs a = make_fixed_args(transposed(g), c, fx::kR4W16, 1, 0, (int64_t)2 * 152);
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
  const int shape = fx::kR4W16;
  const Geom gT = transposed(g);

  // adjoint kernel shape and its dynamic shared memory
  constexpr int smem = 2 * 2 * kAR * 32 * kAW * (int)sizeof(int64_t);
  static bool configured = false;
  if (!configured) {
    cudaFuncSetAttribute(k_adjoint_fixed<kAR, kAW>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         smem);
    configured = true;
  }
  FixedArgs aT = make_fixed_args(gT, c, shape, 1, 0, (int64_t)2 * 152);
  aT.guard = gK;
  aT.err = err;
  aT.scale_log = nullptr;
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
    for (int k = 1; k < len; ++k)
      FDB_TRY(launch_fixed_one(g, c, shape, 1, io.states[k - 1], io.states[k], false, false, fr, k,
                               err, 0, 1, logs + k, st));
    if (io.recompute_ev) {
      cudaEventRecord(e1, st);
      io.recompute_ev->push_back({e0, e1});
    }
    // adjoint steps n = sK+len-1 .. sK
    for (int k = len - 1; k >= 0; --k) {
      aT.slot_in = lr + (li % 3);
      aT.slot_out = lr + ((li + 1) % 3);
      aT.slot_reset = lr + ((li + 2) % 3);
      k_adjoint_fixed<kAR, kAW><<<nblk, 32 * kAW, smem, st>>>(io.lam[lc], io.lam[lc ^ 1],
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
