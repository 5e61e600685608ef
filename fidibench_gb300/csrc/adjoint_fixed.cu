// adjoint_fixed.cu -- the transposed upwind step in 64-bit block-fixed-point
// (no reference counterpart; the transpose of upwind/cxx/upwind.cxx:64-84).
//
// Adjoint step n (lam' = lam^{n+1} -> lam = lam^n, f = f^n):
//   lam[i] = lam'[i] + sum_j a_j (lam'[i - up_j e_j] - lam'[i])
//   dL/da_j += sum_i D_j[i] f[i],   D_j = lam'[i - up_j e_j] - lam'[i]
// (a_j = -c_j are the Courant numbers; the second line follows from
// <lam', S_j f - f> and the periodic shift invariance, so f is read only at
// i).  The lam update is the forward fixed-point update with every axis
// flipped, so the kernel reuses its update and scale ring (step_fixed.cuh)
// with one step per launch: 20 B of HBM per cell-step (lam in and out, f^n
// in as int32), the differences D_j shared between the update and the
// contraction.  The contraction takes F^n in 2^29 units (G, int32,
// 2^-30 of the 2^59 range) and D_j whole: D_j * G / 2^32 from the update's
// own split of D (high word times G by IMAD.WIDE, low word by IMAD.HI),
// summed per thread in int64 over four planes and in a 128-bit integer
// across planes; each CTA adds its three sums into its own slot of a
// per-call array (fixed CTA -> tile map, so the result is deterministic).
//
// Forward states f^n of a checkpoint segment are recomputed by the
// temporally blocked forward kernel (step_fixed.cuh, several steps per
// launch), which also stores every level of its output cells in 2^29 units
// (int32, one array per step of the segment); the int64 chain goes through
// two ping-pong buffers.  Each launch logs the scale of its levels on the
// device, which the adjoint launch for that step reads.  The batched adjoint
// recomputes with the tile kernel below without the transpose and the
// contraction, one step per launch over all instances.  Elementwise kernels
// convert FP64 <-> int64 at the ends.
#include <math.h>

#include <algorithm>
#include <type_traits>
#include <vector>

#include "step_fixed.cuh"

namespace fdb {

using fx::FixedArgs;
using fx::kGShift;
using fx::ScaleSlot;
using fx::state_g;

namespace {

constexpr int kAR = 4;  // rows per thread
constexpr int kAW = 8;  // warps per CTA
constexpr int kAMinBlocks = 3;  // resident CTAs per SM the registers are sized for

// floor(a * b / 2^32) (one IMAD.HI)
__device__ __forceinline__ int32_t mulhi_s(int32_t a, int32_t b) {
  int32_t d;
  asm("mul.hi.s32 %0, %1, %2;" : "=r"(d) : "r"(a), "r"(b));
  return d;
}

// One contraction term D G / 2^32 = D F / 2^(32 + kGShift), from D's high
// word d1 and low word d0 (D = d1 2^32 + d0, the split the update uses):
// d1 G (exact, |.| <= 2^58) into p, and floor((d0 >> 1) G / 2^32) (within
// 1 of d0 G / 2^33, |.| <= 2^29) into q, which the caller adds to p as 2 q
// after at most four terms (|q| <= 2^31 still fits int32).  D = 0 adds 0.
__device__ __forceinline__ void dot_term(int64_t D, int32_t G, int64_t& p, int32_t& q) {
  p += mulw_s((int32_t)(D >> 32), G);
  q += mulhi_s((int32_t)((uint32_t)D >> 1), G);
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
  __device__ __forceinline__ void add(const Acc128& o) {
    const unsigned long long nlo = lo + o.lo;
    hi += o.hi + (long long)(nlo < lo);
    lo = nlo;
  }
  // sum over the warp (integer shuffles), valid in every lane
  __device__ __forceinline__ void warp_sum() {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      Acc128 t;
      t.lo = __shfl_xor_sync(0xffffffffu, lo, o);
      t.hi = __shfl_xor_sync(0xffffffffu, hi, o);
      add(t);
    }
  }
  __device__ __forceinline__ double to_double() const {
    return fma((double)hi, 18446744073709551616.0, (double)lo);
  }
};

// 2^e as a double from its bit pattern (0 below the normal range)
__device__ __forceinline__ double pow2(int e) {
  if (e < -1022) return 0.0;
  if (e > 1023) e = 1024;  // infinity
  return __longlong_as_double((long long)(e + 1023) << 52);
}

// One step per launch, one 32 x 32 (x, y) tile per CTA marching along z.
// Each plane of the input is staged by cp.async into shared memory with its
// upstream halo (row 0 = the y-1 row, column 0 = the x-1 column), so every
// neighbour of a cell is one shared-memory load: no shuffles, no selects,
// one __syncthreads per plane.  kAhead planes are in flight while one is
// computed, so kNL = kAhead + 2 input planes rotate (z-1, z and the ones
// being fetched); the forward state F^n (DOTS, int32 in 2^29 units) is
// staged the same way in kNF = kAhead + 1 buffers.  Without DOTS (the
// batched adjoint's forward recompute) each output value is also stored in
// 2^29 units in out_hi, the form the contraction reads.
// Thread (warp w, lane l) owns cells (x = l, y = w*R + r) of the tile.
constexpr int kAhead = 2;
constexpr int kNL = kAhead + 2;
constexpr int kNF = kAhead + 1;
template <int R, int W, bool DOTS>
struct AdjTileSmem {
  static constexpr int kRows = R * W;              // tile rows (32)
  static constexpr int kLRow = 33;                 // halo column + 32 cells
  static constexpr int kLPlane = (kRows + 1) * kLRow;
  static constexpr int kFPlane = kRows * 32;
  static constexpr int bytes() { return kNL * kLPlane * 8 + (DOTS ? kNF * kFPlane * 4 : 0); }
};

// The tile step of one field: CTA number bid of its grid (tiles x fastest,
// then y, then z-slabs), the scale ring slots of this launch (the lead CTA
// advances the ring and logs the output scale), sf the scale of the state in
// fstate, and dslot this CTA's three partial sums (DOTS).
template <int R, int W, bool DOTS>
__device__ __forceinline__ void adjoint_tile(
    const int64_t* __restrict__ in, int64_t* __restrict__ out, int32_t* __restrict__ out_hi,
    const int32_t* __restrict__ fstate, int sf, const FixedArgs& a, int bid,
    const ScaleSlot* slot_in, ScaleSlot* slot_out, ScaleSlot* slot_reset, int* scale_log,
    int* err, bool lead, double* __restrict__ dslot) {
  using SM = AdjTileSmem<R, W, DOTS>;
  static_assert(SM::kRows == 32, "the halo column is loaded by one warp");
  extern __shared__ __align__(16) int64_t s_dyn[];
  __shared__ unsigned long long s_or[W];
  __shared__ unsigned long long s_red_lo[3][W];
  __shared__ long long s_red_hi[3][W];
  int64_t* sL = s_dyn;                                  // [kNL][kRows + 1][33]
  int32_t* sF = (int32_t*)(s_dyn + kNL * SM::kLPlane);  // [kNF][kRows][32]

  const int tid = threadIdx.x;
  const int lane = tid & 31;
  const int warp = tid >> 5;
  const int tile_x = bid % a.tiles_x;
  bid /= a.tiles_x;
  const int tile_y = bid % a.tiles_y;
  const int tile_z = bid / a.tiles_y;

  // coefficients held in registers (a may live in global memory, which the
  // stores below could alias as far as the compiler knows)
  const QCoeff qz = a.qz, qy = a.qy, qx = a.qx;
  int s, d;
  if (!fx::scale_from_slot(slot_in, a.guard, &s, &d) && tid == 0) atomicOr(err, 1);
  if (lead && tid == 0) {
    slot_reset->m = 0ull;
    slot_reset->kind = 1;
    slot_out->s = s;
    slot_out->kind = 1;
    if (scale_log) *scale_log = s;
  }

  // logical -> physical column and row offsets (periodic wrap, axis flips)
  const int gx = tile_x * 32 + lane;
  const bool in_x = gx < a.nx;
  const int lx = in_x ? gx : a.nx - 1;  // idle lanes read a valid column
  const int px = a.fx ? a.nx - 1 - lx : lx;
  const int lxm = fx::wrap_mod(tile_x * 32 - 1, a.nx);
  const int pxm = a.fx ? a.nx - 1 - lxm : lxm;
  const int Y0 = tile_y * SM::kRows;
  auto prow = [&](int ly) {
    const int w = fx::wrap_mod(ly, a.ny);
    return (a.fy ? a.ny - 1 - w : w) * a.nx;
  };
  int roff[R];
  unsigned row_mask = 0u;
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const int ly = Y0 + warp * R + r;
    roff[r] = prow(ly);
    if (in_x && ly < a.ny) row_mask |= 1u << r;
  }
  // warp 0 also fetches the y-1 row (its lanes' columns) and the x-1 column
  // (lane l: tile row l)
  const int rhalo = prow(Y0 - 1) + px;
  const int chalo = prow(Y0 + lane) + pxm;
  const int64_t plane_sz = (int64_t)a.ny * a.nx;
  const int Z0 = tile_z * a.tz;
  const int nz_tile = min(a.tz, a.nz - Z0);
  auto plane_off = [&](int lz) -> int64_t {
    return (int64_t)(a.fz ? a.nz - 1 - lz : lz) * plane_sz;
  };
  auto lam_at = [&](int buf, int row, int col) -> int64_t* {
    return sL + buf * SM::kLPlane + row * SM::kLRow + col;
  };

  // this thread's cells in lambda buffer 0 (row 1 + warp*R, column 1 + lane)
  // and in F buffer 0, and its in-plane element offsets (ny * nx < 2^31)
  int64_t* const myl = sL + (1 + warp * R) * SM::kLRow + 1 + lane;
  int32_t* const myf = sF + warp * R * 32 + lane;
  int gofs[R];
#pragma unroll
  for (int r = 0; r < R; ++r) gofs[r] = roff[r] + px;
  // fetch a plane (physical offset po) into lambda buffer b and, with_f, its
  // state into F buffer fb
  auto fetch = [&](int b, int64_t po, bool with_f, int fb) {
    const int64_t* pin = in + po;
    int64_t* l = myl + b * SM::kLPlane;
#pragma unroll
    for (int r = 0; r < R; ++r) fx::cp_async8(l + r * SM::kLRow, pin + gofs[r]);
    if (warp == 0) {
      fx::cp_async8(lam_at(b, 0, 1 + lane), pin + rhalo);
      fx::cp_async8(lam_at(b, 1 + lane, 0), pin + chalo);
    }
    if (DOTS && with_f) {
      const int32_t* pf = fstate + po;
      int32_t* f = myf + fb * SM::kFPlane;
#pragma unroll
      for (int r = 0; r < R; ++r) fx::cp_async4(f + r * 32, pf + gofs[r]);
    }
    fx::cp_async_commit();
  };
  // bring this thread's copies in lambda buffer b to the launch scale
  auto rescale = [&](int b) {
    auto sh = [&](int64_t* p) { *p = d > 0 ? (*p << d) : (*p >> (-d)); };
#pragma unroll
    for (int r = 0; r < R; ++r) sh(lam_at(b, 1 + warp * R + r, 1 + lane));
    if (warp == 0) {
      sh(lam_at(b, 0, 1 + lane));
      sh(lam_at(b, 1 + lane, 0));
    }
  };

  // dot_term: per plane at most R = 4 terms in q; per 4 planes 16 terms
  // (|.| <= 2^58) and 4 folds (|2 q| <= 2^32) in the int64 sums before they
  // go into the 128-bit ones.
  static_assert(R <= 4, "q holds at most four terms");
  Acc128 acc[3];
  int64_t part[3] = {0, 0, 0};
  unsigned long long my_or = 0ull;
  // one plane: lambda buffers b (z) and bm (z-1), f buffer fb, output at po
  auto compute = [&](auto full_tag, int b, int bm, int fb, int64_t po) {
    constexpr bool kFull = decltype(full_tag)::value;
    int64_t* dst = out + po;
    int32_t* dst_hi = DOTS ? nullptr : out_hi + po;
    const int64_t* l = myl + b * SM::kLPlane;
    const int64_t* lm = myl + bm * SM::kLPlane;
    int32_t q[3] = {0, 0, 0};
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const int64_t c = l[r * SM::kLRow];
      const int64_t Dz = lm[r * SM::kLRow] - c;
      const int64_t Dy = l[r * SM::kLRow - SM::kLRow] - c;
      const int64_t Dx = l[r * SM::kLRow - 1] - c;
      const int64_t nv = fixed_update_d(c, Dz, Dy, Dx, qz, qy, qx);
      if (kFull || (row_mask & (1u << r))) {
        if (DOTS) {
          const int32_t G = myf[fb * SM::kFPlane + r * 32];
          dot_term(Dz, G, part[0], q[0]);
          dot_term(Dy, G, part[1], q[1]);
          dot_term(Dx, G, part[2], q[2]);
        } else {
          dst_hi[gofs[r]] = state_g(nv);
        }
        my_or |= (unsigned long long)(nv ^ (nv >> 63));
        dst[gofs[r]] = nv;
      }
    }
    if (DOTS) {
#pragma unroll
      for (int k = 0; k < 3; ++k) part[k] += 2 * (int64_t)q[k];
    }
  };
  // the tile lies inside the grid: every thread stores all R rows
  const bool full = (tile_x + 1) * 32 <= a.nx && Y0 + SM::kRows <= a.ny;
  const int64_t dz = a.fz ? -plane_sz : plane_sz;
  const int64_t wrap_po = a.fz ? (int64_t)(a.nz - 1) * plane_sz : 0;

  // plane j (j = 0: z = Z0 - 1, the z-1 history of the first output plane)
  // goes to lambda buffer j % kNL and its state to F buffer j % kNF; planes
  // j + 1 .. j + kAhead are in flight while plane j is computed.  Every
  // iteration commits one cp.async group (empty past the last plane), so
  // waiting for all but the kAhead - 1 newest groups completes plane j.
  auto advance = [&](int& lz, int64_t& po) {
    const bool wraps = lz + 1 == a.nz;
    lz = wraps ? 0 : lz + 1;
    po = wraps ? wrap_po : po + dz;
  };
  int lz = fx::wrap_mod(Z0 - 1, a.nz);  // plane j
  int64_t po = plane_off(lz);
  int lz_f = lz;  // the next plane to fetch
  int64_t po_f = po;
#pragma unroll
  for (int k = 0; k < kAhead; ++k) {
    if (k <= nz_tile) fetch(k, po_f, k > 0, k % kNF);
    else fx::cp_async_commit();
    advance(lz_f, po_f);
  }
  int b = 0, fb = 0;  // buffers of plane j
  for (int j = 0; j <= nz_tile; ++j) {
    fx::cp_async_wait<kAhead - 1>();
    if (d != 0) rescale(b);
    __syncthreads();
    // the buffers of plane j + kAhead held plane j + kAhead - kNL (lambda)
    // and j + kAhead - kNF (F), last read in iteration j - 1
    const int bf = b + kAhead >= kNL ? b + kAhead - kNL : b + kAhead;
    const int fbf = fb + kAhead >= kNF ? fb + kAhead - kNF : fb + kAhead;
    if (j + kAhead <= nz_tile) fetch(bf, po_f, true, fbf);
    else fx::cp_async_commit();
    advance(lz_f, po_f);
    if (j > 0) {
      const int bm = b == 0 ? kNL - 1 : b - 1;
      if (full)
        compute(std::true_type{}, b, bm, fb, po);
      else
        compute(std::false_type{}, b, bm, fb, po);
      if (DOTS && (j & 3) == 0) {
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          acc[k].add(part[k]);
          part[k] = 0;
        }
      }
    }
    b = b + 1 == kNL ? 0 : b + 1;
    fb = fb + 1 == kNF ? 0 : fb + 1;
    advance(lz, po);
  }
  if (DOTS) {
#pragma unroll
    for (int k = 0; k < 3; ++k) acc[k].add(part[k]);
  }

  // CTA sums of the three contractions (exact integers in units of
  // 2^(32 + kGShift - s - sf)); one FP64 conversion per sum and CTA
  if (DOTS) {
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      acc[j].warp_sum();
      if (lane == 0) {
        s_red_lo[j][warp] = acc[j].lo;
        s_red_hi[j][warp] = acc[j].hi;
      }
    }
  }
  fx::cta_or<W>(my_or, s_or, &slot_out->m);  // contains __syncthreads
  if (DOTS && tid < 3) {
    Acc128 t;
    for (int w = 0; w < W; ++w) {
      Acc128 u;
      u.lo = s_red_lo[tid][w];
      u.hi = s_red_hi[tid][w];
      t.add(u);
    }
    dslot[tid] += t.to_double() * pow2(32 + kGShift - s - sf);
  }
}

// One field: the ring slots come with the launch arguments.
template <int R, int W, bool DOTS>
__global__ void __launch_bounds__(32 * W, kAMinBlocks)
k_adjoint_tile(const int64_t* __restrict__ in, int64_t* __restrict__ out,
               int32_t* __restrict__ out_hi, const int32_t* __restrict__ fstate,
               const int* __restrict__ fscale, const FixedArgs a, double* __restrict__ dpart) {
  adjoint_tile<R, W, DOTS>(in, out, out_hi, fstate, DOTS ? *fscale : 0, a, blockIdx.x, a.slot_in,
                           a.slot_out, a.slot_reset, a.scale_log, a.err, blockIdx.x == 0,
                           DOTS ? dpart + 3 * blockIdx.x : nullptr);
}

// Many fields in one launch (the batched adjoint): CTA b works on instance
// cta_inst[b], whose CTAs start at insts[i].cta_base; every instance has its
// own scale ring (position ring_pos of this launch), its own scale log and
// its own place in the buffers.  All instances take the same step.
struct AdjInst {
  FixedArgs a;       // geometry, tiling, coefficients, guard (slot fields unused)
  int64_t offset;    // first cell in the buffers
  ScaleSlot* ring;   // 3 slots
  int* logs;         // scale of each state of the segment
  int cta_base;
};

template <int R, int W, bool DOTS>
__global__ void __launch_bounds__(32 * W, kAMinBlocks)
k_adjoint_tile_multi(const AdjInst* __restrict__ insts, const int* __restrict__ cta_inst,
                     const int64_t* __restrict__ in, int64_t* __restrict__ out,
                     int32_t* __restrict__ out_hi, const int32_t* __restrict__ fstate,
                     int ring_pos, int log_out, int log_f, int* err,
                     double* __restrict__ dpart) {
  const AdjInst& I = insts[cta_inst[blockIdx.x]];
  const int bid = blockIdx.x - I.cta_base;
  ScaleSlot* r = I.ring;
  adjoint_tile<R, W, DOTS>(in + I.offset, out + I.offset,
                           DOTS ? nullptr : out_hi + I.offset,
                           DOTS ? fstate + I.offset : nullptr, DOTS ? I.logs[log_f] : 0, I.a,
                           bid, r + ring_pos % 3, r + (ring_pos + 1) % 3, r + (ring_pos + 2) % 3,
                           log_out >= 0 ? I.logs + log_out : nullptr, err, bid == 0,
                           DOTS ? dpart + 3 * blockIdx.x : nullptr);
}

// f (FP64) -> F (int64) with the scale of a kind-0 slot (max|f| pre-pass);
// writes the output slot (OR of |F|, scale, kind 1), clears the next one and
// logs the scale.  F_hi (nullable) receives F in 2^29 units.
__global__ void __launch_bounds__(256)
k_to_fixed(const double* __restrict__ f, int64_t* __restrict__ F, int32_t* __restrict__ F_hi,
           uint64_t n, const ScaleSlot* slot_in, ScaleSlot* slot_out, ScaleSlot* slot_reset,
           int guard, int* scale_log, int* err) {
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
    if (F_hi) F_hi[i] = state_g(v);
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

// ---- per-instance elementwise kernels of the batched adjoint ---------------
// Block b works on part (b % per_inst) of instance b / per_inst; instance i
// has cells [offs[i], offs[i] + sizes[i]) and the scale ring rings[3i..3i+2].
constexpr int kPerInst = 16;

__global__ void k_ring_init_multi(ScaleSlot* rings, int count) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < 3 * count; k += gridDim.x * blockDim.x) {
    rings[k].m = 0ull;
    rings[k].s = 0;
    rings[k].kind = (k % 3 == 0) ? 0 : 1;
  }
}

// max|f| bit patterns of each instance into slot 0 of its ring (kind 0)
__global__ void __launch_bounds__(256)
k_absmax_multi(const double* __restrict__ f, const int64_t* __restrict__ offs,
               const uint64_t* __restrict__ sizes, ScaleSlot* rings) {
  __shared__ unsigned long long sh[8];
  const int i = blockIdx.x / kPerInst;
  const int part = blockIdx.x - i * kPerInst;
  const double* fi = f + offs[i];
  const uint64_t n = sizes[i];
  unsigned long long m = 0ull;
  for (uint64_t k = (uint64_t)part * 256 + threadIdx.x; k < n; k += (uint64_t)kPerInst * 256) {
    const unsigned long long b =
        (unsigned long long)__double_as_longlong(__ldg(fi + k)) & 0x7FFFFFFFFFFFFFFFull;
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
    atomicMax(&rings[3 * i].m, m);
  }
}

// f (FP64) -> F (int64) per instance, ring position 0 (slot 0 kind 0 in,
// slot 1 out, slot 2 cleared); F_hi (nullable) receives F in 2^29 units and
// logs (nullable) the scale, at logs[i * log_stride].
__global__ void __launch_bounds__(256)
k_to_fixed_multi(const double* __restrict__ f, int64_t* __restrict__ F,
                 int32_t* __restrict__ F_hi, const int64_t* __restrict__ offs,
                 const uint64_t* __restrict__ sizes, ScaleSlot* rings,
                 const int* __restrict__ guards, int* logs, int log_stride, int* err) {
  __shared__ unsigned long long s_or[8];
  const int i = blockIdx.x / kPerInst;
  const int part = blockIdx.x - i * kPerInst;
  ScaleSlot* r = rings + 3 * i;
  int s, d;
  if (!fx::scale_from_slot(r, guards[i], &s, &d) && threadIdx.x == 0) atomicOr(err, 1);
  if (part == 0 && threadIdx.x == 0) {
    r[2].m = 0ull;
    r[2].kind = 1;
    r[1].s = s;
    r[1].kind = 1;
    if (logs) logs[i * log_stride] = s;
  }
  const int64_t o = offs[i];
  const uint64_t n = sizes[i];
  unsigned long long my_or = 0ull;
  for (uint64_t k = (uint64_t)part * 256 + threadIdx.x; k < n; k += (uint64_t)kPerInst * 256) {
    const int64_t v = to_fixed(__ldg(f + o + k), s);
    F[o + k] = v;
    if (F_hi) F_hi[o + k] = state_g(v);
    my_or |= (unsigned long long)(v ^ (v >> 63));
  }
  fx::cta_or<8>(my_or, s_or, &r[1].m);
}

// F (int64, scale from ring slot ring_pos % 3) -> f (FP64) per instance
__global__ void __launch_bounds__(256)
k_to_double_multi(const int64_t* __restrict__ F, double* __restrict__ f,
                  const int64_t* __restrict__ offs, const uint64_t* __restrict__ sizes,
                  const ScaleSlot* rings, int ring_pos) {
  const int i = blockIdx.x / kPerInst;
  const int part = blockIdx.x - i * kPerInst;
  const int s = __ldcg(&rings[3 * i + ring_pos % 3].s);
  const int64_t o = offs[i];
  const uint64_t n = sizes[i];
  for (uint64_t k = (uint64_t)part * 256 + threadIdx.x; k < n; k += (uint64_t)kPerInst * 256)
    f[o + k] = to_double(__ldg(F + o + k), s);
}

// per-instance sums of the CTA partials: block i adds CTAs
// [cta_base[i], cta_base[i+1]) in a fixed order
__global__ void __launch_bounds__(256)
k_sum3_multi(const double* __restrict__ dpart, const int* __restrict__ cta_base,
             double* __restrict__ out3) {
  __shared__ double sh[256];
  const int i = blockIdx.x;
  const int b0 = cta_base[i], b1 = cta_base[i + 1];
  for (int j = 0; j < 3; ++j) {
    double acc = 0.0;
    for (int b = b0 + threadIdx.x; b < b1; b += 256) acc += dpart[3 * b + j];
    sh[threadIdx.x] = acc;
    __syncthreads();
    for (int st = 128; st > 0; st >>= 1) {
      if (threadIdx.x < st) sh[threadIdx.x] += sh[threadIdx.x + st];
      __syncthreads();
    }
    if (threadIdx.x == 0) out3[3 * i + j] = sh[0];
    __syncthreads();
  }
}

}  // namespace

Geom transposed_geom(const Geom& g) {
  Geom t = g;
  t.upz = -g.upz;
  t.upy = -g.upy;
  t.upx = -g.upx;
  return t;
}

size_t adjoint_fixed_scratch_bytes(int seg_len) {
  return 6 * sizeof(ScaleSlot) + 4 * sizeof(int) + (size_t)(seg_len + 1) * sizeof(int);
}

// Dynamic shared memory above the 48 KB default needs an opt-in per kernel
// (and device): set it for both forms before any launch.
static int set_smem_limits() {
  FDB_CUDA_TRY(cudaFuncSetAttribute(k_adjoint_tile<kAR, kAW, true>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    AdjTileSmem<kAR, kAW, true>::bytes()));
  return FDB_OK;
}

// CTAs of the one-step kernel that fit on the current GPU at once.
static int64_t step1_resident() {
  static int per_sm = -1;  // benign race (idempotent)
  if (per_sm < 0) {
    int occ = 0;
    set_smem_limits();
    const cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &occ, k_adjoint_tile<kAR, kAW, true>, 32 * kAW, AdjTileSmem<kAR, kAW, true>::bytes());
    per_sm = (e != cudaSuccess || occ < 1) ? 1 : occ;
  }
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return (int64_t)per_sm * (sms > 0 ? sms : 1);
}

// Tiling of the one-step kernel: 32 columns x (kAR*kAW) rows per CTA and as
// many z-slabs as fill one wave of resident CTAs (long z-runs amortise each
// CTA's set-up, warm-up planes and final reduction; one wave has no partial
// last wave), at least 4 planes each.  transpose = true: the adjoint (every
// upwind direction reversed).
static FixedArgs step1_args(const Geom& g, const Coeffs3& c, bool transpose) {
  FixedArgs a = make_fixed_args(transpose ? transposed_geom(g) : g, c, fx::kR4W8S, 1, 0,
                                (int64_t)2 * 152);
  a.tx = 32;
  a.ty = kAR * kAW;
  a.tiles_x = (a.nx + a.tx - 1) / a.tx;
  a.tiles_y = (a.ny + a.ty - 1) / a.ty;
  const int64_t txy = (int64_t)a.tiles_x * a.tiles_y;
  int64_t cz = step1_resident() / txy;
  if (cz > (a.nz + 3) / 4) cz = (a.nz + 3) / 4;
  if (cz < 1) cz = 1;
  int tz = (int)((a.nz + cz - 1) / cz);
  if (tz > a.nz) tz = a.nz;
  a.tz = tz;
  a.tiles_z = (a.nz + tz - 1) / tz;
  a.guard = guard_bits(c, 1);
  a.scale_log = nullptr;
  return a;
}

static int grid_of(const FixedArgs& a) { return a.tiles_x * a.tiles_y * a.tiles_z; }

int adjoint_fixed_ctas(const Geom& g, const Coeffs3& c) {
  return grid_of(step1_args(g, c, true));
}

int adjoint_fixed_run(const AdjointFixedIO& io, cudaStream_t st) {
  FDB_TRY(set_smem_limits());
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
  const int nblk = grid_of(aT);
  // steps per recompute launch: the forward kernel's own choice for g
  const int kRec = default_depth(g);
  if (nblk > io.dpart_cap) return fail(FDB_ERR_INVALID, "adjoint partial-sum buffer too small");

  // lam_T -> int64 (adjoint ring, launch index 0)
  FDB_CUDA_TRY(cudaMemsetAsync(io.dpart, 0, 3 * sizeof(double) * nblk, st));
  k_ring_init<<<1, 32, 0, st>>>(lr);
  k_absmax_slot<<<grid_for(n), 256, 0, st>>>(io.lam_T, n, lr);
  k_to_fixed<<<grid_for(n), 256, 0, st>>>(io.lam_T, io.lam[0], nullptr, n, lr, lr + 1, lr + 2,
                                         gK, nullptr, err);
  note_launch(3);
  int li = 1;  // adjoint ring position of the next launch
  int lc = 0;
  for (int sgi = io.nseg - 1; sgi >= 0; --sgi) {
    const int len = std::min(io.K, io.S - sgi * io.K);
    cudaEvent_t e0 = nullptr, e1 = nullptr, e2 = nullptr;
    if (io.events && (io.recompute_ev || io.adjoint_ev)) {
      e0 = io.events->make();
      e1 = io.events->make();
      e2 = io.events->make();
      EventPool::record(e0, st);
    }
    {
      NvtxScope nvtx_r("fdb.adjoint.recompute");
      // states f^{sK} .. f^{sK+len-1}: state 0 from the checkpoint (forward
      // ring position 0), then the temporally blocked forward kernel, kRec
      // steps per launch, which stores every level in state_g units; the int64
      // chain ping-pongs between the two chain buffers
      k_ring_init<<<1, 32, 0, st>>>(fr);
      k_absmax_slot<<<grid_for(n), 256, 0, st>>>(io.ckpt[sgi], n, fr);
      k_to_fixed<<<grid_for(n), 256, 0, st>>>(io.ckpt[sgi], io.chain[0], io.state_hi[0], n, fr,
                                             fr + 1, fr + 2, gK, logs + 0, err);
      note_launch(3);
      int cc = 0;   // chain buffer of the latest state
      int pos = 1;  // forward ring position of the next launch
      for (int k = 1; k < len;) {
        const int kb = std::min(kRec, len - k);
        FDB_TRY(launch_fixed_one(g, c, fx::kR4W8S, kb, io.chain[cc], io.chain[cc ^ 1], false,
                                 false, fr, pos, err, 0, kRec, logs + k, st, io.state_hi + k));
        cc ^= 1;
        ++pos;
        k += kb;
      }
    }
    FDB_CUDA_TRY(cudaGetLastError());
    EventPool::record(e1, st);
    if (io.recompute_ev && e0 && e1) io.recompute_ev->push_back({e0, e1});
    NvtxScope nvtx_t("fdb.adjoint.transposed");
    // adjoint steps n = sK+len-1 .. sK
    for (int k = len - 1; k >= 0; --k) {
      aT.slot_in = lr + (li % 3);
      aT.slot_out = lr + ((li + 1) % 3);
      aT.slot_reset = lr + ((li + 2) % 3);
      k_adjoint_tile<kAR, kAW, true>
          <<<nblk, 32 * kAW, AdjTileSmem<kAR, kAW, true>::bytes(), st>>>(
              io.lam[lc], io.lam[lc ^ 1], nullptr, io.state_hi[k], logs + k, aT, io.dpart);
      note_launch();
      FDB_CUDA_TRY(cudaGetLastError());
      lc ^= 1;
      ++li;
    }
    EventPool::record(e2, st);
    if (io.adjoint_ev && e1 && e2) io.adjoint_ev->push_back({e1, e2});
  }
  k_to_double<<<grid_for(n), 256, 0, st>>>(io.lam[lc], io.grad_f0, n, lr + (li % 3));
  k_sum3<<<1, 256, 0, st>>>(io.dpart, nblk, io.dda3);
  note_launch(2);
  FDB_CUDA_TRY(cudaGetLastError());
  return FDB_OK;
}

// ---- batched adjoint ----------------------------------------------------

// z-slab height of the batched launches: one common height such that the
// launch is about two waves of resident CTAs (uneven instances then
// balance), at least 4 planes.
static int batch_slab_height(int count, const Geom* geoms) {
  int64_t tile_planes = 0;
  for (int i = 0; i < count; ++i)
    tile_planes += ((geoms[i].nx + 31) / 32) * ((geoms[i].ny + 31) / 32) * geoms[i].nz;
  const int64_t res = step1_resident();
  return (int)std::max<int64_t>(4, (tile_planes + 2 * res - 1) / (2 * res));
}

static int batch_ctas_of(const Geom& g, int H) {
  const int tz = (int)std::min<int64_t>(H, g.nz);
  return (int)(((g.nx + 31) / 32) * ((g.ny + 31) / 32) * ((g.nz + tz - 1) / tz));
}

int batch_adjoint_grid(int count, const Geom* geoms) {
  const int H = batch_slab_height(count, geoms);
  int grid = 0;
  for (int i = 0; i < count; ++i) grid += batch_ctas_of(geoms[i], H);
  return grid;
}

namespace {
struct BatchScratch {
  AdjInst* insT;
  AdjInst* insF;
  int* cta_inst;
  int* cta_base;
  double* dpart;
  ScaleSlot* ringsF;
  ScaleSlot* ringsT;
  int* logs;
  int* guards;
  size_t bytes;
};
BatchScratch carve(void* base, int count, int K, int grid) {
  BatchScratch sc;
  char* p = (char*)base;
  size_t off = 0;
  auto take = [&](size_t n) {
    char* q = p ? p + off : nullptr;
    off += (n + 255) / 256 * 256;
    return q;
  };
  sc.insT = (AdjInst*)take(sizeof(AdjInst) * count);
  sc.insF = (AdjInst*)take(sizeof(AdjInst) * count);
  sc.cta_inst = (int*)take(sizeof(int) * grid);
  sc.cta_base = (int*)take(sizeof(int) * (count + 1));
  sc.dpart = (double*)take(sizeof(double) * 3 * grid);
  sc.ringsF = (ScaleSlot*)take(sizeof(ScaleSlot) * 3 * count);
  sc.ringsT = (ScaleSlot*)take(sizeof(ScaleSlot) * 3 * count);
  sc.logs = (int*)take(sizeof(int) * K * count);
  sc.guards = (int*)take(sizeof(int) * count);
  sc.bytes = off;
  return sc;
}
}  // namespace

size_t batch_adjoint_scratch_bytes(int count, int K, int grid) {
  return carve(nullptr, count, K, grid).bytes;
}

static int set_multi_smem_limits() {
  FDB_CUDA_TRY(cudaFuncSetAttribute(k_adjoint_tile_multi<kAR, kAW, true>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    AdjTileSmem<kAR, kAW, true>::bytes()));
  FDB_CUDA_TRY(cudaFuncSetAttribute(k_adjoint_tile_multi<kAR, kAW, false>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    AdjTileSmem<kAR, kAW, false>::bytes()));
  return FDB_OK;
}

int batch_adjoint_run(const BatchAdjointIO& io, cudaStream_t st) {
  FDB_TRY(set_multi_smem_limits());
  const int count = io.count;
  const int H = batch_slab_height(count, io.geoms);
  const int grid = batch_adjoint_grid(count, io.geoms);
  const BatchScratch sc = carve(io.scratch, count, io.K, grid);
  // per-instance tables: tiling and coefficients of the transposed and the
  // forward step, ring, scale log and first CTA
  std::vector<AdjInst> hT(count), hF(count);
  std::vector<int> cta_inst, cta_base(count + 1), guards(count);
  cta_inst.reserve(grid);
  int next = 0;
  for (int i = 0; i < count; ++i) {
    const Geom& g = io.geoms[i];
    const Coeffs3& c = io.coeffs[i];
    for (int t = 0; t < 2; ++t) {
      FixedArgs a = make_fixed_args(t == 0 ? transposed_geom(g) : g, c, fx::kR4W8S, 1, 0,
                                    (int64_t)2 * 152);
      a.tx = 32;
      a.ty = kAR * kAW;
      a.tiles_x = (a.nx + a.tx - 1) / a.tx;
      a.tiles_y = (a.ny + a.ty - 1) / a.ty;
      a.tz = std::min(H, a.nz);
      a.tiles_z = (a.nz + a.tz - 1) / a.tz;
      a.guard = guard_bits(c, 1);
      a.scale_log = nullptr;
      AdjInst& I = t == 0 ? hT[i] : hF[i];
      I.a = a;
      I.offset = io.offsets[i];
      I.ring = (t == 0 ? sc.ringsT : sc.ringsF) + 3 * i;
      I.logs = sc.logs + (size_t)i * io.K;
      I.cta_base = next;
    }
    const int n = batch_ctas_of(g, H);
    cta_base[i] = next;
    for (int k = 0; k < n; ++k) cta_inst.push_back(i);
    next += n;
    guards[i] = guard_bits(c, 1);
  }
  cta_base[count] = next;
  if (next != grid) return fail(FDB_ERR_INVALID, "batched adjoint tiling mismatch");
  FDB_CUDA_TRY(cudaMemcpyAsync(sc.insT, hT.data(), sizeof(AdjInst) * count,
                               cudaMemcpyHostToDevice, st));
  FDB_CUDA_TRY(cudaMemcpyAsync(sc.insF, hF.data(), sizeof(AdjInst) * count,
                               cudaMemcpyHostToDevice, st));
  FDB_CUDA_TRY(cudaMemcpyAsync(sc.cta_inst, cta_inst.data(), sizeof(int) * grid,
                               cudaMemcpyHostToDevice, st));
  FDB_CUDA_TRY(cudaMemcpyAsync(sc.cta_base, cta_base.data(), sizeof(int) * (count + 1),
                               cudaMemcpyHostToDevice, st));
  FDB_CUDA_TRY(cudaMemcpyAsync(sc.guards, guards.data(), sizeof(int) * count,
                               cudaMemcpyHostToDevice, st));
  FDB_CUDA_TRY(cudaMemsetAsync(sc.dpart, 0, sizeof(double) * 3 * grid, st));
  const unsigned eg = (unsigned)(count * kPerInst);
  const unsigned rg = (unsigned)((3 * count + 255) / 256);
  constexpr int kSmT = AdjTileSmem<kAR, kAW, true>::bytes();
  constexpr int kSmF = AdjTileSmem<kAR, kAW, false>::bytes();

  // lam_T -> int64 (adjoint rings, position 0)
  k_ring_init_multi<<<rg, 256, 0, st>>>(sc.ringsT, count);
  k_absmax_multi<<<eg, 256, 0, st>>>(io.lam_T, io.d_offs, io.d_sizes, sc.ringsT);
  k_to_fixed_multi<<<eg, 256, 0, st>>>(io.lam_T, io.lam[0], nullptr, io.d_offs, io.d_sizes,
                                       sc.ringsT, sc.guards, nullptr, 0, io.err);
  note_launch(3);
  int li = 1;  // adjoint ring position of the next launch
  int lc = 0;
  for (int sgi = io.nseg - 1; sgi >= 0; --sgi) {
    const int len = std::min(io.K, io.S - sgi * io.K);
    // states of the segment: state k in chain[k & 1] (int64) and in
    // state_hi[k] (2^29 units), forward rings at position k
    k_ring_init_multi<<<rg, 256, 0, st>>>(sc.ringsF, count);
    k_absmax_multi<<<eg, 256, 0, st>>>(io.ckpt[sgi], io.d_offs, io.d_sizes, sc.ringsF);
    k_to_fixed_multi<<<eg, 256, 0, st>>>(io.ckpt[sgi], io.chain[0], io.state_hi[0], io.d_offs,
                                         io.d_sizes, sc.ringsF, sc.guards, sc.logs, io.K, io.err);
    note_launch(3);
    for (int k = 1; k < len; ++k) {
      k_adjoint_tile_multi<kAR, kAW, false><<<grid, 32 * kAW, kSmF, st>>>(
          sc.insF, sc.cta_inst, io.chain[(k - 1) & 1], io.chain[k & 1], io.state_hi[k], nullptr,
          k, k, -1, io.err, nullptr);
      note_launch();
    }
    FDB_CUDA_TRY(cudaGetLastError());
    // adjoint steps sK+len-1 .. sK
    for (int k = len - 1; k >= 0; --k) {
      k_adjoint_tile_multi<kAR, kAW, true><<<grid, 32 * kAW, kSmT, st>>>(
          sc.insT, sc.cta_inst, io.lam[lc], io.lam[lc ^ 1], nullptr, io.state_hi[k], li, -1, k,
          io.err, sc.dpart);
      note_launch();
      lc ^= 1;
      ++li;
    }
    FDB_CUDA_TRY(cudaGetLastError());
  }
  k_to_double_multi<<<eg, 256, 0, st>>>(io.lam[lc], io.grad_f0, io.d_offs, io.d_sizes, sc.ringsT,
                                        li);
  k_sum3_multi<<<count, 256, 0, st>>>(sc.dpart, sc.cta_base, io.dda3);
  note_launch(2);
  FDB_CUDA_TRY(cudaGetLastError());
  return FDB_OK;
}

}  // namespace fdb
