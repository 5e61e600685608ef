// step_fixed.cuh -- the temporally blocked block-fixed-point upwind kernel
// (template), included by the per-shape translation units step_fixed_*.cu.
// The algorithm, precision argument and scale protocol are described in
// step_fixed.cu.
#pragma once

#include "fdb_internal.h"
#include "fixed_point.cuh"

namespace fdb {
namespace fx {

struct ScaleSlot {
  unsigned long long m;  // kind 0: FP64 bits of max|f|; kind 1: OR of |F| at scale s
  int s;
  int kind;
};

constexpr int kMaxSlabs = 24;

struct FixedArgs {
  int nz, ny, nx;
  int fz, fy, fx;  // 1: physical axis reversed relative to the logical one
  int tx, ty, tz;
  int tiles_x, tiles_y, tiles_z;
  // k_advect_fixed: z-slabs [slab_z[i], slab_z[i+1]), i < nslab, one CTA per
  // (slab, tile); the other kernels tile z uniformly by tz
  int nslab;
  int slab_z[kMaxSlabs + 1];
  QCoeff qz, qy, qx;
  int guard;
  const ScaleSlot* slot_in;
  ScaleSlot* slot_out;
  ScaleSlot* slot_reset;
  int* err;
  int* scale_log;  // nullable: block 0 records the scale of this launch's output
  // logical z range [or_z0, or_z1) of the planes whose outputs enter the OR
  // of |F| (all planes, except in a slab of a distributed grid: its own ones)
  int or_z0, or_z1;
  // STORE_G launches (the adjoint's recompute): level t+1 of every output
  // cell, in state_g units, into gout[t]; scale_log[t] receives the scale
  int32_t* gout[4];
};

// A state as the adjoint's contraction reads it: G = floor(F / 2^kGShift).
// Every launch's output has |F| < 2^59 (scale_from_slot puts the input below
// 2^(59 - guard); the guard bits cover the launch's growth; the roundings add
// at most 8 units per step), so |G| <= 2^30 fits int32.  Flooring rather than
// rounding shifts G by half a unit on average, and a constant shift adds
// nothing to the contraction: sum_i D_j[i] = 0 over the periodic grid.
constexpr int kGShift = 29;
__device__ __forceinline__ int32_t state_g(int64_t v) { return (int32_t)(v >> kGShift); }

__device__ __forceinline__ int wrap_mod(int i, int n) {
  int r = i % n;
  return r < 0 ? r + n : r;
}

__device__ __forceinline__ void cp_async8(void* smem, const void* gmem) {
  const unsigned saddr = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(saddr), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async4(void* smem, const void* gmem) {
  const unsigned saddr = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(saddr), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;\n" ::: "memory");
}
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// One level for one cell (fixed_point.cuh fixed_update: nine 32x32->64-bit
// products, one rounding, exactly F when every difference is zero).
__device__ __forceinline__ int64_t update(int64_t c, int64_t zb, int64_t up, int64_t left,
                                          const FixedArgs& a) {
  return fixed_update(c, zb, up, left, a.qz, a.qy, a.qx);
}

// Dynamic shared memory of one CTA: plane prefetch [2][R][threads] (cp.async
// loader only), plus the K-deep plane history [K][R][threads] when HSM.
template <int K, int R, int W, bool HSM, int LOADER = 0>
constexpr int fixed_smem_bytes() {
  return ((LOADER == 0 ? 2 : 0) + (HSM ? K : 0)) * R * 32 * W * (int)sizeof(int64_t);
}

// Scale of a launch (or, in the batched kernel, of one instance's time block)
// from its input slot: s = scale of the fixed-point values used inside, d =
// shift that brings int64 input (held at scale s_in) to scale s.  Returns
// false when the slot reports a non-finite input.
__device__ __forceinline__ bool scale_from_slot(const ScaleSlot* slot, int guard, int* s_out,
                                                int* d_out) {
  // L1-bypassing loads: in the persistent batched kernel the slots are
  // rewritten by other CTAs during the launch
  const unsigned long long M = __ldcg(&slot->m);
  const int kind = __ldcg(&slot->kind);
  const int s_in = __ldcg(&slot->s);
  const int T = 58 - guard;  // highest bit allowed for |F| at the input
  int s = 0, d = 0;
  bool ok = true;
  if (kind == 0) {
    if (M >= 0x7FF0000000000000ull) ok = false;  // NaN/Inf in the input field
    else if (M != 0ull) s = T + 1023 - (int)(M >> 52);  // max|f| < 2^(E-1022) -> |F| < 2^(T+1)
  } else if (M != 0ull) {
    d = T - (63 - __clzll((long long)M));
    d = d > 62 ? 62 : (d < -62 ? -62 : d);
    s = s_in + d;
  } else {
    s = s_in;
  }
  *s_out = s;
  *d_out = d;
  return ok;
}

// Loaders of the next plane: cp.async into shared memory (one tile per launch:
// no other CTA writes the input during the launch), or L1-bypassing register
// loads (the persistent batched kernel reads data that other CTAs wrote
// earlier in the same launch, which L1 may hold stale).
// kLoadRegs: read-only-path register loads one plane ahead (one tile per
// launch, like cp.async, but without the shared-memory staging).
enum Loader { kLoadCpAsync = 0, kLoadL2Regs = 1, kLoadRegs = 2 };

// One rectangle of a packed tile (the persistent batched kernel): the output
// cells x in [x0, x0+xout), y in [y0, y0+yout) of the logical axes, and the
// tile's planes from z0 on, computed by a block of lanes (xout + K of them at
// most) and warps of the CTA.  xout = 0 marks an unused rectangle (nothing
// stored).
struct TileGroup {
  int x0, y0, z0;
  int xout, yout;
};

// Advance one tile of one field by `levels` (<= K) steps.  The tile's output
// region is x in [X0, X0+tx), y in [Y0, Y0+ty), z in [Z0, Z0+nout) of the
// logical axes (Z0 + nout <= nz); the CTA computes a (32) x (R*W) x (nout+K)
// region that starts K cells upstream on every axis.  my_or accumulates |F| bits of the stored
// outputs.  Callers synchronise the CTA before reusing shared memory.
//
// LEFT_SMEM (with HSM): the x-1 neighbour comes from the plane history
// instead of a shuffle: each level's values go into their history slot
// before the update (the previous plane's were read just before), and lane l
// reads lane l-1's slot after a warp barrier.  Same values, fewer FMA-pipe
// moves than the 64-bit shuffle.
//
// GROUPED: the CTA holds several rectangles (TileGroup) side by side in lanes
// and stacked in warps; this thread's rectangle is `grp`, in which it is lane
// `xlane` and its row 0 is row `wrow0`.  The first K lanes and rows of every
// rectangle are its halo: the x-1 and y-1 neighbours they read from another
// rectangle feed only halo cells, whose values are never stored.  tile_x,
// tile_y and Z0 are unused, and every rectangle marches nout + K planes.
template <int K, int R, int W, bool HSM, int LOADER, bool STORE_G = false,
          bool LEFT_SMEM = false, bool GROUPED = false>
__device__ __forceinline__ void advance_tile(const FixedArgs& a, int tile_x, int tile_y, int Z0,
                                             int nout, int levels, bool in_f64, bool out_f64, int s, int d,
                                             const int64_t* __restrict__ in,
                                             int64_t* __restrict__ out, int64_t* s_dyn,
                                             int64_t (*s_row)[W][32],
                                             unsigned long long& my_or,
                                             const TileGroup& grp = TileGroup{}, int xlane = 0,
                                             int wrow0 = 0) {
  constexpr int kThreads = 32 * W;
  int64_t(*s_pre)[R][kThreads] = reinterpret_cast<int64_t(*)[R][kThreads]>(s_dyn);
  int64_t(*s_hist)[R][kThreads] =
      reinterpret_cast<int64_t(*)[R][kThreads]>(s_dyn + (LOADER == kLoadCpAsync ? 2 : 0) * R * kThreads);

  const int tid = threadIdx.x;
  const int lane = tid & 31;
  const int warp = tid >> 5;
  const int X0 = GROUPED ? grp.x0 : tile_x * a.tx;
  const int Y0 = GROUPED ? grp.y0 : tile_y * a.ty;
  const int xl = GROUPED ? xlane : lane;

  const int lx = wrap_mod(X0 - K + xl, a.nx);
  const int px = a.fx ? a.nx - 1 - lx : lx;
  const bool out_x = GROUPED ? (xl >= K && xl - K < grp.xout) : (lane >= K) && (X0 + lane - K < a.nx);

  // offset (py * nx + px) of each of this thread's rows, wrapped once here:
  // the rows stay the same for the whole z-march (unsigned: each address is
  // one 32 x 32 -> 64-bit multiply-add)
  const int ly0 = Y0 - K + (GROUPED ? wrow0 : warp * R);
  unsigned roff[R];
#pragma unroll
  for (int r = 0; r < R; ++r) {
    int ly = ly0 + r;
    ly = ly < 0 ? ly + a.ny : (ly >= a.ny ? ly - a.ny : ly);  // |ly0| < ny: one wrap at most
    if (ly < 0 || ly >= a.ny) ly = wrap_mod(ly, a.ny);         // grids shorter than the tile
    roff[r] = (a.fy ? a.ny - 1 - ly : ly) * a.nx + px;
  }
  // physical offset of the plane at logical z, advanced plane by plane
  const int64_t plane_sz = (int64_t)a.ny * a.nx;
  const int64_t dz = a.fz ? -plane_sz : plane_sz;
  const int64_t po_wrap = a.fz ? (int64_t)(a.nz - 1) * plane_sz : 0;  // logical z = 0
  const int nplanes = nout + K;
  // rows this thread writes: bit r set when row r lies in the tile and the grid
  unsigned row_mask = 0u;
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const int ry = (GROUPED ? wrow0 : warp * R) + r;
    if (out_x && ry >= K && (GROUPED ? ry - K < grp.yout : Y0 + ry - K < a.ny)) row_mask |= 1u << r;
  }


  int64_t hist[HSM ? 1 : K][R];
  int64_t cur[R];
  static_assert(!LEFT_SMEM || HSM, "the x-1 neighbour from shared memory needs the history there");
  static_assert(!(GROUPED && STORE_G), "packed tiles store no adjoint states");
  int64_t pre[LOADER != kLoadCpAsync ? R : 1];
#pragma unroll
  for (int t = 0; t < (HSM ? 1 : K); ++t)
#pragma unroll
    for (int r = 0; r < R; ++r) hist[t][r] = 0;
  if (HSM) {
#pragma unroll
    for (int t = 0; t < K; ++t)
#pragma unroll
      for (int r = 0; r < R; ++r) s_hist[t][r][tid] = 0;
  }

  // logical z of the plane being computed; advanced by one per iteration
  int lz = wrap_mod((GROUPED ? grp.z0 : Z0) - K, a.nz);
  int64_t po = (int64_t)(a.fz ? a.nz - 1 - lz : lz) * plane_sz;
  {
    const int64_t* src = in + po;
    if (LOADER == kLoadCpAsync) {
#pragma unroll
      for (int r = 0; r < R; ++r) cp_async8(&s_pre[0][r][tid], src + roff[r]);
      cp_async_commit();
    } else {
#pragma unroll
      for (int r = 0; r < R; ++r)
        pre[r] = LOADER == kLoadRegs ? __ldg(src + roff[r]) : __ldcg(src + roff[r]);
    }
  }

  int parity = 0;
  for (int p = 0; p < nplanes; ++p) {
    const bool wraps = lz + 1 == a.nz;
    const int lz_next = wraps ? 0 : lz + 1;
    const int64_t po_next = wraps ? po_wrap : po + dz;
    if (LOADER == kLoadCpAsync) {
      if (p + 1 < nplanes) {
        const int64_t* src = in + po_next;
#pragma unroll
        for (int r = 0; r < R; ++r) cp_async8(&s_pre[(p + 1) & 1][r][tid], src + roff[r]);
      }
      cp_async_commit();
      cp_async_wait<1>();
#pragma unroll
      for (int r = 0; r < R; ++r) cur[r] = s_pre[p & 1][r][tid];
    } else {
#pragma unroll
      for (int r = 0; r < R; ++r) cur[r] = pre[r];
      if (p + 1 < nplanes) {
        const int64_t* src = in + po_next;
#pragma unroll
        for (int r = 0; r < R; ++r)
          pre[r] = LOADER == kLoadRegs ? __ldg(src + roff[r]) : __ldcg(src + roff[r]);
      }
    }
    if (in_f64) {
#pragma unroll
      for (int r = 0; r < R; ++r) cur[r] = to_fixed(__longlong_as_double(cur[r]), s);
    } else if (d != 0) {
#pragma unroll
      for (int r = 0; r < R; ++r) cur[r] = d > 0 ? (cur[r] << d) : (cur[r] >> (-d));
    }
#pragma unroll
    for (int t = 0; t < K; ++t) {
      // Level t+1 is skipped (uniformly across the CTA) on warm-up plane p
      // for t >= p, where it is not valid, and for t >= levels; level t is
      // still recorded as the history that level t+1 of the next plane reads.
      if ((p < K && t >= p) || t >= levels) {
#pragma unroll
        for (int r = 0; r < R; ++r) {
          if (HSM) s_hist[t][r][tid] = cur[r];
          else hist[HSM ? 0 : t][r] = cur[r];
        }
        continue;
      }
      int64_t zb[R];
      if (HSM) {
#pragma unroll
        for (int r = 0; r < R; ++r) zb[r] = s_hist[t][r][tid];
      }
      // publish this level's last row for the warp below, then update rows
      // R-1 .. 1 (their y-1 neighbour is the thread's own previous row) while
      // the other warps catch up, and row 0 after the barrier
      s_row[parity][warp][lane] = cur[R - 1];
      // x-1 neighbour; lane 0 (the tile's halo column) receives its own value
      int64_t left[R];
      if (LEFT_SMEM) {
#pragma unroll
        for (int r = 0; r < R; ++r) s_hist[t][r][tid] = cur[r];
        __syncwarp();
        const int src_tid = tid - (lane > 0 ? 1 : 0);
#pragma unroll
        for (int r = 0; r < R; ++r) left[r] = s_hist[t][r][src_tid];
      } else {
#pragma unroll
        for (int r = 0; r < R; ++r) left[r] = __shfl_up_sync(0xffffffffu, cur[r], 1);
      }
      auto row = [&](int r, int64_t upv) {
        const int64_t c = cur[r];
        const int64_t nv = update(c, HSM ? zb[r] : hist[HSM ? 0 : t][r], upv, left[r], a);
        if (HSM) {
          if (!LEFT_SMEM) s_hist[t][r][tid] = c;
        } else {
          hist[HSM ? 0 : t][r] = c;
        }
        cur[r] = nv;
      };
#pragma unroll
      for (int r = R - 1; r >= 1; --r) row(r, cur[r - 1]);
      __syncthreads();
      row(0, (warp > 0) ? s_row[parity][warp - 1][lane] : cur[0]);
      parity ^= 1;
      if (STORE_G && p >= K) {
        int32_t* g = a.gout[t] + po;
#pragma unroll
        for (int r = 0; r < R; ++r)
          if (row_mask & (1u << r)) g[roff[r]] = state_g(cur[r]);
      }
    }
    if (p >= K) {
      int64_t* dst = out + po;
      const bool counted = lz >= a.or_z0 && lz < a.or_z1;  // uniform per plane
#pragma unroll
      for (int r = 0; r < R; ++r) {
        if (row_mask & (1u << r)) {
          const int64_t v = cur[r];
          if (counted) my_or |= (unsigned long long)(v ^ (v >> 63));
          if (out_f64)
            dst[roff[r]] = __double_as_longlong(to_double(v, s));
          else
            dst[roff[r]] = v;
        }
      }
    }
    lz = lz_next;
    po = po_next;
  }
  if (LOADER == kLoadCpAsync) cp_async_wait<0>();
}

// OR of my_or over the CTA -> atomicOr into *dst (thread 0).  Contains a
// __syncthreads.
template <int W>
__device__ __forceinline__ void cta_or(unsigned long long my_or, unsigned long long* s_or,
                                       unsigned long long* dst) {
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) my_or |= __shfl_xor_sync(0xffffffffu, my_or, o);
  if (lane == 0) s_or[warp] = my_or;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long m = 0ull;
#pragma unroll
    for (int w = 0; w < W; ++w) m |= s_or[w];
    if (m) atomicOr(dst, m);
  }
}

// One launch = K steps of one field.  CTA b works on tile b % (tiles_x *
// tiles_y) of z-slab b / (tiles_x * tiles_y): the CTAs that run together share
// their halo rows through L2, and the slabs shrink towards the end of the
// grid so that the last wave is short (the scheduler hands out CTAs in
// index order).
template <int K, int R, int W, bool HSM, int MINB, bool IN_F64, bool OUT_F64, bool STORE_G = false,
          int LOAD = kLoadCpAsync, bool LEFT = false>
__global__ void __launch_bounds__(32 * W, MINB)
k_advect_fixed(const int64_t* __restrict__ in, int64_t* __restrict__ out, const FixedArgs a) {
  extern __shared__ __align__(16) int64_t s_dyn[];
  __shared__ int64_t s_row[2][W][32];
  __shared__ unsigned long long s_or[W];

  const int txy = a.tiles_x * a.tiles_y;
  const int slab = (int)blockIdx.x / txy;
  const int tile = (int)blockIdx.x - slab * txy;
  const int z0 = a.slab_z[slab];
  const int nout = a.slab_z[slab + 1] - z0;

  int s, d;
  if (!scale_from_slot(a.slot_in, a.guard, &s, &d) && threadIdx.x == 0) atomicOr(a.err, 1);
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    a.slot_reset->m = 0ull;
    a.slot_reset->kind = 1;
    a.slot_out->s = s;
    a.slot_out->kind = 1;
    if (a.scale_log) {
      // every level of the launch is held at scale s
      if (STORE_G)
        for (int t = 0; t < K; ++t) a.scale_log[t] = s;
      else
        *a.scale_log = s;
    }
  }
  unsigned long long my_or = 0ull;
  advance_tile<K, R, W, HSM, LOAD, STORE_G, LEFT>(a, tile % a.tiles_x, tile / a.tiles_x, z0,
                                                  nout, K, IN_F64, OUT_F64, s, d, in, out,
                                                  s_dyn, s_row, my_or);
  cta_or<W>(my_or, s_or, &a.slot_out->m);
}

// Kernel shapes compiled into the library: rows per thread x warps per CTA,
// history in registers (reg) or shared memory (smem); the L shapes load the
// next plane into registers and take the x-1 neighbour from the history
// (kLoadRegs, LEFT_SMEM).
enum Shape {
  kR8W8 = 0, kR4W16 = 1, kR8W8S = 2, kR4W16S = 3, kR4W8S = 4, kR4W8L = 5, kR6W8L = 6,
  kNumShapes = 7
};
constexpr int shape_rows(int sh) {
  return (sh == kR8W8 || sh == kR8W8S) ? 8 : (sh == kR6W8L ? 6 : 4);
}
constexpr int shape_warps(int sh) { return (sh == kR4W16 || sh == kR4W16S) ? 16 : 8; }

// z-slabs of one k_advect_fixed launch for `resident` CTAs on the GPU at once:
// slabs of h0 planes (cap if > 0, else about a quarter of the planes per
// resident CTA, at least 32), then slabs that follow the remaining planes per
// resident CTA down to 8.  Sets a.nslab / a.slab_z; returns the CTA count.
long long plan_slabs(FixedArgs& a, int resident, int cap);

template <int K, int R, int W, bool HSM, int MINB, bool IN, bool OUT, bool STORE_G = false,
          int LOAD = kLoadCpAsync, bool LEFT = false>
void launch_k(int cap, const int64_t* in, int64_t* out, FixedArgs a, cudaStream_t st) {
  constexpr int smem = fixed_smem_bytes<K, R, W, HSM, LOAD>();
  auto kern = k_advect_fixed<K, R, W, HSM, MINB, IN, OUT, STORE_G, LOAD, LEFT>;
  static int per_sm = -1;  // per instantiation; benign race (idempotent)
  if (per_sm < 0) {
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    int occ = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, 32 * W, smem) != cudaSuccess)
      occ = 1;
    per_sm = occ > 0 ? occ : 1;
  }
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const long long blocks = plan_slabs(a, per_sm * (sms > 0 ? sms : 1), cap);
  if (blocks <= 0) return;
  kern<<<(unsigned)blocks, 32 * W, smem, st>>>(in, out, a);
}

// int64 in and out, every level also stored in state_g units (a.gout)
template <int R, int W, bool HSM, int MINB>
void launch_shape_store_g(int K, int cap, const int64_t* in, int64_t* out, const FixedArgs& a,
                          cudaStream_t st) {
  switch (K) {
    case 1: launch_k<1, R, W, HSM, MINB, false, false, true>(cap, in, out, a, st); break;
    case 2: launch_k<2, R, W, HSM, MINB, false, false, true>(cap, in, out, a, st); break;
    case 3: launch_k<3, R, W, HSM, MINB, false, false, true>(cap, in, out, a, st); break;
    default: launch_k<4, R, W, HSM, MINB, false, false, true>(cap, in, out, a, st); break;
  }
}

template <int K, int R, int W, bool HSM, int MINB, int LOAD = kLoadCpAsync, bool LEFT = false>
void launch_io(bool in_f64, bool out_f64, int cap, const int64_t* in, int64_t* out,
               const FixedArgs& a, cudaStream_t st) {
  if (in_f64 && out_f64)
    launch_k<K, R, W, HSM, MINB, true, true, false, LOAD, LEFT>(cap, in, out, a, st);
  else if (in_f64)
    launch_k<K, R, W, HSM, MINB, true, false, false, LOAD, LEFT>(cap, in, out, a, st);
  else if (out_f64)
    launch_k<K, R, W, HSM, MINB, false, true, false, LOAD, LEFT>(cap, in, out, a, st);
  else
    launch_k<K, R, W, HSM, MINB, false, false, false, LOAD, LEFT>(cap, in, out, a, st);
}

template <int R, int W, bool HSM, int MINB, int LOAD = kLoadCpAsync, bool LEFT = false>
void launch_shape(int K, bool in_f64, bool out_f64, int cap, const int64_t* in, int64_t* out,
                  const FixedArgs& a, cudaStream_t st) {
  switch (K) {
    case 1: launch_io<1, R, W, HSM, MINB, LOAD, LEFT>(in_f64, out_f64, cap, in, out, a, st); break;
    case 2: launch_io<2, R, W, HSM, MINB, LOAD, LEFT>(in_f64, out_f64, cap, in, out, a, st); break;
    case 3: launch_io<3, R, W, HSM, MINB, LOAD, LEFT>(in_f64, out_f64, cap, in, out, a, st); break;
    default: launch_io<4, R, W, HSM, MINB, LOAD, LEFT>(in_f64, out_f64, cap, in, out, a, st); break;
  }
}

// defined in step_fixed.cu
}  // namespace fx
fx::FixedArgs make_fixed_args(const Geom& g, const Coeffs3& c, int shape, int K, int tz_override,
                              int64_t resident_ctas);
int guard_bits(const Coeffs3& c, int K);
// One launch of the single-field kernel (K steps, explicit buffers and slot
// ring position i); scale_log (nullable, device) receives the output scale.
// gout (nullable; K arrays, int64 in and out, default shape only): every level
// of the launch stored in state_g units, its scale in scale_log[0..K).
int launch_fixed_one(const Geom& g, const Coeffs3& c, int shape, int K, const void* in, void* out,
                     bool in_f64, bool out_f64, fx::ScaleSlot* slots, int i, int* err,
                     int tz_override, int guard_K, int* scale_log, cudaStream_t st,
                     int32_t* const* gout = nullptr);
namespace fx {

// defined in step_fixed_<shape>.cu; cap as in plan_slabs
#define FDB_FX_DECLARE(NAME)                                                               \
  void NAME(int K, bool in_f64, bool out_f64, int cap, const int64_t* in, int64_t* out,    \
            const FixedArgs& a, cudaStream_t st);
FDB_FX_DECLARE(launch_r8w8)
// the default shape with every level stored (the adjoint's recompute)
void launch_r4w8s_store_g(int K, int cap, const int64_t* in, int64_t* out, const FixedArgs& a,
                          cudaStream_t st);
FDB_FX_DECLARE(launch_r4w16)
FDB_FX_DECLARE(launch_r8w8s)
FDB_FX_DECLARE(launch_r4w16s)
FDB_FX_DECLARE(launch_r4w8s)
FDB_FX_DECLARE(launch_r4w8l)
FDB_FX_DECLARE(launch_r6w8l)
#undef FDB_FX_DECLARE

}  // namespace fx
}  // namespace fdb
