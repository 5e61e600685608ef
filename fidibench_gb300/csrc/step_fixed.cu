// step_fixed.cu -- temporally blocked upwind kernel in 64-bit block-fixed-point.
//
// One launch advances the field by K steps (K = 1..4).  Within one advect()
// call the field stays in fixed point in HBM between launches: the first
// launch reads FP64 and converts f -> F = round(f * 2^s), the inner launches
// read and write int64 F (8 B, like FP64), and the last launch converts back
// and writes FP64.  Each launch streams every cell once: 16 B of HBM traffic
// per cell per K steps.  The arithmetic runs on the integer pipes
// (IMAD/IADD3/LOP3/SHFL); GB300 retires only ~2 FP64 operations per clock
// per SM, which would cap a native FP64 step near 150 GCUPS.
//
// Precision.  The scale keeps |F| < 2^(59-g) at a launch's input (g guard
// bits cover the step's max-norm growth G^K), so one unit of F is at most
// 2^-(58-g) of max|f|.  One step adds < 8 units of truncation error per cell,
// so after 100 steps the field is within ~1e-15 of the reference's FP64
// arithmetic relative to max|f| (the bar is 1e-13).  Cells below one unit
// are held as 0, an absolute error below the same bound.
//
// Update.  F' = F + sum_j a_j (F_up_j - F) with a_j in [0, 1] held in Q1.62
// (A = a1 2^32 + a0, a0 balanced to [-2^31, 2^31)).  For D = d1 2^32 + d0:
//   A D / 2^64 = a1 d1 + (a1 d0 + a0 d1) 2^-32 + a0 d0 2^-64
// the a1 d1 products are summed exactly; the six a1 d0 and a0 d1 partial
// products of the three axes are summed exactly in one offset unsigned
// 64-bit word whose high word is taken (one rounding to nearest);
// F' = F + 4 * sum (fixed_point.cuh fixed_update).  The rounding is unbiased
// and a zero difference contributes exactly zero.
//
// Geometry.  Axes are relabelled so that every upstream neighbour is at -1
// (axis j reversed when v_j < 0, upwind.cxx:34-35).  A CTA of W warps owns an
// output tile of (32-K) x (R*W-K) cells in (x, y) and marches along z over tz
// output planes after K warm-up planes.  Lanes are consecutive x (coalesced
// 256 B row accesses), each thread holds R consecutive y rows of one column
// in registers (shapes R x W = 8x8 and 4x16 with the plane history in
// registers or shared memory, and 4x8 with it in shared memory, are
// compiled).  Per level: x-1 from lane-1 by SHFL, y-1 from the thread's
// previous row (row 0 from the warp above through shared memory, one
// __syncthreads per level), z-1 from the thread's K-deep history of the
// previous plane.  The next plane is prefetched with cp.async into shared
// memory while the current one is computed.  The upstream halo (K columns,
// K rows, K planes) is the only redundant work; periodic wrap is applied to
// the coordinates of the loaded rows and planes.
//
// Scale protocol (no host synchronisation).  Three device slots hold
// {m, s, kind}: kind 0 = m is the FP64 bit pattern of max|f| (from the
// pre-pass), kind 1 = m is an OR of |F| over the field held at scale s.
// Launch i reads slot i%3, ORs its output into slot (i+1)%3 (block 0 also
// writes s and kind there) and clears slot (i+2)%3 for launch i+1.
#include <math.h>

#include "step_fixed.cuh"

namespace fdb {

using fx::FixedArgs;
using fx::ScaleSlot;

double growth_bound(const Coeffs3& c) { return fabs(c.w) + c.az + c.ay + c.ax; }

int guard_bits(const Coeffs3& c, int K) {
  const double G = growth_bound(c);
  if (G <= 1.0) return 0;
  return (int)ceil(K * log2(G)) + 1;
}

namespace {

constexpr int kMaxDepth = 4;

// max|f| as the bit pattern of |f| (monotone for non-negative doubles; NaN
// and Inf patterns exceed every finite one) -> slot {m, kind 0}.
__global__ void __launch_bounds__(256)
k_absmax_bits(const double* __restrict__ f, uint64_t n, ScaleSlot* __restrict__ slot) {
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
    atomicMax(&slot->m, m);
  }
}

__global__ void k_slots_init(ScaleSlot* slots) {
  if (threadIdx.x < 3) {
    slots[threadIdx.x].m = 0ull;
    slots[threadIdx.x].s = 0;
    slots[threadIdx.x].kind = threadIdx.x == 0 ? 0 : 1;
  }
}


}  // namespace

// Tiling and coefficients of one field for the fixed kernel (slot pointers
// are left null).  tz_override > 0 fixes the output planes per CTA.
fx::FixedArgs make_fixed_args(const Geom& g, const Coeffs3& c, int shape, int K, int tz_override,
                              int64_t resident_ctas) {
  const int R = fx::shape_rows(shape), W = fx::shape_warps(shape);
  FixedArgs a{};
  a.nz = (int)g.nz;
  a.ny = (int)g.ny;
  a.nx = (int)g.nx;
  a.fz = g.upz > 0;
  a.fy = g.upy > 0;
  a.fx = g.upx > 0;
  a.tx = 32 - K;
  a.ty = R * W - K;
  a.tiles_x = (a.nx + a.tx - 1) / a.tx;
  a.tiles_y = (a.ny + a.ty - 1) / a.ty;
  const int64_t txy = (int64_t)a.tiles_x * a.tiles_y;
  int tz = tz_override;
  if (tz <= 0) {
    // about four waves of the resident CTAs
    const int64_t want = 4 * resident_ctas;
    int64_t cz = (want + txy - 1) / txy;
    if (cz < 1) cz = 1;
    tz = (int)((a.nz + cz - 1) / cz);
    if (tz < 4 * K) tz = 4 * K;
  }
  if (tz > a.nz) tz = a.nz;
  a.tz = tz;
  a.tiles_z = (a.nz + tz - 1) / tz;
  a.qz = make_qcoeff(c.az);
  a.qy = make_qcoeff(c.ay);
  a.qx = make_qcoeff(c.ax);
  a.guard = guard_bits(c, K);
  // the planes whose outputs set the next scale: the geometry's own planes
  // of the internal z axis (all of them unless a slab names its own)
  a.or_z0 = 0;
  a.or_z1 = a.nz;
  if (g.own_n > 0 && g.jz == 0) {
    const int p0 = (int)g.own0, p1 = (int)(g.own0 + g.own_n);  // physical
    a.or_z0 = a.fz ? a.nz - p1 : p0;
    a.or_z1 = a.fz ? a.nz - p0 : p1;
  }
  return a;
}

namespace fx {

long long plan_slabs(FixedArgs& a, int resident, int cap) {
  const long long txy = (long long)a.tiles_x * a.tiles_y;
  const int nz = a.nz;
  if (txy <= 0 || nz <= 0) {
    a.nslab = 0;
    return 0;
  }
  const long long res = resident > 0 ? resident : 1;
  int h0 = cap;
  if (h0 <= 0) {
    h0 = (int)((txy * nz + 4 * res - 1) / (4 * res));
    if (h0 < 32) h0 = 32;
  }
  if (h0 > nz) h0 = nz;
  const int hmin = h0 < 8 ? h0 : 8;
  int z = 0, i = 0;
  while (z < nz) {
    const int rem = nz - z;
    long long h = (txy * rem + res - 1) / res;  // remaining planes per resident CTA
    if (h > h0) h = h0;
    if (h < hmin) h = hmin;
    if (h > rem || i == kMaxSlabs - 1) h = rem;
    a.slab_z[i++] = z;
    z += (int)h;
  }
  a.slab_z[i] = nz;
  a.nslab = i;
  return txy * i;
}

}  // namespace fx

int launch_fixed_one(const Geom& g, const Coeffs3& c, int shape, int K, const void* in, void* out,
                     bool in_f64, bool out_f64, ScaleSlot* slots, int i, int* err,
                     int tz_override, int guard_K, int* scale_log, cudaStream_t st,
                     int32_t* const* gout) {
  if (gout && (shape != fx::kR4W8S || in_f64 || out_f64 || K < 1 || K > 4))
    return fail(FDB_ERR_UNSUPPORTED, "level output needs the default shape and int64 in/out");
  // 8 x 152 resident 256-thread CTAs, scaled to this shape's CTA size
  FixedArgs a = make_fixed_args(g, c, shape, K, tz_override,
                                (int64_t)2 * 152 * 256 / (32 * fx::shape_warps(shape)));
  // guard bits sized for the call's full depth, also on a shorter final
  // launch, so that every launch of a call uses the same headroom rule as the
  // batched kernel (which sizes them once per instance)
  a.guard = guard_bits(c, guard_K);
  a.slot_in = slots + (i % 3);
  a.slot_out = slots + ((i + 1) % 3);
  a.slot_reset = slots + ((i + 2) % 3);
  a.err = err;
  a.scale_log = scale_log;
  // the grid is at most tiles_x * tiles_y * kMaxSlabs CTAs
  if ((int64_t)a.tiles_x * a.tiles_y * fx::kMaxSlabs > 0x7FFFFFFF)
    return fail(FDB_ERR_UNSUPPORTED, "grid too large for the fixed kernel");
  const int64_t* pin = (const int64_t*)in;
  int64_t* pout = (int64_t*)out;
  const int cap = tz_override > 0 ? tz_override : 0;
  if (gout) {
    for (int t = 0; t < K; ++t) a.gout[t] = gout[t];
    fx::launch_r4w8s_store_g(K, cap, pin, pout, a, st);
    note_launch();
    FDB_CUDA_TRY(cudaGetLastError());
    return FDB_OK;
  }
  switch (shape) {
    case fx::kR4W16: fx::launch_r4w16(K, in_f64, out_f64, cap, pin, pout, a, st); break;
    case fx::kR8W8S: fx::launch_r8w8s(K, in_f64, out_f64, cap, pin, pout, a, st); break;
    case fx::kR4W16S: fx::launch_r4w16s(K, in_f64, out_f64, cap, pin, pout, a, st); break;
    case fx::kR4W8S: fx::launch_r4w8s(K, in_f64, out_f64, cap, pin, pout, a, st); break;
    case fx::kR4W8L: fx::launch_r4w8l(K, in_f64, out_f64, cap, pin, pout, a, st); break;
    case fx::kR6W8L: fx::launch_r6w8l(K, in_f64, out_f64, cap, pin, pout, a, st); break;
    default: fx::launch_r8w8(K, in_f64, out_f64, cap, pin, pout, a, st); break;
  }
  note_launch();
  FDB_CUDA_TRY(cudaGetLastError());
  return FDB_OK;
}

namespace {

// Default shape: 4 or 6 rows x 8 warps with the plane history in shared
// memory, the next plane loaded into registers and the x-1 neighbour read
// from the history.  Measured (advect(100), one GB300): 512^3 457 GCUPS for
// 6 rows against 454 for 4 rows and 442 for the cp.async/shuffle 4 x 8 form;
// 384^3 422 / 418 / 418; 320^3 416 / 395 / 391; 256^3 389 / 394 / 382.
// Grids of up to 256^3 cells take 4 rows (more tiles keep the GPU full).
int default_shape(const Geom& g, int K) {
  (void)K;
  return g.ntot > (uint64_t)256 * 256 * 256 ? fx::kR6W8L : fx::kR4W8L;
}

}  // namespace

// Steps per launch for the default shape: the K that minimises the computed
// tiles times the per-launch cost,
//   ceil(nx / (32 - K)) * ceil(ny / (32 - K)) * (1 + 0.5 / K),
// where 0.5 is the per-plane work (load, scale, store) in units of one
// level's update (fitted to 160^3 .. 512^3 sweeps of K = 2..4, whose
// winners this picks: 4 at 160, 3 at 256, 2 at 384, 3 at 512); ties go to
// the deeper K.
int default_depth(const Geom& g) {
  int best = kMaxDepth;
  double best_cost = 0.0;
  for (int K = kMaxDepth; K >= 2; --K) {
    const double w = 32.0 - K;
    const double tiles = std::ceil(g.nx / w) * std::ceil(g.ny / w);
    const double cost = tiles * (1.0 + 0.5 / K);
    if (K == kMaxDepth || cost < best_cost) {
      best = K;
      best_cost = cost;
    }
  }
  return best;
}

int fixed_supported(const Geom& g, const Coeffs3& c, int depth) {
  if (g.ndims > 3) return fail(FDB_ERR_UNSUPPORTED, "fixed kernel serves ndims <= 3");
  const int K = depth > 0 ? depth : default_depth(g);
  if (K > kMaxDepth) return fail(FDB_ERR_UNSUPPORTED, "fixed kernel temporal depth must be <= 4");
  const double as[3] = {c.az, c.ay, c.ax};
  for (double x : as)
    if (!(x >= 0.0 && x <= 1.0))
      return fail(FDB_ERR_UNSUPPORTED, "fixed kernel needs Courant numbers a_j in [0, 1]");
  if (guard_bits(c, K) > 16)
    return fail(FDB_ERR_UNSUPPORTED, "step growth too large for the fixed kernel's headroom");
  if (g.nx >= (1 << 30) || g.ny >= (1 << 30) || g.nz >= (1 << 30) ||
      g.nx * g.ny >= ((int64_t)1 << 31))
    return fail(FDB_ERR_UNSUPPORTED, "fixed kernel needs ny*nx < 2^31");
  return FDB_OK;
}

bool fixed_preferred(const Geom& g) {
  // tiles are (32-K) x (R*W-K) cells in (x, y); small grids are cheaper in FP64
  return g.ndims <= 3 && g.nx >= 16 && g.ny >= 16 && g.nz >= 8 && g.ntot >= (1u << 18);
}

int fx_num_shapes() { return fx::kNumShapes; }

size_t fixed_scratch_bytes() { return 3 * sizeof(ScaleSlot) + 4 * sizeof(int); }

int* fixed_error_word(double* d_scratch) { return (int*)((ScaleSlot*)d_scratch + 3); }

int launch_scale_prepass(const Geom& g, const double* f, double* d_scratch, cudaStream_t s) {
  ScaleSlot* slots = (ScaleSlot*)d_scratch;
  // max|f| over the geometry's own planes of axis 0 (all planes unless a
  // slab names its own: its halo planes hold other ranks' values)
  uint64_t first = 0, count = g.ntot;
  if (g.own_n > 0) {
    const uint64_t plane = g.ntot / g.n[0];
    first = g.own0 * plane;
    count = g.own_n * plane;
  }
  k_slots_init<<<1, 32, 0, s>>>(slots);
  uint64_t blocks = (count + 255) / 256;
  if (blocks > 152 * 8) blocks = 152 * 8;
  if (blocks < 1) blocks = 1;
  k_absmax_bits<<<(unsigned)blocks, 256, 0, s>>>(f + first, count, slots);
  note_launch(2);
  FDB_CUDA_TRY(cudaGetLastError());
  return FDB_OK;
}

int launch_fixed_block(const Geom& g, const Coeffs3& c, int k, const FixedTuning& tune,
                       int guard_K, double** buf, int* cur, bool in_f64, bool out_f64,
                       double* d_scratch, int i, cudaStream_t s) {
  if (fault_injected("launch")) return fail(FDB_ERR_INJECTED, "injected launch failure");
  const int shape =
      (tune.shape >= 0 && tune.shape < fx::kNumShapes) ? tune.shape : default_shape(g, guard_K);
  FDB_TRY(launch_fixed_one(g, c, shape, k, buf[*cur], buf[*cur ^ 1], in_f64, out_f64,
                           (ScaleSlot*)d_scratch, i, fixed_error_word(d_scratch), tune.tz, guard_K,
                           nullptr, s));
  *cur ^= 1;
  return FDB_OK;
}

uint64_t* scale_word(double* d_scratch, int i) {
  return reinterpret_cast<uint64_t*>(&((ScaleSlot*)d_scratch + (i % 3))->m);
}

int launch_advect_fixed(const Geom& g, const Coeffs3& c, int steps, int depth, double** buf,
                        int* cur, double* d_scratch, size_t scratch_bytes, cudaStream_t s) {
  FixedTuning t;
  t.depth = depth;
  return launch_advect_fixed_ex(g, c, steps, t, buf, cur, d_scratch, scratch_bytes, nullptr, s);
}

int launch_advect_fixed_ex(const Geom& g, const Coeffs3& c, int steps, const FixedTuning& tune,
                           double** buf, int* cur, double* d_scratch, size_t scratch_bytes,
                           int* scale_slot, cudaStream_t s) {
  if (fault_injected("launch")) return fail(FDB_ERR_INJECTED, "injected launch failure");
  if (scratch_bytes < fixed_scratch_bytes() || !d_scratch)
    return fail(FDB_ERR_INVALID, "fixed kernel scratch missing");
  if (steps <= 0) return FDB_OK;
  ScaleSlot* slots = (ScaleSlot*)d_scratch;
  int* err = fixed_error_word(d_scratch);
  const int K = tune.depth > 0 ? tune.depth : default_depth(g);
  const int shape =
      (tune.shape >= 0 && tune.shape < fx::kNumShapes) ? tune.shape : default_shape(g, K);
  int i0 = (scale_slot && *scale_slot >= 0) ? *scale_slot : -1;
  if (i0 < 0) {
    FDB_TRY(launch_scale_prepass(g, buf[*cur], d_scratch, s));
    i0 = 0;
  }
  const int nlaunch = (steps + K - 1) / K;
  int i = i0;
  for (int l = 0, done = 0; l < nlaunch; ++l, ++i) {
    const int k = (steps - done) < K ? (steps - done) : K;
    FDB_TRY(launch_fixed_one(g, c, shape, k, buf[*cur], buf[*cur ^ 1], l == 0, l == nlaunch - 1,
                             slots, i, err, tune.tz, K, nullptr, s));
    *cur ^= 1;
    done += k;
  }
  if (scale_slot) *scale_slot = i % 3;
  return FDB_OK;
}

}  // namespace fdb
