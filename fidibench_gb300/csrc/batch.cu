// batch.cu -- many independent upwind problems of uneven sizes and
// velocities advanced in one persistent launch (no reference counterpart;
// each instance is the reference's advect(), upwind/cxx/upwind.cxx:51-86).
//
// Work.  advect(steps) is cut into time blocks of K steps.  A work item is
// one packed tile of one instance in one time block: rectangles of output
// cells laid side by side in the lanes and stacked in the warps of a CTA
// (pack_instance), so that the remainder strips of uneven axes share CTAs
// instead of padding one each.  Items are numbered block-major, instance,
// tile.  One persistent grid (the resident CTAs of the device) takes items
// from an atomic counter in that order.
//
// Dependencies.  A tile of block b reads its upstream halo from the
// neighbouring tiles' block b-1 output, so before starting it waits until
// all block b-1 tiles of *its own instance* are done (a per-instance
// completion counter); other instances keep the GPU busy meanwhile, and no
// grid-wide barrier separates the blocks.  Items are taken in block order,
// so every item a CTA waits for was taken earlier by a running CTA that only
// waits for still earlier items: the waits cannot deadlock.  Every wait is
// bounded (clock64 budget): on expiry the CTA sets an error bit and leaves,
// the others follow, and the host reports FDB_ERR_TIMEOUT.
//
// Storage order.  An instance's three axes may be stored permuted: the order
// whose packed tiles march the fewest tile-planes (choose_order).  The update
// sums exact integer products, so the result does not depend on the order of
// the axes; set_field, get_field and init_sphere translate between the
// caller's order and the stored one.
// Instances that the single-field path advances in FP64 keep their order, so
// the looped comparator stays bit-identical to fdb_upwind_advect for all.
//
// Memory.  All instances' fields live in two arenas (ping-pong by block).
// Halo data written by other CTAs during the launch is read with L1-bypassing
// loads (ld.global.cg); a tile's stores are fenced before its completion is
// published.  Each instance has its own three-slot scale ring (see
// step_fixed.cu), advanced per block by the instance's tile 0.
//
// The launch sequence of an advect (counter resets, per-instance max|f|
// pre-pass, persistent kernel) is captured once in a CUDA graph per
// (steps, dt, tuning) and replayed.
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <array>
#include <chrono>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "step_fixed.cuh"

using fdb::fx::FixedArgs;
using fdb::fx::ScaleSlot;

namespace fdb {
namespace bt {

struct InstDev {
  FixedArgs a;        // geometry, tiling, coefficients, guard (slot pointers unused)
  int64_t offset;     // first cell of the instance in the arenas
  int items;          // tiles per time block
  int item_base;      // first item of the instance within a block
};

// One packed tile: rectangles of gw lanes x gh warps of one instance, laid
// out (32 / gw) across the lanes and (W / gh) down the warps, row-major from
// groups[group_base]; each marches nout + K planes.
struct ItemDev {
  int inst;
  int gw, gh;
  int group_base;
  int nout;
};

constexpr long long kWaitCycles = 4000000000ll;  // ~2 s at 2 GHz

// depth of the persistent launch when none is set (the kernel is issue-bound,
// so the smaller halo of depth 2 outweighs its extra field traffic), and the
// depth the storage order is chosen for
constexpr int kDefaultDepth = 2;

__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// 4-row shapes: at least 32 warps per SM (64 registers per thread, no
// spills); 8-row shapes: 16 warps (their rows need the registers)
template <int K, int R, int W>
__global__ void __launch_bounds__(32 * W, (R > 4 ? 512 : 1024) / (32 * W))
k_batch_fixed(const InstDev* __restrict__ insts, const ItemDev* __restrict__ items,
              const fx::TileGroup* __restrict__ groups, int items_per_block, int nblocks,
              int steps, int64_t* arena0, int64_t* arena1, ScaleSlot* slots, unsigned* done,
              unsigned* queue, int* err, unsigned wait_bias, long long wait_cycles) {
  extern __shared__ __align__(16) int64_t s_dyn[];  // plane history [K][R][threads]
  __shared__ int64_t s_row[2][W][32];
  __shared__ unsigned long long s_or[W];
  __shared__ int s_w;
  __shared__ int s_stop;
  __shared__ __align__(16) FixedArgs s_a;

  const long long total = (long long)nblocks * items_per_block;
  for (;;) {
    if (threadIdx.x == 0) {
      s_w = (int)atomicAdd(queue, 1u);
      s_stop = (*(volatile int*)err != 0);
    }
    __syncthreads();
    const int w = s_w;
    if (w >= total || s_stop) break;
    const int b = w / items_per_block;
    const int item = w - b * items_per_block;
    const ItemDev it = items[item];
    const int i = it.inst;
    const InstDev& I = insts[i];
    const int local = item - I.item_base;
    // the item's FixedArgs into shared memory: under the register cap the
    // tile loop re-reads the coefficients at every level, and a shared-memory
    // read is cheaper than a global one (the previous item's readers passed
    // the barrier at the end of its iteration)
    {
      static_assert(sizeof(FixedArgs) % 4 == 0, "FixedArgs is copied as 32-bit words");
      const int* src = reinterpret_cast<const int*>(&I.a);
      int* dst = reinterpret_cast<int*>(&s_a);
      for (int k = threadIdx.x; k < (int)(sizeof(FixedArgs) / 4); k += blockDim.x) dst[k] = src[k];
    }

    // wait until every block b-1 tile of this instance is done
    if (threadIdx.x == 0 && b > 0) {
      const unsigned need = (unsigned)b * (unsigned)I.items + wait_bias;
      const long long t0 = clock64();
      while (ld_acquire(done + i) < need) {
        if (clock64() - t0 > wait_cycles) {
          atomicOr(err, 2);
          s_stop = 1;
          break;
        }
        __nanosleep(200);
      }
    }
    __syncthreads();
    if (s_stop) break;

    ScaleSlot* sl = slots + 3 * i;
    int s, d;
    if (!scale_from_slot(sl + (b % 3), s_a.guard, &s, &d) && threadIdx.x == 0) atomicOr(err, 1);
    if (local == 0 && threadIdx.x == 0) {
      ScaleSlot* rs = sl + ((b + 2) % 3);
      rs->m = 0ull;
      rs->kind = 1;
      sl[(b + 1) % 3].s = s;
      sl[(b + 1) % 3].kind = 1;
    }
    // this thread's rectangle of the packed tile (lanes and warps past the
    // last full rectangle join the last one, beyond its outputs)
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int ncol = 32 / it.gw, nrow = W / it.gh;
    const int col = min(lane / it.gw, ncol - 1);
    const int rg = min(warp / it.gh, nrow - 1);
    const fx::TileGroup grp = groups[it.group_base + rg * ncol + col];
    const int levels = min(K, steps - b * K);
    const int64_t* in = ((b & 1) ? arena1 : arena0) + I.offset;
    int64_t* out = ((b & 1) ? arena0 : arena1) + I.offset;
    unsigned long long my_or = 0ull;
    fx::advance_tile<K, R, W, true, fx::kLoadL2Regs, false, false, true>(
        s_a, 0, 0, 0, it.nout, levels, b == 0, b == nblocks - 1, s, d, in, out, s_dyn, s_row,
        my_or, grp, lane - col * it.gw, (warp - rg * it.gh) * R);
    fx::cta_or<W>(my_or, s_or, &sl[(b + 1) % 3].m);
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) atomicAdd(done + i, 1u);
  }
}

// max|f| of every instance (FP64 bit patterns) into slot 0 of its ring, kind 0;
// slots 1 and 2 are cleared.  Block b works on instance b / per_inst.
__global__ void __launch_bounds__(256)
k_batch_absmax(const double* __restrict__ arena, const InstDev* __restrict__ insts, int count,
               int per_inst, ScaleSlot* slots) {
  __shared__ unsigned long long sh[8];
  const int i = blockIdx.x / per_inst;
  const int part = blockIdx.x - i * per_inst;
  if (i >= count) return;
  const InstDev& I = insts[i];
  const uint64_t n = (uint64_t)I.a.nx * I.a.ny * I.a.nz;
  unsigned long long m = 0ull;
  for (uint64_t k = (uint64_t)part * 256 + threadIdx.x; k < n; k += (uint64_t)per_inst * 256) {
    const unsigned long long bits =
        (unsigned long long)__double_as_longlong(__ldg(arena + I.offset + k)) & 0x7FFFFFFFFFFFFFFFull;
    m = bits > m ? bits : m;
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
    atomicMax(&slots[3 * i].m, m);
  }
}

__global__ void k_batch_slots_init(ScaleSlot* slots, int count) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < 3 * count; k += gridDim.x * blockDim.x) {
    slots[k].m = 0ull;
    slots[k].s = 0;
    slots[k].kind = (k % 3 == 0) ? 0 : 1;
  }
}

// per-instance sums: block b sums part (b % per_inst) of instance b / per_inst
__global__ void __launch_bounds__(256)
k_batch_sum_partial(const double* __restrict__ arena, const int64_t* __restrict__ offs,
                    const uint64_t* __restrict__ sizes, int count, int per_inst,
                    double* __restrict__ part) {
  __shared__ double sh[256];
  const int i = blockIdx.x / per_inst;
  const int pi = blockIdx.x - i * per_inst;
  const uint64_t n = sizes[i];
  const uint64_t chunk = (n + per_inst - 1) / per_inst;
  const uint64_t lo = (uint64_t)pi * chunk;
  const uint64_t hi = lo + chunk < n ? lo + chunk : n;
  double acc = 0.0;
  for (uint64_t k = lo + threadIdx.x; k < hi; k += 256) acc = acc + arena[offs[i] + k];
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int st = 128; st > 0; st >>= 1) {
    if (threadIdx.x < st) sh[threadIdx.x] = sh[threadIdx.x] + sh[threadIdx.x + st];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

__global__ void k_batch_sum_final(const double* __restrict__ part, int count, int per_inst,
                                  double* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  double acc = 0.0;
  for (int p = 0; p < per_inst; ++p) acc = acc + part[i * per_inst + p];
  out[i] = acc;
}

// One instance between the caller's axis order (the 3-D view (z, y, x) of
// its description, extents n) and the stored order (stored axis k = view
// axis p[k]): to_view = false writes dst in stored order from src in view
// order, true the other way.
__global__ void __launch_bounds__(256)
k_permute3(const double* __restrict__ src, double* __restrict__ dst, uint64_t n0, uint64_t n1,
           uint64_t n2, int p0, int p1, int p2, int to_view) {
  const uint64_t n[3] = {n0, n1, n2};
  const uint64_t e1 = n[p1], e2 = n[p2];
  const uint64_t total = n0 * n1 * n2;
  for (uint64_t i = blockIdx.x * 256ull + threadIdx.x; i < total; i += (uint64_t)gridDim.x * 256ull) {
    const uint64_t c2 = i % e2;
    const uint64_t t = i / e2;
    const uint64_t c1 = t % e1;
    const uint64_t c0 = t / e1;
    uint64_t r[3];
    r[p0] = c0;
    r[p1] = c1;
    r[p2] = c2;
    const uint64_t v = (r[0] * n1 + r[1]) * n2 + r[2];
    if (to_view)
      dst[v] = src[i];
    else
      dst[i] = src[v];
  }
}

// Extents, velocities and lengths of the 3-D view (z, y, x) of a described
// instance (missing leading axes: extent 1, velocity 0).
void view3(const Geom& g, uint64_t n[3], double v[3], double L[3]) {
  const int jj[3] = {g.jz, g.jy, g.jx};
  for (int a = 0; a < 3; ++a) {
    const int j = jj[a];
    n[a] = j < 0 ? 1 : g.n[j];
    v[a] = j < 0 ? 0.0 : g.v[j];
    L[a] = j < 0 ? 1.0 : g.L[j];
  }
}

// Packed tiles of one instance of nx x ny x nz cells (stored axes).  The x axis is cut
// into segments of 32 - K outputs (a warp's width) and a remainder of rx
// outputs (rx + K lanes); the y axis into ranges of R W - K outputs (all W
// warps) and a remainder of ry outputs (ceil((ry + K) / R) warps).  The
// rectangles of one size (lanes x warps) are packed side by side and stacked,
// (32 / lanes) x (W / warps) to a tile.  To fill the tiles, the z axis of
// those rectangles may be cut into s ranges of zl planes, each marched from
// its own K warm-up planes; s minimises tiles x planes (with tz > 0, a range
// holds at most tz planes).  The last range ends at the last plane and may
// overlap the one before: the cells of the overlap are computed from the same
// inputs by the same integer arithmetic in both and stored twice with the
// same value, which no tile reads before the next time block.  Every other
// output cell lies in exactly one rectangle.
int pack_instance(int nx, int ny, int nz, int inst, int K, int R, int W, int tz,
                  std::vector<ItemDev>* items, std::vector<fx::TileGroup>* groups) {
  struct Seg {
    int o, n, units;  // first output, outputs, lanes (x) or warps (y)
  };
  // [0]: full segments, [1]: the remainder (at most one)
  std::vector<Seg> xs[2], ys[2];
  const int Tx = 32 - K, Ty = R * W - K;
  for (int j = 0; j < nx / Tx; ++j) xs[0].push_back({j * Tx, Tx, 32});
  if (nx % Tx) xs[1].push_back({nx / Tx * Tx, nx % Tx, nx % Tx + K});
  for (int j = 0; j < ny / Ty; ++j) ys[0].push_back({j * Ty, Ty, W});
  if (ny % Ty) ys[1].push_back({ny / Ty * Ty, ny % Ty, (ny % Ty + K + R - 1) / R});
  for (int xc = 0; xc < 2; ++xc) {
    for (int yc = 0; yc < 2; ++yc) {
      if (xs[xc].empty() || ys[yc].empty()) continue;
      const int gw = xs[xc][0].units, gh = ys[yc][0].units;
      const int ncol = 32 / gw, nrow = W / gh, P = ncol * nrow;
      const int64_t c = (int64_t)xs[xc].size() * (int64_t)ys[yc].size();
      // z ranges: the count sp of ranges that minimises tiles x planes
      const int s_min = tz > 0 ? (nz + tz - 1) / tz : 1;
      const int s_max = std::min(nz, std::max(s_min, P));
      int zl_best = nz;
      int64_t best_cost = INT64_MAX;
      for (int sp = s_min; sp <= s_max; ++sp) {
        const int64_t zl = (nz + sp - 1) / sp;
        const int64_t zr = (nz + zl - 1) / zl;
        const int64_t cost = ((c * zr + P - 1) / P) * (zl + K);
        if (cost < best_cost) {
          best_cost = cost;
          zl_best = (int)zl;
        }
      }
      const int zl = zl_best;
      const int zr = (nz + zl - 1) / zl;
      int in_item = 0;
      for (const Seg& x : xs[xc]) {
        for (const Seg& y : ys[yc]) {
          for (int k = 0; k < zr; ++k) {
            if (in_item == 0) items->push_back({inst, gw, gh, (int)groups->size(), zl});
            fx::TileGroup g;
            g.x0 = x.o;
            g.xout = x.n;
            g.y0 = y.o;
            g.yout = y.n;
            g.z0 = (int)std::min<int64_t>((int64_t)k * zl, nz - zl);
            groups->push_back(g);
            if (++in_item == P) in_item = 0;
          }
        }
      }
      // the last tile's unused rectangles store nothing
      for (; in_item != 0 && in_item < P; ++in_item) groups->push_back(fx::TileGroup{});
    }
  }
  return FDB_OK;
}

// Tiles x planes marched per time block by pack_instance's tiles.
int64_t packed_cost(int nx, int ny, int nz, int K, int R, int W) {
  std::vector<ItemDev> items;
  std::vector<fx::TileGroup> groups;
  pack_instance(nx, ny, nz, 0, K, R, W, 0, &items, &groups);
  int64_t c = 0;
  for (const ItemDev& it : items) c += it.nout + K;
  return c;
}

// Stored order of an instance with view extents n: the permutation whose
// packed tiles (pack_instance at the default depth with 4 rows x 8 warps)
// march the fewest tile-planes per time block; ties keep the view order.
// Orders whose stored plane has 2^31 cells or more are skipped (the fixed
// kernel's limit).
std::array<int, 3> choose_order(const uint64_t n[3]) {
  static const int ps[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};
  std::array<int, 3> best = {0, 1, 2};
  int64_t best_cost = INT64_MAX;
  for (const auto& p : ps) {
    if (n[p[1]] * n[p[2]] >= (1ull << 31) || n[p[0]] >= (1ull << 31)) continue;
    const int64_t cost =
        packed_cost((int)n[p[2]], (int)n[p[1]], (int)n[p[0]], kDefaultDepth, 4, 8);
    if (cost < best_cost) {
      best_cost = cost;
      best = {p[0], p[1], p[2]};
    }
  }
  return best;
}

template <int K, int R, int W>
int launch_batch_kernel(int grid, const InstDev* insts, const ItemDev* items,
                        const fx::TileGroup* groups, int ipb, int nblocks, int steps, int64_t* a0,
                        int64_t* a1, ScaleSlot* slots, unsigned* done, unsigned* queue, int* err,
                        unsigned wait_bias, long long wait_cycles, cudaStream_t st) {
  constexpr int smem = K * R * 32 * W * (int)sizeof(int64_t);
  static bool configured = false;
  if (!configured) {
    cudaFuncSetAttribute(k_batch_fixed<K, R, W>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         smem);
    configured = true;
  }
  k_batch_fixed<K, R, W><<<grid, 32 * W, smem, st>>>(insts, items, groups, ipb, nblocks, steps,
                                                     a0, a1, slots, done, queue, err, wait_bias,
                                                     wait_cycles);
  return FDB_OK;
}

template <int K, int R, int W>
int resident_ctas_of() {
  constexpr int smem = K * R * 32 * W * (int)sizeof(int64_t);
  cudaFuncSetAttribute(k_batch_fixed<K, R, W>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch_fixed<K, R, W>, 32 * W, smem);
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return std::max(1, per_sm) * std::max(1, sms);
}

using LaunchFn = int (*)(int, const InstDev*, const ItemDev*, const fx::TileGroup*, int, int,
                         int, int64_t*, int64_t*,
                         ScaleSlot*, unsigned*, unsigned*, int*, unsigned, long long,
                         cudaStream_t);
using ResidentFn = int (*)();

struct Variant {
  int K, shape;
  LaunchFn launch;
  ResidentFn resident;
};

// compiled (K, shape) combinations of the batched kernel
const Variant kVariants[] = {
    {2, fx::kR4W16S, launch_batch_kernel<2, 4, 16>, resident_ctas_of<2, 4, 16>},
    {3, fx::kR4W16S, launch_batch_kernel<3, 4, 16>, resident_ctas_of<3, 4, 16>},
    {4, fx::kR4W16S, launch_batch_kernel<4, 4, 16>, resident_ctas_of<4, 4, 16>},
    {2, fx::kR4W8S, launch_batch_kernel<2, 4, 8>, resident_ctas_of<2, 4, 8>},
    {3, fx::kR4W8S, launch_batch_kernel<3, 4, 8>, resident_ctas_of<3, 4, 8>},
    {4, fx::kR4W8S, launch_batch_kernel<4, 4, 8>, resident_ctas_of<4, 4, 8>},
    {2, fx::kR8W8S, launch_batch_kernel<2, 8, 8>, resident_ctas_of<2, 8, 8>},
    {3, fx::kR8W8S, launch_batch_kernel<3, 8, 8>, resident_ctas_of<3, 8, 8>},
    {4, fx::kR8W8S, launch_batch_kernel<4, 8, 8>, resident_ctas_of<4, 8, 8>},
};

const Variant* find_variant(int K, int shape) {
  for (const Variant& v : kVariants)
    if (v.K == K && v.shape == shape) return &v;
  return nullptr;
}

}  // namespace bt
}  // namespace fdb

using namespace fdb;
using namespace fdb::bt;

struct fdb_batch {
  int count = 0;
  std::vector<Geom> geoms;      // as stored (the kernels' geometry)
  std::vector<Geom> geoms_ref;  // as described by the caller
  std::vector<std::array<int, 3>> order;  // stored axis k = view axis order[k]
  std::vector<char> permuted;
  double* d_stage = nullptr;  // one instance in the caller's order
  uint64_t stage_cells = 0;
  // batched adjoint storage (grown on demand): checkpoints, segment buffers
  // (two int64 chains, then int32 states two per buffer), adjoint ping-pong,
  // lambda_T / dL/df0 in the stored layout, the caller-order copy, scratch
  std::vector<double*> adj_ckpt, adj_seg;
  double* adj_lam[2] = {nullptr, nullptr};
  double* adj_io[2] = {nullptr, nullptr};
  double* adj_user = nullptr;
  double* adj_dda = nullptr;
  void* adj_scratch = nullptr;
  size_t adj_scratch_bytes = 0;
  // plans built while set step the transposed problem (every upwind
  // direction reversed, the coefficients unchanged): the dL/df0-only adjoint
  bool transposed_run = false;
  // adjoint form (FDB_TUNE_ADJOINT): 0 = dL/dv in closed form, 1 = step by step
  int adj_mode = 0;
  DeviceScratch contract;  // the closed form's contraction tables and partials
  std::vector<int64_t> offsets;  // cells
  std::vector<uint64_t> sizes;
  int64_t total = 0;
  double* arena[2] = {nullptr, nullptr};
  int cur = 0;
  // device tables
  InstDev* d_insts = nullptr;
  ItemDev* d_items = nullptr;
  size_t item_cap = 0;
  fx::TileGroup* d_groups = nullptr;
  size_t group_cap = 0;
  ScaleSlot* d_slots = nullptr;
  unsigned* d_done = nullptr;
  unsigned* d_queue = nullptr;
  int* d_err = nullptr;
  int64_t* d_offs = nullptr;
  uint64_t* d_sizes = nullptr;
  double* d_part = nullptr;
  double* d_sums = nullptr;
  double* h_sums = nullptr;
  double* d_plain_scratch = nullptr;  // per-instance scratch of the looped comparator
  cudaStream_t own = nullptr, stream = nullptr;
  // tuning (0 / -1 = automatic)
  int K = 0, shape = -1, tz = 0;
  // graph cache
  cudaGraphExec_t graph = nullptr;
  std::string graph_key;
};

namespace {

constexpr int kSumPerInst = 16;

int bcheck(fdb_batch* b) {
  if (!b) return fail(FDB_ERR_INVALID, "null batch");
  return FDB_OK;
}

int bsync(fdb_batch* b) {
  FDB_CUDA_TRY(cudaStreamSynchronize(b->stream));
  int herr = 0;
  FDB_CUDA_TRY(cudaMemcpy(&herr, b->d_err, sizeof(int), cudaMemcpyDeviceToHost));
  if (herr) {
    FDB_CUDA_TRY(cudaMemset(b->d_err, 0, sizeof(int)));
    if (herr & 2)
      return fail(FDB_ERR_TIMEOUT, "batched kernel: a bounded wait for a neighbour tile expired");
    return fail(FDB_ERR_NONFINITE, "batched kernel: an instance field holds NaN or Inf");
  }
  return FDB_OK;
}

template <typename T>
int balloc(T** p, size_t count) {
  if (fault_injected("alloc")) return fail(FDB_ERR_INJECTED, "injected allocation failure");
  cudaError_t e = cudaMalloc((void**)p, std::max<size_t>(count, 1) * sizeof(T));
  if (e != cudaSuccess) {
    *p = nullptr;
    cudaGetLastError();
    return fail(FDB_ERR_ALLOC, std::string("cudaMalloc failed: ") + cudaGetErrorString(e));
  }
  return FDB_OK;
}

void drop_graph(fdb_batch* b) {
  if (b->graph) cudaGraphExecDestroy(b->graph);
  b->graph = nullptr;
  b->graph_key.clear();
}

int check_dts(fdb_batch* b, const double* dt) {
  if (!dt) return fail(FDB_ERR_INVALID, "null dt array");
  for (int i = 0; i < b->count; ++i)
    if (!isfinite(dt[i])) return fail(FDB_ERR_INVALID, "dt must be finite");
  return FDB_OK;
}

struct Plan {
  int K, shape, tz;
  const Variant* v;
  std::vector<InstDev> insts;
  std::vector<ItemDev> items;
  std::vector<fx::TileGroup> groups;
  int ipb = 0;
  int nblocks = 0;
  int grid = 0;
};

int make_plan(fdb_batch* b, int steps, const double* dt, int K, int shape, int tz, Plan* p) {
  p->K = K;
  p->shape = shape;
  p->tz = tz;
  p->v = find_variant(K, shape);
  if (!p->v) return fail(FDB_ERR_UNSUPPORTED, "no batched kernel compiled for this depth/shape");
  p->insts.resize(b->count);
  p->items.clear();
  p->groups.clear();
  const int resident = p->v->resident();
  const int R = fx::shape_rows(shape), W = fx::shape_warps(shape);
  int base = 0;
  for (int i = 0; i < b->count; ++i) {
    const Geom& g = b->geoms[i];
    const Coeffs3 c = coeffs3(g, dt[i]);
    if (fixed_supported(g, c, K) != FDB_OK) return FDB_ERR_UNSUPPORTED;
    InstDev& I = p->insts[i];
    // per instance: whole z extent per tile unless tz is given (many small
    // instances already fill the device)
    I.a = make_fixed_args(b->transposed_run ? transposed_geom(g) : g, c, shape, K,
                          tz > 0 ? tz : (int)g.nz, resident);
    I.a.scale_log = nullptr;
    I.offset = b->offsets[i];
    const size_t first = p->items.size();
    FDB_TRY(pack_instance(I.a.nx, I.a.ny, I.a.nz, i, K, R, W, tz, &p->items, &p->groups));
    const size_t items = p->items.size() - first;
    if (items > (1u << 24)) return fail(FDB_ERR_UNSUPPORTED, "instance has too many tiles");
    I.items = (int)items;
    I.item_base = base;
    base += I.items;
  }
  if (p->groups.size() >= (1ull << 31))
    return fail(FDB_ERR_UNSUPPORTED, "batched plan exceeds 2^31 tile rectangles");
  p->ipb = base;
  p->nblocks = (steps + K - 1) / K;
  if ((int64_t)p->nblocks * p->ipb >= (1ll << 31))
    return fail(FDB_ERR_UNSUPPORTED, "batched work queue exceeds 2^31 items");
  p->grid = (int)std::min<int64_t>((int64_t)p->nblocks * p->ipb, resident);
  return FDB_OK;
}

// Enqueue one batched advect (not captured).
int enqueue_advect(fdb_batch* b, const Plan& p, int steps, cudaStream_t st) {
  FDB_CUDA_TRY(cudaMemsetAsync(b->d_queue, 0, sizeof(unsigned), st));
  FDB_CUDA_TRY(cudaMemsetAsync(b->d_done, 0, b->count * sizeof(unsigned), st));
  k_batch_slots_init<<<(3 * b->count + 255) / 256, 256, 0, st>>>(b->d_slots, b->count);
  const int per_inst = 8;
  k_batch_absmax<<<b->count * per_inst, 256, 0, st>>>(b->arena[b->cur], b->d_insts, b->count,
                                                       per_inst, b->d_slots);
  int64_t* a0 = (int64_t*)b->arena[b->cur];
  int64_t* a1 = (int64_t*)b->arena[b->cur ^ 1];
  // FDB_FAULT=timeout makes every dependency unsatisfiable and the wait
  // budget ~1 ms, so the bounded-wait error path runs without a GPU fault
  const bool inject = fault_injected("timeout");
  p.v->launch(p.grid, b->d_insts, b->d_items, b->d_groups, p.ipb, p.nblocks, steps, a0, a1,
              b->d_slots, b->d_done, b->d_queue, b->d_err, inject ? (1u << 30) : 0u,
              inject ? 2000000ll : kWaitCycles, st);
  note_launch(3);
  FDB_CUDA_TRY(cudaGetLastError());
  return FDB_OK;
}

int upload_plan(fdb_batch* b, const Plan& p) {
  if (p.items.size() > b->item_cap) {
    if (b->d_items) cudaFree(b->d_items);
    b->d_items = nullptr;
    b->item_cap = 0;
    FDB_TRY(balloc(&b->d_items, p.items.size()));
    b->item_cap = p.items.size();
  }
  if (p.groups.size() > b->group_cap) {
    if (b->d_groups) cudaFree(b->d_groups);
    b->d_groups = nullptr;
    b->group_cap = 0;
    FDB_TRY(balloc(&b->d_groups, p.groups.size()));
    b->group_cap = p.groups.size();
  }
  FDB_CUDA_TRY(cudaMemcpyAsync(b->d_insts, p.insts.data(), p.insts.size() * sizeof(InstDev),
                               cudaMemcpyHostToDevice, b->stream));
  FDB_CUDA_TRY(cudaMemcpyAsync(b->d_items, p.items.data(), p.items.size() * sizeof(ItemDev),
                               cudaMemcpyHostToDevice, b->stream));
  FDB_CUDA_TRY(cudaMemcpyAsync(b->d_groups, p.groups.data(),
                               p.groups.size() * sizeof(fx::TileGroup), cudaMemcpyHostToDevice,
                               b->stream));
  return FDB_OK;
}

std::string plan_key(fdb_batch* b, int steps, const double* dt, const Plan& p) {
  std::ostringstream os;
  os << steps << ':' << p.K << ':' << p.shape << ':' << p.tz << ':' << b->cur << ':'
     << (void*)b->stream << ':' << b->transposed_run;
  uint64_t h = 1469598103934665603ull;
  for (int i = 0; i < b->count; ++i) {
    uint64_t x;
    memcpy(&x, &dt[i], 8);
    h = (h ^ x) * 1099511628211ull;
  }
  os << ':' << h;
  return os.str();
}

int run_batched(fdb_batch* b, int steps, const double* dt, int K, int shape, int tz,
                bool use_graph) {
  Plan p;
  const int rc = make_plan(b, steps, dt, K, shape, tz, &p);
  if (rc) return rc;
  const std::string key = plan_key(b, steps, dt, p);
  if (fault_injected("timeout")) use_graph = false;
  if (use_graph && b->graph && key == b->graph_key) {
    FDB_CUDA_TRY(cudaGraphLaunch(b->graph, b->stream));
    note_launch(3);
  } else {
    FDB_TRY(upload_plan(b, p));
    if (use_graph) {
      drop_graph(b);
      cudaStream_t cs = nullptr;
      FDB_CUDA_TRY(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
      // the plan upload above is ordered before the capture stream's work
      cudaStreamSynchronize(b->stream);
      cudaGraph_t graph = nullptr;
      cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
      int rc2 = FDB_OK;
      if (e == cudaSuccess) {
        rc2 = enqueue_advect(b, p, steps, cs);
        e = cudaStreamEndCapture(cs, &graph);
      }
      if (e == cudaSuccess && rc2 == FDB_OK)
        e = cudaGraphInstantiate(&b->graph, graph, 0);
      if (graph) cudaGraphDestroy(graph);
      cudaStreamDestroy(cs);
      if (rc2) return rc2;
      FDB_CUDA_TRY(e);
      b->graph_key = key;
      FDB_CUDA_TRY(cudaGraphLaunch(b->graph, b->stream));
    } else {
      drop_graph(b);  // the device tables now hold this plan, not the cached graph's
      FDB_TRY(enqueue_advect(b, p, steps, b->stream));
    }
  }
  b->cur ^= (p.nblocks & 1);
  return FDB_OK;
}

// The comparator: the plain per-field kernels looped over the instances,
// K steps per fixed-point launch; K <= 0: what fdb_upwind_advect runs for
// each instance (the fixed kernel at its default depth where it is
// supported and preferred, the FP64 kernel otherwise).  Every instance ends
// in the same arena: the one most instances end in; the others are copied
// across.
int run_looped(fdb_batch* b, int steps, const double* dt, int K) {
  const size_t per = (fixed_scratch_bytes() + 7) / 8;
  std::vector<int> fin(b->count);
  for (int i = 0; i < b->count; ++i) {
    const Geom& g = b->geoms[i];
    const Coeffs3 c = coeffs3(g, dt[i]);
    double* bufs[2] = {b->arena[0] + b->offsets[i], b->arena[1] + b->offsets[i]};
    int cur = b->cur;
    // depth and arithmetic as fdb_upwind_advect picks them for the described
    // instance (the stored order does not change the fixed-point result)
    const Geom& gr = b->geoms_ref[i];
    FixedTuning t;
    t.depth = K > 0 ? K : default_depth(gr);
    if (fixed_supported(g, c, t.depth) == FDB_OK && (K > 0 || fixed_preferred(gr))) {
      FDB_TRY(launch_advect_fixed_ex(g, c, steps, t, bufs, &cur, b->d_plain_scratch + i * per,
                                     per * 8, nullptr, b->stream));
    } else {
      for (int s = 0; s < steps; ++s) {
        FDB_TRY(launch_step_f64(g, c, FDB_ARITH_FMA, bufs[cur], bufs[cur ^ 1], b->stream));
        cur ^= 1;
      }
    }
    fin[i] = cur;
  }
  int ones = 0;
  for (int i = 0; i < b->count; ++i) ones += fin[i];
  const int new_cur = 2 * ones > b->count ? 1 : 0;
  for (int i = 0; i < b->count; ++i) {
    if (fin[i] == new_cur) continue;
    FDB_CUDA_TRY(cudaMemcpyAsync(b->arena[new_cur] + b->offsets[i], b->arena[fin[i]] + b->offsets[i],
                                 b->sizes[i] * 8, cudaMemcpyDeviceToDevice, b->stream));
  }
  b->cur = new_cur;
  return FDB_OK;
}

int effective_K(fdb_batch* b) { return b->K > 0 ? b->K : kDefaultDepth; }

void free_batch_adjoint(fdb_batch* b) {
  for (double* p : b->adj_ckpt) cudaFree(p);
  for (double* p : b->adj_seg) cudaFree(p);
  b->adj_ckpt.clear();
  b->adj_seg.clear();
  for (double*& p : b->adj_lam) {
    if (p) cudaFree(p);
    p = nullptr;
  }
  for (double*& p : b->adj_io) {
    if (p) cudaFree(p);
    p = nullptr;
  }
  if (b->adj_user) cudaFree(b->adj_user);
  if (b->adj_dda) cudaFree(b->adj_dda);
  if (b->adj_scratch) cudaFree(b->adj_scratch);
  b->adj_user = nullptr;
  b->adj_dda = nullptr;
  b->adj_scratch = nullptr;
  b->adj_scratch_bytes = 0;
}

// instance i between the caller's order and the stored order (see k_permute3)
int launch_permute(fdb_batch* b, int i, const double* src, double* dst, bool to_view) {
  uint64_t n3[3];
  double v3[3], L3[3];
  view3(b->geoms_ref[i], n3, v3, L3);
  const std::array<int, 3>& o = b->order[i];
  const uint64_t blocks = std::min<uint64_t>((b->sizes[i] + 255) / 256, 152 * 16);
  k_permute3<<<(unsigned)blocks, 256, 0, b->stream>>>(src, dst, n3[0], n3[1], n3[2], o[0], o[1],
                                                       o[2], to_view ? 1 : 0);
  note_launch();
  FDB_CUDA_TRY(cudaGetLastError());
  return FDB_OK;
}
int effective_shape(fdb_batch* b) { return b->shape >= 0 ? b->shape : fx::kR4W8S; }

}  // namespace

extern "C" {

int fdb_batch_create(int count, const fdb_instance_desc* descs, fdb_batch** out) {
  if (!out) return fail(FDB_ERR_INVALID, "null output batch pointer");
  *out = nullptr;
  if (count <= 0 || !descs) return fail(FDB_ERR_INVALID, "count must be > 0 with descriptors");
  fdb_batch* b = new fdb_batch();
  b->count = count;
  for (int i = 0; i < count; ++i) {
    Geom g;
    const fdb_instance_desc& d = descs[i];
    if (d.ndims < 1 || d.ndims > 3) {
      delete b;
      return fail(FDB_ERR_INVALID, "batched instances have 1 to 3 axes");
    }
    int rc = make_geom(d.ndims, d.velocity, d.lengths, d.num_cells, &g);
    if (rc) {
      delete b;
      return rc;
    }
    // stored order: permuted only where the single-field path would run the
    // (order-independent) fixed kernel
    uint64_t n3[3];
    double v3[3], L3[3];
    view3(g, n3, v3, L3);
    const std::array<int, 3> ord =
        fixed_preferred(g) ? choose_order(n3) : std::array<int, 3>{0, 1, 2};
    const bool perm = !(ord[0] == 0 && ord[1] == 1 && ord[2] == 2);
    Geom gs = g;
    if (perm) {
      uint64_t np[3];
      double vp[3], Lp[3];
      for (int k = 0; k < 3; ++k) {
        np[k] = n3[ord[k]];
        vp[k] = v3[ord[k]];
        Lp[k] = L3[ord[k]];
      }
      rc = make_geom(3, vp, Lp, np, &gs);
      if (rc) {
        delete b;
        return rc;
      }
      b->stage_cells = std::max<uint64_t>(b->stage_cells, g.ntot);
    }
    b->geoms.push_back(gs);
    b->geoms_ref.push_back(g);
    b->order.push_back(ord);
    b->permuted.push_back(perm ? 1 : 0);
    b->offsets.push_back(b->total);
    b->sizes.push_back(g.ntot);
    // keep every instance 256-byte aligned in the arenas
    b->total += (int64_t)((g.ntot + 31) / 32 * 32);
  }
  cudaError_t e = cudaStreamCreateWithFlags(&b->own, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete b;
    return cuda_fail(e, "cudaStreamCreate");
  }
  b->stream = b->own;
  const size_t per = (fixed_scratch_bytes() + 7) / 8;
  int rc = FDB_OK;
  if ((rc = balloc(&b->arena[0], b->total)) || (rc = balloc(&b->arena[1], b->total)) ||
      (rc = balloc(&b->d_insts, count)) || (rc = balloc(&b->d_slots, 3 * count)) ||
      (rc = balloc(&b->d_done, count)) || (rc = balloc(&b->d_queue, 1)) ||
      (rc = balloc(&b->d_err, 1)) || (rc = balloc(&b->d_offs, count)) ||
      (rc = balloc(&b->d_sizes, count)) || (rc = balloc(&b->d_part, count * kSumPerInst)) ||
      (rc = balloc(&b->d_sums, count)) || (rc = balloc(&b->d_plain_scratch, per * count)) ||
      (b->stage_cells && (rc = balloc(&b->d_stage, b->stage_cells)))) {
    fdb_batch_destroy(b);
    return rc;
  }
  e = cudaMallocHost((void**)&b->h_sums, count * sizeof(double));
  if (e == cudaSuccess) e = cudaMemsetAsync(b->d_err, 0, sizeof(int), b->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(b->d_plain_scratch, 0, per * count * 8, b->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(b->arena[0], 0, b->total * 8, b->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(b->d_offs, b->offsets.data(), count * 8, cudaMemcpyHostToDevice, b->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(b->d_sizes, b->sizes.data(), count * 8, cudaMemcpyHostToDevice, b->stream);
  if (e != cudaSuccess) {
    fdb_batch_destroy(b);
    return cuda_fail(e, "batch set-up");
  }
  // each instance starts like the reference constructor: f = 0, f[0] = 1
  for (int i = 0; i < count && !rc; ++i)
    rc = launch_fill_corner(b->arena[0] + b->offsets[i], b->sizes[i], b->stream);
  if (!rc) rc = bsync(b);
  if (rc) {
    fdb_batch_destroy(b);
    return rc;
  }
  *out = b;
  return FDB_OK;
}

int fdb_batch_destroy(fdb_batch* b) {
  if (!b) return FDB_OK;
  if (b->stream) cudaStreamSynchronize(b->stream);
  drop_graph(b);
  void* ps[] = {b->arena[0], b->arena[1], b->d_insts, b->d_items,  b->d_groups,
                b->d_slots,  b->d_done,  b->d_queue, b->d_err,    b->d_offs,
                b->d_sizes,  b->d_part,  b->d_sums,  b->d_plain_scratch, b->d_stage};
  for (void* p : ps)
    if (p) cudaFree(p);
  free_batch_adjoint(b);
  b->contract.release();
  if (b->h_sums) cudaFreeHost(b->h_sums);
  if (b->own) cudaStreamDestroy(b->own);
  delete b;
  return FDB_OK;
}

int fdb_batch_set_velocity(fdb_batch* b, int index, const double* velocity) {
  FDB_TRY(bcheck(b));
  if (index < 0 || index >= b->count || !velocity)
    return fail(FDB_ERR_INVALID, "bad index or velocity");
  const Geom& old = b->geoms_ref[index];
  Geom g;
  FDB_TRY(make_geom(old.ndims, velocity, old.L, old.n, &g));
  Geom gs = g;
  if (b->permuted[index]) {
    uint64_t n3[3];
    double v3[3], L3[3];
    view3(g, n3, v3, L3);
    uint64_t np[3];
    double vp[3], Lp[3];
    const std::array<int, 3>& o = b->order[index];
    for (int k = 0; k < 3; ++k) {
      np[k] = n3[o[k]];
      vp[k] = v3[o[k]];
      Lp[k] = L3[o[k]];
    }
    FDB_TRY(make_geom(3, vp, Lp, np, &gs));
  }
  FDB_TRY(bsync(b));
  b->geoms_ref[index] = g;
  b->geoms[index] = gs;
  drop_graph(b);
  return FDB_OK;
}

int fdb_batch_storage_order(fdb_batch* b, int index, int* order3) {
  FDB_TRY(bcheck(b));
  if (index < 0 || index >= b->count || !order3) return fail(FDB_ERR_INVALID, "bad index or output");
  for (int k = 0; k < 3; ++k) order3[k] = b->order[index][k];
  return FDB_OK;
}

int fdb_batch_count(fdb_batch* b, int* count, uint64_t* total_cells) {
  FDB_TRY(bcheck(b));
  if (count) *count = b->count;
  if (total_cells) {
    uint64_t t = 0;
    for (uint64_t s : b->sizes) t += s;
    *total_cells = t;
  }
  return FDB_OK;
}

int fdb_batch_set_field(fdb_batch* b, int index, const double* src, int is_device) {
  FDB_TRY(bcheck(b));
  if (index < 0 || index >= b->count || !src) return fail(FDB_ERR_INVALID, "bad index or source");
  double* dst = b->arena[b->cur] + b->offsets[index];
  const bool perm = b->permuted[index];
  FDB_CUDA_TRY(cudaMemcpyAsync(perm ? b->d_stage : dst, src, b->sizes[index] * 8,
                               is_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                               b->stream));
  if (perm) FDB_TRY(launch_permute(b, index, b->d_stage, dst, false));
  return bsync(b);
}

int fdb_batch_get_field(fdb_batch* b, int index, double* dst, int is_device) {
  FDB_TRY(bcheck(b));
  if (index < 0 || index >= b->count || !dst) return fail(FDB_ERR_INVALID, "bad index or destination");
  const double* src = b->arena[b->cur] + b->offsets[index];
  const bool perm = b->permuted[index];
  if (perm) FDB_TRY(launch_permute(b, index, src, b->d_stage, true));
  FDB_CUDA_TRY(cudaMemcpyAsync(dst, perm ? b->d_stage : src, b->sizes[index] * 8,
                               is_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                               b->stream));
  return bsync(b);
}

int fdb_batch_init_sphere(fdb_batch* b, int index, const double* center, double radius,
                          double noise_amp, uint64_t seed) {
  FDB_TRY(bcheck(b));
  if (index < 0 || index >= b->count || !center) return fail(FDB_ERR_INVALID, "bad index or centre");
  double* dst = b->arena[b->cur] + b->offsets[index];
  const bool perm = b->permuted[index];
  // generated in the caller's order (the generator is a function of the
  // reference's cell index), then stored
  FDB_TRY(launch_sphere_noise(b->geoms_ref[index], center, radius, noise_amp, seed,
                              perm ? b->d_stage : dst, b->stream));
  if (perm) FDB_TRY(launch_permute(b, index, b->d_stage, dst, false));
  return bsync(b);
}

int fdb_batch_set_stream(fdb_batch* b, void* cuda_stream) {
  FDB_TRY(bcheck(b));
  FDB_TRY(bsync(b));
  b->stream = cuda_stream ? (cudaStream_t)cuda_stream : b->own;
  drop_graph(b);
  return FDB_OK;
}

int fdb_batch_set_tuning(fdb_batch* b, int key, int value) {
  FDB_TRY(bcheck(b));
  if (key == FDB_TUNE_DEPTH) {
    if (value < 0 || value == 1 || value > 4) return fail(FDB_ERR_INVALID, "batched depth is 0, 2, 3 or 4");
    b->K = value;
  } else if (key == FDB_TUNE_SHAPE) {
    if (!(value == -1 || value == fx::kR4W16S || value == fx::kR4W8S || value == fx::kR8W8S))
      return fail(FDB_ERR_INVALID, "batched shape is -1, 2 (8x8), 3 (4x16) or 4 (4x8)");
    b->shape = value;
  } else if (key == FDB_TUNE_TILE_Z) {
    if (value < 0) return fail(FDB_ERR_INVALID, "tile_z must be >= 0");
    b->tz = value;
  } else if (key == FDB_TUNE_ADJOINT) {
    if (value < 0 || value > 2) return fail(FDB_ERR_INVALID, "adjoint form must be 0, 1 or 2");
    b->adj_mode = value;
    return FDB_OK;
  } else {
    return fail(FDB_ERR_INVALID, "unknown tuning key");
  }
  drop_graph(b);
  return FDB_OK;
}

int fdb_batch_advect(fdb_batch* b, int num_steps, const double* dt) {
  NvtxScope nvtx_("fdb.batch.advect");
  FDB_TRY(bcheck(b));
  if (num_steps < 0) return fail(FDB_ERR_INVALID, "num_steps must be >= 0");
  FDB_TRY(check_dts(b, dt));
  if (num_steps == 0) return FDB_OK;
  const int rc = run_batched(b, num_steps, dt, effective_K(b), effective_shape(b), b->tz, true);
  if (rc == FDB_ERR_UNSUPPORTED) {
    // some instance is outside the fixed kernel's domain: loop the plain path
    return run_looped(b, num_steps, dt, effective_K(b));
  }
  return rc;
}

int fdb_batch_advect_looped(fdb_batch* b, int num_steps, const double* dt) {
  NvtxScope nvtx_("fdb.batch.advect_looped");
  FDB_TRY(bcheck(b));
  if (num_steps < 0) return fail(FDB_ERR_INVALID, "num_steps must be >= 0");
  FDB_TRY(check_dts(b, dt));
  if (num_steps == 0) return FDB_OK;
  return run_looped(b, num_steps, dt, b->K);
}

// The transposed problems run on the adjoint buffers adj_lam[0..1] (the
// fields are untouched): each instance's upwind directions reversed, its
// coefficients unchanged, in its storage order.
//
// adj_lam[0] = the caller's concatenated fields `in`, permuted into the
// storage order; `pref` receives where each instance starts in the caller's
// layout.
static int batch_lam_load(fdb_batch* b, const double* in, int is_device,
                          std::vector<uint64_t>& pref) {
  const int n = b->count;
  const size_t T = (size_t)b->total;
  int rc = FDB_OK;
  for (auto& p : b->adj_lam)
    if (!rc && !p) rc = balloc(&p, T);
  if (!rc && !b->adj_user) rc = balloc(&b->adj_user, T);
  if (rc) {
    free_batch_adjoint(b);
    return rc;
  }
  pref.assign(n, 0);
  uint64_t cells = 0;
  for (int i = 0; i < n; ++i) {
    pref[i] = cells;
    cells += b->sizes[i];
  }
  const double* lt = in;
  if (!is_device) {
    FDB_CUDA_TRY(cudaMemcpyAsync(b->adj_user, in, cells * 8, cudaMemcpyHostToDevice,
                                 b->stream));
    lt = b->adj_user;
  }
  for (int i = 0; i < n; ++i) {
    double* dst = b->adj_lam[0] + b->offsets[i];
    if (b->permuted[i])
      FDB_TRY(launch_permute(b, i, lt + pref[i], dst, false));
    else
      FDB_CUDA_TRY(cudaMemcpyAsync(dst, lt + pref[i], b->sizes[i] * 8, cudaMemcpyDeviceToDevice,
                                   b->stream));
  }
  return FDB_OK;
}

// S transposed steps of every instance: the persistent launch on the adjoint
// buffers; *lc (in/out) names the buffer that holds the state.
static int batch_lam_steps(fdb_batch* b, int S, const double* dt, int* lc) {
  if (S <= 0) return FDB_OK;
  const int cur = b->cur;
  std::swap(b->arena[0], b->adj_lam[0]);
  std::swap(b->arena[1], b->adj_lam[1]);
  b->cur = *lc;
  b->transposed_run = true;
  const int rc = run_batched(b, S, dt, effective_K(b), effective_shape(b), b->tz, false);
  *lc = b->cur;
  std::swap(b->arena[0], b->adj_lam[0]);
  std::swap(b->arena[1], b->adj_lam[1]);
  b->cur = cur;
  b->transposed_run = false;
  return rc;
}

// adj_lam[lc] back to the caller's order into `out`.
static int batch_lam_store(fdb_batch* b, int lc, double* out, int is_device,
                           const std::vector<uint64_t>& pref) {
  const int n = b->count;
  double* gd = is_device ? out : b->adj_user;
  for (int i = 0; i < n; ++i) {
    const double* src = b->adj_lam[lc] + b->offsets[i];
    if (b->permuted[i])
      FDB_TRY(launch_permute(b, i, src, gd + pref[i], true));
    else
      FDB_CUDA_TRY(cudaMemcpyAsync(gd + pref[i], src, b->sizes[i] * 8, cudaMemcpyDeviceToDevice,
                                   b->stream));
  }
  if (!is_device) {
    const uint64_t cells = n ? pref[n - 1] + b->sizes[n - 1] : 0;
    FDB_CUDA_TRY(cudaMemcpyAsync(out, b->adj_user, cells * 8, cudaMemcpyDeviceToHost,
                                 b->stream));
  }
  return FDB_OK;
}

// out = (A^T)^S in for all instances at once; the fields are untouched.
static int batch_transposed(fdb_batch* b, int S, const double* dt, const double* lambda_T,
                            double* grad_f0, int is_device) {
  std::vector<uint64_t> pref;
  FDB_TRY(batch_lam_load(b, lambda_T, is_device, pref));
  int lc = 0;
  FDB_TRY(batch_lam_steps(b, S, dt, &lc));
  FDB_TRY(batch_lam_store(b, lc, grad_f0, is_device, pref));
  return bsync(b);
}

// dL/dv of every instance from dL/da of its stored axes: stored axis k is
// view axis order[k], i.e. reference axis jj[order[k]];
// a_j = -dt v_j up_j / dx_j  =>  dL/dv_j = dL/da_j (-dt up_j / dx_j).
static void batch_velocity_grad(fdb_batch* b, const double* dt, const double* dda,
                                double* grad_v) {
  for (int i = 0; i < b->count; ++i) {
    const Geom& gr = b->geoms_ref[i];
    const int jj[3] = {gr.jz, gr.jy, gr.jx};
    for (int k = 0; k < 3; ++k) grad_v[3 * i + k] = 0.0;
    for (int k = 0; k < 3; ++k) {
      const int j = jj[b->order[i][k]];
      if (j >= 0) grad_v[3 * i + j] = dda[3 * i + k] * (-dt[i] * (double)gr.up[j] / gr.dx[j]);
    }
  }
}

// The full gradient in closed form for every instance (the single-field
// derivation: A, A^T and every D_j commute on the periodic grid, so
// dL/da_j = S <lam^1, D_j f0> with lam^1 = (A^T)^(S-1) lam_T): S - 1
// transposed steps, one contraction per instance with its field (still f0),
// the last transposed step, then the forward advect to f_T.
static int batch_adjoint_closed_form(fdb_batch* b, int S, const double* dt,
                                     const double* lambda_T, double* grad_f0, double* grad_v,
                                     int is_device, bool advance_fields) {
  const int n = b->count;
  if (!b->adj_dda) FDB_TRY(balloc(&b->adj_dda, 3 * (size_t)n));
  std::vector<uint64_t> pref;
  FDB_TRY(batch_lam_load(b, lambda_T, is_device, pref));
  int lc = 0;
  FDB_TRY(batch_lam_steps(b, S - 1, dt, &lc));
  FDB_TRY(launch_vel_contract(n, b->geoms.data(), b->offsets.data(), b->arena[b->cur],
                              b->adj_lam[lc], b->adj_dda, b->contract, b->stream));
  FDB_TRY(batch_lam_steps(b, 1, dt, &lc));
  FDB_TRY(batch_lam_store(b, lc, grad_f0, is_device, pref));
  if (advance_fields)
    FDB_TRY(run_batched(b, S, dt, effective_K(b), effective_shape(b), b->tz, true));
  std::vector<double> dda(3 * (size_t)n);
  FDB_CUDA_TRY(cudaMemcpyAsync(dda.data(), b->adj_dda, dda.size() * 8, cudaMemcpyDeviceToHost,
                               b->stream));
  FDB_TRY(bsync(b));
  for (double& x : dda) x *= (double)S;
  batch_velocity_grad(b, dt, dda.data(), grad_v);
  return FDB_OK;
}

// dL/df0 only (fdb_batch_adjoint with grad_v = NULL): the batch advances to
// f_T, then the transposed launch gives (A^T)^S lambda_T.
static int batch_adjoint_f0_only(fdb_batch* b, int S, const double* dt, const double* lambda_T,
                                 double* grad_f0, int is_device) {
  if (S > 0 && b->adj_mode != 2)  // form 2 keeps the fields at f0
    FDB_TRY(run_batched(b, S, dt, effective_K(b), effective_shape(b), b->tz, true));
  return batch_transposed(b, S, dt, lambda_T, grad_f0, is_device);
}

int fdb_batch_advect_transposed(fdb_batch* b, int num_steps, const double* dt, const double* in,
                                double* out, int is_device) {
  NvtxScope nvtx_("fdb.batch.advect_transposed");
  FDB_TRY(bcheck(b));
  if (num_steps < 0) return fail(FDB_ERR_INVALID, "num_steps must be >= 0");
  FDB_TRY(check_dts(b, dt));
  if (!in || !out) return fail(FDB_ERR_INVALID, "null input or output");
  return batch_transposed(b, num_steps, dt, in, out, is_device);
}

int fdb_batch_adjoint(fdb_batch* b, int num_steps, const double* dt, const double* lambda_T,
                      double* grad_f0, double* grad_v, int checkpoint_every, int is_device) {
  NvtxScope nvtx_("fdb.batch.adjoint");
  FDB_TRY(bcheck(b));
  if (num_steps < 0) return fail(FDB_ERR_INVALID, "num_steps must be >= 0");
  FDB_TRY(check_dts(b, dt));
  if (!lambda_T || !grad_f0) return fail(FDB_ERR_INVALID, "null lambda_T or grad_f0");
  if (checkpoint_every < 0) return fail(FDB_ERR_INVALID, "checkpoint_every must be >= 0");
  const int S = num_steps;
  int K = checkpoint_every;
  if (K == 0) K = std::max(1, (int)ceil(sqrt((double)std::max(S, 1))));
  if (K > std::max(S, 1)) K = std::max(S, 1);
  const int nseg = (S + K - 1) / K;
  const int n = b->count;
  if (!grad_v) return batch_adjoint_f0_only(b, S, dt, lambda_T, grad_f0, is_device);
  // every instance in the fixed kernel's domain (forward and transposed steps)
  std::vector<Coeffs3> cs(n);
  for (int i = 0; i < n; ++i) {
    cs[i] = coeffs3(b->geoms[i], dt[i]);
    if (fixed_supported(b->geoms[i], cs[i], 1) != FDB_OK ||
        fixed_supported(b->geoms[i], cs[i], effective_K(b)) != FDB_OK)
      return fail(FDB_ERR_UNSUPPORTED, "batched adjoint: instance " + std::to_string(i) +
                                           " is outside the fixed-point kernel's domain");
  }
  if (b->adj_mode != 1) {
    if (S == 0) {  // dL/df0 = lambda_T, dL/dv = 0
      uint64_t cells = 0;
      for (uint64_t z : b->sizes) cells += z;
      FDB_TRY(bsync(b));
      FDB_CUDA_TRY(cudaMemcpy(grad_f0, lambda_T, cells * 8,
                              is_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToHost));
      for (int i = 0; i < 3 * n; ++i) grad_v[i] = 0.0;
      return FDB_OK;
    }
    NvtxScope nvtx_c("fdb.batch.adjoint.closed_form");
    return batch_adjoint_closed_form(b, S, dt, lambda_T, grad_f0, grad_v, is_device,
                                     b->adj_mode == 0);
  }
  // storage
  const size_t T = (size_t)b->total;
  const int nsegbuf = adjoint_fixed_segment_buffers(K);
  const int grid = batch_adjoint_grid(n, b->geoms.data());
  const size_t sb = batch_adjoint_scratch_bytes(n, K, grid);
  if ((int)b->adj_ckpt.size() < nseg || (int)b->adj_seg.size() < nsegbuf || !b->adj_lam[0] ||
      b->adj_scratch_bytes < sb) {
    free_batch_adjoint(b);
    b->adj_ckpt.assign(nseg, nullptr);
    b->adj_seg.assign(nsegbuf, nullptr);
    int rc = FDB_OK;
    for (auto& p : b->adj_ckpt)
      if (!rc) rc = balloc(&p, T);
    for (auto& p : b->adj_seg)
      if (!rc) rc = balloc(&p, T);
    for (auto& p : b->adj_lam)
      if (!rc) rc = balloc(&p, T);
    for (auto& p : b->adj_io)
      if (!rc) rc = balloc(&p, T);
    if (!rc) rc = balloc(&b->adj_user, T);
    if (!rc) rc = balloc(&b->adj_dda, 3 * (size_t)n);
    if (!rc) rc = balloc((char**)&b->adj_scratch, sb);
    if (rc) {
      free_batch_adjoint(b);
      return rc;
    }
    b->adj_scratch_bytes = sb;
  }
  // the caller's concatenated fields: instance i starts at pref[i]
  std::vector<uint64_t> pref(n);
  uint64_t cells = 0;
  for (int i = 0; i < n; ++i) {
    pref[i] = cells;
    cells += b->sizes[i];
  }
  // forward with checkpoints (the persistent launch): ckpt[s] = f^{sK}
  for (int sg = 0; sg < nseg; ++sg) {
    FDB_CUDA_TRY(cudaMemcpyAsync(b->adj_ckpt[sg], b->arena[b->cur], T * 8,
                                 cudaMemcpyDeviceToDevice, b->stream));
    const int len = std::min(K, S - sg * K);
    FDB_TRY(run_batched(b, len, dt, effective_K(b), effective_shape(b), b->tz, true));
  }
  // lambda_T into the stored layout
  const double* lt = lambda_T;
  if (!is_device) {
    FDB_CUDA_TRY(cudaMemcpyAsync(b->adj_user, lambda_T, cells * 8, cudaMemcpyHostToDevice,
                                 b->stream));
    lt = b->adj_user;
  }
  for (int i = 0; i < n; ++i) {
    double* dst = b->adj_io[0] + b->offsets[i];
    if (b->permuted[i])
      FDB_TRY(launch_permute(b, i, lt + pref[i], dst, false));
    else
      FDB_CUDA_TRY(cudaMemcpyAsync(dst, lt + pref[i], b->sizes[i] * 8, cudaMemcpyDeviceToDevice,
                                   b->stream));
  }
  BatchAdjointIO io;
  std::vector<int32_t*> hi(K);
  for (int k = 0; k < K; ++k) hi[k] = (int32_t*)b->adj_seg[2 + k / 2] + (k & 1) * T;
  io.count = n;
  io.geoms = b->geoms.data();
  io.coeffs = cs.data();
  io.offsets = b->offsets.data();
  io.d_offs = b->d_offs;
  io.d_sizes = b->d_sizes;
  io.S = S;
  io.K = K;
  io.nseg = nseg;
  io.ckpt = b->adj_ckpt.data();
  io.chain[0] = (int64_t*)b->adj_seg[0];
  io.chain[1] = (int64_t*)b->adj_seg[1];
  io.state_hi = hi.data();
  io.lam[0] = (int64_t*)b->adj_lam[0];
  io.lam[1] = (int64_t*)b->adj_lam[1];
  io.lam_T = b->adj_io[0];
  io.grad_f0 = b->adj_io[1];
  io.dda3 = b->adj_dda;
  io.err = b->d_err;
  io.scratch = b->adj_scratch;
  FDB_TRY(batch_adjoint_run(io, b->stream));
  // dL/df0 back to the caller's order
  double* gd = is_device ? grad_f0 : b->adj_user;
  for (int i = 0; i < n; ++i) {
    const double* src = b->adj_io[1] + b->offsets[i];
    if (b->permuted[i])
      FDB_TRY(launch_permute(b, i, src, gd + pref[i], true));
    else
      FDB_CUDA_TRY(cudaMemcpyAsync(gd + pref[i], src, b->sizes[i] * 8, cudaMemcpyDeviceToDevice,
                                   b->stream));
  }
  if (!is_device)
    FDB_CUDA_TRY(cudaMemcpyAsync(grad_f0, b->adj_user, cells * 8, cudaMemcpyDeviceToHost,
                                 b->stream));
  std::vector<double> dda(3 * (size_t)n);
  FDB_CUDA_TRY(cudaMemcpyAsync(dda.data(), b->adj_dda, dda.size() * 8, cudaMemcpyDeviceToHost,
                               b->stream));
  FDB_TRY(bsync(b));
  if (grad_v) batch_velocity_grad(b, dt, dda.data(), grad_v);
  return FDB_OK;
}

int fdb_batch_checksums(fdb_batch* b, double* out) {
  FDB_TRY(bcheck(b));
  if (!out) return fail(FDB_ERR_INVALID, "null output");
  k_batch_sum_partial<<<b->count * kSumPerInst, 256, 0, b->stream>>>(
      b->arena[b->cur], b->d_offs, b->d_sizes, b->count, kSumPerInst, b->d_part);
  k_batch_sum_final<<<(b->count + 127) / 128, 128, 0, b->stream>>>(b->d_part, b->count,
                                                                   kSumPerInst, b->d_sums);
  note_launch(2);
  FDB_CUDA_TRY(cudaGetLastError());
  FDB_CUDA_TRY(cudaMemcpyAsync(b->h_sums, b->d_sums, b->count * sizeof(double),
                               cudaMemcpyDeviceToHost, b->stream));
  FDB_TRY(bsync(b));
  memcpy(out, b->h_sums, b->count * sizeof(double));
  return FDB_OK;
}

// Small autotuner: times each compiled (depth, shape) of the batched kernel,
// and whole-z versus 32-plane tiles, on a copy of the current fields for
// `num_steps` steps; keeps the fastest.  With a cache path, results are
// stored per problem class (instance count, cell-count bucket, largest axis,
// GPU name) and reused without timing.
int fdb_batch_autotune(fdb_batch* b, int num_steps, const double* dt, const char* cache_path,
                       int* chosen) {
  FDB_TRY(bcheck(b));
  FDB_TRY(check_dts(b, dt));
  if (num_steps <= 0) return fail(FDB_ERR_INVALID, "num_steps must be > 0");
  uint64_t cells = 0;
  uint64_t maxn = 0;
  for (const Geom& g : b->geoms) {
    cells += g.ntot;
    maxn = std::max<uint64_t>(maxn, std::max<uint64_t>(g.nx, std::max<uint64_t>(g.ny, g.nz)));
  }
  int dev = 0;
  cudaDeviceProp prop;
  FDB_CUDA_TRY(cudaGetDevice(&dev));
  FDB_CUDA_TRY(cudaGetDeviceProperties(&prop, dev));
  std::ostringstream cls;
  cls << "count=" << b->count << ";cells_log2=" << (int)floor(log2((double)std::max<uint64_t>(cells, 1)))
      << ";maxn=" << maxn << ";steps=" << num_steps << ";gpu=" << prop.name;
  std::string key = cls.str();
  for (char& ch : key)
    if (ch == ' ') ch = '_';
  if (cache_path && *cache_path) {
    std::ifstream in(cache_path);
    std::string line;
    while (std::getline(in, line)) {
      std::istringstream ls(line);
      std::string k;
      int K, sh, tz;
      if (ls >> k >> K >> sh >> tz && k == key && find_variant(K, sh)) {
        b->K = K;
        b->shape = sh;
        b->tz = tz;
        drop_graph(b);
        if (chosen) {
          chosen[0] = K;
          chosen[1] = sh;
          chosen[2] = tz;
        }
        return FDB_OK;
      }
    }
  }
  // time candidates on a copy: the fields are restored afterwards
  double* save = nullptr;
  FDB_TRY(balloc(&save, b->total));
  FDB_CUDA_TRY(cudaMemcpyAsync(save, b->arena[b->cur], b->total * 8, cudaMemcpyDeviceToDevice,
                               b->stream));
  const int cur0 = b->cur;
  EventPool events;
  cudaEvent_t e0 = events.make(), e1 = events.make();
  if (!e0 || !e1) {
    cudaFree(save);
    return fail(FDB_ERR_CUDA, "autotune: cudaEventCreate failed");
  }
  float best = 1e30f;
  int bK = kDefaultDepth, bsh = fx::kR4W8S, btz = 0;
  int rc = FDB_OK;
  for (const Variant& v : kVariants) {
    for (int tzc : {0, 32}) {
      for (int rep = 0; rep < 2 && !rc; ++rep) {  // rep 0 warms up (and builds nothing)
        b->cur = cur0;
        cudaMemcpyAsync(b->arena[cur0], save, b->total * 8, cudaMemcpyDeviceToDevice, b->stream);
        cudaEventRecord(e0, b->stream);
        rc = run_batched(b, num_steps, dt, v.K, v.shape, tzc, false);
        cudaEventRecord(e1, b->stream);
        if (rc == FDB_ERR_UNSUPPORTED) {
          rc = FDB_OK;
          break;
        }
        if (!rc) rc = bsync(b);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (!rc && rep == 1 && ms < best) {
          best = ms;
          bK = v.K;
          bsh = v.shape;
          btz = tzc;
        }
      }
    }
  }
  b->cur = cur0;
  cudaMemcpyAsync(b->arena[cur0], save, b->total * 8, cudaMemcpyDeviceToDevice, b->stream);
  cudaStreamSynchronize(b->stream);
  cudaFree(save);
  if (rc) return rc;
  b->K = bK;
  b->shape = bsh;
  b->tz = btz;
  drop_graph(b);
  if (chosen) {
    chosen[0] = bK;
    chosen[1] = bsh;
    chosen[2] = btz;
  }
  if (cache_path && *cache_path) {
    std::ofstream o(cache_path, std::ios::app);
    o << key << ' ' << bK << ' ' << bsh << ' ' << btz << '\n';
  }
  return FDB_OK;
}

}  // extern "C"
