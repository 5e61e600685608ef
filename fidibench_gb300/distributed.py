"""Distributed upwind advection: a periodic grid split into slabs of axis 0
across ranks (one GPU each), with the upwind halo exchanged once every K
steps.

The reference distributes its upwind run with the MPI Filter
(upwind/cxx/upwindMpi.cxx:30-165): CubeDecomp splits the grid into
sub-domains (cxx/Filter.cpp:26-56), every applyFilter fetches the neighbour's
halo window with MPI_Get (Filter.cpp:114-129, :212-221) for every stencil
term, and computeCheckSum reduces the local sums with MPI_Reduce
(Filter.cpp:465-485).  Here:

- a rank owns planes [z0, z1) of axis 0, the slowest axis, so its field and
  every plane range of it are contiguous blocks of HBM (no packing);
- the step is one-sided, so only the planes on the upwind side are needed:
  cell z reads z - 1 when v_0 >= 0 (upwind.cxx:34-35) and z + 1 otherwise;
- with K halo planes a rank advances K steps between exchanges: after k <= K
  steps the k planes nearest the halo end of its slab are stale and all its
  own planes are exact (the slab handle, fdb_upwind_create_slab, treats its
  extended slab as periodic and uses the global grid's spacings, so every
  own cell is updated exactly as in the whole-grid run);
- the exchange is a ring shift: every rank sends its K boundary planes to the
  downwind rank and receives K planes from the upwind rank (torch.distributed
  point-to-point: NCCL on device tensors, or gloo through host buffers);
- the checksum is the sum of the ranks' own-plane checksums (all-reduced).

Every slab advances in a block chain (fdb_upwind_block_begin /
fdb_upwind_advect_block): under the block-fixed-point arithmetic the field
stays int64 between blocks, the halo planes travel as int64, and before each
block the ranks make their scale words equal to the maximum over all ranks
(the scale is measured over each slab's own planes only), so every slab
advances with the scale of the whole grid.  The result is then the
single-field advect's bit for bit, in every arithmetic (EXACT and FMA are
per-cell FP64 and need no agreement).  `SlabRing` runs all slabs of a
decomposition in one process on one GPU with the same exchange done by
device copies (tests, and single-GPU runs of the sharded form).

The slab protocol (`UpwindSlab` on the GPU; any object with the same methods,
such as a CPU stand-in in the tests): own / halo / send plane ranges,
get_planes / set_planes / block_begin / advect_block / get_scale_word /
set_scale_word / checksum_own / set_own / get_own.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _capi
from ._capi import check, lib


def slab_bounds(n0: int, world: int) -> list[tuple[int, int]]:
    """Contiguous split of n0 planes over `world` ranks, the first n0 % world
    ranks one plane longer (the balanced 1-D case of CubeDecomp)."""
    if world < 1 or n0 < world:
        raise ValueError(f"cannot split {n0} planes over {world} ranks")
    base, extra = divmod(n0, world)
    out, z = [], 0
    for r in range(world):
        h = base + (1 if r < extra else 0)
        out.append((z, z + h))
        z += h
    return out


def halo_depth(bounds, requested: int) -> int:
    """Steps between exchanges: the requested depth, at most the thinnest
    slab (a halo comes from one neighbour)."""
    return max(1, min([requested] + [z1 - z0 for z0, z1 in bounds]))


class SlabLayout:
    """Where a rank's planes sit in its extended slab of K + nloc planes.

    v_0 >= 0 (upwind neighbour at z - 1): [halo K | own nloc]; the halo is the
    upwind rank's last K own planes, and this rank's last K own planes go to
    the downwind rank (rank + 1).  v_0 < 0: [own nloc | halo K], halo = the
    upwind rank's (rank + 1) first K own planes."""

    def __init__(self, z0: int, z1: int, halo: int, v0: float, world: int, rank: int):
        self.z0, self.z1, self.halo = z0, z1, halo
        self.nloc = z1 - z0
        self.planes = halo + self.nloc
        self.low_halo = not (v0 < 0.0)
        if self.low_halo:
            self.own = (halo, self.nloc)
            self.halo_at = (0, halo)
            self.send = (self.nloc, halo)  # own planes [nloc - K, nloc) at offset K
            self.upwind = (rank - 1) % world
            self.downwind = (rank + 1) % world
        else:
            self.own = (0, self.nloc)
            self.halo_at = (self.nloc, halo)
            self.send = (0, halo)
            self.upwind = (rank + 1) % world
            self.downwind = (rank - 1) % world


class UpwindSlab:
    """One rank's slab on the current GPU (fdb_upwind_create_slab)."""

    def __init__(self, velocity, lengths, numCells, layout: SlabLayout, arith: str = "auto",
                 depth: int = 0, coeff_form: str = "cxx"):
        self.layout = layout
        v = np.ascontiguousarray(velocity, dtype=np.float64)
        L = np.ascontiguousarray(lengths, dtype=np.float64)
        n = np.ascontiguousarray([int(x) for x in numCells], dtype=np.uint64)
        self.ndims = len(n)
        self.plane = int(np.prod(n[1:])) if self.ndims > 1 else 1
        h = ctypes.c_void_p()
        check(lib.fdb_upwind_create_slab(self.ndims, v.ctypes.data, L.ctypes.data,
                                         n.ctypes.data, layout.planes, ctypes.byref(h)))
        self._h = h
        # blocks of up to `halo` steps: the fixed kernel's depth is the halo
        # depth unless one is asked for (at least the halo depth)
        check(lib.fdb_upwind_set_arith(self._h, _capi.ARITH_NAMES[arith],
                                       int(depth) if depth else layout.halo))
        if coeff_form != "cxx":
            check(lib.fdb_upwind_set_coeff_form(self._h, _capi.COEFF_NAMES[coeff_form]))
        check(lib.fdb_upwind_set_own_planes(self._h, layout.own[0], layout.own[1]))

    def close(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            lib.fdb_upwind_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_stream(self, stream) -> None:
        check(lib.fdb_upwind_set_stream(self._h, getattr(stream, "cuda_stream", stream)))

    def get_planes(self, first: int, count: int, out) -> None:
        is_dev = 1 if getattr(out, "is_cuda", False) else 0
        check(lib.fdb_upwind_get_planes(self._h, first, count, _capi.dptr(out), is_dev))

    def set_planes(self, first: int, count: int, src) -> None:
        is_dev = 1 if getattr(src, "is_cuda", False) else 0
        check(lib.fdb_upwind_set_planes(self._h, first, count, _capi.dptr(src), is_dev))

    def advect(self, steps: int, dt: float) -> None:
        check(lib.fdb_upwind_advect(self._h, int(steps), float(dt)))

    def block_begin(self, dt: float) -> bool:
        """Open a block chain; True when it runs the fixed-point arithmetic
        (whose scale word the ranks must agree on before every block)."""
        fixed = ctypes.c_int()
        check(lib.fdb_upwind_block_begin(self._h, float(dt), ctypes.byref(fixed)))
        return bool(fixed.value)

    def advect_block(self, steps: int, dt: float, last: bool) -> None:
        check(lib.fdb_upwind_advect_block(self._h, int(steps), float(dt), 1 if last else 0))

    def get_scale_word(self, out) -> None:
        is_dev = 1 if getattr(out, "is_cuda", False) else 0
        check(lib.fdb_upwind_get_scale_word(self._h, _capi.dptr(out), is_dev))

    def set_scale_word(self, src) -> None:
        is_dev = 1 if getattr(src, "is_cuda", False) else 0
        check(lib.fdb_upwind_set_scale_word(self._h, _capi.dptr(src), is_dev))

    def checksum_own(self) -> float:
        out = ctypes.c_double()
        first, count = self.layout.own
        check(lib.fdb_upwind_checksum_planes(self._h, first, count, ctypes.byref(out)))
        return out.value

    def set_own(self, values) -> None:
        first, count = self.layout.own
        if getattr(values, "is_cuda", False):
            import torch
            t = values.contiguous()
            if t.numel() != count * self.plane:
                raise ValueError(f"slab has {count * self.plane} values, got {t.numel()}")
            torch.cuda.current_stream(t.device).synchronize()  # written on torch's stream
            self.set_planes(first, count, t)
        else:
            a = np.ascontiguousarray(values, dtype=np.float64).reshape(-1)
            if a.size != count * self.plane:
                raise ValueError(f"slab has {count * self.plane} values, got {a.size}")
            self.set_planes(first, count, a)

    def get_own(self, out=None):
        first, count = self.layout.own
        if out is None:
            out = np.empty(count * self.plane, dtype=np.float64)
        self.get_planes(first, count, out)
        return out

    @property
    def arith_used(self) -> str:
        ntot = ctypes.c_uint64()
        a = ctypes.c_int()
        check(lib.fdb_upwind_info(self._h, ctypes.byref(ntot), ctypes.byref(a)))
        return {v: k for k, v in _capi.ARITH_NAMES.items()}.get(a.value, str(a.value))


def _advance(slabs, exchange, agree, steps: int, dt: float, halo: int) -> None:
    """steps steps in blocks of up to `halo`: the halo exchange before every
    block and, under the fixed-point arithmetic, the scale agreement."""
    if steps == 0:
        return
    fixed = [s.block_begin(dt) for s in slabs]
    if any(fixed) != all(fixed):
        raise RuntimeError("slabs disagree on the arithmetic")
    fixed = fixed[0]
    done = 0
    while done < steps:
        k = min(halo, steps - done)
        exchange()
        if fixed:
            agree()
        for s in slabs:
            s.advect_block(k, dt, done + k == steps)
        done += k


class DistributedUpwind:
    """upwindMpi.cxx's distributed advect on one GPU per rank.

    velocity, lengths, numCells: the global problem (>= 1 axes; axis 0 is
    split).  group: a torch.distributed process group (None: the default
    group when initialised, else one rank).  halo: steps between exchanges
    (capped by the thinnest slab).  slab_factory: callable(SlabLayout) ->
    slab object (tests put a CPU stand-in here); default an UpwindSlab on the
    current GPU.  The GPU slab enqueues on its own torch stream (`stream`),
    and the NCCL transfers are issued with that stream current, so copies,
    transfers and steps are ordered on the device without host waits."""

    def __init__(self, velocity, lengths, numCells, group=None, halo: int = 3,
                 arith: str = "auto", depth: int = 0, coeff_form: str = "cxx",
                 slab_factory=None):
        import torch
        import torch.distributed as dist
        self.numCells = [int(x) for x in numCells]
        self.group = group
        if dist.is_available() and dist.is_initialized():
            self.world = dist.get_world_size(group)
            self.rank = dist.get_rank(group)
            self.backend = str(dist.get_backend(group))
        else:
            self.world, self.rank, self.backend = 1, 0, None
        self.bounds = slab_bounds(self.numCells[0], self.world)
        self.halo = halo_depth(self.bounds, halo)
        z0, z1 = self.bounds[self.rank]
        self.layout = SlabLayout(z0, z1, self.halo, float(velocity[0]), self.world, self.rank)
        self.plane = int(np.prod(self.numCells[1:])) if len(self.numCells) > 1 else 1
        # device buffers for NCCL and for the single-rank self-exchange on the
        # GPU; host buffers for gloo (and for CPU stand-in slabs)
        self.on_device = self.backend == "nccl" or (self.world == 1 and slab_factory is None)
        self.stream = None
        if slab_factory is None:
            slab = UpwindSlab(velocity, lengths, self.numCells, self.layout, arith, depth,
                              coeff_form)
            self.stream = torch.cuda.Stream()
            slab.set_stream(self.stream)
        else:
            slab = slab_factory(self.layout)
        self.slab = slab
        n = self.halo * self.plane
        # halo planes hold FP64 or int64 values: 8-byte words moved as they are
        if self.on_device:
            dev = torch.device("cuda", torch.cuda.current_device())
            self._send = torch.empty(n, dtype=torch.float64, device=dev)
            self._recv = torch.empty(n, dtype=torch.float64, device=dev)
            self._word = torch.zeros(1, dtype=torch.int64, device=dev)
        else:
            pin = torch.cuda.is_available() and isinstance(self.slab, UpwindSlab)
            self._send = torch.empty(n, dtype=torch.float64, pin_memory=pin)
            self._recv = torch.empty(n, dtype=torch.float64, pin_memory=pin)
            self._word = torch.zeros(1, dtype=torch.int64, pin_memory=pin)

    def close(self) -> None:
        if hasattr(self.slab, "close"):
            self.slab.close()

    # -- field ---------------------------------------------------------------------
    def set_global_field(self, f) -> None:
        """Each rank takes its own planes of the global field (host array)."""
        a = np.asarray(f, dtype=np.float64).reshape(-1)
        z0, z1 = self.bounds[self.rank]
        self.slab.set_own(a[z0 * self.plane:z1 * self.plane])

    def gather(self):
        """The global field on every rank (host array; all-gather of the
        own planes, the slabs padded to the thickest one)."""
        import torch
        import torch.distributed as dist
        own = np.asarray(self.slab.get_own(), dtype=np.float64)
        if self.world == 1:
            return own.copy()
        hmax = max(z1 - z0 for z0, z1 in self.bounds)
        pad = np.zeros(hmax * self.plane)
        pad[:own.size] = own
        if self.on_device:
            with torch.cuda.stream(self.stream):
                t = torch.from_numpy(pad).to(torch.device("cuda", torch.cuda.current_device()))
                parts = [torch.empty_like(t) for _ in range(self.world)]
                dist.all_gather(parts, t, group=self.group)
                self.stream.synchronize()
        else:
            t = torch.from_numpy(pad)
            parts = [torch.empty_like(t) for _ in range(self.world)]
            dist.all_gather(parts, t, group=self.group)
        return np.concatenate([parts[r].cpu().numpy()[:(z1 - z0) * self.plane]
                               for r, (z0, z1) in enumerate(self.bounds)])

    # -- the step ------------------------------------------------------------------
    def exchange(self) -> None:
        """Halo planes <- the upwind rank's boundary planes (ring shift)."""
        import torch.distributed as dist
        lay = self.layout
        self.slab.get_planes(lay.send[0], lay.send[1], self._send)
        if self.world == 1:
            self.slab.set_planes(lay.halo_at[0], lay.halo_at[1], self._send)
            return
        ops = [dist.P2POp(dist.isend, self._send, lay.downwind, self.group),
               dist.P2POp(dist.irecv, self._recv, lay.upwind, self.group)]
        if self.on_device:
            import torch
            # NCCL waits for, and is waited on by, the current stream: the slab's
            with torch.cuda.stream(self.stream):
                for req in dist.batch_isend_irecv(ops):
                    req.wait()
        else:
            for req in dist.batch_isend_irecv(ops):
                req.wait()
        self.slab.set_planes(lay.halo_at[0], lay.halo_at[1], self._recv)

    def agree_scale(self) -> None:
        """Every rank's scale word <- the maximum over the ranks (the scale
        words are FP64 bit patterns of max|f| or ORs of |F|: non-negative,
        ordered as integers)."""
        import torch
        import torch.distributed as dist
        if self.world == 1:
            return
        self.slab.get_scale_word(self._word)
        if self.on_device:
            with torch.cuda.stream(self.stream):
                dist.all_reduce(self._word, op=dist.ReduceOp.MAX, group=self.group)
        else:
            dist.all_reduce(self._word, op=dist.ReduceOp.MAX, group=self.group)
        self.slab.set_scale_word(self._word)

    def advect(self, numTimeSteps: int, deltaTime: float) -> None:
        """numTimeSteps steps of the global problem: exchange (and agree on
        the scale), then up to K steps on every slab, repeated."""
        if numTimeSteps < 0:
            raise ValueError("numTimeSteps must be >= 0")
        _advance([self.slab], self.exchange, self.agree_scale, int(numTimeSteps),
                 float(deltaTime), self.halo)

    def checksum(self) -> float:
        """Sum of the global field (Filter::computeCheckSum, Filter.cpp:465-485;
        all-reduced so that every rank returns it)."""
        import torch
        import torch.distributed as dist
        local = float(self.slab.checksum_own())
        if self.world == 1:
            return local
        if self.on_device:
            with torch.cuda.stream(self.stream):
                t = torch.tensor([local], dtype=torch.float64,
                                 device=torch.device("cuda", torch.cuda.current_device()))
                dist.all_reduce(t, op=dist.ReduceOp.SUM, group=self.group)
                return float(t.item())
        t = torch.tensor([local], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.SUM, group=self.group)
        return float(t.item())


class SlabRing:
    """Every slab of a `world`-way decomposition in this process, on the
    current GPU: the exchange of DistributedUpwind with device copies between
    the slabs' buffers in place of sends.  All slabs enqueue on one torch
    stream (`stream`), so the copies and the steps are ordered."""

    def __init__(self, velocity, lengths, numCells, world: int, halo: int = 3,
                 arith: str = "auto", depth: int = 0, coeff_form: str = "cxx"):
        import torch
        self.numCells = [int(x) for x in numCells]
        self.world = world
        self.bounds = slab_bounds(self.numCells[0], world)
        self.halo = halo_depth(self.bounds, halo)
        self.plane = int(np.prod(self.numCells[1:])) if len(self.numCells) > 1 else 1
        self.layouts = [SlabLayout(z0, z1, self.halo, float(velocity[0]), world, r)
                        for r, (z0, z1) in enumerate(self.bounds)]
        self.slabs = []
        self.stream = torch.cuda.Stream()
        for lay in self.layouts:
            s = UpwindSlab(velocity, lengths, self.numCells, lay, arith, depth, coeff_form)
            s.set_stream(self.stream)
            self.slabs.append(s)
        dev = torch.device("cuda", torch.cuda.current_device())
        self._tmp = [torch.empty(self.halo * self.plane, dtype=torch.float64, device=dev)
                     for _ in range(world)]
        self._words = torch.zeros(world, dtype=torch.int64, device=dev)

    def close(self) -> None:
        for s in self.slabs:
            s.close()

    def set_global_field(self, f) -> None:
        a = np.asarray(f, dtype=np.float64).reshape(-1)
        for s, (z0, z1) in zip(self.slabs, self.bounds):
            s.set_own(a[z0 * self.plane:z1 * self.plane])

    def gather(self) -> np.ndarray:
        return np.concatenate([s.get_own() for s in self.slabs])

    def exchange(self) -> None:
        # every rank's boundary planes first, then every halo: the ring shift
        for r, s in enumerate(self.slabs):
            lay = self.layouts[r]
            s.get_planes(lay.send[0], lay.send[1], self._tmp[r])
        for r, s in enumerate(self.slabs):
            lay = self.layouts[r]
            s.set_planes(lay.halo_at[0], lay.halo_at[1], self._tmp[lay.upwind])

    def agree_scale(self) -> None:
        # every slab's scale word -> one tensor, its maximum back to every slab
        import torch
        for r, s in enumerate(self.slabs):
            s.get_scale_word(self._words[r:r + 1])
        with torch.cuda.stream(self.stream):
            m = torch.max(self._words).reshape(1)
            for s in self.slabs:
                s.set_scale_word(m)
            self._m = m  # kept alive until the copies out of it have run

    def advect(self, numTimeSteps: int, deltaTime: float) -> None:
        if numTimeSteps < 0:
            raise ValueError("numTimeSteps must be >= 0")
        _advance(self.slabs, self.exchange, self.agree_scale, int(numTimeSteps),
                 float(deltaTime), self.halo)

    def checksum(self) -> float:
        return float(sum(s.checksum_own() for s in self.slabs))


__all__ = ["DistributedUpwind", "SlabLayout", "SlabRing", "UpwindSlab", "halo_depth",
           "slab_bounds"]
