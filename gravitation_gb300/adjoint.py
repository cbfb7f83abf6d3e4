"""Differentiable rollout: K steps forward with FP64 checkpoints, discrete adjoint back.

``rollout(r0, v0, m, G, T, steps, every)`` is a torch.autograd.Function: its forward
runs ``steps`` GB300 steps (FP32 stage 1, FP64 stage 2) and keeps the FP64 state at
the start of every ``every``-step segment; its backward sweeps the segments from last
to first.  Each segment starts from the exact stored state at its end and reverses the
update step by step in FP64, while the adjoint pair kernel recomputes stage 1 at each
reconstructed position and applies the transposed stage 2 and stage 1 (see
csrc/adjoint.cu).  Gradients are returned for the initial positions, velocities and
masses.  Memory: one FP64 state per segment, no per-step storage.

Option ``store_a`` trades memory for time: the forward keeps every step's FP64
accelerations (steps x 32 bytes per body), the reversal uses them and the pair kernel
forms only the transposed terms, without recomputing stage 1.  By default ('auto') they
are kept whenever they fit the slot budget (engine.slot_budget_bytes: 1000 steps of
65536 bodies take 2.1 GB), which measured forward + adjoint 10-13 % faster from 8192
bodies up on GB300.
"""

import ctypes

import numpy as np
import torch

from . import _lib
from ._lib import check
from .engine import Engine, device_info, make_plan, _ctypes_to_device

ADJ_TILE = (2, 128, 128)


def default_adjoint_pairs(sizes, budget=None):
    """The unique-pair backward kernel from ~4k bodies (1.6e7 ordered pairs) on.
    Measured on GB300, backward step (graph-replayed), all pairs vs unique pairs:
    N = 4096 -- 32.5 vs 31.2 us (8 warps, 2 rows/thread, 64-body j-tiles), N = 8192 --
    116 vs 94 us, N = 16384 -- 385 vs 313 us, N = 65536 -- 5.63 vs 4.15 ms.
    Above the slot budget (engine.slot_budget_bytes, or `budget` bytes) the all-pairs
    kernel is used: the unique-pair plan keeps 7-component slots per pair of row blocks."""
    if sum(int(n) * int(n) for n in sizes) < 16_000_000:
        return False
    from .engine import pair_plan_fits
    t = default_adjoint_tile(sizes, True)
    return pair_plan_fits(sizes, budget, comps=7, tiles=[_lib.Tile(t[0], t[1], t[2], 1)])


def default_adjoint_tile(sizes, pairs=False):
    """Tile of the backward pair kernel.  Unique pairs: 2 rows/thread, 8 warps and
    64-body j-tiles up to ~20k bodies, 4 rows/thread (compensated sums in shared memory),
    4 warps and 128-body j-tiles above.  Measured on GB300, backward step with the
    accelerations recomputed / kept, tiles 2/256/64, 2/128/64, 4/128/128: N = 8192 --
    85 / 71, 84 / 69, 81 / 70 us; N = 16384 -- 274 / 232, 283 / 235, 289 / 254 us;
    N = 32768 -- 1035 / 871, 1091 / 895, 967 / 854 us; N = 65536 -- 4.08 / 3.43,
    4.28 / 3.52, 3.77 / 3.33 ms.  All pairs: up to ~10k bodies (1e8 ordered pairs) a step
    is latency bound and one body per thread (the finest work units) is fastest; above,
    two bodies per thread.  Measured on GB300, backward step: N = 4096 -- 37.8 us with
    (1, 128, 128), 40.4 us with (2, 128, 128), 37.9 / 40.3 / 43.3 / 48.8 us with
    (1, 64, 128) / (2, 64, 128) / (1, 128, 64) / (2, 64, 64); N = 65536 -- 5.16 ms with
    (2, 128, 128), 5.62 ms with (1, 128, 128)."""
    if pairs:
        n2 = sum(int(n) * int(n) for n in sizes)
        return (2, 256, 64) if n2 <= 400_000_000 else (4, 128, 128)
    if sum(int(n) * int(n) for n in sizes) <= 100_000_000:
        return (1, 128, 128)
    return ADJ_TILE


class AdjointEngine:
    """Buffers and plan of the backward sweep for a packed batch of universes.

    pairs: True -- the unique-pair backward kernel (each unordered pair once, plan of
    grav_plan_pairs); False -- every ordered pair (plan of grav_plan); None -- by size.
    tile: (bpt, threads, jtile) of that kernel, default by size, optionally with a fourth
    entry, the persistent grid (default: SMs x resident CTAs)."""

    def __init__(self, sizes, T, device=None, tile=None, pairs=None):
        self.lib = _lib.load()
        self.dev_info = device_info(device)
        self.device = torch.device('cuda', self.dev_info.index)
        self.sizes = [int(n) for n in sizes]
        if pairs is None:
            pairs = default_adjoint_pairs(self.sizes)
        self.pairs = bool(pairs)
        mode = _lib.GRAV_MODE_FP32U if self.pairs else _lib.GRAV_MODE_FP32
        if tile is None:
            tile = default_adjoint_tile(self.sizes, self.pairs)
        t = _lib.Tile(tile[0], tile[1], tile[2], 0)
        if not self.lib.grav_adjoint_tile_supported(mode, ctypes.byref(t)):
            raise ValueError('no %s adjoint kernel for tile %r' % (
                'unique-pair' if self.pairs else 'all-pairs', tile))
        occ = ctypes.c_int32()
        with torch.cuda.device(self.device):
            check(self.lib.grav_adjoint_occupancy(mode, ctypes.byref(t), ctypes.byref(occ)))
        t.grid = self.dev_info.sm_count * max(occ.value, 1)
        if len(tile) > 3 and tile[3]:
            t.grid = max(1, int(tile[3]))
        self.info, univ, seg = make_plan(self.sizes, T, t, 'fp32u' if self.pairs else 'fp32')
        info, dev = self.info, self.device
        self.univ_dev = _ctypes_to_device(univ, ctypes.sizeof(_lib.UnivDesc) * info.n_univ, dev)
        self.seg_dev = _ctypes_to_device(seg, ctypes.sizeof(_lib.SegDesc) * info.n_seg, dev)
        nb = max(info.n_bodies, 1)
        f64 = dict(dtype=torch.float64, device=dev)
        self.r = torch.zeros((nb, 4), **f64)
        self.v = torch.zeros((nb, 4), **f64)
        self.gr = torch.zeros((nb, 4), **f64)
        self.gv = torch.zeros((nb, 4), **f64)
        self.ggm = torch.zeros(nb, **f64)
        self.pos = torch.zeros(max(info.n_pad_total, 1) * 4, dtype=torch.float32, device=dev)
        self.upos = torch.zeros_like(self.pos)
        self.part7 = torch.zeros(max(info.n_slots * 7 * info.itile, 1), **f64)
        self.err = torch.zeros(1, dtype=torch.int32, device=dev)
        b = _lib.Batch()
        b.mode = mode
        b.n_univ, b.n_seg, b.n_slots = info.n_univ, info.n_seg, info.n_slots
        b.n_bodies, b.n_pad_total, b.n_units = info.n_bodies, info.n_pad_total, info.n_units
        b.tile = _lib.Tile(t.bpt, t.threads, t.jtile, info.grid)
        b.eps2 = 1e-30
        b.univ, b.seg = self.univ_dev.data_ptr(), self.seg_dev.data_ptr()
        b.r, b.v, b.pos = self.r.data_ptr(), self.v.data_ptr(), self.pos.data_ptr()
        b.part, b.a_out, b.err = self.part7.data_ptr(), None, self.err.data_ptr()
        self.batch = b
        a = _lib.Adjoint()
        a.b = ctypes.pointer(b)
        a.gr, a.gv, a.ggm = self.gr.data_ptr(), self.gv.data_ptr(), self.ggm.data_ptr()
        a.upos, a.part7 = self.upos.data_ptr(), self.part7.data_ptr()
        a.a_in = None
        self.adj = a
        self._aref = ctypes.byref(a)

    def _h(self, stream):
        s = stream if stream is not None else torch.cuda.current_stream(self.device)
        return ctypes.c_void_p(s.cuda_stream)

    def set_state(self, r4, v4):
        """State (FP64 rows x, y, z, G*m / vx, vy, vz, 0) the next step reverses from."""
        self.r.copy_(r4)
        self.v.copy_(v4)

    def prepare(self, stream=None):
        check(self.lib.grav_adjoint_prepare(self._aref, self._h(stream)))

    def step(self, stream=None, a_in=None):
        """One backward step.  a_in: the forward's accelerations of the step being
        reversed (float64 [n_bodies, 4] device tensor, as stage 2 wrote them with
        GRAV_S2_WRITE_A); None lets the pair kernel recompute them."""
        self.adj.a_in = None if a_in is None else a_in.data_ptr()
        try:
            check(self.lib.grav_adjoint_step(self._aref, self._h(stream)))
        finally:
            self.adj.a_in = None

    def raise_on_device_error(self):
        code = int(self.err.item())
        if code != _lib.GRAV_DEV_OK:
            self.err.zero_()
            raise _lib.GravError(_lib.GRAV_E_CUDA, 'device error flag %d in the adjoint' % code)


class Rollout:
    """Forward engine + adjoint engine for one batch of universes (reusable).

    store_a: False -- checkpoints only; the backward pair kernel recomputes stage 1 at
    every reconstructed position.  True -- the forward also keeps its FP64 accelerations
    of every step (steps x n_bodies x 32 bytes), so that the backward pair kernel forms
    only J^T u and the mass term (40 instead of 46 FMA-pipe operations per pair, 4 slot
    components instead of 7) and the reversal v_k = v_{k+1} - T a_k uses the very a_k
    of the forward.  'auto' (default): True when that fits the slot budget
    (engine.slot_budget_bytes).  Measured on GB300 (forward + adjoint over forward,
    uniform cube, forward fp32un): N = 8192 -- 2.75 kept, 3.07 recomputed; N = 16384 --
    2.91 kept, 3.26 recomputed."""

    def __init__(self, sizes, T, steps, every=32, device=None, fwd_tile=None, tuner=None,
                 mode=None, graphs=True, adj_pairs=None, store_a='auto'):
        self.sizes = [int(n) for n in sizes]
        self.T = float(T)
        self.steps = int(steps)
        self.every = max(1, int(every))
        if mode is None:
            # the forward's FP32 kernel by size, as the plugin picks it: all pairs for
            # small universes, unique pairs from 4608 bodies while the batch's slots fit,
            # near pairs from double-single separations.  A final-state loss against a
            # nearby target is ill-conditioned (at the differentiable-rollout workload
            # r_K - t is ~1e-9 of r_K), so the forward's force error reaches the
            # gradients through dL/dr_K: plain FP32 separations put them ~1e-3 off the
            # exact FP64 gradients there, the near-corrected ones ~7e-5
            from .plugin import UNIQUE_PAIRS_FROM_N
            from .engine import pair_plan_fits
            mode = 'fp32n'
            if max(self.sizes, default=0) >= UNIQUE_PAIRS_FROM_N and pair_plan_fits(
                    self.sizes, mode='fp32un'):
                mode = 'fp32un'
        self.fwd = Engine(self.sizes, self.T, mode=mode, tile=fwd_tile, device=device,
                          tuner=tuner)
        self.adj = AdjointEngine(self.sizes, self.T, device=device, pairs=adj_pairs)
        self.graphs = bool(graphs)
        self._fwd_graphs = {}
        self._adj_graphs = {}
        n = self.fwd.info.n_bodies
        nseg = -(-self.steps // self.every)
        # FP64 state at the start of every segment, plus the final state
        self.ck_r = torch.zeros((nseg + 1, n, 4), dtype=torch.float64, device=self.fwd.device)
        self.ck_v = torch.zeros_like(self.ck_r)
        self.checkpoints = []
        if store_a == 'auto':
            from .engine import slot_budget_bytes
            store_a = self.steps * max(n, 1) * 32 <= slot_budget_bytes(self.fwd.device)
        self.store_a = bool(store_a)
        # accelerations of every forward step (rows ax, ay, az, 0), written by stage 2
        self.acc = (torch.zeros((max(self.steps, 1), max(n, 1), 4), dtype=torch.float64,
                                device=self.fwd.device) if self.store_a else None)

    def _segments(self):
        starts = list(range(0, self.steps, self.every))
        return [(s, min(s + self.every, self.steps)) for s in starts]

    def _fwd_launch(self, s0, s1, stream):
        """Forward steps s0 .. s1-1; with store_a each writes its accelerations to acc[k]
        (the batch's a_out is pointed there for that launch and restored after)."""
        f = self.fwd
        if not self.store_a:
            f.step(s1 - s0, stream=stream)
            return
        flags = _lib.GRAV_S2_INTEGRATE | _lib.GRAV_S2_WRITE_A
        h = f._h(stream)
        keep = f.batch.a_out
        try:
            for k in range(s0, s1):
                f.batch.a_out = self.acc[k].data_ptr()
                check(f.lib.grav_step(f._bref, flags, h))
        finally:
            f.batch.a_out = keep

    def _graph(self, cache, key, device, enqueue):
        g = cache.get(key)
        if g is None:
            side = torch.cuda.Stream(device=device)
            side.wait_stream(torch.cuda.current_stream(device))
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g, stream=side):
                enqueue(side)
            torch.cuda.current_stream(device).wait_stream(side)
            cache[key] = g
        return g

    def _fwd_segment(self, si, s0, s1, stream):
        """Checkpoint the state at the segment's start, then run its steps."""
        n = self.fwd.info.n_bodies
        with torch.cuda.stream(self.fwd._stream(stream)):
            self.ck_r[si].copy_(self.fwd.r[:n])
            self.ck_v[si].copy_(self.fwd.v[:n])
        self._fwd_launch(s0, s1, stream)

    def _adj_segment(self, si, s0, s1, stream):
        """From the stored state at the segment's end, backward steps s1-1 down to s0."""
        a = self.adj
        with torch.cuda.stream(self.fwd._stream(stream)):
            a.set_state(self.ck_r[si + 1], self.ck_v[si + 1])
        a.prepare(stream)
        for k in reversed(range(s0, s1)):
            a.step(stream, a_in=self.acc[k] if self.store_a else None)

    def forward(self, r0, v0, gm, stream=None):
        """Run the steps; keep the FP64 state at the start of every segment.
        Returns device views (r[n,3], v[n,3]) of the final state.  With graphs=True each
        segment (its checkpoint copy and steps) replays from a CUDA graph captured on
        first use."""
        n = self.fwd.info.n_bodies
        self.fwd.set_state(r0, v0, gm, stream=stream)
        segs = self._segments()
        for si, (s0, s1) in enumerate(segs):
            if self.graphs:
                self._graph(self._fwd_graphs, si, self.fwd.device,
                            lambda st, a=si, b=s0, c=s1: self._fwd_segment(a, b, c, st)).replay()
            else:
                self._fwd_segment(si, s0, s1, stream)
        with torch.cuda.stream(self.fwd._stream(stream)):
            self.ck_r[len(segs)].copy_(self.fwd.r[:n])
            self.ck_v[len(segs)].copy_(self.fwd.v[:n])
        self.checkpoints = [(self.ck_r[i], self.ck_v[i]) for i in range(len(segs))]
        self.final = (self.ck_r[len(segs)], self.ck_v[len(segs)])
        return self.fwd.r[:n, :3], self.fwd.v[:n, :3]

    def backward(self, g_r, g_v, stream=None):
        """Gradients (dL/dr0 [n,3], dL/dv0 [n,3], dL/dGm [n]) from dL/dr_K, dL/dv_K.
        With graphs=True each segment (state reset, prepare and steps) replays from a
        CUDA graph captured on first use."""
        a = self.adj
        n = a.info.n_bodies
        with torch.cuda.stream(self.fwd._stream(stream)):
            a.gr.zero_()
            a.gv.zero_()
            a.ggm.zero_()
            a.gr[:n, :3].copy_(g_r)
            a.gv[:n, :3].copy_(g_v)
        segs = self._segments()
        for si in reversed(range(len(segs))):
            s0, s1 = segs[si]
            if self.graphs:
                self._graph(self._adj_graphs, si, a.device,
                            lambda st, x=si, y=s0, z=s1: self._adj_segment(x, y, z, st)).replay()
            else:
                self._adj_segment(si, s0, s1, stream)
        self.reversed_state = (a.r[:n, :3].clone(), a.v[:n, :3].clone())
        return a.gr[:n, :3].clone(), a.gv[:n, :3].clone(), a.ggm[:n].clone()


class _RolloutFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, r0, v0, m, G, ro):
        gm = (float(G) * m).detach()
        rK, vK = ro.forward(r0.detach(), v0.detach(), gm)
        ctx.ro = ro
        ctx.G = float(G)
        return rK.clone(), vK.clone()

    @staticmethod
    def backward(ctx, g_rK, g_vK):
        ro = ctx.ro
        if g_rK is None:
            g_rK = torch.zeros_like(ro.final[0][:, :3])
        if g_vK is None:
            g_vK = torch.zeros_like(ro.final[1][:, :3])
        gr, gv, ggm = ro.backward(g_rK.to(torch.float64), g_vK.to(torch.float64))
        ro.adj.raise_on_device_error()
        return gr, gv, ctx.G * ggm, None, None


def rollout(r0, v0, m, G, T, steps, every=32, ro=None):
    """Differentiable K-step rollout of one universe (or a packed batch when ``ro`` is
    given).  r0, v0: [n,3] float64 CUDA tensors; m: [n] masses (scaled); G: scaled
    gravitational constant.  Returns (r_K, v_K)."""
    if ro is None:
        ro = Rollout([r0.shape[0]], T, steps, every, device=r0.device.index)
    return _RolloutFn.apply(r0, v0, m, G, ro)


def torch_reference_rollout(r0, v0, m, G, T, steps):
    """Plain PyTorch FP64 integrator (autograd reference): the same law and update."""
    n = r0.shape[0]
    eye = torch.eye(n, dtype=r0.dtype, device=r0.device)
    r, v = r0, v0
    for _ in range(steps):
        d = r[None, :, :] - r[:, None, :]          # d[i, j] = r_j - r_i
        r2 = (d * d).sum(-1) + eye
        inv3 = r2.pow(-1.5) * (1.0 - eye)
        a = G * (d * (m[None, :, None] * inv3[:, :, None])).sum(1)
        v = v + T * a
        r = r + T * v
    return r, v


def reference_gradients_fp64(r0, v0, m, G, T, steps, g_rK, g_vK, every=8):
    """Gradients (dL/dr0, dL/dv0, dL/dm) of a final-state loss with incoming gradients
    g_rK, g_vK, by autograd through the plain PyTorch FP64 integrator
    (torch_reference_rollout) with checkpoints every ``every`` steps: the forward keeps
    only the segment starts, and each segment is replayed with autograd in reverse
    order, so device memory stays at a few N x N x 3 FP64 tensors per step of one
    segment.  A reference for the adjoint kernels, not a fast path."""
    r, v = r0.detach(), v0.detach()
    m = m.detach()
    starts = list(range(0, steps, every))
    ckpt = []
    with torch.no_grad():
        for s0 in starts:
            ckpt.append((r, v))
            r, v = torch_reference_rollout(r, v, m, G, T, min(every, steps - s0))
    gr, gv = g_rK.detach(), g_vK.detach()
    gm = torch.zeros_like(m)
    for s0, (rc, vc) in zip(reversed(starts), reversed(ckpt)):
        rs = rc.clone().requires_grad_(True)
        vs = vc.clone().requires_grad_(True)
        ms = m.clone().requires_grad_(True)
        re, ve = torch_reference_rollout(rs, vs, ms, G, T, min(every, steps - s0))
        gr, gv, gms = torch.autograd.grad((re, ve), (rs, vs, ms), (gr, gv))
        gm = gm + gms
        del re, ve
    return gr, gv, gm
