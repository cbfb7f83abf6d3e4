"""Device engine: FP64 state, work-list plan and stage launches for one or more universes.

PyTorch owns every device buffer; the C ABI (libgravgb300.so) borrows raw pointers.
One ``Engine`` holds a packed batch of universes (a single universe is a batch of
one) and drives the persistent stage-1 kernel and the FP64 stage-2 kernel on a CUDA
stream.  There is no CPU path: without the library or a GB300 every call raises.

Layout in HBM (all packed universe after universe):
  r, v     float64 [n_bodies, 4]   (x, y, z, G*m) and (vx, vy, vz, 0); or, after
           bind_host_state, the caller's pinned host tensors of that layout
  pos      padded stage-1 positions: float4 hi (+ float4 lo in fp32c/fp32cu/fp32n/fp32un)
           or double4
  part     8-byte entries [n_slots, 3, itile]  partial sums written by stage 1: FP32
           (hi, lo) pairs in the row slots (FP64 values in fp64 mode); the unique-pair
           column slots hold FP32 sums in their first half
  univ/seg plan tables (grav_univ_desc / grav_seg_desc)
"""

import ctypes

import numpy as np
import torch

from . import _lib
from ._lib import check

_DEVICE_CACHE = {}


class DeviceInfo:
    def __init__(self, index, sm_count, cc):
        self.index = index
        self.sm_count = sm_count
        self.cc = cc
        self.name = torch.cuda.get_device_name(index)

    def __repr__(self):
        return 'DeviceInfo(%d, %s, sms=%d, cc=%d.%d)' % (
            self.index, self.name, self.sm_count, self.cc[0], self.cc[1])


def device_info(device=None):
    """SM count and compute capability; raises unless the GPU is sm_103 (GB300)."""
    if not torch.cuda.is_available():
        raise RuntimeError('gravitation_gb300 needs a CUDA GPU (GB300); none is visible')
    index = torch.device('cuda', torch.cuda.current_device()).index if device is None else \
        torch.device(device).index
    if index is None:
        index = torch.cuda.current_device()
    if index not in _DEVICE_CACHE:
        L = _lib.load()
        sms, ma, mi = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
        with torch.cuda.device(index):
            check(L.grav_device_query(index, ctypes.byref(sms), ctypes.byref(ma), ctypes.byref(mi)))
        _DEVICE_CACHE[index] = DeviceInfo(index, sms.value, (ma.value, mi.value))
    return _DEVICE_CACHE[index]


def tile_list(mode):
    L = _lib.load()
    m = _lib.MODES[mode] if isinstance(mode, str) else mode
    n = L.grav_tile_list(m, None, 0)
    if n < 0:
        check(n)
    arr = (_lib.Tile * n)()
    L.grav_tile_list(m, arr, n)
    return [_lib.Tile(t.bpt, t.threads, t.jtile, 0) for t in arr]


def occupancy(mode, tile, device=None):
    L = _lib.load()
    m = _lib.MODES[mode] if isinstance(mode, str) else mode
    out = ctypes.c_int32()
    info = device_info(device)
    with torch.cuda.device(info.index):
        check(L.grav_occupancy(m, ctypes.byref(tile), ctypes.byref(out)))
    return out.value


def make_plan(sizes, T, tile, mode='fp32'):
    """Host-side plan (no GPU needed): (PlanInfo, univ ctypes array, seg ctypes array).
    The unique-pair modes (fp32u, fp32cu, fp32un) use grav_plan_pairs, the others
    grav_plan."""
    L = _lib.load()
    fn = L.grav_plan_pairs if mode in _lib.PAIR_MODES else L.grav_plan
    sizes = [int(x) for x in sizes]
    nu = len(sizes)
    n_arr = (ctypes.c_int32 * max(nu, 1))(*sizes)
    T_list = list(T) if np.ndim(T) else [float(T)] * nu
    T_arr = (ctypes.c_double * max(nu, 1))(*[float(x) for x in T_list])
    info = _lib.PlanInfo()
    check(fn(nu, n_arr, T_arr, ctypes.byref(tile), ctypes.byref(info), None, None))
    univ = (_lib.UnivDesc * max(info.n_univ, 1))()
    seg = (_lib.SegDesc * max(info.n_seg, 1))()
    check(fn(nu, n_arr, T_arr, ctypes.byref(tile), ctypes.byref(info), univ, seg))
    return info, univ, seg


def plan_part_bytes(sizes, tile, mode, comps=3):
    """Bytes of partial-sum slots the plan of `mode` (all pairs or unique pairs) needs for
    `sizes` with `tile`: grav_part_bytes, scaled to `comps` components per slot entry (3
    for stage 1; the backward pair kernel keeps 7).  Host-side, no GPU needed.

    The unique-pair plan keeps one column slot per pair of row blocks, so its slots grow
    as N^2 / (rows per block): 12.9 GB at N = 2^20 with 1024-row blocks, 206 GB at 2^22.
    The all-pairs plan keeps one slot per CTA piece of a row block: 36 MB at 2^20."""
    L = _lib.load()
    fn = L.grav_plan_pairs if mode in _lib.PAIR_MODES else L.grav_plan
    sizes = [int(x) for x in sizes]
    nu = len(sizes)
    n_arr = (ctypes.c_int32 * max(nu, 1))(*sizes)
    T_arr = (ctypes.c_double * max(nu, 1))(*([1.0] * max(nu, 1)))
    t = _lib.Tile(tile.bpt, tile.threads, tile.jtile, max(int(tile.grid), 1))
    info = _lib.PlanInfo()
    check(fn(nu, n_arr, T_arr, ctypes.byref(t), ctypes.byref(info), None, None))
    return int(L.grav_part_bytes(ctypes.byref(info))) * comps // 3


SLOT_BUDGET_FRACTION = 0.125
SLOT_BUDGET_NO_GPU = 32 << 30


def slot_budget_bytes(device=None):
    """Device memory that a unique-pair plan chosen by default may spend on partial-sum
    slots: an eighth of the GPU's memory (about 35 GB on a GB300); 32 GiB when no GPU is
    visible (host-side planning)."""
    if not torch.cuda.is_available():
        return SLOT_BUDGET_NO_GPU
    idx = torch.cuda.current_device() if device is None else torch.device(device).index
    if idx is None:
        idx = torch.cuda.current_device()
    return int(torch.cuda.get_device_properties(idx).total_memory * SLOT_BUDGET_FRACTION)


def fitting_tiles(sizes, mode, budget=None, comps=3, tiles=None):
    """The shapes in `tiles` (default: every compiled shape of `mode`) whose plan keeps
    its partial-sum slots within `budget` bytes (default slot_budget_bytes()); every shape
    in the all-pairs modes, whose slots do not grow with N^2.  The autotuner and the
    default shape choose among these."""
    tiles = list(tile_list(mode) if tiles is None else tiles)
    if mode not in _lib.PAIR_MODES:
        return tiles
    if budget is None:
        budget = slot_budget_bytes()
    return [t for t in tiles if plan_part_bytes(sizes, t, mode, comps) <= budget]


def pair_plan_fits(sizes, budget=None, mode='fp32u', comps=3, tiles=None):
    """True when some shape in `tiles` (default: every compiled shape of `mode`) keeps the
    unique-pair plan's slots within `budget` bytes (default slot_budget_bytes()); the
    autotuner and the default shape then pick only such shapes (fitting_tiles)."""
    return len(fitting_tiles(sizes, mode, budget, comps, tiles)) > 0


def _ctypes_to_device(arr, nbytes, device):
    host = torch.frombuffer(bytearray(ctypes.string_at(ctypes.addressof(arr), nbytes)),
                            dtype=torch.uint8) if nbytes else torch.zeros(0, dtype=torch.uint8)
    dev = torch.empty(max(nbytes, 16), dtype=torch.uint8, device=device)
    if nbytes:
        dev[:nbytes].copy_(host)
    return dev


def default_tile(mode, sizes, device=None):
    """Tile shape used when no tuned entry exists: the largest i-tile that still gives
    every resident CTA several work units."""
    info = device_info(device)
    cands = fitting_tiles(sizes, mode) or tile_list(mode)
    best = None
    for t in cands:
        occ = occupancy(mode, t, device)
        if occ <= 0:
            continue
        grid = info.sm_count * occ
        t.grid = grid
        pinfo, _, _ = make_plan(sizes, 1.0, t, mode)
        if pinfo.n_units == 0:
            # no pairs at all (only empty universes): stage 1 launches nothing, any
            # compiled shape serves
            if best is None:
                best = (float('inf'), _lib.Tile(t.bpt, t.threads, t.jtile, grid))
            continue
        # padded work (interactions) and the slowest CTA's share of it
        work = pinfo.n_units * pinfo.itile * t.jtile
        per_cta = -(-pinfo.n_units // min(grid, pinfo.n_units)) * pinfo.itile * t.jtile
        # register-blocked shapes issue fewer shared loads per interaction
        eff = {1: 0.80, 2: 0.90, 4: 0.97, 8: 1.0}.get(t.bpt, 0.9)
        score = per_cta / eff + 0.02 * work / grid
        if best is None or score < best[0]:
            best = (score, _lib.Tile(t.bpt, t.threads, t.jtile, grid))
    if best is None:
        raise RuntimeError('no compiled tile shape fits mode %r' % (mode,))
    return best[1]


FUSED_MODES = ('fp32', 'fp32n', 'fp32c')
# (largest n, (threads, rows)) of the single-launch step, the fastest measured on GB300
# (graph-replayed steps, fp32n / fp32, against the two-launch step's 8.7-9.0 / 7.7-8.3
# us): n <= 32 -- 3.6 / 3.5 us (one CTA); 64 -- 4.2 / 4.0 (one CTA); 128 -- 4.8 / 4.5 (a
# cluster of 4 CTAs); 256 -- 5.3 / 5.2 (8); 512 -- 6.5 / 5.9 (16).  From 1024 bodies
# the two-launch step, whose stage 1 spreads the pairs over every SM, is faster (9.4 us
# against 9.9 at 1024, 10.2 against 13.6 at 2048).
FUSED_RULE = ((32, (256, 64)), (64, (512, 64)), (128, (256, 32)), (512, (512, 32)))


def default_fused(mode, sizes, dev_info=None):
    """(threads, rows) of the single-launch step (grav_step_fused) for this workload, or
    None for the two-launch step: one universe of at most 512 bodies in an all-pairs
    FP32 mode."""
    if len(sizes) != 1 or mode not in FUSED_MODES:
        return None
    n = int(sizes[0])
    for n_max, cfg in FUSED_RULE:
        if 0 < n <= n_max:
            return cfg
    return None


class Engine:
    """Packed batch of universes on one GB300 with FP64 state.

    Parameters
      sizes : list of body counts (one per universe)
      T     : time step (scalar or one per universe)
      mode  : 'fp32' (default, all pairs), 'fp32u' (unique pairs), 'fp32n' / 'fp32un'
              (near pairs from double-single separations), 'fp32c' / 'fp32cu'
              (double-single separations for every pair) or 'fp64'
      tile  : _lib.Tile, or None to use the autotuner's choice / the default shape
      fused : single-launch step (grav_step_fused) for one small universe: (threads,
              rows) per CTA, False for the two-launch step, None to decide by size
              (default_fused)
    """

    def __init__(self, sizes, T, mode='fp32', tile=None, device=None, tuner=None, fused=None):
        self.lib = _lib.load()
        self.dev_info = device_info(device)
        self.device = torch.device('cuda', self.dev_info.index)
        if isinstance(mode, str):
            if mode not in _lib.MODES:
                raise ValueError('unknown precision mode %r (%s)' % (mode, ', '.join(_lib.MODES)))
            self.mode_name, self.mode = mode, _lib.MODES[mode]
        else:
            self.mode = int(mode)
            self.mode_name = {v: k for k, v in _lib.MODES.items()}[self.mode]
        self.sizes = [int(x) for x in sizes]
        self.T = list(T) if np.ndim(T) else [float(T)] * len(self.sizes)
        if fused is None:
            fused = default_fused(self.mode_name, self.sizes, self.dev_info)
        if tile is None:
            if tuner is not None and not fused:
                tile = tuner.choose(self.mode_name, self.sizes, self.dev_info, T=self.T)
            else:
                tile = default_tile(self.mode_name, self.sizes, self.dev_info.index)
        elif tile.grid <= 0:
            tile = _lib.Tile(tile.bpt, tile.threads, tile.jtile,
                             self.dev_info.sm_count * occupancy(self.mode, tile, self.dev_info.index))
        if not self.lib.grav_tile_supported(self.mode, ctypes.byref(tile)):
            raise ValueError('tile %r is not compiled for mode %s' % (tile, self.mode_name))
        self.tile = tile
        self.info, univ, seg = make_plan(self.sizes, self.T, tile, self.mode_name)
        info = self.info
        dev = self.device
        self.univ_dev = _ctypes_to_device(univ, ctypes.sizeof(_lib.UnivDesc) * info.n_univ, dev)
        self.seg_dev = _ctypes_to_device(seg, ctypes.sizeof(_lib.SegDesc) * info.n_seg, dev)
        self.univ_host = univ
        self.seg_host = seg
        nb = max(info.n_bodies, 1)
        self.r = torch.zeros((nb, 4), dtype=torch.float64, device=dev)
        self.v = torch.zeros((nb, 4), dtype=torch.float64, device=dev)
        self.a = torch.zeros((nb, 4), dtype=torch.float64, device=dev)
        pos_bytes = int(self.lib.grav_pos_bytes(self.mode, info.n_pad_total))
        self.pos = torch.zeros(max(pos_bytes // 4, 4), dtype=torch.float32, device=dev)
        part_bytes = int(self.lib.grav_part_bytes(ctypes.byref(info)))
        self.part = torch.zeros(max(part_bytes // 8, 1), dtype=torch.float64, device=dev)
        self.err = torch.zeros(1, dtype=torch.int32, device=dev)
        b = _lib.Batch()
        b.mode = self.mode
        b.n_univ = info.n_univ
        b.n_seg = info.n_seg
        b.n_slots = info.n_slots
        b.n_bodies = info.n_bodies
        b.n_pad_total = info.n_pad_total
        b.n_units = info.n_units
        b.tile = _lib.Tile(tile.bpt, tile.threads, tile.jtile, info.grid)
        b.eps2 = 1e-30
        b.univ = self.univ_dev.data_ptr()
        b.seg = self.seg_dev.data_ptr()
        b.r = self.r.data_ptr()
        b.v = self.v.data_ptr()
        b.pos = self.pos.data_ptr()
        b.part = self.part.data_ptr()
        b.a_out = self.a.data_ptr()
        b.err = self.err.data_ptr()
        self.batch = b
        self._bref = ctypes.byref(b)
        self.offsets = np.array([u.body_off for u in list(univ)[:info.n_univ]], dtype=np.int64)
        self.fused = None
        if fused:
            threads, rows = int(fused[0]), int(fused[1])
            n = self.sizes[0] if len(self.sizes) == 1 else -1
            if len(self.sizes) != 1 or not self.lib.grav_fused_supported(self.mode, n, threads, rows):
                raise ValueError('no single-launch step for mode %s, sizes %s, %d threads, %d rows'
                                 % (self.mode_name, self.sizes[:4], threads, rows))
            occ = ctypes.c_int32()
            with torch.cuda.device(dev):
                check(self.lib.grav_fused_occupancy(self.mode, n, threads, rows, ctypes.byref(occ)))
            if -(-n // rows) > occ.value * self.dev_info.sm_count:
                raise ValueError('%d CTAs of the single-launch step are not resident at once'
                                 % -(-n // rows))
            self.fused = (threads, rows)
            # grid-barrier counters of grav_step_fused (zero between calls)
            self.sync = torch.zeros(2, dtype=torch.int32, device=dev)

    # ---- state ----------------------------------------------------------------------
    def set_state(self, r, v, gm, stream=None):
        """Load positions, velocities and G*m (already scaled) for all bodies, packed."""
        n = self.info.n_bodies
        r = torch.as_tensor(np.asarray(r, dtype=np.float64).reshape(n, 3) if not torch.is_tensor(r)
                            else r.reshape(n, 3), dtype=torch.float64)
        v = torch.as_tensor(np.asarray(v, dtype=np.float64).reshape(n, 3) if not torch.is_tensor(v)
                            else v.reshape(n, 3), dtype=torch.float64)
        gm = torch.as_tensor(np.asarray(gm, dtype=np.float64).reshape(n) if not torch.is_tensor(gm)
                             else gm.reshape(n), dtype=torch.float64)
        if not bool(torch.isfinite(gm).all()) or bool((gm < 0).any()):
            raise ValueError('G*m must be finite and >= 0')
        max_gm = float(gm.max()) if n else 0.0
        self.batch.eps2 = float(self.lib.grav_eps2(max_gm))
        with torch.cuda.stream(self._stream(stream)):
            self.r[:n, :3].copy_(r, non_blocking=False)
            self.r[:n, 3].copy_(gm)
            self.v[:n, :3].copy_(v)
            self.v[:n, 3].zero_()
        self.prepare(stream)

    def generate_state(self, scenarios, G, stream=None):
        """Fill r and v on the device from seeded scenarios (gravitation_gb300.generate):
        one list of parts per universe, covering exactly that universe's bodies; G is
        the (scaled) constant the G*m column is formed with (one per universe or one
        for all).  Sets eps2 from the largest G*m and refreshes the stage-1 positions."""
        from . import generate as gen
        if len(scenarios) != len(self.sizes):
            raise ValueError('%d scenarios for %d universes' % (len(scenarios), len(self.sizes)))
        Gs = list(G) if np.ndim(G) else [float(G)] * len(self.sizes)
        st = self._stream(stream)
        for u, parts in enumerate(scenarios):
            n = self.sizes[u]
            if gen.total_bodies(parts) != n or sum(p.n for p in parts) != n:
                raise ValueError('scenario of universe %d does not cover its %d bodies' % (u, n))
            o = int(self.offsets[u])
            gen.generate(parts, self.r[o:o + n], self.v[o:o + n], Gs[u], st)
        nb = self.info.n_bodies
        st.synchronize()  # r may be host memory the device wrote (bind_host_state)
        with torch.cuda.stream(st):
            max_gm = float(self.r[:nb, 3].max()) if nb else 0.0
        self.batch.eps2 = float(self.lib.grav_eps2(max_gm))
        self.prepare(st)

    def bind_host_state(self, hr, hv):
        """Keep r and v in page-locked host tensors hr, hv (float64 [n_bodies, 4], same
        layout): prepare and stage 2 then read and write them in place over the CPU-GPU
        link, and the device copies are no longer used.  Returns False, changing
        nothing, if the tensors are not page-locked memory the device can address."""
        n = self.info.n_bodies
        for t in (hr, hv):
            if (t.device.type != 'cpu' or t.dtype != torch.float64 or tuple(t.shape) != (n, 4)
                    or not t.is_contiguous()):
                raise ValueError('host state must be contiguous float64 [%d, 4] CPU tensors' % n)
        ptrs = []
        for t in (hr, hv):
            p = ctypes.c_void_p()
            if not t.is_pinned() or self.lib.grav_host_device_pointer(
                    ctypes.c_void_p(t.data_ptr()), ctypes.byref(p)) != _lib.GRAV_OK:
                return False
            ptrs.append(p.value)
        self.r, self.v = hr, hv
        self.batch.r, self.batch.v = ptrs
        return True

    def _stream(self, stream):
        return stream if stream is not None else torch.cuda.current_stream(self.device)

    def _h(self, stream):
        return ctypes.c_void_p(self._stream(stream).cuda_stream)

    # ---- stages ---------------------------------------------------------------------
    def prepare(self, stream=None):
        """Refresh the padded stage-1 positions after r was changed."""
        check(self.lib.grav_prepare(self._bref, self._h(stream)))

    def stage1(self, stream=None):
        check(self.lib.grav_stage1(self._bref, self._h(stream)))

    def stage2(self, flags=_lib.GRAV_S2_INTEGRATE, stream=None):
        check(self.lib.grav_stage2(self._bref, int(flags), self._h(stream)))

    def step(self, steps=1, stream=None, write_a=False):
        """`steps` full steps (stage 1 + stage 2, or the single-launch step) queued on the
        stream."""
        flags = _lib.GRAV_S2_INTEGRATE | (_lib.GRAV_S2_WRITE_A if write_a else 0)
        h = self._h(stream)
        if self.fused:
            threads, rows = self.fused
            sync = ctypes.c_void_p(self.sync.data_ptr())
            for _ in range(int(steps)):
                check(self.lib.grav_step_fused(self._bref, flags, threads, rows, sync, h))
            return
        for _ in range(int(steps)):
            check(self.lib.grav_step(self._bref, flags, h))

    def capture_graph(self, steps=1):
        """CUDA graph of `steps` full steps (the steady-state step: stage 1 + stage 2,
        2 launches per step); returns a torch.cuda.CUDAGraph whose replay() runs them.
        The launches are recorded on a side stream that torch puts into capture mode."""
        side = torch.cuda.Stream(device=self.device)
        side.wait_stream(torch.cuda.current_stream(self.device))
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=side):
            self.step(steps, stream=side)
        torch.cuda.current_stream(self.device).wait_stream(side)
        return g

    def forces(self, stream=None):
        """Stage 1 only; returns the accelerations (float64 [n_bodies, 3], device)."""
        self.stage1(stream)
        self.stage2(_lib.GRAV_S2_WRITE_A, stream)
        return self.a[:self.info.n_bodies, :3]

    # ---- diagnostics ----------------------------------------------------------------
    DIAG_TILE = (2, 128, 128)

    def _fp64_view(self):
        """An FP64-mode batch sharing r and v, with its own all-pairs plan, padded double4
        positions and partial-sum scratch (so a diagnostic never clobbers stage 1)."""
        if getattr(self, '_b64', None) is None:
            t = _lib.Tile(*self.DIAG_TILE, 0)
            t.grid = self.dev_info.sm_count * max(
                occupancy(_lib.GRAV_MODE_FP64, t, self.dev_info.index), 1)
            info, univ, seg = make_plan(self.sizes, self.T, t, 'fp64')
            dev = self.device
            self._univ64 = _ctypes_to_device(univ, ctypes.sizeof(_lib.UnivDesc) * info.n_univ, dev)
            self._seg64 = _ctypes_to_device(seg, ctypes.sizeof(_lib.SegDesc) * info.n_seg, dev)
            nbytes = int(self.lib.grav_pos_bytes(_lib.GRAV_MODE_FP64, info.n_pad_total))
            self._pos64 = torch.zeros(max(nbytes // 8, 4), dtype=torch.float64, device=dev)
            self._part64 = torch.zeros(max(int(self.lib.grav_part_bytes(ctypes.byref(info))) // 8,
                                           1), dtype=torch.float64, device=dev)
            self._out64 = torch.zeros(max(info.n_univ, 1) * 8, dtype=torch.float64, device=dev)
            b = _lib.Batch()
            b.mode = _lib.GRAV_MODE_FP64
            b.n_univ, b.n_seg, b.n_slots = info.n_univ, info.n_seg, info.n_slots
            b.n_bodies, b.n_pad_total, b.n_units = info.n_bodies, info.n_pad_total, info.n_units
            b.tile = _lib.Tile(t.bpt, t.threads, t.jtile, info.grid)
            b.eps2 = 1e-30
            b.univ, b.seg = self._univ64.data_ptr(), self._seg64.data_ptr()
            b.r, b.v = self.r.data_ptr(), self.v.data_ptr()
            b.pos, b.part = self._pos64.data_ptr(), self._part64.data_ptr()
            b.a_out, b.err = self.a.data_ptr(), self.err.data_ptr()
            self._b64 = b
        return self._b64

    def energy(self, G, stream=None):
        """FP64 (kinetic, potential, momentum[3]) per universe as a numpy array
        [n_univ, 5]; G is the (scaled) gravitational constant of the universes."""
        b = self._fp64_view()
        h = self._h(stream)
        check(self.lib.grav_prepare(ctypes.byref(b), h))
        check(self.lib.grav_energy(ctypes.byref(b), ctypes.c_void_p(self._out64.data_ptr()), h))
        out = self._out64.view(-1, 8)[:self.info.n_univ, :5].cpu().numpy() / float(G)
        self.raise_on_device_error()
        return out

    # ---- errors ---------------------------------------------------------------------
    def device_error(self):
        """Device error flag (GRAV_DEV_*); synchronises the stream."""
        return int(self.err.item())

    def raise_on_device_error(self):
        code = self.device_error()
        if code != _lib.GRAV_DEV_OK:
            self.err.zero_()
            raise _lib.GravError(_lib.GRAV_E_CUDA, 'device error flag %d (%s)' % (
                code, 'bounded wait expired: a bulk copy or a grid barrier'
                if code == _lib.GRAV_DEV_TIMEOUT else 'unknown'))

    # ---- views ----------------------------------------------------------------------
    def universe_slice(self, u):
        o = int(self.offsets[u])
        return slice(o, o + self.sizes[u])

    def interactions_per_step(self):
        """Algorithmic interactions per step: sum over universes of N^2."""
        return sum(n * n for n in self.sizes)
