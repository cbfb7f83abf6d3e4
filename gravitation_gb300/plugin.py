"""GB300 implementation of the plugin hooks of ``universe_base``.

``GB300Stages`` is mixed in front of ``universe_base`` by the ``gb1`` kernel package
(class universe(GB300Stages, universe_base)).  It overrides only the hooks the
reference lets kernels override (_base_.py:131-177): start_kernel, step_stage1,
step_stage2 and stop_kernel.  ``__init__``, ``add_object``, ``step`` and iteration
stay the base class's.

Behaviour seen from the front end (README.md:50, worker.py:119-136):
  - after every step() the position and velocity of each point mass are valid
    iterables: ``pm._r`` / ``pm._v`` are numpy row views of a pinned FP64 host mirror
    (the binding pattern of np2.py:70-75);
  - step() is synchronous, so wall-clock timing of step() is valid;
  - with host_sync='full' (default) the mirror is the source of truth: edits of
    pm._r / pm._v between steps are uploaded at the next step, as the reference's
    kernels re-read pm._r every stage 1 (np1.py:101-102, pc2.py:147-151).

Kernel options (keyword arguments of the constructor, kept in self._meta):
  precision  'fp32n' | 'fp32un' | 'fp32' | 'fp32u' | 'fp32c' | 'fp32cu' | 'fp64'   default
             from dtype: 'float32' -> fp32n below 4608 bodies, fp32un from there on while
             its partial-sum slots fit an eighth of the GPU's memory (~1.7 M bodies);
             fp32c / fp32cu instead when more than 1e-3 of sampled pairs are near
             (default_mode, near_pair_fraction: discs, dense clusters far out);
             'float64' -> fp64.  fp32/fp32u: plain FP32 separations (fp32u visits each
             pair once); fp32n/fp32un: the same plus double-single separations for near
             pairs (closer than |x|/20), which keeps every body within ~1e-6 of the FP64
             forces wherever the bodies are; fp32c/fp32cu: double-single separations for
             every pair
  host_sync  'full' (upload + download every step) | 'pull' (download only) |
             'none' (device state only; call sync_host() to refresh the mirror)
  fuse       True (default): stage 1 and stage 2 both run in step_stage1 on the GPU
             (for one universe of up to 512 bodies in a single kernel, the engine's
             single-launch step) and step_stage2 refreshes the mirror; False:
             step_stage1 fills pm._a like the reference's kernels and step_stage2
             integrates on the GPU
  tile       (bpt, threads, jtile) to force a tile shape; default: autotuned
  autotune   True (default) to use the autotuner cache / tuning
  device     CUDA device index (default: current device)
  graph      True (default): with fuse, a step is one CUDA-graph replay of upload,
             stage 1, stage 2 and download (the velocity upload overlaps stage 1);
             False: the same work launched call by call
  zero_copy  True (default): with host_sync='full', r and v stay in the pinned host
             mirror, which the GPU reads and writes in place over the CPU-GPU link
             (NVLink-C2C on Grace); False: device copies, uploaded and downloaded
  scenario   instead of add_object calls: a dict such as {'kind': 'plummer_pair',
             'n': 16384, 'seed': 2} or a list of gravitation_gb300.generate parts; the
             bodies are generated on the device in the universe's scaled units and
             the point masses are made on first access (see _MirrorMasses)
"""

import ctypes
import sys

import numpy as np
import torch

from . import _lib, generate
from .engine import Engine

# float32 runs the FP32 arithmetic with near pairs corrected, either on unique pairs
# (fp32un: each pair once, like the reference's CPU kernels) or on all ordered pairs
# (fp32n: finer work units, faster for small universes); the results agree to FP32
# rounding.  Measured on GB300 (graph-replayed steps on an evolved cube, each mode with
# its tuned tile), fp32n against fp32un: 3072 bodies 12.9 / 17.1 us, 4096 17.8 / 18.6,
# 4608 21.3 / 21.4, 6144 30.0 / 25.5, 8192 49.4 / 39.1, 16384 156 / 118.
_DTYPE_MODE = {'float32': 'fp32n', 'float64': 'fp64'}
UNIQUE_PAIRS_FROM_N = 4608


# Above this fraction of near pairs the near-corrected kernels spend more time on their
# correction path than double-single separations for every pair cost (fp32c / fp32cu,
# ~1.4x the plain loop): the near path then runs on most steps of the loop.
NEAR_DS_FRACTION = 1e-3


def near_pair_fraction(r, samples=1 << 16, seed=0, rows=8):
    """Fraction of `samples` seeded random pairs (i != j) of positions r (n x >=3) that
    the near-corrected kernels treat as near: |r_j - r_i| below m / GRAV_NEAR_KAPPA,
    where m is the largest |coordinate| among the `rows` bodies a thread holds (i and
    rows - 1 others drawn at random, as the kernels' rows are spread over the body
    order).  About 5e-5 for the uniform cube of the benchmark; dense clusters far from
    the origin, and discs whose outer bodies set the radius for the inner ones, reach
    1e-3 and more."""
    r = np.asarray(r, dtype=np.float64)[:, :3]
    n = len(r)
    if n < 2:
        return 0.0
    rng = np.random.default_rng(seed)
    i = rng.integers(n, size=samples)
    j = rng.integers(n - 1, size=samples)
    j += j >= i
    d2 = ((r[j] - r[i]) ** 2).sum(1)
    scale = np.abs(r).max(1)
    others = rng.integers(n, size=(samples, max(rows - 1, 0)))
    m = np.maximum(scale[i], scale[others].max(1) if rows > 1 else 0.0)
    thr = (m / _lib.GRAV_NEAR_KAPPA) ** 2
    return float((d2 < thr).mean())


def default_mode(dtype, n, budget=None, r=None):
    """Precision mode for a dtype and body count: float32 runs on unique pairs from
    UNIQUE_PAIRS_FROM_N bodies while the unique-pair plan's partial-sum slots fit the
    slot budget (engine.slot_budget_bytes, or `budget` bytes), on all pairs otherwise
    (above ~1.7 million bodies on a GB300); near pairs are corrected (fp32n / fp32un),
    or, given positions r whose near-pair fraction exceeds NEAR_DS_FRACTION, every pair
    takes double-single separations (fp32c / fp32cu).  Both keep the forces within
    1e-5 of FP64."""
    mode = _DTYPE_MODE.get(str(dtype))
    if mode == 'fp32n' and n >= UNIQUE_PAIRS_FROM_N:
        from .engine import pair_plan_fits
        if pair_plan_fits([n], budget, mode='fp32un'):
            mode = 'fp32un'
    if mode in ('fp32n', 'fp32un') and r is not None and \
            near_pair_fraction(r) > NEAR_DS_FRACTION:
        mode = {'fp32n': 'fp32c', 'fp32un': 'fp32cu'}[mode]
    return mode


class _MirrorMasses:
    """The point-mass list of a universe whose bodies were generated on the device.

    Behaves as the base class's ``_mass_list`` does for its readers (``len``,
    iteration, indexing: _base_.py:95-100): each body is a ``_point_mass`` of the
    base class, made on first access, whose ``_r``, ``_v`` and ``_a`` are rows of the
    pinned host mirror and whose ``_m`` is the scaled mass.  Nothing per body is
    built before the front end asks for it."""

    def __init__(self, cls, hr, hv, ha, G, parts):
        self._cls, self._hr, self._hv, self._ha, self._G = cls, hr, hv, ha, G
        self._items = [None] * len(hr)
        self._names = []
        for p in parts:
            self._names.append((p.offset, p.offset + p.n, p.kind))

    def __len__(self):
        return len(self._items)

    def __getitem__(self, i):
        if isinstance(i, slice):
            return [self[k] for k in range(*i.indices(len(self._items)))]
        i = range(len(self._items))[i]
        pm = self._items[i]
        if pm is None:
            name = next((k for lo, hi, k in self._names if lo <= i < hi), 'body')
            m = float(self._hr[i, 3]) / self._G if self._G else 0.0
            pm = self._cls(name='%s %d' % (name, i), r=self._hr[i, :3], v=self._hv[i, :3], m=m)
            pm._a = self._ha[i, :3]
            self._items[i] = pm
        return pm

    def __iter__(self):
        for i in range(len(self._items)):
            yield self[i]


class GB300Stages:
    """start/step/stop hooks of a gravitation kernel running on one GB300."""

    def start_kernel(self):
        meta = self._meta
        parts = None
        if meta.get('scenario') is not None:
            if len(self._mass_list):
                raise ValueError('a scenario generated on the device replaces add_object: '
                                 'use one or the other')
            spec = meta['scenario']
            parts = list(spec) if isinstance(spec, (list, tuple)) else generate.from_spec(spec)
            n = generate.total_bodies(parts)
        else:
            n = len(self._mass_list)
        mode = meta.get('precision') or default_mode(self._dtype, n)
        if mode not in _lib.MODES:
            raise ValueError('unsupported dtype/precision %r (float32, float64, %s)' % (
                meta.get('precision') or self._dtype, ', '.join(_lib.MODES)))
        self._gb_sync = meta.get('host_sync', 'full')
        if self._gb_sync not in ('full', 'pull', 'none'):
            raise ValueError('host_sync must be full, pull or none')
        self._gb_fuse = bool(meta.get('fuse', True))
        if n == 0:
            raise ValueError('no point masses were added before start()')
        tile = meta.get('tile')
        tuner = None
        if tile is not None:
            tile = _lib.Tile(int(tile[0]), int(tile[1]), int(tile[2]), 0)
        elif meta.get('autotune', True):
            from .tune import default_tuner
            tuner = default_tuner()
        device = meta.get('device')

        def make_engine(m):
            return Engine([n], float(self._T), mode=m, tile=tile, device=device, tuner=tuner)
        self._gb = make_engine(mode)
        dev = self._gb.device
        # pinned FP64 host mirror (x, y, z, G*m) / (vx, vy, vz, 0) / (ax, ay, az, 0)
        pin = torch.cuda.is_available()
        self._gb_hr = torch.zeros((n, 4), dtype=torch.float64, pin_memory=pin)
        self._gb_hv = torch.zeros((n, 4), dtype=torch.float64, pin_memory=pin)
        self._gb_ha = torch.zeros((n, 4), dtype=torch.float64, pin_memory=pin)
        hr, hv, ha = self._gb_hr.numpy(), self._gb_hv.numpy(), self._gb_ha.numpy()
        self._gb_herr = torch.zeros(1, dtype=torch.int32, pin_memory=pin)
        self._gb_herr_np = self._gb_herr.numpy()
        self._gb_stream = torch.cuda.Stream(device=dev)
        self._gb_side = torch.cuda.Stream(device=dev)
        self._gb_wait = self._gb_stream  # the stream the queued step runs on
        if parts is not None:
            # bodies written by the device, then one copy into the host mirror
            self._gb.generate_state([parts], G=self._G, stream=self._gb_stream)
            with torch.cuda.stream(self._gb_stream):
                self._gb_hr.copy_(self._gb.r[:n], non_blocking=True)
                self._gb_hv.copy_(self._gb.v[:n], non_blocking=True)
            self._gb_stream.synchronize()
            self._mass_list = _MirrorMasses(self._point_mass_class(), hr, hv, ha, self._G,
                                            parts)
        else:
            for i, pm in enumerate(self._mass_list):
                hr[i, :3] = pm._r[:3]
                hr[i, 3] = self._G * pm._m
                hv[i, :3] = pm._v[:3]
            if not np.all(np.isfinite(hr)) or not np.all(np.isfinite(hv)):
                raise ValueError('positions, velocities and masses must be finite')
            self._gb.set_state(hr[:, :3], hv[:, :3], hr[:, 3], stream=self._gb_stream)
            self._gb_stream.synchronize()
            # np2-style binding: the point masses see rows of the host mirror
            for i, pm in enumerate(self._mass_list):
                pm._r = hr[i, :3]
                pm._v = hv[i, :3]
                pm._a = ha[i, :3]
        if not meta.get('precision') and mode in ('fp32n', 'fp32un'):
            # with the positions known: dense configurations far from the origin take
            # double-single separations for every pair (default_mode)
            chosen = default_mode(self._dtype, n, r=hr)
            if chosen != mode:
                if tile is not None and not self._gb.lib.grav_tile_supported(
                        _lib.MODES[chosen], ctypes.byref(tile)):
                    chosen = mode
            if chosen != mode:
                self._gb = make_engine(chosen)
                self._gb.set_state(hr[:, :3], hv[:, :3], hr[:, 3], stream=self._gb_stream)
                self._gb_stream.synchronize()
        self._gb_a_dirty = False
        # host_sync='full' keeps the state in the host mirror itself when the device can
        # address it: prepare and stage 2 read and write it in place
        self._gb_zero_copy = False
        if self._gb_sync == 'full' and meta.get('zero_copy', True):
            self._gb_zero_copy = self._gb.bind_host_state(self._gb_hr, self._gb_hv)
        self._gb_graph = None
        if self._gb_fuse and meta.get('graph', True):
            self._gb_graph = self._gb_capture()

    def _point_mass_class(self):
        """The ``_point_mass`` class of the module that defines this universe's base."""
        for c in type(self).__mro__:
            if c.__name__ == 'universe_base':
                return getattr(sys.modules[c.__module__], '_point_mass')
        raise TypeError('no universe_base among the bases of %r' % (type(self),))

    # ---- stages ----------------------------------------------------------------------
    def _gb_enqueue_step(self):
        """Queue one fused step on the kernel's stream: upload (host_sync='full'),
        stage 1, stage 2, download (full/pull) and the device error flag.  With an
        upload, positions go first and the velocities travel on a side stream while
        stage 1 runs (stage 1 reads only positions).  With the state in the host
        mirror (zero_copy) prepare reads the positions and stage 2 updates r and v in
        place, so only the error flag is copied."""
        g, s, side = self._gb, self._gb_stream, self._gb_side
        if self._gb_zero_copy:
            g.prepare(stream=s)
            g.step(1, stream=s)
            self._gb_enqueue_download(state=False)
            return
        if self._gb_sync == 'full':
            side.wait_stream(s)
            with torch.cuda.stream(side):
                g.v.copy_(self._gb_hv, non_blocking=True)
            with torch.cuda.stream(s):
                g.r.copy_(self._gb_hr, non_blocking=True)
            g.prepare(stream=s)
            g.stage1(stream=s)
            s.wait_stream(side)
            g.stage2(_lib.GRAV_S2_INTEGRATE, stream=s)
        else:
            g.step(1, stream=s)
        self._gb_enqueue_download(state=self._gb_sync in ('full', 'pull'))

    def _gb_enqueue_download(self, state=True, with_a=False):
        g, s = self._gb, self._gb_stream
        with torch.cuda.stream(s):
            if state and not self._gb_zero_copy:
                self._gb_hr.copy_(g.r, non_blocking=True)
                self._gb_hv.copy_(g.v, non_blocking=True)
            if with_a:
                self._gb_ha.copy_(g.a, non_blocking=True)
            self._gb_herr.copy_(g.err, non_blocking=True)

    def _gb_capture(self):
        """CUDA graph of one fused step (memory copies and kernels; the pinned host
        mirror and the device buffers keep their addresses for the universe's life)."""
        s = self._gb_stream
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph, stream=s):
            self._gb_enqueue_step()
        return graph

    def _gb_finish(self):
        """Wait for the queued work; raise on the device error flag it copied back."""
        self._gb_wait.synchronize()
        self._gb_wait = self._gb_stream
        if int(self._gb_herr_np[0]) != _lib.GRAV_DEV_OK:
            self._gb.raise_on_device_error()

    def _gb_download(self, state=True):
        self._gb_enqueue_download(state=state)
        self._gb_finish()

    def step_stage1(self):
        if self._gb_fuse:
            if self._gb_graph is not None:
                # replay() launches on the current stream; the step is synchronous, so
                # step_stage2 waits for that stream (entering a stream context for the
                # replay would cost more than the replay's own launch)
                if torch.cuda.current_device() == self._gb.device.index:
                    self._gb_wait = torch.cuda.current_stream()
                    self._gb_graph.replay()
                else:
                    with torch.cuda.stream(self._gb_stream):
                        self._gb_graph.replay()
            else:
                self._gb_enqueue_step()
            return
        g, s = self._gb, self._gb_stream
        if self._gb_sync == 'full':
            if not self._gb_zero_copy:
                with torch.cuda.stream(s):
                    g.r.copy_(self._gb_hr, non_blocking=True)
                    g.v.copy_(self._gb_hv, non_blocking=True)
            g.prepare(stream=s)
        g.stage1(stream=s)
        g.stage2(_lib.GRAV_S2_WRITE_A, stream=s)
        self._gb_enqueue_download(state=False, with_a=True)
        self._gb_finish()
        self._gb_a_dirty = True

    def step_stage2(self):
        if self._gb_fuse:
            # the step queued by step_stage1 already holds its download
            self._gb_finish()
            return
        self._gb.stage2(_lib.GRAV_S2_INTEGRATE, stream=self._gb_stream)
        self._gb_download(state=self._gb_sync in ('full', 'pull'))
        # the base class's stage 2 leaves the accelerations zeroed (_base_.py:62);
        # only the unfused stage 1 writes them
        if self._gb_a_dirty:
            self._gb_ha[:, :3] = 0.0
            self._gb_a_dirty = False

    def sync_host(self):
        """Refresh the host mirror (pm._r, pm._v) from the device state."""
        self._gb_download()

    def stop_kernel(self):
        if getattr(self, '_gb', None) is not None:
            self._gb_stream.synchronize()
            self.sync_host()
            self._gb_graph = None
            self._gb = None
