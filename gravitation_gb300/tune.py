"""Autotuner for the stage-1 tile shape (bodies per thread, threads per CTA, j-tile).

For a workload key -- the GPU (name, SM count), the precision mode, the library's
source hash and the size bucket (single universe: N rounded up to a quarter octave,
m * 2^k with m in 4..7; batch: the size classes of its universe count and of its
largest universe and the binary order of magnitude of its sum of N^2, so that batches of
the same make-up share a tuned tile whatever their exact sizes) -- every compiled tile
shape whose partial-sum slots fit the slot budget, at 1, 1/2 and 1/4 of the resident
persistent grid, is timed as full steps replayed from a CUDA graph (CUDA events, at
least ~2 ms of steps) on a seeded synthetic state of the sizes that asked, at their
time step, and the fastest is cached as JSON (the four fastest of that pass timed
again, longer, and the best of those kept).

Cache robustness: an unreadable or malformed cache file is ignored (and rewritten),
entries from another library build (different source hash) or naming a tile that is
not compiled are ignored, and nothing is trusted that does not pass
``grav_tile_supported``.  The cache path is $GRAV_TUNE_CACHE or
gravitation_gb300/_tune_cache.json.
"""

import json
import os
import tempfile
import threading

import numpy as np

from . import _lib
from .build import source_hash

HERE = os.path.dirname(os.path.abspath(__file__))


def size_class(n):
    """Power-of-two class of a universe size: the smallest 2^k >= n (0 for no bodies)."""
    n = int(n)
    return 0 if n <= 0 else 1 << (n - 1).bit_length()


def fine_class(n):
    """Quarter-octave class of one universe's size: the smallest m * 2^k >= n with m in
    {4, 5, 6, 7} (n itself below 4; 0 for no bodies)."""
    n = int(n)
    if n < 4:
        return max(n, 0)
    k = max(0, (n - 1).bit_length() - 3)
    m = -(-n // (1 << k))          # 4 < m <= 8
    return (m << k) if m < 8 else (1 << (k + 3))


def bucket_of(sizes):
    """Tuner key of a size list.  One universe: its quarter-octave class (fine_class).  A
    batch: the size class of its universe count, the binary order of magnitude of its
    work (sum of N^2) and the size class of its largest universe, e.g.
    'batch:u256:w32:max16384' -- what the tile choice depends on -- so that batches
    drawn from one distribution (other seeds of the same log-uniform range) share their
    tuned tile."""
    sizes = [int(s) for s in sizes]
    if len(sizes) == 1:
        return 'single:%d' % fine_class(max(sizes[0], 1))
    work = sum(n * n for n in sizes)
    return 'batch:u%d:w%d:max%d' % (size_class(len(sizes)), max(work, 1).bit_length() - 1,
                                    size_class(max(sizes + [0])))


class Tuner:
    def __init__(self, path=None, build_hash=None):
        self.path = path or os.environ.get('GRAV_TUNE_CACHE') or os.path.join(
            HERE, '_tune_cache.json')
        self._build_hash = build_hash
        self._lock = threading.Lock()
        self._cache = None

    @property
    def build_hash(self):
        if self._build_hash is None:
            self._build_hash = source_hash()
        return self._build_hash

    # ---- cache ----------------------------------------------------------------------
    def load(self):
        if self._cache is not None:
            return self._cache
        data = {}
        try:
            with open(self.path) as f:
                raw = json.load(f)
            if isinstance(raw, dict) and isinstance(raw.get('entries'), dict):
                data = raw['entries']
        except (OSError, ValueError):
            data = {}
        self._cache = data
        return data

    def save(self):
        data = {'format': 1, 'entries': self._cache or {}}
        d = os.path.dirname(os.path.abspath(self.path))
        os.makedirs(d, exist_ok=True)
        fd, tmp = tempfile.mkstemp(dir=d, prefix='.tune', suffix='.json')
        with os.fdopen(fd, 'w') as f:
            json.dump(data, f, indent=1, sort_keys=True)
        os.replace(tmp, self.path)

    def key(self, mode, sizes, dev_info):
        return '|'.join([dev_info.name, str(dev_info.sm_count), mode, bucket_of(sizes),
                         self.build_hash])

    def lookup(self, mode, sizes, dev_info):
        """Cached tile for the key, or None (missing, stale or invalid entry)."""
        ent = self.load().get(self.key(mode, sizes, dev_info))
        if not isinstance(ent, dict):
            return None
        try:
            t = _lib.Tile(int(ent['bpt']), int(ent['threads']), int(ent['jtile']), int(ent['grid']))
        except (KeyError, TypeError, ValueError):
            return None
        if t.grid <= 0:
            return None
        L = _lib.load()
        m = _lib.MODES[mode]
        import ctypes
        if not L.grav_tile_supported(m, ctypes.byref(t)):
            return None
        return t

    def store(self, mode, sizes, dev_info, tile, ms):
        with self._lock:
            self.load()[self.key(mode, sizes, dev_info)] = {
                'bpt': tile.bpt, 'threads': tile.threads, 'jtile': tile.jtile,
                'grid': tile.grid, 'ms': ms}
            self.save()

    # ---- tuning ---------------------------------------------------------------------
    def choose(self, mode, sizes, dev_info, tune_if_missing=None, T=None):
        """Tile for the workload: cached, else tuned (if enabled, with time step T), else
        the default.  The entry is tuned at the sizes that asked first and serves their
        whole bucket.  Single universes are bucketed by quarter octave (fine_class): with
        octave classes, the fp32un entry of the 4097-8192 class was tuned at ~5000
        bodies and ran a 8192-body step in 55 us against 39 us for the tile tuned at 8192
        (the stream-K work units quantise differently); tuning every entry at its
        class's upper edge instead cost sizes far below the edge up to 10 % (fp32n at
        5000 bodies: 53 against 48 us) and the per-universe loop of the batched
        workload 13 %."""
        from .engine import default_tile
        t = self.lookup(mode, sizes, dev_info)
        if t is not None:
            return t
        if sum(int(n) for n in sizes) == 0:
            return default_tile(mode, sizes, dev_info.index)   # nothing to time
        if tune_if_missing is None:
            tune_if_missing = os.environ.get('GRAV_AUTOTUNE', '1') != '0'
        if tune_if_missing:
            return self.tune(mode, sizes, dev_info, T=T)
        return default_tile(mode, sizes, dev_info.index)

    def tune(self, mode, sizes, dev_info, reps=5, grid_factors=(1, 0.5, 0.25), T=None):
        """Time every compiled tile shape, with the persistent grid at each of
        `grid_factors` x (SMs x resident CTAs), on a seeded state and cache the fastest.
        What is timed is the full step (stage 1 + stage 2) replayed from a CUDA graph: a
        smaller grid gives each CTA more work units but leaves fewer partial-sum slots
        per row for stage 2, which at a few thousand bodies is worth as much.  Above
        2^38 interactions per step a replay holds one step instead of `reps`.  The steps
        use the workload's time step T (one per universe or one for all; default the
        reference's 1e3): the near-pair kernels' cost follows the state, and a uniform
        cube streaming for a few steps at T = 1e3 takes the shape of its velocity
        distribution, where more pairs are near than in the cube (at T = 1 nothing
        moves, and the tiles with 8 rows per thread timed 12 % faster than they run)."""
        import torch
        from .engine import Engine, fitting_tiles, make_plan, occupancy, tile_list
        from .scenarios import uniform_cube
        sizes = [int(s) for s in sizes]
        rs, vs, ms = [], [], []
        for u, n in enumerate(sizes):
            r, v, m = uniform_cube(n, seed=1000 + u)
            rs.append(r)
            vs.append(v)
            ms.append(m * 6.6740831e-11)
        r = np.concatenate(rs) if rs else np.zeros((0, 3))
        v = np.concatenate(vs) if vs else np.zeros((0, 3))
        gm = np.concatenate(ms) if ms else np.zeros(0)
        best = None
        seen = set()
        step_T = 1e3 if T is None else T
        if sum(n * n for n in sizes) >= 1 << 38:
            # steps of 0.1 s and more (above ~500k bodies): one step per replay is
            # already far above the timing noise, and keeps tuning to about a minute
            reps = 1
        def time_tile(t, min_ms):
            """ms per step of tile t: full steps replayed from a CUDA graph, enough
            replays for about `min_ms` of steps (short steps time noisily)."""
            eng = Engine(sizes, step_T, mode=mode, tile=t, device=dev_info.index, fused=False)
            eng.set_state(r, v, gm)
            s = torch.cuda.current_stream(eng.device)
            g = eng.capture_graph(reps)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            g.replay()
            e0.record(s)
            g.replay()
            e1.record(s)
            e1.synchronize()
            k = max(1, min(100, int(min_ms / max(e0.elapsed_time(e1), 1e-3))))
            e0.record(s)
            for _ in range(k):
                g.replay()
            e1.record(s)
            e1.synchronize()
            eng.raise_on_device_error()
            out = e0.elapsed_time(e1) / (k * reps)
            del g, eng
            return out

        timed = []
        # unique-pair shapes whose partial-sum slots exceed the slot budget at these
        # sizes are not candidates (rows per block set the slots' N^2 / R growth)
        for cand in fitting_tiles(sizes, mode) or tile_list(mode):
            occ = occupancy(mode, cand, dev_info.index)
            if occ <= 0:
                continue
            for gf in grid_factors:
                grid = max(1, int(dev_info.sm_count * occ * gf))
                t = _lib.Tile(cand.bpt, cand.threads, cand.jtile, grid)
                pinfo = make_plan(sizes, 1.0, t, mode)[0]
                key = (t.bpt, t.threads, t.jtile, pinfo.grid)  # the plan caps the grid
                if key in seen:
                    continue
                seen.add(key)
                # the grid as tried, not as this size's plan capped it: the entry serves
                # every size of the bucket, each plan capping the grid at its own units
                timed.append((time_tile(t, 2.0), t))
        # a second pass over the closest candidates, with longer timings and in another
        # order: a single short timing picked tiles 10 % off the best on GB300
        timed.sort(key=lambda x: x[0])
        for ms_, t in timed[:4][::-1]:
            again = min(time_tile(t, 6.0), time_tile(t, 6.0))
            if best is None or again < best[0]:
                best = (again, t)
        if best is None:
            raise RuntimeError('no tile shape could be timed for mode %s' % mode)
        self.store(mode, sizes, dev_info, best[1], best[0])
        return best[1]


_DEFAULT = None


def default_tuner():
    global _DEFAULT
    if _DEFAULT is None:
        _DEFAULT = Tuner()
    return _DEFAULT
