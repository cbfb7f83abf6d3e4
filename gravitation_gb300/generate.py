"""Seeded scenarios generated on the GB300, straight into the packed FP64 state.

The reference builds its initial conditions in Python, one ``add_object`` call per
body (gravitation/lib/simulation.py:85-184, kernel/_base_.py:107-118).  Here the
bodies are written by the device (``grav_scenario_generate``: Philox4x64-10 counter-
based random numbers, one thread per body) into ``r`` = (x, y, z, G*m) and ``v`` =
(vx, vy, vz, 0), so a universe of 2^17 or 2^24 bodies starts without a per-body host
loop.  The values are in the universe's (scaled) units, i.e. what ``add_object``
stores after scaling.

A scenario is a list of ``Part`` objects, each filling ``n`` consecutive bodies of one
universe from ``offset`` on:

  uniform_cube(n, seed)   r ~ U[-1000,1000]^3, v ~ N(0,1)^3, m ~ U[1,100] (defaults)
  plummer_pair(n, seed)   two Plummer spheres (scale radius 50, centres at x = -500 and
                          +500, closing at 5 along x, masses log-uniform [0.1, 1000])
  galaxy(n, seed)         the reference's galaxy recipe (central mass + disc + bulge)
  from_spec(dict)         one of the above from {'kind': ..., 'n': ..., 'seed': ..., ...}

The same seed gives the same bits on every GB300 and for every launch shape.  These
are not the numpy streams of ``gravitation_gb300.scenarios`` (a different generator);
the CPU restatement used to check them lives with the tests' oracle.
"""

import ctypes

import torch

from . import _lib
from ._lib import check
from .scenarios import G_DEFAULT

KINDS = {'uniform_cube': _lib.GRAV_SCEN_UNIFORM_CUBE, 'plummer': _lib.GRAV_SCEN_PLUMMER,
         'galaxy': _lib.GRAV_SCEN_GALAXY}


class Part:
    """`n` bodies of one scenario kind written from body `offset` of a universe."""

    def __init__(self, kind, n, seed, stream=0, params=(), offset=0):
        if kind not in KINDS:
            raise ValueError('unknown scenario kind %r (%s)' % (kind, ', '.join(KINDS)))
        self.kind, self.n, self.seed, self.stream = kind, int(n), int(seed), int(stream)
        self.params = [float(x) for x in params]
        self.offset = int(offset)
        if self.n < 0 or self.offset < 0 or len(self.params) > 10:
            raise ValueError('bad scenario part')

    def struct(self, G):
        s = _lib.Scenario()
        s.kind = KINDS[self.kind]
        s.seed = self.seed & (2 ** 64 - 1)
        s.stream = self.stream & (2 ** 64 - 1)
        s.G = float(G)
        for k, x in enumerate(self.params):
            s.p[k] = x
        return s

    def __repr__(self):
        return 'Part(%s, n=%d, seed=%d, stream=%d, offset=%d, %r)' % (
            self.kind, self.n, self.seed, self.stream, self.offset, self.params)


def uniform_cube(n, seed=0, stream=0, half=1000.0, v_sigma=1.0, m_lo=1.0, m_hi=100.0):
    return [Part('uniform_cube', n, seed, stream, (half, v_sigma, m_lo, m_hi))]


def plummer_pair(n, seed=2, stream=0, a=50.0, sep=1000.0, vrel=5.0, m_lo=0.1, m_hi=1000.0):
    """Two Plummer spheres: the first n - n//2 bodies centred at (-sep/2, 0, 0) moving
    with +vrel/2 along x, the rest at (+sep/2, 0, 0) moving with -vrel/2."""
    n1 = n - n // 2
    return [Part('plummer', n1, seed, 2 * stream, (a, m_lo, m_hi, -0.5 * sep, 0, 0, 0.5 * vrel, 0, 0)),
            Part('plummer', n - n1, seed, 2 * stream + 1,
                 (a, m_lo, m_hi, 0.5 * sep, 0, 0, -0.5 * vrel, 0, 0), offset=n1)]


def galaxy(n, seed=0, stream=0, radius=1e20, m_hole=4e40, m_star=2e30, scale_r=1e-10,
           scale_m=1e-30):
    """The reference's galaxy scenario (simulation.py:57-77, 99-184): SI inputs, scaled
    by scale_r / scale_m; generate it with the universe's scaled G
    (G * scale_r^3 / scale_m, _base_.py:85-88), which the recipe also uses for the
    orbital speeds."""
    return [Part('galaxy', n, seed, stream, (radius, m_hole, m_star, scale_r, scale_m))]


def galaxy_universe_params(scale_r=1e-10, scale_m=1e-30):
    """Constructor arguments of the reference's galaxy simulation (simulation.py:57-63)."""
    return dict(T=2.0e12, scale_m=scale_m, scale_r=scale_r)


_BUILDERS = {'uniform_cube': uniform_cube, 'plummer_pair': plummer_pair, 'galaxy': galaxy}


def from_spec(spec):
    """Parts from a dict such as {'kind': 'plummer_pair', 'n': 16384, 'seed': 2}; other
    keys are the builder's keyword arguments."""
    spec = dict(spec)
    kind = spec.pop('kind')
    if kind not in _BUILDERS:
        raise ValueError('unknown scenario %r (%s)' % (kind, ', '.join(_BUILDERS)))
    n = int(spec.pop('n'))
    return _BUILDERS[kind](n, **spec)


def total_bodies(parts):
    return max((p.offset + p.n for p in parts), default=0)


def generate(parts, r, v, G=G_DEFAULT, stream=None):
    """Write the parts into r, v (float64 [n, 4] CUDA tensors, or pinned host tensors
    the device can address) on `stream`.  Returns nothing; work is queued."""
    lib = _lib.load()
    n = total_bodies(parts)
    for t in (r, v):
        if t.dtype != torch.float64 or t.dim() != 2 or t.shape[1] != 4 or not t.is_contiguous():
            raise ValueError('r and v must be contiguous float64 [n, 4] tensors')
        if t.shape[0] < n:
            raise ValueError('r and v hold %d rows; the scenario needs %d' % (t.shape[0], n))
    if r.is_cuda:
        device = r.device
        r_ptr, v_ptr = r.data_ptr(), v.data_ptr()
    else:
        device = torch.device('cuda', torch.cuda.current_device())
        ptrs = []
        for t in (r, v):
            p = ctypes.c_void_p()
            check(lib.grav_host_device_pointer(ctypes.c_void_p(t.data_ptr()), ctypes.byref(p)))
            ptrs.append(p.value)
        r_ptr, v_ptr = ptrs
    st = stream if stream is not None else torch.cuda.current_stream(device)
    h = ctypes.c_void_p(st.cuda_stream)
    scratch = []
    for part in parts:
        s = part.struct(G)
        nbytes = int(lib.grav_scenario_scratch_bytes(ctypes.byref(s), part.n))
        if nbytes < 0:
            check(nbytes)
        buf = None
        if nbytes > 0:
            with torch.cuda.stream(st):
                buf = torch.empty(nbytes // 8, dtype=torch.float64, device=device)
            scratch.append(buf)
        check(lib.grav_scenario_generate(
            ctypes.byref(s), ctypes.c_void_p(r_ptr + 32 * part.offset),
            ctypes.c_void_p(v_ptr + 32 * part.offset), part.n,
            ctypes.c_void_p(buf.data_ptr() if buf is not None else None), h))
    # scratch tensors were allocated on `st`: the caching allocator reuses them only
    # after the work queued on that stream
    del scratch
