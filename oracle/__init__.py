"""CPU oracle for the all-pairs n-body step -- TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py`` (its ``cpu_baseline``
leg and its ``--impl reference`` arm) may import this package, and only as the
checker or as the timed CPU baseline.  The product package ``gravitation_gb300``
never imports it and has no CPU fallback.

Parity pin: the FP64 oracle is checked against golden vectors produced by the
reference's own kernels (np1, np2 and py1, run from the reference tree by
``tests/golden/make_golden.py``) in ``tests/test_oracle.py``.

Contents
  accel_fp64          FP64 all-pairs accelerations (C, compensated sums)
  accel_fp64_numpy    same law in vectorised numpy (cross-check of the C code)
  accel_np1_order     restatement of np1's row loop (np1.py:81-108), any dtype
  accel_py1           restatement of py1 (py1.py:57-69), pure Python, tiny N
  stage2_fp64         base-class stage 2 (_base_.py:58-62)
  rollout_fp64        stage 1 (FP64) + stage 2 (FP64) for k steps
  energy_fp64         kinetic, potential and momentum in FP64
  vjp_fp64            discrete adjoint of one stage 1 (J_A^T u and dA/dm terms)
  adjoint_rollout_fp64  discrete adjoint of a checkpointed FP64 rollout (gradients of a
                      final-state loss with respect to r0, v0 and m)
  port_stage1         portable restatement of the reference's fastest CPU kernel
                      design (c4a/cy4), FP32, OpenMP -- the CPU baseline
"""

import ctypes
import math
import os

import numpy as np

from . import build as _build

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None
_PORT = None

_dp = ctypes.POINTER(ctypes.c_double)
_fp = ctypes.POINTER(ctypes.c_float)
_i64p = ctypes.POINTER(ctypes.c_int64)


def _ptr(a, kind):
    return a.ctypes.data_as(kind)


def lib():
    """The FP64 oracle library (built on first use)."""
    global _LIB
    if _LIB is None:
        path = _build.build_oracle()
        L = ctypes.CDLL(path)
        L.orc_accel_fp64.argtypes = [_dp, _dp, ctypes.c_double, ctypes.c_int64, _i64p,
                                     ctypes.c_int64, _dp, ctypes.c_int, ctypes.c_int]
        L.orc_accel_fp64.restype = None
        L.orc_stage2_fp64.argtypes = [_dp, _dp, _dp, ctypes.c_double, ctypes.c_int64]
        L.orc_stage2_fp64.restype = None
        L.orc_energy_fp64.argtypes = [_dp, _dp, _dp, ctypes.c_double, ctypes.c_int64,
                                      _dp, ctypes.c_int]
        L.orc_energy_fp64.restype = None
        L.orc_vjp_fp64.argtypes = [_dp, _dp, ctypes.c_double, _dp, ctypes.c_int64,
                                   _dp, _dp, ctypes.c_int]
        L.orc_vjp_fp64.restype = None
        _u64p = ctypes.POINTER(ctypes.c_uint64)
        L.orc_philox4x64_10.argtypes = [_u64p, _u64p, _u64p]
        L.orc_philox4x64_10.restype = None
        L.orc_scenario.argtypes = [ctypes.c_int, ctypes.c_uint64, ctypes.c_uint64,
                                   ctypes.c_double, _dp, ctypes.c_int64, _dp, _dp]
        L.orc_scenario.restype = ctypes.c_int
        _LIB = L
    return _LIB


# ---------------------------------------------------------------------------------
# seeded scenarios (restatement of the device generator, oracle/scenario.c)
# ---------------------------------------------------------------------------------

SCENARIO_KINDS = {'uniform_cube': 1, 'plummer': 2, 'galaxy': 3}


def philox4x64_10(ctr, key):
    """Philox4x64-10 block for a 4-word counter and a 2-word key (uint64 array [4])."""
    c = np.ascontiguousarray(ctr, dtype=np.uint64)
    k = np.ascontiguousarray(key, dtype=np.uint64)
    out = np.zeros(4, dtype=np.uint64)
    u64 = ctypes.POINTER(ctypes.c_uint64)
    lib().orc_philox4x64_10(_ptr(c, u64), _ptr(k, u64), _ptr(out, u64))
    return out


def scenario(kind, n, seed, stream, G, params):
    """(r, v): n x 4 float64 arrays (x, y, z, G*m) / (vx, vy, vz, 0) of a scenario."""
    p = np.zeros(10)
    p[:len(params)] = params
    r = np.zeros((n, 4))
    v = np.zeros((n, 4))
    k = SCENARIO_KINDS[kind] if isinstance(kind, str) else int(kind)
    if lib().orc_scenario(k, int(seed), int(stream), float(G), _ptr(p, _dp), int(n),
                          _ptr(r, _dp), _ptr(v, _dp)) != 0:
        raise ValueError('unknown scenario kind %r' % (kind,))
    return r, v


def load_port(path):
    """ctypes binding of a build of oracle/ref_port.c."""
    L = ctypes.CDLL(path)
    L.port_stage1_rows.argtypes = [_fp, _fp, _fp, _fp, ctypes.c_float, ctypes.c_int64,
                                   ctypes.c_int64, ctypes.c_int64, _fp, _fp, _fp, _fp,
                                   ctypes.c_int]
    L.port_stage1_rows.restype = None
    L.port_segments.argtypes = [ctypes.c_int64, ctypes.c_int64, ctypes.c_int64,
                                ctypes.c_int, _i64p]
    L.port_segments.restype = None
    L.port_stage2.argtypes = [_fp] * 9 + [ctypes.c_float, ctypes.c_int64]
    L.port_stage2.restype = None
    return L


def port_lib():
    """The portable CPU-baseline library (built on first use)."""
    global _PORT
    if _PORT is None:
        _PORT = load_port(_build.build_port())
    return _PORT


def default_threads():
    try:
        return max(1, len(os.sched_getaffinity(0)))
    except AttributeError:
        return max(1, os.cpu_count() or 1)


# ---------------------------------------------------------------------------------
# FP64 oracle
# ---------------------------------------------------------------------------------

def accel_fp64(r, m, G, rows=None, coincident=False, threads=None):
    """FP64 accelerations a_i = sum_{j!=i} G m_j (r_j - r_i)/|r_j - r_i|^3.

    Follows np1.py:81-95 (rel = r_i - r_j, inv = 1/sqrt(s), f = G/s) with
    compensated summation.  ``rows`` selects the bodies i (default: all).
    ``coincident=True`` skips distinct bodies at zero distance instead of producing
    inf/nan as the reference does.
    """
    r = np.ascontiguousarray(r, dtype=np.float64).reshape(-1, 3)
    m = np.ascontiguousarray(m, dtype=np.float64).reshape(-1)
    n = r.shape[0]
    if rows is None:
        rows_arr = None
        nrows = n
    else:
        rows_arr = np.ascontiguousarray(rows, dtype=np.int64)
        nrows = rows_arr.shape[0]
    out = np.zeros((nrows, 3), dtype=np.float64)
    lib().orc_accel_fp64(_ptr(r, _dp), _ptr(m, _dp), float(G), n,
                         None if rows_arr is None else _ptr(rows_arr, _i64p), nrows,
                         _ptr(out, _dp), int(bool(coincident)),
                         int(threads or default_threads()))
    return out


def accel_fp64_numpy(r, m, G, rows=None, chunk=256):
    """Vectorised numpy FP64 all-pairs (plain summation), used to cross-check the C."""
    r = np.asarray(r, dtype=np.float64).reshape(-1, 3)
    m = np.asarray(m, dtype=np.float64).reshape(-1)
    idx = np.arange(r.shape[0]) if rows is None else np.asarray(rows)
    out = np.zeros((len(idx), 3))
    for s in range(0, len(idx), chunk):
        ii = idx[s:s + chunk]
        rel = r[ii][:, None, :] - r[None, :, :]
        sq = (rel * rel).sum(axis=2)
        sq[np.arange(len(ii)), ii] = 1.0
        inv = 1.0 / np.sqrt(sq)
        f = G / sq
        w = f * m[None, :] * inv
        w[np.arange(len(ii)), ii] = 0.0
        out[s:s + chunk] = -(rel * w[:, :, None]).sum(axis=1)
    return out


def accel_np1_order(r, m, G, dtype='float32'):
    """Restatement of the np1 stage 1 (np1.py:81-108) in the given dtype.

    Row loop over i with the symmetric update of rows i+1..N-1, the same ufunc
    sequence and the same temporaries' dtype, so that results agree with the
    reference's np1 to rounding of the same operations.
    """
    dt = np.dtype(dtype)
    R = np.asarray(r, dtype=np.float64).reshape(-1, 3).astype(dt)
    M = np.asarray(m, dtype=np.float64).astype(dt)
    n = R.shape[0]
    A = np.zeros((n, 3), dtype=dt)
    Gd = G
    for i in range(n - 1):
        k = n - 1 - i
        rel = np.subtract(R[i, :], R[i + 1:, :])
        sq = np.add.reduce(np.multiply(rel, rel), axis=1)
        dinv = np.sqrt(sq)
        dinv = np.divide(1.0, dinv, out=dinv)
        rel = np.multiply(rel, dinv.reshape(k, 1), out=rel)
        af = np.divide(Gd, sq)
        a1 = np.multiply(af, M[i + 1:])
        a2 = np.multiply(af, M[i])
        a1v = np.add.reduce(np.multiply(rel, a1.reshape(k, 1)), axis=0)
        np.subtract(A[i, :], a1v, out=A[i, :])
        np.add(A[i + 1:, :], np.multiply(rel, a2.reshape(k, 1)), out=A[i + 1:, :])
    return A


def accel_py1(r, m, G):
    """Restatement of py1 (py1.py:57-69): unique pairs in pure Python, FP64."""
    n = len(r)
    a = [[0.0, 0.0, 0.0] for _ in range(n)]
    for i in range(n - 1):
        for j in range(i + 1, n):
            rel = [r[i][k] - r[j][k] for k in range(3)]
            dist = math.sqrt(sum(x ** 2 for x in rel))
            rel = [x / dist for x in rel]
            a1 = G * m[j] / dist ** 2
            a2 = G * m[i] / dist ** 2
            a[i] = [aa - x * a1 for x, aa in zip(rel, a[i])]
            a[j] = [aa + x * a2 for x, aa in zip(rel, a[j])]
    return a


def stage2_fp64(r, v, a, T):
    """Base-class stage 2 (_base_.py:58-62) in FP64: v = a*T + v; r = v*T + r."""
    r = np.ascontiguousarray(r, dtype=np.float64).copy()
    v = np.ascontiguousarray(v, dtype=np.float64).copy()
    a = np.ascontiguousarray(a, dtype=np.float64)
    lib().orc_stage2_fp64(_ptr(r, _dp), _ptr(v, _dp), _ptr(a, _dp), float(T), r.size)
    return r, v


def rollout_fp64(r, v, m, G, T, steps, threads=None, record=False):
    """``steps`` FP64 steps (stage 1 + stage 2).  Returns (r, v[, list of a_k])."""
    r = np.array(r, dtype=np.float64).reshape(-1, 3)
    v = np.array(v, dtype=np.float64).reshape(-1, 3)
    acc = []
    for _ in range(steps):
        a = accel_fp64(r, m, G, threads=threads)
        if record:
            acc.append(a)
        r, v = stage2_fp64(r, v, a, T)
    return (r, v, acc) if record else (r, v)


def energy_fp64(r, v, m, G, threads=None):
    """(kinetic, potential, momentum[3]) in FP64 with compensated sums."""
    r = np.ascontiguousarray(r, dtype=np.float64).reshape(-1, 3)
    v = np.ascontiguousarray(v, dtype=np.float64).reshape(-1, 3)
    m = np.ascontiguousarray(m, dtype=np.float64)
    out = np.zeros(5)
    lib().orc_energy_fp64(_ptr(r, _dp), _ptr(v, _dp), _ptr(m, _dp), float(G), r.shape[0],
                          _ptr(out, _dp), int(threads or default_threads()))
    return out[0], out[1], out[2:5].copy()


def vjp_fp64(r, m, G, u, threads=None):
    """(h, gmk) of one stage 1: h = J_A(r)^T u,  gmk_k = sum_j u_j.(r_j-r_k)/|r_j-r_k|^3."""
    r = np.ascontiguousarray(r, dtype=np.float64).reshape(-1, 3)
    m = np.ascontiguousarray(m, dtype=np.float64)
    u = np.ascontiguousarray(u, dtype=np.float64).reshape(-1, 3)
    n = r.shape[0]
    h = np.zeros((n, 3))
    g = np.zeros(n)
    lib().orc_vjp_fp64(_ptr(r, _dp), _ptr(m, _dp), float(G), _ptr(u, _dp), n,
                       _ptr(h, _dp), _ptr(g, _dp), int(threads or default_threads()))
    return h, g


def adjoint_rollout_fp64(r0, v0, m, G, T, steps, g_rK, g_vK, every=32, threads=None):
    """Discrete adjoint of ``steps`` FP64 symplectic-Euler steps (stage 1 all pairs,
    stage 2 of _base_.py:58-62), reverse sweep with checkpoints every ``every`` steps
    and the states of a segment recomputed from its checkpoint.  Per step k, with
    u = gv_{k+1} + T gr_{k+1} and (h, g) = vjp_fp64(r_k, m, G, u):
        gr_k = gr_{k+1} + T h,   gv_k = u,   dL/d(G m) += -T g.
    Returns (dL/dr0, dL/dv0, dL/dm) for the incoming final-state gradients g_rK, g_vK."""
    r = np.array(r0, dtype=np.float64).reshape(-1, 3)
    v = np.array(v0, dtype=np.float64).reshape(-1, 3)
    m = np.ascontiguousarray(m, dtype=np.float64)
    starts = list(range(0, steps, every))
    ckpt = []
    for s0 in starts:
        ckpt.append((r.copy(), v.copy()))
        r, v = rollout_fp64(r, v, m, G, T, min(every, steps - s0), threads=threads)
    gr = np.array(g_rK, dtype=np.float64).reshape(-1, 3)
    gv = np.array(g_vK, dtype=np.float64).reshape(-1, 3)
    g_gm = np.zeros(len(m))
    for s0, (rc, vc) in zip(reversed(starts), reversed(ckpt)):
        k = min(every, steps - s0)
        states = [rc]
        rr, vv = rc, vc
        for _ in range(k - 1):
            rr, vv = rollout_fp64(rr, vv, m, G, T, 1, threads=threads)
            states.append(rr)
        for rk in reversed(states):
            u = gv + T * gr
            h, g = vjp_fp64(rk, m, G, u, threads=threads)
            gr = gr + T * h
            gv = u
            g_gm -= T * g
    return gr, gv, G * g_gm


# ---------------------------------------------------------------------------------
# CPU baseline: portable restatement of the reference's fastest CPU kernel design
# ---------------------------------------------------------------------------------

class PortStage1:
    """FP32 SoA buffers + scratch for ``port_stage1_rows`` (c4a/cy4 design)."""

    def __init__(self, r, m, G, threads=None, lib=None):
        self.lib = lib  # another build of ref_port.c (load_port), default port_lib()
        r = np.asarray(r, dtype=np.float64).reshape(-1, 3)
        self.n = r.shape[0]
        self.threads = int(threads or default_threads())
        self.x = np.ascontiguousarray(r[:, 0], dtype=np.float32)
        self.y = np.ascontiguousarray(r[:, 1], dtype=np.float32)
        self.z = np.ascontiguousarray(r[:, 2], dtype=np.float32)
        self.m = np.ascontiguousarray(m, dtype=np.float32)
        self.G = float(G)
        self.a = np.zeros((3, self.n), dtype=np.float32)
        self.work = np.zeros(self.threads * 3 * self.n, dtype=np.float32)

    def run(self, row0=0, row1=None):
        row1 = self.n if row1 is None else row1
        (self.lib or port_lib()).port_stage1_rows(
            _ptr(self.x, _fp), _ptr(self.y, _fp), _ptr(self.z, _fp), _ptr(self.m, _fp),
            self.G, self.n, int(row0), int(row1),
            _ptr(self.a[0], _fp), _ptr(self.a[1], _fp), _ptr(self.a[2], _fp),
            _ptr(self.work, _fp), self.threads)
        return self.a.T.copy()

    @staticmethod
    def pairs_in_rows(n, row0, row1):
        """Unique pairs (i<j) whose row i lies in [row0, row1)."""
        return sum(n - 1 - i for i in range(row0, row1))


def port_segments(n, threads, row0=0, row1=None):
    row1 = n if row1 is None else row1
    b = np.zeros(threads + 1, dtype=np.int64)
    port_lib().port_segments(n, row0, row1, threads, _ptr(b, _i64p))
    return b


# ---------------------------------------------------------------------------------
# error metrics
# ---------------------------------------------------------------------------------

def rel_err_per_body(a, ref):
    """|a_i - ref_i| / |ref_i| per body (Euclidean norms)."""
    a = np.asarray(a, dtype=np.float64).reshape(-1, 3)
    ref = np.asarray(ref, dtype=np.float64).reshape(-1, 3)
    num = np.linalg.norm(a - ref, axis=1)
    den = np.linalg.norm(ref, axis=1)
    return num / np.where(den == 0, 1.0, den)
