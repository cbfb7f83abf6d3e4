"""Time the CPU baseline port (oracle/ref_port.c) against the reference's own CPU kernels
on this host, where the reference tree is present: the cy4 Cython/OpenMP kernel
(gravitation/kernel/cy4/core.pyx, the reference's fastest portable CPU kernel) and the
single-threaded c1a C kernel (gravitation/kernel/_lib1_/lib.c), both compiled from the
reference's sources by oracle/build.py.  Stage 1 only, FP32, uniform cube of N bodies
(seed 0), best of `runs` wall-clock runs each, every kernel in a process of its own (two
OpenMP thread pools in one process would spin against each other).  Prints one JSON line.

Test infrastructure: shows that the design of the timed CPU baseline (kind "port") is at
least as fast as the reference's own kernels when compiled alike, so that it is not a
weaker stand-in.

    python -m oracle.compare_reference_cpu [N] [threads]
"""

import ctypes
import importlib.util
import json
import os
import platform
import subprocess
import sys
import time
from array import array

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

import oracle  # noqa: E402
from oracle import build as obuild  # noqa: E402


def best(fn, runs):
    ts = []
    for _ in range(runs):
        t0 = time.perf_counter()
        fn()
        ts.append(time.perf_counter() - t0)
    return min(ts)


def row_segments(n, workers):
    """Contiguous row ranges [p0, p1) covering rows 0 .. n-2 (row i holds the pairs
    (i, j > i)), each with about 1/workers of the n(n-1)/2 pairs; the same split the
    reference's cy4 wrapper makes before launching its workers."""
    total = n * (n - 1) // 2
    target = total / workers
    p0, p1, start, acc = [], [], 0, 0
    for line in range(n - 1):
        acc += n - 1 - line
        if acc >= target and len(p0) < workers - 1:
            p0.append(start)
            p1.append(line + 1)
            start, acc = line + 1, 0
    p0.append(start)
    p1.append(n - 1)
    return p0, p1


def measure(kind, n, threads, runs=3):
    """Seconds per stage-1 call of one kernel (run in a process of its own)."""
    built = obuild.build_reference()
    from gravitation_gb300.scenarios import G_DEFAULT, uniform_cube
    r, _, m = uniform_cube(n, seed=0)
    G = G_DEFAULT
    out = {}
    if kind in ('port', 'port_refflags'):
        lib = None
        if kind == 'port_refflags':
            lib = oracle.load_port(obuild.build_port_reference_flags())
        port = oracle.PortStage1(r, m, G, threads=threads, lib=lib)
        port.run()
        out['s'] = best(port.run, runs)
        np.save(os.path.join(os.environ.get('TMPDIR', '/tmp'), 'cmp_port_%d.npy' % n), port.run())
    elif kind == 'cy4':
        path = built.get('cy4')
        if not path or path.startswith('unbuildable'):
            return {'unavailable': path}
        spec = importlib.util.spec_from_file_location('core', path)
        core = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(core)
        rx, ry, rz = (array('f', r[:, k].astype(np.float32).tolist()) for k in range(3))
        acc = [array('f', [0.0] * n) for _ in range(3)]
        amp = [array('f', [0.0] * (n * threads)) for _ in range(3)]
        mm = array('f', m.astype(np.float32).tolist())
        p0, p1 = row_segments(n, threads)
        i0, i1 = array('l', p0), array('l', p1)

        def cy4():
            core._step_stage1_(rx, ry, rz, *acc, *amp, mm, i0, i1, len(p0), n, float(G))
        cy4()
        out['s'] = best(cy4, runs)
        a_cy4 = np.stack([np.array(x) for x in acc], 1)
        ref = os.path.join(os.environ.get('TMPDIR', '/tmp'), 'cmp_port_%d.npy' % n)
        if os.path.exists(ref):
            out['max_rel_diff_vs_port'] = float(
                oracle.rel_err_per_body(np.load(ref), a_cy4).max())
    elif kind == 'c1a':
        path = built.get('lib1')
        if not path or path.startswith('unbuildable'):
            return {'unavailable': path}
        L = ctypes.CDLL(path)
        arr_t = ctypes.c_float * n

        class univ(ctypes.Structure):  # struct univ of _lib1_/lib.c
            _fields_ = [(f, ctypes.POINTER(arr_t)) for f in
                        ('X', 'Y', 'Z', 'AX', 'AY', 'AZ', 'M')] + \
                [('G', ctypes.c_float), ('N', ctypes.c_long)]
        u = univ()
        bufs = {f: arr_t() for f in ('X', 'Y', 'Z', 'AX', 'AY', 'AZ', 'M')}
        for f, b in bufs.items():
            setattr(u, f, ctypes.pointer(b))
        for k, f in enumerate(('X', 'Y', 'Z')):
            ctypes.memmove(bufs[f], r[:, k].astype(np.float32).tobytes(), 4 * n)
        ctypes.memmove(bufs['M'], m.astype(np.float32).tobytes(), 4 * n)
        u.G = float(G)
        u.N = n
        L.step_stage1.argtypes = [ctypes.POINTER(univ)]
        out['s'] = best(lambda: L.step_stage1(ctypes.byref(u)), runs)
        out['threads'] = 1
    return out


def main():
    if len(sys.argv) > 1 and sys.argv[1] == '--one':
        kind, n, threads = sys.argv[2], int(sys.argv[3]), int(sys.argv[4])
        print(json.dumps(measure(kind, n, threads)))
        return 0
    n = int(sys.argv[1]) if len(sys.argv) > 1 else 16384
    threads = int(sys.argv[2]) if len(sys.argv) > 2 else (os.cpu_count() or 1)
    if not obuild.reference_present():
        print(json.dumps({'skipped': 'reference tree not present on this host'}))
        return 0
    obuild.build_reference()
    pairs = n * (n - 1) // 2
    out = {'n': n, 'threads': threads, 'host': platform.machine(), 'cpus': os.cpu_count(),
           'pairs': pairs, 'unit': 'interactions/s (2 per unique pair)'}
    # cy4 keeps one partial sum per (body, worker) interleaved in memory
    # (cy4/wrapper.py: mass_amp_array), so its workers write neighbouring floats and it
    # slows down as threads are added: it is timed on 1 and 2 threads only
    # port: the portable build that bench.py times; port_refflags: the same source with
    # the reference's flags on this host, like for like with c1a
    plan = [('port', 1), ('port', threads), ('port_refflags', 1), ('port_refflags', threads),
            ('c1a', 1), ('cy4', 1), ('cy4', min(2, threads))]
    for kind, t in plan:
        p = subprocess.run([sys.executable, '-m', 'oracle.compare_reference_cpu', '--one', kind,
                            str(n), str(t)], cwd=os.path.dirname(HERE),
                           capture_output=True, text=True, check=True)
        res = json.loads(p.stdout.strip().splitlines()[-1])
        if 's' in res:
            res['value'] = 2 * pairs / res['s']
        out['%s_%dt' % (kind, t)] = res
    print(json.dumps(out))
    return 0


if __name__ == '__main__':
    sys.exit(main())
