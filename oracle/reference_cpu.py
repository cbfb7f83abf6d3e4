"""The reference's own CPU kernels timed on this host, through their plugin classes, on
bounded samples of the single-universe workload -- the reference arm of bench.py
(``--impl reference``).  Test/measurement infrastructure: nothing in the package uses it.

The kernels are the reference's sources staged in baseline/_ref (oracle/build.py,
stage_reference) and compiled on this host (build_reference):
  c1a  gravitation/kernel/c1a.py + _lib1_/lib.c: C, one thread, every unique pair once
       (step_stage1, _lib1_/lib.c:52-126) with the plugin's Python copy loops
       (c1a.py:84-96); sample: its full step_stage1 on the first k bodies of the workload
  cy4  gravitation/kernel/cy4: Cython + OpenMP prange (cy4/core.pyx:120-170) through its
       plugin (cy4/wrapper.py:43-115), `threads` workers; sample: step_stage1 on the
       first k bodies
  np2  gravitation/kernel/np2.py: numpy row loop (np2.py:89-108); sample: update_pair on
       rows 0 .. k-1 of the full universe (the calls its step_stage1 makes first)
c4a/c4b (_lib4_, x86 SSE) do not compile with GCC 13 and not at all on Arm.  Every
kernel runs in a process of its own (OpenMP thread pools of different kernels would
compete).  Interactions are counted as 2 per unique pair, the unit of bench.py.

    python -m oracle.reference_cpu --one KIND N SEED SECONDS THREADS [REPEATS]
"""

import importlib
import json
import os
import subprocess
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
KINDS = ('c1a', 'cy4', 'np2')


def _import_reference():
    from oracle import build as obuild
    if not obuild.staged_reference():
        raise ImportError('the reference package is not staged in baseline/_ref')
    if obuild.BASELINE_REF not in sys.path:
        sys.path.insert(0, obuild.BASELINE_REF)
    return importlib.import_module('gravitation.kernel._base_')


def _universe(kind, r, v, m, threads):
    mod = importlib.import_module('gravitation.kernel.%s' % (
        'cy4.wrapper' if kind == 'cy4' else kind))
    u = mod.universe(threads=threads)  # defaults: T, G, scale 1, dtype float32
    for i in range(len(m)):
        u.add_object(name='b', r=[float(x) for x in r[i]], v=[float(x) for x in v[i]],
                     m=float(m[i]))
    u.start()
    return u


def measure(kind, n, seed, seconds, threads, repeats=3):
    """Interactions/s of one kernel on a sample of about `seconds` of work: the sample
    size is found first, then `repeats` timed runs of it (values: each run's rate;
    value: their mean)."""
    _import_reference()
    sys.path.insert(0, ROOT)
    from gravitation_gb300.scenarios import uniform_cube
    r, v, m = uniform_cube(n, seed=seed)
    if kind == 'np2':
        u = _universe('np2', r, v, m, 1)
        rows = 8
        while True:
            t0 = time.perf_counter()
            for i in range(rows):
                u.update_pair(i, n - 1 - i)
            dt = time.perf_counter() - t0
            if dt >= seconds / 4 or rows >= n - 1:
                break
            rows = min(n - 1, rows * 4)
        pairs = sum(n - 1 - i for i in range(rows))
        times = []
        for _ in range(repeats):
            t0 = time.perf_counter()
            for i in range(rows):
                u.update_pair(i, n - 1 - i)
            times.append(time.perf_counter() - t0)
        sample = 'np2 update_pair on rows 0..%d of the N=%d universe' % (rows - 1, n)
        return _result(pairs, times, 1, sample)
    k = 512
    while True:
        u = _universe(kind, r[:k], v[:k], m[:k], threads)
        u.step_stage1()
        t0 = time.perf_counter()
        u.step_stage1()
        dt = time.perf_counter() - t0
        if dt >= seconds / 4 or k >= n:
            break
        k = min(n, k * 2)
    times = []
    for _ in range(repeats):
        t0 = time.perf_counter()
        u.step_stage1()
        times.append(time.perf_counter() - t0)
    pairs = k * (k - 1) // 2
    sample = '%s step_stage1 on the first %d bodies of the N=%d workload' % (kind, k, n)
    return _result(pairs, times, threads if kind == 'cy4' else 1, sample)


def _result(pairs, times, threads, sample):
    rates = [2.0 * pairs / t for t in times]
    return {'value': sum(rates) / len(rates), 'best': max(rates), 'values': rates,
            'threads': threads, 'sample': sample, 'seconds_per_run': sum(times) / len(times)}


def available():
    """The reference kernels whose compiled parts exist on this host."""
    from oracle import build as obuild
    if not obuild.staged_reference():
        return []
    import sysconfig
    out = ['np2']
    if os.path.isfile(os.path.join(obuild.STAGED_KERNEL, '_lib1_', 'lib.so')):
        out.insert(0, 'c1a')
    if os.path.isfile(os.path.join(obuild.STAGED_KERNEL, 'cy4',
                                   'core' + sysconfig.get_config_var('EXT_SUFFIX'))):
        out.insert(1, 'cy4')
    return out


def run(kind, n, seed, seconds, threads, repeats=3, timeout=900):
    """measure() in a subprocess of its own; returns its dict (or {'error': ...})."""
    env = dict(os.environ)
    env['OMP_NUM_THREADS'] = str(threads)   # set before the process starts
    p = subprocess.run([sys.executable, '-m', 'oracle.reference_cpu', '--one', kind, str(n),
                        str(seed), str(seconds), str(threads), str(repeats)], cwd=ROOT, env=env,
                       capture_output=True, text=True, timeout=timeout)
    if p.returncode != 0:
        return {'error': (p.stderr or p.stdout).strip().splitlines()[-1:]}
    return json.loads(p.stdout.strip().splitlines()[-1])


def main():
    if len(sys.argv) > 1 and sys.argv[1] == '--one':
        kind, n, seed, seconds, threads = sys.argv[2], int(sys.argv[3]), int(sys.argv[4]), \
            float(sys.argv[5]), int(sys.argv[6])
        repeats = int(sys.argv[7]) if len(sys.argv) > 7 else 3
        print(json.dumps(measure(kind, n, seed, seconds, threads, repeats)))
        return 0
    n = int(sys.argv[1]) if len(sys.argv) > 1 else 65536
    out = {}
    for kind in available():
        out[kind] = run(kind, n, 0, 2.0, os.cpu_count() or 1)
    print(json.dumps(out))
    return 0


if __name__ == '__main__':
    sys.exit(main())
