"""The reference's own command-line front end driving the gb1 kernel: its `benchmark`
command (cli/benchmark.py:164-205, one `worker` subprocess per size, lib/proc.py:76-104)
over its galaxy scenario, then its `analyze` command (cli/analyze.py:40-116) on the log.

The reference package is the staged copy in baseline/_ref (oracle/build.py,
stage_reference); a temporary copy of it gets the gb1 package in its kernel directory,
where the reference's loader discovers kernels (lib/load.py:44-66).  Imports that neither
host has are served by oracle/standins (h5py, psutil, asciiplotlib, plotly); click comes
from the local wheelhouse into baseline/_ref.  Nothing of the reference is changed.
Test infrastructure: the GPU test and the front-end summary use it.

    python -m oracle.frontend B_MIN B_MAX OUT_DIR [MIN_ITERATIONS MIN_TOTAL_RUNTIME]

writes OUT_DIR/benchmark.log (the workers' log) and OUT_DIR/benchmark.json (analyze's
output) and prints a one-line summary.
"""

import json
import os
import shutil
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
GB1 = os.path.join(ROOT, 'gravitation_gb300', 'kernel', 'gb1')
STANDINS = os.path.join(HERE, 'standins')


def available():
    """(True, '') when the staged reference and click are there, else (False, why)."""
    from oracle import build as obuild
    if not obuild.staged_reference():
        return False, 'the reference package is not staged in baseline/_ref'
    if not os.path.isdir(os.path.join(obuild.BASELINE_REF, 'click')):
        return False, 'click is not installed in baseline/_ref'
    return True, ''


def prepare(workdir):
    """Copy the staged reference package into workdir/pkg with gb1 among its kernels;
    returns the environment for the front end's processes."""
    from oracle import build as obuild
    pkg = os.path.join(os.path.abspath(workdir), 'pkg')
    shutil.rmtree(pkg, ignore_errors=True)
    shutil.copytree(os.path.join(obuild.BASELINE_REF, 'gravitation'),
                    os.path.join(pkg, 'gravitation'),
                    ignore=shutil.ignore_patterns('__pycache__', '*.so'))
    shutil.copytree(GB1, os.path.join(pkg, 'gravitation', 'kernel', 'gb1'),
                    ignore=shutil.ignore_patterns('__pycache__'))
    env = dict(os.environ)
    env['PYTHONPATH'] = os.pathsep.join([pkg, STANDINS, ROOT, obuild.BASELINE_REF] + (
        [env['PYTHONPATH']] if env.get('PYTHONPATH') else []))
    # the loader reads kernel metadata with ast.Str/Num (lib/load.py:113-144), deprecated
    # on Python 3.12; keep the warnings out of the workers' JSON logs
    env['PYTHONWARNINGS'] = 'ignore::DeprecationWarning'
    return env


def cli(env, args, timeout, cwd):
    cmd = [sys.executable, '-c', 'from gravitation.cli import cli; cli()'] + list(args)
    return subprocess.run(cmd, env=env, cwd=cwd, capture_output=True, text=True,
                          timeout=timeout)


def run(b_min, b_max, outdir, min_iterations=10, min_total_runtime=1, timeout=3600):
    """gravitation benchmark -k gb1 -b b_min b_max, then gravitation analyze on its log
    (both written to outdir; the package copy lives in a temporary directory).
    Returns (analyze's data as a list of dicts, log path, benchmark process)."""
    outdir = os.path.abspath(outdir)
    os.makedirs(outdir, exist_ok=True)
    workdir = tempfile.mkdtemp(prefix='gravitation_frontend_')
    env = prepare(workdir)
    log = os.path.join(outdir, 'benchmark.log')
    out = os.path.join(outdir, 'benchmark.json')
    b = cli(env, ['benchmark', '--kernel', 'gb1', '--n_body_power_boundaries', str(b_min),
                  str(b_max), '--logfile', log, '--data_out_file',
                  os.path.join(outdir, 'data.h5'), '--interpreter', sys.executable,
                  '--min_iterations', str(min_iterations), '--min_total_runtime',
                  str(min_total_runtime), '--display', 'none', '--threads', '1'],
            timeout, workdir)
    if b.returncode != 0:
        raise RuntimeError('benchmark failed: %s' % (b.stderr or b.stdout)[-2000:])
    a = cli(env, ['analyze', '--logfile', log, '--data', out], 600, workdir)
    shutil.rmtree(workdir, ignore_errors=True)
    if a.returncode != 0:
        raise RuntimeError('analyze failed: %s' % (a.stderr or a.stdout)[-2000:])
    with open(out) as f:
        return json.load(f), log, b


def summary(data):
    """One row per worker run of the analyzed log: size, steps, best and mean step time."""
    rows = []
    for item in data:
        sim = item['meta']['simulation']
        rt = item['runtime']
        rows.append({'kernel': sim['kernel'], 'n': sim['size'], 'steps': len(rt),
                     'best_ns': min(rt), 'mean_ns': sum(rt) / len(rt),
                     'interactions_per_s_best': sim['size'] ** 2 / (min(rt) * 1e-9)})
    return rows


def main():
    b_min, b_max, workdir = int(sys.argv[1]), int(sys.argv[2]), sys.argv[3]
    it = int(sys.argv[4]) if len(sys.argv) > 4 else 10
    tt = int(sys.argv[5]) if len(sys.argv) > 5 else 1
    data, log, _ = run(b_min, b_max, workdir, it, tt)
    print(json.dumps({'log': log, 'runs': summary(data)}))
    return 0


if __name__ == '__main__':
    sys.path.insert(0, ROOT)
    sys.exit(main())
