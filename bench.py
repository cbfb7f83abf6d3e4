#!/usr/bin/env python
"""Benchmark of the GB300 all-pairs n-body step (prints one JSON line on rank 0).

Workload (default): one universe of N = 65536 bodies, positions U[-1000,1000]^3,
velocities N(0,1), masses U[1,100] (seed 0), G = 6.6740831e-11, T = 1e3 -- FP32
pairwise stage 1 over unique pairs with compensated sums, near pairs from
double-single separations, and FP64 stage 2 ("fp32un", the plugin's float32 default at
this size; --mode picks another).  Synthetic data: the reference has no dataset, its
own scenarios are generated too.

  accuracy   every body's acceleration in the timed mode against the GPU's FP64 mode on
             the same FP64 state (max and tail of |a - a64| / |a64| over all N bodies);
             the GPU tests pin the FP64 mode to the CPU FP64 oracle at 1e-12
  precision  the Plummer-pair stress (N = 16384, 1000 steps): force errors over every
             body at the first and last step and energy / momentum drift, per mode
  sweep      the step over N = 2^4 .. 2^17 in the plugin's float32 default at each size,
             with the CPU baseline beside every size

  value      pair interactions per second (N^2 per step), device-timed steps with the
             state resident in HBM; L2 flushed (256 MiB write) between timed steps
  e2e        the same metric through the reference-facing plugin (gb1.universe.step()
             with host_sync='full'): the FP64 r, v live in pinned host memory (the
             point masses' pm._r / pm._v) and cross the CPU-GPU link every step,
             wall-clock timed; the upload/download copy path is timed beside it
  roofline   stage-1 kernel: 20 FLOP per interaction / kernel time, against the FP32
             FMA peak measured live by grav_fp32_peak_probe (SMs x 128 x 2 x clock)
  cpu_baseline  the reference's fastest CPU design (portable restatement in
             oracle/ref_port.c: unique pairs, OpenMP, private accumulators) on the
             host cores, on a bounded sample of the same workload

--impl reference times the reference's own CPU kernels (c1a, cy4, np2, compiled on this
host from its sources staged in baseline/_ref) and reports the fastest, with the port
beside it (rank 0; other ranks exit).
Multi-GPU: the path runs one universe per GPU (replicas only, no collective);
value = sum over ranks of interactions / the slowest rank's time.
"""

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = ('pair-interactions/s/GPU at N=65536 and fwd+adjoint steps/s at ≤1e-5 FP64 err')
UNIT = 'interactions/s'
FLOP_PER_INTERACTION = 20
STAGE1_KERNEL = {'fp32': 'stage1_f32_kernel<FP32>', 'fp32c': 'stage1_f32_kernel<FP32C>',
                 'fp32n': 'stage1_f32_kernel<FP32N>', 'fp64': 'stage1_f64_kernel',
                 'fp32u': 'stage1_sym_kernel<SYM_PLAIN>', 'fp32cu': 'stage1_sym_kernel<SYM_DS>',
                 'fp32un': 'stage1_sym_kernel<SYM_NEAR>'}
MODES = ('fp32', 'fp32u', 'fp32n', 'fp32un', 'fp32c', 'fp32cu', 'fp64')
L2_FLUSH_BYTES = 256 << 20


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=200)
    ap.add_argument('--warmup', type=int, default=3)
    ap.add_argument('--impl', choices=('ours', 'reference'), default='ours')
    ap.add_argument('--n', type=int, default=65536)
    ap.add_argument('--mode', default='fp32un', choices=MODES)
    ap.add_argument('--cpu-seconds', type=float, default=4.0,
                    help='target seconds per CPU-baseline sample run (3 runs)')
    ap.add_argument('--no-cpu', action='store_true')
    ap.add_argument('--no-e2e', action='store_true')
    ap.add_argument('--no-batched', action='store_true')
    ap.add_argument('--no-adjoint', action='store_true')
    ap.add_argument('--no-precision', action='store_true')
    ap.add_argument('--no-sweep', action='store_true')
    ap.add_argument('--workload', default=None,
                    choices=('precision', 'sweep', 'adjoint', 'adjoint-check', 'scenario',
                             'frontend', 'batched'),
                    help='run one secondary workload instead of the headline step')
    ap.add_argument('--profile', action='store_true',
                    help='only set up the workload and run --steps stage-1 launches '
                         '(for ncu captures); prints nothing on success')
    ap.add_argument('--profile-all', action='store_true',
                    help='with --profile: also run steps, the energy diagnostic and adjoint '
                         'steps (for captures of those kernels)')
    ap.add_argument('--adjoint-n', type=int, default=4096,
                    help='bodies of the adjoint workload (1000 steps, checkpoint every 32)')
    ap.add_argument('--tile', default=None,
                    help='force the stage-1 tile as bpt,threads,jtile (default: autotuned)')
    a = ap.parse_args()
    a.warmup = max(a.warmup, 3)
    a.mode_given = a.mode if '--mode' in sys.argv else None
    return a


def measured_peaks():
    """The machine's measured HBM and tensor peaks (MEASURED_PEAKS.json at the repo root)."""
    try:
        with open(os.path.join(ROOT, 'MEASURED_PEAKS.json')) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


# ---- distributed plumbing ----------------------------------------------------------------

def dist_env():
    world = int(os.environ.get('WORLD_SIZE', '1'))
    rank = int(os.environ.get('RANK', '0'))
    local = int(os.environ.get('LOCAL_RANK', '0'))
    return world, rank, local


def dist_init(world, backend):
    import torch.distributed as dist
    if world > 1 and not dist.is_initialized():
        os.environ.setdefault('MASTER_ADDR', '127.0.0.1')
        dist.init_process_group(backend)
    return dist


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def allreduce_max(x, world, device):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ---- clocks ---------------------------------------------------------------------------------

class ClockSampler:
    """nvidia-smi sampling (every 100 ms) of SM clock, power and throttle reasons.
    Samples are time-stamped; the summary keeps those taken inside the window that
    mark()/unmark() bracket (the timed region), and falls back to every sample only
    when the window is shorter than the sampling period."""
    FIELDS = ('timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,'
              'clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,'
              'clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap')
    PERIOD_MS = 100

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None
        self.window = [None, None]

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix='.csv')
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ['nvidia-smi', '-i', str(self.index), '--query-gpu=' + self.FIELDS,
                 '--format=csv,noheader,nounits', '-lms', str(self.PERIOD_MS)],
                stdout=open(self.path, 'w'), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)

    def mark(self):
        self.window[0] = time.time()

    def unmark(self):
        self.window[1] = time.time()

    @staticmethod
    def _epoch(stamp):
        import datetime
        try:
            return datetime.datetime.strptime(stamp, '%Y/%m/%d %H:%M:%S.%f').timestamp()
        except ValueError:
            return None

    def stop(self):
        if self.proc is None:
            return {'sm_mhz': None, 'sm_max_mhz': None, 'reasons': ['nvidia-smi unavailable']}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = []
        names = ('hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap')
        with open(self.path) as f:
            for line in f:
                p = [x.strip() for x in line.split(',')]
                if len(p) < 10:
                    continue
                try:
                    vals = (float(p[2]), float(p[3]), float(p[4]))
                except ValueError:
                    continue
                active = {nm for nm, val in zip(names, p[6:10]) if val.lower() == 'active'}
                rows.append((self._epoch(p[0]), vals, active))
        os.unlink(self.path)
        t0, t1 = self.window
        inside = [x for x in rows if x[0] is not None and t0 is not None and t1 is not None
                  and t0 <= x[0] <= t1]
        scope = 'timed region'
        if not inside:
            inside, scope = rows, 'whole run (timed region shorter than the sampling period)'
        if not inside:
            return {'sm_mhz': None, 'sm_max_mhz': None, 'reasons': ['no samples']}
        sm = [x[1][0] for x in inside]
        reasons = set().union(*[x[2] for x in inside])
        return {'sm_mhz': statistics.median(sm), 'sm_mhz_min': min(sm),
                'sm_max_mhz': max(x[1][1] for x in inside),
                'power_w_max': max(x[1][2] for x in inside), 'samples': len(sm),
                'samples_scope': scope, 'period_ms': self.PERIOD_MS,
                'reasons': sorted(reasons)}


def workload_name(n, mode):
    """The headline workload, named the same by both arms."""
    from gravitation_gb300.scenarios import G_DEFAULT, T_DEFAULT
    return ('one universe, N=%d uniform cube seed 0, G=%.8g, T=%g, FP32 pair terms (%s on '
            'the GPU) + FP64 stage 2' % (n, G_DEFAULT, T_DEFAULT, mode))


# ---- CPU baseline (the reference's CPU design, restated portably) -------------------------

def cpu_model():
    """The host CPU's model name (lscpu), for the CPU-baseline record."""
    try:
        out = subprocess.run(['lscpu'], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.strip().lower().startswith('model name'):
                return line.split(':', 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    import platform
    return platform.processor() or platform.machine()


def cpu_baseline_run(n, seed, target_s, runs=3):
    """Time the unique-pair OpenMP stage 1 (oracle/ref_port.c) on rows [0, k) of the pair
    triangle of the workload, k sized for about target_s seconds; best of `runs`.
    Returns (interactions/s, threads, sample description)."""
    import oracle
    from gravitation_gb300.scenarios import G_DEFAULT, uniform_cube
    r, _, m = uniform_cube(n, seed=seed)
    port = oracle.PortStage1(r, m, G_DEFAULT)
    k0 = max(1, min(n, 256))
    port.run(0, k0)  # first call starts the OpenMP thread team
    t0 = time.perf_counter()
    port.run(0, k0)
    dt = time.perf_counter() - t0
    rate = oracle.PortStage1.pairs_in_rows(n, 0, k0) / max(dt, 1e-6)
    want = rate * target_s
    k = k0
    pairs = oracle.PortStage1.pairs_in_rows(n, 0, k)
    while k < n and pairs < want:
        step = max(1, min(n - k, int((want - pairs) / max(n - 1 - k, 1)) + 1))
        pairs += sum(n - 1 - i for i in range(k, k + step))
        k += step
    best = None
    for _ in range(runs):
        t0 = time.perf_counter()
        port.run(0, k)
        dt = time.perf_counter() - t0
        best = dt if best is None else min(best, dt)
    value = 2.0 * pairs / best
    sample = ('rows 0..%d of the unique-pair triangle of the N=%d workload (%d pairs = %d '
              'interactions), FP32, best of %d runs of %.2f s' % (k, n, pairs, 2 * pairs, runs, best))
    return value, port.threads, sample


def run_reference(args):
    """The reference arm: the reference's own CPU kernels (c1a, cy4, np2; staged from its
    sources and compiled on this host, oracle/reference_cpu.py) each timed once on a
    bounded sample of the workload, then the fastest of them `--steps` times; the
    portable restatement of its c4a design (the cpu_baseline port of our arm) beside
    it.  Without the staged reference the port is the arm (kind "port")."""
    world, rank, _ = dist_env()
    if rank != 0:
        return 0
    from oracle import reference_cpu
    threads = os.cpu_count() or 1
    kernels = {}
    for kind in reference_cpu.available():
        kernels[kind] = reference_cpu.run(kind, args.n, 0, 1.5, threads if kind == 'cy4' else 1,
                                          repeats=1)
    ok = {k: v for k, v in kernels.items() if 'value' in v}
    # each step one bounded sample; keep the whole --steps run within ~2 minutes
    target = min(args.cpu_seconds, max(0.3, 120.0 / max(1, args.steps)))
    port_value, port_threads, port_sample = cpu_baseline_run(args.n, 0, target,
                                                              runs=max(1, min(args.steps, 5)))
    port = {'value': port_value, 'cores': port_threads, 'kind': 'port', 'sample': port_sample,
            'what': 'oracle/ref_port.c: portable restatement of the reference c4a design '
                    '(unique pairs, OpenMP row segments balanced by pair count, private '
                    'accumulators, serial reduction), all host threads'}
    if ok:
        fastest = max(ok, key=lambda k: ok[k]['value'])
        res = reference_cpu.run(fastest, args.n, 0, max(0.3, min(2.0, target)),
                                ok[fastest]['threads'], repeats=max(1, args.steps))
        if 'value' not in res:
            res = ok[fastest]
        value = res['value']
        cpu = {'value': value, 'unit': UNIT, 'cores': res['threads'], 'kind': 'reference',
               'kernel': fastest, 'cpu_model': cpu_model(), 'sample': res['sample'],
               'statistic': 'mean over %d samples' % len(res.get('values', [1]))}
        note = ('the reference\'s own CPU kernels, staged from its sources and compiled on '
                'this host, timed through their plugin classes; %s is the fastest; c4a/c4b '
                '(x86 SSE) do not compile here' % fastest)
    else:
        value = port_value
        cpu = dict(port, unit=UNIT, cpu_model=cpu_model())
        note = 'reference package not staged on this host: the port is the arm'
    line = {
        'impl': 'reference', 'metric': METRIC, 'value': value, 'unit': UNIT,
        'n_gpus': args.gpus, 'steps': args.steps, 'warmup': args.warmup,
        'ms_per_step': 1e3 * args.n * args.n / value,
        'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f32',
        'data': 'synthetic (seeded uniform cube)',
        'config': {'workload': workload_name(args.n, args.mode), 'n': args.n,
                   'mode': args.mode,
                   'parallelism': 'CPU, %d thread(s) on the host cores' % cpu['cores'],
                   'timed': 'stage 1 (FP32); the O(N) stage 2 is under 1e-4 of a CPU step '
                            'at this size and not timed'},
        'cpu_baseline': cpu,
        'reference_kernels': {k: {x: v.get(x) for x in ('value', 'threads', 'sample', 'error')
                                  if x in v} for k, v in kernels.items()},
        'port': port,
        'e2e': {'value': value, 'unit': UNIT, 'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': 0},
        'note': note,
    }
    print(json.dumps(line))
    return 0


# ---- ours --------------------------------------------------------------------------------------

def measure_fp32_peak(torch, lib, info, device):
    """FP32 FLOP/s of the FMA probe (best of 3 launches of ~20 ms)."""
    import ctypes
    blocks = info.sm_count * 8
    out = torch.empty(blocks * 256, dtype=torch.float32, device=device)
    s = torch.cuda.current_stream(device)
    h = ctypes.c_void_p(s.cuda_stream)
    iters = 2048
    lib.grav_fp32_peak_probe(out.data_ptr(), blocks, 64, h)
    best = None
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(s)
        lib.grav_fp32_peak_probe(out.data_ptr(), blocks, iters, h)
        e1.record(s)
        e1.synchronize()
        ms = e0.elapsed_time(e1)
        best = ms if best is None else min(best, ms)
    fmas = blocks * 256 * iters * 8 * 16
    return 2.0 * fmas / (best * 1e-3)


def all_body_errors(eng, r, m, G, device):
    """Per-body relative acceleration error of the engine's mode on the FP64 state, over
    every body, against the GPU's FP64 mode (FP64 all pairs, pinned to the CPU FP64
    oracle at 1e-12 by the GPU tests)."""
    from gravitation_gb300.workloads import fp64_forces, rel_err_per_body
    a = eng.forces().cpu().numpy()
    err = rel_err_per_body(a, fp64_forces(r, G * m, device))
    return {'max_rel_err_all_bodies_fp64_state': float(err.max()),
            'p999_rel_err': float(np.quantile(err, 0.999)),
            'median_rel_err': float(np.median(err)),
            'bodies_above_1e-5': int((err > 1e-5).sum()),
            'bodies': int(len(m)),
            'reference': 'GPU FP64 mode on the same FP64 state (every body)'}


def compact_precision(device):
    """Plummer-pair precision stress, shortened to 1000 steps: per mode the force error
    over every body at the first and last step against the GPU FP64 forces of that
    state, and the FP64 energy / momentum drift (every 100 steps)."""
    from gravitation_gb300.workloads import run_precision
    res = run_precision(n=16384, steps=1000, every=100, device=device)
    keys = ('accel_err_first', 'accel_err_last', 'bodies_above_1e-5_first',
            'bodies_above_1e-5_last', 'energy_drift_max', 'momentum_drift_max', 'wall_s',
            'final_pos_dev_vs_fp64_rel')
    out = {'workload': res['workload']}
    for mode, val in res.items():
        if isinstance(val, dict):
            out[mode] = {k: val[k] for k in keys if k in val}
    return out


def compact_sweep(tuner, cpu=True):
    """Single-universe step over N = 2^4 .. 2^17 in the plugin's float32 default at each
    size (up to 512 bodies the single-launch step), device-timed, with the CPU baseline
    (the port on the host cores) beside it."""
    from gravitation_gb300.workloads import run_sweep
    rows = run_sweep(sizes=[2 ** k for k in range(4, 18)], tuner=tuner)
    for row in rows:
        if cpu:
            cv, threads, _ = cpu_baseline_run(row['n'], 0, 0.3, runs=2)
            row['cpu_interactions_per_s'] = cv
            row['cpu_threads'] = threads
            row['gpu_over_cpu'] = row['interactions_per_s'] / cv
    return rows


def run_ours(args):
    import torch
    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    device = torch.device('cuda', local)
    dist_init(world, 'nccl')
    from gravitation_gb300 import _lib
    from gravitation_gb300.engine import Engine, device_info
    from gravitation_gb300.scenarios import G_DEFAULT, T_DEFAULT, uniform_cube
    from gravitation_gb300.tune import default_tuner

    lib = _lib.load()
    info = device_info(local)
    n = args.n
    r, v, m = uniform_cube(n, seed=0)
    gm = G_DEFAULT * m
    if args.tile:
        bpt, thr, jt = (int(x) for x in args.tile.split(','))
        eng = Engine([n], T_DEFAULT, mode=args.mode, tile=_lib.Tile(bpt, thr, jt, 0), device=local)
    else:
        eng = Engine([n], T_DEFAULT, mode=args.mode, tuner=default_tuner(), device=local)
    eng.set_state(r, v, gm)
    stream = torch.cuda.current_stream(device)
    if args.profile:
        # stage 1 alone, then (for the other kernels' captures) full steps, the FP64
        # energy diagnostic and backward adjoint steps, each --warmup + --steps times
        for _ in range(args.warmup + args.steps):
            eng.stage1()
        if args.profile_all:
            from gravitation_gb300.adjoint import AdjointEngine
            adj = AdjointEngine([n], T_DEFAULT, device=local)
            adj.set_state(eng.r[:n], eng.v[:n])
            adj.gr[:n, :3].normal_()
            for _ in range(args.warmup + args.steps):
                eng.step(1, write_a=True)
                eng.energy(G_DEFAULT)
                # the backward step with the forward's accelerations, then recomputing them
                adj.prepare()
                adj.step(a_in=eng.a)
                adj.prepare()
                adj.step()
            adj.raise_on_device_error()
        torch.cuda.synchronize()
        eng.raise_on_device_error()
        return 0
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=device)

    # accuracy of every body before timing, against the GPU FP64 mode
    accuracy = None
    if rank == 0:
        accuracy = all_body_errors(eng, r, m, G_DEFAULT, local)
        eng.set_state(r, v, gm)

    for _ in range(args.warmup):
        eng.step(1)
    torch.cuda.synchronize()
    eng.raise_on_device_error()

    clocks = ClockSampler(local)
    clocks.start()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
           for _ in range(args.steps)]
    barrier(world)
    torch.cuda.synchronize()
    clocks.mark()
    t_wall0 = time.perf_counter()
    for k in range(args.steps):
        flush.zero_()
        evs[k][0].record(stream)
        eng.step(1)
        evs[k][1].record(stream)
    torch.cuda.synchronize()
    barrier(world)
    t_wall = time.perf_counter() - t_wall0
    step_ms = [a.elapsed_time(b) for a, b in evs]
    eng.raise_on_device_error()

    # stage-1 kernel alone (the dominant kernel) for the roofline
    s1 = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    for k in range(args.steps):
        flush.zero_()
        s1[k][0].record(stream)
        eng.stage1()
        s1[k][1].record(stream)
    torch.cuda.synchronize()
    clocks.unmark()
    clk = clocks.stop()
    s1_ms = [a.elapsed_time(b) for a, b in s1]
    peak = measure_fp32_peak(torch, lib, info, device)

    total_ms = sum(step_ms)
    my_ms = total_ms / args.steps
    max_ms = allreduce_max(my_ms, world, device)
    value = world * n * n / (max_ms * 1e-3)

    e2e = None
    if not args.no_e2e:
        e2e = run_e2e(args, r, v, m, local)

    batched = None
    if not args.no_batched:
        from gravitation_gb300.workloads import run_batched
        batched = run_batched(steps=100, warmup=args.warmup, mode=args.mode,
                              tuner=default_tuner(), device=local)

    adjoint = None
    if not args.no_adjoint:
        from gravitation_gb300.workloads import run_adjoint
        adjoint = run_adjoint(tuner=default_tuner(), device=local)
        # forward + adjoint against forward beyond the specified size (fewer steps, same
        # checkpoint interval)
        adjoint['by_n'] = {}
        for n_adj, steps_adj in ((8192, 256), (16384, 128)):
            res = run_adjoint(n=n_adj, steps=steps_adj, tuner=default_tuner(), device=local)
            adjoint['by_n'][str(n_adj)] = {
                'steps': steps_adj,
                'ratio_fwd_plus_adjoint_over_fwd': res['ratio_fwd_plus_adjoint_over_fwd'],
                'backward_kernel': res['graphs']['backward_kernel'],
                'ratio_recomputed_accelerations': res['recomputed_accelerations'][
                    'ratio_fwd_plus_adjoint_over_fwd'],
                'fwd_adjoint_steps_per_s': res['fwd_adjoint_steps_per_s'],
                'forward_ms': res['forward_ms'], 'forward_adjoint_ms': res['forward_adjoint_ms'],
                'forward_mode': res['forward_mode']}

    precision = None
    if rank == 0 and not args.no_precision:
        precision = compact_precision(local)

    sweep = None
    if rank == 0 and not args.no_sweep:
        sweep = compact_sweep(default_tuner(), cpu=world == 1 and not args.no_cpu)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        cv, threads, sample = cpu_baseline_run(n, 0, args.cpu_seconds)
        cpu = {'value': cv, 'unit': UNIT, 'cores': threads, 'kind': 'port',
               'cpu_model': cpu_model(), 'sample': sample}

    if rank != 0:
        return 0
    s1_avg = statistics.mean(s1_ms)
    achieved = FLOP_PER_INTERACTION * n * n / (s1_avg * 1e-3)
    traffic = read_profile_traffic(args.mode)
    line = {
        'metric': METRIC, 'value': value, 'unit': UNIT, 'n_gpus': world,
        'steps': args.steps, 'warmup': args.warmup, 'ms_per_step': max_ms,
        'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None,
        'dtype': 'f32',
        'dtype_detail': ('FP32 pair terms into compensated FP32 (hi, lo) sums%s; FP64 state and '
                         'stage 2' % (', near pairs from double-single separations'
                                      if args.mode in ('fp32n', 'fp32un') else '')),
        'data': 'synthetic (seeded uniform cube; the reference ships no dataset)',
        'config': {'workload': workload_name(n, args.mode),
                   'n': n, 'mode': args.mode,
                   'tile': {'bpt': eng.tile.bpt, 'threads': eng.tile.threads,
                            'jtile': eng.tile.jtile, 'grid': eng.info.grid},
                   'l2': 'flushed between timed steps (256 MiB write)',
                   'parallelism': 'replicas' if world > 1 else 'single GPU'},
        'stage1_ms': s1_avg, 'step_ms_min': min(step_ms), 'wall_s_timed_region': t_wall,
        'roofline': {'bound': 'fp32', 'achieved': achieved / 1e12, 'peak': peak / 1e12,
                     'unit': 'TFLOP/s', 'frac': achieved / peak, 'traffic': traffic,
                     'kernel': STAGE1_KERNEL.get(args.mode, args.mode),
                     'flop_per_interaction': FLOP_PER_INTERACTION,
                     'peak_kind': 'measured live (grav_fp32_peak_probe FFMA kernel)',
                     'peak_formula_tflops_at_max_clock':
                         info.sm_count * 128 * 2 * (clk.get('sm_max_mhz') or 2070) * 1e6 / 1e12},
        'accuracy': accuracy,
        'clocks': clk,
        'gpu_launches': 2 * args.steps,
        'e2e': e2e,
        'cpu_baseline': cpu,
        'batched': batched,
        'adjoint': adjoint,
        'precision': precision,
        'sweep': sweep,
    }
    print(json.dumps(line))
    return 0


def _e2e_once(args, r, v, m, local, zero_copy):
    from gravitation_gb300.kernel import gb1
    n = len(m)
    u = gb1.universe(dtype='float32', precision=args.mode, host_sync='full', device=local,
                     zero_copy=zero_copy)
    for i in range(n):
        u.add_object(name='s', r=[float(r[i, 0]), float(r[i, 1]), float(r[i, 2])],
                     v=[float(v[i, 0]), float(v[i, 1]), float(v[i, 2])], m=float(m[i]))
    u.start()
    for _ in range(args.warmup):
        u.step()
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        u.step()
        times.append(time.perf_counter() - t0)
    used = u._gb_zero_copy
    u.stop()
    return times, used


def run_e2e(args, r, v, m, local):
    """gb1.universe.step() timed by wall clock with the FP64 state in pinned host memory
    (the mirror pm._r / pm._v are views of), crossing the CPU-GPU link every step.
    Default plugin path: prepare reads r and stage 2 reads and writes r, v in place in
    host memory (h2d 96 B/body, d2h 64 B/body + the 4-byte error flag).  The copy path
    (upload r, v; download r, v: 64 B/body each way) is timed beside it."""
    n = len(m)
    times, zc = _e2e_once(args, r, v, m, local, zero_copy=True)
    copies, _ = _e2e_once(args, r, v, m, local, zero_copy=False)
    mean, mean_c = statistics.mean(times), statistics.mean(copies)
    return {'value': n * n / mean, 'unit': UNIT,
            'h2d_bytes_per_step': (96 if zc else 64) * n,
            'd2h_bytes_per_step': 64 * n + 4, 'ms_per_step': 1e3 * mean,
            'ms_per_step_min': 1e3 * min(times),
            'path': 'gb1.universe.step(), host_sync=full, %s' % (
                'state in pinned host memory (zero_copy)' if zc else 'copies'),
            'copies_path': {'value': n * n / mean_c, 'ms_per_step': 1e3 * mean_c,
                            'h2d_bytes_per_step': 64 * n, 'd2h_bytes_per_step': 64 * n + 4}}


def read_profile_traffic(mode):
    """DRAM bytes per stage-1 launch from the committed ncu summary, if present."""
    p = os.path.join(ROOT, 'profiles', 'stage1_%s_n65536.md' % mode)
    try:
        with open(p) as f:
            for line in f:
                if line.startswith('dram_bytes_per_launch:'):
                    return float(line.split(':', 1)[1].split()[0])
    except OSError:
        pass
    return None


def run_workload(args):
    """Secondary workloads, one JSON line each: precision (Plummer pair, 3 modes,
    energy/momentum drift), sweep (N = 2^4 .. 2^17), adjoint (forward+adjoint), batched
    (256 universes vs the per-universe loop; with --profile the batched step alone),
    scenario generation and the reference's benchmark protocol through gb1 (frontend)."""
    import torch
    torch.cuda.set_device(0)
    from gravitation_gb300 import workloads
    from gravitation_gb300.tune import default_tuner
    if args.workload == 'precision':
        res = workloads.run_precision(n=args.n if args.n != 65536 else 16384,
                                      steps=args.steps)
    elif args.workload == 'sweep':
        mode = None if args.mode_given is None else args.mode
        res = {'sweep': workloads.run_sweep(mode=mode, tuner=default_tuner())}
        # the CPU baseline (the reference's design, restated portably) at every size
        for row in res['sweep']:
            cv, threads, sample = cpu_baseline_run(row['n'], 0, 0.5)
            row['cpu_baseline'] = {'value': cv, 'cores': threads, 'sample': sample}
            row['gpu_over_cpu'] = row['interactions_per_s'] / cv
        res['cpu_model'] = cpu_model()
    elif args.workload == 'adjoint':
        res = workloads.run_adjoint(n=args.adjoint_n, tuner=default_tuner())
    elif args.workload == 'adjoint-check':
        res = workloads.run_adjoint_check()
    elif args.workload == 'scenario':
        res = workloads.run_generate(hbm_gbs=measured_peaks().get('hbm_gbs'))
    elif args.workload == 'frontend':
        res = workloads.run_frontend()
    elif args.workload == 'batched':
        if args.profile:
            # the batched step alone, with a fixed tile (for ncu captures)
            from gravitation_gb300 import _lib
            from gravitation_gb300.engine import Engine
            from gravitation_gb300.scenarios import T_DEFAULT
            sizes, states = workloads.batch_universes(256, 1)
            bpt, thr, jt = (int(x) for x in (args.tile or '4,128,128').split(','))
            eng = Engine(sizes, T_DEFAULT, mode=args.mode, tile=_lib.Tile(bpt, thr, jt, 0))
            eng.set_state(np.concatenate([x[0] for x in states]),
                          np.concatenate([x[1] for x in states]),
                          workloads.G_DEFAULT * np.concatenate([x[2] for x in states]))
            eng.step(args.warmup + args.steps)
            torch.cuda.synchronize()
            eng.raise_on_device_error()
            return 0
        tile = None
        if args.tile:
            from gravitation_gb300 import _lib
            tile = _lib.Tile(*(int(x) for x in args.tile.split(',')), 0)
        res = workloads.run_batched(steps=100, warmup=args.warmup, mode=args.mode,
                                    tuner=default_tuner(), tile=tile)
    else:
        raise SystemExit('unknown workload %r' % args.workload)
    res['workload_name'] = args.workload
    print(json.dumps(res))
    return 0


def main():
    args = parse()
    if args.impl == 'reference':
        return run_reference(args)
    if args.workload:
        return run_workload(args)
    return run_ours(args)


if __name__ == '__main__':
    sys.exit(main())
