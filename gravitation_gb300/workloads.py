"""Measured workloads beyond the single-universe step (used by bench.py).

  run_batched   many universes of log-uniform size (64..16384) in one persistent launch
                per stage, the steady-state step replayed from a CUDA graph, tile shape
                from the autotuner -- against looping the single-universe step over the
                universes (one Engine per universe, each with its own tuned tile)
  run_adjoint   forward rollout vs forward + adjoint (N = 4096, 1000 steps)
  run_adjoint_check  adjoint gradients vs FP64 central differences
  run_precision Plummer-pair precision stress of the modes (errors, energy drift)
  run_sweep     one step per graph replay over N = 2^4 .. 2^17
  run_generate  scenario generation on the device; plugin start-up from a scenario
  run_frontend  the reference's benchmark/worker protocol over its galaxy scenario
"""

import statistics
import time

import numpy as np
import torch

from .engine import Engine
from .scenarios import G_DEFAULT, T_DEFAULT, batch_universes


def run_adjoint(n=4096, steps=1000, every=32, seed=3, reps=3, tuner=None, device=None):
    """Forward rollout vs forward + adjoint (gradients of the mean squared distance to a
    target made by the same run with masses scaled by a seeded factor in [0.99, 1.01]).
    Returns timings and the steps/s of forward+adjoint with the Rollout's defaults
    (checkpoints every `every` steps, the forward's accelerations kept where they fit:
    graph-replayed and launched) and, beside it, the variant that recomputes stage 1
    in the backward sweep instead (store_a=False)."""
    from .adjoint import Rollout
    from .scenarios import mass_perturbation, uniform_cube
    r, v, m = uniform_cube(n, seed=seed)
    dev = torch.device('cuda', torch.cuda.current_device() if device is None else device)
    gm = torch.tensor(G_DEFAULT * m, device=dev)
    gm_t = torch.tensor(G_DEFAULT * m * mass_perturbation(n, seed), device=dev)
    r0 = torch.tensor(r, device=dev)
    v0 = torch.tensor(v, device=dev)
    stream = torch.cuda.current_stream(dev)

    def measure(graphs, store_a='auto'):
        ro = Rollout([n], T_DEFAULT, steps, every, device=dev.index, tuner=tuner,
                     graphs=graphs, store_a=store_a)
        rt, _ = ro.forward(r0, v0, gm_t)
        rt = rt.clone()
        fwd_ms, tot_ms = [], []
        for _ in range(reps + 1):            # the first round captures the graphs
            e0, e1 = _events(1)[0]
            e2 = torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            e0.record(stream)
            rK, _ = ro.forward(r0, v0, gm)
            e1.record(stream)
            g_r = (2.0 / n) * (rK - rt)
            ro.backward(g_r, torch.zeros_like(g_r))
            e2.record(stream)
            e2.synchronize()
            fwd_ms.append(e0.elapsed_time(e1))
            tot_ms.append(e0.elapsed_time(e2))
        ro.adj.raise_on_device_error()
        ro.fwd.raise_on_device_error()
        f, t = min(fwd_ms[1:]), min(tot_ms[1:])
        return {'forward_ms': f, 'forward_adjoint_ms': t, 'forward_mode': ro.fwd.mode_name,
                'ratio_fwd_plus_adjoint_over_fwd': t / f,
                'fwd_adjoint_steps_per_s': steps / (t * 1e-3),
                'forward_tile': [ro.fwd.tile.bpt, ro.fwd.tile.threads, ro.fwd.tile.jtile,
                                 ro.fwd.info.grid],
                'backward_kernel': '%s, %s' % (
                    'unique pairs' if ro.adj.pairs else 'all pairs',
                    'forward accelerations kept' if ro.store_a else 'accelerations recomputed')}

    out = {'workload': 'N=%d uniform cube seed %d, %d steps, checkpoint every %d, loss = mean '
                       '|r_K - r_target|^2 (target: masses x U[0.99,1.01])' % (n, seed, steps,
                                                                             every),
           'launches_per_step': {'forward': 2, 'adjoint': 2}}
    out['graphs'] = measure(True)
    out['launched'] = measure(False)
    out['recomputed_accelerations'] = measure(True, store_a=False)
    out.update({k: out['graphs'][k] for k in ('forward_ms', 'forward_adjoint_ms',
                                             'ratio_fwd_plus_adjoint_over_fwd',
                                             'fwd_adjoint_steps_per_s', 'forward_mode')})
    return out


def run_adjoint_check(n=4096, steps=1000, every=32, seed=3, ncoords=16, eps=1e-6,
                      device=None, reference=True):
    """Gradients of the differentiable-rollout workload (N=4096, 1000 steps, checkpoint
    every 32) against FP64 central finite differences with step eps on `ncoords` seeded
    coordinates of (r0, v0, m).  The finite differences run full FP64 rollouts on the
    GPU (fp64 mode); the target is the same FP64 run with masses scaled by the seeded
    factor in [0.99, 1.01].  Returns per-coordinate gradients and relative errors, and
    (reference=True) every body's gradients against the exact FP64 discrete gradients
    (adjoint_reference_errors), which also resolve the mass gradients that finite
    differences cannot at this configuration."""
    from .adjoint import Rollout
    from .scenarios import mass_perturbation, uniform_cube
    r, v, m = uniform_cube(n, seed=seed)
    f = mass_perturbation(n, seed)
    dev = torch.device('cuda', torch.cuda.current_device() if device is None else device)
    e64 = Engine([n], T_DEFAULT, mode='fp64', device=dev.index)
    g64 = {}

    def final64(rr, vv, mm):
        e64.set_state(rr, vv, G_DEFAULT * mm)
        if every not in g64:
            g64[every] = e64.capture_graph(every)
        done = 0
        while done + every <= steps:
            g64[every].replay()
            done += every
        if done < steps:
            e64.step(steps - done)
        return e64.r[:n, :3].cpu().numpy()

    t = final64(r, v, m * f)

    def loss(rr, vv, mm):
        rk = final64(rr, vv, mm)
        return float(((rk - t) ** 2).sum(1).mean())

    # adjoint gradients (FP32 pairs, FP64 state) of the same loss
    ro = Rollout([n], T_DEFAULT, steps, every, device=dev.index)
    r0 = torch.tensor(r, device=dev)
    v0 = torch.tensor(v, device=dev)
    rK, _ = ro.forward(r0, v0, torch.tensor(G_DEFAULT * m, device=dev))
    tt = torch.tensor(t, device=dev)
    loss_adj = float(((rK - tt) ** 2).sum(1).mean())
    g_r, g_v, g_gm = ro.backward((2.0 / n) * (rK - tt), torch.zeros_like(rK))
    g_r, g_v = g_r.cpu().numpy(), g_v.cpu().numpy()
    g_m = G_DEFAULT * g_gm.cpu().numpy()
    rng = np.random.default_rng(np.random.SeedSequence([seed, 16]))
    rows = []
    for _ in range(ncoords):
        which = int(rng.integers(3))
        i = int(rng.integers(n))
        c = int(rng.integers(3))
        args_p = [r.copy(), v.copy(), m.copy()]
        args_m = [r.copy(), v.copy(), m.copy()]
        if which == 2:
            args_p[2][i] += eps
            args_m[2][i] -= eps
            g = float(g_m[i])
        else:
            args_p[which][i, c] += eps
            args_m[which][i, c] -= eps
            g = float((g_r, g_v)[which][i, c])
        fd = (loss(*args_p) - loss(*args_m)) / (2 * eps)
        rows.append({'var': ('r0', 'v0', 'm')[which], 'body': i, 'comp': c, 'adjoint': g,
                     'fd': fd, 'rel_err': abs(g - fd) / max(abs(fd), 1e-300)})
    e64.raise_on_device_error()
    errs = {k: [x['rel_err'] for x in rows if x['var'] == k] for k in ('r0', 'v0', 'm')}
    out = {'workload': 'N=%d uniform cube seed %d, %d steps, checkpoint every %d; FD eps %g '
                       'on %d seeded coordinates' % (n, seed, steps, every, eps, ncoords),
           'loss_fp64': loss(r, v, m), 'loss_adjoint_forward': loss_adj,
           'max_rel_err': {k: (max(vs) if vs else None) for k, vs in errs.items()},
           'median_rel_err': {k: (float(np.median(vs)) if vs else None) for k, vs in errs.items()},
           'coords': rows}
    if reference:
        out['fp64_reference'] = adjoint_reference_errors(
            r, v, m, tt, steps, (g_r, g_v, g_m), rows, dev)
    return out


def adjoint_reference_errors(r, v, m, target, steps, grads, coords, dev, every=8):
    """The adjoint's gradients (FP32 pair terms, FP64 state) against the exact FP64
    discrete gradients of the same loss, by autograd through the plain PyTorch FP64
    integrator with checkpoints (adjoint.reference_gradients_fp64), over every body:
    ||g - g64|| / ||g64|| for r0, v0 and m, the largest per-body error relative to the
    largest per-body gradient, and the finite differences' own error on `coords`."""
    from .adjoint import reference_gradients_fp64, torch_reference_rollout
    n = len(m)
    t0 = time.perf_counter()
    r0 = torch.tensor(r, device=dev)
    v0 = torch.tensor(v, device=dev)
    mm = torch.tensor(m, device=dev)
    with torch.no_grad():
        rk64, _ = torch_reference_rollout(r0, v0, mm, G_DEFAULT, T_DEFAULT, steps)
    g_rK = (2.0 / n) * (rk64 - target)
    ref = reference_gradients_fp64(r0, v0, mm, G_DEFAULT, T_DEFAULT, steps, g_rK,
                                   torch.zeros_like(g_rK), every=every)
    ref = [x.cpu().numpy() for x in ref]
    res = {'reference': 'autograd through a plain PyTorch FP64 integrator (checkpoints '
                        'every %d steps), same loss, every body' % every,
           'seconds': time.perf_counter() - t0}
    for name, g, g64 in zip(('r0', 'v0', 'm'), grads, ref):
        g = np.asarray(g).reshape(g64.shape)
        diff = np.abs(g - g64).reshape(n, -1).max(1)
        res[name] = {'rel_err_norm': float(np.linalg.norm(g - g64) / np.linalg.norm(g64)),
                     'max_body_err_over_max_grad': float(diff.max() / np.abs(g64).max())}
    fd_err = {'r0': [], 'v0': [], 'm': []}
    for c in coords:
        g64 = ref[('r0', 'v0', 'm').index(c['var'])]
        val = g64[c['body']] if c['var'] == 'm' else g64[c['body'], c['comp']]
        c['fp64_reference'] = float(val)
        fd_err[c['var']].append(abs(c['fd'] - val) / max(abs(val), 1e-300))
    res['fd_rel_err_vs_reference_max'] = {k: (max(x) if x else None) for k, x in fd_err.items()}
    return res


def fp64_forces(r, gm, device=None):
    """Every body's acceleration from the GPU FP64 mode (FP64 all pairs; the tests pin
    that mode to the CPU FP64 oracle at 1e-12) for positions r and G*m gm."""
    n = len(gm)
    e = Engine([n], 1.0, mode='fp64', device=device)
    e.set_state(r, np.zeros((n, 3)), gm)
    a = e.forces().cpu().numpy()
    e.raise_on_device_error()
    return a


def rel_err_per_body(a, ref):
    """|a_i - ref_i| / |ref_i| per body (0 where both vanish)."""
    num = np.linalg.norm(np.asarray(a) - np.asarray(ref), axis=1)
    den = np.linalg.norm(np.asarray(ref), axis=1)
    return np.where(den > 0, num / np.where(den > 0, den, 1.0), np.where(num > 0, np.inf, 0.0))


def run_precision(n=16384, steps=10000, every=100, seed=2,
                  modes=('fp32u', 'fp32un', 'fp32cu', 'fp32c', 'fp64'),
                  check=None, device=None):
    """Precision stress: two Plummer spheres (scale radius 50, centres 1000 apart,
    approaching at 5 along x, masses log-uniform in [0.1, 1000]).  For each mode: the
    per-body acceleration error at the first and the last step over every body, against
    the FP64 forces of the same FP64 state (``check(r, gm, a)`` returning per-body
    errors, default: the GPU FP64 mode, fp64_forces), and the relative drift of the FP64
    energy and momentum every `every` steps.  Returns a dict per mode."""
    from .scenarios import plummer_pair
    r, v, m = plummer_pair(n, seed=seed)
    gm = G_DEFAULT * m
    dev = torch.device('cuda', torch.cuda.current_device() if device is None else device)
    if check is None:
        def check(rs, gms, a):
            return rel_err_per_body(a, fp64_forces(rs, gms, dev.index))
    out = {'workload': 'Plummer pair N=%d seed %d, %d steps, T=%g; force errors over every '
                       'body against the FP64 forces of the same state' % (n, seed, steps,
                                                                           T_DEFAULT)}
    finals = {}
    for mode in modes:
        eng = Engine([n], T_DEFAULT, mode=mode, device=dev.index)
        eng.set_state(r, v, gm)
        errs = []
        e0 = eng.energy(G_DEFAULT)[0]
        E0 = e0[0] + e0[1]
        P0 = e0[2:5]
        pscale = float((m * np.linalg.norm(v, axis=1)).sum())
        drift_e, drift_p = [], []

        def accel_err():
            rs = eng.r[:n, :3].cpu().numpy()
            a = eng.forces().cpu().numpy()
            e = np.asarray(check(rs, gm, a))
            return float(e.max()), int((e > 1e-5).sum())
        errs.append(accel_err())
        graph = eng.capture_graph(every)
        t0 = time.perf_counter()
        done = 0
        while done < steps:
            graph.replay()
            done += every
            e = eng.energy(G_DEFAULT)[0]
            drift_e.append(abs((e[0] + e[1]) - E0) / abs(E0))
            drift_p.append(float(np.linalg.norm(e[2:5] - P0)) / pscale)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        errs.append(accel_err())
        finals[mode] = eng.r[:n, :3].cpu().numpy()
        eng.raise_on_device_error()
        out[mode] = {'accel_err_first': errs[0][0], 'accel_err_last': errs[1][0],
                     'bodies_above_1e-5_first': errs[0][1], 'bodies_above_1e-5_last': errs[1][1],
                     'energy_drift_max': max(drift_e), 'energy_drift_final': drift_e[-1],
                     'momentum_drift_max': max(drift_p), 'wall_s': wall, 'steps': done,
                     'energy_every': every}
    if 'fp64' in finals:
        ref = finals['fp64']
        scale = np.abs(ref).max()
        for mode in modes:
            if mode != 'fp64':
                out[mode]['final_pos_dev_vs_fp64_rel'] = float(np.abs(finals[mode] - ref).max() / scale)
    return out


def run_sweep(sizes=None, mode=None, reps=50, tuner=None, device=None):
    """Interactions/s of the single-universe step over an N sweep (2^4 .. 2^17), with
    the state in HBM.  mode None: the plugin's float32 default at each size (all pairs
    below 4608 bodies, unique pairs from there, near pairs corrected).  Below 8192 bodies
    one graph replay holds 20 steps, so that the host's graph-launch rate does not set
    the measured step time; above, one step per replay.  Up to 512 bodies the engine
    takes the single-launch step (grav_step_fused).  At least `reps` steps are
    timed: the near-pair kernels' cost follows the state, which at the reference's time
    step streams from the cube towards the shape of its velocity distribution."""
    from .plugin import default_mode
    from .scenarios import uniform_cube
    sizes = sizes or [2 ** k for k in range(4, 18)]
    dev = torch.device('cuda', torch.cuda.current_device() if device is None else device)
    stream = torch.cuda.current_stream(dev)
    res = []
    for n in sizes:
        m_n = mode or default_mode('float32', n)
        r, v, m = uniform_cube(n, seed=0)
        eng = Engine([n], T_DEFAULT, mode=m_n, tuner=tuner, device=dev.index)
        eng.set_state(r, v, G_DEFAULT * m)
        per = 20 if n < 8192 else 1
        g = eng.capture_graph(per)
        for _ in range(3):
            g.replay()
        e0, e1 = _events(1)[0]
        k = max(reps, int(2e10 // (n * n * per)) if n < 8192 else reps)
        k = min(k, 200)
        e0.record(stream)
        for _ in range(k):
            g.replay()
        e1.record(stream)
        e1.synchronize()
        ms = e0.elapsed_time(e1) / (k * per)
        res.append({'n': n, 'mode': m_n, 'ms_per_step': ms,
                    'interactions_per_s': n * n / (ms * 1e-3),
                    'steps_per_replay': per,
                    'kernel': ('single launch (threads, rows) = %d, %d' % eng.fused
                               if eng.fused else 'stage 1 + stage 2'),
                    'tile': [eng.tile.bpt, eng.tile.threads, eng.tile.jtile, eng.info.grid]})
        eng.raise_on_device_error()
    return res


def _events(n):
    return [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
            for _ in range(n)]


def _loop_timings(engines, stream, dev, warmup, loop_steps):
    """Per-universe loop of single-universe steps: wall clock of launched steps (host
    launch overhead included) and device time of the same loop captured in one graph."""
    for _ in range(warmup):
        for e in engines:
            e.step(1)
    torch.cuda.synchronize()
    walls = []
    for _ in range(loop_steps):
        t0 = time.perf_counter()
        for e in engines:
            e.step(1)
        torch.cuda.synchronize()
        walls.append(time.perf_counter() - t0)
    side = torch.cuda.Stream(device=dev)
    side.wait_stream(stream)
    g2 = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g2, stream=side):
        for e in engines:
            e.step(1, stream=side)
    stream.wait_stream(side)
    g2.replay()
    torch.cuda.synchronize()
    e0, e1 = _events(1)[0]
    e0.record(stream)
    for _ in range(loop_steps):
        g2.replay()
    e1.record(stream)
    e1.synchronize()
    for e in engines:
        e.raise_on_device_error()
    return 1e3 * statistics.mean(walls), e0.elapsed_time(e1) / loop_steps


def run_batched(steps=100, warmup=3, mode='fp32un', n_univ=256, seed=1, loop_steps=10,
                tuner=None, device=None, tile=None):
    """Batched step vs the per-universe loop.  Returns a dict of measurements.

    The batch runs in `mode` with the tile the autotuner picks for the batch.  The loop
    is timed twice: with every universe in the mode and tile the plugin itself would
    use for it alone (plugin.default_mode: all pairs below 4608 bodies, unique pairs
    from there; each universe's own tuned tile) -- the fair comparison, reported as
    speedup_vs_loop / speedup_vs_graphed_loop -- and with every universe in the batch's
    mode (each its own tuned tile)."""
    from .plugin import default_mode
    sizes, states = batch_universes(n_univ, seed)
    sizes = [int(s) for s in sizes]
    r = np.concatenate([s[0] for s in states])
    v = np.concatenate([s[1] for s in states])
    gm = G_DEFAULT * np.concatenate([s[2] for s in states])
    inter = float(sum(n * n for n in sizes))
    dev = torch.device('cuda', torch.cuda.current_device() if device is None else device)
    stream = torch.cuda.current_stream(dev)

    eng = Engine(sizes, T_DEFAULT, mode=mode, tile=tile, tuner=tuner, device=dev.index)
    eng.set_state(r, v, gm)
    graph = eng.capture_graph(1)
    for _ in range(warmup):
        graph.replay()
    torch.cuda.synchronize()
    e0, e1 = _events(1)[0]
    e0.record(stream)
    for _ in range(steps):
        graph.replay()
    e1.record(stream)
    e1.synchronize()
    eng.raise_on_device_error()
    batched_ms = e0.elapsed_time(e1) / steps

    # the same batch, launched step by step without the graph
    e0.record(stream)
    eng.step(steps)
    e1.record(stream)
    e1.synchronize()
    nograph_ms = e0.elapsed_time(e1) / steps

    def loop_engines(mode_of):
        engines, off = [], 0
        for n in sizes:
            e = Engine([n], T_DEFAULT, mode=mode_of(n), tuner=tuner, device=dev.index)
            e.set_state(r[off:off + n], v[off:off + n], gm[off:off + n])
            engines.append(e)
            off += n
        return engines

    def plugin_mode(n):
        # the float32 default for one universe of n bodies; a batch forced to another
        # precision compares with universes forced to it too
        return default_mode('float32', n) if mode in ('fp32n', 'fp32un') else mode

    engines = loop_engines(plugin_mode)
    loop_ms, loop_graph_ms = _loop_timings(engines, stream, dev, warmup, loop_steps)
    modes_used = sorted({e.mode_name for e in engines})
    del engines
    engines = loop_engines(lambda n: mode)
    same_ms, same_graph_ms = _loop_timings(engines, stream, dev, warmup, loop_steps)
    del engines

    return {
        'workload': '%d universes, N log-uniform in [64,16384] (seed %d), uniform cube each, '
                    '%s stage 1 + FP64 stage 2' % (n_univ, seed, mode),
        'interactions_per_step': inter,
        'bodies': int(sum(sizes)),
        'batched_ms_per_step': batched_ms,
        'batched_interactions_per_s': inter / (batched_ms * 1e-3),
        'batched_no_graph_ms_per_step': nograph_ms,
        'loop': 'each universe in the mode and tile the plugin picks for it alone (%s)' %
                ', '.join(modes_used),
        'loop_ms_per_step': loop_ms,
        'loop_graph_ms_per_step': loop_graph_ms,
        'speedup_vs_loop': loop_ms / batched_ms,
        'speedup_vs_graphed_loop': loop_graph_ms / batched_ms,
        'loop_same_mode_ms_per_step': same_ms,
        'loop_same_mode_graph_ms_per_step': same_graph_ms,
        'speedup_vs_graphed_loop_same_mode': same_graph_ms / batched_ms,
        'tile': {'bpt': eng.tile.bpt, 'threads': eng.tile.threads, 'jtile': eng.tile.jtile,
                 'grid': eng.info.grid},
        'launches_per_step': 2,
        'loop_launches_per_step': 2 * n_univ,
    }


def run_generate(n_big=1 << 24, n_plugin=1 << 17, reps=5, hbm_gbs=None, device=None):
    """Scenario generation on the device (gravitation_gb300.generate).

    Throughput: n_big bodies of each scenario written into device r, v (64 B per body
    written: two rows of 4 doubles; nothing read but the Plummer's per-CTA sums), CUDA
    events around each call, best of `reps`, against the HBM copy bandwidth.  Start-up:
    a gb1 universe of n_plugin bodies started from a scenario against the same universe
    built by n_plugin add_object calls with numpy-generated bodies (wall clock)."""
    from . import generate as gen
    from .kernel import gb1
    from .scenarios import uniform_cube
    dev = torch.device('cuda', torch.cuda.current_device() if device is None else device)
    stream = torch.cuda.current_stream(dev)
    r = torch.empty((n_big, 4), dtype=torch.float64, device=dev)
    v = torch.empty((n_big, 4), dtype=torch.float64, device=dev)
    out = {'n': n_big, 'bytes_written_per_body': 64}
    cases = {'uniform_cube': gen.uniform_cube(n_big, seed=0),
             'plummer_pair': gen.plummer_pair(n_big, seed=2),
             'galaxy': gen.galaxy(n_big, seed=0)}
    for name, parts in cases.items():
        G = G_DEFAULT * (1e-10 ** 3 / 1e-30 if name == 'galaxy' else 1.0)
        gen.generate(parts, r, v, G, stream)
        ms = []
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            gen.generate(parts, r, v, G, stream)
            e1.record(stream)
            e1.synchronize()
            ms.append(e0.elapsed_time(e1))
        best = min(ms)
        gbs = 64.0 * n_big / (best * 1e-3) / 1e9
        # FP64 log/exp/sin/cos per body on GB300's reduced FP64 pipe bound these
        # kernels, not the 64 B/body of writes (fraction of HBM reported for scale)
        out[name] = {'ms': best, 'bodies_per_s': n_big / (best * 1e-3), 'write_gbs': gbs,
                     'hbm_frac': gbs / hbm_gbs if hbm_gbs else None,
                     'launches': 3 * len(parts) if name == 'plummer_pair' else len(parts)}
    del r, v
    torch.cuda.synchronize()

    # one untimed start first: the tile autotuner's first visit to this size class and
    # the first graph capture would otherwise be charged to whichever path runs first
    w = gb1.universe(scenario={'kind': 'uniform_cube', 'n': n_plugin, 'seed': 1})
    w.start()
    w.stop()
    t0 = time.perf_counter()
    u = gb1.universe(scenario={'kind': 'uniform_cube', 'n': n_plugin, 'seed': 0})
    u.start()
    t_scen = time.perf_counter() - t0
    u.step()
    u.stop()
    t0 = time.perf_counter()
    rr, vv, mm = uniform_cube(n_plugin, seed=0)
    w = gb1.universe()
    for i in range(n_plugin):
        w.add_object(name='b', r=[float(rr[i, 0]), float(rr[i, 1]), float(rr[i, 2])],
                     v=[float(vv[i, 0]), float(vv[i, 1]), float(vv[i, 2])], m=float(mm[i]))
    t_objects = time.perf_counter() - t0
    w.start()
    t_add = time.perf_counter() - t0
    w.stop()
    out['plugin_start'] = {'n': n_plugin, 'scenario_s': t_scen, 'add_object_s': t_add,
                           'add_object_loop_s': t_objects, 'speedup': t_add / t_scen}
    return out


def run_frontend(b_min=10, b_max=17, min_iterations=10, min_total_runtime=1.0, seed=0,
                 device=None):
    """The reference's benchmark over its galaxy scenario, measured the way its worker
    measures a kernel, with the gb1 plugin as the kernel.

    `gravitation benchmark -k gb1 -b 10 17` starts one worker per size 2^b
    (cli/benchmark.py) on the galaxy scenario with stars_len = 2^b (simulation.py:57-77);
    the worker (cli/worker.py:109-245) disables the garbage collector, and for each step
    runs gc.collect(), times s.step() by wall clock (lib/timing.py:41-78, best_run_timer),
    takes at least min_iterations steps, then more until min_total_runtime has passed,
    and reports the best step time.  Here the universes start from the galaxy generated
    on the device (the reference's generator is unseeded Python) with the recipe's
    universe parameters; dtype float32 as in the scenario, so the plugin picks all pairs
    below 4608 bodies and unique pairs above."""
    import gc
    from . import generate as gen
    from .kernel import gb1
    rows = []
    for b in range(b_min, b_max + 1):
        n = 1 << b
        u = gb1.universe(scenario={'kind': 'galaxy', 'n': n, 'seed': seed}, dtype='float32',
                         device=device, **gen.galaxy_universe_params())
        u.start()
        times = []
        gc_was = gc.isenabled()
        gc.disable()
        try:
            t_start = time.perf_counter_ns()

            def one():
                gc.collect()
                t0 = time.perf_counter_ns()
                u.step()
                times.append(time.perf_counter_ns() - t0)
                gc.collect()

            for _ in range(min_iterations):
                one()
            elapsed = time.perf_counter_ns() - t_start
            target = int(min_total_runtime * 1e9)
            if elapsed < target:
                for _ in range((target - elapsed) // elapsed * min_iterations):
                    one()
        finally:
            if gc_was:
                gc.enable()
        mode = u._gb.mode_name
        u.stop()
        best = min(times)
        rows.append({'n': n, 'mode': mode, 'steps': len(times), 'best_ns': best,
                     'avg_ns': sum(times) // len(times),
                     'interactions_per_s_best': n * n / (best * 1e-9)})
    return {'workload': 'galaxy scenario (reference parameters), N = 2^%d..2^%d, worker '
                        'protocol: gc off, gc.collect() between steps, wall clock, best of '
                        '>= %d steps and >= %g s' % (b_min, b_max, min_iterations,
                                                     min_total_runtime),
            'path': 'gb1.universe.step(), host_sync=full (pm._r/pm._v valid after every step)',
            'sizes': rows}
