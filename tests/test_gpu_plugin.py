"""GPU tests of the drop-in kernel (gb1) through the plugin API, the way the
reference's front end drives any kernel (worker.py:119-136: add_object, start,
step, iterate over point masses)."""

import numpy as np
import pytest

import oracle
from gravitation_gb300.kernel import gb1
from gravitation_gb300.scenarios import G_DEFAULT, uniform_cube

pytestmark = pytest.mark.gpu


def make_universe(r, v, m, **kw):
    u = gb1.universe(**kw)
    for i in range(len(m)):
        u.add_object(name='b%d' % i, r=[float(x) for x in r[i]], v=[float(x) for x in v[i]],
                     m=float(m[i]))
    u.start()
    return u


def state(u):
    return (np.array([[float(c) for c in pm._r] for pm in u]),
            np.array([[float(c) for c in pm._v] for pm in u]))


def test_lifecycle_errors(gpu):
    r, v, m = uniform_cube(8, seed=1)
    u = gb1.universe()
    with pytest.raises(SyntaxError):
        u.step()
    u.add_object(name='a', r=list(r[0]), v=list(v[0]), m=float(m[0]))
    u.add_object(name='b', r=list(r[1]), v=list(v[1]), m=float(m[1]))
    u.start()
    with pytest.raises(SyntaxError):
        u.add_object(name='c', r=[0.0, 0, 0], v=[0.0, 0, 0], m=1.0)
    with pytest.raises(SyntaxError):
        u.start()
    u.step()
    u.stop()
    with pytest.raises(SyntaxError):
        u.step()


def test_plugin_fp32_matches_np1_golden(gpu, golden):
    u = make_universe(golden['c0_r0'], golden['c0_v0'], golden['c0_m'], dtype='float32')
    for _ in range(10):
        u.step()
        pm = next(iter(u))
        assert len(list(pm._r)) == 3 and len(list(pm._v)) == 3
        assert list(pm._a) == [0.0, 0.0, 0.0]
    r, v = state(u)
    # FP64 stage 2: the FP64 oracle trajectory to rounding of the FP32 forces
    r64, _ = oracle.rollout_fp64(golden['c0_r0'], golden['c0_v0'], golden['c0_m'],
                                 float(golden['G_scaled']), 1e3, 10)
    assert np.max(np.abs(r - r64) / np.abs(r64)) < 1e-12
    # np1 integrates in FP32 (its pm._a holds numpy float32): agreement to FP32 rounding
    ref = golden['np1_f32_r10']
    assert np.max(np.abs(r - ref) / np.abs(ref)) < 1e-4
    assert abs(u._t - 10 * 1e3) == 0.0
    u.stop()


def test_plugin_fp64_matches_np1_golden(gpu, golden):
    u = make_universe(golden['c0_r0'], golden['c0_v0'], golden['c0_m'], dtype='float64')
    for _ in range(10):
        u.step()
    r, v = state(u)
    ref = golden['np1_f64_r10']
    assert np.max(np.abs(r - ref) / np.abs(ref)) < 1e-13
    assert np.max(np.abs(v - golden['np1_f64_v10'])) < 1e-12


def test_host_mirror_edits_are_uploaded(gpu):
    """As with the reference's kernels, stage 1 sees pm._r edited between steps."""
    r, v, m = uniform_cube(300, seed=4)
    u = make_universe(r, v, m, dtype='float64')
    u.step()
    pms = list(u)
    pms[5]._r[:] = [1.0, 2.0, 3.0]
    pms[7]._v[:] = [0.0, 0.0, 0.0]
    r1, v1 = state(u)
    u.step()
    a = oracle.accel_fp64(r1, G_DEFAULT * m, 1.0)
    r_exp, v_exp = oracle.stage2_fp64(r1, v1, a, 1e3)
    r2, v2 = state(u)
    assert np.max(np.abs(r2 - r_exp) / np.maximum(np.abs(r_exp), 1.0)) < 1e-12


def test_unfused_stage1_fills_accelerations(gpu):
    r, v, m = uniform_cube(500, seed=6)
    u = make_universe(r, v, m, dtype='float64', fuse=False)
    u.step_stage1()
    a = np.array([[float(c) for c in pm._a] for pm in u])
    ref = oracle.accel_fp64(r, G_DEFAULT * m, 1.0)
    assert oracle.rel_err_per_body(a, ref).max() < 1e-12
    u.step_stage2()
    u.step_stage3()
    r1, v1 = state(u)
    r_exp, v_exp = oracle.stage2_fp64(r, v, ref, 1e3)
    assert np.max(np.abs(r1 - r_exp) / np.abs(r_exp)) < 1e-13


def test_precision_option_and_scaling(gpu, golden):
    """The reference's galaxy parameters (T=2e12, scale_m=1e-30, scale_r=1e-10,
    simulation.py:57-63) through add_object's scaling."""
    r, v, m = golden['gal_r0'], golden['gal_v0'], golden['gal_m']
    u = make_universe(r, v, m, T=float(golden['gal_T']), scale_m=float(golden['gal_scale_m']),
                      scale_r=float(golden['gal_scale_r']), dtype='float32', precision='fp32c',
                      fuse=False)
    assert u._G == float(golden['gal_G_scaled'])
    u.step_stage1()
    a = np.array([[float(c) for c in pm._a] for pm in u])
    sr, sm = float(golden['gal_scale_r']), float(golden['gal_scale_m'])
    ref = oracle.accel_fp64(r * sr, m * sm, u._G)
    assert oracle.rel_err_per_body(a, ref).max() < 1e-5
    # and the reference's own FP32 kernel on the same bodies
    assert np.median(oracle.rel_err_per_body(golden['gal_np1_f32_a0'], a)) < 1e-5


def test_frontend_protocol_workload(gpu):
    """The reference's worker protocol (gc off, gc.collect() between steps, best wall
    time) over device-generated galaxies, small sizes."""
    from gravitation_gb300.workloads import run_frontend
    import gc
    enabled = gc.isenabled()
    out = run_frontend(b_min=6, b_max=9, min_iterations=3, min_total_runtime=0.01)
    assert gc.isenabled() == enabled
    assert [r['n'] for r in out['sizes']] == [64, 128, 256, 512]
    for r in out['sizes']:
        assert r['steps'] >= 3 and 0 < r['best_ns'] <= r['avg_ns']
        # the float32 default below 4608 bodies: near pairs corrected, or double-single
        # separations for every pair where near pairs are common (the galaxy's disc)
        assert r['mode'] in ('fp32n', 'fp32c')


@pytest.mark.parametrize('sync', ['full', 'pull', 'none'])
def test_graph_step_matches_launched_step(gpu, sync):
    """The graph-replayed fused step (default), the same work launched call by call,
    the host-resident state (zero_copy, host_sync='full') and the unfused stages give
    bit-identical states, for every host_sync mode; with 'full' an edit of the host
    mirror between steps reaches all of them."""
    r, v, m = uniform_cube(700, seed=8)
    variants = [dict(graph=True), dict(graph=False)]
    if sync == 'full':
        variants = [dict(graph=True, zero_copy=True), dict(graph=False, zero_copy=True),
                    dict(graph=True, zero_copy=False), dict(graph=False, zero_copy=False),
                    dict(fuse=False, zero_copy=True), dict(fuse=False, zero_copy=False)]
    out = []
    for kw in variants:
        u = make_universe(r, v, m, dtype='float32', precision='fp32u', host_sync=sync, **kw)
        assert (u._gb_graph is not None) == (kw.get('graph', True) and kw.get('fuse', True))
        assert u._gb_zero_copy == (sync == 'full' and kw.get('zero_copy', True))
        for k in range(4):
            u.step()
            if k == 1 and sync == 'full':
                next(iter(u))._v[:] = [0.5, -0.25, 0.0]
        if sync == 'none':
            u.sync_host()
        assert all(list(pm._a) == [0.0, 0.0, 0.0] for pm in u)
        out.append(state(u))
        u.stop()
    for rv in out[1:]:
        assert np.array_equal(out[0][0], rv[0]) and np.array_equal(out[0][1], rv[1])
    assert not np.array_equal(out[0][0], r)


def test_plugin_small_universe_single_launch(gpu):
    """A small universe through the plugin takes the single-launch step, with the state
    in the pinned host mirror (read and written in place by the kernel) and the step
    replayed from a CUDA graph: the trajectory is the FP64 oracle's to the rounding of
    the FP32 forces, and pm._r / pm._v follow every step."""
    n = 300
    r0, v0, m = uniform_cube(n, seed=4)
    u = make_universe(r0, v0, m, dtype='float32')
    assert u._gb.fused and u._gb_zero_copy and u._gb_graph is not None
    for k in range(1, 6):
        u.step()
        r, v = state(u)
        r64, v64 = oracle.rollout_fp64(r0, v0, m, G_DEFAULT, 1e3, k)
        # per body: |r - r64| / |r64| (a coordinate near zero would inflate a
        # per-component ratio)
        err = np.linalg.norm(r - r64, axis=1) / np.linalg.norm(r64, axis=1)
        assert err.max() < 1e-12, (k, err.max())
        assert np.max(np.abs(v - v64)) < 1e-9, k
    u.stop()
