"""GPU tests of the single-launch step (grav_step_fused) for one small universe.

Each CTA holds every position in shared memory, completes its rows' accelerations and
integrates them; one CTA alone, a thread-block cluster's barrier or (more than 16 CTAs)
a grid barrier on two device counters keeps every CTA's reads ahead of the writes.
Checked here, through the C ABI (Engine with fused=(threads, rows)):
  - the accelerations it writes (GRAV_S2_WRITE_A) against the FP64 oracle at the same
    tolerances as the two-launch step (test_gpu_parity.py), for every compiled thread
    count, rows per CTA that are and are not multiples of 32, one CTA and many;
  - the FP64 update bit-exact against v = a*T + v ; r = v*T + r given those
    accelerations (_base_.py:58-62), and the refreshed stage-1 positions bit-equal to
    what grav_prepare writes from the new state;
  - agreement with the two-launch step over 20 steps, run-to-run and graph-replay
    bit-equality, and the barrier counters back at zero after every step;
  - the counter barrier's bounded wait: made to expire, it reports GRAV_DEV_TIMEOUT,
    writes nothing and leaves the counters ready for the next step.
"""

import ctypes

import numpy as np
import pytest
import torch

import oracle
from gravitation_gb300 import _lib
from gravitation_gb300.engine import Engine, default_fused
from gravitation_gb300.scenarios import G_DEFAULT, uniform_cube, plummer_pair

pytestmark = pytest.mark.gpu

TOL = 1e-5
CONFIGS = [(256, 32), (256, 48), (512, 128), (1024, 32), (1024, 1024), (256, 256)]


def r32(r):
    return np.asarray(r, dtype=np.float64).astype(np.float32).astype(np.float64)


def oracle_accel(mode, r, gm):
    if mode == 'fp32':
        gm32 = np.asarray(gm).astype(np.float32).astype(np.float64)
        return oracle.accel_fp64(r32(r), gm32, 1.0, coincident=True)
    return oracle.accel_fp64(r, np.asarray(gm), 1.0, coincident=True)


def fused_engine(mode, n, cfg, T=1e3):
    try:
        return Engine([n], T, mode=mode, fused=cfg)
    except ValueError:
        return None   # more CTAs than can be resident at once for this configuration


@pytest.mark.parametrize('mode', ['fp32', 'fp32n', 'fp32c'])
@pytest.mark.parametrize('n', [1, 2, 31, 33, 100, 257, 512, 1000, 4096])
def test_fused_step_against_oracle(gpu, mode, n):
    r, v, m = uniform_cube(n, seed=300 + n)
    gm = G_DEFAULT * m
    ref = oracle_accel(mode, r, gm)
    ran = 0
    for cfg in CONFIGS:
        eng = fused_engine(mode, n, cfg)
        if eng is None:
            continue
        eng.set_state(r, v, gm)
        eng.step(1, write_a=True)
        torch.cuda.synchronize()
        eng.raise_on_device_error()
        a = eng.a[:n, :3].cpu().numpy()
        if n > 1:
            assert oracle.rel_err_per_body(a, ref).max() < TOL, cfg
        else:
            assert np.all(a == 0.0)
        # the FP64 update, bit for bit, from the accelerations it used
        r_exp, v_exp = oracle.stage2_fp64(r, v, a, 1e3)
        assert np.array_equal(eng.v[:n, :3].cpu().numpy(), v_exp), cfg
        assert np.array_equal(eng.r[:n, :3].cpu().numpy(), r_exp), cfg
        # the stage-1 positions it wrote are those grav_prepare derives from the state
        pos = eng.pos.clone()
        eng.prepare()
        torch.cuda.synchronize()
        assert torch.equal(pos, eng.pos), cfg
        assert eng.sync.cpu().tolist() == [0, 0], cfg
        ran += 1
    assert ran > 0


@pytest.mark.parametrize('mode', ['fp32', 'fp32n', 'fp32c'])
def test_fused_matches_two_launch_step(gpu, mode):
    """20 steps: the single-launch step and the two-launch step agree to the FP32
    rounding of the partial sums (a different summation order)."""
    n = 700
    r, v, m = uniform_cube(n, seed=7)
    gm = G_DEFAULT * m
    a = Engine([n], 1e3, mode=mode, fused=(512, 32))
    b = Engine([n], 1e3, mode=mode, fused=False)
    assert a.fused == (512, 32) and b.fused is None
    for e in (a, b):
        e.set_state(r, v, gm)
        e.step(20)
    torch.cuda.synchronize()
    ra, rb = a.r[:n, :3].cpu().numpy(), b.r[:n, :3].cpu().numpy()
    assert np.max(np.abs(ra - rb) / np.abs(rb)) < 1e-12
    fa, fb = a.forces().cpu().numpy(), b.forces().cpu().numpy()
    assert oracle.rel_err_per_body(fa, fb).max() < 2e-6


def test_fused_near_pairs(gpu):
    """Near-pair correction in the single-launch step: a Plummer pair far from the origin
    (near pairs common) against the FP64 oracle on the FP64 state."""
    n = 512
    r, v, m = plummer_pair(n, seed=4)
    r = r + 1e4
    gm = G_DEFAULT * m
    eng = Engine([n], 1e3, mode='fp32n', fused=(512, 32))
    eng.set_state(r, v, gm)
    eng.step(1, write_a=True)
    torch.cuda.synchronize()
    a = eng.a[:n, :3].cpu().numpy()
    assert oracle.rel_err_per_body(a, oracle_accel('fp32n', r, gm)).max() < TOL
    # and without the correction the same state is visibly worse
    plain = Engine([n], 1e3, mode='fp32', fused=(512, 32))
    plain.set_state(r, v, gm)
    plain.step(1, write_a=True)
    torch.cuda.synchronize()
    a_plain = plain.a[:n, :3].cpu().numpy()
    assert oracle.rel_err_per_body(a_plain, oracle_accel('fp32n', r, gm)).max() > TOL


def test_fused_deterministic_and_graph_replay(gpu):
    n = 1000
    r, v, m = uniform_cube(n, seed=8)
    gm = G_DEFAULT * m
    engines = [Engine([n], 1e3, mode='fp32n', fused=(1024, 32)) for _ in range(3)]
    for e in engines:
        e.set_state(r, v, gm)
    engines[0].step(6)
    engines[1].step(6)
    g = engines[2].capture_graph(3)
    g.replay()
    g.replay()
    torch.cuda.synchronize()
    for e in engines[1:]:
        assert torch.equal(engines[0].r, e.r) and torch.equal(engines[0].v, e.v)
        assert torch.equal(engines[0].pos, e.pos)
    for e in engines:
        e.raise_on_device_error()
        assert e.sync.cpu().tolist() == [0, 0]


def test_default_rule(gpu):
    """The engine takes the single-launch step by itself for one small universe in an
    all-pairs FP32 mode, and the two-launch step otherwise."""
    assert Engine([100], 1e3, mode='fp32n').fused is not None
    assert Engine([512], 1e3, mode='fp32').fused is not None
    assert Engine([4096], 1e3, mode='fp32n').fused is None
    assert Engine([100], 1e3, mode='fp64').fused is None
    assert Engine([100, 50], 1e3, mode='fp32').fused is None
    assert default_fused('fp32un', [100]) is None
    with pytest.raises(ValueError):
        Engine([100, 50], 1e3, mode='fp32', fused=(256, 32))


def test_fused_rejects_non_resident_grid(gpu):
    """A grid that cannot be resident at once is refused on the host (the cooperative
    launch would fail): 4096 bodies at 1 row per CTA."""
    with pytest.raises(ValueError):
        Engine([4096], 1e3, mode='fp32', fused=(1024, 1))
    eng = Engine([64], 1e3, mode='fp32', fused=(256, 32))
    L = _lib.load()
    occ = ctypes.c_int32()
    assert L.grav_fused_occupancy(_lib.GRAV_MODE_FP32, 64, 256, 32, ctypes.byref(occ)) == 0
    assert occ.value >= 1
    eng.set_state(*uniform_cube(64, seed=1)[:2], G_DEFAULT * uniform_cube(64, seed=1)[2])
    eng.step(2)
    eng.raise_on_device_error()


def test_counter_barrier_timeout_is_reported(gpu):
    """The grid barrier of a cooperative single-launch step (128 CTAs) gives up after its
    bounded wait when the arrivals never add up -- its arrive counter is preset so far
    below zero that nothing brings it to the grid size (a flag that nothing sets) --
    records GRAV_DEV_TIMEOUT, writes nothing, and the last CTA out still resets the
    counters, so the next step runs normally."""
    n = 4096
    eng = Engine([n], 1e3, mode='fp32', fused=(256, 32))
    assert -(-n // 32) > 16          # more CTAs than one cluster: the counter barrier
    r, v, m = uniform_cube(n, seed=9)
    eng.set_state(r, v, G_DEFAULT * m)
    r_before, v_before = eng.r.clone(), eng.v.clone()
    eng.sync[0] = -(1 << 30)
    eng.step(1)
    torch.cuda.synchronize()
    assert int(eng.err.item()) == _lib.GRAV_DEV_TIMEOUT
    assert torch.equal(eng.r, r_before) and torch.equal(eng.v, v_before)
    assert eng.sync.cpu().tolist() == [0, 0]
    with pytest.raises(_lib.GravError):
        eng.raise_on_device_error()
    eng.err.zero_()
    eng.step(1)
    torch.cuda.synchronize()
    eng.raise_on_device_error()
    assert not torch.equal(eng.r, r_before)
