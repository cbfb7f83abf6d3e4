"""GPU parity tests: the CUDA path (through the C ABI) against the CPU oracle and the
reference's golden vectors.

Tolerances (relative per-body acceleration error |a - a_ref| / |a_ref|):
  fp32, fp32u    1e-5 against the FP64 oracle evaluated on the FP32-rounded positions
                 the kernel reads (arithmetic error), as the reference's own FP32
                 kernels (np1/np2) are measured from identical states
  fp32n, fp32un  1e-5 against the FP64 oracle on the FP64 state itself (the plugin's
                 float32 default: near pairs from double-single separations)
  fp32c, fp32cu  1e-5 against the FP64 oracle on the FP64 state itself
  fp64           1e-12 against the FP64 oracle on the FP64 state
Stage 2 is bit-exact against the FP64 update of _base_.py:58-62.
"""

import numpy as np
import pytest
import torch

import oracle
from gravitation_gb300 import _lib
from gravitation_gb300.engine import Engine, tile_list
from gravitation_gb300.scenarios import G_DEFAULT, uniform_cube, plummer_pair

pytestmark = pytest.mark.gpu

TOL = {'fp32': 1e-5, 'fp32u': 1e-5, 'fp32n': 1e-5, 'fp32un': 1e-5, 'fp32c': 1e-5,
       'fp32cu': 1e-5, 'fp64': 1e-12}
ALL_MODES = ['fp32', 'fp32u', 'fp32n', 'fp32un', 'fp32c', 'fp32cu', 'fp64']


def r32(r):
    return np.asarray(r, dtype=np.float64).astype(np.float32).astype(np.float64)


def oracle_accel(mode, r, m, G, rows=None):
    """FP64 oracle on the state the mode is compared against (see module doc)."""
    if mode in ('fp32', 'fp32u'):
        gm32 = (G * np.asarray(m)).astype(np.float32).astype(np.float64)
        return oracle.accel_fp64(r32(r), gm32, 1.0, rows=rows, coincident=True)
    return oracle.accel_fp64(r, G * np.asarray(m), 1.0, rows=rows, coincident=True)


def engine_forces(mode, r, v, m, G=G_DEFAULT, tile=None):
    eng = Engine([len(m)], 1e3, mode=mode, tile=tile)
    eng.set_state(r, v, G * np.asarray(m))
    a = eng.forces().cpu().numpy()
    eng.raise_on_device_error()
    return a, eng


@pytest.mark.parametrize('mode', ALL_MODES)
@pytest.mark.parametrize('n', [1, 2, 3, 31, 33, 127, 129, 257, 1000])
def test_forces_small_n(gpu, mode, n):
    r, v, m = uniform_cube(n, seed=100 + n)
    a, _ = engine_forces(mode, r, v, m)
    ref = oracle_accel(mode, r, m, G_DEFAULT)
    if n == 1:
        assert np.all(a == 0.0)
        return
    err = oracle.rel_err_per_body(a, ref)
    assert err.max() < TOL[mode], (mode, n, err.max())


@pytest.mark.parametrize('mode', ALL_MODES)
def test_every_tile_shape(gpu, mode):
    n = 777
    r, v, m = uniform_cube(n, seed=7)
    ref = oracle_accel(mode, r, m, G_DEFAULT)
    for t in tile_list(mode):
        for grid in (1, 3, 1000):
            try:
                a, _ = engine_forces(mode, r, v, m, tile=_lib.Tile(t.bpt, t.threads, t.jtile, grid))
            except _lib.GravError as e:
                raise AssertionError('%s tile %r grid %d: %s' % (mode, t, grid, e)) from e
            err = oracle.rel_err_per_body(a, ref).max()
            assert err < TOL[mode], (mode, t, grid, err)


def test_np1_golden_fp32(gpu, golden):
    """The reference's np1 FP32 per-step accelerations, from the same state."""
    G = float(golden['G_scaled'])
    r0, v0, m = golden['c0_r0'], golden['c0_v0'], golden['c0_m']
    a, _ = engine_forces('fp32', r0, v0, m, G)
    ref64 = oracle_accel('fp32', r0, m, G)
    assert oracle.rel_err_per_body(a, ref64).max() < 1e-5
    assert oracle.rel_err_per_body(a, golden['np1_f32_a'][0]).max() < 2e-5


def test_np1_golden_trajectory_fp32(gpu, golden):
    """10 steps with FP32 stage 1 and FP64 stage 2 -- the same split as np1 with the
    base class's stage 2 -- against np1's states and accelerations."""
    G, T = float(golden['G_scaled']), float(golden['T'])
    r0, v0, m = golden['c0_r0'], golden['c0_v0'], golden['c0_m']
    eng = Engine([len(m)], T, mode='fp32')
    eng.set_state(r0, v0, G * m)
    for k in range(10):
        rk = eng.r[:len(m), :3].cpu().numpy()
        eng.step(1, write_a=True)
        a = eng.a[:len(m), :3].cpu().numpy()
        # ours against the FP64 oracle on the positions stage 1 reads
        ref = oracle_accel('fp32', rk, m, G)
        assert oracle.rel_err_per_body(a, ref).max() < 1e-5, k
        # and against np1's own FP32 result: np1 itself is up to ~2e-5 away from the
        # FP64 oracle on some bodies, so agreement is bounded by np1's own error + 1e-5
        e_np1 = oracle.rel_err_per_body(golden['np1_f32_a'][k], ref)
        e_pair = oracle.rel_err_per_body(a, golden['np1_f32_a'][k])
        assert np.all(e_pair <= e_np1 * 1.01 + 1e-5), k
    r = eng.r[:len(m), :3].cpu().numpy()
    v = eng.v[:len(m), :3].cpu().numpy()
    # FP64 integration: the FP32 force error (~1e-6 of a) moves r by ~1e-6 a T^2,
    # far below the positions' size
    r64, v64 = oracle.rollout_fp64(r0, v0, m, G, T, 10)
    assert np.max(np.abs(r - r64) / np.abs(r64)) < 1e-12
    assert np.max(np.abs(v - v64)) < 1e-12
    # np1's state: its stage 2 runs on numpy float32 scalars (pm._a holds float32
    # after np1.py:107-108, so a*T + v stays float32), i.e. FP32 integration
    assert np.max(np.abs(r - golden['np1_f32_r10']) / np.abs(golden['np1_f32_r10'])) < 1e-4


def test_np1_golden_trajectory_fp64(gpu, golden):
    G, T = float(golden['G_scaled']), float(golden['T'])
    r0, v0, m = golden['c0_r0'], golden['c0_v0'], golden['c0_m']
    eng = Engine([len(m)], T, mode='fp64')
    eng.set_state(r0, v0, G * m)
    eng.step(1, write_a=True)
    assert oracle.rel_err_per_body(eng.a[:len(m), :3].cpu().numpy(),
                                   golden['np1_f64_a0']).max() < 1e-12
    eng.step(9)
    r = eng.r[:len(m), :3].cpu().numpy()
    assert np.max(np.abs(r - golden['np1_f64_r10']) / np.abs(golden['np1_f64_r10'])) < 1e-13
    eng.raise_on_device_error()


def test_py1_golden_fp64(gpu, golden):
    a, _ = engine_forces('fp64', golden['py1_r0'], golden['py1_v0'], golden['py1_m'])
    assert oracle.rel_err_per_body(a, golden['py1_a0']).max() < 1e-12


@pytest.mark.parametrize('mode', ['fp32', 'fp64'])
def test_stage2_bit_exact(gpu, mode):
    """Given the accelerations, stage 2 equals v = a*T + v ; r = v*T + r in FP64."""
    n = 3000
    r, v, m = uniform_cube(n, seed=21)
    eng = Engine([n], 1e3, mode=mode)
    eng.set_state(r, v, G_DEFAULT * m)
    a = eng.forces().cpu().numpy().copy()
    eng.stage2(_lib.GRAV_S2_INTEGRATE)
    r_exp, v_exp = oracle.stage2_fp64(r, v, a, 1e3)
    assert np.array_equal(eng.v[:n, :3].cpu().numpy(), v_exp)
    assert np.array_equal(eng.r[:n, :3].cpu().numpy(), r_exp)


def test_full_size_sampled_65536(gpu):
    """N = 65536: sampled bodies against the FP64 oracle, every FP32 mode."""
    n = 65536
    r, v, m = uniform_cube(n, seed=0)
    rows = np.random.default_rng(9).choice(n, 192, replace=False)
    for mode in ('fp32', 'fp32u', 'fp32n', 'fp32un', 'fp32c', 'fp32cu'):
        a, _ = engine_forces(mode, r, v, m)
        ref = oracle_accel(mode, r, m, G_DEFAULT, rows=rows)
        err = oracle.rel_err_per_body(a[rows], ref)
        assert err.max() < 1e-5, (mode, err.max())


def fp64_forces_gpu(r, m):
    """Every body's acceleration in the GPU FP64 mode (itself pinned to the oracle at
    1e-12 by the small-N, golden-vector and sampled tests of this module)."""
    a, _ = engine_forces('fp64', r, np.zeros_like(r), m)
    return a


@pytest.mark.parametrize('mode,n,seed', [('fp32un', 65536, 0), ('fp32n', 8192, 0),
                                         ('fp32n', 4096, 3), ('fp32un', 16384, 1)])
def test_default_float32_every_body_fp64_state(gpu, mode, n, seed):
    """The float32 near-corrected modes (the plugin default: fp32n below 4608 bodies,
    fp32un from there; fp32n also at 8192) on the FP64 state itself: every body within 1e-5 of the FP64 forces (bodies of the uniform
    cube sit up to 1000 from the origin, where rounding a coordinate to FP32 moves it by
    up to 3e-5: the plain FP32 modes exceed 1e-5 on ~0.2 % of the bodies there)."""
    r, v, m = uniform_cube(n, seed=seed)
    a64 = fp64_forces_gpu(r, m)
    rows = np.random.default_rng(seed + 5).choice(n, 16, replace=False)
    ref = oracle.accel_fp64(r, G_DEFAULT * m, 1.0, rows=rows, coincident=True)
    assert oracle.rel_err_per_body(a64[rows], ref).max() < 1e-12
    a, eng = engine_forces(mode, r, v, m)
    err = oracle.rel_err_per_body(a, a64)
    assert err.max() < 1e-5, (mode, n, err.max(), int((err > 1e-5).sum()))
    assert np.array_equal(eng.forces().cpu().numpy(), a)     # deterministic
    # the plain FP32 mode of the same arithmetic, for contrast: only its tail is wrong
    plain = {'fp32un': 'fp32u', 'fp32n': 'fp32'}[mode]
    a_plain, _ = engine_forces(plain, r, v, m)
    e_plain = oracle.rel_err_per_body(a_plain, a64)
    assert np.median(e_plain) < 1e-5
    assert err.max() <= e_plain.max()


def test_size_independent_properties_65536(gpu):
    n = 65536
    r, v, m = uniform_cube(n, seed=0)
    a1, eng = engine_forces('fp32', r, v, m)
    a2 = eng.forces().cpu().numpy()
    assert np.array_equal(a1, a2)                         # deterministic
    # momentum: sum_i m_i a_i = 0 (pairwise antisymmetry), relative to sum m|a|
    p = (m[:, None] * a1).sum(0)
    assert np.linalg.norm(p) < 1e-6 * (m * np.linalg.norm(a1, axis=1)).sum()
    # tile shape does not change the answer beyond FP32 rounding
    t = tile_list('fp32')[0]
    a3, _ = engine_forces('fp32', r, v, m, tile=_lib.Tile(t.bpt, t.threads, t.jtile, 97))
    assert oracle.rel_err_per_body(a3, a1).max() < 2e-6


def test_unique_pairs_matches_all_pairs_65536(gpu):
    """The unique-pair kernel (fp32u) against the all-pairs kernel (fp32) at N = 65536:
    same FP32 arithmetic per pair, different summation order."""
    n = 65536
    r, v, m = uniform_cube(n, seed=0)
    rows = np.random.default_rng(19).choice(n, 256, replace=False)
    ref = oracle_accel('fp32u', r, m, G_DEFAULT, rows=rows)
    a_all, _ = engine_forces('fp32', r, v, m)
    a_u, eng = engine_forces('fp32u', r, v, m)
    # both within 1e-5 of the FP64 oracle, hence within 1e-5 of each other
    assert oracle.rel_err_per_body(a_u, a_all).max() < 1e-5
    assert np.array_equal(a_u, eng.forces().cpu().numpy())   # deterministic
    p = (m[:, None] * a_u).sum(0)
    assert np.linalg.norm(p) < 1e-6 * (m * np.linalg.norm(a_u, axis=1)).sum()
    for t in tile_list('fp32u'):
        a_t, _ = engine_forces('fp32u', r, v, m, tile=_lib.Tile(t.bpt, t.threads, t.jtile, 0))
        assert oracle.rel_err_per_body(a_t[rows], ref).max() < 1e-5, t
        assert oracle.rel_err_per_body(a_t, a_all).max() < 1e-5, t


def test_plummer_pair_precision_modes(gpu):
    """Clustered input far from the origin: fp32c and fp64 hold their bounds on the
    FP64 state; plain fp32 holds its bound on the positions it reads."""
    n = 4096
    r, v, m = plummer_pair(n, seed=2)
    rows = np.arange(0, n, 16)
    for mode in ALL_MODES:
        a, _ = engine_forces(mode, r, v, m)
        ref = oracle_accel(mode, r, m, G_DEFAULT, rows=rows)
        err = oracle.rel_err_per_body(a[rows], ref).max()
        assert err < TOL[mode], (mode, err)


def test_edge_cases(gpu):
    # two bodies: analytic
    r = np.array([[0.0, 0, 0], [3.0, 4.0, 0]])
    m = np.array([2.0, 5.0]) / G_DEFAULT
    for mode in ('fp32', 'fp64'):
        a, _ = engine_forces(mode, r, np.zeros((2, 3)), m)
        d = np.array([3.0, 4.0, 0]) / 125.0
        assert np.allclose(a[0], 5.0 * d, rtol=1e-6) and np.allclose(a[1], -2.0 * d, rtol=1e-6)
    # coincident bodies exert no force on each other (the reference gives inf/nan)
    r = np.array([[0.0, 0, 0], [1.0, 0, 0], [1.0, 0, 0]])
    m = np.ones(3) / G_DEFAULT
    for mode in ALL_MODES:
        a, _ = engine_forces(mode, r, np.zeros((3, 3)), m)
        assert np.all(np.isfinite(a))
        assert np.allclose(a[1], [-1.0, 0, 0], rtol=1e-6)
        assert np.allclose(a[0], [2.0, 0, 0], rtol=1e-6)
    # coincident bodies far apart in the body order (different row blocks of the
    # unique-pair kernel, so they meet on its unique-pair path, not the diagonal one)
    r, v, m = uniform_cube(5000, seed=31)
    r[4321] = r[7]
    for mode in ALL_MODES:
        a, _ = engine_forces(mode, r, v, m)
        assert np.all(np.isfinite(a)), mode
        ref = oracle_accel(mode, r, m, G_DEFAULT, rows=np.array([7, 4321, 0]))
        assert oracle.rel_err_per_body(a[[7, 4321, 0]], ref).max() < TOL[mode], mode
    # two bodies 1e-3 apart at x = 1000, where FP32 resolves 6.1e-5: the near modes
    # take their separation from the double-single positions (within FP32 rounding of the
    # exact force); the plain modes see the FP32-rounded separation
    r = np.array([[1000.0, 0, 0], [1000.001, 0, 0], [-1000.0, 0.0, 0]])
    m = np.array([1.0, 2.0, 3.0]) / G_DEFAULT
    ref = oracle.accel_fp64(r, G_DEFAULT * m, 1.0, coincident=True)
    for mode in ('fp32n', 'fp32un', 'fp32c', 'fp32cu'):
        a, _ = engine_forces(mode, r, np.zeros((3, 3)), m)
        assert oracle.rel_err_per_body(a, ref).max() < 1e-5, mode
    a, _ = engine_forces('fp32', r, np.zeros((3, 3)), m)
    assert oracle.rel_err_per_body(a, ref)[:2].max() > 1e-3
    # closer than the FP32 resolution of their coordinates: the FP32 separation is
    # exactly zero, and such a pair contributes nothing in every FP32 mode but the
    # double-single ones
    r = np.array([[1000.0, 0, 0], [1000.00001, 0, 0], [0.0, 10.0, 0]])
    ref = oracle.accel_fp64(r32(r), G_DEFAULT * m, 1.0, coincident=True)
    for mode in ('fp32n', 'fp32un', 'fp32', 'fp32u'):
        a, _ = engine_forces(mode, r, np.zeros((3, 3)), m)
        assert np.all(np.isfinite(a)), mode
        assert oracle.rel_err_per_body(a, ref).max() < 1e-5, mode
    # massless bodies feel forces but exert none
    r, v, m = uniform_cube(100, seed=3)
    m[::3] = 0.0
    a, _ = engine_forces('fp64', r, v, m)
    ref = oracle.accel_fp64(r, G_DEFAULT * m, 1.0)
    assert oracle.rel_err_per_body(a, ref).max() < 1e-12
    # negative masses are rejected on the host
    with pytest.raises(ValueError):
        engine_forces('fp32', r, v, -m)


def test_batched_matches_single(gpu):
    """Several universes in one persistent launch == each universe alone."""
    sizes = [64, 1000, 3, 4096, 517]
    rs, vs, ms = zip(*[uniform_cube(n, seed=50 + i) for i, n in enumerate(sizes)])
    for mode in ('fp32', 'fp32u', 'fp32n', 'fp32un', 'fp64'):
        eng = Engine(sizes, [1e3] * len(sizes), mode=mode)
        eng.set_state(np.concatenate(rs), np.concatenate(vs), G_DEFAULT * np.concatenate(ms))
        a = eng.forces().cpu().numpy()
        for u, n in enumerate(sizes):
            ref = oracle_accel(mode, rs[u], ms[u], G_DEFAULT)
            err = oracle.rel_err_per_body(a[eng.universe_slice(u)], ref).max()
            assert err < TOL[mode], (mode, u, err)
        eng.step(3)
        eng.raise_on_device_error()


@pytest.mark.parametrize('mode', ALL_MODES)
def test_empty_and_ragged_batches(gpu, mode):
    """Universes without bodies anywhere in a batch (first, between, last) take no rows
    and leave the others' answers unchanged; batches of nothing but empty universes step
    without a launch error (stage 1 and stage 2 then launch nothing)."""
    sizes = [0, 5, 0, 1, 300, 0, 2, 0]
    parts = [uniform_cube(n, seed=110 + i) for i, n in enumerate(sizes)]
    r = np.concatenate([p[0] for p in parts])
    v = np.concatenate([p[1] for p in parts])
    m = np.concatenate([p[2] for p in parts])
    eng = Engine(sizes, 1e3, mode=mode)
    eng.set_state(r, v, G_DEFAULT * m)
    a = eng.forces().cpu().numpy()
    eng.raise_on_device_error()
    for u, n in enumerate(sizes):
        sl = eng.universe_slice(u)
        assert a[sl].shape[0] == n
        if n < 2:
            assert np.all(a[sl] == 0.0)
            continue
        ref = oracle_accel(mode, parts[u][0], parts[u][2], G_DEFAULT)
        assert oracle.rel_err_per_body(a[sl], ref).max() < TOL[mode], (mode, u)
    eng.step(2)
    out = eng.energy(G_DEFAULT)
    assert np.all(np.isfinite(out))
    eng.raise_on_device_error()
    for empty in ([0], [0, 0, 0]):
        e = Engine(empty, 1e3, mode=mode)
        e.set_state(np.zeros((0, 3)), np.zeros((0, 3)), np.zeros(0))
        assert e.forces().shape[0] == 0
        e.step(2)
        torch.cuda.synchronize()
        e.raise_on_device_error()


@pytest.mark.parametrize('mode', ['fp32u', 'fp32', 'fp32un'])
def test_maximum_size_2_20(gpu, mode):
    """N = 2^20 bodies in one universe (one step is 1.1e12 interactions; the unique-pair
    plan holds ~525k partial-sum slots): sampled bodies against the FP64 oracle, the
    total momentum change, and determinism of a repeated evaluation on those bodies."""
    n = 1 << 20
    r, v, m = uniform_cube(n, seed=4)
    rows = np.random.default_rng(20).choice(n, 48, replace=False)
    a, eng = engine_forces(mode, r, v, m)
    ref = oracle_accel(mode, r, m, G_DEFAULT, rows=rows)
    assert oracle.rel_err_per_body(a[rows], ref).max() < TOL[mode]
    assert np.all(np.isfinite(a))
    p = (m[:, None] * a).sum(0)
    assert np.linalg.norm(p) < 1e-5 * (m * np.linalg.norm(a, axis=1)).sum()
    assert np.array_equal(eng.forces().cpu().numpy()[rows], a[rows])


@pytest.mark.parametrize('n', [1024, 4096])
def test_matches_reference_gpu_kernel(gpu, n):
    """The reference's own GPU kernel (pc2's update_all, pc2.py:59-91, compiled for
    sm_103a from the reference's source where the reference tree exists) run on the same
    GB300 on the same inputs: both are within 1e-5 of the FP64 oracle and within 2e-5 of
    each other on every body, in fp32 and fp32u."""
    from oracle import refgpu
    if not refgpu.available(n):
        pytest.skip('pc2 cubin not built (the reference tree is not on this host)')
    r, v, m = uniform_cube(n, seed=0)
    f32 = dict(dtype=torch.float32, device='cuda')
    cols = [torch.tensor(r[:, k], **f32) for k in range(3)]
    acc = [torch.zeros(n, **f32) for _ in range(3)]
    mm = torch.tensor(m, **f32)
    k = refgpu.Pc2Kernel(n)
    k.launch(*(t.data_ptr() for t in cols), *(t.data_ptr() for t in acc), mm.data_ptr(),
             torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    k.close()
    a_pc2 = torch.stack(acc, 1).double().cpu().numpy()
    ref = oracle_accel('fp32', r, m, G_DEFAULT)
    assert oracle.rel_err_per_body(a_pc2, ref).max() < 1e-5
    for mode in ('fp32', 'fp32u'):
        a, _ = engine_forces(mode, r, v, m)
        assert oracle.rel_err_per_body(a, ref).max() < 1e-5, mode
        assert oracle.rel_err_per_body(a, a_pc2).max() < 2e-5, mode


def test_energy_momentum_fp64(gpu):
    """Energy and momentum of every universe of a batch against the FP64 oracle."""
    sizes = [2, 300, 1500, 77]
    rs, vs, ms = zip(*[uniform_cube(n, seed=70 + i) for i, n in enumerate(sizes)])
    for mode in ('fp32', 'fp32u', 'fp64'):
        eng = Engine(sizes, 1e3, mode=mode)
        eng.set_state(np.concatenate(rs), np.concatenate(vs), G_DEFAULT * np.concatenate(ms))
        out = eng.energy(G_DEFAULT)
        for u in range(len(sizes)):
            k, p, mom = oracle.energy_fp64(rs[u], vs[u], ms[u], G_DEFAULT)
            assert abs(out[u, 0] - k) <= 1e-12 * abs(k)
            assert abs(out[u, 1] - p) <= 1e-12 * abs(p)
            assert np.allclose(out[u, 2:5], mom, rtol=1e-12, atol=1e-12 * np.abs(ms[u]).sum())
        # a step in between and the diagnostic does not disturb the state
        eng.step(2)
        out2 = eng.energy(G_DEFAULT)
        assert np.all(np.isfinite(out2))


@pytest.mark.parametrize('mode', ['fp32', 'fp32n', 'fp32un'])
def test_graph_replay_matches_launches(gpu, mode):
    """The CUDA-graph step replays exactly what the launched steps compute."""
    sizes = [300, 64, 2000, 9000]
    rs, vs, ms = zip(*[uniform_cube(n, seed=90 + i) for i, n in enumerate(sizes)])
    r, v, gm = np.concatenate(rs), np.concatenate(vs), G_DEFAULT * np.concatenate(ms)
    a = Engine(sizes, 1e3, mode=mode)
    a.set_state(r, v, gm)
    a.step(4)
    b = Engine(sizes, 1e3, mode=mode, tile=a.tile)
    b.set_state(r, v, gm)
    g = b.capture_graph(2)
    g.replay()
    g.replay()
    torch.cuda.synchronize()
    assert torch.equal(a.r, b.r) and torch.equal(a.v, b.v)


def test_context_usable_after_many_launches(gpu):
    r, v, m = uniform_cube(2048, seed=1)
    eng = Engine([2048], 1e3, mode='fp32')
    eng.set_state(r, v, G_DEFAULT * m)
    eng.step(50)
    torch.cuda.synchronize()
    eng.raise_on_device_error()
    assert torch.isfinite(eng.r).all()


def test_plummer_pair_default_mode_every_body(gpu):
    """The precision-stress configuration (two Plummer spheres, N = 16384, seed 2): the
    float32 default (fp32un) at the first step, every body within 1e-5 of the FP64
    forces of the FP64 state; the FP64 mode pinned to the oracle on sampled bodies."""
    n = 16384
    r, v, m = plummer_pair(n, seed=2)
    a64 = fp64_forces_gpu(r, m)
    rows = np.random.default_rng(2).choice(n, 24, replace=False)
    ref = oracle.accel_fp64(r, G_DEFAULT * m, 1.0, rows=rows, coincident=True)
    assert oracle.rel_err_per_body(a64[rows], ref).max() < 1e-12
    a, _ = engine_forces('fp32un', r, v, m)
    assert oracle.rel_err_per_body(a, a64).max() < 1e-5


def test_precision_workload_short(gpu):
    """The precision workload (shortened): errors over every body against the GPU FP64
    forces at the first and last step, energy and momentum drift recorded."""
    from gravitation_gb300.workloads import run_precision
    out = run_precision(n=2048, steps=20, every=10, modes=('fp32un', 'fp32u', 'fp64'))
    assert out['fp32un']['accel_err_first'] < 1e-5
    assert out['fp32un']['accel_err_last'] < 1e-5
    assert out['fp32un']['bodies_above_1e-5_first'] == 0
    assert out['fp64']['accel_err_first'] < 1e-12
    for mode in ('fp32un', 'fp32u', 'fp64'):
        assert np.isfinite(out[mode]['energy_drift_max'])
        assert out[mode]['momentum_drift_max'] < 1e-9
