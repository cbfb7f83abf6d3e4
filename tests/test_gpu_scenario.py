"""GPU tests of the scenario generator (grav_scenario_generate) against the oracle's
restatement: uniform-derived values bit for bit, values through log/exp/sin/cos/expm1
to a few ulp, the Plummer centre-of-mass sums (a fixed tree on the device, body order
on the CPU) to rounding; determinism, host-resident targets, batches through the
engine, and universes started from a scenario through the plugin."""

import numpy as np
import pytest
import torch

import oracle
from gravitation_gb300 import generate
from gravitation_gb300.engine import Engine
from gravitation_gb300.kernel import gb1
from gravitation_gb300.scenarios import G_DEFAULT

pytestmark = pytest.mark.gpu

GAL = [1e20, 4e40, 2e30, 1e-10, 1e-30]
G_GAL = G_DEFAULT * 1e-10 ** 3 / 1e-30


def on_device(parts, G, n=None):
    n = generate.total_bodies(parts) if n is None else n
    r = torch.full((n, 4), float('nan'), dtype=torch.float64, device='cuda')
    v = torch.full((n, 4), float('nan'), dtype=torch.float64, device='cuda')
    generate.generate(parts, r, v, G)
    torch.cuda.synchronize()
    return r.cpu().numpy(), v.cpu().numpy()


def on_cpu(parts, G):
    n = generate.total_bodies(parts)
    r, v = np.zeros((n, 4)), np.zeros((n, 4))
    for p in parts:
        pr, pv = oracle.scenario(p.kind, p.n, p.seed, p.stream, G, p.params)
        r[p.offset:p.offset + p.n], v[p.offset:p.offset + p.n] = pr, pv
    return r, v


@pytest.mark.parametrize('n', [1, 2, 3, 255, 257, 4099, 262145])
def test_cube_matches_oracle(gpu, n):
    parts = generate.uniform_cube(n, seed=11, stream=3)
    r, v = on_device(parts, G_DEFAULT)
    r0, v0 = on_cpu(parts, G_DEFAULT)
    assert np.array_equal(r, r0)                       # positions and G*m: bit for bit
    assert np.array_equal(v[:, 3], v0[:, 3])
    np.testing.assert_allclose(v[:, :3], v0[:, :3], rtol=1e-14, atol=1e-15)


@pytest.mark.parametrize('n', [1, 2, 5, 1000, 70001])
def test_plummer_matches_oracle(gpu, n):
    parts = [generate.Part('plummer', n, 9, 1, (50.0, 0.1, 1000.0, -500, 20, 0, 2.5, 0, -1))]
    r, v = on_device(parts, G_DEFAULT)
    r0, v0 = on_cpu(parts, G_DEFAULT)
    np.testing.assert_allclose(r[:, 3], r0[:, 3], rtol=1e-15, atol=0)
    # relative to the sphere's scale (radius 50 around x = -500) and speeds (~1e-3)
    assert np.abs(r[:, :3] - r0[:, :3]).max() < 1e-11
    assert np.abs(v[:, :3] - v0[:, :3]).max() < 1e-15
    assert np.all(v[:, 3] == 0)


@pytest.mark.parametrize('n', [1, 2, 6, 300, 5001])
def test_galaxy_matches_oracle(gpu, n):
    parts = generate.galaxy(n, seed=5)
    r, v = on_device(parts, G_GAL)
    r0, v0 = on_cpu(parts, G_GAL)
    assert np.array_equal(r[:, 3], r0[:, 3])
    assert oracle.rel_err_per_body(r[:, :3], r0[:, :3]).max() < 4e-15
    assert oracle.rel_err_per_body(v[:, :3], v0[:, :3]).max() < 4e-15


def test_galaxy_matches_reference_create_galaxy(gpu, golden):
    n = len(golden['galdev_m'])
    G = float(golden['galdev_G'])
    r, v = on_device(generate.galaxy(n, seed=int(golden['galdev_seed']),
                                     stream=int(golden['galdev_stream'])), G)
    assert oracle.rel_err_per_body(r[:, :3], golden['galdev_r']).max() < 1e-14
    assert oracle.rel_err_per_body(v[1:, :3], golden['galdev_v'][1:]).max() < 1e-14
    assert np.array_equal(r[:, 3], G * golden['galdev_m'])


def test_deterministic_and_prefix_stable(gpu):
    parts = generate.plummer_pair(20000, seed=2)
    a = on_device(parts, G_DEFAULT)
    b = on_device(parts, G_DEFAULT)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    big = on_device(generate.uniform_cube(300000, seed=1), 1.0)
    small = on_device(generate.uniform_cube(1000, seed=1), 1.0)
    assert np.array_equal(big[0][:1000], small[0]) and np.array_equal(big[1][:1000], small[1])


def test_host_resident_target(gpu):
    """The device writes straight into pinned host memory (grav_host_device_pointer)."""
    parts = generate.plummer_pair(3001, seed=7)
    hr = torch.zeros((3001, 4), dtype=torch.float64, pin_memory=True)
    hv = torch.zeros((3001, 4), dtype=torch.float64, pin_memory=True)
    generate.generate(parts, hr, hv, G_DEFAULT)
    torch.cuda.synchronize()
    r, v = on_device(parts, G_DEFAULT)
    assert np.array_equal(hr.numpy(), r) and np.array_equal(hv.numpy(), v)


def test_engine_batch_generate_and_forces(gpu):
    sizes = [700, 64, 3001]
    scen = [generate.uniform_cube(700, seed=0, stream=0),
            generate.galaxy(64, seed=1),
            generate.plummer_pair(3001, seed=2, stream=5)]
    Gs = [G_DEFAULT, G_GAL, G_DEFAULT]
    eng = Engine(sizes, [1e3, 2e12, 1e3], mode='fp32u')
    eng.generate_state(scen, Gs)
    a = eng.forces().cpu().numpy()
    torch.cuda.synchronize()
    eng.raise_on_device_error()
    r = eng.r.cpu().numpy()
    for u, parts in enumerate(scen):
        sl = eng.universe_slice(u)
        r0, v0 = on_cpu(parts, Gs[u])
        np.testing.assert_allclose(r[sl], r0, rtol=1e-13, atol=1e-11)
        ref = oracle.accel_fp64(r0[:, :3], r0[:, 3], 1.0)
        assert oracle.rel_err_per_body(a[sl], ref).max() < 1e-4


def test_plugin_universe_from_scenario(gpu):
    u = gb1.universe(scenario={'kind': 'plummer_pair', 'n': 2001, 'seed': 3})
    u.start()
    assert len(u) == 2001
    r0, v0 = on_cpu(generate.plummer_pair(2001, seed=3), u._G)
    pms = list(u)
    assert pms[0]._name == 'plummer 0' and pms[2000]._name == 'plummer 2000'
    got = np.array([[float(c) for c in pm._r] for pm in pms])
    assert np.abs(got - r0[:, :3]).max() < 1e-11
    assert abs(pms[10]._m * u._G / r0[10, 3] - 1) < 1e-15
    u.step()
    a = oracle.accel_fp64(r0[:, :3], r0[:, 3], 1.0)
    r1, _ = oracle.stage2_fp64(r0[:, :3], v0[:, :3], a, u._T)
    got = np.array([[float(c) for c in pm._r] for pm in u])
    # FP32 pair terms: the error of the step is a small fraction of its force part a T^2
    err = np.linalg.norm(got - r1, axis=1)
    bound = 1e-4 * np.linalg.norm(a, axis=1) * u._T ** 2 + 1e-12 * np.linalg.norm(r1, axis=1)
    assert np.all(err <= bound)
    u.stop()
    with pytest.raises(ValueError):
        w = gb1.universe(scenario={'kind': 'uniform_cube', 'n': 10})
        w.add_object(name='x', r=[0.0, 0, 0], v=[0.0, 0, 0], m=1.0)
        w.start()


def test_plugin_galaxy_with_reference_scaling(gpu):
    params = generate.galaxy_universe_params()
    u = gb1.universe(scenario={'kind': 'galaxy', 'n': 1000, 'seed': 8}, **params)
    u.start()
    assert u._G == G_GAL
    r0, _ = on_cpu(generate.galaxy(1000, seed=8), u._G)
    got = np.array([[float(c) for c in pm._r] for pm in u])
    assert oracle.rel_err_per_body(got, r0[:, :3]).max() < 4e-15
    u.step()
    u.stop()
