"""CPU tests of the seeded scenario generator: the oracle's Philox4x64-10 against
numpy's own Philox bit generator, the galaxy restatement against the reference's own
create_galaxy (golden vectors), statistical properties of the cube and Plummer
restatements, host-side argument checks of grav_scenario_generate, and the plugin's
lazily built point-mass list."""

import ctypes

import numpy as np
import pytest

import oracle
from gravitation_gb300 import _lib, build as gbuild, generate
from gravitation_gb300.kernel._base_ import _point_mass
from gravitation_gb300.plugin import _MirrorMasses

U64 = 2 ** 64 - 1


def _minus_one(ctr):
    """Counter one below `ctr` (with borrow): numpy's Philox advances before a block."""
    c = [int(x) for x in ctr]
    for i in range(4):
        if c[i]:
            c[i] -= 1
            break
        c[i] = U64
    return np.array(c, dtype=np.uint64)


@pytest.mark.parametrize('key,ctr', [
    ([0, 0], [0, 0, 0, 0]),
    ([123456789, 42], [5, 7, 0, 0]),
    ([U64, 2 ** 63 + 11], [U64, 3, 0, 0]),
    ([0xDEADBEEF, 1], [17, U64, U64, 9]),
    ([2, 1], [65535, 33, 0, 0]),
])
def test_philox_matches_numpy(key, ctr):
    ref = np.random.Philox(key=np.array(key, dtype=np.uint64), counter=_minus_one(ctr))
    assert np.array_equal(oracle.philox4x64_10(ctr, key), ref.random_raw(4))


def test_uniform_conversion_matches_numpy():
    key, ctr = [7, 3], [100, 2, 0, 0]
    g = np.random.Generator(np.random.Philox(key=np.array(key, dtype=np.uint64),
                                             counter=_minus_one(ctr)))
    w = oracle.philox4x64_10(ctr, key)
    assert np.array_equal(g.random(4), (w >> np.uint64(11)).astype(np.float64) * 2.0 ** -53)


def test_galaxy_matches_reference_create_galaxy(golden):
    """The reference's create_galaxy, fed the generator's draws (make_golden.py), against
    the restatement: the reference's zero-angle rotations (atan2/cos/sin round trips,
    simulation.py:151-176) leave a few ulp."""
    n = len(golden['galdev_m'])
    G = float(golden['galdev_G'])
    r, v = oracle.scenario('galaxy', n, int(golden['galdev_seed']),
                           int(golden['galdev_stream']), G, [1e20, 4e40, 2e30, 1e-10, 1e-30])
    assert oracle.rel_err_per_body(r[:, :3], golden['galdev_r']).max() < 4e-15
    assert oracle.rel_err_per_body(v[1:, :3], golden['galdev_v'][1:]).max() < 4e-15
    assert np.array_equal(r[:, 3], G * golden['galdev_m'])
    assert np.array_equal(v[0], np.zeros(4))


def test_cube_properties():
    n = 200000
    r, v = oracle.scenario('uniform_cube', n, 0, 0, 2.0, [1000.0, 1.0, 1.0, 100.0])
    x = r[:, :3]
    assert x.min() >= -1000.0 and x.max() < 1000.0
    assert abs(x.mean()) < 5 * 1000 / np.sqrt(3 * 3 * n)
    assert abs(x.var() / (1000.0 ** 2 / 3) - 1) < 0.01
    m = r[:, 3] / 2.0
    assert m.min() >= 1.0 and m.max() < 100.0
    assert abs(v[:, :3].mean()) < 0.01 and abs(v[:, :3].var() - 1) < 0.01
    assert np.all(v[:, 3] == 0)
    # the first bodies do not depend on n (each body has its own counter)
    r2, v2 = oracle.scenario('uniform_cube', 1000, 0, 0, 2.0, [1000.0, 1.0, 1.0, 100.0])
    assert np.array_equal(r2, r[:1000]) and np.array_equal(v2, v[:1000])
    # another stream of the same seed is another sequence
    r3, _ = oracle.scenario('uniform_cube', 1000, 0, 1, 2.0, [1000.0, 1.0, 1.0, 100.0])
    assert not np.any(r3[:, 0] == r[:1000, 0])


def test_plummer_properties():
    n, a, G = 50000, 50.0, 6.6740831e-11
    c, cv = np.array([-500.0, 0, 0]), np.array([2.5, 0, 0])
    r, v = oracle.scenario('plummer', n, 2, 0, G, [a, 0.1, 1000.0, *c, *cv])
    gm = r[:, 3]
    assert np.all(gm > 0)
    com = (gm[:, None] * r[:, :3]).sum(0) / gm.sum()
    comv = (gm[:, None] * v[:, :3]).sum(0) / gm.sum()
    assert np.allclose(com, c, rtol=0, atol=1e-9 * a)
    assert np.allclose(comv, cv, rtol=0, atol=1e-12)
    # half-mass radius of a Plummer sphere: a / sqrt(2^(2/3) - 1) = 1.3048 a (by number,
    # since the masses are drawn independently of the radii)
    rad = np.linalg.norm(r[:, :3] - c, axis=1)
    assert abs(np.median(rad) / a / 1.3048 - 1) < 0.03
    # every body is bound: speed below the local escape speed of the sphere
    vesc = np.sqrt(2 * gm.sum() / a) * (1 + (rad / a) ** 2) ** -0.25
    speed = np.linalg.norm(v[:, :3] - cv, axis=1)
    assert np.quantile(speed / vesc, 0.999) < 1.0 + 1e-3


@pytest.fixture(scope='module')
def L():
    gbuild.build()
    return _lib.load()


def test_scenario_abi_checks_on_host(L):
    s = generate.uniform_cube(10)[0].struct(1.0)
    assert L.grav_scenario_scratch_bytes(ctypes.byref(s), 10) == 0
    # n = 0 is a no-op that needs no pointers
    assert L.grav_scenario_generate(ctypes.byref(s), None, None, 0, None, None) == _lib.GRAV_OK
    assert L.grav_scenario_generate(ctypes.byref(s), None, None, 10, None, None) == _lib.GRAV_E_ARG
    # misaligned rows
    assert L.grav_scenario_generate(ctypes.byref(s), ctypes.c_void_p(8), ctypes.c_void_p(64),
                                    10, None, None) == _lib.GRAV_E_ARG
    bad = generate.Part('uniform_cube', 10, 0, params=(1.0, 1.0, 5.0, 1.0)).struct(1.0)
    assert L.grav_scenario_generate(ctypes.byref(bad), ctypes.c_void_p(64), ctypes.c_void_p(128),
                                    10, None, None) == _lib.GRAV_E_ARG
    assert b'm_lo' in L.grav_last_error()
    p = generate.plummer_pair(1000)[0].struct(1.0)
    nb = L.grav_scenario_scratch_bytes(ctypes.byref(p), 500)
    assert nb == 2 * 8 * 8  # two CTAs of 256 bodies, 8 doubles each
    assert L.grav_scenario_generate(ctypes.byref(p), ctypes.c_void_p(64), ctypes.c_void_p(128),
                                    500, None, None) == _lib.GRAV_E_ARG
    assert b'scratch' in L.grav_last_error()
    unknown = _lib.Scenario()
    unknown.kind = 99
    assert L.grav_scenario_generate(ctypes.byref(unknown), ctypes.c_void_p(64),
                                    ctypes.c_void_p(128), 4, None, None) == _lib.GRAV_E_ARG
    nan = generate.galaxy(10)[0].struct(float('nan'))
    assert L.grav_scenario_generate(ctypes.byref(nan), ctypes.c_void_p(64), ctypes.c_void_p(128),
                                    10, None, None) == _lib.GRAV_E_ARG


def test_specs_and_parts():
    parts = generate.from_spec({'kind': 'plummer_pair', 'n': 1001, 'seed': 4})
    assert [(p.kind, p.n, p.offset, p.stream) for p in parts] == [
        ('plummer', 501, 0, 0), ('plummer', 500, 501, 1)]
    assert generate.total_bodies(parts) == 1001
    assert generate.from_spec({'kind': 'galaxy', 'n': 7})[0].params[:3] == [1e20, 4e40, 2e30]
    with pytest.raises(ValueError):
        generate.from_spec({'kind': 'torus', 'n': 7})


def test_mirror_masses_build_point_masses_on_access():
    n, G = 5, 2.0
    hr = np.arange(4 * n, dtype=np.float64).reshape(n, 4)
    hv = -hr
    ha = np.zeros((n, 4))
    mm = _MirrorMasses(_point_mass, hr, hv, ha, G, generate.uniform_cube(n))
    assert len(mm) == n and all(x is None for x in mm._items)
    pm = mm[2]
    assert pm._name == 'uniform_cube 2' and pm._m == hr[2, 3] / G
    assert list(pm._r) == list(hr[2, :3]) and list(pm._v) == list(hv[2, :3])
    pm._r[:] = [7.0, 8.0, 9.0]          # a view of the mirror
    assert list(hr[2, :3]) == [7.0, 8.0, 9.0]
    assert mm[2] is pm and mm[-1] is mm[4]
    assert [p._name for p in mm][:2] == ['uniform_cube 0', 'uniform_cube 1']
    assert len(mm[1:3]) == 2
