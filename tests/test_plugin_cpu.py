"""CPU tests of the drop-in boundary: the kernel package's metadata is what the
reference's AST loader reads, the reference's own inventory discovers and imports it
from a copy of the reference tree, and the stand-alone universe_base restatement
behaves like the reference's class (scaling, state machine, default stage 2)."""

import ast
import os
import shutil
import subprocess
import sys
import textwrap

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GB1 = os.path.join(ROOT, 'gravitation_gb300', 'kernel', 'gb1')
from oracle.build import REF_ROOT as REF  # noqa: E402  (the reference tree, if present)
REF_SRC = os.path.join(REF, 'src')
META = ('longname', 'version', 'description', 'requirements', 'externalrequirements',
        'interpreters', 'parallel', 'license', 'authors')


def test_metadata_is_literal():
    tree = ast.parse(open(os.path.join(GB1, '__init__.py')).read())
    found = {}
    for item in tree.body:
        if isinstance(item, ast.Assign):
            for t in item.targets:
                # the reference's loader reads target.id of every top-level assignment
                assert isinstance(t, ast.Name)
                found[t.id] = ast.literal_eval(item.value)
    for k in META:
        assert '__%s__' % k in found, k
    assert found['__parallel__'] is True
    assert 'cuda' in found['__externalrequirements__']


@pytest.mark.skipif(not os.path.isdir(REF_SRC), reason='reference tree not present')
def test_reference_inventory_discovers_gb1(tmp_path):
    src = tmp_path / 'src'
    shutil.copytree(os.path.join(REF_SRC, 'gravitation'), src / 'gravitation',
                    ignore=shutil.ignore_patterns('__pycache__', '*.so'))
    shutil.copytree(GB1, src / 'gravitation' / 'kernel' / 'gb1',
                    ignore=shutil.ignore_patterns('__pycache__'))
    script = textwrap.dedent('''
        import sys, warnings
        warnings.simplefilter("ignore", DeprecationWarning)
        sys.path[:0] = [%r, %r]
        from gravitation.lib.load import inventory
        from gravitation.kernel._base_ import universe_base
        k = inventory["gb1"]
        k.load_meta()
        assert k["longname"].startswith("gb300"), k["longname"]
        assert k["name"] == "gb1"
        k.load_module()
        cls = k.get_class()
        assert issubclass(cls, universe_base), cls.__mro__
        assert cls.__module__ == "gravitation.kernel.gb1"
        u = cls(T=2.0e12, scale_m=1e-30, scale_r=1e-10)
        u.add_object(name="a", r=[1.0, 2.0, 3.0], v=[0.0, 0.0, 0.0], m=2e30)
        assert u._G == 6.6740831e-11 * 1e-30 / 1e-30
        print("OK", sorted(inventory.keys())[:3])
    ''' % (str(src), ROOT))
    res = subprocess.run([sys.executable, '-c', script], capture_output=True, text=True,
                         timeout=300)
    assert res.returncode == 0, res.stderr[-2000:]
    assert 'OK' in res.stdout


_FAKE_H5PY = open(os.path.join(ROOT, 'oracle', 'standins', 'h5py.py')).read()


@pytest.mark.skipif(not os.path.isdir(REF_SRC), reason='reference tree not present')
def test_reference_store_load_with_gb1(tmp_path):
    """The reference's own store_simulation / load_simulation (simulation.py:186-258,
    the worker's snapshot path, worker.py:138-155) run on gb1 universes: the state
    model they read and write (pm._name, pm._r, pm._v, pm._m and the universe's scale,
    time step and G attributes) is the reference's.  h5py itself is absent on both hosts,
    so an in-memory stand-in takes its place; the HDF5 file format is not exercised.  The
    reference's store also needs numpy's chararray, which numpy 2 keeps under np.char."""
    src = tmp_path / 'src'
    shutil.copytree(os.path.join(REF_SRC, 'gravitation'), src / 'gravitation',
                    ignore=shutil.ignore_patterns('__pycache__', '*.so'))
    shutil.copytree(GB1, src / 'gravitation' / 'kernel' / 'gb1',
                    ignore=shutil.ignore_patterns('__pycache__'))
    fake = tmp_path / 'fake'
    fake.mkdir()
    (fake / 'h5py.py').write_text(_FAKE_H5PY)
    script = textwrap.dedent('''
        import sys, warnings
        warnings.simplefilter("ignore", DeprecationWarning)
        sys.path[:0] = [%r, %r, %r]
        import numpy as np
        if not hasattr(np, "chararray"):
            # simulation.py:241 calls np.chararray, which numpy 2 moved to np.char
            np.chararray = np.char.chararray
        from gravitation.lib.load import inventory
        from gravitation.lib.simulation import store_simulation, load_simulation
        k = inventory["gb1"]
        k.load_meta()
        k.load_module()
        cls = k.get_class()
        rng = np.random.default_rng(5)
        u = cls(T=1.5e3, scale_m=1e-30, scale_r=1e-10, dtype="float32", t=7.0)
        for i in range(50):
            u.add_object(name="body %%d" %% i, r=list(rng.uniform(-1e12, 1e12, 3)),
                         v=list(rng.normal(0, 1e3, 3)), m=float(rng.uniform(1e29, 1e31)))
        fn = %r
        store_simulation(u, fn, "kernel=gb1;len=50;step=0")
        store_simulation(u, fn, "kernel=gb1;len=50;step=1")
        w = load_simulation(cls, fn, "kernel=gb1;len=50;step=1")
        assert type(w) is cls and len(w) == 50
        assert w._G == u._G and w._T == u._T and w._t == u._t
        assert w._scale_m == u._scale_m and w._scale_r == u._scale_r and w._dtype == u._dtype
        for a, b in zip(u, w):
            assert a._name == b._name
            # the store keeps the universe's dtype (float32 here), as the reference does
            assert np.allclose(np.float32(a._r), b._r, rtol=0) and np.float32(a._m) == b._m
            assert np.allclose(np.float32(a._v), b._v, rtol=0)
        print("OK")
    ''' % (str(fake), str(src), ROOT, str(tmp_path / 'sim.h5')))
    res = subprocess.run([sys.executable, '-c', script], capture_output=True, text=True,
                         timeout=300)
    assert res.returncode == 0, res.stderr[-2000:]
    assert 'OK' in res.stdout


def _ref_base():
    if not os.path.isdir(REF_SRC):
        pytest.skip('reference tree not present')
    import importlib.util
    spec = importlib.util.spec_from_file_location(
        '_ref_base_', os.path.join(REF_SRC, 'gravitation', 'kernel', '_base_.py'))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_base_restatement_matches_reference():
    ref = _ref_base()
    from gravitation_gb300.kernel import _base_ as ours
    for kw in ({}, {'scale_m': 1e-30, 'scale_r': 1e-10, 'T': 2e12},
               {'scale_m': 3.0, 'scale_r': 2.0, 'scale_off': True, 'foo': 1}):
        a = ref.universe_base(**dict(kw))
        b = ours.universe_base(**dict(kw))
        assert a._G == b._G and a._T == b._T and a._meta == b._meta
        for u in (a, b):
            u.add_object(name='x', r=[1.0, 2.0, 3.0], v=[0.5, 0.0, -1.0], m=7.0)
            u.add_object(name='y', r=[-1.0, 0.0, 3.0], v=[0.0, 0.0, 0.0], m=1.0, scale_off=True)
        for pa, pb in zip(a, b):
            assert pa._r == pb._r and pa._v == pb._v and pa._m == pb._m and pa._a == pb._a
            assert str(pa) == str(pb)
        # state machine
        for u in (a, b):
            with pytest.raises(SyntaxError):
                u.step()
            with pytest.raises(SyntaxError):
                u.stop()
            u.start()
            with pytest.raises(SyntaxError):
                u.start()
            with pytest.raises(SyntaxError):
                u.add_object(name='z', r=[0.0] * 3, v=[0.0] * 3, m=1.0)
            with pytest.raises(NotImplementedError):
                u.step()
        # default stage 2 on identical accelerations
        for u in (a, b):
            for i, pm in enumerate(u):
                pm._a[:] = [1e-3 * (i + 1), -2e-3, 3e-3]
            u.step_stage2()
            u.step_stage3()
        for pa, pb in zip(a, b):
            assert pa._r == pb._r and pa._v == pb._v and pa._a == pb._a
        assert a._t == b._t
        for u in (a, b):
            u.stop()
            with pytest.raises(SyntaxError):
                u.stop()


def test_default_precision_by_dtype_and_size():
    from gravitation_gb300 import build as gbuild
    gbuild.build()
    from gravitation_gb300.plugin import default_mode
    from gravitation_gb300.adjoint import default_adjoint_pairs
    from gravitation_gb300.engine import plan_part_bytes, tile_list
    from gravitation_gb300 import _lib
    gib = 1 << 30
    assert default_mode('float32', 1024) == 'fp32n'
    assert default_mode('float32', 65536) == 'fp32un'
    assert default_mode('float64', 65536) == 'fp64'
    assert default_mode('float16', 10) is None
    # the unique-pair slots grow as N^2 / rows-per-block; the all-pairs slots do not
    t = _lib.Tile(8, 128, 256, 456)
    assert plan_part_bytes([1 << 20], t, 'fp32u') > 12 * 10 ** 9
    assert plan_part_bytes([1 << 20], t, 'fp32') < 64 * 10 ** 6
    assert plan_part_bytes([1 << 22], t, 'fp32u') > 15 * plan_part_bytes([1 << 20], t, 'fp32u')
    assert plan_part_bytes([4096], t, 'fp32u', comps=7) * 3 == plan_part_bytes([4096], t, 'fp32u') * 7
    # beyond the slot budget float32 falls back to all pairs (forward and backward);
    # unique pairs stay while some compiled shape fits, and only those are candidates
    from gravitation_gb300.engine import fitting_tiles
    sizes = [1 << 20]
    per_tile = [plan_part_bytes(sizes, x, 'fp32un') for x in tile_list('fp32un')]
    best, worst = min(per_tile), max(per_tile)
    assert best < worst        # rows per block set the slots' N^2 / R growth
    assert default_mode('float32', 1 << 20, budget=best) == 'fp32un'
    assert default_mode('float32', 1 << 20, budget=best - 1) == 'fp32n'
    fit = fitting_tiles(sizes, 'fp32un', budget=best)
    assert fit and all(plan_part_bytes(sizes, x, 'fp32un') <= best for x in fit)
    assert len(fitting_tiles(sizes, 'fp32un', budget=worst)) == len(per_tile)
    assert len(fitting_tiles(sizes, 'fp32n', budget=1)) == len(tile_list('fp32n'))
    assert default_mode('float32', 1 << 23, budget=32 * gib) == 'fp32n'
    assert default_adjoint_pairs([4096], budget=32 * gib)
    assert not default_adjoint_pairs([4096], budget=1)
    assert not default_adjoint_pairs([1 << 22], budget=32 * gib)
    assert not default_adjoint_pairs([1024])


def test_default_stage2_matches_oracle():
    import oracle
    from gravitation_gb300.kernel._base_ import universe_base
    rng = np.random.default_rng(2)
    r, v, a = rng.normal(size=(5, 3)), rng.normal(size=(5, 3)), rng.normal(size=(5, 3))
    u = universe_base(T=123.0)
    for i in range(5):
        u.add_object(name='b', r=list(r[i]), v=list(v[i]), m=1.0)
    u.start()
    for i, pm in enumerate(u):
        pm._a[:] = list(a[i])
    u.step_stage2()
    r2, v2 = oracle.stage2_fp64(r, v, a, 123.0)
    assert np.array_equal(np.array([pm._r for pm in u]), r2)
    assert np.array_equal(np.array([pm._v for pm in u]), v2)


def test_reference_cli_loads_with_gb1_among_its_kernels(tmp_path):
    """The reference's command-line front end (staged in baseline/_ref) imports with the
    stand-ins of oracle/standins and offers gb1 as a kernel of its worker command."""
    from oracle import frontend
    ok, why = frontend.available()
    if not ok:
        pytest.skip(why)
    env = frontend.prepare(str(tmp_path))
    res = frontend.cli(env, ['worker', '--help'], 300, str(tmp_path))
    assert res.returncode == 0, res.stderr[-2000:]
    assert 'gb1' in res.stdout


def test_near_pair_fraction_picks_the_precision_mode():
    """float32 with positions known: the near-corrected modes for configurations with few
    near pairs (the uniform cube), double-single separations for every pair where near
    pairs are common (two dense clusters far from the origin)."""
    from gravitation_gb300 import build as gbuild
    gbuild.build()
    from gravitation_gb300.plugin import default_mode, near_pair_fraction, NEAR_DS_FRACTION
    from gravitation_gb300.scenarios import plummer_pair, uniform_cube
    cube = uniform_cube(16384, seed=0)[0]
    pair = plummer_pair(16384, seed=2)[0]
    assert near_pair_fraction(cube) < NEAR_DS_FRACTION < near_pair_fraction(pair)
    assert default_mode('float32', 16384, r=cube) == 'fp32un'
    assert default_mode('float32', 16384, r=pair) == 'fp32cu'
    assert default_mode('float32', 4096, r=pair[:4096]) == 'fp32c'
    assert default_mode('float64', 16384, r=pair) == 'fp64'
    assert near_pair_fraction(cube[:1]) == 0.0
