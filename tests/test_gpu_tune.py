"""GPU test of the tile autotuner: it times full steps over tiles and grid sizes, caches
the fastest, and the cached choice drives a correct step."""

import ctypes

import numpy as np
import pytest

import oracle
from gravitation_gb300 import _lib
from gravitation_gb300.engine import Engine, device_info
from gravitation_gb300.scenarios import G_DEFAULT, uniform_cube
from gravitation_gb300.tune import Tuner

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize('mode,n', [('fp32', 3000), ('fp32u', 9000), ('fp32n', 3000), ('fp32un', 9000)])
def test_tune_caches_a_valid_choice(gpu, tmp_path, mode, n):
    info = device_info(0)
    t = Tuner(str(tmp_path / 'cache.json'))
    tile = t.tune(mode, [n], info, reps=2)
    L = _lib.load()
    assert L.grav_tile_supported(_lib.MODES[mode], ctypes.byref(tile))
    assert tile.grid >= 1
    again = Tuner(str(tmp_path / 'cache.json')).choose(mode, [n], info, tune_if_missing=False)
    assert (again.bpt, again.threads, again.jtile, again.grid) == (
        tile.bpt, tile.threads, tile.jtile, tile.grid)
    r, v, m = uniform_cube(n, seed=21)
    eng = Engine([n], 1e3, mode=mode, tile=again)
    # the cached grid is the one tried; each plan caps it at its own number of units
    assert eng.info.grid == min(tile.grid, eng.info.n_units)
    eng.set_state(r, v, G_DEFAULT * m)
    a = eng.forces().cpu().numpy()
    eng.raise_on_device_error()
    rows = np.arange(0, n, 97)
    ref = oracle.accel_fp64(r, G_DEFAULT * m, 1.0, rows=rows)
    assert oracle.rel_err_per_body(a[rows], ref).max() < 1e-5
