"""Failure detection without a GPU fault: a device-side wait that expires is reported to
the host through the device error flag, the host raises, and the context stays usable.
(Argument errors are covered on the CPU in test_abi_cpu.py: they are rejected before any
launch.)"""

import ctypes
import time

import numpy as np
import pytest
import torch

import oracle
from gravitation_gb300 import _lib
from gravitation_gb300.engine import Engine
from gravitation_gb300.scenarios import G_DEFAULT, uniform_cube

pytestmark = pytest.mark.gpu


def test_expired_wait_is_reported_and_context_survives(gpu):
    L = _lib.load()
    r, v, m = uniform_cube(500, seed=4)
    eng = Engine([500], 1e3, mode='fp32u')
    eng.set_state(r, v, G_DEFAULT * m)
    s = torch.cuda.current_stream()
    t0 = time.perf_counter()
    _lib.check(L.grav_wait_check(eng.err.data_ptr(), 50_000_000, ctypes.c_void_p(s.cuda_stream)))
    assert eng.device_error() == _lib.GRAV_DEV_TIMEOUT
    assert time.perf_counter() - t0 < 10.0
    with pytest.raises(_lib.GravError, match='bounded wait'):
        eng.raise_on_device_error()
    assert eng.device_error() == _lib.GRAV_DEV_OK          # cleared by the raise
    # the context is still usable: a normal step gives correct forces
    a = eng.forces().cpu().numpy()
    eng.raise_on_device_error()
    ref = oracle.accel_fp64(r.astype(np.float32).astype(np.float64),
                            (G_DEFAULT * m).astype(np.float32).astype(np.float64), 1.0,
                            coincident=True)
    assert oracle.rel_err_per_body(a, ref).max() < 1e-5


def test_wait_check_rejects_bad_arguments(gpu):
    L = _lib.load()
    assert L.grav_wait_check(None, 1000, None) == _lib.GRAV_E_ARG
    err = torch.zeros(1, dtype=torch.int32, device='cuda')
    assert L.grav_wait_check(err.data_ptr(), 0, None) == _lib.GRAV_E_ARG
    assert L.grav_wait_check(err.data_ptr(), 3_000_000_000, None) == _lib.GRAV_E_ARG
