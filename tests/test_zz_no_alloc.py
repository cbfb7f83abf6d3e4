"""GPU test of grav_forces_noalloc, the entry point for callers that cannot allocate
device memory where they need forces (code inside another framework's memory pool,
threads that must not enter the CUDA allocator, hosts that reserve all device memory up
front).  It keeps its scratch in a fixed device array inside the library, so this test
checks that calls in a row -- the largest size the entry point accepts, then smaller
ones, so that anything left over from an earlier call would show -- give the same
accelerations as the regular entry points (grav_stage1 + grav_stage2 through the
Engine), within the tolerance the other tests allow between tile shapes; that a call
after the first allocates no device memory (free device memory and the PyTorch
allocator's counters unchanged across it); that a caller's error flag is left as the
caller set it; and that sizes above the limit are refused.

The file is named to be collected last; it passes alone in a fresh process (its first
call does the per-device set-up) and after the other tests.
"""

import ctypes

import numpy as np
import pytest
import torch

import oracle
from gravitation_gb300 import _lib
from gravitation_gb300.engine import Engine
from gravitation_gb300.scenarios import G_DEFAULT, uniform_cube

pytestmark = pytest.mark.gpu


def device_memory_state():
    """Free device memory (cudaMemGetInfo) and the PyTorch caching allocator's counters."""
    torch.cuda.synchronize()
    st = torch.cuda.memory_stats()
    return (torch.cuda.mem_get_info()[0], st.get('allocated_bytes.all.current', 0),
            st.get('reserved_bytes.all.current', 0), st.get('num_alloc_retries', 0))


def forces_noalloc(r, gm, err_init=0, check_no_alloc=False):
    """Accelerations through grav_forces_noalloc (every buffer allocated before the
    call).  With check_no_alloc the device-memory state is compared across the call."""
    L = _lib.load()
    n = len(gm)
    dev = torch.device('cuda', torch.cuda.current_device())
    rr = torch.zeros((n, 4), dtype=torch.float64, device=dev)
    rr[:, :3] = torch.as_tensor(r, dtype=torch.float64)
    rr[:, 3] = torch.as_tensor(gm, dtype=torch.float64)
    a = torch.full((n, 4), float('nan'), dtype=torch.float64, device=dev)
    err = torch.full((1,), err_init, dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream(dev)
    before = device_memory_state() if check_no_alloc else None
    _lib.check(L.grav_forces_noalloc(rr.data_ptr(), a.data_ptr(), n, float(np.max(gm)),
                                     err.data_ptr(), ctypes.c_void_p(stream.cuda_stream)))
    stream.synchronize()
    if check_no_alloc:
        assert device_memory_state() == before
    # the call never clears the caller's flag: it holds what the caller put there
    assert int(err.item()) == err_init
    return a[:, :3].cpu().numpy(), a[:, 3].cpu().numpy()


def forces_regular(r, gm):
    eng = Engine([len(gm)], 1e3, mode='fp32')
    eng.set_state(r, np.zeros_like(r), gm)
    a = eng.forces().cpu().numpy()
    eng.raise_on_device_error()
    return a


def test_noalloc_matches_regular_entry_points_twice(gpu):
    sizes = ((_lib.GRAV_NOALLOC_MAX_N, 10), (5000, 11), (3001, 12))
    for n, seed in sizes:
        r, _, m = uniform_cube(n, seed=seed)
        gm = G_DEFAULT * m
        # a repeated call of the same size runs the kernels the first one loaded, so
        # nothing at all may be allocated by it
        forces_noalloc(r, gm)
        a_na, w = forces_noalloc(r, gm, err_init=0, check_no_alloc=True)
        assert np.all(w == 0.0)
        a_reg = forces_regular(r, gm)
        # both FP32 stage 1 with FP64 sums, different tile and grid
        assert oracle.rel_err_per_body(a_na, a_reg).max() < 2e-6, n
        gm32 = gm.astype(np.float32).astype(np.float64)
        ref = oracle.accel_fp64(r.astype(np.float32).astype(np.float64), gm32, 1.0,
                                coincident=True)
        assert oracle.rel_err_per_body(a_na, ref).max() < 1e-5, n


def test_noalloc_leaves_the_callers_error_flag(gpu):
    """A flag the caller already set (say by earlier work sharing it) stays set."""
    r, _, m = uniform_cube(700, seed=13)
    gm = G_DEFAULT * m
    a_na, _ = forces_noalloc(r, gm, err_init=_lib.GRAV_DEV_TIMEOUT)
    a_reg = forces_regular(r, gm)
    assert oracle.rel_err_per_body(a_na, a_reg).max() < 2e-6


def test_noalloc_refuses_sizes_above_the_limit(gpu):
    L = _lib.load()
    n = _lib.GRAV_NOALLOC_MAX_N + 1
    assert L.grav_forces_noalloc(None, None, n, 1.0, None, None) == _lib.GRAV_E_SIZE
    assert '16384' in _lib.last_error()
