"""The reference's own GPU kernel (pc2's update_all, gravitation/kernel/pc2.py:59-91) run
on the GB300 from the cubin oracle/build.py compiles, through the CUDA driver API
(ctypes on libcuda; PyCUDA, which pc2 itself uses, is absent).

Test infrastructure: a comparator for parity tests and for timing beside the product's
kernels, never part of the product path.  The kernel takes FP32 columns rx, ry, rz, the
unscaled masses m, writes ax, ay, az = G * sum_{i != j} m_i d / |d|^3 (G and N are
compiled in), one thread per body, 256 threads per block, as pc2.py:133-162 launches it.
"""

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
THREADS = 256  # pc2.py:137


def cubin_path(n):
    return os.path.join(HERE, '_ref', 'pc2_n%d.cubin' % int(n))


def available(n):
    return os.path.exists(cubin_path(n))


class _Driver:
    _lib = None

    @classmethod
    def lib(cls):
        if cls._lib is None:
            L = ctypes.CDLL('libcuda.so.1')
            L.cuModuleLoad.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_char_p]
            L.cuModuleGetFunction.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_void_p,
                                              ctypes.c_char_p]
            L.cuLaunchKernel.argtypes = [ctypes.c_void_p] + [ctypes.c_uint] * 7 + [
                ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p), ctypes.c_void_p]
            L.cuModuleUnload.argtypes = [ctypes.c_void_p]
            L.cuCtxGetCurrent.argtypes = [ctypes.POINTER(ctypes.c_void_p)]
            L.cuGetErrorString.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_char_p)]
            cls._lib = L
        return cls._lib

    @classmethod
    def check(cls, rc, what):
        if rc != 0:
            msg = ctypes.c_char_p()
            cls.lib().cuGetErrorString(rc, ctypes.byref(msg))
            raise RuntimeError('%s: CUDA driver error %d (%s)' % (
                what, rc, (msg.value or b'?').decode()))


class Pc2Kernel:
    """pc2's update_all for N bodies; launch(rx, ry, rz, ax, ay, az, m, stream) takes
    device pointers (float32 arrays of N) and a CUstream handle (0: the legacy stream).
    A CUDA context must be current (torch's, once it has touched the device)."""

    def __init__(self, n):
        self.n = int(n)
        path = cubin_path(self.n)
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        L = _Driver.lib()
        ctx = ctypes.c_void_p()
        _Driver.check(L.cuCtxGetCurrent(ctypes.byref(ctx)), 'cuCtxGetCurrent')
        if not ctx.value:
            raise RuntimeError('no current CUDA context (touch the device with torch first)')
        self.mod = ctypes.c_void_p()
        _Driver.check(L.cuModuleLoad(ctypes.byref(self.mod), path.encode()), 'cuModuleLoad')
        self.fn = ctypes.c_void_p()
        _Driver.check(L.cuModuleGetFunction(ctypes.byref(self.fn), self.mod, b'update_all'),
                      'cuModuleGetFunction')
        self.blocks = -(-self.n // THREADS)  # pc2.py:138-140

    def launch(self, rx, ry, rz, ax, ay, az, m, stream=0):
        vals = [ctypes.c_void_p(int(p)) for p in (rx, ry, rz, ax, ay, az, m)]
        params = (ctypes.c_void_p * 7)(*[ctypes.cast(ctypes.pointer(v), ctypes.c_void_p)
                                         for v in vals])
        _Driver.check(_Driver.lib().cuLaunchKernel(
            self.fn, self.blocks, 1, 1, THREADS, 1, 1, 0, ctypes.c_void_p(int(stream)),
            params, None), 'cuLaunchKernel')

    def close(self):
        if self.mod:
            _Driver.lib().cuModuleUnload(self.mod)
            self.mod = ctypes.c_void_p()
