"""ctypes binding of libgravgb300.so (the C ABI declared in include/gravitation_gb300.h).

There is no fallback: if the library is missing or fails to load, every entry point
of this package raises.  Build it with ``python -m gravitation_gb300.build``.
"""

import ctypes
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, 'libgravgb300.so')

# ---- constants (mirror of the header) -------------------------------------------
GRAV_ABI_VERSION = 5
GRAV_OK = 0
GRAV_E_ARG = -1
GRAV_E_TILE = -2
GRAV_E_CUDA = -3
GRAV_E_SIZE = -4
GRAV_E_DEVICE = -5
GRAV_DEV_OK = 0
GRAV_DEV_TIMEOUT = 1
GRAV_MODE_FP32 = 0
GRAV_MODE_FP32C = 1
GRAV_MODE_FP64 = 2
GRAV_MODE_FP32U = 3
GRAV_S2_INTEGRATE = 1
GRAV_S2_WRITE_A = 2
GRAV_S2_PREPARE = 4

GRAV_MODE_FP32CU = 4
GRAV_MODE_FP32N = 5
GRAV_MODE_FP32UN = 6
GRAV_NEAR_KAPPA = 20
GRAV_FUSED_MAX_N = 4096
MODES = {'fp32': GRAV_MODE_FP32, 'fp32c': GRAV_MODE_FP32C, 'fp64': GRAV_MODE_FP64,
         'fp32u': GRAV_MODE_FP32U, 'fp32cu': GRAV_MODE_FP32CU, 'fp32n': GRAV_MODE_FP32N,
         'fp32un': GRAV_MODE_FP32UN}
PAIR_MODES = ('fp32u', 'fp32cu', 'fp32un', GRAV_MODE_FP32U, GRAV_MODE_FP32CU, GRAV_MODE_FP32UN)


class GravError(RuntimeError):
    """A C-ABI call returned a non-zero status."""

    def __init__(self, code, msg):
        super().__init__('gravitation_gb300 error %d: %s' % (code, msg))
        self.code = code


# ---- structs (mirror of the header) ---------------------------------------------
class UnivDesc(ctypes.Structure):
    _fields_ = [('body_off', ctypes.c_int64), ('pad_off', ctypes.c_int64),
                ('n', ctypes.c_int32), ('n_jtiles', ctypes.c_int32), ('T', ctypes.c_double)]


class SegDesc(ctypes.Structure):
    _fields_ = [('unit_begin', ctypes.c_int64), ('u', ctypes.c_int32), ('il0', ctypes.c_int32),
                ('n_units', ctypes.c_int32), ('cta_first', ctypes.c_int32),
                ('slot_base', ctypes.c_int32), ('nslots', ctypes.c_int32)]


class Tile(ctypes.Structure):
    _fields_ = [('bpt', ctypes.c_int32), ('threads', ctypes.c_int32),
                ('jtile', ctypes.c_int32), ('grid', ctypes.c_int32)]

    def key(self):
        return (self.bpt, self.threads, self.jtile)

    def __repr__(self):
        return 'Tile(bpt=%d, threads=%d, jtile=%d, grid=%d)' % (
            self.bpt, self.threads, self.jtile, self.grid)


class PlanInfo(ctypes.Structure):
    _fields_ = [('n_bodies', ctypes.c_int64), ('n_pad_total', ctypes.c_int64),
                ('n_units', ctypes.c_int64), ('n_univ', ctypes.c_int32),
                ('n_seg', ctypes.c_int32), ('n_slots', ctypes.c_int32),
                ('itile', ctypes.c_int32), ('pad_unit', ctypes.c_int32),
                ('grid', ctypes.c_int32)]


class Batch(ctypes.Structure):
    _fields_ = [('mode', ctypes.c_int32), ('n_univ', ctypes.c_int32), ('n_seg', ctypes.c_int32),
                ('n_slots', ctypes.c_int32), ('n_bodies', ctypes.c_int64),
                ('n_pad_total', ctypes.c_int64), ('n_units', ctypes.c_int64),
                ('tile', Tile), ('eps2', ctypes.c_float), ('_pad0', ctypes.c_float),
                ('univ', ctypes.c_void_p), ('seg', ctypes.c_void_p),
                ('r', ctypes.c_void_p), ('v', ctypes.c_void_p), ('pos', ctypes.c_void_p),
                ('part', ctypes.c_void_p), ('a_out', ctypes.c_void_p),
                ('err', ctypes.c_void_p)]


class Adjoint(ctypes.Structure):
    _fields_ = [('b', ctypes.POINTER(Batch)), ('gr', ctypes.c_void_p), ('gv', ctypes.c_void_p),
                ('ggm', ctypes.c_void_p), ('upos', ctypes.c_void_p), ('part7', ctypes.c_void_p),
                ('a_in', ctypes.c_void_p)]


GRAV_SCEN_UNIFORM_CUBE = 1
GRAV_SCEN_PLUMMER = 2
GRAV_SCEN_GALAXY = 3


class Scenario(ctypes.Structure):
    _fields_ = [('kind', ctypes.c_int32), ('_pad0', ctypes.c_int32), ('seed', ctypes.c_uint64),
                ('stream', ctypes.c_uint64), ('G', ctypes.c_double), ('p', ctypes.c_double * 10)]


# ---- declarations -----------------------------------------------------------------
_P = ctypes.POINTER
_DECLS = {
    'grav_abi_version': (ctypes.c_int, []),
    'grav_last_error': (ctypes.c_char_p, []),
    'grav_device_query': (ctypes.c_int, [ctypes.c_int, _P(ctypes.c_int32), _P(ctypes.c_int32),
                                         _P(ctypes.c_int32)]),
    'grav_tile_supported': (ctypes.c_int, [ctypes.c_int, _P(Tile)]),
    'grav_tile_list': (ctypes.c_int, [ctypes.c_int, _P(Tile), ctypes.c_int]),
    'grav_occupancy': (ctypes.c_int, [ctypes.c_int, _P(Tile), _P(ctypes.c_int32)]),
    'grav_plan': (ctypes.c_int, [ctypes.c_int32, _P(ctypes.c_int32), _P(ctypes.c_double),
                                 _P(Tile), _P(PlanInfo), _P(UnivDesc), _P(SegDesc)]),
    'grav_plan_pairs': (ctypes.c_int, [ctypes.c_int32, _P(ctypes.c_int32), _P(ctypes.c_double),
                                       _P(Tile), _P(PlanInfo), _P(UnivDesc), _P(SegDesc)]),
    'grav_pos_bytes': (ctypes.c_int64, [ctypes.c_int, ctypes.c_int64]),
    'grav_part_bytes': (ctypes.c_int64, [_P(PlanInfo)]),
    'grav_eps2': (ctypes.c_float, [ctypes.c_double]),
    'grav_prepare': (ctypes.c_int, [_P(Batch), ctypes.c_void_p]),
    'grav_stage1': (ctypes.c_int, [_P(Batch), ctypes.c_void_p]),
    'grav_stage2': (ctypes.c_int, [_P(Batch), ctypes.c_int, ctypes.c_void_p]),
    'grav_step': (ctypes.c_int, [_P(Batch), ctypes.c_int, ctypes.c_void_p]),
    'grav_fused_supported': (ctypes.c_int, [ctypes.c_int, ctypes.c_int32, ctypes.c_int32,
                                            ctypes.c_int32]),
    'grav_fused_occupancy': (ctypes.c_int, [ctypes.c_int, ctypes.c_int32, ctypes.c_int32,
                                            ctypes.c_int32, _P(ctypes.c_int32)]),
    'grav_step_fused': (ctypes.c_int, [_P(Batch), ctypes.c_int, ctypes.c_int32, ctypes.c_int32,
                                       ctypes.c_void_p, ctypes.c_void_p]),
    'grav_fp32_peak_probe': (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32,
                                            ctypes.c_void_p]),
    'grav_energy': (ctypes.c_int, [_P(Batch), ctypes.c_void_p, ctypes.c_void_p]),
    'grav_wait_check': (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p]),
    'grav_host_device_pointer': (ctypes.c_int, [ctypes.c_void_p, _P(ctypes.c_void_p)]),
    'grav_scenario_scratch_bytes': (ctypes.c_int64, [_P(Scenario), ctypes.c_int64]),
    'grav_scenario_generate': (ctypes.c_int, [_P(Scenario), ctypes.c_void_p, ctypes.c_void_p,
                                              ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p]),
    'grav_adjoint_tile_supported': (ctypes.c_int, [ctypes.c_int, _P(Tile)]),
    'grav_adjoint_occupancy': (ctypes.c_int, [ctypes.c_int, _P(Tile), _P(ctypes.c_int32)]),
    'grav_adjoint_prepare': (ctypes.c_int, [_P(Adjoint), ctypes.c_void_p]),
    'grav_adjoint_step': (ctypes.c_int, [_P(Adjoint), ctypes.c_void_p]),
    'grav_forces_noalloc': (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32,
                                           ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p]),
}
GRAV_NOALLOC_MAX_N = 16384

_lock = threading.Lock()
_lib = None


def load():
    """Load the library (once).  Raises if it is missing: there is no fallback."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIB_PATH):
            raise ImportError(
                'libgravgb300.so is missing at %s: build it with '
                '"python -m gravitation_gb300.build" (no CPU fallback exists)' % LIB_PATH)
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in _DECLS.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        if L.grav_abi_version() != GRAV_ABI_VERSION:
            raise ImportError('libgravgb300.so ABI %d != expected %d' % (
                L.grav_abi_version(), GRAV_ABI_VERSION))
        _lib = L
    return _lib


def declared_symbols():
    return sorted(_DECLS)


def last_error():
    return load().grav_last_error().decode(errors='replace')


def check(rc):
    """Raise GravError for a non-zero status code."""
    if rc != GRAV_OK:
        raise GravError(rc, last_error())
    return rc
