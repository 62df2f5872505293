"""ctypes binding of liblbm_cuda.so (include/lbm_cuda.h).

The library is the product: this module only declares its C signatures.
Loading fails loudly when the library has not been built; there is no
fallback implementation.
"""
from __future__ import annotations

import ctypes
import os
import re
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "liblbm_cuda.so")
HEADER_DIR = os.path.join(os.path.dirname(HERE), "include")

# status codes
LBM_OK = 0
LBM_ERR_INVALID_ARGUMENT = -1
LBM_ERR_OUT_OF_MEMORY = -2
LBM_ERR_CUDA = -3
LBM_ERR_UNSTABLE = -4
LBM_ERR_TIMEOUT = -5
LBM_ERR_NOT_SUPPORTED = -6
LBM_ERR_STATE = -7
# precision
F32, F64, F16DEV, BF16DEV = 0, 1, 2, 3
# flags
X_ZEROPAD, X_PERIODIC, X_WALL = 0x00, 0x01, 0x02
Y_ZEROPAD, Y_PERIODIC, Y_WALL = 0x00, 0x04, 0x08
SOLID_FULLWAY, SOLID_HALFWAY = 0x00, 0x10
FRAME_REF, FRAME_XY = 0x00, 0x20
FAST = 0x40
ROUND_NEAREST = 0x80
REFERENCE_FLAGS = 0x00
# collision
COLLISION_BGK, COLLISION_TRT = 0, 1


class LBMHealth(ctypes.Structure):
    _fields_ = [
        ("mass", ctypes.c_double),
        ("momentum_x", ctypes.c_double),
        ("momentum_y", ctypes.c_double),
        ("min_population", ctypes.c_double),
        ("min_eq0", ctypes.c_double),
        ("nonfinite_count", ctypes.c_int64),
        ("steps", ctypes.c_int64),
        ("unstable", ctypes.c_int32),
        ("reserved", ctypes.c_int32),
    ]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_ if k != "reserved"}


class LBMDesc(ctypes.Structure):
    _fields_ = [
        ("w", ctypes.c_int), ("h", ctypes.c_int), ("tau", ctypes.c_float),
        ("flags", ctypes.c_int), ("fx", ctypes.c_float), ("fy", ctypes.c_float),
        ("solid", ctypes.c_void_p),
    ]


class LBMError(RuntimeError):
    """A negative status of the C ABI (the reference panics in these cases)."""

    def __init__(self, status: int, message: str):
        super().__init__(f"lbm status {status}: {message}")
        self.status = status


_vp = ctypes.c_void_p
_i32 = ctypes.c_int
_f32 = ctypes.c_float
_i64 = ctypes.c_int64
_f32p = ctypes.POINTER(ctypes.c_float)
_f64p = ctypes.POINTER(ctypes.c_double)
_u8p = ctypes.POINTER(ctypes.c_uint8)

# name -> (restype, argtypes)
SIGNATURES = {
    "lbm_last_error_string": (ctypes.c_char_p, []),
    "lbm_version": (_i32, []),
    "lbm_create": (_i32, [_i32, _i32, _f32, _i32, _i32, ctypes.POINTER(_vp)]),
    "lbm_destroy": (_i32, [_vp]),
    "lbm_set_discretization": (_i32, [_vp, _f32, _f32]),
    "lbm_set_collision": (_i32, [_vp, _i32, _f32, _f32]),
    "lbm_init_equilibrium": (_i32, [_vp, _vp, _vp, _vp]),
    "lbm_set_populations": (_i32, [_vp, _vp]),
    "lbm_get_populations": (_i32, [_vp, _vp]),
    "lbm_set_populations_f64": (_i32, [_vp, _vp]),
    "lbm_get_populations_f64": (_i32, [_vp, _vp]),
    "lbm_set_geometry": (_i32, [_vp, _vp]),
    "lbm_set_force": (_i32, [_vp, _f32, _f32]),
    "lbm_step": (_i32, [_vp, _i32]),
    "lbm_step_moments": (_i32, [_vp, _i32]),
    "lbm_read_moments": (_i32, [_vp, _vp, _vp, _vp, _i32]),
    "lbm_check": (_i32, [_vp, ctypes.POINTER(LBMHealth)]),
    "lbm_get_time": (_i32, [_vp, ctypes.POINTER(_f32), ctypes.POINTER(_i64)]),
    "lbm_set_stream": (_i32, [_vp, _vp]),
    "lbm_synchronize": (_i32, [_vp]),
    "lbm_device_populations": (_i32, [_vp, ctypes.POINTER(_vp), ctypes.POINTER(_i64),
                                      ctypes.POINTER(_i32)]),
    "lbm_set_tile": (_i32, [_vp, _i32, _i32]),
    "lbm_check_device_noalloc": (_i32, [_vp, _i32, _i32, _i32, _i32, _i64, _f32, _f32, _vp,
                                        ctypes.POINTER(LBMHealth)]),
    "lbm_batch_create": (_i32, [_i32, ctypes.POINTER(LBMDesc), _i32, ctypes.POINTER(_vp)]),
    "lbm_batch_destroy": (_i32, [_vp]),
    "lbm_batch_size": (_i32, [_vp, ctypes.POINTER(_i32)]),
    "lbm_batch_lattice": (_i32, [_vp, _i32, ctypes.POINTER(_vp)]),
    "lbm_batch_step": (_i32, [_vp, _i32]),
    "lbm_batch_synchronize": (_i32, [_vp]),
    "lbm_batch_set_stream": (_i32, [_vp, _vp]),
    "lbm_batch_set_tile": (_i32, [_vp, _i32]),
    "lbm_batch_tile": (_i32, [_vp, ctypes.POINTER(_i32)]),
    "lbm_batch_autotune": (_i32, [_vp, ctypes.c_char_p, _i32]),
    "lbm_read_moments_async": (_i32, [_vp, _vp, _vp, _vp]),
    "lbm_step_moments_to": (_i32, [_vp, _i32, _vp, _vp, _vp]),
    "lbm_readback_wait": (_i32, [_vp]),
    "lbm_render": (_i32, [_vp, _i32, _i32, _vp, _i32]),
    "lbm_render_async": (_i32, [_vp, _i32, _i32, _vp]),
    "lbm_save": (_i32, [_vp, ctypes.c_char_p]),
    "lbm_load": (_i32, [_vp, ctypes.c_char_p]),
    "lbm_cnn_create": (_i32, [_i32, _i32, _i32, ctypes.c_uint64, ctypes.POINTER(_vp)]),
    "lbm_cnn_destroy": (_i32, [_vp]),
    "lbm_cnn_param_count": (_i32, [_vp, ctypes.POINTER(_i64)]),
    "lbm_cnn_get_params": (_i32, [_vp, _vp]),
    "lbm_cnn_set_params": (_i32, [_vp, _vp]),
    "lbm_cnn_forward": (_i32, [_vp, _vp, _i32, _vp]),
    "lbm_cnn_gradients": (_i32, [_vp, _vp, _vp, _i32, ctypes.POINTER(_f32), _vp]),
    "lbm_cnn_train_step": (_i32, [_vp, _vp, _vp, _i32, _f32, ctypes.POINTER(_f32)]),
    "lbm_cnn_set_stream": (_i32, [_vp, _vp]),
    "lbm_selftest_wait_timeout": (_i32, [ctypes.c_uint32, ctypes.POINTER(_i32)]),
    "lbm_cnn_save": (_i32, [_vp, ctypes.c_char_p]),
    "lbm_cnn_load": (_i32, [_vp, ctypes.c_char_p]),
    "lbm_coarse_run": (_i32, [_vp, _vp, _i32, _i32, _f32, _f32, _f32, _f32, _i32, _f32,
                              ctypes.POINTER(_i64)]),
    "lbm_cnn_synchronize": (_i32, [_vp]),
    "lbm_restrict": (_i32, [_vp, _vp, _i32]),
    "lbm_coarse_features": (_i32, [_vp, _f32, _f32, _i32, _vp]),
    "lbm_coarse_apply": (_i32, [_vp, _vp, _i32, _f32, _f32]),
    "lbm_coarse_target": (_i32, [_vp, _vp, _f32, _i32, _vp]),
}

_lock = threading.Lock()
_lib = None


def header_functions() -> list[str]:
    """Names of every function declared in include/*.h."""
    names = []
    for fn in sorted(os.listdir(HEADER_DIR)):
        if not fn.endswith(".h"):
            continue
        with open(os.path.join(HEADER_DIR, fn)) as fh:
            text = fh.read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(lbm_\w+)\s*\(", text, re.M):
            names.append(m.group(1))
    return names


def load() -> ctypes.CDLL:
    """Load the built library (raises if it is missing)."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise OSError(
                    f"{LIB_PATH} is missing: build it with chemsim_gb300.build.build() "
                    "(there is no CPU fallback)")
            lib = ctypes.CDLL(LIB_PATH)
            for name, (res, args) in SIGNATURES.items():
                fn = getattr(lib, name, None)
                if fn is None:
                    continue
                fn.restype = res
                fn.argtypes = args
            _lib = lib
    return _lib


def last_error() -> str:
    msg = load().lbm_last_error_string()
    return msg.decode() if msg else ""


def check(status: int) -> int:
    if status != LBM_OK:
        raise LBMError(status, last_error())
    return status
