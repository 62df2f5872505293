"""ctypes front-end and build recipe of the C++ oracle (lbm_oracle.cpp).

TEST INFRASTRUCTURE ONLY — see the package docstring.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SRC = os.path.join(_HERE, "lbm_oracle.cpp")
_HDR = os.path.join(os.path.dirname(_HERE), "include", "lbm_cuda.h")
_OUT_DIR = os.path.join(_HERE, "_build")
_LIB = os.path.join(_OUT_DIR, "liblbm_oracle.so")

F32, F64 = 0, 1
_lock = threading.Lock()
_lib = None


def lib_path() -> str:
    return _LIB


def build(force: bool = False) -> str:
    """Compile lbm_oracle.cpp into oracle/_build/liblbm_oracle.so.

    -ffp-contract=off keeps one rounding per operation on every host
    (aarch64 GCC would otherwise fuse multiply-adds).
    """
    os.makedirs(_OUT_DIR, exist_ok=True)
    newest = max(os.path.getmtime(_SRC), os.path.getmtime(_HDR))
    if not force and os.path.exists(_LIB) and os.path.getmtime(_LIB) >= newest:
        return _LIB
    tmp = _LIB + f".tmp{os.getpid()}"
    cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-fopenmp",
           "-ffp-contract=off", "-fno-fast-math", _SRC, "-o", tmp]
    subprocess.run(cmd, check=True)
    os.replace(tmp, _LIB)
    return _LIB


def _load():
    global _lib
    with _lock:
        if _lib is None:
            build()
            lib = ctypes.CDLL(_LIB)
            vp, i32, f64 = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
            lib.orc_step.argtypes = [i32, i32, i32, i32, i32, f64, f64, f64, f64,
                                     f64, f64, vp, vp, i32, i32, i32]
            lib.orc_step.restype = i32
            lib.orc_equilibrium.argtypes = [i32, i32, i32, f64, f64, vp, vp, vp, vp]
            lib.orc_equilibrium.restype = i32
            lib.orc_moments.argtypes = [i32, i32, i32, f64, f64, vp, vp, vp, vp]
            lib.orc_moments.restype = i32
            lib.orc_health.argtypes = [i32, i32, i32, f64, f64, vp,
                                       ctypes.POINTER(ctypes.c_double),
                                       ctypes.POINTER(ctypes.c_int64)]
            lib.orc_health.restype = i32
            lib.orc_max_threads.argtypes = []
            lib.orc_max_threads.restype = i32
            _lib = lib
    return _lib


def _prec(a: np.ndarray) -> int:
    if a.dtype == np.float32:
        return F32
    if a.dtype == np.float64:
        return F64
    raise TypeError(f"oracle supports float32/float64, got {a.dtype}")


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def step(f: np.ndarray, nsteps: int, *, tau: float, flags: int = 0,
         collision: int = 0, tau_minus: float = 1.0, dx: float = 1.0,
         dt: float = 1.0, force=(0.0, 0.0), solid=None, structured=False,
         threads: int = 1) -> np.ndarray:
    """Advance a (9, h, w) population array nsteps (returns a new array)."""
    f = np.ascontiguousarray(f).copy()
    if f.ndim != 3 or f.shape[0] != 9:
        raise ValueError("populations must be shaped (9, h, w)")
    _, h, w = f.shape
    if solid is not None:
        solid = np.ascontiguousarray(solid, dtype=np.uint8)
        if solid.shape != (h, w):
            raise ValueError("solid mask must be shaped (h, w)")
    rc = _load().orc_step(_prec(f), w, h, flags, collision, tau, tau_minus, dx,
                          dt, float(force[0]), float(force[1]), _ptr(solid),
                          _ptr(f), int(nsteps), int(bool(structured)), int(threads))
    if rc != 0:
        raise RuntimeError(f"orc_step failed with status {rc}")
    return f


def equilibrium(rho, ux, uy, *, dx: float = 1.0, dt: float = 1.0) -> np.ndarray:
    """compute_equilibrium (src/lbm.rs:43-71) over (h, w) fields -> (9, h, w)."""
    rho = np.ascontiguousarray(rho)
    ux = np.ascontiguousarray(ux, dtype=rho.dtype)
    uy = np.ascontiguousarray(uy, dtype=rho.dtype)
    h, w = rho.shape
    f = np.empty((9, h, w), dtype=rho.dtype)
    rc = _load().orc_equilibrium(_prec(rho), w, h, dx, dt, _ptr(rho), _ptr(ux),
                                 _ptr(uy), _ptr(f))
    if rc != 0:
        raise RuntimeError(f"orc_equilibrium failed with status {rc}")
    return f


def moments(f: np.ndarray, force=(0.0, 0.0)):
    """(rho, ux, uy) of a state (src/lbm.rs:117-149)."""
    f = np.ascontiguousarray(f)
    _, h, w = f.shape
    rho = np.empty((h, w), dtype=f.dtype)
    ux = np.empty_like(rho)
    uy = np.empty_like(rho)
    rc = _load().orc_moments(_prec(f), w, h, float(force[0]), float(force[1]),
                             _ptr(f), _ptr(rho), _ptr(ux), _ptr(uy))
    if rc != 0:
        raise RuntimeError(f"orc_moments failed with status {rc}")
    return rho, ux, uy


def health(f: np.ndarray, *, dx: float = 1.0, dt: float = 1.0) -> dict:
    f = np.ascontiguousarray(f)
    _, h, w = f.shape
    out = (ctypes.c_double * 6)()
    bad = ctypes.c_int64(0)
    rc = _load().orc_health(_prec(f), w, h, dx, dt, _ptr(f), out, ctypes.byref(bad))
    if rc != 0:
        raise RuntimeError(f"orc_health failed with status {rc}")
    return {"mass": out[0], "momentum_x": out[1], "momentum_y": out[2],
            "min_population": out[3], "min_eq0": out[4],
            "nonfinite_count": int(bad.value)}


def max_threads() -> int:
    return int(_load().orc_max_threads())
