"""lbm_check_device_noalloc: the health check for callers that cannot call
cudaMalloc (render/game loops that must avoid cudaMalloc's implicit device
synchronisation, hosts whose memory pool owns the whole device, plugin hosts
that forbid library allocations).

It reduces populations the caller already holds on the device, using a
static device scratch array instead of allocating; its results must agree
with lbm_check's on the same state, call after call (the array keeps the
previous call's contents).  This file is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

from chemsim_gb300 import _lib
from chemsim_gb300.lbm import BF16DEV, F16DEV, F32, F64, X_PERIODIC, Y_PERIODIC, Lattice

pytestmark = pytest.mark.gpu

MAX_CELLS = 16384 * 16384


def _noalloc(lib, lat, dx=1.0, dt=1.0):
    base, plane, pitch = lat.device_populations()
    out = _lib.LBMHealth()
    rc = lib.lbm_check_device_noalloc(ctypes.c_void_p(base), lat.precision, lat.w, lat.h, pitch,
                                      plane, dx, dt, None, ctypes.byref(out))
    assert rc == _lib.LBM_OK, _lib.last_error()
    return out.as_dict()


def _state(w, h, seed):
    rng = np.random.default_rng(seed)
    rho = (1 + rng.uniform(-0.01, 0.01, (h, w))).astype(np.float32)
    ux = rng.uniform(-0.05, 0.05, (h, w)).astype(np.float32)
    uy = rng.uniform(-0.05, 0.05, (h, w)).astype(np.float32)
    return rho, ux, uy


def _close(a, b, scale):
    if np.isnan(a) or np.isnan(b):          # a NaN population makes both sums NaN
        return bool(np.isnan(a) and np.isnan(b))
    if not np.isfinite(scale):              # e.g. the mass when a population is NaN
        scale = max(abs(a), abs(b), 1.0)
    return abs(a - b) <= 1e-12 * abs(scale)


def _agree(got, ref):
    # The two reductions partition the cells differently, so the f64 sums may
    # differ in the last bits; extrema and counts are exact.
    assert _close(got["mass"], ref["mass"], ref["mass"])
    assert _close(got["momentum_x"], ref["momentum_x"], ref["mass"])
    assert _close(got["momentum_y"], ref["momentum_y"], ref["mass"])
    assert got["min_population"] == ref["min_population"]
    assert got["min_eq0"] == ref["min_eq0"]
    assert got["nonfinite_count"] == ref["nonfinite_count"]
    assert got["unstable"] == ref["unstable"]


@pytest.mark.parametrize("precision", [F32, F64, F16DEV, BF16DEV])
def test_noalloc_matches_lbm_check_twice(gpu, precision):
    lib = _lib.load()
    with Lattice(700, 300, 0.7, precision, X_PERIODIC | Y_PERIODIC) as big, \
            Lattice(37, 11, 0.9, precision, X_PERIODIC | Y_PERIODIC) as small:
        big.init_equilibrium(*_state(700, 300, 1))
        small.init_equilibrium(*_state(37, 11, 2))
        big.step(3)
        small.step(5)
        # two calls in a row on each lattice; the small one follows the big
        # one, so stale partials from the first call sit in the array
        for lat in (big, big, small, small):
            _agree(_noalloc(lib, lat), lat.health())


def test_noalloc_reports_planted_nan(gpu):
    lib = _lib.load()
    rho, ux, uy = _state(64, 48, 3)
    with Lattice(64, 48, 0.8, F32, 0) as lat:
        lat.init_equilibrium(rho, ux, uy)
        f = lat.get_populations()
        f[4, 10, 20] = np.nan
        lat.set_populations(f)
        first = _noalloc(lib, lat)
        second = _noalloc(lib, lat)
        ref = lat.health()
    assert first["nonfinite_count"] == 1 and first["unstable"] == 1
    _agree(first, ref)
    _agree(second, ref)


def test_noalloc_rejects_oversize_and_bad_arguments(gpu):
    lib = _lib.load()
    out = _lib.LBMHealth()
    # rejected on the host before any device access: the pointer is never used
    dummy = ctypes.c_void_p(256)
    rc = lib.lbm_check_device_noalloc(dummy, F32, 16385, 16384, 16385, 16385 * 16384,
                                      1.0, 1.0, None, ctypes.byref(out))
    assert rc == _lib.LBM_ERR_INVALID_ARGUMENT
    assert "268435456" in _lib.last_error()
    rc = lib.lbm_check_device_noalloc(dummy, 9, 8, 8, 8, 64, 1.0, 1.0, None, ctypes.byref(out))
    assert rc == _lib.LBM_ERR_INVALID_ARGUMENT and "precision" in _lib.last_error()
    rc = lib.lbm_check_device_noalloc(dummy, F32, 8, 8, 4, 64, 1.0, 1.0, None, ctypes.byref(out))
    assert rc == _lib.LBM_ERR_INVALID_ARGUMENT
    rc = lib.lbm_check_device_noalloc(None, F32, 8, 8, 8, 64, 1.0, 1.0, None, ctypes.byref(out))
    assert rc == _lib.LBM_ERR_INVALID_ARGUMENT
    assert 16384 * 16384 == MAX_CELLS


@pytest.mark.parametrize("dx,dt", [(0.25, 1.0), (1.0, 0.5), (2.0, 1.5)])
def test_noalloc_with_discretization_and_solids(gpu, dx, dt):
    """delta_x and delta_t set the speed of sound, which sets min f_eq[0]
    and with it the unstable flag: the caller passes the lattice's own
    values and gets lbm_check's answer, on a lattice with solid cells."""
    lib = _lib.load()
    w, h = 96, 40
    rng = np.random.default_rng(7)
    rho = (1 + rng.uniform(-0.01, 0.01, (h, w))).astype(np.float32)
    ux = rng.uniform(-0.25, 0.25, (h, w)).astype(np.float32)
    uy = rng.uniform(-0.25, 0.25, (h, w)).astype(np.float32)
    solid = (rng.uniform(size=(h, w)) < 0.1).astype(np.uint8)
    with Lattice(w, h, 0.8, F32, X_PERIODIC | Y_PERIODIC) as lat:
        lat.set_discretization(dx, dt)
        lat.set_geometry(solid)
        lat.init_equilibrium(rho, ux, uy)
        lat.step(2)
        ref = lat.health()
        for _ in range(2):
            _agree(_noalloc(lib, lat, dx, dt), ref)
        # the unit discretization gives a different min f_eq[0] on this state
        unit = _noalloc(lib, lat, 1.0, 1.0)
    assert unit["min_eq0"] != ref["min_eq0"]
