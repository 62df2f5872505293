"""Checkpoint / resume (lbm_save, lbm_load): a resumed run continues bit for
bit, in every storage precision."""
import numpy as np
import pytest

from chemsim_gb300 import lbm
from chemsim_gb300.lbm import (BF16DEV, F16DEV, F32, F64, FAST, FRAME_XY, SOLID_HALFWAY,
                               X_PERIODIC, Y_PERIODIC, Y_WALL, Lattice)
from chemsim_gb300.workloads import channel_spec

pytestmark = pytest.mark.gpu
FLAGS = X_PERIODIC | Y_WALL | SOLID_HALFWAY | FRAME_XY | FAST


def _lattice(spec, precision):
    lat = Lattice(spec.w, spec.h, spec.tau, precision, FLAGS)
    lat.set_force(*spec.force)
    lat.set_geometry(spec.solid)
    lat.init_equilibrium(spec.rho, spec.ux, spec.uy)
    return lat


@pytest.mark.parametrize("precision", [F32, F64, F16DEV, BF16DEV])
def test_resume_continues_bit_for_bit(gpu, tmp_path, precision):
    spec = channel_spec(192, n_obstacles=4, r_lo=5, r_hi=12, force=1e-5, seed=8, h=96)
    path = tmp_path / "state.lbm"
    with _lattice(spec, precision) as a:
        a.step(37)
        a.save(path)
        with Lattice(spec.w, spec.h, 0.9, precision, FLAGS) as b:   # other tau, no geometry
            b.load(path)
            assert b.time() == a.time()
            a.step(25)
            b.step(25)
            assert np.array_equal(a.get_populations(np.float64), b.get_populations(np.float64))
            assert b.time() == a.time()


def test_load_rejects_mismatches(gpu, tmp_path):
    spec = channel_spec(128, n_obstacles=2, r_lo=4, r_hi=8, force=1e-5, seed=9, h=64)
    path = tmp_path / "state.lbm"
    with _lattice(spec, F32) as a:
        a.save(path)
    with Lattice(128, 32, 0.6, F32, FLAGS) as b, pytest.raises(lbm.LBMError):
        b.load(path)                                    # other size
    with Lattice(128, 64, 0.6, F16DEV, FLAGS) as b, pytest.raises(lbm.LBMError):
        b.load(path)                                    # other precision
    with Lattice(128, 64, 0.6, F32, X_PERIODIC | Y_PERIODIC | FRAME_XY) as b, \
            pytest.raises(lbm.LBMError):
        b.load(path)                                    # other boundaries
    (tmp_path / "short.lbm").write_bytes(path.read_bytes()[:500])
    with Lattice(128, 64, 0.6, F32, FLAGS) as b, pytest.raises(lbm.LBMError):
        b.load(tmp_path / "short.lbm")                  # truncated


# offsets of header fields (the 96-byte checkpoint header of lbm_save)
_OFF = {"collision": 28, "tau": 40, "tau_minus": 44, "dx": 48, "dt": 52, "fx": 56, "time": 64,
        "steps": 72}


@pytest.mark.parametrize("field,value", [("tau", -1.0), ("dt", 0.0), ("fx", float("nan")),
                                         ("dx", float("inf")), ("collision", 7), ("steps", -3)])
def test_load_of_a_corrupt_header_leaves_the_lattice_unchanged(gpu, tmp_path, field, value):
    """A header value that a setter would reject fails the load before the
    lattice changes: populations, time, step count and the step rule stay."""
    import struct
    spec = channel_spec(128, n_obstacles=2, r_lo=4, r_hi=8, force=1e-5, seed=9, h=64)
    path = tmp_path / "state.lbm"
    with _lattice(spec, F32) as a:
        a.step(5)
        a.save(path)
    raw = bytearray(path.read_bytes())
    fmt = {"collision": "<i", "steps": "<q"}.get(field, "<f")
    struct.pack_into(fmt, raw, _OFF[field], value)
    (tmp_path / "bad.lbm").write_bytes(bytes(raw))
    other = channel_spec(128, n_obstacles=3, r_lo=4, r_hi=8, force=2e-5, seed=10, h=64)
    with _lattice(other, F32) as b, _lattice(other, F32) as ref:
        b.step(3)
        ref.step(3)
        with pytest.raises(lbm.LBMError):
            b.load(tmp_path / "bad.lbm")
        assert b.time() == ref.time()
        b.step(4)
        ref.step(4)
        assert np.array_equal(b.get_populations(), ref.get_populations())
