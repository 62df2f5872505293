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
