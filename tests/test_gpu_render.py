"""lbm_render (the colour map of src/render.rs) against the numpy oracle."""
import numpy as np
import pytest

from oracle import render_oracle as ro
from chemsim_gb300 import lbm
from chemsim_gb300.lbm import (F32, FAST, FRAME_XY, RENDER_DENSITY, RENDER_MOMENTUM, RENDER_SPEED,
                               RENDER_VELOCITY, SOLID_HALFWAY, X_PERIODIC, Y_WALL, Lattice)

pytestmark = pytest.mark.gpu
MODES = (RENDER_DENSITY, RENDER_SPEED, RENDER_VELOCITY, RENDER_MOMENTUM)


def _channel(w, h, seed):
    from chemsim_gb300.workloads import channel_spec
    return channel_spec(w, n_obstacles=5, r_lo=4, r_hi=12, force=1e-5, seed=seed, h=h)


@pytest.fixture(scope="module")
def flowing():
    spec = _channel(256, 160, 4)
    lat = Lattice(256, 160, 0.6, F32, X_PERIODIC | Y_WALL | SOLID_HALFWAY | FRAME_XY | FAST)
    lat.set_force(*spec.force)
    lat.set_geometry(spec.solid)
    rng = np.random.default_rng(2)
    rho = (1 + 0.01 * rng.normal(size=(160, 256))).astype(np.float32)
    ux = (0.02 * rng.normal(size=(160, 256))).astype(np.float32)
    uy = (0.02 * rng.normal(size=(160, 256))).astype(np.float32)
    lat.init_equilibrium(rho, ux, uy)
    lat.step(20)
    yield lat, spec.solid
    lat.close()


def _compare(got, ref):
    d = np.abs(got.astype(int) - ref.astype(int))
    # exp / atan2 may differ in the last ulp between the GPU and numpy: one
    # unit in a channel, on a small fraction of pixels
    assert d.max() <= 1
    assert (d.max(axis=-1) > 0).mean() < 5e-3


@pytest.mark.parametrize("mode", MODES)
def test_render_matches_oracle(gpu, flowing, mode):
    lat, solid = flowing
    got = lat.render(mode, geometry_overlay=True)
    rho, ux, uy = lat.moments()
    _compare(got, ro.render(rho, ux, uy, mode, solid))
    # without the overlay, solid cells take the colour of their field value
    got = lat.render(mode, geometry_overlay=False)
    _compare(got, ro.render(rho, ux, uy, mode, None))


def test_render_to_device_equals_host(gpu, flowing):
    torch = pytest.importorskip("torch")
    lat, _ = flowing
    buf = torch.zeros((160, 256, 4), dtype=torch.uint8, device="cuda")
    lat.render_to_device(buf.data_ptr(), RENDER_VELOCITY)
    assert np.array_equal(buf.cpu().numpy(), lat.render(RENDER_VELOCITY))


def test_uniform_density_renders_white(gpu):
    with Lattice(128, 64, 0.7, F32, X_PERIODIC | Y_WALL | FRAME_XY) as lat:
        one = np.ones((64, 128), np.float32)
        lat.init_equilibrium(one, one * 0, one * 0)
        img = lat.render(RENDER_DENSITY)
        assert (img == 255).all()


def test_bad_mode_rejected(gpu, flowing):
    lat, _ = flowing
    with pytest.raises(lbm.LBMError):
        lat.render(7)


def test_record_writes_the_rendered_frames(gpu, tmp_path):
    from chemsim_gb300.record import read_png, record
    spec = _channel(128, 64, 6)
    flags = X_PERIODIC | Y_WALL | SOLID_HALFWAY | FRAME_XY | FAST
    with Lattice(128, 64, 0.6, F32, flags) as a, Lattice(128, 64, 0.6, F32, flags) as b:
        for lat in (a, b):
            lat.set_force(*spec.force)
            lat.set_geometry(spec.solid)
            lat.init_equilibrium(spec.rho, spec.ux, spec.uy)
        paths = record(a, 3, str(tmp_path / "frame{:03d}.png"), steps_per_frame=5)
        assert [p[-12:] for p in paths] == ["frame000.png", "frame001.png", "frame002.png"]
        for p in paths:
            b.step(5)
            with open(p, "rb") as fh:
                assert np.array_equal(read_png(fh.read()), b.render(RENDER_VELOCITY))


def test_render_async_is_a_snapshot(gpu):
    torch = pytest.importorskip("torch")
    spec = _channel(128, 64, 7)
    flags = X_PERIODIC | Y_WALL | SOLID_HALFWAY | FRAME_XY | FAST
    with Lattice(128, 64, 0.6, F32, flags) as a, Lattice(128, 64, 0.6, F32, flags) as b:
        for lat in (a, b):
            lat.set_force(*spec.force)
            lat.set_geometry(spec.solid)
            lat.init_equilibrium(spec.rho, spec.ux, spec.uy)
        imgs = [torch.zeros((64, 128, 4), dtype=torch.uint8).pin_memory().numpy() for _ in range(2)]
        a.step(6)
        a.render_async(imgs[0], RENDER_SPEED)
        a.step(6)                       # runs while the copy may be in flight
        a.render_async(imgs[1], RENDER_SPEED)
        a.readback_wait()
        b.step(6)
        assert np.array_equal(imgs[0], b.render(RENDER_SPEED))
        b.step(6)
        assert np.array_equal(imgs[1], b.render(RENDER_SPEED))
