"""The colour-map oracle's building blocks (CPU)."""
import numpy as np

from oracle import render_oracle as ro


def test_hsv_primaries_and_grey():
    r, g, b = ro.hsv2rgb(np.array([0.0, 1 / 3, 2 / 3, 1.0], np.float32), np.float32(1), np.float32(1))
    np.testing.assert_allclose(np.stack([r, g, b]), [[1, 0, 0, 1], [0, 1, 0, 0], [0, 0, 1, 0]], atol=1e-6)
    r, g, b = ro.hsv2rgb(np.float32(0.3), np.float32(0), np.float32(0.25))
    assert r == g == b == np.float32(0.25)


def test_channel_rounding():
    # round half away from zero, 256 * 1.0 clamps to 255, NaN renders 255
    c = np.array([1.0, 0.5, 1.5 / 256, 0.5 / 256, -0.2, np.nan], np.float32)
    assert ro.to_u8(c).tolist() == [255, 128, 2, 1, 0, 255]


def test_uniform_field_is_white_and_overlay_blue():
    rho = np.ones((4, 5), np.float32)
    solid = np.zeros((4, 5), np.uint8)
    solid[1, 2] = 1
    img = ro.render(rho, rho * 0, rho * 0, ro.DENSITY, solid)
    assert (img[1, 2] == [0, 0, 255, 255]).all()
    rest = np.delete(img.reshape(-1, 4), 1 * 5 + 2, axis=0)
    assert (rest == 255).all()


def test_scalar_field_value_channel():
    # hue 0 and saturation 1: red = value, green = blue = 0
    rng = np.random.default_rng(0)
    rho = (1 + 0.01 * rng.normal(size=(8, 16))).astype(np.float32)
    img = ro.render(rho, rho * 0, rho * 0, ro.DENSITY)
    z = (rho.astype(np.float64) - rho.mean()) / rho.std()
    expect = np.clip(np.floor(256 / (1 + np.exp(-z)) + 0.5), 0, 255)
    assert np.abs(img[..., 0].astype(int) - expect).max() <= 1
    assert (img[..., 1] == 0).all() and (img[..., 2] == 0).all()


def test_vector_field_hue_follows_direction():
    ux = np.array([[1.0, -1.0, 0.0, 0.0]], np.float32) * 0.01
    uy = np.array([[0.0, 0.0, 1.0, -1.0]], np.float32) * 0.01
    img = ro.render(np.ones_like(ux), ux, uy, ro.VELOCITY)
    # equal magnitudes: std 0, the value is NaN and every channel white
    assert (img == 255).all()
    ux2 = ux * np.array([[1, 2, 3, 4]], np.float32)
    uy2 = uy * np.array([[1, 2, 3, 4]], np.float32)
    img = ro.render(np.ones_like(ux), ux2, uy2, ro.VELOCITY)
    # +x: hue 0.5 (cyan family: red lowest); -x: hue 0 or 1 (red highest)
    assert img[0, 0, 0] < img[0, 0, 1] and img[0, 1, 0] >= img[0, 1, 1]
