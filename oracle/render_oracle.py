"""CPU oracle of the colour map — TEST INFRASTRUCTURE ONLY.

numpy restatement of taktoa/chemsim src/render.rs, the checker of
liblbm_cuda.so's lbm_render:

  render_scalar_field (src/render.rs:23-89): hue 0, saturation 1,
    value = logistic((x - mean_all) * (1 / stdev_all)), each clamped to [0, 1]
  render_vector_field (src/render.rs:91-207): hue = (arg(vx + i vy) + pi) *
    (FRAC_1_PI * 0.5), saturation 0.8, value = logistic of the z-score of
    vx^2 + vy^2
  af::hsv2rgb: the hexcone model (sector i = floor(6h), f = 6h - i,
    p = v(1 - s), q = v(1 - f s), t = v(1 - (1 - f) s))
  pixel channel = (256 c).round().min(255).max(0) as u8 (src/render.rs:77-82)
  render_geometry (src/render.rs:7-21): solid cells (0, 0, 255).

ArrayFire (the arrayfire crate 3.6.0, Cargo.lock:59-61) is not in the source
tree; mean_all / stdev_all are restated as the mean and the population
standard deviation (division by the element count) of all elements, in f64.
Per-pixel arithmetic is f32, one rounding per operation; exp and atan2 are
numpy's float32 functions (their last-ulp results may differ from the GPU's,
which the tests allow for: one unit in a colour channel).
"""
from __future__ import annotations

import numpy as np

DENSITY, SPEED, VELOCITY, MOMENTUM = 0, 1, 2, 3
F32 = np.float32


def field(rho, ux, uy, mode):
    rho, ux, uy = (np.asarray(a, dtype=F32) for a in (rho, ux, uy))
    if mode == DENSITY:
        return rho
    if mode == SPEED:
        return np.sqrt(ux * ux + uy * uy)
    if mode == VELOCITY:
        return ux * ux + uy * uy
    jx, jy = rho * ux, rho * uy
    return jx * jx + jy * jy


def clamp01(x):
    with np.errstate(invalid="ignore"):
        return np.where(np.isnan(x), x, np.minimum(np.maximum(x, F32(0)), F32(1))).astype(F32)


def hsv2rgb(h, s, v):
    h, s, v = (np.asarray(a, dtype=F32) for a in (h, s, v))
    h, s, v = np.broadcast_arrays(h, s, v)
    with np.errstate(invalid="ignore"):
        h6 = h * F32(6)
        i = np.where(np.isnan(h6), 0, np.trunc(np.nan_to_num(h6))).astype(np.int64)
        f = (h6 - i.astype(F32)).astype(F32)
        p = v * (F32(1) - s)
        q = v * (F32(1) - f * s)
        t = v * (F32(1) - (F32(1) - f) * s)
    sec = i % 6
    r = np.select([sec == 0, sec == 1, sec == 2, sec == 3, sec == 4], [v, q, p, p, t], v)
    g = np.select([sec == 0, sec == 1, sec == 2, sec == 3, sec == 4], [t, v, v, q, p], p)
    b = np.select([sec == 0, sec == 1, sec == 2, sec == 3, sec == 4], [p, p, t, v, v], q)
    return r.astype(F32), g.astype(F32), b.astype(F32)


def to_u8(c):
    """(256 c).round().min(255).max(0) as u8: half away from zero, NaN -> 255."""
    x = np.asarray(c, dtype=F32) * F32(256)
    with np.errstate(invalid="ignore"):
        r = np.floor(x.astype(np.float64) + 0.5)          # x >= 0; negatives clamp to 0
        out = np.clip(np.nan_to_num(r, nan=255.0), 0, 255)
    return out.astype(np.uint8)


def render(rho, ux, uy, mode, solid=None):
    """RGBA8 image (h, w, 4)."""
    x = field(rho, ux, uy, mode)
    x64 = x.astype(np.float64)
    mean = x64.mean()
    std = np.sqrt(np.mean((x64 - mean) ** 2))
    avg = F32(mean)
    with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
        inv = F32(1) / F32(std)
        z = (x - avg) * inv
        val = clamp01(F32(1) / (F32(1) + np.exp(-z)))
    if mode in (VELOCITY, MOMENTUM):
        vx, vy = np.asarray(ux, F32), np.asarray(uy, F32)
        if mode == MOMENTUM:
            vx, vy = np.asarray(rho, F32) * vx, np.asarray(rho, F32) * vy
        half_over_pi = F32(np.float32(1 / np.pi) * F32(0.5))
        hue = clamp01((np.arctan2(vy, vx).astype(F32) + F32(np.pi)) * half_over_pi)
        sat = F32(0.8)
    else:
        hue, sat = F32(0), F32(1)
    r, g, b = hsv2rgb(hue, sat, val)
    img = np.empty(x.shape + (4,), dtype=np.uint8)
    img[..., 0], img[..., 1], img[..., 2], img[..., 3] = to_u8(r), to_u8(g), to_u8(b), 255
    if solid is not None:
        img[np.asarray(solid).astype(bool)] = (0, 0, 255, 255)
    return img
