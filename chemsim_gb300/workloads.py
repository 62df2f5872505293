"""Seeded synthetic lattices (Taylor-Green vortex, obstacle channel, batches).

The reference has no datasets: its demo builds its state in code
(initial_state, taktoa/chemsim src/main.rs:180-328).  These generators build
the named benchmark lattices the same way, from a counter-based splitmix64
stream: value k of stream `seed` is splitmix64(seed + (k+1) * 0x9E3779B97F4A7C15),
so any consumer (GPU run, oracle, another language) regenerates identical
inputs from (seed, k).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from ._lib import FRAME_XY, SOLID_HALFWAY, X_PERIODIC, Y_PERIODIC, Y_WALL

_GOLDEN = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def splitmix64(seed: int, start: int, count: int) -> np.ndarray:
    """count uint64 outputs of stream `seed` from counter `start`."""
    with np.errstate(over="ignore"):
        k = np.arange(start + 1, start + 1 + count, dtype=np.uint64)
        z = np.uint64(seed & 0xFFFFFFFFFFFFFFFF) + k * _GOLDEN
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        return z ^ (z >> np.uint64(31))


def uniform(seed: int, start: int, count: int, lo: float = 0.0, hi: float = 1.0) -> np.ndarray:
    """Uniform f64 in [lo, hi) from the top 53 bits."""
    u = (splitmix64(seed, start, count) >> np.uint64(11)).astype(np.float64) * (2.0 ** -53)
    return lo + (hi - lo) * u


def taylor_green(n_x: int, n_y: int, *, u0: float = 0.02, noise: float = 1e-4,
                 seed: int = 1, frame_xy: bool = True):
    """rho = 1 + U(-noise, noise), u = u0 (sin kX cos kY, -(kx/ky) cos kX sin kY).

    The kx/ky factor (1 on square lattices) keeps u divergence-free when the
    two periods differ.

    x, y are cell indices.  In the XY frame x is the column and y the row.
    In the reference frame the lattice c-frame axes run along (-row, +column)
    (the convolve2 displacement of src/lbm.rs:716-729), so the same vortex is
    laid out on X = -row, Y = column.  Returns f32 (rho, ux, uy), (h, w).
    """
    rows, cols = np.meshgrid(np.arange(n_y, dtype=np.float64),
                             np.arange(n_x, dtype=np.float64), indexing="ij")
    if frame_xy:
        X, Y = cols, rows
        kx, ky = 2.0 * math.pi / n_x, 2.0 * math.pi / n_y
    else:
        X, Y = -rows, cols
        kx, ky = 2.0 * math.pi / n_y, 2.0 * math.pi / n_x
    ux = u0 * np.sin(kx * X) * np.cos(ky * Y)
    uy = -u0 * (kx / ky) * np.cos(kx * X) * np.sin(ky * Y)
    rho = 1.0 + uniform(seed, 0, n_x * n_y, -noise, noise).reshape(n_y, n_x)
    return rho.astype(np.float32), ux.astype(np.float32), uy.astype(np.float32)


def circles_mask(w: int, h: int, n: int, r_lo: float, r_hi: float, seed: int,
                 start: int = 1 << 40) -> np.ndarray:
    """n solid discs, centres uniform in the domain, radii U[r_lo, r_hi]."""
    solid = np.zeros((h, w), dtype=np.uint8)
    if n == 0:
        return solid
    u = uniform(seed, start, 3 * n).reshape(n, 3)
    cx, cy = u[:, 0] * w, u[:, 1] * h
    rr = r_lo + (r_hi - r_lo) * u[:, 2]
    for x0, y0, r in zip(cx, cy, rr):
        xa, xb = max(0, int(x0 - r) - 1), min(w, int(x0 + r) + 2)
        ya, yb = max(0, int(y0 - r) - 1), min(h, int(y0 + r) + 2)
        if xa >= xb or ya >= yb:
            continue
        yy, xx = np.mgrid[ya:yb, xa:xb]
        inside = (xx + 0.5 - x0) ** 2 + (yy + 0.5 - y0) ** 2 < r * r
        solid[ya:yb, xa:xb] |= inside.astype(np.uint8)
    return solid


@dataclass
class LatticeSpec:
    """One synthetic lattice: size, relaxation, boundaries, initial fields."""
    w: int
    h: int
    tau: float
    flags: int
    force: tuple = (0.0, 0.0)
    solid: np.ndarray | None = None
    rho: np.ndarray | None = None
    ux: np.ndarray | None = None
    uy: np.ndarray | None = None
    name: str = ""
    extra: dict = field(default_factory=dict)


CHANNEL_FLAGS = X_PERIODIC | Y_WALL | SOLID_HALFWAY | FRAME_XY
PERIODIC_FLAGS = X_PERIODIC | Y_PERIODIC | FRAME_XY


def taylor_green_spec(n: int = 256, tau: float = 0.8, seed: int = 1, u0: float = 0.02,
                      frame_xy: bool = True) -> LatticeSpec:
    """Plain D2Q9 BGK, n x n fully periodic Taylor-Green vortex."""
    rho, ux, uy = taylor_green(n, n, u0=u0, seed=seed, frame_xy=frame_xy)
    flags = X_PERIODIC | Y_PERIODIC | (FRAME_XY if frame_xy else 0)
    return LatticeSpec(n, n, tau, flags, rho=rho, ux=ux, uy=uy, name=f"taylor_green_{n}")


def channel_spec(n: int = 4096, tau: float = 0.56, n_obstacles: int = 64,
                 r_lo: float = 16.0, r_hi: float = 64.0, force: float = 1e-6,
                 seed: int = 2, h: int | None = None) -> LatticeSpec:
    """Channel: periodic in x, half-way bounce-back walls in y, body force
    along x, seeded circular obstacles; starts at rest (rho = 1, u = 0)."""
    h = n if h is None else h
    solid = circles_mask(n, h, n_obstacles, r_lo, r_hi, seed)
    rho = np.ones((h, n), dtype=np.float32)
    z = np.zeros((h, n), dtype=np.float32)
    return LatticeSpec(n, h, tau, CHANNEL_FLAGS, force=(force, 0.0), solid=solid,
                       rho=rho, ux=z, uy=z.copy(), name=f"channel_{n}x{h}")


def batch_specs(count: int = 512, lo: int = 64, hi: int = 1024, seed: int = 3,
                tau_lo: float = 0.52, tau_hi: float = 1.0, max_obstacles: int = 16):
    """Independent lattices of uneven sizes and relaxation times."""
    out = []
    u = uniform(seed, 0, 6 * count).reshape(count, 6)
    for k in range(count):
        w = int(lo + (hi - lo + 1) * u[k, 0])
        h = int(lo + (hi - lo + 1) * u[k, 1])
        tau = tau_lo + (tau_hi - tau_lo) * u[k, 2]
        n_obs = int((max_obstacles + 1) * u[k, 4])
        if u[k, 3] < 0.5:
            rho, ux, uy = taylor_green(w, h, u0=0.02, seed=seed * 1000003 + k)
            solid = circles_mask(w, h, n_obs, 2.0, max(3.0, min(w, h) / 16), seed * 7919 + k)
            spec = LatticeSpec(w, h, tau, PERIODIC_FLAGS | SOLID_HALFWAY, solid=solid,
                               rho=rho, ux=ux, uy=uy, name=f"tg_{k}")
        else:
            solid = circles_mask(w, h, n_obs, 2.0, max(3.0, min(w, h) / 16), seed * 7919 + k)
            rho = np.ones((h, w), dtype=np.float32)
            z = np.zeros((h, w), dtype=np.float32)
            spec = LatticeSpec(w, h, tau, CHANNEL_FLAGS, force=(1e-6, 0.0), solid=solid,
                               rho=rho, ux=z, uy=z.copy(), name=f"ch_{k}")
        out.append(spec)
    return out
