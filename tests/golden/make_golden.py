#!/usr/bin/env python3
"""Generate the golden fixtures of the D2Q9 step (tests/golden/*.npz).

The reference (taktoa/chemsim, Rust over ArrayFire 3.6) cannot run here and
ships no golden data.  This script is a second, independent restatement of
its hot path, written against ArrayFire's semantics rather than per cell:
every lbm.rs expression becomes the numpy array operation ArrayFire would
run, in f32, one rounding per operation:

  Matrix::new(slice, (w, h)) -> array[h, w] with A[y, x] = slice[y*w + x]
                                (af::Array::new + af::transpose, src/matrix.rs:24-30)
  af::convolve2(f, K, DEFAULT, SPATIAL)
                             -> scipy.signal.convolve2d(f, K, mode="same",
                                boundary="fill"): true convolution, same size,
                                zeros outside (ArrayFire documents convolve2
                                as convolution, i.e. with the kernel flipped)
  af::replace(a, cond, b)    -> np.where(cond, a, b)
  Matrix::recip              -> np.float32(1) / x   (src/matrix.rs:133-136)

The C++ oracle (oracle/lbm_oracle.cpp) must reproduce these arrays bit for
bit.  Run:  python tests/golden/make_golden.py  (writes next to this file).
"""
from __future__ import annotations

import os

import numpy as np
from scipy.signal import convolve2d

F = np.float32
HERE = os.path.dirname(os.path.abspath(__file__))

# src/lbm.rs:205-215
WS = [F(16.0) / F(36.0), F(4.0) / F(36.0), F(4.0) / F(36.0), F(4.0) / F(36.0),
      F(4.0) / F(36.0), F(1.0) / F(36.0), F(1.0) / F(36.0), F(1.0) / F(36.0),
      F(1.0) / F(36.0)]
# src/lbm.rs:217-227
CS = [(0.0, 0.0), (1.0, 0.0), (0.0, 1.0), (-1.0, 0.0), (0.0, -1.0),
      (1.0, 1.0), (-1.0, 1.0), (-1.0, -1.0), (1.0, -1.0)]
# src/lbm.rs:229-269, each passed through make_m -> Matrix::new(&temp, (3, 3))
MS = [
    [0, 0, 0, 0, 1, 0, 0, 0, 0],
    [0, 0, 0, 1, 0, 0, 0, 0, 0],
    [0, 0, 0, 0, 0, 0, 0, 1, 0],
    [0, 0, 0, 0, 0, 1, 0, 0, 0],
    [0, 1, 0, 0, 0, 0, 0, 0, 0],
    [0, 0, 0, 0, 0, 0, 1, 0, 0],
    [0, 0, 0, 0, 0, 0, 0, 0, 1],
    [0, 0, 1, 0, 0, 0, 0, 0, 0],
    [1, 0, 0, 0, 0, 0, 0, 0, 0],
]


def matrix_new(slice_, dims):
    """Matrix::new (src/matrix.rs:24-30): Array::new(slice, [w, h]) is
    column-major with w rows; af::transpose then gives [h, w] with
    M[r, c] = slice[r*w + c]."""
    w, h = dims
    a = np.asarray(slice_, dtype=F).reshape(h, w, order="C")
    col_major_w_by_h = a.T          # dims [w, h], element (i, j) = slice[i + j*w]
    return np.ascontiguousarray(col_major_w_by_h.T)   # af::transpose


def stencils():
    return [matrix_new(m, (3, 3)) for m in MS]


def compute_equilibrium(density, vx, vy, dx=F(1), dt=F(1)):
    """src/lbm.rs:43-71."""
    v2 = vx * vx + vy * vy
    cs = F(dx) / (np.sqrt(F(3.0)) * F(dt))
    cs2 = cs * cs
    cs4 = cs2 * cs2
    k1 = F(1.0) / cs2
    k2 = F(1.0) / (F(2.0) * cs4)
    k3 = F(-1.0) / (F(2.0) * cs2)
    out = []
    for w, (cx, cy) in zip(WS, CS):
        vc = vx * F(cx) + vy * F(cy)
        vc2 = vc * vc
        s = np.full(density.shape, F(1.0), dtype=F)
        s = s + vc * k1
        s = s + vc2 * k2
        s = s + v2 * k3
        out.append((density * w) * s)
    return out


def density(pops):
    r = np.zeros(pops[0].shape, dtype=F)          # Matrix::new_filled(0.0)
    for p in pops:
        r += p                                    # src/lbm.rs:119
    return r


def momentum_density(pops):
    mx = np.zeros(pops[0].shape, dtype=F)
    my = np.zeros(pops[0].shape, dtype=F)
    for (cx, cy), p in zip(CS, pops):
        mx = mx + p * F(cx)
        my = my + p * F(cy)
    return mx, my


def velocity(pops):
    inv = np.full(pops[0].shape, F(1.0), dtype=F) / density(pops)   # recip
    mx, my = momentum_density(pops)
    return inv * mx, inv * my


def stream(pops):
    """src/lbm.rs:716-729."""
    out = []
    for s, p in zip(stencils(), pops):
        k = s.T                                    # stencil.transpose()
        r = convolve2d(p, k, mode="same", boundary="fill", fillvalue=0)
        out.append(r.astype(F))
    return out


def swap_populations(pops):
    """src/lbm.rs:298-309."""
    opp = [0, 3, 4, 1, 2, 7, 8, 5, 6]
    return [pops[o] for o in opp]


def bounce_back(pops, geometry):
    """src/lbm.rs:741-751: replace(sw, geometry, pop) keeps sw where the
    geometry is true and takes pop elsewhere."""
    sw = swap_populations(pops)
    return [np.where(geometry, s, p) for s, p in zip(sw, pops)]


def collide_bgk(pops, tau, dt=F(1)):
    """src/lbm.rs:731-739 + 350-364."""
    vx, vy = velocity(pops)
    feq = compute_equilibrium(density(pops), vx, vy)
    factor = -F(dt) / F(tau)
    return [f + (f - e) * factor for f, e in zip(pops, feq)]


def step(pops, geometry, tau):
    """src/lbm.rs:694-714."""
    pops = stream(pops)
    pops = bounce_back(pops, geometry)
    return collide_bgk(pops, tau)


def make_case(name, w, h, steps, tau, seed, n_solid):
    rng = np.random.default_rng(seed)
    rho = (1.0 + rng.uniform(-0.01, 0.01, size=w * h)).astype(F)
    ux = rng.uniform(-0.05, 0.05, size=w * h).astype(F)
    uy = rng.uniform(-0.05, 0.05, size=w * h).astype(F)
    geom_flat = np.zeros(w * h, dtype=bool)
    if n_solid:
        geom_flat[rng.choice(w * h, size=n_solid, replace=False)] = True
    # initial_state builds host vectors indexed y*w + x, then Matrix::new
    # (src/main.rs:201-265) and the geometry via Array::new + transpose
    # (src/main.rs:269-312).
    R, UX, UY = (matrix_new(a, (w, h)) for a in (rho, ux, uy))
    G = matrix_new(geom_flat.astype(F), (w, h)).astype(bool)
    pops0 = compute_equilibrium(R, UX, UY)
    pops = pops0
    for _ in range(steps):
        pops = step(pops, G, tau)
    vx, vy = velocity(pops)
    out = dict(
        w=np.int32(w), h=np.int32(h), steps=np.int32(steps), tau=F(tau),
        rho0=R, ux0=UX, uy0=UY, solid=G.astype(np.uint8),
        f0=np.stack(pops0), f=np.stack(pops),
        density=density(pops), vx=vx, vy=vy,
        stream1=np.stack(stream(pops0)),
    )
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)
    return out


CASES = [
    # (name, w, h, steps, tau, seed, solid cells)
    ("lbmrs_12x9_solid", 12, 9, 6, 0.8, 1, 14),
    ("lbmrs_16x16_open", 16, 16, 10, 0.6, 2, 0),
    ("lbmrs_7x13_solid", 7, 13, 4, 1.3, 3, 20),
]


if __name__ == "__main__":
    for c in CASES:
        make_case(*c)
        print("wrote", c[0])
