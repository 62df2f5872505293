"""CPU-rank simulation of a y-slab partition of one lattice — TEST
INFRASTRUCTURE ONLY.

The design the GPU path would use on several GPUs (the library itself steps
one lattice per GPU; several GPUs run replicas): rank r owns rows [r h / n, (r + 1) h / n) of a
lattice that is periodic in y, plus one halo row above and below.  Before
each step a rank sends the boundary rows of the three populations that stream
across each face (c_y = +1 up, c_y = -1 down, in the XY frame) to its
neighbours and receives theirs into its halo rows; then it steps its slab with
the oracle and keeps the interior rows.  Halo rows of the other six
populations are never read by an interior row, so only 3 * w values cross a
face per step.  The tests run this over torch.distributed (gloo) ranks on the
CPU and compare with the oracle's single-domain step, bit for bit.
"""
from __future__ import annotations

import numpy as np

from . import oracle

# D2Q9 directions with c_y = +1 (moving to the next row) and c_y = -1, in the
# XY frame (row = y): src/lbm.rs:217-227.
UP = (2, 5, 6)
DOWN = (4, 7, 8)
FLAG_Y_ZEROPAD = 0x0          # the slab's own y edges: the halo rows carry the neighbours


def slab_rows(h: int, rank: int, world: int) -> tuple[int, int]:
    return rank * h // world, (rank + 1) * h // world


def step_slab(f_halo: np.ndarray, *, tau: float, x_flags: int, frame_xy: int,
              **step_kw) -> np.ndarray:
    """One step of a slab with its halo rows (9, rows + 2, w); returns the
    interior rows (9, rows, w).  step_kw (force, collision, tau_minus) go to
    the oracle's step: the body force and the collision are local to a cell."""
    out = oracle.step(f_halo, 1, tau=tau, flags=x_flags | FLAG_Y_ZEROPAD | frame_xy, **step_kw)
    return out[:, 1:-1]


def run_rank(f_global: np.ndarray, nsteps: int, tau: float, x_flags: int, frame_xy: int, dist,
             solid=None, **step_kw):
    """The slab of this rank after nsteps steps, exchanging halos with its
    neighbours through `dist` (torch.distributed, any backend).  A solid mask
    (h, w) is static, so every rank cuts its slab's rows and the two halo
    rows from it without an exchange."""
    import torch
    rank, world = dist.get_rank(), dist.get_world_size()
    _, h, w = f_global.shape
    y0, y1 = slab_rows(h, rank, world)
    slab = np.ascontiguousarray(f_global[:, y0:y1])
    if solid is not None:
        rows = [(y0 - 1) % h] + list(range(y0, y1)) + [y1 % h]
        step_kw = dict(step_kw, solid=np.ascontiguousarray(np.asarray(solid)[rows]))
    above, below = (rank + 1) % world, (rank - 1) % world
    for _ in range(nsteps):
        halo = np.zeros((9, slab.shape[1] + 2, w), dtype=slab.dtype)
        halo[:, 1:-1] = slab
        # populations moving up leave through the top row into the rank above;
        # those moving down leave through the bottom row into the rank below
        send_up = torch.from_numpy(np.ascontiguousarray(slab[list(UP), -1]))
        send_dn = torch.from_numpy(np.ascontiguousarray(slab[list(DOWN), 0]))
        recv_from_below = torch.empty_like(send_up)
        recv_from_above = torch.empty_like(send_dn)
        reqs = [dist.isend(send_up, above), dist.isend(send_dn, below),
                dist.irecv(recv_from_below, below), dist.irecv(recv_from_above, above)]
        for r in reqs:
            r.wait()
        halo[list(UP), 0] = recv_from_below.numpy()
        halo[list(DOWN), -1] = recv_from_above.numpy()
        slab = step_slab(halo, tau=tau, x_flags=x_flags, frame_xy=frame_xy, **step_kw)
    return slab
