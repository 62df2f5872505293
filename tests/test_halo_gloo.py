"""The y-slab partition of one lattice (oracle/halo.py) over two and three gloo
ranks on the CPU: halo exchange of the three populations crossing each face,
then the slabs stepped independently, equals the single-domain step bit for
bit, also with a body force, TRT and full- or half-way solids on the faces."""
import os
import socket

import numpy as np
import pytest

import oracle
from oracle import halo

torch = pytest.importorskip("torch")
X_PERIODIC, Y_PERIODIC, SOLID_HALFWAY, FRAME_XY = 0x1, 0x4, 0x10, 0x20


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, f_path, out_dir, nsteps, tau, x_flags, step_kw, solid):
    import torch.distributed as dist
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank,
                            world_size=world)
    try:
        f = np.load(f_path)
        slab = halo.run_rank(f, nsteps, tau, x_flags, FRAME_XY, dist, solid=solid, **step_kw)
        np.save(os.path.join(out_dir, f"slab{rank}.npy"), slab)
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("world,h,step_kw,mask", [
    (2, 24, {}, None),
    (3, 31, {}, None),
    (2, 26, {"force": (2e-4, -1e-4), "collision": 1, "tau_minus": 0.9}, None),   # Guo force, TRT
    (3, 30, {}, "full-way"),
    (3, 30, {"force": (1e-4, 0.0)}, "half-way"),
])
def test_slab_partition_matches_single_domain(tmp_path, world, h, step_kw, mask):
    oracle.build()
    rng = np.random.default_rng(world)
    w, tau, nsteps = 20, 0.7, 6
    rho = (1 + 0.02 * rng.normal(size=(h, w))).astype(np.float32)
    ux = (0.05 * rng.normal(size=(h, w))).astype(np.float32)
    uy = (0.05 * rng.normal(size=(h, w))).astype(np.float32)
    f = oracle.equilibrium(rho, ux, uy)
    f_path = str(tmp_path / "f.npy")
    np.save(f_path, f)
    solid = None
    x_flags = X_PERIODIC
    if mask is not None:
        # about 15% solid cells, slab faces included (the mask is static and
        # every rank cuts its rows and halo rows from it)
        solid = (rng.uniform(size=(h, w)) < 0.15).astype(np.uint8)
        if mask == "half-way":
            x_flags |= SOLID_HALFWAY
    torch.multiprocessing.spawn(_rank_main, args=(world, _free_port(), f_path, str(tmp_path),
                                                  nsteps, tau, x_flags, dict(step_kw), solid),
                                nprocs=world, join=True)
    got = np.concatenate([np.load(tmp_path / f"slab{r}.npy") for r in range(world)], axis=1)
    ref = oracle.step(f, nsteps, tau=tau, flags=x_flags | Y_PERIODIC | FRAME_XY, solid=solid,
                      **step_kw)
    assert np.array_equal(got, ref)
