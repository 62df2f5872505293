"""The y-slab partition of one lattice (oracle/halo.py) over two gloo ranks on
the CPU: halo exchange of the three populations crossing each face, then the
slabs stepped independently, equals the single-domain step bit for bit."""
import os
import socket

import numpy as np
import pytest

import oracle
from oracle import halo

torch = pytest.importorskip("torch")
X_PERIODIC, Y_PERIODIC, FRAME_XY = 0x1, 0x4, 0x20


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, f_path, out_dir, nsteps, tau, step_kw):
    import torch.distributed as dist
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank,
                            world_size=world)
    try:
        f = np.load(f_path)
        slab = halo.run_rank(f, nsteps, tau, X_PERIODIC, FRAME_XY, dist, **step_kw)
        np.save(os.path.join(out_dir, f"slab{rank}.npy"), slab)
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("world,h,step_kw", [
    (2, 24, {}),
    (3, 31, {}),
    (2, 26, {"force": (2e-4, -1e-4), "collision": 1, "tau_minus": 0.9}),   # Guo force, TRT
])
def test_slab_partition_matches_single_domain(tmp_path, world, h, step_kw):
    oracle.build()
    rng = np.random.default_rng(world)
    w, tau, nsteps = 20, 0.7, 6
    rho = (1 + 0.02 * rng.normal(size=(h, w))).astype(np.float32)
    ux = (0.05 * rng.normal(size=(h, w))).astype(np.float32)
    uy = (0.05 * rng.normal(size=(h, w))).astype(np.float32)
    f = oracle.equilibrium(rho, ux, uy)
    f_path = str(tmp_path / "f.npy")
    np.save(f_path, f)
    torch.multiprocessing.spawn(_rank_main, args=(world, _free_port(), f_path, str(tmp_path),
                                                  nsteps, tau, step_kw), nprocs=world, join=True)
    got = np.concatenate([np.load(tmp_path / f"slab{r}.npy") for r in range(world)], axis=1)
    ref = oracle.step(f, nsteps, tau=tau, flags=X_PERIODIC | Y_PERIODIC | FRAME_XY, **step_kw)
    assert np.array_equal(got, ref)
