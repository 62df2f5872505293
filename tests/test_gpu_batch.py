"""Batched lattices (lbm_batch_*) against single lattices and the oracle."""
import json

import numpy as np
import pytest

import oracle
from chemsim_gb300 import lbm
from chemsim_gb300.lbm import F32, FAST, FRAME_XY, Batch, Lattice
from chemsim_gb300.workloads import LatticeSpec, batch_specs

pytestmark = pytest.mark.gpu


def _specs(count=10, seed=7):
    specs = batch_specs(count, lo=20, hi=300, seed=seed, max_obstacles=4)
    # a few shapes that stress the tiling: 1-tile rows, partial tiles, tall
    extra = [(33, 70), (1, 9), (129, 5), (256, 64)]
    for k, (w, h) in enumerate(extra):
        s = batch_specs(1, lo=w, hi=w, seed=100 + k)[0]
        specs.append(LatticeSpec(w, h, 0.7, s.flags, force=s.force, solid=None,
                                 rho=np.ones((h, w), np.float32),
                                 ux=np.full((h, w), 0.01, np.float32),
                                 uy=np.zeros((h, w), np.float32), name=f"extra{k}"))
    return specs


def _single(spec, flags, steps):
    with Lattice(spec.w, spec.h, spec.tau, F32, (spec.flags & ~(FRAME_XY | FAST)) | flags) as lat:
        lat.set_force(*spec.force)
        if spec.solid is not None and spec.solid.any():
            lat.set_geometry(spec.solid)
        lat.init_equilibrium(spec.rho, spec.ux, spec.uy)
        lat.step(steps)
        return lat.get_populations(), lat.time()


def _init(batch, specs):
    for m, sp in zip(batch.members, specs):
        m.init_equilibrium(sp.rho, sp.ux, sp.uy)


def test_batch_equals_single_lattices(gpu):
    specs = _specs()
    with Batch(specs, FRAME_XY | FAST) as b:
        _init(b, specs)
        b.step(37)                    # two 16-step graph replays + 5 single steps
        for m, sp in zip(b.members, specs):
            ref, (t_ref, n_ref) = _single(sp, FRAME_XY | FAST, 37)
            assert np.array_equal(m.get_populations(), ref), sp.name
            assert m.time() == (t_ref, n_ref)


def test_batch_strict_equals_oracle(gpu):
    specs = _specs(4, seed=11)
    with Batch(specs, FRAME_XY) as b:
        _init(b, specs)
        b.step(9)
        for m, sp in zip(b.members, specs):
            f0 = oracle.equilibrium(sp.rho, sp.ux, sp.uy)
            solid = sp.solid if sp.solid is not None and sp.solid.any() else None
            ref = oracle.step(f0, 9, tau=float(np.float32(sp.tau)), flags=sp.flags | FRAME_XY,
                              solid=solid, force=tuple(float(np.float32(v)) for v in sp.force))
            assert np.array_equal(m.get_populations(), ref), sp.name


def test_member_calls_between_batch_steps(gpu):
    """A member stepped on its own, re-forced and re-shaped between batch steps
    stays consistent with the same sequence on a single lattice."""
    specs = _specs(3, seed=5)
    sp = specs[0]
    with Batch(specs, FRAME_XY | FAST) as b:
        _init(b, specs)
        b.step(4)
        m = b[0]
        m.step(3)                                # odd: parities differ now
        m.set_force(2e-6, -1e-6)
        m.set_tile(2, 8)
        b.step(20)
        got = m.get_populations()
    with Lattice(sp.w, sp.h, sp.tau, F32, (sp.flags & ~(FRAME_XY | FAST)) | FRAME_XY | FAST) as lat:
        lat.set_force(*sp.force)
        if sp.solid is not None and sp.solid.any():
            lat.set_geometry(sp.solid)
        lat.init_equilibrium(sp.rho, sp.ux, sp.uy)
        lat.step(7)
        lat.set_force(2e-6, -1e-6)
        lat.step(20)
        assert np.array_equal(got, lat.get_populations())


def test_autotune_writes_and_reuses_cache(gpu, tmp_path):
    specs = _specs(6, seed=21)
    cache = tmp_path / "tiles.json"
    with Batch(specs, FRAME_XY | FAST) as b:
        _init(b, specs)
        before = [m.get_populations() for m in b.members]
        b.autotune(str(cache), steps_per_trial=4)
        # tuning steps the members, then restores their state exactly
        for m, f in zip(b.members, before):
            assert np.array_equal(m.get_populations(), f)
            assert m.time() == (0.0, 0)
        doc = json.loads(cache.read_text())
        entries = doc["lbm_batch_autotune"]
        assert len(entries) == 1 and entries[0]["V"] in (2, 4)
        assert entries[0]["mlups_v2"] > 0 and entries[0]["mlups_v4"] > 0
        chosen = entries[0]["V"]
        first = cache.read_text()
        b.autotune(str(cache))            # cached: nothing timed, file unchanged
        assert cache.read_text() == first
        b.step(21)
        for m, sp in zip(b.members, specs):
            ref, _ = _single(sp, FRAME_XY | FAST, 21)
            assert np.array_equal(m.get_populations(), ref), sp.name
    # a new batch of the same mode takes the cached width without timing
    with Batch(specs[:2], FRAME_XY | FAST) as b:
        b.autotune(str(cache))
        assert cache.read_text() == first
        assert b.tile() == chosen


@pytest.mark.parametrize("tile", [2, 4])
def test_batch_tile_widths_equal_single_lattices(gpu, tile):
    """Both batch kernels (2 and 4 cells per thread), with members whose own
    tile width differs from the batch's (reset to it at the next step)."""
    specs = _specs(8, seed=13)
    with Batch(specs, FRAME_XY | FAST) as b:
        _init(b, specs)
        b.set_tile(tile)
        b.members[1].set_tile(8 if tile == 4 else 4, 2)
        b.step(19)
        for m, sp in zip(b.members, specs):
            ref, _ = _single(sp, FRAME_XY | FAST, 19)
            assert np.array_equal(m.get_populations(), ref), sp.name
        assert b.tile() == tile
    with Batch(specs[:1], FRAME_XY | FAST) as b, pytest.raises(lbm.LBMError):
        b.set_tile(8)


def test_batch_rejects_bad_flags(gpu):
    specs = _specs(2)
    with pytest.raises(lbm.LBMError):
        Batch(specs, FRAME_XY | FAST | 0x01)
