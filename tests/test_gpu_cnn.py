"""The correction network (tcgen05 convolutions) and the coarse-grid calls
against the CPU oracles."""
import numpy as np
import pytest

import oracle
from oracle import cnn_oracle as co
from chemsim_gb300 import lbm
from chemsim_gb300.lbm import F32, FAST, FRAME_XY, SOLID_HALFWAY, X_PERIODIC, Y_WALL, Lattice

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

from chemsim_gb300.learned import (CorrectionNet, apply_correction, coarse_run,  # noqa: E402
                                   features, restrict, target)


def _rel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / max(np.linalg.norm(b), 1e-30))


@pytest.fixture(scope="module")
def small_case():
    B, H, W = 2, 8, 128
    rng = np.random.default_rng(0)
    p = co.init_params(1).astype(np.float32)
    x = rng.normal(size=(B, 4, H, W)).astype(np.float32)
    t = (rng.normal(size=(B, 9, H, W)) * 0.1).astype(np.float32)
    return p, x, t


def test_forward_matches_oracle(gpu, small_case):
    p, x, _ = small_case
    B, _, H, W = x.shape
    with CorrectionNet(H, W, B) as net:
        net.set_params(p)
        assert np.array_equal(net.get_params(), p)
        out = torch.empty((B, 9, H, W), device="cuda")
        net.forward(torch.from_numpy(x).cuda(), out)
        ref, _ = co.forward(p.astype(np.float64), x.astype(np.float64))
        # bf16 activations: the oracle rounds at the same points; sums differ
        # in order only (f32 on the tensor cores vs f64)
        assert _rel(out.cpu().numpy(), ref) < 2e-3


def test_gradients_match_oracle(gpu, small_case):
    p, x, t = small_case
    B, _, H, W = x.shape
    with CorrectionNet(H, W, B) as net:
        net.set_params(p)
        loss, g = net.gradients(torch.from_numpy(x).cuda(), torch.from_numpy(t).cuda())
        lref, gref = co.gradients(p.astype(np.float64), x.astype(np.float64), t.astype(np.float64))
        assert abs(loss - lref) <= 1e-3 * lref
        k = 0
        for ci, cout in zip(co.CIN, co.COUT):
            for n in (9 * ci * cout, cout):
                assert _rel(g[k:k + n], gref[k:k + n]) < 5e-3, k
                k += n


def test_training_reduces_loss(gpu):
    B, H, W = 2, 16, 128
    rng = np.random.default_rng(4)
    x = rng.normal(size=(B, 4, H, W)).astype(np.float32)
    # a target the network can represent: a smoothed function of the input
    t = np.tanh(x[:, :3].mean(axis=1, keepdims=True)).repeat(9, axis=1).astype(np.float32) * 0.3
    with CorrectionNet(H, W, B, seed=7) as net:
        xd, td = torch.from_numpy(x).cuda(), torch.from_numpy(t).cuda()
        first = net.train_step(xd, td, 1e-3)
        for _ in range(150):
            last = net.train_step(xd, td, 1e-3)
        assert last < 0.3 * first


def test_batch_bounds_checked(gpu):
    with CorrectionNet(8, 128, 2) as net:
        x = torch.zeros((3, 4, 8, 128), device="cuda")
        out = torch.zeros((3, 9, 8, 128), device="cuda")
        with pytest.raises(lbm.LBMError):
            net.forward(x, out)
    with pytest.raises(lbm.LBMError):
        CorrectionNet(8, 100, 1)          # width must be a multiple of 128


def _channel(w, h, seed):
    from chemsim_gb300.workloads import channel_spec
    return channel_spec(w, n_obstacles=3, r_lo=4, r_hi=9, force=1e-5, seed=seed, h=h)


def test_restrict_matches_block_average(gpu):
    spec = _channel(128, 64, 3)
    flags = X_PERIODIC | Y_WALL | SOLID_HALFWAY | FRAME_XY | FAST
    with Lattice(128, 64, 0.6, F32, flags) as fine, Lattice(32, 16, 0.525, F32, flags) as coarse:
        fine.set_force(*spec.force)
        fine.set_geometry(spec.solid)
        fine.init_equilibrium(spec.rho, spec.ux, spec.uy)
        fine.step(50)
        rho, ux, uy = fine.moments()
        coarse.set_force(4 * spec.force[0], 0.0)
        restrict(fine, coarse, 4)
        got = coarse.get_populations()
        fl = (spec.solid == 0).reshape(16, 4, 32, 4)
        r4 = rho.reshape(16, 4, 32, 4).astype(np.float64)
        n = fl.sum(axis=(1, 3))
        sr = (r4 * fl).sum(axis=(1, 3))
        rc = np.where(n > 0, sr / np.maximum(n, 1), 1.0)
        jx = (r4 * ux.reshape(16, 4, 32, 4) * fl).sum(axis=(1, 3))
        jy = (r4 * uy.reshape(16, 4, 32, 4) * fl).sum(axis=(1, 3))
        vx = np.where(sr > 0, jx / np.where(sr > 0, sr, 1), 0) + np.where(n > 0, 0.5 * 4 * spec.force[0] / rc, 0)
        vy = np.where(sr > 0, jy / np.where(sr > 0, sr, 1), 0)
        ref = oracle.equilibrium(rc.astype(np.float32), vx.astype(np.float32), vy.astype(np.float32))
        assert np.max(np.abs(got - ref)) < 2e-6


def test_features_apply_target(gpu):
    spec = _channel(128, 32, 5)
    flags = X_PERIODIC | Y_WALL | SOLID_HALFWAY | FRAME_XY | FAST
    with Lattice(128, 32, 0.6, F32, flags) as a, Lattice(128, 32, 0.6, F32, flags) as b:
        for lat in (a, b):
            lat.set_geometry(spec.solid)
        rng = np.random.default_rng(9)
        rho = (1 + 0.01 * rng.normal(size=(32, 128))).astype(np.float32)
        ux = (0.01 * rng.normal(size=(32, 128))).astype(np.float32)
        uy = (0.01 * rng.normal(size=(32, 128))).astype(np.float32)
        a.init_equilibrium(rho, ux, uy)
        b.init_equilibrium(np.ones_like(rho), ux * 0, uy * 0)
        solid = spec.solid.astype(bool)
        x = torch.zeros((2, 4, 32, 128), device="cuda")
        features(a, x, 1, 100.0, 50.0)
        r, vx, vy = a.moments()
        xs = x[1].cpu().numpy()
        np.testing.assert_allclose(xs[0], np.where(solid, 0, (r - 1) * 100), rtol=1e-6, atol=1e-6)
        np.testing.assert_allclose(xs[1], np.where(solid, 0, vx * 50), rtol=1e-6, atol=1e-7)
        np.testing.assert_array_equal(xs[3], solid.astype(np.float32))
        assert float(x[0].abs().sum()) == 0.0
        t = torch.zeros((1, 9, 32, 128), device="cuda")
        target(a, b, t, 0, 1e-3)
        fa, fb = a.get_populations().astype(np.float64), b.get_populations().astype(np.float64)
        cx = np.array([0, 1, 0, -1, 0, 1, -1, -1, 1])[:, None, None]
        cy = np.array([0, 0, 1, 0, -1, 1, 1, -1, -1])[:, None, None]
        ra = fa.sum(axis=0)
        uxa, uya = (fa * cx).sum(axis=0) / ra, (fa * cy).sum(axis=0) / ra
        tg = t[0].cpu().numpy().astype(np.float64)
        rb = fb.sum(axis=0)
        # b is at rest: the target is f_eq(rho_b, u(a)) - f_eq(rho_b, 0), over the scale
        shift = (oracle.equilibrium(rb.astype(np.float32), uxa.astype(np.float32), uya.astype(np.float32))
                 .astype(np.float64) - oracle.equilibrium(rb.astype(np.float32), 0 * rho, 0 * rho))
        np.testing.assert_allclose(tg, np.where(solid[None], 0, shift / 1e-3), rtol=0, atol=2e-4)
        apply_correction(b, t, 0, 1e-3)
        got = b.get_populations().astype(np.float64)
        w = np.array([16, 4, 4, 4, 4, 1, 1, 1, 1], np.float64)[:, None, None] / 36
        d = tg * 1e-3
        np.testing.assert_allclose(got, np.where(solid[None], fb, fb + d - w * d.sum(axis=0)),
                                   rtol=0, atol=3e-7)
        # mass per fluid cell unchanged by the correction
        np.testing.assert_allclose(got.sum(axis=0), fb.sum(axis=0), rtol=0, atol=1e-6)
        # clamped correction: each population change limited to +-max_abs first
        b.init_equilibrium(np.ones_like(rho), ux * 0, uy * 0)
        apply_correction(b, t, 0, 1e-3, max_abs=2e-4)
        got = b.get_populations().astype(np.float64)
        dc = np.clip(d, -2e-4, 2e-4)
        np.testing.assert_allclose(got, np.where(solid[None], fb, fb + dc - w * dc.sum(axis=0)),
                                   rtol=0, atol=3e-7)


def test_weights_save_load(gpu, tmp_path):
    with CorrectionNet(8, 128, 1, seed=1) as a, CorrectionNet(8, 128, 1, seed=2) as b:
        assert not np.array_equal(a.get_params(), b.get_params())
        a.save(tmp_path / "w.bin")
        b.load(tmp_path / "w.bin")
        assert np.array_equal(a.get_params(), b.get_params())
        (tmp_path / "bad.bin").write_bytes(b"LBMCNN01" + b"\0" * 8)
        with pytest.raises(lbm.LBMError):
            b.load(tmp_path / "bad.bin")


def _coarse_pair(seed):
    spec = _channel(128, 32, seed)
    flags = X_PERIODIC | Y_WALL | SOLID_HALFWAY | FRAME_XY | FAST
    lats = []
    for _ in range(2):
        lat = Lattice(128, 32, 0.55, F32, flags)
        lat.set_force(*spec.force)
        lat.set_geometry(spec.solid)
        lat.init_equilibrium(spec.rho, spec.ux, spec.uy)
        lats.append(lat)
    return lats


def test_coarse_run_with_zero_scale_is_plain_stepping(gpu):
    a, b = _coarse_pair(6)
    with CorrectionNet(32, 128, 1, seed=3) as net, a, b:
        assert coarse_run(a, net, 30, 8, 0.0, 100.0, 0.0, check_every=1) is None
        b.step(30)
        assert np.array_equal(a.get_populations(), b.get_populations())
        assert a.time()[1] == 30


def test_coarse_run_falls_back_on_a_failed_check(gpu):
    a, _ = _coarse_pair(7)
    with CorrectionNet(32, 128, 1, seed=3) as net, a:
        f = a.get_populations()
        f[0, 10, 40] = np.nan                # a planted non-finite population
        a.set_populations(f)
        assert coarse_run(a, net, 64, 4, 0.0, 100.0, 1e-6, check_every=1) == 4


def test_learned_correction_beats_coarse_only(gpu):
    """The coarse-plus-correction run against the coarse-only run of a held-out
    geometry (fine 512^2, coarse 128^2, 4000 fine-equivalent steps): the
    trained correction lowers the velocity L2 error at every checkpoint and
    the corrected run stays healthy (no fine-grid fallback)."""
    from chemsim_gb300.learned import CorrectionConfig, run_correction_experiment
    cfg = CorrectionConfig(fine=512, n_obstacles=8, r_lo=6, r_hi=16, pairs=1000, horizon_fine=4000,
                           batch=8, buffer=1000, final_iters=800, checkpoints=8, train_lattices=8)
    res = run_correction_experiment(cfg)
    ev = res["evaluation"]
    corr = ev["corrected"][0]
    print({"coarse_only": ev["u_l2_coarse_only"], "corrected": corr["u_l2"]})
    assert corr["fallback_triggered_at_fine_step"] is None
    assert all(c < b for c, b in zip(corr["u_l2"], ev["u_l2_coarse_only"]))


def test_bounded_wait_times_out_and_context_survives(gpu):
    """A wait on an mbarrier that nothing signals gives up after its poll
    limit and reports it; the device keeps working afterwards."""
    import ctypes
    lib = lbm._lib.load()
    out = ctypes.c_int(0)
    lbm._lib.check(lib.lbm_selftest_wait_timeout(1000, ctypes.byref(out)))
    assert out.value == 1
    with pytest.raises(lbm.LBMError):
        lbm._lib.check(lib.lbm_selftest_wait_timeout(0, ctypes.byref(out)))
    with Lattice(64, 32, 0.8, F32, X_PERIODIC | Y_WALL | FRAME_XY) as lat:
        lat.step(5)
        assert not lat.health()["unstable"]
