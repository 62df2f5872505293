"""The oracle against the golden fixtures and physics known-answer tests (CPU)."""
import glob
import math
import os

import numpy as np
import pytest

import oracle
from chemsim_gb300._lib import (COLLISION_TRT, FRAME_XY, SOLID_HALFWAY, X_PERIODIC,
                                X_WALL, Y_PERIODIC, Y_WALL)

GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz")))
W = np.array([16, 4, 4, 4, 4, 1, 1, 1, 1], dtype=np.float64) / 36.0
CX = np.array([0, 1, 0, -1, 0, 1, -1, -1, 1])
CY = np.array([0, 0, 1, 0, -1, 1, 1, -1, -1])
OPP = [0, 3, 4, 1, 2, 7, 8, 5, 6]


def random_state(w, h, dtype, seed=0, du=0.05):
    rng = np.random.default_rng(seed)
    rho = (1 + rng.uniform(-0.01, 0.01, (h, w))).astype(dtype)
    ux = rng.uniform(-du, du, (h, w)).astype(dtype)
    uy = rng.uniform(-du, du, (h, w)).astype(dtype)
    return oracle.equilibrium(rho, ux, uy)


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p) for p in GOLDEN])
@pytest.mark.parametrize("structured", [False, True])
def test_golden_bit_exact(oracle_lib, path, structured):
    g = np.load(path)
    f0 = oracle.equilibrium(g["rho0"], g["ux0"], g["uy0"])
    assert np.array_equal(f0, g["f0"])
    solid = g["solid"] if g["solid"].any() else None
    f = oracle.step(g["f0"], int(g["steps"]), tau=float(g["tau"]), solid=solid,
                    structured=structured)
    assert np.array_equal(f, g["f"])
    rho, ux, uy = oracle.moments(f)
    assert np.array_equal(rho, g["density"])
    assert np.array_equal(ux, g["vx"])
    assert np.array_equal(uy, g["vy"])


def test_golden_stream_only(oracle_lib):
    """Streaming alone: tau -> inf makes the collision the identity up to an
    absolute residue ~1e-31 on the zero-padded edge populations."""
    for path in GOLDEN:
        g = np.load(path)
        f = oracle.step(g["f0"], 1, tau=1e30)
        nz = g["stream1"] != 0
        assert np.array_equal(f[nz], g["stream1"][nz])
        assert np.max(np.abs(f[~nz])) < 1e-29


ALL_MODES = [
    0,
    X_PERIODIC | Y_PERIODIC,
    X_PERIODIC | Y_PERIODIC | FRAME_XY,
    X_PERIODIC | Y_WALL | SOLID_HALFWAY | FRAME_XY,
    X_WALL | Y_WALL | SOLID_HALFWAY,
    X_WALL | Y_PERIODIC,
    SOLID_HALFWAY,
]


@pytest.mark.parametrize("flags", ALL_MODES)
@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("collision", [0, COLLISION_TRT])
def test_structured_equals_fused(oracle_lib, flags, dtype, collision):
    w, h = 13, 11
    f0 = random_state(w, h, dtype, seed=5)
    solid = (np.random.default_rng(9).uniform(size=(h, w)) < 0.15).astype(np.uint8)
    kw = dict(tau=0.7, flags=flags, collision=collision, tau_minus=0.9, solid=solid,
              force=(1e-5, -2e-5))
    a = oracle.step(f0, 4, structured=False, **kw)
    b = oracle.step(f0, 4, structured=True, **kw)
    assert np.array_equal(a, b)


def test_equilibrium_invariant(oracle_lib):
    """KAT 1: a uniform equilibrium is invariant under periodic steps."""
    w = h = 16
    rho = np.full((h, w), 1.02)
    ux = np.full((h, w), 0.03)
    uy = np.full((h, w), -0.01)
    f0 = oracle.equilibrium(rho, ux, uy)
    f = oracle.step(f0, 20, tau=0.6, flags=X_PERIODIC | Y_PERIODIC)
    np.testing.assert_allclose(f, f0, rtol=1e-13, atol=1e-15)


@pytest.mark.parametrize("flags", [X_PERIODIC | Y_PERIODIC, X_PERIODIC | Y_PERIODIC | FRAME_XY])
def test_conservation_periodic(oracle_lib, flags):
    """KAT 2: mass and momentum are conserved (f64 to ~1e-12)."""
    f0 = random_state(24, 20, np.float64, seed=3)
    h0 = oracle.health(f0)
    f = oracle.step(f0, 50, tau=0.55, flags=flags)
    h1 = oracle.health(f)
    assert abs(h1["mass"] - h0["mass"]) <= 1e-12 * h0["mass"]
    assert abs(h1["momentum_x"] - h0["momentum_x"]) <= 1e-12 * h0["mass"]
    assert abs(h1["momentum_y"] - h0["momentum_y"]) <= 1e-12 * h0["mass"]


@pytest.mark.parametrize("frame_xy", [True, False])
def test_taylor_green_decay(oracle_lib, frame_xy):
    """KAT 3: TG kinetic energy decays as exp(-4 nu k^2 t), nu = (tau - 1/2)/3
    (src/lbm.rs:366-369 with dx = dt = 1)."""
    from chemsim_gb300.workloads import taylor_green
    n, tau, steps = 48, 0.8, 300
    rho, ux, uy = taylor_green(n, n, u0=0.01, noise=0.0, frame_xy=frame_xy)
    f0 = oracle.equilibrium(rho.astype(np.float64), ux.astype(np.float64), uy.astype(np.float64))
    flags = X_PERIODIC | Y_PERIODIC | (FRAME_XY if frame_xy else 0)
    f = oracle.step(f0, steps, tau=tau, flags=flags)
    _, vx0, vy0 = oracle.moments(f0)
    _, vx, vy = oracle.moments(f)
    e0 = np.sum(vx0 ** 2 + vy0 ** 2)
    e1 = np.sum(vx ** 2 + vy ** 2)
    nu = (tau - 0.5) / 3.0
    k2 = 2 * (2 * math.pi / n) ** 2
    expect = math.exp(-2 * nu * k2 * steps)
    assert abs(e1 / e0 - expect) / expect < 0.01


@pytest.mark.parametrize("frame_xy", [0, FRAME_XY])
def test_stream_delta_displacement(oracle_lib, frame_xy):
    """KAT 4: streaming moves a perturbation of plane i by its displacement."""
    w, h = 9, 7
    for i in range(9):
        f0 = np.broadcast_to(W[:, None, None], (9, h, w)).copy()
        f0[i, 3, 4] += 1e-3
        f = oracle.step(f0, 1, tau=1e300, flags=X_PERIODIC | Y_PERIODIC | frame_xy)
        d = f[i] - W[i]
        r, c = np.argwhere(np.abs(d) > 1e-9)[0]
        if frame_xy:
            assert (c - 4, r - 3) == (CX[i], CY[i])
        else:
            assert (r - 3, c - 4) == (-CX[i], CY[i])


def test_halfway_wall_reverses(oracle_lib):
    """KAT 5: a population leaving through a half-way wall returns reversed."""
    w, h = 6, 5
    f0 = np.broadcast_to(W[:, None, None], (9, h, w)).copy()
    f0[4, 0, 2] += 1e-3    # c = (0, -1) heading into the y = -1/2 wall (XY frame)
    f = oracle.step(f0, 1, tau=1e300, flags=X_PERIODIC | Y_WALL | FRAME_XY)
    assert abs(f[2, 0, 2] - W[2] - 1e-3) < 1e-12
    assert abs(f[4].sum() + f[2].sum() - (W[4] + W[2]) * w * h - 1e-3) < 1e-12


def test_wall_channel_zero_wall_momentum(oracle_lib):
    """Walls at rest: a forced channel develops a symmetric profile."""
    w, h = 4, 16
    f0 = np.broadcast_to(W[:, None, None], (9, h, w)).copy()
    f = oracle.step(f0, 400, tau=0.8, flags=X_PERIODIC | Y_WALL | FRAME_XY, force=(1e-5, 0.0))
    _, ux, uy = oracle.moments(f, force=(1e-5, 0.0))
    prof = ux[:, 0]
    np.testing.assert_allclose(prof, prof[::-1], rtol=1e-9, atol=1e-14)
    assert np.all(prof > 0)
    assert np.max(np.abs(uy)) < 1e-12


def test_force_adds_momentum(oracle_lib):
    """Guo forcing adds exactly F per cell per step to the momentum."""
    w, h, steps, F = 8, 8, 10, (2e-5, -1e-5)
    f0 = random_state(w, h, np.float64, seed=4, du=0.01)
    h0 = oracle.health(f0)
    f = oracle.step(f0, steps, tau=0.9, flags=X_PERIODIC | Y_PERIODIC, force=F)
    h1 = oracle.health(f)
    assert abs(h1["momentum_x"] - h0["momentum_x"] - steps * w * h * F[0]) < 1e-12
    assert abs(h1["momentum_y"] - h0["momentum_y"] - steps * w * h * F[1]) < 1e-12
    assert abs(h1["mass"] - h0["mass"]) < 1e-12


def test_trt_matches_reference_formula(oracle_lib):
    """TRT as src/lbm.rs:399-446 writes it (swap_equilibrium fills entries
    1..8 from the populations): one collision restated in numpy."""
    w, h = 5, 4
    f = random_state(w, h, np.float64, seed=8)
    tau_p, tau_m = 0.8, 1.1
    out = oracle.step(f, 1, tau=tau_p, tau_minus=tau_m, collision=COLLISION_TRT,
                      flags=X_PERIODIC | Y_PERIODIC)
    # streaming first (tau -> inf), then the collision formula
    s = oracle.step(f, 1, tau=1e300, flags=X_PERIODIC | Y_PERIODIC)
    rho, ux, uy = oracle.moments(s)
    feq = oracle.equilibrium(rho, ux, uy)
    sw = s[OPP]
    feq_sw = s[OPP].copy()
    feq_sw[0] = feq[0]
    om = ((s + sw) - (feq + feq_sw)) / tau_p + ((s - sw) - (feq - feq_sw)) / tau_m
    np.testing.assert_allclose(out, s + om * (-0.5), rtol=1e-13, atol=1e-15)


def test_reference_mode_solid_nodes_swap(oracle_lib):
    """Reference full-way mode: after streaming, a solid node holds the
    reversed populations, then collides (src/lbm.rs:741-751)."""
    w, h = 7, 6
    f0 = random_state(w, h, np.float64, seed=11)
    solid = np.zeros((h, w), np.uint8)
    solid[2, 3] = 1
    s = oracle.step(f0, 1, tau=1e300)
    s_solid = oracle.step(f0, 1, tau=1e300, solid=solid)
    np.testing.assert_array_equal(s_solid[:, 2, 3], s[OPP, 2, 3])
    mask = np.ones((h, w), bool)
    mask[2, 3] = False
    np.testing.assert_array_equal(s_solid[:, mask], s[:, mask])


def test_health_detects_instability(oracle_lib):
    f = random_state(6, 6, np.float64, seed=1)
    assert oracle.health(f)["nonfinite_count"] == 0
    assert oracle.health(f)["min_eq0"] > 0
    f[3, 2, 2] = np.nan
    assert oracle.health(f)["nonfinite_count"] == 1
    g = random_state(6, 6, np.float64, seed=1)
    g[1, 1, 1] += 5.0      # |u| > sqrt(2/3): f_eq[0] < 0, is_unstable()
    assert oracle.health(g)["min_eq0"] < 0
