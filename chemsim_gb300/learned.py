"""Learned coarse-grid correction: the network and the lattice-side calls.

Thin wrappers over liblbm_cuda.so (lbm_cnn_*, lbm_restrict, lbm_coarse_*);
device tensors are torch CUDA tensors (plumbing only — every computation runs
in the library's kernels).
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from ._lib import check


def _ptr(t) -> ctypes.c_void_p:
    if not t.is_cuda or not t.is_contiguous() or t.dtype.itemsize != 4:
        raise ValueError("expected a contiguous 32-bit CUDA tensor")
    return ctypes.c_void_p(t.data_ptr())


class CorrectionNet:
    """4 x (3x3 conv), 4 -> 32 -> 32 -> 32 -> 9, GELU (lbm_cnn_*)."""

    def __init__(self, h: int, w: int, max_batch: int, seed: int = 0):
        self._lib = _lib.load()
        self._n = ctypes.c_void_p()
        check(self._lib.lbm_cnn_create(int(h), int(w), int(max_batch), ctypes.c_uint64(seed),
                                       ctypes.byref(self._n)))
        self.h, self.w, self.max_batch = int(h), int(w), int(max_batch)
        cnt = ctypes.c_int64()
        check(self._lib.lbm_cnn_param_count(self._n, ctypes.byref(cnt)))
        self.nparams = int(cnt.value)

    def close(self):
        if self._n:
            self._lib.lbm_cnn_destroy(self._n)
            self._n = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def get_params(self) -> np.ndarray:
        out = np.empty(self.nparams, dtype=np.float32)
        check(self._lib.lbm_cnn_get_params(self._n, out.ctypes.data_as(ctypes.c_void_p)))
        return out

    def set_params(self, params):
        p = np.ascontiguousarray(params, dtype=np.float32)
        if p.size != self.nparams:
            raise ValueError(f"expected {self.nparams} parameters")
        check(self._lib.lbm_cnn_set_params(self._n, p.ctypes.data_as(ctypes.c_void_p)))

    def forward(self, x, out):
        check(self._lib.lbm_cnn_forward(self._n, _ptr(x), int(x.shape[0]), _ptr(out)))

    def gradients(self, x, target):
        loss = ctypes.c_float()
        g = np.empty(self.nparams, dtype=np.float32)
        check(self._lib.lbm_cnn_gradients(self._n, _ptr(x), _ptr(target), int(x.shape[0]),
                                          ctypes.byref(loss), g.ctypes.data_as(ctypes.c_void_p)))
        return float(loss.value), g

    def train_step(self, x, target, lr: float) -> float:
        loss = ctypes.c_float()
        check(self._lib.lbm_cnn_train_step(self._n, _ptr(x), _ptr(target), int(x.shape[0]),
                                           float(lr), ctypes.byref(loss)))
        return float(loss.value)

    def synchronize(self):
        check(self._lib.lbm_cnn_synchronize(self._n))


def restrict(fine, coarse, factor: int = 4):
    check(_lib.load().lbm_restrict(fine.handle, coarse.handle, int(factor)))


def features(lat, x, image: int, s_rho: float, s_u: float):
    check(_lib.load().lbm_coarse_features(lat.handle, float(s_rho), float(s_u), int(image), _ptr(x)))


def apply_correction(lat, corr, image: int, scale: float):
    check(_lib.load().lbm_coarse_apply(lat.handle, _ptr(corr), int(image), float(scale)))


def target(ref, cur, t, image: int, scale: float):
    check(_lib.load().lbm_coarse_target(ref.handle, cur.handle, float(scale), int(image), _ptr(t)))


# ---------------------------------------------------------------------------
# the coarse-plus-correction experiment
# ---------------------------------------------------------------------------

from dataclasses import dataclass, field  # noqa: E402
import time  # noqa: E402


@dataclass
class CorrectionConfig:
    """Fine channel lattice (periodic x, half-way walls y, body force, seeded
    obstacles) against a factor-x coarser lattice of equal viscosity under
    acoustic scaling: tau_c = 1/2 + (tau_f - 1/2) / factor, F_c = factor * F_f."""
    fine: int = 2048
    factor: int = 4
    tau_fine: float = 0.55
    force_fine: float = 1e-6
    n_obstacles: int = 64
    r_lo: float = 8.0
    r_hi: float = 32.0
    k: int = 8                    # coarse steps between corrections
    train_lattices: int = 8
    pairs: int = 4000
    horizon_fine: int = 20000     # fine-equivalent steps of the evaluation
    batch: int = 8
    buffer: int = 512
    iters_per_round: int = 2
    final_iters: int = 400
    lr: float = 1e-3
    s_rho: float = 1000.0
    s_u: float = 100.0
    s_out: float = 1e-4
    seed: int = 11
    eval_seed: int = 9999
    checkpoints: int = 10
    check_every: int = 64
    mass_tolerance: float = 1e-3
    extra: dict = field(default_factory=dict)

    @property
    def coarse(self) -> int:
        return self.fine // self.factor

    @property
    def tau_coarse(self) -> float:
        return 0.5 + (self.tau_fine - 0.5) / self.factor


def coarse_geometry(solid, factor: int) -> np.ndarray:
    """A coarse cell is solid when at least half of its fine cells are."""
    h, w = solid.shape
    blocks = solid.reshape(h // factor, factor, w // factor, factor).astype(np.int32)
    return (blocks.sum(axis=(1, 3)) * 2 >= factor * factor).astype(np.uint8)


def _block_velocity(rho, ux, uy, solid, factor):
    """Fluid-weighted block averages of rho u / rho on the coarse grid."""
    h, w = rho.shape
    fl = (solid == 0).reshape(h // factor, factor, w // factor, factor)
    r = rho.astype(np.float64).reshape(fl.shape) * fl
    sr = r.sum(axis=(1, 3))
    jx = (r * ux.reshape(fl.shape)).sum(axis=(1, 3))
    jy = (r * uy.reshape(fl.shape)).sum(axis=(1, 3))
    with np.errstate(invalid="ignore", divide="ignore"):
        return np.where(sr > 0, jx / sr, 0.0), np.where(sr > 0, jy / sr, 0.0)


def _l2(cx, cy, rx, ry, mask):
    num = np.sqrt(np.sum(((cx - rx) ** 2 + (cy - ry) ** 2)[mask]))
    den = np.sqrt(np.sum((rx ** 2 + ry ** 2)[mask]))
    return float(num / max(den, 1e-300))


def run_correction_experiment(cfg: CorrectionConfig, log=None) -> dict:
    """Generates snapshot pairs with the batched fine LBM, trains the network
    on the GPU, and judges coarse-only and coarse-plus-correction runs against
    the fine run of a held-out geometry.  Returns a result dict."""
    import torch
    from . import lbm
    from .workloads import CHANNEL_FLAGS, channel_spec
    say = log or (lambda *a: None)
    flags = CHANNEL_FLAGS | lbm.FAST
    nf, nc, fac = cfg.fine, cfg.coarse, cfg.factor
    force_c = cfg.force_fine * fac
    dev = torch.device("cuda")
    res = {"config": {k: v for k, v in cfg.__dict__.items() if k != "extra"},
           "tau_coarse": cfg.tau_coarse, "force_coarse": force_c}

    # ---- snapshot pairs from the batched fine LBM, online training ---------
    specs = [channel_spec(nf, tau=cfg.tau_fine, n_obstacles=cfg.n_obstacles, r_lo=cfg.r_lo,
                          r_hi=cfg.r_hi, force=cfg.force_fine, seed=cfg.seed + i)
             for i in range(cfg.train_lattices)]
    cmasks = [coarse_geometry(s.solid, fac) for s in specs]
    from .workloads import LatticeSpec
    cspecs = [LatticeSpec(nc, nc, cfg.tau_coarse, s.flags, force=(force_c, 0.0), solid=m)
              for s, m in zip(specs, cmasks)]
    fine_b = lbm.Batch(specs, lbm.FRAME_XY | lbm.FAST)
    cur_b = lbm.Batch(cspecs, lbm.FRAME_XY | lbm.FAST)
    refs = []
    for m in cmasks:
        r = lbm.Lattice(nc, nc, cfg.tau_coarse, lbm.F32, flags)
        r.set_force(force_c, 0.0)
        r.set_geometry(m)
        refs.append(r)
    net = CorrectionNet(nc, nc, max(cfg.batch, 1), seed=cfg.seed)
    xb = torch.zeros((cfg.buffer, 4, nc, nc), device=dev)
    tb = torch.zeros((cfg.buffer, 9, nc, nc), device=dev)
    rounds = max(1, cfg.pairs // cfg.train_lattices)
    spacing = max(cfg.k * fac, (cfg.horizon_fine * cfg.train_lattices) // max(cfg.pairs, 1))
    rng = np.random.default_rng(cfg.seed)
    filled, slot, losses = 0, 0, []
    t_gen = t_train = 0.0
    for rd in range(rounds):
        t0 = time.perf_counter()
        for m, c in zip(fine_b.members, cur_b.members):
            restrict(m, c, fac)
        cur_b.step(cfg.k)
        fine_b.step(cfg.k * fac)
        for i, (m, c, r) in enumerate(zip(fine_b.members, cur_b.members, refs)):
            restrict(m, r, fac)
            features(c, xb, slot, cfg.s_rho, cfg.s_u)
            target(r, c, tb, slot, cfg.s_out)
            slot = (slot + 1) % cfg.buffer
            filled = min(filled + 1, cfg.buffer)
        fine_b.step(spacing - cfg.k * fac)
        cur_b.synchronize()
        t_gen += time.perf_counter() - t0
        t0 = time.perf_counter()
        for _ in range(cfg.iters_per_round):
            idx = torch.from_numpy(rng.choice(filled, size=min(cfg.batch, filled), replace=False)).to(dev)
            losses.append(net.train_step(xb[idx].contiguous(), tb[idx].contiguous(), cfg.lr))
        t_train += time.perf_counter() - t0
        if rd % 50 == 0:
            say(f"round {rd}/{rounds} loss {losses[-1]:.4e}")
    t0 = time.perf_counter()
    for it in range(cfg.final_iters):
        idx = torch.from_numpy(rng.choice(filled, size=min(cfg.batch, filled), replace=False)).to(dev)
        lr = cfg.lr * (0.5 if it > cfg.final_iters // 2 else 1.0)
        losses.append(net.train_step(xb[idx].contiguous(), tb[idx].contiguous(), lr))
    net.synchronize()
    t_train += time.perf_counter() - t0
    fine_b.close()
    cur_b.close()
    for r in refs:
        r.close()
    del xb, tb
    res["training"] = {"pairs": rounds * cfg.train_lattices, "iterations": len(losses),
                       "first_loss": losses[0], "final_loss": float(np.mean(losses[-20:])),
                       "data_seconds": round(t_gen, 2), "train_seconds": round(t_train, 2),
                       "fine_steps_between_pairs": spacing}

    # ---- judge on a held-out geometry ---------------------------------------
    es = channel_spec(nf, tau=cfg.tau_fine, n_obstacles=cfg.n_obstacles, r_lo=cfg.r_lo,
                      r_hi=cfg.r_hi, force=cfg.force_fine, seed=cfg.eval_seed)
    cm = coarse_geometry(es.solid, fac)
    fluid_c = cm == 0
    stream = torch.cuda.Stream()

    def coarse_lattice():
        lat = lbm.Lattice(nc, nc, cfg.tau_coarse, lbm.F32, flags)
        lat.set_force(force_c, 0.0)
        lat.set_geometry(cm)
        return lat

    fine = lbm.Lattice(nf, nf, cfg.tau_fine, lbm.F32, flags)
    fine.set_force(cfg.force_fine, 0.0)
    fine.set_geometry(es.solid)
    base, corr = coarse_lattice(), coarse_lattice()
    restrict(fine, base, fac)
    restrict(fine, corr, fac)
    for lat in (fine, base, corr):
        lat.set_stream(stream.cuda_stream)
    chunk_f = cfg.horizon_fine // cfg.checkpoints
    chunk_c = chunk_f // fac
    x1 = torch.zeros((1, 4, nc, nc), device=dev)
    o1 = torch.zeros((1, 9, nc, nc), device=dev)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t_fine = t_base = t_corr = 0.0
    err_base, err_corr = [], []
    fallback_at = None
    mass0 = corr.health()["mass"]
    for cp in range(cfg.checkpoints):
        ev0.record(stream)
        fine.step(chunk_f)
        ev1.record(stream)
        ev1.synchronize()
        t_fine += ev0.elapsed_time(ev1) / 1e3
        ev0.record(stream)
        base.step(chunk_c)
        ev1.record(stream)
        ev1.synchronize()
        t_base += ev0.elapsed_time(ev1) / 1e3
        ev0.record(stream)
        done = 0
        while done < chunk_c:
            n = min(cfg.k, chunk_c - done)
            corr.step(n)
            done += n
            if n == cfg.k:
                features(corr, x1, 0, cfg.s_rho, cfg.s_u)
                net.forward(x1, o1)
                apply_correction(corr, o1, 0, cfg.s_out)
        ev1.record(stream)
        ev1.synchronize()
        t_corr += ev0.elapsed_time(ev1) / 1e3
        # periodic check of the corrected run (the fine grid is the fallback)
        h = corr.health()
        if fallback_at is None and (h["unstable"] or abs(h["mass"] - mass0) > cfg.mass_tolerance * mass0):
            fallback_at = (cp + 1) * chunk_f
        rho, ux, uy = fine.moments()
        rx, ry = _block_velocity(rho, ux, uy, es.solid, fac)
        _, bx, by = base.moments()
        _, cx, cy = corr.moments()
        err_base.append(_l2(bx, by, rx, ry, fluid_c))
        err_corr.append(_l2(cx, cy, rx, ry, fluid_c))
        say(f"checkpoint {cp + 1}: coarse {err_base[-1]:.4f} corrected {err_corr[-1]:.4f}")
    u_rms = float(np.sqrt(np.mean((rx ** 2 + ry ** 2)[fluid_c])))
    for lat in (fine, base, corr):
        lat.close()
    net.close()
    res["evaluation"] = {
        "fine_equivalent_steps": cfg.horizon_fine, "checkpoints": cfg.checkpoints,
        "u_l2_coarse_only": err_base, "u_l2_corrected": err_corr,
        "u_l2_coarse_only_mean": float(np.mean(err_base)),
        "u_l2_corrected_mean": float(np.mean(err_corr)),
        "u_l2_coarse_only_final": err_base[-1], "u_l2_corrected_final": err_corr[-1],
        "u_rms_fine_final": u_rms,
        "fine_seconds": round(t_fine, 4), "coarse_seconds": round(t_base, 4),
        "corrected_seconds": round(t_corr, 4),
        "time_to_solution_ratio": round(t_fine / max(t_corr, 1e-12), 2),
        "fallback_triggered_at_fine_step": fallback_at,
    }
    return res
