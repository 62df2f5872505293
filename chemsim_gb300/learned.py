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

    def save(self, path: str):
        check(self._lib.lbm_cnn_save(self._n, str(path).encode()))

    def load(self, path: str):
        check(self._lib.lbm_cnn_load(self._n, str(path).encode()))

    def set_stream(self, stream_ptr: int | None):
        """Issue the net's work on this cudaStream_t (None: its own stream)."""
        check(self._lib.lbm_cnn_set_stream(self._n, ctypes.c_void_p(stream_ptr or 0)))

    def synchronize(self):
        check(self._lib.lbm_cnn_synchronize(self._n))


def restrict(fine, coarse, factor: int = 4):
    check(_lib.load().lbm_restrict(fine.handle, coarse.handle, int(factor)))


def features(lat, x, image: int, s_rho: float, s_u: float):
    check(_lib.load().lbm_coarse_features(lat.handle, float(s_rho), float(s_u), int(image), _ptr(x)))


def apply_correction(lat, corr, image: int, scale: float, max_abs: float = 0.0):
    check(_lib.load().lbm_coarse_apply(lat.handle, _ptr(corr), int(image), float(scale), float(max_abs)))


def target(ref, cur, t, image: int, scale: float):
    check(_lib.load().lbm_coarse_target(ref.handle, cur.handle, float(scale), int(image), _ptr(t)))


def coarse_run(lat, net, nsteps: int, k: int, s_rho: float, s_u: float, scale: float,
               max_abs: float = 0.0, check_every: int = 16, mass_tolerance: float = 1e-3):
    """lbm_coarse_run: nsteps corrected coarse steps; returns the step count at
    which the periodic check asked for the fine-grid fallback, or None."""
    out = ctypes.c_int64()
    check(_lib.load().lbm_coarse_run(lat.handle, net._n, int(nsteps), int(k), float(s_rho),
                                     float(s_u), float(scale), float(max_abs), int(check_every),
                                     float(mass_tolerance), ctypes.byref(out)))
    return None if out.value < 0 else int(out.value)


# ---------------------------------------------------------------------------
# the coarse-plus-correction experiment
# ---------------------------------------------------------------------------

from dataclasses import dataclass  # noqa: E402
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
    pairs: int = 4000             # snapshot pairs: (intervals of k coarse steps) x train_lattices
    horizon_fine: int = 20000     # fine-equivalent steps of the evaluation
    batch: int = 8
    buffer: int = 4000            # pairs kept for training (evenly thinned when fewer)
    final_iters: int = 3000       # Adam iterations
    lr: float = 1e-3
    s_rho: float = 0.0             # density input off: its acoustic part is noise here
    s_u: float = 100.0
    s_out: float = 1e-4
    seed: int = 11
    eval_seed: int = 9999
    checkpoints: int = 10
    mass_tolerance: float = 1e-3
    check_every: int = 16         # corrections between health checks of a corrected run
    gain: float = 0.1             # fraction of the predicted correction applied
    clip: float = 4.0             # |d_i| limit in RMS of the training targets (0: none)
    data_policy: str = "teacher"  # first data pass: "teacher" or "none" (coarse-only run)
    onpolicy_passes: int = 0      # data passes with the network's own corrections applied
    onpolicy_iters: int = 1500

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


def _coarse_specs(cfg: CorrectionConfig, seeds):
    from .workloads import LatticeSpec, channel_spec
    fine = [channel_spec(cfg.fine, tau=cfg.tau_fine, n_obstacles=cfg.n_obstacles, r_lo=cfg.r_lo,
                         r_hi=cfg.r_hi, force=cfg.force_fine, seed=s) for s in seeds]
    coarse = [LatticeSpec(cfg.coarse, cfg.coarse, cfg.tau_coarse, f.flags,
                          force=(cfg.force_fine * cfg.factor, 0.0),
                          solid=coarse_geometry(f.solid, cfg.factor)) for f in fine]
    return fine, coarse


def train_correction(cfg: CorrectionConfig, stream, log=None):
    """Snapshot pairs from the batched fine LBM, then Adam on the GPU.

    Every lattice pair runs side by side from rest: each interval the coarse
    lattice takes k steps and the fine one k * factor; the restricted fine
    state is the reference and the pair (features of the coarse state, the
    population change that moves its velocity onto the reference's) is
    stored.  In the first pass that change itself is then applied to the
    coarse lattice (teacher forcing); in each later pass the network's own
    prediction is applied instead (the states a corrected run visits, so the
    network learns to pull its own drift back), the new pairs replace the
    buffer and training continues.

    Returns (net, s_eff, info): the applied correction is net output * s_eff.
    """
    import torch
    from . import lbm
    say = log or (lambda *a: None)
    nc, fac, nl = cfg.coarse, cfg.factor, cfg.train_lattices
    dev = torch.device("cuda")
    specs, cspecs = _coarse_specs(cfg, [cfg.seed + i for i in range(nl)])
    refs = []
    for cs in cspecs:
        r = lbm.Lattice(nc, nc, cfg.tau_coarse, lbm.F32, cs.flags | lbm.FAST)
        r.set_force(*cs.force)
        r.set_geometry(cs.solid)
        r.set_stream(stream.cuda_stream)
        refs.append(r)
    net = CorrectionNet(nc, nc, max(cfg.batch, nl), seed=cfg.seed)
    net.set_stream(stream.cuda_stream)
    rounds = max(1, cfg.pairs // nl)
    keep = max(1, (rounds * nl + cfg.buffer - 1) // cfg.buffer)
    nbuf = min(cfg.buffer, rounds * nl)
    rng = np.random.default_rng(cfg.seed)
    losses, passes = [], []
    t_gen = t_train = 0.0

    with torch.cuda.stream(stream):
        xb = torch.zeros((nbuf, 4, nc, nc), device=dev)
        tb = torch.zeros((nbuf, 9, nc, nc), device=dev)
        xs = torch.zeros((nl, 4, nc, nc), device=dev)
        ts = torch.zeros((nl, 9, nc, nc), device=dev)
        os_ = torch.zeros((nl, 9, nc, nc), device=dev)
        stream.synchronize()

        def generate(scale, policy):
            """One pass over the training horizon; fills the buffer (targets
            in units of `scale`).  policy "teacher": the target itself is
            applied; "none": nothing is applied (the coarse-only run, whose
            accumulated gap to the fine run becomes the target); a number:
            the network's correction with that gain."""
            fine_b = lbm.Batch(specs, lbm.FRAME_XY | lbm.FAST)
            cur_b = lbm.Batch(cspecs, lbm.FRAME_XY | lbm.FAST)
            fine_b.set_stream(stream.cuda_stream)
            cur_b.set_stream(stream.cuda_stream)
            for m, c in zip(fine_b.members, cur_b.members):
                restrict(m, c, fac)
            slot = count = 0
            for _ in range(rounds):
                cur_b.step(cfg.k)
                fine_b.step(cfg.k * fac)
                for i, (m, c, r) in enumerate(zip(fine_b.members, cur_b.members, refs)):
                    restrict(m, r, fac)
                    features(c, xs, i, cfg.s_rho, cfg.s_u)
                    target(r, c, ts, i, scale)
                if not isinstance(policy, str):
                    net.forward(xs, os_)
                for i, c in enumerate(cur_b.members):
                    if policy == "teacher":
                        apply_correction(c, ts, i, scale)
                    elif not isinstance(policy, str):
                        apply_correction(c, os_, i, s_eff * policy, cfg.clip * s_eff)
                    if count % keep == 0 and slot < nbuf:
                        xb[slot].copy_(xs[i])
                        tb[slot].copy_(ts[i])
                        slot += 1
                    count += 1
            stream.synchronize()
            fine_b.close()
            cur_b.close()
            return slot

        def train(filled, iters, lr0):
            for it in range(iters):
                idx = torch.from_numpy(rng.choice(filled, size=min(cfg.batch, filled),
                                                  replace=False)).to(dev)
                lr = lr0 * (0.1 if it >= 0.8 * iters else 0.3 if it >= 0.5 * iters else 1.0)
                losses.append(net.train_step(xb[idx].contiguous(), tb[idx].contiguous(), lr))
                if it % 500 == 0:
                    say(f"iteration {it}/{iters} loss {losses[-1]:.4e}")
            net.synchronize()

        t0 = time.perf_counter()
        filled = generate(cfg.s_out, cfg.data_policy)
        # targets to unit RMS; the applied correction is net output * s_eff
        rms = float(torch.sqrt(torch.mean(tb[:filled] ** 2)))
        rms = rms if rms > 0 else 1.0
        tb[:filled] /= rms
        s_eff = cfg.s_out * rms
        t_gen += time.perf_counter() - t0
        t0 = time.perf_counter()
        train(filled, cfg.final_iters, cfg.lr)
        t_train += time.perf_counter() - t0
        passes.append({"policy": cfg.data_policy, "final_loss": float(np.mean(losses[-20:]))})
        for p in range(cfg.onpolicy_passes):
            t0 = time.perf_counter()
            filled = generate(s_eff, cfg.gain)
            t_gen += time.perf_counter() - t0
            t0 = time.perf_counter()
            train(filled, cfg.onpolicy_iters, cfg.lr * 0.3)
            t_train += time.perf_counter() - t0
            passes.append({"policy": f"network, gain {cfg.gain}",
                           "first_loss": losses[-cfg.onpolicy_iters],
                           "final_loss": float(np.mean(losses[-20:]))})
        del xb, tb, xs, ts, os_
    for r in refs:
        r.close()
    info = {"pairs_per_pass": filled, "iterations": len(losses), "passes": passes,
            "first_loss": losses[0], "final_loss": float(np.mean(losses[-20:])),
            "loss_unit": "mean squared error / target variance",
            "data_seconds": round(t_gen, 2), "train_seconds": round(t_train, 2),
            "fine_steps_covered": rounds * cfg.k * fac}
    return net, s_eff, info


def evaluate_correction(cfg: CorrectionConfig, net, s_eff: float, stream, gains=(1.0,),
                        log=None) -> dict:
    """Fine, coarse-only and coarse-plus-correction runs (one per gain) of a
    held-out geometry, side by side on one stream; velocity L2 errors of the
    coarse runs against the block-averaged fine run at each checkpoint and the
    time of each run (CUDA events).  A corrected run goes through
    lbm_coarse_run, whose periodic health check (mass drift or instability)
    hands the run over to the fine grid: from then on it is charged the fine
    run's time and carries the fine state."""
    import torch
    from . import lbm
    say = log or (lambda *a: None)
    nf, nc, fac = cfg.fine, cfg.coarse, cfg.factor
    (es,), (cs,) = _coarse_specs(cfg, [cfg.eval_seed])
    fluid_c = cs.solid == 0
    flags = es.flags | lbm.FAST

    def lattice(n, tau, force, solid):
        lat = lbm.Lattice(n, n, tau, lbm.F32, flags)
        lat.set_force(*force)
        lat.set_geometry(solid)
        lat.set_stream(stream.cuda_stream)
        return lat

    fine = lattice(nf, cfg.tau_fine, es.force, es.solid)
    base = lattice(nc, cfg.tau_coarse, cs.force, cs.solid)
    corrs = [lattice(nc, cfg.tau_coarse, cs.force, cs.solid) for _ in gains]
    for lat in [base] + corrs:
        restrict(fine, lat, fac)
    chunk_f = cfg.horizon_fine // cfg.checkpoints
    chunk_c = chunk_f // fac
    stream.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def timed(fn):
        ev0.record(stream)
        fn()
        ev1.record(stream)
        ev1.synchronize()
        return ev0.elapsed_time(ev1) / 1e3

    t_fine = t_base = 0.0
    t_corr = [0.0] * len(gains)
    err_base, err_corr = [], [[] for _ in gains]
    fallback_at = [None] * len(gains)
    for cp in range(cfg.checkpoints):
        t_chunk = timed(lambda: fine.step(chunk_f))
        t_fine += t_chunk
        t_base += timed(lambda: base.step(chunk_c))
        for g, (gain, corr) in enumerate(zip(gains, corrs)):
            if fallback_at[g] is not None:
                # that run has handed over to the fine grid: it costs the fine
                # chunk and carries the fine state
                t_corr[g] += t_chunk
                restrict(fine, corr, fac)
                continue
            stop = []

            def run():
                stop.append(coarse_run(corr, net, chunk_c, cfg.k, cfg.s_rho, cfg.s_u,
                                       s_eff * gain, cfg.clip * s_eff, cfg.check_every,
                                       cfg.mass_tolerance))
            t_corr[g] += timed(run)
            if stop[0] is not None:
                fallback_at[g] = stop[0] * fac
        rho, ux, uy = fine.moments()
        rx, ry = _block_velocity(rho, ux, uy, es.solid, fac)
        _, bx, by = base.moments()
        err_base.append(_l2(bx, by, rx, ry, fluid_c))
        for g, corr in enumerate(corrs):
            _, cx, cy = corr.moments()
            err_corr[g].append(_l2(cx, cy, rx, ry, fluid_c))
        say(f"checkpoint {cp + 1}: coarse {err_base[-1]:.4f} corrected "
            + " ".join(f"{e[-1]:.4f}" for e in err_corr))
    u_rms = float(np.sqrt(np.mean((rx ** 2 + ry ** 2)[fluid_c])))
    for lat in [fine, base] + corrs:
        lat.close()
    out = {"fine_equivalent_steps": cfg.horizon_fine, "checkpoints": cfg.checkpoints,
           "u_l2_coarse_only": err_base, "u_l2_coarse_only_mean": float(np.mean(err_base)),
           "u_l2_coarse_only_final": err_base[-1], "u_rms_fine_final": u_rms,
           "fine_seconds": round(t_fine, 4), "coarse_seconds": round(t_base, 4), "corrected": []}
    for g, gain in enumerate(gains):
        out["corrected"].append({
            "gain": gain, "u_l2": err_corr[g], "u_l2_mean": float(np.mean(err_corr[g])),
            "u_l2_final": err_corr[g][-1], "seconds": round(t_corr[g], 4),
            "time_to_solution_ratio": round(t_fine / max(t_corr[g], 1e-12), 2),
            "fallback_triggered_at_fine_step": fallback_at[g]})
    return out


def run_correction_experiment(cfg: CorrectionConfig, log=None, gains=None) -> dict:
    """Trains the correction (train_correction) and evaluates it on a held-out
    geometry (evaluate_correction).  Returns a result dict."""
    import torch
    stream = torch.cuda.Stream()
    res = {"config": dict(cfg.__dict__),
           "tau_coarse": cfg.tau_coarse, "force_coarse": cfg.force_fine * cfg.factor}
    net, s_eff, res["training"] = train_correction(cfg, stream, log)
    res["training"]["target_rms"] = s_eff
    try:
        res["evaluation"] = evaluate_correction(cfg, net, s_eff, stream,
                                                gains=gains or (cfg.gain,), log=log)
    finally:
        net.close()
    return res


def forward_throughput(images: int = 8, side: int = 512, reps: int = 20) -> dict:
    """Times the correction network's forward pass on `images` random images
    of side x side (CUDA events on the net's stream); TFLOP/s counted with the
    real channel counts (4 -> 32 -> 32 -> 32 -> 9, 3x3 taps)."""
    import torch
    stream = torch.cuda.Stream()
    macs = 9 * (4 * 32 + 32 * 32 + 32 * 32 + 32 * 9)
    with CorrectionNet(side, side, images, seed=1) as net:
        net.set_stream(stream.cuda_stream)
        with torch.cuda.stream(stream):
            x = torch.randn((images, 4, side, side), device="cuda")
            out = torch.empty((images, 9, side, side), device="cuda")
        stream.synchronize()
        for _ in range(3):
            net.forward(x, out)
        start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        start.record(stream)
        for _ in range(reps):
            net.forward(x, out)
        end.record(stream)
        end.synchronize()
        secs = start.elapsed_time(end) / 1e3 / reps
    flops = 2.0 * macs * images * side * side
    return {"images": images, "side": side, "ms": round(secs * 1e3, 3),
            "algorithmic_gflop": round(flops / 1e9, 2), "tflops": round(flops / secs / 1e12, 1)}


def gradient_throughput(images: int = 8, side: int = 512, reps: int = 10) -> dict:
    """Times lbm_cnn_gradients (forward with the pre-activations kept, loss,
    input gradients and the tcgen05 weight gradients) on `images` random
    images of side x side; each call waits for its loss."""
    import torch
    with CorrectionNet(side, side, images, seed=1) as net:
        x = torch.randn((images, 4, side, side), device="cuda")
        t = torch.randn((images, 9, side, side), device="cuda") * 0.1
        torch.cuda.synchronize()
        for _ in range(2):
            net.gradients(x, t)
        t0 = time.perf_counter()
        for _ in range(reps):
            net.gradients(x, t)
        secs = (time.perf_counter() - t0) / reps
    return {"images": images, "side": side, "ms": round(secs * 1e3, 3)}


if __name__ == "__main__":
    # python -m chemsim_gb300.learned forward|gradients [images] [side]
    import json
    import sys
    if len(sys.argv) < 2 or sys.argv[1] not in ("forward", "gradients"):
        sys.exit("usage: python -m chemsim_gb300.learned forward|gradients [images] [side]")
    n = int(sys.argv[2]) if len(sys.argv) > 2 else 8
    side = int(sys.argv[3]) if len(sys.argv) > 3 else 512
    fn = forward_throughput if sys.argv[1] == "forward" else gradient_throughput
    print(json.dumps(fn(n, side)))
