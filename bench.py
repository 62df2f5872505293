#!/usr/bin/env python3
"""Benchmark of the fused D2Q9 step (one JSON line on rank 0).

Workload (the lattice the headline metric is quoted on): D2Q9 BGK channel,
4096 x 4096, tau = 0.56, periodic in x, half-way bounce-back walls in y, body
force 1e-6 along x, 64 seeded circular obstacles with radius U[16, 64];
synthetic, seeded (chemsim_gb300.workloads.channel_spec).  A "step" is one
time step of the whole lattice; the timed region is K back-to-back steps
(default 5000, the configuration's run length).  Inputs (1.2 GB of f32
populations per step) are larger than L2, so no L2 flush is needed.

  value   MLUPS of the f32 step, state resident in HBM, CUDA events on the
          lattice's stream, max over ranks.
  e2e     the same metric through the C ABI with host buffers: the initial
          fields are uploaded from pinned host memory and, every frame of two
          steps (the reference demo's speed_factor, src/main.rs:393), rho/u
          reach pinned host memory (LBMSim::step + render, src/main.rs:128-177):
          staged on the device and copied with lbm_read_moments_async, each
          frame's host copy overlapping the next frame's steps and staging
          (two staging areas in turn); the last frame is waited for inside
          the timed region.  e2e.direct_readback: written by the frame's last
          step kernel straight into the host buffers (lbm_step_moments_to);
          e2e.blocking_readback: the blocking lbm_read_moments;
          e2e.rendered_frames: reading back the finished RGBA8 frame of
          lbm_render_async (render.rs's colour map).
  fp16    the same lattice with half-precision deviation storage: the default
          stochastic rounding, and round_nearest (LBM_ROUND_NEAREST).
  accuracy  rho/u L2 errors of f32/f16/bf16 storage against the f64 run of
          the same kernel on the headline channel after --accuracy-steps
          steps (default 5000, the channel configuration's run length,
          whatever K is), and the same on the laminar 1024^2 Taylor-Green
          vortex (taylor_green_1024).
  taylor_green_256  the 256^2 periodic Taylor-Green lattice (tau 0.8, 1000
          steps; L2-resident): GPU MLUPS in both arithmetics and both CPU
          steppers on the host cores.
  roofline  algorithmic bytes (9 loads + 9 stores of 4 B + 1 B solid mask =
          73 B per cell) / average step time against the measured HBM copy
          bandwidth.
  batch   512 uneven lattices (sides U[64, 1024]) stepped together, autotuned.
  large   16384^2 with 16-bit deviation storage (both roundings) against
          8192^2 f32, and their rho/u L2 errors against f64 on a 1024^2 window.
  learned the coarse-grid correction: 2048^2 fine vs 512^2 coarse channel,
          training on the GPU, velocity L2 of coarse-only and corrected runs
          against the fine run, time-to-solution ratio, and the network's
          forward throughput on the tensor cores.

  cpu_baseline  the oracle's op-by-op CPU stepper (and the fused one) on all
          host cores, 3 steps of the full lattice.
  clocks  SM clock samples (nvidia-smi) during the timed region.

--impl reference times the CPU implementation of the same step, restated op
by op the way lbm.rs drives ArrayFire (oracle/, the reference cannot be built
on this machine), on the host cores.
"""
from __future__ import annotations

import argparse
import json
import os
import re
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

BYTES_F32 = 72          # 9 loads + 9 stores x 4 B
BYTES_F16 = 36
BYTES_MASK = 1          # u8 solid mask read once per cell
def workload_name(n: int) -> str:
    """The headline workload at side n (channel_spec(n): 64 obstacles at every size)."""
    return f"channel_{n}x{n}_tau0.56_walls_y_periodic_x_force1e-6_64obstacles_r16-64"


def bench_config(args, world: int) -> dict:
    """The workload both arms report (the same dict, so they compare)."""
    cells = args.size * args.size
    return {"workload": workload_name(args.size), "cells": cells,
            "l2": (f"inputs larger than L2 ({72 * cells / 1e9:.1f} GB of populations per "
                   "step); no flush") if 72 * cells > 129e6 else
                  "inputs smaller than L2: no flush, the roofline fraction is not an HBM figure",
            "parallelism": "replicas" if world > 1 else "single GPU"}


def parse_args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5000)
    p.add_argument("--warmup", type=int, default=20)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--size", type=int, default=4096)
    p.add_argument("--no-cpu", action="store_true", help="skip the cpu_baseline leg")
    p.add_argument("--no-accuracy", action="store_true")
    p.add_argument("--accuracy-steps", type=int, default=5000,
                   help="steps of the accuracy leg (the channel configuration's 5000 by default)")
    p.add_argument("--strict", action="store_true",
                   help="time the reference operation order instead of LBM_FAST")
    p.add_argument("--no-batch", action="store_true", help="skip the 512-lattice batch")
    p.add_argument("--batch-steps", type=int, default=2000)
    p.add_argument("--batch-lattices", type=int, default=512)
    p.add_argument("--batch-tile", type=int, default=0, choices=(0, 2, 4),
                   help="batch tile width in cells per thread (0: autotuned)")
    p.add_argument("--no-large", action="store_true",
                   help="skip the 16384^2 f16 / 8192^2 f32 comparison")
    p.add_argument("--large-steps", type=int, default=500)
    p.add_argument("--no-learned", action="store_true",
                   help="skip the learned coarse-grid correction (train + evaluate)")
    p.add_argument("--learned-iters", type=int, default=3000, help="Adam iterations")
    return p.parse_args()


def dist_env():
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("LOCAL_RANK", "0")),
            int(os.environ.get("WORLD_SIZE", "1")))


# ---------------------------------------------------------------------------
# clocks
# ---------------------------------------------------------------------------

class ClockSampler:
    """nvidia-smi sampled every 200 ms while the timed region runs."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.tmp = None

    def start(self):
        try:
            self.tmp = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.tmp, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.tmp.flush()
        self.tmp.seek(0)
        rows = [r.split(",") for r in self.tmp.read().splitlines() if r.strip()]
        os.unlink(self.tmp.name)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            r = [x.strip() for x in r]
            try:
                sm.append(float(r[0]))
                mx.append(float(r[1]))
            except (ValueError, IndexError):
                continue
            for name, val in zip(names, r[4:8]):
                if val.lower() in ("active", "1"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------
# helpers
# ---------------------------------------------------------------------------

def measured_peak_gbs():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as fh:
            return float(json.load(fh)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def profiled_traffic(kernel_tag: str):
    """DRAM bytes per cell of the step kernel from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", f"{kernel_tag}.txt")
    try:
        with open(path) as fh:
            m = re.search(r"dram_bytes_per_cell:\s*([0-9.]+)", fh.read())
        return float(m.group(1)) if m else None
    except OSError:
        return None


def l2_rel(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def make_lattice(spec, precision, flags):
    from chemsim_gb300 import lbm
    lat = lbm.Lattice(spec.w, spec.h, spec.tau, precision, flags)
    lat.set_force(*spec.force)
    lat.set_geometry(spec.solid)
    lat.init_equilibrium(spec.rho, spec.ux, spec.uy)
    return lat


def timed_steps(lat, steps, warmup, torch, stream, dist=None):
    """W untimed steps, then exactly K steps between CUDA events on the
    lattice's stream; returns elapsed seconds (max over ranks)."""
    lat.set_stream(stream.cuda_stream)
    lat.step(warmup)
    lat.synchronize()
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    start = torch.cuda.Event(enable_timing=True)
    end = torch.cuda.Event(enable_timing=True)
    start.record(stream)
    lat.step(steps)
    end.record(stream)
    end.synchronize()
    torch.cuda.synchronize()
    secs = start.elapsed_time(end) / 1e3
    if dist is not None:
        t = torch.tensor([secs], device="cuda", dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        secs = float(t.item())
    return secs


def cpu_sample(spec, steps, threads, structured=True):
    """The oracle's CPU step on the full lattice, `steps` steps; MLUPS."""
    import oracle
    f0 = oracle.equilibrium(spec.rho, spec.ux, spec.uy)
    oracle.step(f0[:, :64], 1, tau=spec.tau, flags=spec.flags,
                solid=None if spec.solid is None else spec.solid[:64],
                force=spec.force, structured=structured, threads=threads)
    t0 = time.perf_counter()
    oracle.step(f0, steps, tau=spec.tau, flags=spec.flags, solid=spec.solid,
                force=spec.force, structured=structured, threads=threads)
    secs = time.perf_counter() - t0
    return spec.w * spec.h * steps / secs / 1e6, secs


# ---------------------------------------------------------------------------
# reference arm
# ---------------------------------------------------------------------------

def run_reference(args):
    rank, _, world = dist_env()
    if rank != 0:
        return 0
    import oracle
    from chemsim_gb300.workloads import channel_spec
    oracle.build()
    threads = os.cpu_count() or 1
    full = channel_spec(args.size)
    # Calibrate on a 512-row band, then size the band so W + K steps take
    # about 90 s of host time.
    band = 512
    spec = crop(full, band)
    f = oracle.equilibrium(spec.rho, spec.ux, spec.uy)
    t0 = time.perf_counter()
    f = oracle.step(f, 2, tau=spec.tau, flags=spec.flags, solid=spec.solid, force=spec.force,
                    structured=True, threads=threads)
    per_cell = (time.perf_counter() - t0) / (2 * spec.w * spec.h)
    budget = 90.0
    rows = int(budget / max(per_cell * spec.w * (args.steps + args.warmup), 1e-12))
    rows = max(16, min(full.h, rows))
    spec = crop(full, rows)
    f = oracle.equilibrium(spec.rho, spec.ux, spec.uy)
    f = oracle.step(f, args.warmup, tau=spec.tau, flags=spec.flags, solid=spec.solid,
                    force=spec.force, structured=True, threads=threads)
    t0 = time.perf_counter()
    oracle.step(f, args.steps, tau=spec.tau, flags=spec.flags, solid=spec.solid,
                force=spec.force, structured=True, threads=threads)
    secs = time.perf_counter() - t0
    mlups = spec.w * spec.h * args.steps / secs / 1e6
    sample = (f"{args.steps} time steps of a {spec.w}x{spec.h} band (rows 0..{spec.h - 1}) of "
              f"the {full.w}x{full.h} channel lattice, same tau/force/walls/obstacles; f32, "
              "op-by-op full-plane passes as lbm.rs drives ArrayFire (oracle/lbm_oracle.cpp "
              "step_structured), OpenMP")
    line = {
        "metric": "D2Q9 MLUPS", "value": round(mlups, 3), "unit": "MLUPS", "impl": "reference",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": secs / args.steps * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": bench_config(args, world),
        "arithmetic": "reference order (the op-by-op stepper)",
        "cpu_baseline": {"value": round(mlups, 3), "unit": "MLUPS", "cores": threads,
                         "kind": "port", "sample": sample},
        "e2e": {"value": round(mlups, 3), "unit": "MLUPS", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "note": "taktoa/chemsim (Rust over ArrayFire 3.6) cannot be built here: no Rust "
                "toolchain and no ArrayFire; timed is the oracle's restatement of its step",
    }
    print(json.dumps(line), flush=True)
    return 0


def crop(spec, rows):
    from chemsim_gb300.workloads import LatticeSpec
    r = min(rows, spec.h)
    return LatticeSpec(spec.w, r, spec.tau, spec.flags, force=spec.force,
                       solid=np.ascontiguousarray(spec.solid[:r]),
                       rho=np.ascontiguousarray(spec.rho[:r]),
                       ux=np.ascontiguousarray(spec.ux[:r]),
                       uy=np.ascontiguousarray(spec.uy[:r]), name=spec.name + f"_band{r}")


# ---------------------------------------------------------------------------
# our arm
# ---------------------------------------------------------------------------

def run_ours(args):
    import torch
    rank, local_rank, world = dist_env()
    dist = None
    if world > 1:
        import torch.distributed as tdist
        torch.cuda.set_device(local_rank)
        tdist.init_process_group("nccl")
        dist = tdist
    else:
        torch.cuda.set_device(0)
    from chemsim_gb300 import build, lbm
    from chemsim_gb300.workloads import channel_spec
    build()

    spec = channel_spec(args.size)
    cells = spec.w * spec.h
    base_flags = spec.flags | (0 if args.strict else lbm.FAST)
    stream = torch.cuda.Stream()
    clocks = ClockSampler(torch.cuda.current_device())

    # The accuracy leg runs first: besides its own result, its seconds of
    # full-load GPU work bring the clocks up before the timed legs.
    accuracy = None
    if not args.no_accuracy and rank == 0:
        accuracy = accuracy_channel(spec, base_flags, args.accuracy_steps)
        accuracy["taylor_green_1024"] = accuracy_taylor_green(args.accuracy_steps)

    # f32: the headline
    lat32 = make_lattice(spec, lbm.F32, base_flags)
    clocks.start()
    t32 = timed_steps(lat32, args.steps, args.warmup, torch, stream, dist)
    # f16 deviation storage (stochastic rounding, the default), and with
    # round-to-nearest
    lat16 = make_lattice(spec, lbm.F16DEV, base_flags)
    t16 = timed_steps(lat16, args.steps, args.warmup, torch, stream, dist)
    lat16n = make_lattice(spec, lbm.F16DEV, base_flags | lbm.ROUND_NEAREST)
    t16n = timed_steps(lat16n, args.steps, args.warmup, torch, stream, dist)
    clk = clocks.stop()
    mlups32 = cells * args.steps / t32 / 1e6 * world
    mlups16 = cells * args.steps / t16 / 1e6 * world
    mlups16n = cells * args.steps / t16n / 1e6 * world

    lat32.close()
    lat16.close()
    lat16n.close()

    # e2e through the C ABI with pinned host buffers
    e2e = run_e2e(spec, args, torch, dist)
    e2e["direct_readback"] = run_e2e(spec, args, torch, dist, readback="mapped")
    e2e["blocking_readback"] = run_e2e(spec, args, torch, dist, readback="moments")
    e2e["rendered_frames"] = run_e2e(spec, args, torch, dist, readback="frame")
    batch = None if args.no_batch or world > 1 else run_batch(args, torch)
    large = None if args.no_large or world > 1 else run_large(args, torch)
    learned = None if args.no_learned or world > 1 else run_learned(args, torch)

    peak, peak_kind = measured_peak_gbs()
    bpc = BYTES_F32 + BYTES_MASK
    step_s = t32 / args.steps
    achieved = bpc * cells / step_s / 1e9
    traffic_pc = profiled_traffic("lbm_step_f32_channel")
    roofline = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4),
                "traffic": None if traffic_pc is None else round(traffic_pc * cells / 1e9, 4),
                "algorithmic_bytes_per_cell": bpc, "peak_source": peak_kind,
                "traffic_unit": "GB per launch"}
    fp16 = {"mlups": round(mlups16, 1), "speedup_vs_f32": round(mlups16 / mlups32, 3),
            "achieved_gbs": round((BYTES_F16 + BYTES_MASK) * cells / (t16 / args.steps) / 1e9, 1),
            "rounding": "stochastic (random bits from the pair's own f32 bits)",
            "round_nearest": {"mlups": round(mlups16n, 1),
                              "speedup_vs_f32": round(mlups16n / mlups32, 3)}}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        threads = os.cpu_count() or 1
        import oracle
        oracle.build()
        v, secs = cpu_sample(spec, 3, threads, structured=True)
        vf, _ = cpu_sample(spec, 3, threads, structured=False)
        cpu = {"value": round(v, 3), "unit": "MLUPS", "cores": threads, "kind": "port",
               "sample": f"3 full {spec.w}x{spec.h} time steps ({secs:.1f} s), f32, the oracle's "
                         "op-by-op restatement of lbm.rs's ArrayFire passes, OpenMP",
               "fused_cpu_mlups": round(vf, 3)}
    config1 = None if (args.no_cpu or rank != 0) else run_config1(torch)

    if rank == 0:
        line = {
            "metric": "D2Q9 MLUPS", "value": round(mlups32, 1), "unit": "MLUPS",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(step_s * 1e3, 5), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": bench_config(args, world),
            "arithmetic": "reference order" if args.strict else "LBM_FAST (FMA)",
            "hbm_gbs": round(achieved, 1),
            "roofline": roofline,
            "fp16": fp16,
            "accuracy": accuracy,
            "taylor_green_256": config1,
            "e2e": e2e,
            "gpu_launches": args.steps,
            "clocks": clk,
            "cpu_baseline": cpu,
            "batch": batch,
            "large": large,
            "learned": learned,
        }
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()
    return 0


def run_config1(torch):
    """The 256^2 periodic Taylor-Green lattice (tau 0.8, 1000 steps): GPU MLUPS
    (f32, LBM_FAST and strict) and both CPU steppers on the host cores.  Its
    4.7 MB per step stay in L2, so no HBM roofline applies."""
    from chemsim_gb300 import lbm
    from chemsim_gb300.workloads import taylor_green_spec
    spec = taylor_green_spec(256)
    steps = 1000
    out = {"workload": "taylor_green_256x256_tau0.8_periodic", "steps": steps,
           "l2": "L2-resident (4.7 MB per step): MLUPS only, no HBM roofline"}
    stream = torch.cuda.Stream()
    for name, flags in (("gpu_fast_mlups", spec.flags | lbm.FAST), ("gpu_strict_mlups", spec.flags)):
        lat = make_lattice(spec, lbm.F32, flags)
        secs = timed_steps(lat, steps, 20, torch, stream)
        lat.close()
        out[name] = round(spec.w * spec.h * steps / secs / 1e6, 1)
    threads = os.cpu_count() or 1
    out["cpu_cores"] = threads
    out["cpu_structured_mlups"] = round(cpu_sample(spec, 50, threads, structured=True)[0], 2)
    out["cpu_fused_mlups"] = round(cpu_sample(spec, 200, threads, structured=False)[0], 2)
    out["cpu_sample"] = "50 (structured) and 200 (fused) time steps of the same lattice"
    return out


def accuracy_channel(spec, flags, steps):
    """rho/u L2 errors of f32, f16-deviation (both roundings) and
    bf16-deviation storage against the f64 run of the same kernel on the
    headline channel, each lattice run from the same initial state for
    `steps` steps (the channel configuration's run length by default,
    independent of the timed step count)."""
    from chemsim_gb300 import lbm
    runs = {}
    for name, prec, extra in (("f64", lbm.F64, 0), ("f32", lbm.F32, 0), ("f16dev", lbm.F16DEV, 0),
                              ("f16dev_round_nearest", lbm.F16DEV, lbm.ROUND_NEAREST),
                              ("bf16dev", lbm.BF16DEV, 0)):
        lat = make_lattice(spec, prec, flags | extra)
        lat.step(steps)
        runs[name] = lat.moments()
        lat.close()
    m64 = runs["f64"]
    fluid = spec.solid == 0

    def errs(m):
        return {"rho_dev_l2": l2_rel(m[0][fluid] - 1.0, m64[0][fluid] - 1.0),
                "rho_l2": l2_rel(m[0][fluid], m64[0][fluid]),
                "u_l2": l2_rel(np.stack([m[1][fluid], m[2][fluid]]),
                               np.stack([m64[1][fluid], m64[2][fluid]]))}
    out = {"workload": f"{spec.w}x{spec.h} channel (the timed lattice)", "steps": steps,
           "against": "f64 run of the same kernel"}
    for name in ("f32", "f16dev", "f16dev_round_nearest", "bf16dev"):
        out[name] = errs(runs[name])
    out["u_rms_f64"] = float(np.sqrt(np.mean(m64[1][fluid] ** 2 + m64[2][fluid] ** 2)))
    return out


def accuracy_taylor_green(steps):
    """rho/u L2 of f32, f16-deviation and bf16-deviation storage against the
    f64 run of the same kernel on a laminar flow: the 1024^2 Taylor-Green
    vortex (tau 0.8, u0 0.02), where the error is the storage's own and not
    the phase drift of an unsteady flow."""
    from chemsim_gb300 import lbm
    from chemsim_gb300.workloads import taylor_green_spec
    spec = taylor_green_spec(1024)
    runs = {}
    for name, prec, extra in (("f64", lbm.F64, 0), ("f32", lbm.F32, 0), ("f16dev", lbm.F16DEV, 0),
                              ("f16dev_round_nearest", lbm.F16DEV, lbm.ROUND_NEAREST),
                              ("bf16dev", lbm.BF16DEV, 0)):
        lat = make_lattice(spec, prec, spec.flags | lbm.FAST | extra)
        lat.step(steps)
        runs[name] = lat.moments()
        lat.close()
    r64, x64, y64 = runs["f64"]
    out = {"steps": steps, "u_rms_f64": float(np.sqrt(np.mean(x64 ** 2 + y64 ** 2)))}
    for name in ("f32", "f16dev", "f16dev_round_nearest", "bf16dev"):
        r, x, y = runs[name]
        out[name] = {"rho_l2": l2_rel(r, r64), "u_l2": l2_rel(np.stack([x, y]), np.stack([x64, y64]))}
    return out


def run_batch(args, torch):
    """512 independent lattices, sides U[64, 1024], tau U[0.52, 1.0], Taylor-Green
    or channel initial state by seed, 0-16 obstacles, f32: autotuned tiles,
    then --batch-steps steps of all lattices timed with CUDA events."""
    import tempfile
    from chemsim_gb300 import lbm
    from chemsim_gb300.workloads import batch_specs
    specs = batch_specs(args.batch_lattices)
    cells = sum(s.w * s.h for s in specs)
    b = lbm.Batch(specs, lbm.FRAME_XY | lbm.FAST)
    for m, sp in zip(b.members, specs):
        m.init_equilibrium(sp.rho, sp.ux, sp.uy)
    stream = torch.cuda.Stream()
    b.set_stream(stream.cuda_stream)
    cache = os.path.join(tempfile.gettempdir(), "lbm_batch_tiles.json")
    if os.path.exists(cache):
        os.unlink(cache)
    t0 = time.perf_counter()
    if args.batch_tile:
        b.set_tile(args.batch_tile)
        tuned = None
    else:
        b.autotune(cache)
        with open(cache) as fh:
            tuned = json.load(fh)["lbm_batch_autotune"][-1]
    tune_s = time.perf_counter() - t0
    b.step(args.warmup)
    b.synchronize()
    start = torch.cuda.Event(enable_timing=True)
    end = torch.cuda.Event(enable_timing=True)
    start.record(stream)
    b.step(args.batch_steps)
    end.record(stream)
    end.synchronize()
    secs = start.elapsed_time(end) / 1e3
    health = [m.health() for m in b.members[:8]]
    tile = b.tile()
    b.close()
    peak, _ = measured_peak_gbs()
    gbs = (BYTES_F32 + BYTES_MASK) * cells * args.batch_steps / secs / 1e9
    return {"workload": f"{args.batch_lattices} lattices, sides U[64,1024], tau U[0.52,1.0], TG or "
                        "channel, 0-16 obstacles, f32",
            "cells": cells, "steps": args.batch_steps, "mlups": round(cells * args.batch_steps / secs / 1e6, 1),
            "achieved_gbs": round(gbs, 1), "frac": round(gbs / peak, 4),
            "ms_per_step": round(secs / args.batch_steps * 1e3, 4), "autotune_s": round(tune_s, 2),
            "tile_cells_per_thread": tile,
            "autotune_mlups": {"2": tuned["mlups_v2"], "4": tuned["mlups_v4"]} if tuned else None,
            "launches_per_step": 1,
            "stable": all(not h["unstable"] for h in health)}


def run_learned(args, torch):
    """The learned coarse-grid correction: 2048^2 fine channel (tau 0.55, 64
    obstacles) against the 512^2 coarse lattice of equal viscosity (tau_c =
    0.5125, F_c = 4 F), snapshot pairs from the batched fine LBM, training on
    the GPU, then the held-out geometry over 20000 fine-equivalent steps:
    velocity L2 of coarse-only and corrected runs against the fine run and the
    time-to-solution ratio.  Also the correction network's forward throughput
    (tcgen05 implicit-GEMM convolutions) on 8 coarse images."""
    from chemsim_gb300.learned import (CorrectionConfig, evaluate_correction, forward_throughput,
                                       gradient_throughput, train_correction)
    cfg = CorrectionConfig(final_iters=args.learned_iters)
    stream = torch.cuda.Stream()
    t0 = time.perf_counter()
    net, s_eff, info = train_correction(cfg, stream)
    try:
        ev = evaluate_correction(cfg, net, s_eff, stream, gains=(cfg.gain,))
    finally:
        net.close()
    wall = time.perf_counter() - t0
    fwd = forward_throughput(8, cfg.coarse)
    grads = gradient_throughput(8, cfg.coarse)
    corr = ev["corrected"][0]
    return {"workload": f"fine {cfg.fine}^2 tau {cfg.tau_fine} vs coarse {cfg.coarse}^2 tau "
                        f"{cfg.tau_coarse:.4f}, {cfg.n_obstacles} obstacles, correction every "
                        f"{cfg.k} coarse steps, {cfg.horizon_fine} fine-equivalent steps",
            "training": info, "u_l2_coarse_only_mean": round(ev["u_l2_coarse_only_mean"], 5),
            "u_l2_coarse_only_final": round(ev["u_l2_coarse_only_final"], 5),
            "u_l2_corrected_mean": round(corr["u_l2_mean"], 5),
            "u_l2_corrected_final": round(corr["u_l2_final"], 5), "gain": corr["gain"],
            "fine_seconds": ev["fine_seconds"], "coarse_only_seconds": ev["coarse_seconds"],
            "corrected_seconds": corr["seconds"],
            "time_to_solution_ratio": corr["time_to_solution_ratio"],
            "fallback_triggered_at_fine_step": corr["fallback_triggered_at_fine_step"],
            "wall_seconds": round(wall, 1),
            "forward": fwd,
            "gradients": dict(grads, note="lbm_cnn_gradients: forward keeping the pre-activations, "
                                           "loss, input gradients and weight gradients, all on "
                                           "tcgen05; each call waits for its loss")}


def run_large(args, torch):
    """16384^2 f16-deviation channel (256 cylinders r U[20,120], tau 0.52, force
    5e-7) against 8192^2 f32, and the rho/u L2 error of f16 / f32 against
    f64 on a 1024^2 sub-problem cut from the same geometry (same window of
    the mask, same tau and force)."""
    from chemsim_gb300 import lbm
    from chemsim_gb300.workloads import CHANNEL_FLAGS, circles_mask
    flags = CHANNEL_FLAGS | lbm.FAST
    out = {}
    big = circles_mask(16384, 16384, 256, 20.0, 120.0, seed=5)
    for name, n, prec, bpc, extra in (
            ("f16dev_16384", 16384, lbm.F16DEV, BYTES_F16 + BYTES_MASK, 0),
            ("f16dev_16384_round_nearest", 16384, lbm.F16DEV, BYTES_F16 + BYTES_MASK, lbm.ROUND_NEAREST),
            ("f32_8192", 8192, lbm.F32, BYTES_F32 + BYTES_MASK, 0)):
        solid = np.ascontiguousarray(big[:n, :n])
        lat = lbm.Lattice(n, n, 0.52, prec, flags | extra)   # starts at rest: rho = 1, u = 0
        lat.set_force(5e-7, 0.0)
        lat.set_geometry(solid)
        stream = torch.cuda.Stream()
        secs = timed_steps(lat, args.large_steps, args.warmup, torch, stream)
        h = lat.health()
        lat.close()
        mlups = n * n * args.large_steps / secs / 1e6
        out[name] = {"cells": n * n, "steps": args.large_steps, "mlups": round(mlups, 1),
                     "achieved_gbs": round(bpc * n * n * args.large_steps / secs / 1e9, 1),
                     "stable": not h["unstable"]}
    out["f16_speedup_vs_f32"] = round(out["f16dev_16384"]["mlups"] / out["f32_8192"]["mlups"], 3)
    out["f16_round_nearest_speedup_vs_f32"] = round(
        out["f16dev_16384_round_nearest"]["mlups"] / out["f32_8192"]["mlups"], 3)
    # accuracy on the 1024^2 window
    crop = np.ascontiguousarray(big[:1024, :1024])
    steps = 2000
    res = {}
    for key, prec, extra in (("f64", lbm.F64, 0), ("f32", lbm.F32, 0), ("f16dev", lbm.F16DEV, 0),
                             ("f16dev_round_nearest", lbm.F16DEV, lbm.ROUND_NEAREST)):
        lat = lbm.Lattice(1024, 1024, 0.52, prec, flags | extra)
        lat.set_force(5e-7, 0.0)
        lat.set_geometry(crop)
        lat.step(steps)
        res[key] = lat.moments()
        lat.close()
    fluid = crop == 0
    acc = {}
    for name in ("f32", "f16dev", "f16dev_round_nearest"):
        r, x, y = res[name]
        r6, x6, y6 = res["f64"]
        acc[name] = {"rho_l2": l2_rel(r[fluid], r6[fluid]),
                     "u_l2": l2_rel(np.stack([x[fluid], y[fluid]]), np.stack([x6[fluid], y6[fluid]]))}
    out["accuracy_1024_window"] = {"steps": steps, "against": "f64 run of the same kernel", **acc}
    return out


def run_e2e(spec, args, torch, dist, readback="async"):
    """K steps through the C ABI: upload fields from pinned host memory, then
    frames of 2 steps each followed by a readback to pinned memory:
      "async"   rho/u (what render.rs takes) with lbm_read_moments_async into
                two alternating pinned host buffer sets, so each frame's host
                copy overlaps the next frame's steps and staging; the last one
                is waited for inside the timed region;
      "moments" the same fields with the blocking lbm_read_moments;
      "frame"   the finished RGBA8 velocity frame of lbm_render_async (the
                colour map of render.rs on the device) into two alternating
                pinned images, overlapped like "async";
      "mapped"  rho/u written by each frame's last step kernel straight into
                two alternating pinned host buffer sets (lbm_step_moments_to),
                no staging copy; the last frame is waited for inside the timed
                region."""
    from chemsim_gb300 import lbm
    from chemsim_gb300._lib import check
    flags = spec.flags | (0 if args.strict else lbm.FAST)
    pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()  # noqa: E731
    rho, ux, uy = pin(spec.rho), pin(spec.ux), pin(spec.uy)
    pinned = [[torch.empty((spec.h, spec.w), dtype=torch.float32).pin_memory() for _ in range(3)]
              for _ in range(2)]
    outs = [[t.numpy() for t in group] for group in pinned]
    ptrs = [[t.data_ptr() for t in group] for group in pinned]
    imgs = [torch.empty((spec.h, spec.w, 4), dtype=torch.uint8).pin_memory().numpy()
            for _ in range(2)]
    lat = lbm.Lattice(spec.w, spec.h, spec.tau, lbm.F32, flags)
    lat.set_force(*spec.force)
    lat.set_geometry(spec.solid)
    lat.init_equilibrium(rho, ux, uy)
    lat.step(args.warmup)
    # untimed: allocate the staging areas and make one transfer into every
    # host buffer the timed frames use (a buffer's first transfer pays its
    # host-side mapping setup)
    for j in range(2):
        if readback == "mapped":
            lat.step_moments_to(1, *ptrs[j])
        elif readback == "frame":
            lat.render_async(imgs[j], lbm.RENDER_VELOCITY)
        else:
            lat.read_moments_async(*outs[j])
        lat.readback_wait()
    lat.synchronize()
    frames = max(1, args.steps // 2)
    lib = lat._lib
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    lat.init_equilibrium(rho, ux, uy)
    for k in range(frames):
        if readback == "mapped":
            lat.step_moments_to(2, *ptrs[k & 1])
            continue
        lat.step_moments(2)
        if readback == "async":
            lat.read_moments_async(*outs[k & 1])
        elif readback == "moments":
            o = outs[0]
            check(lib.lbm_read_moments(lat.handle, o[0].ctypes.data, o[1].ctypes.data,
                                       o[2].ctypes.data, 0))
        else:
            lat.render_async(imgs[k & 1], lbm.RENDER_VELOCITY)
    lat.readback_wait()
    lat.synchronize()
    secs = time.perf_counter() - t0
    if dist is not None:
        t = torch.tensor([secs], device="cuda", dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        secs = float(t.item())
    lat.close()
    world = dist.get_world_size() if dist is not None else 1
    cells = spec.w * spec.h
    steps = 2 * frames
    per_frame = 4 * cells if readback == "frame" else 3 * 4 * cells
    notes = {"mapped": "rho/ux/uy every frame, written by the frame's last step kernel straight "
                       "into alternating pinned host buffers (lbm_step_moments_to, over the "
                       "host link; no staging copy)",
             "async": "rho/ux/uy every frame, lbm_read_moments_async into alternating pinned "
                      "buffers (staged in two device areas in turn; each host copy overlaps "
                      "the next frame's steps and staging)",
             "moments": "rho/ux/uy every frame, blocking lbm_read_moments",
             "frame": "one RGBA8 velocity frame every frame (lbm_render_async, render.rs colour "
                      "map; copy overlaps the next frame's steps)"}
    return {"value": round(cells * steps / secs / 1e6 * world, 1), "unit": "MLUPS",
            "h2d_bytes_per_step": int(3 * 4 * cells / steps),
            "d2h_bytes_per_step": int(per_frame / 2),
            "frames": frames, "steps_per_frame": 2,
            "note": "h2d: rho/ux/uy fields once per run, amortised; d2h: " + notes[readback]}


def main():
    args = parse_args()
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
