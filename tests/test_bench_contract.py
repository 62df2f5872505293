"""bench.py's reference arm prints the JSON line of the benchmark contract
(CPU only: the arm times the oracle's restatement of the reference step)."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_json_line():
    out = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--size", "256",
                          "--steps", "3", "--warmup", "3"],
                         cwd=ROOT, capture_output=True, text=True, timeout=600, check=True)
    line = json.loads(out.stdout.strip().splitlines()[-1])
    for key in ("metric", "value", "unit", "impl", "n_gpus", "steps", "warmup", "ms_per_step",
                "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config",
                "cpu_baseline", "e2e"):
        assert key in line, key
    assert line["impl"] == "reference" and line["metric"] == "D2Q9 MLUPS"
    assert line["unit"] == "MLUPS" and line["higher_is_better"] is True
    assert line["steps"] == 3 and line["warmup"] == 3 and line["n_gpus"] == 1
    assert line["value"] > 0 and line["ms_per_step"] > 0
    assert line["config"]["workload"].startswith("channel_256x256_")
    # the same config dict as the GPU arm's line, so the two arms compare
    sys.path.insert(0, ROOT)
    import argparse
    import bench
    assert line["config"] == bench.bench_config(argparse.Namespace(size=256), 1)
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == line["value"]
    e2e = line["e2e"]
    assert e2e["value"] == line["value"] and e2e["h2d_bytes_per_step"] == 0
    assert e2e["d2h_bytes_per_step"] == 0


def test_reference_arm_under_torchrun_prints_once():
    """Launched as the multi-GPU runs are (torchrun, 2 ranks): rank 0 alone
    times and prints; the other rank exits 0 without work."""
    import socket
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    out = subprocess.run([sys.executable, "-m", "torch.distributed.run", "--nnodes=1",
                          "--nproc-per-node", "2", "--master-addr", "127.0.0.1",
                          "--master-port", str(port), "bench.py", "--impl", "reference",
                          "--size", "256", "--steps", "3", "--warmup", "3"],
                         cwd=ROOT, capture_output=True, text=True, timeout=600, check=True)
    lines = [json.loads(l) for l in out.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    assert lines[0]["impl"] == "reference" and lines[0]["n_gpus"] == 2
