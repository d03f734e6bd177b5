"""Multi-process path of bench.py on CPU (gloo, world size 2): rank 0 alone runs the reference
arm and prints one JSON line; the other rank exits 0 without output."""
import json
import os
import socket
import subprocess
import sys

from conftest import ROOT


def free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def test_reference_arm_under_torchrun_world2():
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
           "--master-addr", "127.0.0.1", "--master-port", str(free_port()),
           os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2", "--steps", "2", "--warmup", "3"]
    env = dict(os.environ, OMP_NUM_THREADS="1")
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, env=env, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["cpu_baseline"]["cores"] >= 1


def test_serving_leg_reports_the_median_p99_run():
    """bench.py's serving leg runs the load several times and reports the run with the median
    p99 (one host-side stall should not decide the line), listing every run."""
    sys.path.insert(0, ROOT)
    import bench
    runs = [{"gsps": 2.0, "p50_us": 2200.0, "p99_us": 63000.0, "max_us": 160000.0, "requests": 1},
            {"gsps": 2.0, "p50_us": 2100.0, "p99_us": 3100.0, "max_us": 3600.0, "requests": 2},
            {"gsps": 2.0, "p50_us": 2150.0, "p99_us": 3200.0, "max_us": 3900.0, "requests": 3}]
    out = bench.median_p99_run(runs)
    assert out["requests"] == 3 and out["p99_us"] == 3200.0
    assert [r["p99_us"] for r in out["runs"]] == [63000.0, 3100.0, 3200.0]
    assert bench.median_p99_run(runs[:1])["requests"] == 1
