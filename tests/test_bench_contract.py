"""bench.py's reference arm without a GPU: the JSON line it prints (the keys and meanings
the GPU arm shares), and the torchrun form, where rank 0 alone runs and prints and the
other ranks exit 0 without work."""
import json
import os
import socket
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ARGS = ["--impl", "reference", "--steps", "2", "--warmup", "1", "--workload", "sweep_1M_g64",
        "--cpu-sample-tracks", "40"]


def json_lines(out: str):
    return [json.loads(x) for x in out.splitlines() if x.startswith("{")]


def check_line(r: dict, n_gpus: int):
    assert r["impl"] == "reference"
    assert r["value"] > 0 and r["ms_per_step"] > 0
    assert r["unit"] == r["cpu_baseline"]["unit"] == r["e2e"]["unit"]
    assert r["value"] == r["cpu_baseline"]["value"] == r["e2e"]["value"]
    assert (r["n_gpus"], r["steps"], r["warmup"]) == (n_gpus, 2, 1)
    assert r["higher_is_better"] is True and r["vs_baseline"] is None
    assert r["dtype"] == "f32" and r["data"].startswith("synthetic")
    assert r["config"]["workload"] == "sweep_1M_g64"
    assert (r["config"]["segments"], r["config"]["groups"]) == (1_000_000, 64)
    cb = r["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and "of 1000 tracks" in cb["sample"]
    assert r["e2e"]["h2d_bytes_per_step"] == 0 and r["e2e"]["d2h_bytes_per_step"] == 0


def test_reference_arm_line():
    out = subprocess.run([sys.executable, "bench.py", *ARGS], cwd=ROOT, capture_output=True,
                         text=True, timeout=600)
    assert out.returncode == 0, out.stderr
    lines = json_lines(out.stdout)
    assert len(lines) == 1
    check_line(lines[0], 1)


def free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_reference_arm_under_torchrun():
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node",
           "2", "--master-addr", "127.0.0.1", "--master-port", str(free_port()), "bench.py",
           "--gpus", "2", *ARGS]
    out = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr
    lines = json_lines(out.stdout)
    assert len(lines) == 1
    check_line(lines[0], 2)
