"""bench.py's reference arm on the CPU: the JSON line it prints (the keys,
types and fixed values every bench line carries, plus the reference arm's
impl, cpu_baseline and e2e), at one rank and under torchrun with two ranks,
where rank 0 alone runs the sample and prints.  A small R-MAT scale keeps
each run under a few seconds."""
import json
import os
import socket
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ARGS = ["--impl", "reference", "--scale", "14", "--steps", "2", "--warmup", "3"]


def json_lines(stdout):
    out = []
    for line in stdout.splitlines():
        line = line.strip()
        if line.startswith("{"):
            out.append(json.loads(line))
    return out


def check_line(d, n_gpus):
    assert d["metric"] == "walker steps/s (PageRank walks on R-MAT)"
    assert d["unit"] == "steps/s" and d["higher_is_better"] is True
    assert isinstance(d["value"], float) and d["value"] > 0
    assert d["n_gpus"] == n_gpus and d["steps"] == 2 and d["warmup"] == 3
    assert d["ms_per_step"] > 0
    assert d["scaling"] == "weak" and d["vs_baseline"] is None
    assert d["dtype"] == "u32" and d["data"] == "synthetic"
    assert "R-MAT scale 14" in d["config"]["workload"]
    assert d["impl"] == "reference"
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["value"] == d["value"] and cb["unit"] == d["unit"]
    assert isinstance(cb["cores"], int) and cb["cores"] >= 1 and cb["sample"]
    e2e = d["e2e"]
    assert e2e["value"] == d["value"] and e2e["unit"] == d["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0


def test_reference_arm_line():
    r = subprocess.run([sys.executable, "bench.py", *ARGS], cwd=ROOT, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = json_lines(r.stdout)
    assert len(lines) == 1
    check_line(lines[0], 1)


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_reference_arm_under_torchrun_prints_once():
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(free_port()), "bench.py", "--gpus", "2", *ARGS]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = json_lines(r.stdout)
    assert len(lines) == 1
    check_line(lines[0], 2)
