"""bench.py's reference arm (`--impl reference`) on the host cores: the keys of its JSON line,
and under torchrun with two ranks a single line, from rank 0.  A small dusty ring (64
planetesimals, 2,048 grains) keeps it to seconds."""
import json
import os
import socket
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]
ARGS = ["--impl", "reference", "--steps", "1", "--warmup", "0", "--n-dust", "2048", "--n-plsml", "64"]


def json_lines(out):
    return [json.loads(line) for line in out.splitlines() if line.startswith("{")]


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_reference_arm_line_has_the_contract_keys():
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), *ARGS], capture_output=True, text=True,
                       timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    (d,) = json_lines(r.stdout)
    assert d["impl"] == "reference" and d["metric"] and d["unit"] == "body-steps/s"
    assert d["value"] > 0 and d["higher_is_better"] is True and d["n_gpus"] == 1
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"] and cb["sample"]
    e = d["e2e"]
    assert e["value"] == d["value"] and e["unit"] == d["unit"]
    assert e["h2d_bytes_per_step"] == 0 and e["d2h_bytes_per_step"] == 0
    assert "n_grav - 1" in d["sample_note"]


def test_reference_arm_under_two_ranks_prints_one_line():
    env = dict(os.environ, OMP_NUM_THREADS="2")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(free_port()), str(ROOT / "bench.py"), "--gpus", "2",
           *ARGS]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    (d,) = json_lines(r.stdout)
    assert d["impl"] == "reference" and d["n_gpus"] == 2
