"""``bench.py --gpus N`` started as one plain process launches N ranks itself.

The reference arm runs on the CPU with the gloo backend, so this checks the
launcher here: two local ranks join one process group, rank 0 alone prints the
JSON line, and that line reports both ranks (``n_gpus`` is the process group's
size, not the flag).  The sample is a few time steps of the bench's grid.
"""
import json
import os
import subprocess
import sys

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_gpus_flag_launches_ranks():
    env = dict(os.environ, OMP_NUM_THREADS="2")
    env.pop("WORLD_SIZE", None)
    env.pop("RANK", None)
    env.pop("LOCAL_RANK", None)
    p = subprocess.run([sys.executable, os.path.join(REPO, "bench.py"), "--impl", "reference",
                        "--gpus", "2", "--steps", "1", "--warmup", "0", "--cpu-nt", "4"],
                       cwd=REPO, env=env, capture_output=True, text=True, timeout=600)
    assert p.returncode == 0, p.stderr[-3000:]
    lines = [ln for ln in p.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, p.stdout[-2000:]  # rank 0 alone prints
    out = json.loads(lines[0])
    assert out["impl"] == "reference" and out["n_gpus"] == 2
    assert out["value"] > 0 and out["e2e"]["value"] == out["value"]
