"""The bench's reference arm runs on the CPU (the oracle restatement of the
reference's path) and prints one JSON line with the contract's keys."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_json_line():
    env = dict(os.environ, OMP_NUM_THREADS="2")
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "1",
                        "--warmup", "1", "--cpu-nt", "20"], cwd=ROOT, env=env,
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.strip().splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
              "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config",
              "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["value"] > 0 and d["unit"] == "Gpts/s"
    cb = d["cpu_baseline"]
    for k in ("value", "unit", "cores", "kind", "sample"):
        assert k in cb, k
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1
    assert cb["one_thread"]["cores"] == 1 and cb["one_thread"]["value"] > 0
    e2e = d["e2e"]
    assert e2e["value"] == d["value"] and e2e["h2d_bytes_per_step"] == 0


def test_roofline_inputs_of_the_default_line():
    """The default line's roofline reads its DRAM traffic from the committed ncu summary
    (both regimes present and below the algorithmic bytes per launch), and its algorithmic
    bytes per shot follow the stated per-point counts at the benchmark size."""
    sys.path.insert(0, ROOT)
    import bench
    warm, cold = bench.committed_traffic(), bench.committed_traffic("cold_traffic_bytes_per_launch")
    assert warm is not None and cold is not None
    assert 0 < warm < cold < 112e6  # below the largest launch's algorithmic bytes

    class Survey:
        nz, nx, nt = 1000, 4000, 8000
    P = 1000 * 4000
    # 16 B per point per step in both passes; every second step of each pass adds 12 B
    # (snapshot store + illumination, or snapshot read + image)
    assert bench.bytes_per_shot(Survey, 2) == 2 * 8000 * P * 16 + 4000 * P * 12 * 2
    # per counted point (2 nz nx nt per shot): 22 B, as the batch line assumes
    assert bench.bytes_per_shot(Survey, 2) / (2 * P * 8000) == 22.0
