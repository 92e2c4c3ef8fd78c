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


def test_served_trace_follows_its_configuration():
    """The served trace: Poisson arrivals at 20 jobs/s; grid sides log-uniform from
    128 x 256 to 1024 x 4096; nt in [1000, 8000]; 1-32 shots per job sharing the job's
    model; about 80 % acoustic and 20 % elastic jobs; reproducible from the seed."""
    sys.path.insert(0, ROOT)
    import numpy as np
    import bench
    tr = bench._served_trace(40, 20.0, 0)
    assert len(tr) == 40
    arr = np.array([r.arrival for r in tr])
    assert np.all(np.diff(arr) >= 0)
    rate = (len(tr) - 1) / (arr[-1] - arr[0])
    assert 10.0 < rate < 40.0  # 20 jobs/s, 39 exponential gaps
    kinds = [r.kind for r in tr]
    assert 0.1 <= kinds.count("elastic") / len(tr) <= 0.35
    for r in tr:
        s0 = r.shots[0]
        assert 1 <= len(r.shots) <= 32
        assert 128 <= s0.nz <= 1024 and 256 <= s0.nx <= 4096
        assert 1000 <= len(s0.wavelet) <= 8000
        assert all((s.nz, s.nx, len(s.wavelet)) == (s0.nz, s0.nx, len(s0.wavelet))
                   for s in r.shots)
        assert all(s.vel_fwd is s0.vel_fwd for s in r.shots)  # one model per job
    again = bench._served_trace(40, 20.0, 0)
    assert [(r.kind, r.shots[0].nz, r.shots[0].nx, len(r.shots)) for r in again] == \
        [(r.kind, r.shots[0].nz, r.shots[0].nx, len(r.shots)) for r in tr]
