"""Benchmark of the GB300 RTM engine on the large plain 2D acoustic RTM workload.

Workload (one "step" = one RTM shot: forward modelling with illumination +
backward propagation with zero-lag imaging): grid 1000 x 4000, dx = dz = 2.5 m,
6 Hz Ricker, dt = 0.25 ms, nt = 8000, 4000 surface receivers, source on row 2;
seeded synthetic layered-gradient model with three faults, migration model
Gaussian-smoothed.  Metric: RTM Gpts/s, counting 2 * nz * nx * nt point-updates
per shot (forward + backward; recomputation not counted).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

* ``value``: device-timed (CUDA events on the engine stream), shot inputs already
  resident in HBM (``w2d_migrate_staged``), images stacked on the device.
* ``e2e``: the public drop-in call ``TSWRTMEngine.migrate_shot`` with host arrays
  in page-locked memory; the host->device copies of the gather, wavelet and both
  velocity models and the device->host copies of image and illumination are
  inside the timed region.
* ``roofline``: the fused step kernel, algorithmic bytes of all step launches in
  the timed region over the device time of the region, against the measured HBM
  copy bandwidth.
* ``cpu_baseline``: the reference's CPU path (wave2d.c + its Python time loops,
  restated in oracle/) timed on this host's cores over a bounded sample.
* ``--impl reference``: that CPU implementation alone, each step a bounded sample
  of the same workload (rank 0 only).

Other workloads (``--workload``), one JSON line each:

* ``small``: the reference's own example size (150 x 400, nt 2000, 20 shots), the whole
  ``TSWRTMEngine.migrate_multiple_shots`` call against the per-shot loop and the CPU path
  over all 20 shots.
* ``batched``: 256 uneven virtual-source gathers through the batch engine against the
  plain per-shot loop (shots/s).
* ``served``: a Poisson trace of acoustic and elastic jobs through the server against the
  plain FIFO per-shot loop (shots/s, p50 / p99 latency).
* ``elastic``: one elastic shot's forward modelling and exact adjoint gradient.
* ``interferometry``: virtual-source cross-correlation stacking (windows/s).
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import re
import statistics
import subprocess
import tempfile
import sys
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

METRIC = "RTM Gpts/s"
UNIT = "Gpts/s"
L2_NOTE = ("inputs larger than L2: every shot streams a 128 MB gather and a 64 GB forward "
           "snapshot store through HBM")


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class Dist:
    """Barrier / max-reduce over ranks (torch.distributed only when WORLD_SIZE > 1)."""

    def __init__(self, backend):
        self.rank, self.world, self.local = dist_env()
        self.pg = None
        if self.world > 1:
            import torch.distributed as td
            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            td.init_process_group(backend=backend)
            self.td = td

    def barrier(self):
        if self.world > 1:
            self.td.barrier()

    def max(self, v: float) -> float:
        if self.world == 1:
            return v
        import torch
        dev = "cuda" if self.td.get_backend() == "nccl" else "cpu"
        t = torch.tensor([v], dtype=torch.float64, device=dev)
        self.td.all_reduce(t, op=self.td.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.world > 1:
            self.td.destroy_process_group()


def launch_ranks(n: int) -> int:
    """``--gpus N`` started as a plain process: run this script again as N local ranks
    (one process per GPU, torch.distributed.run on 127.0.0.1) with the same arguments,
    and return the launcher's exit status.  Rank 0 prints the JSON line."""
    import socket
    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        port = sk.getsockname()[1]
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1",
           f"--nproc-per-node={n}", "--master-addr=127.0.0.1", f"--master-port={port}",
           os.path.abspath(__file__)] + sys.argv[1:]
    return subprocess.run(cmd).returncode


def measured_peaks():
    p = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def committed_traffic(key="traffic_bytes_per_launch"):
    """Per-launch DRAM bytes of the step kernel from the committed ncu summary, or None:
    `traffic_bytes_per_launch` in the live (warm-cache) regime, `cold_traffic_bytes_per_launch`
    with the caches flushed before each launch."""
    p = os.path.join(REPO, "profiles", "acoustic_step_large_plain.md")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        m = re.search(r"(?m)^" + key + r":\s*([0-9.eE+]+)", f.read())
    return float(m.group(1)) if m else None


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_id: str, rank: int):
        self.proc = None
        self.gpu = gpu_id
        # the samples go to BENCH_CLOCKS_DIR when set (to keep them), else a temporary folder
        out_dir = os.environ.get("BENCH_CLOCKS_DIR") or tempfile.gettempdir()
        self.path = os.path.join(out_dir, f"das_gb300_clocks_rank{rank}.csv")

    def start(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        rows = []
        with open(self.path) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    rows.append((float(parts[1]), float(parts[2]), float(parts[3]), parts[5:9]))
                except ValueError:
                    continue
        if not rows:
            return None
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i, v in enumerate(r[3]) if v.lower() == "active"})
        loaded = [r[0] for r in rows if r[2] > 200.0] or [r[0] for r in rows]
        return {"sm_mhz": statistics.median(loaded), "sm_max_mhz": max(r[1] for r in rows),
                "reasons": reasons, "samples": len(rows), "power_w_max": max(r[2] for r in rows)}


# Clock sampler running around a whole non-default workload (its line carries the record
# of the run; samples under load are those drawing more than 200 W).
_WORKLOAD_CLOCKS = None


def _emit(out: dict) -> None:
    """Print a workload's JSON line with the clock record of its run."""
    if _WORKLOAD_CLOCKS is not None:
        out["clocks"] = _WORKLOAD_CLOCKS.stop()
    print(json.dumps(out), flush=True)


def _gpu_bus_id(local: int) -> str:
    import das_gb300
    lib = das_gb300.lib()
    bus = ctypes.create_string_buffer(64)
    return bus.value.decode() if lib.w2d_device_pci_bus_id(bus, 64) == 0 else str(local)


# ------------------------------------------------------------------------------ workload

def make_survey(nt):
    from das_gb300.synthetic import plain_large
    return plain_large(seed=0, nt=nt)


def bytes_per_shot(sv, interval):
    """Algorithmic HBM bytes of the fused step launches of one RTM shot.

    Forward step: read p_curr, p_prev, vel^2 dt^2, write p_next = 16 B/pt; on
    snapshot steps +4 (snapshot store) +8 (illumination read-modify-write).
    Backward step: 16 B/pt; on imaging steps +4 (snapshot read) +8 (image RMW).
    """
    P = sv.nz * sv.nx
    n_snaps = (sv.nt - 1) // interval + 1
    return 2 * sv.nt * P * 16 + n_snaps * P * 12 * 2


def cpu_sample(sv, gather, nt_sample, threads):
    """Reference CPU path (oracle restatement of wave2d.c + its Python loops) on a sample."""
    os.environ["OMP_NUM_THREADS"] = str(threads)
    from oracle import oracle as o
    kind = "reference" if o.reference_available() else "port"
    prev = o.backend()
    o.set_backend("reference" if kind == "reference" else "native")
    o.set_num_threads(threads)
    g = o.Grid(sv.nx, sv.nz, sv.dx, sv.dz, sv.dt, sv.n_sponge, sv.sponge_alpha, True)
    sponge = g.sponge()
    w = sv.wavelet[:nt_sample]
    data = np.ascontiguousarray(gather[:nt_sample])
    try:
        t0 = time.perf_counter()
        o.migrate_shot(g, sv.vel_mig, sv.vel_mig, w, int(sv.src_ix[0]), sv.src_iz, data,
                       sv.rec_ix, sv.rec_iz, 2, sponge=sponge, native=True)
        el = time.perf_counter() - t0
    finally:
        o.set_backend(prev)  # the parity checks use the bit-exact restatement
    pts = 2 * sv.nz * sv.nx * nt_sample
    return pts / el / 1e9, el, kind


def cpu_one_thread(sv, gather, nt_sample, threads):
    """The same sample on one host thread, over 1/threads of the steps (same wall time
    as the all-core sample at ideal scaling); restores the all-core setting."""
    from oracle import oracle as o
    nt1 = max(20, nt_sample // max(threads, 1))
    v, el, _ = cpu_sample(sv, gather, nt1, 1)
    o.set_num_threads(threads)
    os.environ["OMP_NUM_THREADS"] = str(threads)
    return {"value": v, "cores": 1,
            "sample": f"the same migrate_shot truncated to nt={nt1}, {el:.1f} s"}


def run_reference(args, dist):
    """--impl reference: the CPU implementation timed on the host cores (rank 0 only)."""
    if dist.rank != 0:
        return
    threads = len(os.sched_getaffinity(0))
    os.environ["OMP_NUM_THREADS"] = str(threads)
    from das_gb300.synthetic import plain_large
    nt_sample = args.cpu_nt
    sv = plain_large(seed=0, nt=8000)
    rng = np.random.default_rng(1)
    gather = (rng.standard_normal((nt_sample, sv.nx)) * 1e-9).astype(np.float32)
    vals = []
    kind = None
    for k in range(args.warmup + args.steps):
        v, el, kind = cpu_sample(sv, gather, nt_sample, threads)
        if k >= args.warmup:
            vals.append((v, el))
    gpts = sum(2 * sv.nz * sv.nx * nt_sample for _ in vals) / sum(e for _, e in vals) / 1e9
    ms = 1e3 * sum(e for _, e in vals) / len(vals)
    one = cpu_one_thread(sv, gather, nt_sample, threads)
    sample = (f"migrate_shot on the 1000x4000 grid truncated to nt={nt_sample} steps "
              f"(forward+backward, snapshot interval 2, 4000 receivers) per step")
    out = {"impl": "reference", "metric": METRIC, "value": gpts, "unit": UNIT, "n_gpus": dist.world,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
           "config": {"workload": sv.name, "nz": sv.nz, "nx": sv.nx, "nt": sv.nt,
                      "sampled_nt": nt_sample, "parallelism": "cpu"},
           "cpu_baseline": {"value": gpts, "unit": UNIT, "cores": threads, "kind": kind,
                            "sample": sample, "one_thread": one},
           "e2e": {"value": gpts, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def accuracy_statement(storage="auto"):
    """Parity and float64 error of the GPU migration on the benchmarked 1000 x 4000 grid
    (same models, sponge, 4000 receivers) cut to 240 time steps, with the 6 Hz Ricker
    taken from sample 560 on so its main lobe falls inside the window: one mid-line
    shot, observed gather forward-modelled on the GPU in the true model and checked
    against the oracle, then migrated; image and illumination against the oracle's
    float32 restatement (the reference's arithmetic, expected bit-identical) and
    against its float64 run of the same stencil.  The oracle runs on the host (test
    infrastructure; not part of the timed work)."""
    from oracle import oracle as o
    from das_gb300.rtm_engine import TSWRTMEngine
    from das_gb300.synthetic import plain_large_window
    from das_gb300.velocity_flood import FloodModels
    from das_gb300.wave_solver import WaveSolver2D
    o.set_backend("port")  # the restatement without FMA contraction: the reference's rounding
    sv = plain_large_window(240)
    six = int(sv.src_ix[117])
    grid = o.Grid(sv.nx, sv.nz, sv.dx, sv.dz, sv.dt, sv.n_sponge, sv.sponge_alpha, True)
    s = WaveSolver2D(sv.nx, sv.nz, sv.dx, sv.dz, sv.dt, sv.n_sponge, sv.sponge_alpha, True)
    data, _ = s.forward_propagate_acoustic(sv.vel_true, sv.wavelet, six, sv.src_iz, sv.rec_ix,
                                           sv.rec_iz)
    data_o, _ = o.forward_propagate_acoustic(grid, sv.vel_true, sv.wavelet, six, sv.src_iz,
                                             sv.rec_ix, sv.rec_iz)
    img, ill = TSWRTMEngine(s, storage).migrate_shot(
        FloodModels(sv.vel_true, sv.vel_mig, sv.vel_mig, 0, 0), sv.wavelet, six, sv.src_iz, data,
        sv.rec_ix, sv.rec_iz, 2)
    used = s.last_stats()["storage"]
    s.close()
    img32, ill32 = o.migrate_shot(grid, sv.vel_mig, sv.vel_mig, sv.wavelet, six, sv.src_iz, data,
                                  sv.rec_ix, sv.rec_iz, 2)
    img64, ill64 = o.migrate_shot(grid, sv.vel_mig, sv.vel_mig, sv.wavelet, six, sv.src_iz, data,
                                  sv.rec_ix, sv.rec_iz, 2, precision="f64")
    return {"case": f"{sv.name}, one shot at column {six}, storage {used}",
            "traces_vs_reference_f32_rel_l2": o.rel_l2(data, data_o),
            "traces_max_abs_diff_vs_reference_f32": float(np.max(np.abs(data - data_o))),
            "image_vs_reference_f32_rel_l2": o.rel_l2(img, img32),
            "image_max_abs_diff_vs_reference_f32": float(np.max(np.abs(img - img32))),
            "illum_vs_reference_f32_rel_l2": o.rel_l2(ill, ill32),
            "image_vs_fp64_rel_l2": o.rel_l2(img, img64),
            "illum_vs_fp64_rel_l2": o.rel_l2(ill, ill64),
            "tolerance_image_rel_l2": 1e-4, "tolerance_traces_rel_l2": 1e-5}


def run_ours(args, dist):
    import das_gb300
    from das_gb300 import _lib
    from das_gb300.rtm_engine import TSWRTMEngine
    from das_gb300.velocity_flood import FloodModels
    from das_gb300.wave_solver import WaveSolver2D
    from das_gb300.pinned import pinned_array

    lib = das_gb300.lib()
    if dist.world > 1:
        _lib.check(lib.w2d_set_device(dist.local))
    bus = ctypes.create_string_buffer(64)
    gpu_id = bus.value.decode() if lib.w2d_device_pci_bus_id(bus, 64) == 0 else str(dist.local)
    sv = make_survey(args.nt)
    interval = 2
    solver = WaveSolver2D(sv.nx, sv.nz, sv.dx, sv.dz, sv.dt, sv.n_sponge, sv.sponge_alpha, True)
    if args.tile:
        solver.tile = tuple(int(t) for t in args.tile.split(","))
    solver.l2_hints = bool(args.l2_hints)
    solver.set_launch(args.launch, bool(args.pdl))
    solver.set_graphs(bool(args.graphs))
    if args.two_step:
        solver.set_two_step(int(args.two_step))
    eng = solver._eng()
    K, W = args.steps, args.warmup
    n_sh = K + W
    # this rank's shots (weak scaling: every rank migrates its own K + W shots)
    shots = [int(sv.src_ix[(dist.rank * n_sh + k) * 7 % len(sv.src_ix)]) for k in range(n_sh)]

    # observed gathers: forward modelling in the true model on the GPU (untimed set-up)
    gathers = []
    for six in shots[: min(n_sh, args.distinct_gathers)]:
        rec, _ = solver.forward_propagate_acoustic(sv.vel_true, sv.wavelet, six, sv.src_iz,
                                                   sv.rec_ix, sv.rec_iz)
        gathers.append(rec)
    gathers = [gathers[k % len(gathers)] for k in range(n_sh)]
    rix = sv.rec_ix.astype(np.int32)
    fm = FloodModels(sv.vel_true, sv.vel_mig, sv.vel_mig, 0, 0)
    solver._set_velocity(0, sv.vel_mig)
    solver._set_velocity(1, sv.vel_mig)
    for k in range(n_sh):
        _lib.check(lib.w2d_shot_stage(eng, k, sv.wavelet.ctypes.data, sv.nt,
                                      gathers[k].ctypes.data, sv.nx))
    _lib.check(lib.w2d_stack_reset(eng))
    storage = {"auto": 0, "all": 1, "checkpoint": 2}[args.storage]

    def staged(k):
        _lib.check(lib.w2d_migrate_staged(eng, k, shots[k], sv.src_iz, rix.ctypes.data, sv.nx,
                                          sv.rec_iz, interval, storage, None, None))
        return solver.last_stats()

    for k in range(W):
        staged(k)
    clocks = Clocks(gpu_id, dist.rank)
    clocks.start()
    dist.barrier()
    _lib.check(lib.w2d_engine_timer_start(eng))
    launches = 0
    recompute = 0
    used = None
    t_wall = time.perf_counter()
    for k in range(W, W + K):
        st = staged(k)
        launches += st["step_launches"]
        recompute += st["recomputed_steps"]
        used = st["storage"]
    ms = ctypes.c_float()
    _lib.check(lib.w2d_engine_timer_stop(eng, ctypes.byref(ms)))
    wall = time.perf_counter() - t_wall
    free_b, total_b = _lib.device_memory()  # the engine still holds its buffers here
    dist.barrier()
    clk = clocks.stop()
    dev_s = dist.max(ms.value / 1e3)
    pts = sv.counted_points_per_shot()
    value = pts * K * dist.world / dev_s / 1e9

    # roofline of the fused step kernel over the timed region
    peak, peak_kind = measured_peaks()
    step_launches_per_shot = 2 * sv.nt + recompute // max(K, 1)
    algo_bytes = bytes_per_shot(sv, interval) * K + recompute * sv.nz * sv.nx * 16
    achieved = algo_bytes / (ms.value / 1e3) / 1e9
    per_launch = algo_bytes / (step_launches_per_shot * K)
    traffic = committed_traffic()

    # end-to-end through the public drop-in call, inputs in page-locked host memory
    ke = max(1, min(K, args.e2e_steps))
    pin_g = [pinned_array(gathers[W + k].shape) for k in range(ke)]
    for k in range(ke):
        pin_g[k][...] = gathers[W + k]
    pin_w = pinned_array(sv.wavelet.shape)
    pin_w[...] = sv.wavelet
    pin_vs = pinned_array(sv.vel_mig.shape)
    pin_vs[...] = sv.vel_mig
    pin_vr = pinned_array(sv.vel_mig.shape)
    pin_vr[...] = sv.vel_mig
    fm_p = FloodModels(sv.vel_true, pin_vs, pin_vr, 0, 0)
    eng_api = TSWRTMEngine(solver, storage=args.storage)
    eng_api.migrate_shot(fm_p, pin_w, shots[0], sv.src_iz, pin_g[0], sv.rec_ix, sv.rec_iz, interval)
    dist.barrier()
    t0 = time.perf_counter()
    calls = []
    for k in range(ke):
        tc = time.perf_counter()
        img, ill = eng_api.migrate_shot(fm_p, pin_w, shots[W + k], sv.src_iz, pin_g[k], sv.rec_ix,
                                        sv.rec_iz, interval)
        calls.append(((time.perf_counter() - tc) * 1e3, solver.last_stats()["device_ms"]))
    e2e_s = dist.max(time.perf_counter() - t0)
    e2e = pts * ke * dist.world / e2e_s / 1e9
    h2d = gathers[0].nbytes + sv.wavelet.nbytes + 2 * sv.vel_mig.nbytes + rix.nbytes
    d2h = 2 * sv.nz * sv.nx * 4

    cpu = None
    if dist.rank == 0 and args.cpu_nt > 0:
        threads = len(os.sched_getaffinity(0))
        v, el, kind = cpu_sample(sv, gathers[0], args.cpu_nt, threads)
        cpu = {"value": v, "unit": UNIT, "cores": threads, "kind": kind,
               "sample": f"migrate_shot on the 1000x4000 grid truncated to nt={args.cpu_nt} "
                         f"(forward+backward, interval 2, 4000 receivers), {el:.1f} s",
               "one_thread": cpu_one_thread(sv, gathers[0], args.cpu_nt, threads)}

    acc = accuracy_statement(args.storage) if dist.rank == 0 and args.accuracy else None

    if dist.rank == 0:
        out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": dist.world, "steps": K,
               "warmup": W, "ms_per_step": dev_s * 1e3 / K, "higher_is_better": True,
               "scaling": "weak", "vs_baseline": None, "dtype": "f32",
               "data": "synthetic (seeded layered-gradient model with 3 faults; gathers "
                       "forward-modelled on the GPU in the true model)",
               "config": {"workload": sv.name, "nz": sv.nz, "nx": sv.nx, "nt": sv.nt,
                          "dx": sv.dx, "dt": sv.dt, "receivers": int(len(sv.rec_ix)),
                          "shots_per_step": 1, "snapshot_interval": interval,
                          "storage": used, "tile": list(solver.tile or (4, 4)),
                          "launch": args.launch, "pdl": bool(args.pdl),
                          "graphs": bool(args.graphs), "two_step": args.two_step,
                          "l2": L2_NOTE, "parallelism": f"shots sharded over {dist.world} GPU(s)"},
               "shots_per_s": K * dist.world / dev_s,
               "recomputed_steps_per_shot": recompute / max(K, 1),
               "device_memory_in_use_gb": (total_b - free_b) / 1e9,
               "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                            "frac": achieved / peak, "traffic": traffic,
                            "traffic_cold": committed_traffic("cold_traffic_bytes_per_launch"),
                            "limiter": "latency: the three wave planes and the model (64 MB) "
                                       "stay in L2 from step to step, so DRAM carries the "
                                       "snapshot stream and write-backs (traffic: warm-cache "
                                       "ncu, per launch) and each CTA waits on its own TMA "
                                       "round trip; frac is algorithmic bytes over the HBM "
                                       "copy rate",
                            "peak_source": f"{peak_kind} hbm_gbs",
                            "kernel": "acoustic_step_kernel (fused forward / backward+imaging)",
                            "algorithmic_bytes_per_launch": per_launch},
               "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                       "d2h_bytes_per_step": int(d2h), "steps": ke,
                       "per_call_ms": [round(c, 2) for c, _ in calls],
                       "per_call_device_ms": [round(d, 2) for _, d in calls],
                       "api": "TSWRTMEngine.migrate_shot (pinned host arrays)"},
               "cpu_baseline": cpu, "clocks": clk, "gpu_launches": int(launches),
               "wall_s_timed_region": wall, "accuracy": acc}
        print(json.dumps(out), flush=True)


def _batched_jobs(n, seed, nt_scale=1.0, pinned=False):
    """Uneven virtual-source gathers (nx 400-2000, nz 200-600, dx 5 m, nt 1500-4000):
    seeded smoothed faulted models, 3-5 Hz Ricker, band-limited random traces as
    observed gathers (their values do not change the work).  pinned: models and
    gathers in page-locked host memory, so admission copies run as DMA."""
    from das_gb300.batch import ShotJob
    from das_gb300.pinned import pinned_array
    from das_gb300.synthetic import batched_gathers
    jobs = []
    rng = np.random.default_rng(seed + 1)
    for gth in batched_gathers(n, seed=seed):
        nt = max(16, int(gth.nt * nt_scale))
        w = gth.wavelet[:nt]
        rix = np.arange(gth.nx)
        data = (rng.standard_normal((nt, gth.nx)) * 1e-8).astype(np.float32)
        vel = gth.vel
        if pinned:
            pd, pv = pinned_array(data.shape), pinned_array(vel.shape)
            pd[...] = data
            pv[...] = vel
            data, vel = pd, pv
        jobs.append(ShotJob(gth.nx, gth.nz, gth.dx, gth.dx, gth.dt, vel, vel, w, data, rix,
                            gth.src_ix, 2, 2, 2, 40, 0.0015, True))
    return jobs


def cpu_job_rate(job, nt_sample):
    """The reference's CPU path (oracle port of wave2d.c and its Python loops, all host
    cores) on one ShotJob truncated to nt_sample steps: (counted Gpts/s, seconds)."""
    threads = len(os.sched_getaffinity(0))
    os.environ["OMP_NUM_THREADS"] = str(threads)
    from oracle import oracle as o
    kind = "reference" if o.reference_available() else "port"
    prev = o.backend()
    o.set_backend("reference" if kind == "reference" else "native")
    o.set_num_threads(threads)
    g = o.Grid(job.nx, job.nz, job.dx, job.dz, job.dt, job.n_sponge, job.sponge_alpha,
               job.free_surface_top)
    n = min(nt_sample, len(job.wavelet))
    try:
        t0 = time.perf_counter()
        o.migrate_shot(g, job.vel_fwd, job.vel_bwd, job.wavelet[:n], job.source_ix,
                       job.source_iz, np.ascontiguousarray(job.data[:n]), job.receiver_ix,
                       job.receiver_iz, job.snapshot_interval, sponge=g.sponge(), native=True)
        el = time.perf_counter() - t0
    finally:
        o.set_backend(prev)
    return 2.0 * job.nx * job.nz * n / el / 1e9, el, threads, kind


def run_batched(args, dist):
    """Batched workload: batched persistent engine vs the plain per-shot GPU loop."""
    from das_gb300.batch import BatchEngine
    from das_gb300.rtm_engine import TSWRTMEngine
    from das_gb300.velocity_flood import FloodModels
    from das_gb300.wave_solver import WaveSolver2D
    jobs = _batched_jobs(args.batch_shots, seed=0, nt_scale=args.batch_nt_scale, pinned=True)
    pts = sum(j.counted_points for j in jobs)
    tile = tuple(int(t) for t in (args.tile or "4,4").split(","))
    tune_table = None
    form = args.batch_form
    if args.autotune:
        from das_gb300.autotune import tune_batch
        (tile, args.spl, args.lpg, form), tune_table = tune_batch(jobs, use_cache=False)
    eng = BatchEngine(arena_bytes=int(args.arena_gb * (1 << 30)), max_shots=len(jobs), tile=tile,
                      steps_per_launch=args.spl, launches_per_graph=args.lpg, form=form)
    eng.run(jobs[: min(4, len(jobs))])  # warm-up: graph capture, first-touch of the arena
    t0 = time.perf_counter()
    _, st = eng.run(jobs)
    wall = time.perf_counter() - t0
    # plain per-shot loop over a sample of the same shots
    k = min(args.plain_shots, len(jobs))
    plain_s, plain_pts = 0.0, 0
    for j in jobs[:k]:
        s = WaveSolver2D(j.nx, j.nz, j.dx, j.dz, j.dt, j.n_sponge, j.sponge_alpha, True)
        e = TSWRTMEngine(s, "all")
        fm = FloodModels(j.vel_fwd, j.vel_fwd, j.vel_bwd, 0, 0)
        e.migrate_shot(fm, j.wavelet[:32], j.source_ix, j.source_iz, j.data[:32], j.receiver_ix,
                       2, 2)  # warm the engine
        t = time.perf_counter()
        e.migrate_shot(fm, j.wavelet, j.source_ix, j.source_iz, j.data, j.receiver_ix, 2, 2)
        plain_s += time.perf_counter() - t
        plain_pts += j.counted_points
        s.close()
    out = {"metric": "batched RTM shots/s", "value": len(jobs) / wall, "unit": "shots/s",
           "n_gpus": 1, "higher_is_better": True, "dtype": "f32", "data": "synthetic",
           "config": {"workload": f"{len(jobs)} uneven virtual-source gathers (nx 400-2000, nz "
                                  f"200-600, dx 5 m, nt scale {args.batch_nt_scale}), models "
                                  f"and gathers in pinned host memory",
                      "tile": list(tile), "steps_per_launch": args.spl,
                      "launches_per_graph": args.lpg, "form": form, "arena_gb": args.arena_gb},
           "gpts_per_s_wall": pts / wall / 1e9,
           "gpts_per_s_device": st["counted_points"] / (st["device_ms"] / 1e3) / 1e9,
           "wall_s": wall, "max_active_shots": st["max_active"],
           "plain_loop": {"shots": k, "shots_per_s": k / plain_s,
                          "gpts_per_s": plain_pts / plain_s / 1e9},
           "speedup_vs_plain_loop_gpts": (pts / wall) / (plain_pts / plain_s),
           "autotune": tune_table}
    if args.cpu_nt > 0:
        rate, el, threads, kind = cpu_job_rate(jobs[0], args.cpu_nt)
        cpu_s = pts / (rate * 1e9)
        out["cpu_baseline"] = {
            "value": len(jobs) / cpu_s, "unit": "shots/s", "cores": threads, "kind": kind,
            "sample": f"migrate_shot of gather 0 ({jobs[0].nz}x{jobs[0].nx}) truncated to "
                      f"nt={min(args.cpu_nt, len(jobs[0].wavelet))}: {rate:.2f} Gpts/s in "
                      f"{el:.1f} s, extrapolated to the {len(jobs)} gathers' {pts / 1e12:.2f} T "
                      f"counted points"}
    # roofline of the batch kernel at the device rate: 22 algorithmic bytes per counted
    # point at snapshot interval 2 (16 per step; every second forward step adds 12 for the
    # snapshot and illumination, every second backward step 12 for the imaging)
    peak, peak_kind = measured_peaks()
    dev = out["gpts_per_s_device"] * 1e9 * 22.0 / 1e9
    out["roofline"] = {"bound": "hbm", "achieved": dev, "peak": peak, "unit": "GB/s",
                       "frac": dev / peak, "peak_source": f"{peak_kind} hbm_gbs",
                       "kernel": "acoustic_batch_step_kernel", "bytes_per_counted_point": 22.0}
    _emit(out)


def _served_trace(n_jobs, rate, seed, side_scale=1.0, nt_scale=1.0):
    """Poisson arrivals at `rate` jobs/s; grid sides log-uniform from 128 x 256 to
    1024 x 4096 (times side_scale), nt uniform in [1000, 8000] (times nt_scale), 1-32
    shots per job sharing the job's smoothed faulted model; 80 % acoustic / 20 % elastic
    (the same size distribution for both kinds)."""
    from das_gb300.batch import ShotJob
    from das_gb300.serving import poisson_trace
    from das_gb300.synthetic import _layered_faulted
    from das_gb300.wave_solver import ricker_wavelet
    from scipy.ndimage import gaussian_filter

    def make(i, rng):
        nz = int(np.exp(rng.uniform(np.log(128), np.log(1024))) * side_scale)
        nx = int(np.exp(rng.uniform(np.log(256), np.log(4096))) * side_scale)
        nt = max(64, int(rng.integers(1000, 8001) * nt_scale))
        kind = "elastic" if rng.uniform() < 0.2 else "acoustic"
        nz, nx = max(nz, 48), max(nx, 96)
        d = 5.0
        zmax = (nz - 1) * d
        faults = [(rng.uniform(0.2, 0.8) * (nx - 1) * d, rng.uniform(45.0, 80.0),
                   rng.uniform(-0.08, 0.08) * zmax) for _ in range(int(rng.integers(1, 4)))]
        v = _layered_faulted(nz, nx, d, d, 0.45 * zmax, 0.12 * zmax, 0.0, faults, v1=3000.0)
        v = gaussian_filter(v, 3.0).astype(np.float32)
        dt = 5e-4
        w, _ = ricker_wavelet(float(rng.uniform(3.0, 5.0)), dt, nt * dt)
        n_sh = int(rng.integers(1, 33))
        if kind == "elastic":
            # shear velocity from the same model; vertical-strain observations
            vs = (v / 1.73).astype(np.float32)  # vp = 1.73 vs = v: same CFL as the acoustic
            dte, nte = dt, nt
            we, _ = ricker_wavelet(float(rng.uniform(3.0, 5.0)), dte, nte * dte)
            we = (we * 1e6).astype(np.float32)
            rix = np.arange(2, nx - 2)
            data = (rng.standard_normal((nte, len(rix))) * 1e-3).astype(np.float32)
            shots = [ShotJob(nx, nz, d, d, dte, vs, vs, we, data, rix,
                             int(2 + (k + 0.5) * (nx - 4) / n_sh), 2, 2, 2, 30, 0.0015, True)
                     for k in range(n_sh)]
            return kind, shots
        rix = np.arange(nx)
        data = (rng.standard_normal((nt, nx)) * 1e-8).astype(np.float32)
        shots = [ShotJob(nx, nz, d, d, dt, v, v, w, data, rix,
                         int((k + 0.5) * nx / n_sh), 2, 2, 2, 30, 0.0015, True)
                 for k in range(n_sh)]
        return kind, shots

    return poisson_trace(n_jobs, rate, make, seed=seed)


def run_elastic(args, dist):
    """Elastic gradient workload: 1024 x 2048 grid, dx 2 m, free surface, vs 300 -> 1200 m/s
    with a 20 m low-velocity zone dipping 70 degrees, vp = 1.73 vs, Gardner density; 5 Hz
    Ricker, dt 0.2 ms, nt 6000; vertical-strain receivers on every interior column; 64
    surface sources.  A step is one shot's forward modelling + adjoint gradient through
    torch.autograd, accumulated into the survey gradient; by default the timed steps are
    the 64 sources once each (``--el-shots``), after warm-up shots on the first sources."""
    import torch
    from scipy.ndimage import gaussian_filter
    from das_gb300.elastic import ElasticSolver2D, elastic_traces
    from das_gb300.synthetic import elastic_fault_zone
    from das_gb300.wave_solver import ricker_wavelet
    nz, nx, d, dt = 1024, 2048, 2.0, 2e-4
    nt = args.el_nt
    vs_true = elastic_fault_zone(nz, nx, d)
    vs_mig = gaussian_filter(vs_true.astype(np.float64), 5.0).astype(np.float32)
    w, _ = ricker_wavelet(5.0, dt, nt * dt)
    w = (w * 1e6).astype(np.float32)
    rix = np.arange(2, nx - 2)
    solver = ElasticSolver2D(nx, nz, d, d, dt, n_sponge=40, sponge_alpha=0.0015)
    solver.set_adjoint(args.el_adjoint)
    el_step, el_adj = ([int(v) for v in t.split(",")] for t in args.el_tiles.split(":"))
    solver.set_tiles(el_step, el_adj)
    src = [int(s) for s in np.linspace(40, nx - 41, 64).astype(int)]
    K = args.el_shots if args.el_shots > 0 else args.steps
    W = max(3, args.warmup)
    order = [src[k % 64] for k in range(W)] + [src[k % 64] for k in range(K)]
    vt = torch.tensor(vs_true, device="cuda")
    obs = {}
    for six in order:
        if six not in obs:
            with torch.no_grad():
                obs[six] = elastic_traces(vt, solver, w, six, 2, rix, 2).clone()
    times = []
    fwd_ms, grad_ms = [], []
    v = torch.tensor(vs_mig, device="cuda", requires_grad=True)
    for k, six in enumerate(order):
        if k == W:
            v.grad = None  # the survey gradient sums the timed shots only
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        dd = elastic_traces(v, solver, w, six, 2, rix, 2)
        f_ms = solver.last_ms
        J = 0.5 * torch.sum((dd - obs[six]) ** 2)
        J.backward()
        torch.cuda.synchronize()
        if k >= W:
            times.append(time.perf_counter() - t0)
            fwd_ms.append(f_ms)
            grad_ms.append(solver.last_ms)
    g = v.grad.detach()
    survey = {"shots": K, "distinct_sources": len(set(order[W:])),
              "gradient_finite": bool(torch.isfinite(g).all().item()),
              "gradient_max_abs": float(g.abs().max().item())}
    pts = 2.0 * nz * nx * nt
    # roofline of the gradient phase (the device time of J.backward): per time step and
    # grid point the recomputation moves 56 B (the forward step: five fields read and
    # written, lambda, mu and the two buoyancies read) + 20 B (the five fields stored
    # into the segment), and the two tiled adjoint passes 28 + 14 planes = 168 B
    peak, peak_kind = measured_peaks()
    grad_bytes = nz * nx * nt * (56 + 20 + 168)
    achieved = grad_bytes / (statistics.mean(grad_ms) / 1e3) / 1e9
    fwd_achieved = nz * nx * nt * 56 / (statistics.mean(fwd_ms) / 1e3) / 1e9
    out = {"metric": "elastic RTM gradient Gpts/s", "value": pts * K / sum(times) / 1e9,
           "unit": "Gpts/s", "n_gpus": 1, "higher_is_better": True, "dtype": "f32",
           "data": "synthetic", "steps": K, "warmup": W,
           "config": {"workload": f"elastic velocity-stress gradient 1024x2048, dx 2 m, nt {nt}, "
                                  f"{len(rix)} vertical-strain receivers, 5 Hz, checkpointed, "
                                  f"{K} shots over the 64 surface sources into one gradient",
                      "adjoint": args.el_adjoint, "tiles": args.el_tiles},
           "s_per_shot": sum(times) / K, "survey": survey,
           "device_ms_forward": statistics.mean(fwd_ms),
           "device_ms_gradient": statistics.mean(grad_ms),
           "counted_points_per_shot": pts,
           "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                        "frac": achieved / peak, "traffic": None,
                        "peak_source": f"{peak_kind} hbm_gbs",
                        "kernel": "gradient phase: el_adj_a + el_adj_b (tiled adjoint passes) "
                                  "and the segment recomputation's step kernels",
                        "algorithmic_bytes_per_step_point": 56 + 20 + 168,
                        "forward_phase_achieved_gbs": fwd_achieved,
                        "forward_phase_frac": fwd_achieved / peak}}
    _emit(out)


def run_gradient(args, dist):
    """Acoustic velocity gradient (the differentiable form): the 1000 x 4000 grid, nt 8000,
    receivers on every written column of row 2; per step one shot's forward modelling
    through ``das_gb300.autograd`` and the misfit's backward (the hand-written adjoint
    kernel over the forward wavefield recomputed segment by segment from checkpoints),
    accumulated into one gradient over the shots of the run."""
    import torch
    from das_gb300.autograd import model_traces
    from das_gb300.wave_solver import WaveSolver2D
    sv = make_survey(args.nt)
    nz, nx, nt = sv.nz, sv.nx, sv.nt
    rix = np.asarray(sv.rec_ix)[2:-2]  # receivers must sit on cells the scheme writes
    s = WaveSolver2D(sv.nx, sv.nz, sv.dx, sv.dz, sv.dt, sv.n_sponge, sv.sponge_alpha, True)
    K, W = args.steps, max(3, args.warmup)
    order = [int(sv.src_ix[(17 * k) % len(sv.src_ix)]) for k in range(W + K)]
    vt = torch.tensor(sv.vel_true, device="cuda")
    obs = {}
    with torch.no_grad():
        for six in order:
            if six not in obs:
                obs[six] = model_traces(vt, s, sv.wavelet, six, sv.src_iz, rix, sv.rec_iz).clone()
    v = torch.tensor(sv.vel_mig, device="cuda", requires_grad=True)
    fwd_s, grad_s, times = [], [], []
    for k, six in enumerate(order):
        if k == W:
            v.grad = None  # the gradient sums the timed shots only
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        d = model_traces(v, s, sv.wavelet, six, sv.src_iz, rix, sv.rec_iz)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        J = 0.5 * torch.sum((d - obs[six]) ** 2)
        J.backward()
        torch.cuda.synchronize()
        t2 = time.perf_counter()
        if k >= W:
            fwd_s.append(t1 - t0)
            grad_s.append(t2 - t1)
            times.append(t2 - t0)
    recomputed = s.last_stats()["recomputed_steps"]
    g = v.grad.detach()
    s.close()
    pts = 2.0 * nz * nx * nt
    # gradient phase per time step and grid point: the recomputed forward step (16 B) and
    # its store into the segment (4 B), the adjoint step (a[n+1], c, P[n], a[n+2] read,
    # a[n] written: 20 B) and the gradient's read-modify-write (8 B)
    peak, peak_kind = measured_peaks()
    per_pt = 16 + 4 + 20 + 8
    achieved = nz * nx * nt * per_pt / statistics.mean(grad_s) / 1e9
    fwd_achieved = nz * nx * nt * 16 / statistics.mean(fwd_s) / 1e9
    _emit({"metric": "acoustic RTM gradient Gpts/s", "value": pts * K / sum(times) / 1e9,
           "unit": "Gpts/s", "n_gpus": 1, "higher_is_better": True, "dtype": "f32",
           "data": "synthetic", "steps": K, "warmup": W,
           "config": {"workload": f"acoustic velocity gradient {nz}x{nx}, nt {nt}, {len(rix)} "
                                  f"receivers, checkpointed; {K} shots into one gradient"},
           "s_per_shot": sum(times) / K, "s_forward": statistics.mean(fwd_s),
           "s_gradient": statistics.mean(grad_s), "recomputed_steps_per_shot": recomputed,
           "counted_points_per_shot": pts,
           "gradient": {"finite": bool(torch.isfinite(g).all().item()),
                        "max_abs": float(g.abs().max().item())},
           "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                        "frac": achieved / peak, "traffic": None,
                        "peak_source": f"{peak_kind} hbm_gbs",
                        "kernel": "gradient phase: acoustic_adjoint_kernel and the segment "
                                  "recomputation's step kernels (host-timed phase)",
                        "algorithmic_bytes_per_step_point": per_pt,
                        "forward_phase_achieved_gbs": fwd_achieved,
                        "forward_phase_frac": fwd_achieved / peak}})


def run_served(args, dist):
    """Served workload: continuous batching server vs the plain per-shot loop (FIFO)."""
    from das_gb300.batch import BatchEngine
    from das_gb300.rtm_engine import TSWRTMEngine
    from das_gb300.serving import RTMServer, percentile
    from das_gb300.velocity_flood import FloodModels
    from das_gb300.wave_solver import WaveSolver2D
    trace = _served_trace(args.serve_jobs, args.serve_rate, 0, args.serve_side_scale,
                          args.serve_nt_scale)
    n_el = sum(r.kind == "elastic" for r in trace)
    tile = tuple(int(t) for t in (args.tile or "4,4").split(","))
    # the elastic workers hold up to ~17 GB each (checkpoints and one recomputed segment
    # of a 1024 x 4096, nt 8000 grid): leave them room beside the acoustic arena
    eng = BatchEngine(arena_bytes=int(min(args.arena_gb, 160.0) * (1 << 30)), max_shots=4096,
                      tile=tile, steps_per_launch=args.spl, launches_per_graph=args.lpg,
                      form=args.batch_form)
    from das_gb300.elastic import ElasticExecutor, ElasticSolver2D
    eng.run([s for r in trace if r.kind == "acoustic" for s in r.shots][:1])  # graph capture
    ex = ElasticExecutor()
    out, st = RTMServer(eng, elastic_executor=ex).serve(trace, realtime=True)
    st["elastic_worker_busy_s"] = ex.busy_s
    st["acoustic_device_busy_s"] = st["device_busy_frac"] * st["makespan_s"]
    ex.busy_s = 0.0
    eng.close()
    # plain per-shot loop over the same trace (or its first --plain-jobs jobs), FIFO,
    # arrivals on the wall clock
    m = len(trace) if args.plain_jobs <= 0 else min(args.plain_jobs, len(trace))
    t0 = time.perf_counter()
    lat, shots_done = [], 0
    kind_s = {"acoustic": 0.0, "elastic": 0.0}
    for r in trace[:m]:
        wait = r.arrival - (time.perf_counter() - t0)
        if wait > 0:
            time.sleep(wait)
        tj = time.perf_counter()
        j0 = r.shots[0]
        if r.kind == "elastic":
            es = ElasticSolver2D(j0.nx, j0.nz, j0.dx, j0.dz, j0.dt, j0.n_sponge, j0.sponge_alpha,
                                 j0.free_surface_top)
            for j in r.shots:
                ex.migrate_shot(es, j)
                shots_done += 1
            es.close()
        else:
            s = WaveSolver2D(j0.nx, j0.nz, j0.dx, j0.dz, j0.dt, j0.n_sponge, j0.sponge_alpha, True)
            e = TSWRTMEngine(s, "all")
            fm = FloodModels(j0.vel_fwd, j0.vel_fwd, j0.vel_bwd, 0, 0)
            for j in r.shots:
                e.migrate_shot(fm, j.wavelet, j.source_ix, j.source_iz, j.data, j.receiver_ix, 2,
                               2)
                shots_done += 1
            s.close()
        kind_s[r.kind] += time.perf_counter() - tj
        lat.append(time.perf_counter() - t0 - r.arrival)
    ex.close()
    plain_span = time.perf_counter() - t0
    plain = {"jobs": m, "shots": shots_done, "shots_per_s": shots_done / plain_span,
             "p50_latency_s": percentile(lat, 50), "p99_latency_s": percentile(lat, 99),
             "busy_s_by_kind": kind_s}
    served_first = [x.latency for x in out[:m]]
    plain["makespan_s"] = plain_span
    plain["achieved_gpts_per_s"] = sum(j.counted_points for r in trace[:m]
                                       for j in r.shots) / plain_span / 1e9
    out_line = {"metric": "served RTM shots/s", "value": st["shots_per_s"], "unit": "shots/s",
                "n_gpus": 1, "higher_is_better": True, "dtype": "f32", "data": "synthetic",
                "config": {"workload": f"Poisson trace of {len(trace)} jobs at {args.serve_rate} "
                                       f"jobs/s, sides log-uniform 128x256..1024x4096 x "
                                       f"{args.serve_side_scale}, nt U[1000,8000] x "
                                       f"{args.serve_nt_scale}, 1-32 shots/job",
                           "elastic_jobs_in_trace": n_el, "tile": list(tile),
                           "form": args.batch_form,
                           "steps_per_launch": args.spl, "launches_per_graph": args.lpg},
                "served": st, "plain_loop": plain,
                "served_first_jobs": {"p50_latency_s": percentile(served_first, 50),
                                      "p99_latency_s": percentile(served_first, 99)},
                "speedup_vs_plain_loop_shots": st["shots_per_s"] / plain["shots_per_s"]}
    if args.cpu_nt > 0:
        # the reference has a CPU path for the acoustic jobs only (no elastic time loop
        # or gradient): rate of one acoustic shot, extrapolated to the acoustic shots
        ac = [r for r in trace if r.kind == "acoustic"]
        rate, el, threads, kind = cpu_job_rate(ac[0].shots[0], args.cpu_nt)
        ac_pts = sum(j.counted_points for r in ac for j in r.shots)
        n_ac = sum(len(r.shots) for r in ac)
        out_line["cpu_baseline"] = {
            "value": n_ac / (ac_pts / (rate * 1e9)), "unit": "shots/s", "cores": threads,
            "kind": kind,
            "sample": f"acoustic jobs only: migrate_shot of the first acoustic shot truncated to "
                      f"nt={min(args.cpu_nt, len(ac[0].shots[0].wavelet))}: {rate:.2f} Gpts/s in "
                      f"{el:.1f} s, extrapolated to the trace's {n_ac} acoustic shots "
                      f"({ac_pts / 1e12:.2f} T counted points)"}
    _emit(out_line)


def run_interferometry(args, dist):
    """Virtual-source cross-correlation stack: 600 channels at 50 Hz, 60 s windows
    (nt = 3000), 16 virtual sources, receivers every 4th channel from 200 (95),
    maximum lag 3.5 s (351 rows); --xc-windows windows of seeded synthetic noise with
    coherent arrivals.  value: windows/s with the windows resident on the device;
    e2e: the same through CrossCorrelationStack.add from pinned host arrays.  CPU
    baseline: the reference's FFT correlation (restated in the oracle) on a sample."""
    import torch
    from das_gb300.interferometry import CrossCorrelationStack
    from das_gb300.pinned import pinned_array
    from oracle import interferometry_oracle as io
    n_ch, dt, nt, n_win = 600, 0.02, 3000, args.xc_windows
    src = np.linspace(20, 150, 16).astype(int)
    rec = np.arange(200, 580, 4)
    rng = np.random.default_rng(3)
    base = rng.standard_normal((nt + 64 * n_win, n_ch)).astype(np.float32)
    wins = [np.ascontiguousarray(base[64 * k:64 * k + nt]) for k in range(n_win)]
    st = CrossCorrelationStack(nt, n_ch, src, rec, 3.5, dt)
    rows = st.n_rows
    macs = len(src) * len(rec) * rows * nt  # per window
    dev = [torch.tensor(w, device="cuda") for w in wins]
    for w in dev[:3]:
        st.add_device(w)  # warm-up
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for w in dev:
        st.add_device(w)
    st.result()
    dev_s = time.perf_counter() - t0
    pins = [pinned_array(w.shape) for w in wins]
    for p_, w in zip(pins, wins):
        p_[...] = w
    st2 = CrossCorrelationStack(nt, n_ch, src, rec, 3.5, dt)
    t0 = time.perf_counter()
    for p_ in pins:
        st2.add(p_)
    st2.result()
    e2e_s = time.perf_counter() - t0
    # CPU: the reference's FFT correlation, all sources, a sample of windows
    k = max(1, min(4, n_win))
    t0 = time.perf_counter()
    for w in wins[:k]:
        for s_ in src:
            io.cross_correlation(w, int(s_), 3.5, dt, rec)
    cpu_s = (time.perf_counter() - t0) / k
    # ten float32 operations per product (exact split, two-sum, error accumulation);
    # issue peak: 152 SMs x 128 float32 lanes x 2.07 GHz, one operation per lane and clock
    ops = 10.0 * macs * n_win / dev_s
    peak = 152 * 128 * 2.07e9
    out = {"metric": "virtual-source CCF windows/s", "value": n_win / dev_s, "unit": "windows/s",
           "n_gpus": 1, "higher_is_better": True, "dtype": "f32 (double-float accumulation)",
           "data": "synthetic (seeded noise windows)",
           "config": {"workload": f"{n_win} windows of 3000 samples x 600 channels, 16 virtual "
                                  f"sources, {len(rec)} receivers, {rows} lag rows"},
           "ms_per_window": dev_s * 1e3 / n_win,
           "roofline": {"bound": "fp32 issue", "achieved": ops / 1e12, "peak": peak / 1e12,
                        "unit": "Tops/s", "frac": ops / peak,
                        "peak_source": "152 SMs x 128 lanes x 2.07 GHz (no measured fp32 peak)"},
           "e2e": {"value": n_win / e2e_s, "unit": "windows/s",
                   "h2d_bytes_per_step": nt * n_ch * 4,
                   "d2h_bytes_per_step": 0},
           "cpu_baseline": {"value": 1.0 / cpu_s, "unit": "windows/s", "cores": 1,
                            "kind": "port", "sample": f"{k} windows, numpy FFT (float32)"}}
    st.close()
    st2.close()
    _emit(out)


def run_small(args, dist):
    """Small plain RTM (150 x 400, dx 10 m, nt 2000, 20 shots x 400 receivers, interval 2):
    the whole TSWRTMEngine.migrate_multiple_shots call (20 shots, stack, post-stack) on
    the GPU in its default form (grids this small run their shots as one batch: every
    launch advances all shots, images stacked in shot order) and as the plain per-shot
    loop (batch="off"), and the reference's CPU path (oracle port of wave2d.c + its
    Python loops) over the same 20 shots on all host cores.  Observed gathers: forward
    modelling in the true model on the GPU."""
    from das_gb300.rtm_engine import TSWRTMEngine
    from das_gb300.synthetic import plain_small
    from das_gb300.velocity_flood import FloodModels
    from das_gb300.wave_solver import WaveSolver2D
    sv = plain_small(seed=0)
    n = len(sv.src_ix)
    solver = WaveSolver2D(sv.nx, sv.nz, sv.dx, sv.dz, sv.dt, n_sponge=sv.n_sponge,
                          sponge_alpha=sv.sponge_alpha)
    gathers = [solver.forward_propagate_acoustic(sv.vel_true, sv.wavelet, int(s), sv.src_iz,
                                                 sv.rec_ix, sv.rec_iz)[0] for s in sv.src_ix]
    fm = FloodModels(sv.vel_true, sv.vel_mig, sv.vel_mig, 0, 0)
    waves = [sv.wavelet] * n
    siz = [sv.src_iz] * n
    timing = {}
    results = {}
    for mode in ("off", "auto"):
        eng = TSWRTMEngine(solver, batch=mode)

        def survey():
            return eng.migrate_multiple_shots(fm, waves, list(sv.src_ix), siz, gathers,
                                              sv.rec_ix, sv.rec_iz, 2)

        for _ in range(args.warmup):
            survey()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            results[mode] = survey()
        timing[mode] = (time.perf_counter() - t0) / args.steps
        eng.close()
    same = all(np.array_equal(getattr(results["auto"], f), getattr(results["off"], f))
               for f in ("raw_image", "laplacian_image", "normalized_image"))
    pts = n * sv.counted_points_per_shot()
    cpu = None
    if args.small_cpu_shots > 0:
        threads = len(os.sched_getaffinity(0))
        os.environ["OMP_NUM_THREADS"] = str(threads)
        from oracle import oracle as o
        kind = "reference" if o.reference_available() else "port"
        o.set_backend("reference" if kind == "reference" else "native")
        o.set_num_threads(threads)
        g = o.Grid(sv.nx, sv.nz, sv.dx, sv.dz, sv.dt, sv.n_sponge, sv.sponge_alpha, True)
        k = min(n, args.small_cpu_shots)
        t0 = time.perf_counter()
        o.migrate_multiple_shots(g, sv.vel_mig, sv.vel_mig, waves[:k], list(sv.src_ix[:k]),
                                 siz[:k], gathers[:k], sv.rec_ix, sv.rec_iz, 2, native=True)
        cpu_s = time.perf_counter() - t0
        cpu = {"value": k * sv.counted_points_per_shot() / cpu_s / 1e9, "unit": UNIT,
               "cores": threads, "kind": kind,
               "sample": f"migrate_multiple_shots over {k} of the {n} shots, {cpu_s:.1f} s"}
    out = {"metric": METRIC, "value": pts / timing["auto"] / 1e9, "unit": UNIT, "n_gpus": 1,
           "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
           "dtype": "f32", "data": "synthetic",
           "config": {"workload": sv.name, "nz": sv.nz, "nx": sv.nx, "nt": sv.nt, "shots": n,
                      "interval": 2, "timed": "migrate_multiple_shots with host arrays"},
           "s_per_survey": timing["auto"], "s_per_survey_per_shot_loop": timing["off"],
           "gpts_per_s_per_shot_loop": pts / timing["off"] / 1e9,
           "shots_per_s": n / timing["auto"], "shots_per_s_per_shot_loop": n / timing["off"],
           "batched_equals_per_shot_loop": same, "cpu_baseline": cpu}
    solver.close()
    _emit(out)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--workload", default="large",
                    choices=["large", "small", "batched", "served", "elastic", "gradient",
                             "interferometry"])
    ap.add_argument("--xc-windows", type=int, default=32)
    ap.add_argument("--el-nt", type=int, default=6000)
    ap.add_argument("--el-shots", type=int, default=64)  # 0: --steps shots
    ap.add_argument("--el-adjoint", default="tiled", choices=["tiled", "cells"])
    ap.add_argument("--el-tiles", default="4,2:4,1")  # step warps,rows : adjoint warps,rows
    ap.add_argument("--small-cpu-shots", type=int, default=20)
    ap.add_argument("--l2-hints", type=int, default=0)
    ap.add_argument("--launch", default="grid", choices=["grid", "persistent"])
    ap.add_argument("--pdl", type=int, default=1)
    ap.add_argument("--graphs", type=int, default=1)
    ap.add_argument("--two-step", type=int, default=0)  # rows per warp of the two-step kernel
    ap.add_argument("--serve-jobs", type=int, default=40)
    ap.add_argument("--serve-rate", type=float, default=20.0)
    ap.add_argument("--serve-side-scale", type=float, default=1.0)
    ap.add_argument("--serve-nt-scale", type=float, default=1.0)
    ap.add_argument("--plain-jobs", type=int, default=0)  # 0: the whole trace
    ap.add_argument("--batch-shots", type=int, default=256)
    ap.add_argument("--batch-nt-scale", type=float, default=1.0)
    ap.add_argument("--plain-shots", type=int, default=16)
    ap.add_argument("--arena-gb", type=float, default=200.0)
    ap.add_argument("--spl", type=int, default=16)
    ap.add_argument("--lpg", type=int, default=16)
    ap.add_argument("--autotune", type=int, default=1)
    ap.add_argument("--batch-form", default="grid", choices=["grid", "queue"])
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--nt", type=int, default=8000)
    ap.add_argument("--storage", default="auto", choices=["auto", "all", "checkpoint"])
    ap.add_argument("--tile", default="")
    ap.add_argument("--cpu-nt", type=int, default=1500)
    ap.add_argument("--e2e-steps", type=int, default=10)
    ap.add_argument("--accuracy", type=int, default=1)
    ap.add_argument("--distinct-gathers", type=int, default=2)
    args = ap.parse_args()
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        sys.exit(launch_ranks(args.gpus))
    os.environ.setdefault("OMP_NUM_THREADS", str(len(os.sched_getaffinity(0))))
    if args.warmup < 3 and args.impl == "ours":
        args.warmup = 3
    if args.impl == "reference":
        dist = Dist("gloo")
        try:
            run_reference(args, dist)
        finally:
            dist.close()
        return
    rank, world, local = dist_env()
    if world > 1:
        import torch
        from das_gb300 import _lib
        torch.cuda.set_device(local)
        _lib.check(_lib.load().w2d_set_device(local))  # handles made on this thread bind here
    dist = Dist("nccl" if world > 1 else "gloo")
    global _WORKLOAD_CLOCKS
    if args.workload != "large":
        _WORKLOAD_CLOCKS = Clocks(_gpu_bus_id(local), rank)
        _WORKLOAD_CLOCKS.start()
    try:
        if args.workload == "batched":
            run_batched(args, dist)
        elif args.workload == "served":
            run_served(args, dist)
        elif args.workload == "elastic":
            run_elastic(args, dist)
        elif args.workload == "gradient":
            run_gradient(args, dist)
        elif args.workload == "interferometry":
            run_interferometry(args, dist)
        elif args.workload == "small":
            run_small(args, dist)
        else:
            run_ours(args, dist)
    finally:
        c = _WORKLOAD_CLOCKS
        if c is not None and c.proc is not None and c.proc.poll() is None:
            c.stop()  # a workload that failed before its line: end the sampler
        dist.close()


if __name__ == "__main__":
    main()
