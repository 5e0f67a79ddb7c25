#!/usr/bin/env python3
"""Benchmark of the FDFK2D hot path on GB300: the hybrid FD-FK time loop.

A step is one time step of the loop of simulate_wavefield (src/FDFK2D.f90:465-532):
receiver sampling + the fused updatedispl_ step over the whole grid.  The
workload is the 4001 x 2001 heterogeneous model (config 2: 400 x 200 km at
100 m, 40-cell PML, FD order 6, 401 receivers) with seeded synthetic inputs.

value: K steps with material and the FK background (computed on the GPU beforehand)
resident in HBM.  e2e: one whole K-step solve through the C ABI from host buffers -
session creation with the material copied from pinned memory, the FK background
computed on the GPU from the host's 1-D models, K steps with the launch shapes the
autotuner found for the model, seismograms copied back (after one untimed warm-up
solve of the same shape).
fk_background: the FK background of the full workload (nt = 12000) alone.

Prints one JSON line (rank 0).  Arms:
  default           the GPU path (this repository)
  --impl reference  the reference's CPU algorithm on this host's cores (the oracle
                    restatement in oracle/; the reference's own gfortran build
                    ships x86-64 binaries only)
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

BYTES_PER_CELL_STEP = 36  # read u^n, u^{n-1} (2 comps), write u^{n+1} (2 comps), read rho, lambda, mu: FP32
METRIC = "Mcell-steps/s"


def measured_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def profile_traffic():
    """Per-launch DRAM traffic of the dominant kernel from the committed ncu summary, if present."""
    path = os.path.join(ROOT, "profiles", "fdfk_march_kernel_config2.md")
    try:
        for line in open(path):
            if line.startswith("traffic_bytes_per_launch:"):
                return float(line.split(":", 1)[1].split()[0])
    except OSError:
        pass
    return None


class ClockSampler:
    """nvidia-smi clocks/throttle sampling every 50 ms, from the warm-up of the device-resident arm
    to the end of the end-to-end solve (the timed region alone can be a few milliseconds)."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_reference(w, budget_s=15.0, max_steps=40):
    """The reference algorithm (oracle restatement) on the host cores over a bounded sample."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    from fdfk2d_gb300 import workloads as W
    p = dict(w["p"], izt=1)
    cells = (p["nz"] + p["npml"]) * (p["nx"] + 2 * p["npml"])
    cores = os.cpu_count() or 1
    os.environ.setdefault("OMP_NUM_THREADS", str(cores))

    def run(steps):
        q = dict(p, nt=steps - 1)
        strips = W.plane_wave_background(dict(w, p=q), 0, steps)
        t = time.perf_counter()
        oracle.simulate(q, strips, w["c"], w["rx"], w["rz"], w["x0"], w["z0"], 1, steps - 1, steps_limit=steps)
        return time.perf_counter() - t

    t1 = run(1)
    steps = int(max(2, min(max_steps, budget_s / max(t1, 1e-3))))
    dt = run(steps)
    value = cells * steps / dt / 1e6
    return value, cores, f"{steps} time steps of the full {p['nz'] + p['npml']}x{p['nx'] + 2 * p['npml']} grid " \
                         f"({dt:.1f} s, OMP threads={cores})"


def cpu_reference_steps(w, K, W, budget_s=90.0):
    """The reference arm: W untimed and then exactly K timed time steps of the reference algorithm
    (the oracle restatement, OpenMP on every host core).  Each step covers a bounded sample of the
    workload - the top R rows of the grid with all its columns, R chosen so that the W + K steps take
    about budget_s (the whole grid when that fits) - since the whole 2041 x 4081 grid takes about
    0.2 s per step on 16 cores.  Returns (Mcell-steps/s, seconds for the K steps, R, cores)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    from fdfk2d_gb300 import workloads as W_
    p = dict(w["p"], izt=1)
    NZ, NX = p["nz"] + p["npml"], p["nx"] + 2 * p["npml"]
    cores = os.cpu_count() or 1
    os.environ.setdefault("OMP_NUM_THREADS", str(cores))

    def run(rows, steps):
        q = dict(p, nz=rows - p["npml"], nt=max(steps - 1, 1))
        wq = dict(w, p=q)
        strips = W_.plane_wave_background(wq, 0, q["nt"] + 1)
        c = np.asfortranarray(w["c"][:, :rows, :])
        t = time.perf_counter()
        oracle.simulate(q, strips, c, w["rx"], w["rz"], w["x0"], w["z0"], 1, q["nt"], steps_limit=steps)
        return time.perf_counter() - t

    probe_rows = min(NZ, 400)
    per_cell_step = run(probe_rows, 2) / (2 * probe_rows * NX)
    rows = int(budget_s / max((W + K) * NX * per_cell_step, 1e-30))
    rows = max(p["npml"] + 2 * p["norder"] + 2, min(NZ, rows))
    if W > 0:
        run(rows, W)
    dt = run(rows, K)
    return rows * NX * K / dt / 1e6, dt, rows, cores


def batched_uneven(F, WL, args, torch, dev):
    """Config 4: solves of uneven grid sizes and lengths (seeded draw from the config-4
    distribution) in one batch against the same solves run one after another (a sample of them),
    each solve from host inputs to host seismograms, FK background on the GPU included."""
    solves = WL.config4_solves(args.uneven_solves)
    cells = lambda w: (w["p"]["nz"] + w["p"]["npml"]) * (w["p"]["nx"] + 2 * w["p"]["npml"])
    work = [cells(w) * (w["p"]["nt"] + 1) for w in solves]

    def session(w):
        p = w["p"]
        s = F.Session(p, w["c"])
        fp, bazs, fl, fr = WL.config4_inputs(w)
        s.fk_background(fp, bazs, fl, fr)
        s.set_receivers(w["rx"], w["rz"], w["x0"], w["z0"], 1, p["nt"])
        return s

    # sequential: every k-th solve alone (a sample spread over the size distribution)
    k = max(1, len(solves) // max(1, args.uneven_seq_sample))
    sample = list(range(0, len(solves), k))[:args.uneven_seq_sample]
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    for i in sample:
        with session(solves[i]) as s:
            s.advance(solves[i]["p"]["nt"] + 1)
            s.seismograms()
    t_seq = time.perf_counter() - t0
    seq_rate = sum(work[i] for i in sample) / t_seq             # cell-steps per second
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    b = F.Batch(3)
    sessions = []
    for w in solves:
        s = session(w)
        b.add(s)
        sessions.append(s)
    b.advance(max(w["p"]["nt"] for w in solves) + 1)
    traces = [s.seismograms() for s in sessions]
    t_batch = time.perf_counter() - t0
    b.close()
    for s in sessions:
        s.close()
    assert all(np.isfinite(tz).all() for _, tz in traces)
    n = len(solves)
    seq_solves_h = 3600.0 * seq_rate / (sum(work) / n)           # at the mean work per solve
    return {"batched_uneven": {
        "workload": f"config4 (scaled): {n} seeded solves, nx 500-6000 and nz 250-2500 log-uniform, dx 100-500 m, "
                    f"20-120 s (nt {min(w['p']['nt'] for w in solves)}-{max(w['p']['nt'] for w in solves)}), "
                    f"2-4 layers, 0-5 % perturbation, P/S",
        "solves": n, "cell_steps": float(sum(work)), "wall_s": round(t_batch, 3),
        "solves_per_hour": round(n / t_batch * 3600, 1),
        "mcell_steps_per_s": round(sum(work) / t_batch / 1e6, 1),
        "sequential_sample": len(sample), "sequential_mcell_steps_per_s": round(seq_rate / 1e6, 1),
        "sequential_solves_per_hour": round(seq_solves_h, 1),
        "speedup_vs_sequential": round(sum(work) / t_batch / seq_rate, 2),
        "note": "each solve from host inputs to host seismograms, FK background on the GPU; sequential rate "
                "from a sample of the same solves, per cell-step"}}


def tune_batch(F, p, c, tune, n, torch, dev, steps=24):
    """Launch shapes of a batch of n solves of this model, (fast-path segment columns, 0 = the
    batch's own plan; absorbing-layer tile length): the tile lengths with the planned segments,
    then segment lengths with the best tile length, then the three fastest shapes again in two
    interleaved rounds; every candidate timed on a scratch batch (zero state and background, a
    short record) outside the timed regions."""
    runs = (16, 24, 32, 48)
    segs = (0, 64, 80, 101, 128)
    trials = len(runs) + len(segs) + 6
    q = dict(p, nt=trials * (steps + 8) + 2)
    nbd = 2 * int(p["norder"]) - 1
    zeros = {k: np.zeros(sh, np.float32, order="F") for k, sh in F.strip_shapes(q["nx"], q["nz"], nbd, q["nt"]).items()}
    sessions = []
    for _ in range(n):
        s = F.Session(q, c)
        if tune:
            s.set_tuning(*tune)
        s.upload_background(zeros)
        sessions.append(s)
    b = F.Batch(int(p["norder"]))
    for s in sessions:
        b.add(s)

    def time_it(seg, run):
        b.set_tuning(seg, run)
        b.advance(8)
        torch.cuda.synchronize(dev)
        b.synchronize()
        t0 = time.perf_counter()
        b.advance(steps)
        b.synchronize()
        return time.perf_counter() - t0

    seen = {}
    for run in runs:
        seen[(0, run)] = time_it(0, run)
    best_run = min(seen, key=seen.get)[1]
    for seg in segs:
        seen[(seg, best_run)] = min(seen.get((seg, best_run), 1e30), time_it(seg, best_run))
    final = sorted(seen, key=seen.get)[:3]
    total = {k: 0.0 for k in final}
    for _ in range(2):
        for k in final:
            total[k] += time_it(*k)
    best = min(total, key=total.get)
    b.close()
    for s in sessions:
        s.close()
    return best


def batched_and_served(F, WL, args, torch, dev):
    """Config 3 (64 events on the config-1 model, batched vs sequential plain-GPU solves, each
    solve from host inputs to host seismograms including its FK background on the GPU) and
    config 5 (an open-loop Poisson stream of config-3 requests through the serving loop at 80 %
    of the measured batched capacity, 160 GB admission budget)."""
    w1 = WL.config1()
    p1 = w1["p"]
    nt = p1["nt"]
    cells1 = (p1["nz"] + p1["npml"]) * (p1["nx"] + 2 * p1["npml"])
    events = WL.config3_events(args.batch_events)
    rx, rz = w1["rx"], w1["rz"]
    out = {}
    # launch shapes tuned once for the model, outside the timed regions, used by both arms; the
    # batch's launch shapes (segments, absorbing-layer tiles) tuned once more for the batch itself
    tune = None if args.no_autotune else F.autotune(p1, w1["c"], steps=20)[:2]
    batch_shape = None if args.no_autotune else tune_batch(F, p1, w1["c"], tune, len(events), torch, dev)

    def new_session():
        s = F.Session(p1, w1["c"])
        if tune:
            s.set_tuning(*tune)
        return s

    def solve_inputs(ev):
        fp, bazs, fl, fr = WL.event_inputs(w1, ev)
        return fp, bazs, fl, fr

    # sequential plain-GPU solves (a bounded sample, same events)
    nseq = min(args.seq_sample, len(events))
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    for ev in events[:nseq]:
        fp, bazs, fl, fr = solve_inputs(ev)
        with new_session() as s:
            s.fk_background(fp, bazs, fl, fr)
            s.set_receivers(rx, rz, w1["x0"], w1["z0"], 1, nt)
            s.advance(nt + 1)
            s.seismograms()
    t_seq = (time.perf_counter() - t0) / nseq
    # batched: every event at once
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    sessions = []
    b = F.Batch(p1["norder"])
    if batch_shape:
        b.set_tuning(*batch_shape)
    for ev in events:
        fp, bazs, fl, fr = solve_inputs(ev)
        s = new_session()
        s.fk_background(fp, bazs, fl, fr)
        s.set_receivers(rx, rz, w1["x0"], w1["z0"], 1, nt)
        b.add(s)
        sessions.append(s)
    b.advance(nt + 1)
    traces = [s.seismograms() for s in sessions]
    t_batch = time.perf_counter() - t0
    b.close()
    for s in sessions:
        s.close()
    assert all(np.isfinite(tz).all() for _, tz in traces)
    n = len(events)
    out["batched"] = {"workload": f"config3: {n} events (P 0.04-0.08, S 0.10-0.12 s/km, baz 0-360, 0.5-1 Hz) "
                                  f"on the config-1 model, nt={nt}",
                      "solves_per_hour": round(n / t_batch * 3600, 1), "wall_s": round(t_batch, 3),
                      "mcell_steps_per_s": round(n * cells1 * (nt + 1) / t_batch / 1e6, 1),
                      "sequential_solves_per_hour": round(3600 / t_seq, 1), "sequential_sample": nseq,
                      "speedup_vs_sequential": round(t_seq * n / t_batch, 2),
                      "tuning": {"seg_len": tune[0], "pml_run": tune[1],
                                 "batch_seg_len": batch_shape[0] if batch_shape else None,
                                 "batch_pml_run": batch_shape[1] if batch_shape else None} if tune else None,
                      "note": "each solve from host inputs to host seismograms, FK background on the GPU"}
    if args.serve_requests <= 0:
        return out
    # serving: open-loop Poisson arrivals at 80 % of the batched capacity
    cap = n / t_batch
    rate = 0.8 * cap
    rng = np.random.default_rng(11)
    reqs = WL.config3_events(args.serve_requests, seed=13)
    rng.shuffle(reqs)
    arrivals = np.cumsum(rng.exponential(1.0 / rate, len(reqs)))
    srv = F.Server(p1["norder"], budget_bytes=160 << 30, chunk=64)
    ids, sched, peak = [], [], 0
    t0 = time.monotonic()
    i = 0
    while True:
        now = time.monotonic() - t0
        while i < len(reqs) and arrivals[i] <= now:
            fp, bazs, fl, fr = solve_inputs(reqs[i])
            ids.append(srv.submit(p1, w1["c"], fp, bazs, fl, fr, rx, rz, w1["x0"], w1["z0"], 1, nt))
            sched.append(t0 + arrivals[i])
            i += 1
        left = srv.pump()
        peak = max(peak, srv.stats()["running"])
        if left == 0:
            if i >= len(reqs):
                break
            time.sleep(max(0.0, min(0.05, arrivals[i] - (time.monotonic() - t0))))
    t_all = time.monotonic() - t0
    lat = []
    for rid, ta in zip(ids, sched):
        st, _, _, t_done = srv.request(rid)
        assert st == F.api.REQ_DONE
        lat.append(t_done - ta)
        srv.release(rid)
    srv.close()
    lat = np.array(lat)
    out["serving"] = {"workload": f"config5 (scaled): {len(reqs)} Poisson requests drawn from config 3, "
                                  f"arrival rate {rate:.2f}/s = 80 % of the batched capacity, budget 160 GB",
                      "requests": len(reqs), "arrival_rate_per_s": round(rate, 3),
                      "solves_per_hour": round(len(reqs) / t_all * 3600, 1),
                      "p50_s": round(float(np.percentile(lat, 50)), 3),
                      "p95_s": round(float(np.percentile(lat, 95)), 3),
                      "p99_s": round(float(np.percentile(lat, 99)), 3),
                      "max_running": peak, "wall_s": round(t_all, 2),
                      "sequential_solves_per_hour": out["batched"]["sequential_solves_per_hour"]}
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    # default: the workload's whole record (nt = 12000 -> 12001 steps), so that e2e is one full solve
    # and the clock sampler sees more than a second of load
    ap.add_argument("--steps", type=int, default=12001)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="config2", choices=["config2", "config1"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fk-full", action="store_true")
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--tuning", default="", help="SEG,RUN: the workload's launch shapes (fast-path segment "
                    "columns, absorbing-layer run) given instead of autotuned")
    ap.add_argument("--batch-events", type=int, default=64, help="config-3 events (0: skip batched and serving)")
    ap.add_argument("--seq-sample", type=int, default=16, help="sequential solves timed for the comparison")
    ap.add_argument("--serve-requests", type=int, default=2000, help="config-5 requests (0: skip serving)")
    ap.add_argument("--uneven-solves", type=int, default=24, help="config-4 solves (0: skip the uneven batch)")
    ap.add_argument("--uneven-seq-sample", type=int, default=4, help="config-4 solves timed one by one")
    args = ap.parse_args()
    K, Wm = args.steps, max(3, args.warmup)

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))

    from fdfk2d_gb300 import workloads as WL
    w = WL.config2() if args.workload == "config2" else WL.config1()
    p = w["p"]
    NZ, NX = p["nz"] + p["npml"], p["nx"] + 2 * p["npml"]
    cells = NZ * NX
    config = {"workload": w["name"], "grid": f"{NZ}x{NX} cells incl. PML", "fd_order": 2 * p["norder"],
              "receivers": len(w["rx"]),
              "background": "FK background computed on the GPU (P, 0.07 s/km, 1 Hz; crust 33 / 50 km left / right)",
              "l2": "state 7 x 33 MB > 129 MB L2 (no flush needed)", "parallelism": f"replicas x{args.gpus}"}

    if args.impl == "reference":
        if rank != 0:
            return
        value, secs, rows, cores = cpu_reference_steps(w, K, Wm)
        sample = (f"each step one time step of the top {rows} of {NZ} rows x all {NX} columns of the grid "
                  f"({rows * NX} cells); {Wm} untimed + {K} timed steps, {secs:.1f} s timed, OMP threads={cores}")
        line = {"metric": METRIC, "value": round(value, 3), "unit": METRIC, "impl": "reference", "n_gpus": args.gpus,
                "steps": K, "warmup": Wm, "ms_per_step": round(secs / K * 1e3, 3),
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": config,
                "cpu_baseline": {"value": round(value, 3), "unit": METRIC, "cores": cores, "kind": "port",
                                 "sample": sample},
                "e2e": {"value": round(value, 3), "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return

    import torch
    import fdfk2d_gb300 as F
    from fdfk2d_gb300 import replicas
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", init_method="env://")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    stream = torch.cuda.Stream(device=dev)

    def barrier():
        torch.cuda.synchronize(dev)
        replicas.barrier()

    # ---- device-resident arm: material and the FK background (computed on the GPU) in HBM
    # before the timed region; time axis = warm-up + timed steps
    q = dict(p, nt=Wm + K - 1)
    fkp, bazs, fk_left, fk_right = WL.fk_inputs(dict(w, p=q))
    tuning = None
    if args.tuning:
        seg, run = (int(v) for v in args.tuning.split(","))
        tuning = {"seg_len": seg, "pml_run": run, "given": True}
    elif not args.no_autotune:
        seg, run, ms_tuned = F.autotune(p, w["c"], steps=20)
        tuning = {"seg_len": seg, "pml_run": run, "ms_per_step_in_tuner": round(ms_tuned, 4)}
    sess = F.Session(q, w["c"], stream=stream.cuda_stream)
    if tuning:
        sess.set_tuning(tuning["seg_len"], tuning["pml_run"])
    sess.fk_background(fkp, bazs, fk_left, fk_right)
    sess.set_receivers(w["rx"], w["rz"], w["x0"], w["z0"], 1, q["nt"])
    clocks = ClockSampler(local)
    clocks.start()
    sess.advance(Wm)
    sess.synchronize()
    barrier()
    n0 = F.kernel_launches()
    # K steps between two CUDA events on the launching stream, with event pairs around the kernels
    # of every 8th step of the same loop (the roofline kernel's time is part of the timed steps;
    # sampling keeps the events' own cost out of most steps)
    ms_int, ms_edge, ms = sess.advance_timed(K, 8)
    barrier()
    launches = F.kernel_launches() - n0
    ms = replicas.max_over_ranks(ms, dev)        # the slowest replica's time
    ms_step = ms / K
    value = replicas.whole_job_rate(cells * K, ms / 1e3) / 1e6

    cells_int, cells_edge = sess.cell_split()
    sess.close()

    # ---- end-to-end arm: one whole K-step solve through the C ABI from host buffers: material
    # (pinned) and FK inputs in, FK background on the GPU, K steps, seismograms out
    # (the FK damping alpha = 10 / (nt dt) needs a record of realistic length: at least 1000 samples)
    qe = dict(p, nt=max(K - 1, 999))
    fke, bazs_e, fl_e, fr_e = WL.fk_inputs(dict(w, p=qe))
    c_pin = torch.empty((NX, NZ, 3), dtype=torch.float32, pin_memory=True)
    c_host = c_pin.numpy().transpose(2, 1, 0)          # Fortran (3, NZ, NX) view
    c_host[...] = w["c"]
    outx = np.empty((K, len(w["rx"])), np.float32, order="F")
    outz = np.empty_like(outx, order="F")

    def solve_e2e():
        se = F.Session(qe, c_host, stream=stream.cuda_stream)
        if tuning:                                       # the launch shapes tuned once for this model
            se.set_tuning(tuning["seg_len"], tuning["pml_run"])
        se.fk_background(fke, bazs_e, fl_e, fr_e)
        se.set_receivers(w["rx"], w["rz"], w["x0"], w["z0"], 1, qe["nt"])
        se.advance(K)
        se.seismogram_range(0, K, outx, outz)
        return se

    solve_e2e().close()        # warm-up: module loading and the first launches of every kernel
    barrier()
    t0 = time.perf_counter()
    se = solve_e2e()
    barrier()
    t_e2e = time.perf_counter() - t0
    se.close()
    clk = clocks.stop()
    t_e2e = replicas.max_over_ranks(t_e2e, dev)
    e2e_value = replicas.whole_job_rate(cells * K, t_e2e) / 1e6
    h2d = (c_host.nbytes + bazs_e.nbytes + fl_e.nbytes + fr_e.nbytes + 2 * 4 * len(w["rx"])) / K
    d2h = (outx.nbytes + outz.nbytes) / K
    assert np.isfinite(outz).all()

    # ---- FK background alone at the workload's full length (nt of the workload), device-resident
    fk_ms = None
    if rank == 0 and not args.no_fk_full:
        sf = F.Session(p, w["c"], stream=stream.cuda_stream)
        fkf, bazs_f, fl_f, fr_f = WL.fk_inputs(w)
        sf.fk_background(fkf, bazs_f, fl_f, fr_f)          # warm-up (first launches, first touch)
        barrier()
        t0 = time.perf_counter()
        sf.fk_background(fkf, bazs_f, fl_f, fr_f)
        barrier()
        fk_ms = (time.perf_counter() - t0) * 1e3
        sf.close()
        n_fft = 1
        while n_fft < 2 * (p["nt"] + 1):
            n_fft *= 2
        series = sum(int(np.prod(s_[:2])) for s_ in F.strip_shapes(p["nx"], p["nz"], p["nbd"], p["nt"]).values())

    extra = {}
    if rank == 0 and args.batch_events > 0:
        extra.update(batched_and_served(F, WL, args, torch, dev))
    if rank == 0 and args.uneven_solves > 0:
        extra.update(batched_uneven(F, WL, args, torch, dev))

    peak, peak_kind = measured_peak()
    # dominant kernel: the interior fast path (its own cells, its own event-timed duration)
    if cells_int > 0 and ms_int > 0:
        dom, dom_cells, dom_ms = "fdfk_march_kernel", cells_int, ms_int
    else:
        dom, dom_cells, dom_ms = "fdfk_step_kernel", cells_edge, ms_edge
    achieved = BYTES_PER_CELL_STEP * dom_cells / (dom_ms / 1e3) / 1e9
    step_equiv = BYTES_PER_CELL_STEP * cells / (ms_step / 1e3) / 1e9
    traffic = profile_traffic()
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        value_cpu, cores, sample = cpu_reference(w)
        cpu = {"value": round(value_cpu, 3), "unit": METRIC, "cores": cores, "kind": "port", "sample": sample}
    if rank == 0:
        line = {"metric": METRIC, "value": round(value, 1), "unit": METRIC, "n_gpus": world, "steps": K, "warmup": Wm,
                "ms_per_step": round(ms_step, 4), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f32", "data": "synthetic", "config": config,
                "e2e": {"value": round(e2e_value, 1), "unit": METRIC, "h2d_bytes_per_step": int(h2d),
                        "d2h_bytes_per_step": int(d2h)},
                "gpu_launches": int(launches),
                "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                             "frac": round(achieved / peak, 4), "traffic": traffic, "peak_kind": peak_kind,
                             "kernel": dom, "bytes_per_cell_step": BYTES_PER_CELL_STEP,
                             "cells_per_launch": dom_cells, "ms_per_launch": round(dom_ms, 4),
                             "edge_kernel_ms_per_launch": round(ms_edge, 4),
                             "whole_step_equiv_gbs": round(step_equiv, 1),
                             "whole_step_frac": round(step_equiv / peak, 4)},
                "cpu_baseline": cpu, "clocks": clk}
        if tuning:
            line["config"]["tuning"] = dict(tuning, note="launch shapes given on the command line" if
                                            tuning.get("given") else "launch shapes picked by fdfk_autotune")
        if extra:
            line.update(extra)
        if fk_ms is not None:
            line["fk_background"] = {"ms": round(fk_ms, 1), "nt": p["nt"], "series": series, "n_fft": n_fft,
                                     "precision": "fp64 spectra and transforms, f32 strips",
                                     "note": "whole FK background of the workload, device-resident output"}
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
