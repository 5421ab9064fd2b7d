"""Benchmark: Nesterov iterations per second on the 1M-cell / 1024x1024-bin
synthetic placement (the reference's headline workload), one JSON line.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

A step is one Nesterov iteration (all its back-tracking evaluations) of the
placement of a seeded synthetic netlist: 1,000,000 movable cells, 1,050,000
nets, 2,000 IO pins, target density 0.75, 1024x1024 bins.  `value` is
iterations/s with the job resident in HBM, timed with CUDA events on the
job's stream; `e2e` is the same metric for a whole job through the C ABI from
host arrays (netlist upload, init, iterations, location read-back).  The
reference arm times the CPU restatement of the reference's path (the oracle)
on this host.  Multi-GPU runs are independent replicas (no collectives).

At one GPU the line also carries `serving`: the batch of config 4 (64 jobs
of 2k-50k cells submitted at once to the placement server, against the same
jobs placed one at a time), its batched form (the jobs' Nesterov loops in
one persistent launch per phase, and the server in batched mode) and the
serving form (the first --stream-jobs requests of the 500-job Poisson stream
at 2 jobs/s, 5k-500k cells, against a one-job-at-a-time server; and the
first --saturating-jobs requests at 20 jobs/s, where arrivals outpace the
GPU): placements/h and p50/p99 job latency.
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = "1m_cells_1024bins"
METRIC = "Nesterov iters/s @1M cells; placements/h + p99 latency @HPWL within 0.5%"


def dist_env():
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("LOCAL_RANK", "0")),
            int(os.environ.get("WORLD_SIZE", "1")))


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons, sampled every 50 ms from the
    start of the warm-up to the end of the end-to-end job (the timed region
    alone is often shorter than one sample period); `mark()` brackets the
    timed region so the samples inside it are counted separately."""

    def __init__(self, gpu_index: int):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.window = None
        q = ("timestamp,clocks.sm,clocks.max.sm,power.draw,utilization.gpu,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--id={gpu_index}", f"--query-gpu={q}",
                                       "--format=csv,noheader,nounits", "-lms", "50"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except FileNotFoundError:
            self.p = None

    def mark(self, t0: float, t1: float):
        self.window = (t0, t1)

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"],
                    "samples": 0}
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
        self.f.seek(0)
        rows = [l.strip().split(",") for l in self.f.read().splitlines() if l.strip()]
        os.unlink(self.f.name)
        sm, smax, busy, inside, reasons = [], [], [], 0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            r = [x.strip() for x in r]
            if len(r) < 9:
                continue
            try:
                f_sm, f_max, util = float(r[1]), float(r[2]), float(r[4])
                ts = time.mktime(time.strptime(r[0].split(".")[0], "%Y/%m/%d %H:%M:%S"))
            except ValueError:
                continue
            sm.append(f_sm); smax.append(f_max)
            if util >= 50:
                busy.append(f_sm)
            if self.window and self.window[0] - 1 <= ts <= self.window[1] + 1:
                inside += 1
            for n, v in zip(names, r[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(busy) if busy else (statistics.median(sm) if sm else None),
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm), "samples_under_load": len(busy),
                "samples_near_timed_region": inside,
                "window": "from the warm-up to the end of the end-to-end job, every 50 ms; "
                          "sm_mhz = median of the samples with GPU utilisation >= 50 %"}


# Algorithmic bytes per launch group (each array touched once), for the
# roofline of the dominant kernel.  Units: Ng gcells, Np pins, Nn nets, B bins.
def algorithmic_bytes(kind, ng, npins, nn, nb):
    return {
        "density_scatter": 53 * ng + 32 * nb,
        "poisson_rows_dct": 48 * nb,
        "poisson_cols_solve": 12 * nb,
        "poisson_rows_inverse": 16 * nb,
        # int4 pin record + pin gradient per pin, net CSR, gcell centres once
        "wa_wirelength": 24 * npins + 4 * nn + 8 * ng,
        "gcell_gradient": 57 * ng + 12 * npins + 8 * nb,
    }.get(kind)


# DRAM bytes per launch (read + write) from one ncu capture of each kernel on
# the 1M-cell workload (dram__bytes_read.sum + dram__bytes_write.sum),
# refreshed when a kernel changes: the `traffic` of the roofline object when
# the dominant kernel is one of these.  A static figure: bench.py does not
# run under ncu.
NCU_TRAFFIC = {
    "1m_cells_1024bins": {
        "wa_wirelength": 100.9e6, "gcell_gradient": 109.1e6, "density_scatter": 39.5e6,
        "poisson_rows_dct": 29.4e6, "poisson_cols_solve": 4.3e6, "poisson_rows_inverse": 8.5e6,
    },
}


def max_over_ranks(ms: float, world: int, device: str) -> float:
    """The slowest rank's timed region (replicas: one job per GPU)."""
    if world == 1:
        return ms
    import torch
    import torch.distributed as dist
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_value(world: int, iters_per_rank: int, ms: float) -> float:
    """Whole-job iterations/s: every rank ran iters_per_rank iterations of its
    own replica within ms milliseconds (the slowest rank's time)."""
    return world * iters_per_rank / (ms / 1000.0)


def host_cpu() -> dict:
    """This host's CPU: model (lscpu) and the threads available to the process."""
    model = None
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for l in out.splitlines():
            if l.startswith("Model name:"):
                model = l.split(":", 1)[1].strip()
                break
    except (OSError, subprocess.SubprocessError):
        pass
    import platform
    return {"nproc": os.cpu_count(), "cpu": model, "arch": platform.machine()}


# The CPU sample of both CPU legs (cpu_baseline and the reference arm): the
# same job, the same warm-up and the same timed iterations, so the two agree.
CPU_WARMUP = 3
CPU_STEPS = 5


def cpu_baseline_sample(nl, td, bins, warmup=CPU_WARMUP, steps=CPU_STEPS):
    """Oracle (single-threaded CPU restatement) on this host: setup and init
    from the centred placement, `warmup` Nesterov iterations, then `steps`
    timed iterations.  Returns (iterations/s, evaluations per iteration,
    seconds of CPU work in all)."""
    from oracle import oracle as O
    t0 = time.perf_counter()
    o = O.Oracle(nl, target_density=td, bin_grid_cnt_x=bins, bin_grid_cnt_y=bins,
                 initial_place_max_iter=0)
    o.initial_place()
    o.nesterov_init()
    _, s0, _ = o.nesterov_run(warmup)
    t1 = time.perf_counter()
    _, s1, _ = o.nesterov_run(steps)
    t2 = time.perf_counter()
    evals = (s1.evaluations - s0.evaluations) / max(steps, 1)
    return steps / (t2 - t1), evals, t2 - t0


def cpu_sample_text(steps, warmup, evals, seconds, workload=WORKLOAD):
    return (f"{steps} Nesterov iterations ({evals:.2f} evaluations each) of the same {workload} job "
            f"after setup, init and {warmup} warm-up iterations, from the centred placement "
            f"({seconds:.1f} s of single-threaded CPU work; the oracle restatement of the "
            "reference's path, which has no threads: its initial place alone would take minutes "
            "on one core, and the work of a Nesterov iteration does not depend on where the "
            "cells are)")


def serving_batch(n_jobs, slots, device):
    """The batched form: n_jobs netlists (2k-50k cells, log-uniform) submitted
    at once to a server with `slots` slots, against the same jobs placed one
    at a time through the plain job API.  Netlists are generated before the
    timed regions; every job runs initial place + Nesterov to its stop rule."""
    import numpy as np
    from replace_gb300 import Placer, PlacementServer, netlist as N
    jobs = N.job_batch(n_jobs, seed=4)
    t0 = time.perf_counter()
    seq = []
    for nl, td in jobs:
        p = Placer(nl, target_density=td, device=device)
        p.initial_place()
        p.nesterov_init()
        rc, st, _ = p.nesterov_run(0)
        seq.append((rc, st.iterations, st.hpwl))
        p.close()
    t_seq = time.perf_counter() - t0
    with PlacementServer(device=device, max_active=slots) as srv:
        t0 = time.perf_counter()
        ts = [srv.submit(nl, target_density=td) for nl, td in jobs]
        res = {r["ticket"]: r for r in srv.wait_all(1800)}
        t_srv = time.perf_counter() - t0
    lat = np.array([res[t]["latency_s"] for t in ts])
    same = all(res[t]["hpwl"] == q[2] and res[t]["iterations"] == q[1] for t, q in zip(ts, seq))
    return {
        "jobs": n_jobs, "slots": slots, "cells": "2k-50k log-uniform", "td": "0.60-0.85",
        "placements_per_hour": n_jobs / t_srv * 3600.0, "makespan_s": t_srv,
        "one_at_a_time_placements_per_hour": n_jobs / t_seq * 3600.0, "one_at_a_time_s": t_seq,
        "speedup_vs_one_at_a_time": t_seq / t_srv,
        "p50_latency_s": float(np.percentile(lat, 50)), "p99_latency_s": float(np.percentile(lat, 99)),
        "converged": int(sum(res[t]["status"] == 0 and res[t]["finished"] and res[t]["overflow"] <= 0.1
                             for t in ts)),
        "same_result_alone_and_in_mix": bool(same),
    }


def batched_form(n_jobs, slots, device):
    """The batched form of config 4's jobs: (1) each job's whole flow
    (initial place, Nesterov init, loop) one job at a time through the plain
    job API, against the batched flow: all initial places together
    (gpl_batch_initial_place: lockstep rounds, one launch per phase over a
    work table of (job, block, axis)), each job's init, then all loops
    together (gpl_batch_nesterov_run: one persistent launch per phase over a
    work table of (job, block), rounds replayed as one CUDA graph); (2) whole
    jobs through the placement server in batched mode (jobs join the running
    batch after their initial place).  Results must be bit-identical between
    the forms.  Netlist conversion (gpl_create) is outside the timings."""
    import numpy as np
    from replace_gb300 import Placer, PlacementServer, batch_initial_place, batch_nesterov_run, netlist as N
    jobs = N.job_batch(n_jobs, seed=4)

    def make():
        return [Placer(nl, target_density=td, device=device, poisson_path=1) for nl, td in jobs]
    ps = make()
    t_ip = t_init = t_loop = 0.0
    ip_alone, alone = [], []
    for p in ps:
        t0 = time.perf_counter()
        ip_alone.append(p.initial_place())
        t1 = time.perf_counter()
        p.nesterov_init()
        t2 = time.perf_counter()
        alone.append(p.nesterov_run(0, allow_divergence=True)[1])
        t3 = time.perf_counter()
        t_ip += t1 - t0
        t_init += t2 - t1
        t_loop += t3 - t2
    loc_alone = [p.inst_locations() for p in ps]
    for p in ps:
        p.close()
    ps = make()
    t0 = time.perf_counter()
    ip_batch, _, ip_launches = batch_initial_place(ps)
    t1 = time.perf_counter()
    for p in ps:
        p.nesterov_init()
    t2 = time.perf_counter()
    stats, status, launches = batch_nesterov_run(ps)
    t3 = time.perf_counter()
    b_ip, b_init, t_batch = t1 - t0, t2 - t1, t3 - t2
    loc_batch = [p.inst_locations() for p in ps]
    for p in ps:
        p.close()
    same_ip = all(a.iterations == b.iterations and a.last_error == b.last_error
                  and a.solver_iters_x == b.solver_iters_x and a.solver_iters_y == b.solver_iters_y
                  for a, b in zip(ip_alone, ip_batch))
    same = same_ip and all(a.hpwl == b.hpwl and a.iterations == b.iterations and np.array_equal(la[0], lb[0])
                           and np.array_equal(la[1], lb[1])
                           for a, b, la, lb in zip(alone, stats, loc_alone, loc_batch))
    iters = sum(s.iterations for s in stats)
    t_whole_alone = t_ip + t_init + t_loop
    t_whole_batch = b_ip + b_init + t_batch
    with PlacementServer(device=device, max_active=slots, batched=True) as srv:
        t0 = time.perf_counter()
        ts = [srv.submit(nl, target_density=td, poisson_path=1) for nl, td in jobs]
        res = {r["ticket"]: r for r in srv.wait_all(1800)}
        t_srv = time.perf_counter() - t0
    lat = np.array([res[t]["latency_s"] for t in ts])
    same_srv = all(res[t]["hpwl"] == a.hpwl for t, a in zip(ts, alone))
    return {
        "whole_flow": {"jobs": n_jobs, "one_at_a_time_s": t_whole_alone, "batched_s": t_whole_batch,
                       "speedup": t_whole_alone / t_whole_batch,
                       "placements_per_hour": n_jobs / t_whole_batch * 3600.0,
                       "same_result": bool(same)},
        "initial_place_phase": {"rounds": int(sum(s.iterations for s in ip_batch)),
                                "one_at_a_time_s": t_ip, "batched_s": b_ip, "speedup": t_ip / b_ip,
                                "kernel_launches": ip_launches, "same_result": bool(same_ip)},
        "init_phase": {"one_at_a_time_s": t_init, "batched_flow_s": b_init},
        "nesterov_phase": {"jobs": n_jobs, "iterations": iters, "one_at_a_time_s": t_loop,
                           "batched_s": t_batch, "speedup": t_loop / t_batch,
                           "batched_iters_per_s": iters / t_batch, "kernel_launches": launches,
                           "same_result": bool(same)},
        "server_batched": {"slots": slots, "placements_per_hour": n_jobs / t_srv * 3600.0,
                           "makespan_s": t_srv, "p50_latency_s": float(np.percentile(lat, 50)),
                           "p99_latency_s": float(np.percentile(lat, 99)),
                           "same_result_as_one_at_a_time": bool(same_srv)},
    }


def batched_ip_only(n_jobs, device=0):
    """The batched initial place of the batched form's job set, alone: one
    JSON line with its wall time, rounds and kernel launches (the case the
    batched kernels are profiled on)."""
    from replace_gb300 import Placer, batch_initial_place, netlist as N
    ps = [Placer(nl, target_density=td, device=device, poisson_path=1) for nl, td in N.job_batch(n_jobs, seed=4)]
    t0 = time.perf_counter()
    st, status, launches = batch_initial_place(ps)
    t = time.perf_counter() - t0
    for p in ps:
        p.close()
    print(json.dumps({"batched_initial_place": {"jobs": n_jobs, "seconds": t, "rounds": int(sum(s.iterations for s in st)),
                                                "kernel_launches": launches, "ok": all(s == 0 for s in status)}}))


def serving_stream(n_jobs, slots, device, rate_scale=1.0, arms=("server", "one_at_a_time")):
    """The serving form: the first n_jobs requests of the 500-job Poisson
    stream (2 jobs/s; 5k-500k cells; 10 % mixed-size), submitted at their
    arrival times (divided by rate_scale: 10 means ten times as many jobs
    per second) to a server with `slots` slots ("server"), the same server
    in batched mode ("server_batched") and a one-slot server, one job at a
    time, FIFO ("one_at_a_time").  Latency = end of the job - its arrival
    (host netlist conversion and submission included)."""
    import numpy as np
    from replace_gb300 import PlacementServer, netlist as N
    spec = N.job_stream_spec(500, 2.0, seed=5)[:n_jobs]
    nets = [N.stream_job(s) for s in spec]
    base = spec[0]["arrival_s"]

    def run(k, batched):
        with PlacementServer(device=device, max_active=k, batched=batched) as srv:
            t_create = time.perf_counter()
            arrive = {}
            for s, nl in zip(spec, nets):
                due = t_create + (s["arrival_s"] - base) / rate_scale
                while time.perf_counter() < due:
                    time.sleep(min(0.005, max(due - time.perf_counter(), 0)))
                ta = time.perf_counter()
                t = srv.submit(nl, target_density=s["td"], poisson_path=1)
                arrive[t] = ta - t_create
            res = srv.wait_all(3600)
        lat = np.array([r["finish_s"] - arrive[r["ticket"]] for r in res])
        span = max(r["finish_s"] for r in res)
        ok = sum(r["status"] == 0 and r["finished"] and r["overflow"] <= 0.1 for r in res)
        return {"slots": k, "placements_per_hour": len(res) / span * 3600.0, "span_s": span,
                "p50_latency_s": float(np.percentile(lat, 50)),
                "p99_latency_s": float(np.percentile(lat, 99)), "converged": int(ok),
                "hpwl": {int(r["ticket"]): int(r["hpwl"]) for r in res}}

    out = {"jobs": n_jobs, "of_stream": 500, "rate_per_s": 2.0 * rate_scale,
           "arrival_span_s": (spec[-1]["arrival_s"] - base) / rate_scale,
           "cells": "5k-500k log-uniform", "td": "0.60-0.90", "mixed_size_share": 0.10,
           "poisson_form": "FFT (pinned, so that every arm computes the same placements)"}
    runs = {}
    for arm in arms:
        runs[arm] = run(1, False) if arm == "one_at_a_time" else run(slots, arm == "server_batched")
    hp = [r.pop("hpwl") for r in runs.values()]
    out.update(runs)
    out["same_results_in_every_arm"] = all(sorted(h.values()) == sorted(hp[0].values()) for h in hp)
    if "server" in runs and "one_at_a_time" in runs:
        out["server_vs_one_at_a_time_placements_per_hour"] = (runs["server"]["placements_per_hour"] /
                                                              runs["one_at_a_time"]["placements_per_hour"])
    return out


def precision_form(nl, td, bins, device, stream, steps, warmup, fft_job):
    """The precision form of the same workload: the Poisson solve as tcgen05
    GEMMs (bf16 three-term split, fp32 accumulation), from the same start as
    the timed job.  Reports its iterations/s (CUDA events on the job stream),
    its potential / field / density-gradient difference against the FFT form
    at the same placement state (`fft_job`, one gpl_eval on each), and the
    whole job to its stop rule (final overflow and HPWL)."""
    import numpy as np
    import torch
    from replace_gb300 import Placer, _abi
    q = Placer(nl, _abi.default_params(target_density=td, bin_grid_cnt_x=bins, bin_grid_cnt_y=bins,
                                       device=device, stream=stream.cuda_stream, poisson_path=2))
    q.initial_place()
    q.nesterov_init()
    if q.info.poisson_path != 2:
        q.close()
        return {"available": False, "reason": "grid not a multiple of 128 bins per axis"}
    q.nesterov_run(warmup)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    rc, st, _ = q.nesterov_run(steps)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    its = st.iterations - warmup
    # both forms evaluated at the GEMM job's current state
    xy = q.gcell_coords()
    coef = float(st.wire_length_coef)
    _, dg_g, _ = q.eval(xy, coef)
    bg = q.bins(bins, bins)
    _, dg_f, _ = fft_job.eval(xy, coef)
    bf = fft_job.bins(bins, bins)

    def rel(a, b):
        a = np.asarray(a, np.float64); b = np.asarray(b, np.float64)
        return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))
    out = {"available": True, "iters_per_s": its * 1000.0 / ms, "steps": its,
           "poisson_gemm_us": round(q.info.poisson_gemm_us, 1),
           "phi_rel_l2_vs_fft": rel(bg["phi"], bf["phi"]),
           "field_rel_l2_vs_fft": rel(np.stack([bg["ex"], bg["ey"]]), np.stack([bf["ex"], bf["ey"]])),
           "density_grad_rel_l2_vs_fft": rel(dg_g, dg_f),
           "note": "fft form within 2.2e-7 (potential) of an fp64 oracle on 1024x1024 grids"}
    rc, st, _ = q.nesterov_run(0)
    out.update({"finished": bool(st.finished), "iterations_to_stop": int(st.iterations),
                "final_overflow": float(st.overflow), "final_hpwl": int(st.hpwl)})
    q.close()
    return out


def reference_parity(nl, td, bins, device, workload):
    """Final HPWL of the whole Nesterov loop against the reference's own
    NesterovPlace run on the same netlist (tests/golden/scale_place_*.npz,
    recorded from the reference build).  Both start without initial place
    (every movable instance at the core centre): the reference's initial
    place needs Eigen, which its build here does not have.  The GPU job runs
    the FFT Poisson form."""
    import numpy as np
    from replace_gb300 import Placer
    path = os.path.join(ROOT, "tests", "golden", f"scale_place_{workload}.npz")
    if not os.path.exists(path):
        return {"available": False, "reason": "no recorded reference run for this workload"}
    ref = np.load(path)
    p = Placer(nl, target_density=td, bin_grid_cnt_x=bins, bin_grid_cnt_y=bins,
               initial_place_max_iter=0, poisson_path=1, device=device)
    p.initial_place()
    p.nesterov_init()
    rc, st, _ = p.nesterov_run(0)
    p.close()
    fh = int(ref["final_hpwl"])
    return {"available": True, "start": "centred placement, no initial place",
            "status": int(rc), "iterations": int(st.iterations), "final_overflow": float(st.overflow),
            "final_hpwl": int(st.hpwl),
            "reference_status": int(ref["rc"]), "reference_iterations": int(ref["iters"][-1]),
            "reference_final_overflow": float(ref["final_overflow"]), "reference_final_hpwl": fh,
            "hpwl_rel_diff": (int(st.hpwl) - fh) / fh if fh > 0 else None,
            "within_0_5_percent": bool(fh > 0 and abs(int(st.hpwl) - fh) <= 0.005 * fh
                                       and st.overflow <= 0.1)}


def run_reference(args):
    rank, _, world = dist_env()
    if rank != 0:
        return
    from replace_gb300 import netlist as N
    nl, td, bins = N.generate_workload(args.workload, seed=1)
    from oracle import oracle as O
    O.build()
    # Each CPU iteration of the 1M-cell job takes about a second: the arm
    # times the same bounded sample as the cpu_baseline leg of the GPU arm.
    warm = CPU_WARMUP
    steps = CPU_STEPS
    v, evals, secs = cpu_baseline_sample(nl, td, bins, warm, steps)
    dt = steps / v
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "iters/s", "n_gpus": args.gpus,
        "steps": steps, "warmup": warm, "ms_per_step": 1000 * dt / steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded generator, %d movable cells)" % int((nl.inst_kind == 0).sum()),
        "config": {"workload": args.workload, "cells": int((nl.inst_kind == 0).sum()), "nets": nl.n_nets,
                   "bins": f"{bins}x{bins}", "target_density": td, "parallelism": "single-threaded CPU"},
        "cpu_baseline": {"value": v, "unit": "iters/s", "cores": 1, "kind": "port",
                         "host": host_cpu(),
                         "sample": cpu_sample_text(steps, warm, evals, secs, args.workload) +
                                   "; the reference's own build needs the reference sources, "
                                   "OpenDB and Eigen, none of which is on this host"},
        "e2e": {"value": v, "unit": "iters/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=300)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--e2e-iters", type=int, default=0,
                    help="Nesterov iteration cap of the end-to-end job (0 = run to the stop rule)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-serving", action="store_true")
    ap.add_argument("--no-parity", action="store_true",
                    help="skip the whole-loop comparison with the reference's recorded run")
    ap.add_argument("--batch-jobs", type=int, default=64)
    ap.add_argument("--stream-jobs", type=int, default=40,
                    help="requests of the 500-job stream replayed at 2 jobs/s (500: the whole stream)")
    ap.add_argument("--saturating-jobs", type=int, default=120,
                    help="requests of the stream replayed at 20 jobs/s, where the GPU is the limit")
    ap.add_argument("--slots", type=int, default=16)
    ap.add_argument("--workload", default=WORKLOAD,
                    help="named synthetic workload (replace_gb300.netlist.WORKLOADS)")
    ap.add_argument("--poisson-path", type=int, default=0, choices=[0, 1, 2],
                    help="Poisson form of the timed job: 0 auto (timed per grid), 1 FFT, 2 tensor-core GEMM")
    ap.add_argument("--ip-solver", type=int, default=0, choices=[0, 1, 2, 3],
                    help="BiCGSTAB form of the initial place: 0 auto, 1 phase kernels, 2 cooperative grid, 3 cluster")
    ap.add_argument("--no-precision", action="store_true",
                    help="skip the tensor-core Poisson (precision) form beside the timed job")
    ap.add_argument("--scatter-tile", type=int, default=0, choices=[0, 16, 32, 64],
                    help="scatter tile side in bins (0: chosen by timing at init; pin it for profiling runs)")
    ap.add_argument("--scatter-chunk", type=int, default=0, choices=[0, 1024, 2048],
                    help="gcells per scatter block (0: chosen with the tile)")
    ap.add_argument("--only-batched-ip", action="store_true",
                    help="time only the batched initial place of the --batch-jobs job set (profiling case)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        return run_reference(args)
    if args.only_batched_ip:
        return batched_ip_only(args.batch_jobs)

    import torch
    rank, local_rank, world = dist_env()
    torch.cuda.set_device(local_rank)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from replace_gb300 import Placer, netlist as N
    from replace_gb300 import _abi

    nl, td, bins = N.generate_workload(args.workload, seed=1 + rank)
    stream = torch.cuda.Stream()
    # the reference flow: initial place (20 B2B rounds), then the Nesterov
    # loop; the timed iterations start after the warm-up ones
    params = _abi.default_params(target_density=td, bin_grid_cnt_x=bins, bin_grid_cnt_y=bins,
                                 device=local_rank, stream=stream.cuda_stream,
                                 poisson_path=args.poisson_path, ip_solver=args.ip_solver,
                                 scatter_tile=args.scatter_tile, scatter_chunk=args.scatter_chunk)
    p = Placer(nl, params)
    ip_stats = p.initial_place()
    p.nesterov_init()
    info = p.info
    clocks = ClockSampler(local_rank)
    p.nesterov_run(args.warmup)

    # timed region: K iterations, resident data, CUDA events on the job stream
    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()
    barrier()
    torch.cuda.synchronize()
    launches0 = p.kernel_launches()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    t_wall0 = time.time()
    e0.record(stream)
    rc, st, _ = p.nesterov_run(args.steps)
    e1.record(stream)
    torch.cuda.synchronize()
    clocks.mark(t_wall0, time.time())
    barrier()
    ms = e0.elapsed_time(e1)
    launches = p.kernel_launches() - launches0
    iters_done = st.iterations - args.warmup
    ms = max_over_ranks(ms, world, "cuda")
    value = replica_value(world, iters_done, ms)

    # per-kernel CUDA-event timing over further iterations (same stream)
    p.kernel_times_reset(True)
    p.nesterov_run(min(args.steps, 10))
    kt = p.kernel_times()
    p.kernel_times_reset(False)
    hbm, peak_kind = peaks()
    dom = max((k for k in kt if algorithmic_bytes(k, 1, 1, 1, 1) is not None), key=lambda k: kt[k][0])
    dom_ms, dom_launches = kt[dom]
    bytes_per = algorithmic_bytes(dom, info.n_gcells, nl.n_pins, nl.n_nets,
                                  info.bin_cnt_x * info.bin_cnt_y)
    # (a job that reached its stop rule inside the timed region runs no
    # further iterations here: no kernel times, no roofline)
    achieved = bytes_per * dom_launches / (dom_ms / 1000.0) / 1e9 if dom_ms > 0 else None
    total_ms = sum(v[0] for v in kt.values())
    kernel_share = {k: round(v[0] / total_ms, 4) for k, v in kt.items() if v[1] and total_ms > 0}
    kernel_ms = {k: round(v[0] / v[1], 4) for k, v in kt.items() if v[1]}
    precision = None
    if not args.no_precision and world == 1:
        precision = precision_form(nl, td, bins, local_rank, stream, min(args.steps, 100),
                                   args.warmup, p)
    p.close()

    # end to end through the C ABI from host arrays
    e2e_line = None
    if not args.no_e2e:
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        q = Placer(nl, _abi.default_params(target_density=td, bin_grid_cnt_x=bins,
                                          bin_grid_cnt_y=bins, device=local_rank))
        q.initial_place()
        q.nesterov_init()
        # a workload on which the reference itself diverges (the 200k-cell /
        # 40-macro one: REPL-4) ends with that code here too; it is reported
        rc2, st2, _ = q.nesterov_run(args.e2e_iters, allow_divergence=True)
        lx, ly = q.inst_locations()
        t1 = time.perf_counter()
        q.close()
        e2e_iters = st2.iterations
        e2e_line = {"value": e2e_iters / (t1 - t0), "unit": "iters/s",
                    "h2d_bytes_per_step": _abi.DescHolder(nl).nbytes,
                    "d2h_bytes_per_step": lx.nbytes + ly.nbytes,
                    "note": f"one step = a whole placement job through the C ABI from host arrays: "
                            "netlist upload, host setup, initial place, Nesterov loop to its stop "
                            f"rule ({e2e_iters} iterations), location read-back",
                    "job_seconds": t1 - t0, "status": int(rc2), "finished": bool(st2.finished),
                    "final_overflow": float(st2.overflow), "final_hpwl": int(st2.hpwl)}
    clk = clocks.stop()
    parity = None
    if rank == 0 and not args.no_parity:
        parity = reference_parity(nl, td, bins, local_rank, args.workload)

    serving = None
    if world == 1 and not args.no_serving:
        serving = {"batch": serving_batch(args.batch_jobs, args.slots, local_rank),
                   "batched_form": batched_form(args.batch_jobs, args.slots, local_rank),
                   "stream": serving_stream(args.stream_jobs, args.slots, local_rank),
                   "stream_saturating": serving_stream(args.saturating_jobs, args.slots, local_rank,
                                                       rate_scale=10.0,
                                                       arms=("server", "server_batched", "one_at_a_time"))}

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        v_cpu, ev_cpu, t_cpu = cpu_baseline_sample(nl, td, bins)
        cpu = {"value": v_cpu, "unit": "iters/s", "cores": 1, "kind": "port", "host": host_cpu(),
               "sample": cpu_sample_text(CPU_STEPS, CPU_WARMUP, ev_cpu, t_cpu, args.workload)}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "iters/s", "n_gpus": world,
            "steps": iters_done, "warmup": args.warmup, "ms_per_step": ms / max(iters_done, 1),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded generator, %d movable cells)" % int((nl.inst_kind == 0).sum()),
            "config": {"workload": args.workload, "cells": int((nl.inst_kind == 0).sum()),
                       "nets": nl.n_nets, "io_pins": int((nl.pin_inst < 0).sum()),
                       "bins": f"{info.bin_cnt_x}x{info.bin_cnt_y}", "gcells": info.n_gcells,
                       "pins": nl.n_pins, "target_density": td,
                       "evals_per_iter": round((st.evaluations) / max(st.iterations, 1), 3),
                       "poisson_form": {1: "shared-memory FFT", 2: "tensor-core GEMM"}.get(info.poisson_path),
                       "scatter_shape": f"{info.scatter_tile} bins / {info.scatter_chunk} gcells",
                       # the autotuner's timings (None: not timed; auto mode
                       # skips the GEMM form above 512 bins per axis)
                       "poisson_fft_us": round(info.poisson_fft_us, 1) or None,
                       "poisson_gemm_us": round(info.poisson_gemm_us, 1) or None,
                       "start": f"after initial place ({ip_stats.iterations} B2B rounds) and "
                                f"{args.warmup} warm-up Nesterov iterations",
                       "l2": "inputs larger than L2 (job working set %.0f MB)" % (info.device_bytes / 1e6),
                       "parallelism": "replicas" if world > 1 else "single GPU"},
            "e2e": e2e_line,
            "gpu_launches": int(launches),
            "roofline": None if achieved is None else {
                         "bound": "hbm", "kernel": dom, "achieved": achieved, "peak": hbm,
                         "unit": "GB/s", "frac": achieved / hbm, "peak_kind": f"of {peak_kind}",
                         "traffic": NCU_TRAFFIC.get(args.workload, {}).get(dom),
                         "traffic_kind": "static: dram__bytes_read.sum + dram__bytes_write.sum per "
                                         "launch from one ncu capture of this kernel on this "
                                         "workload, not measured in this run",
                         "algorithmic_bytes": bytes_per, "kernel_share": kernel_share,
                         "kernel_ms_per_launch": kernel_ms},
            "cpu_baseline": cpu,
            "clocks": clk,
            "final_hpwl_vs_reference": parity,
            "serving": serving,
            "precision_form": precision,
        }
        print(json.dumps(line))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
