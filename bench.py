#!/usr/bin/env python
"""Benchmark: Newton steps/s of the batched mixed-precision GB300 solver.

Workload (one bench step): 256 independent beam models (element counts
log-uniform in [10, 4000], +/-20 % properties around the 5 m cantilever pipe,
random clamp and load triads, 0.1-10 kN step loads, HHT-alpha alpha = -0.1,
dt = 1 ms) each advanced through 500 time steps.  Synthetic, seeded inputs.
A "Newton step" is one Newton iteration of one model (forces, residual,
tangent assembly and factorisation when updated, solve, update, norms).

value: Newton iterations of all models / device time of the batched run,
       state already resident in HBM (restored device-to-device between steps).
e2e:   the same through the C ABI from host buffers: upload (fgpu_batch_create),
       run, download of every triad position, per step.
Also reported: the plain per-model FP64 GPU path on a sample of models, the
max relative displacement error of the mixed path against the FP64 path, the
CPU oracle on a bounded sample (cpu_baseline), sampled phase roofline, clocks.

--impl reference: the CPU oracle (restatement of the reference algorithm; the
reference itself does not build here) on a bounded sample with all host cores.
"""
import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time
from concurrent.futures import ThreadPoolExecutor

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "fedem-solvers_gb300"))
sys.path.insert(0, ROOT)

METRIC = "Newton steps/s batched+served vs plain GPU at 1e-8 rel err; p50/p99 latency"
UNIT = "Newton steps/s"
# algorithmic bytes of the element pass after the increment, per beam element, on
# this workload (compressed 26-value K and M, no damping, no gravity), triad data
# counted once per triad (a chain has one triad per element):
#   in:  model 4, triads 8, frame 96, reference points 12, offsets 72, relative
#        frame 96, undeformed triad frames 192, stiffness scale 8, flags 2,
#        K 208, M 208, triad position 96 + accelerations 48 + first DOF 4
#   out: frame 96, deformation 96, FS, FI, FD, Q 4 x 96
ELEM_BYTES = 1630
# DRAM bytes (read + write) of one launch on this workload (256 models), from
# ncu captures of kForwardCascade<float> and of kFactorForwardCascade<float>
# in an iteration where every model factors (profiles/)
FORWARD_TRAFFIC_256 = 153.6e6
FACTOR_TRAFFIC_256 = 307.4e6


def forward_bytes(models, elem_bytes):
    """Algorithmic bytes of one forward elimination over all fronts: the L
    blocks (nrow x npiv), the front row lists, the right-hand side (FP64) of
    the pivot rows, the solution (pivots) and update vector (non-pivot rows)
    written, and each update vector read back with its relative index by the
    parent front."""
    import numpy as np

    total = 0
    for m in models:
        _, info = m.symbolic()
        npiv, nrow, parent = info[:, 0].astype(np.int64), info[:, 1].astype(np.int64), info[:, 2]
        nu = nrow - npiv
        total += int((elem_bytes * nrow * npiv + 4 * nrow + 8 * npiv + elem_bytes * npiv + elem_bytes * nu).sum())
        total += int(((4 + elem_bytes) * nu[parent >= 0]).sum())
    return total


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--models", type=int, default=256)
    ap.add_argument("--sim-steps", type=int, default=500)
    ap.add_argument("--sweeps", type=int, default=2)
    ap.add_argument("--plain-sample", type=int, default=24, help="models timed on the plain FP64 per-model path")
    ap.add_argument("--cpu-sample-steps", type=int, default=40)
    ap.add_argument("--no-extras", action="store_true", help="skip plain/error/cpu/served legs (profiling runs)")
    ap.add_argument("--timed-only", action="store_true", help="one timed run, no warm-up, e2e or extras (ncu)")
    ap.add_argument("--fp64", action="store_true", help="time the batched plain FP64 path instead of mixed")
    ap.add_argument("--error-only", action="store_true", help="of the extras, run only the mixed-vs-FP64 check")
    ap.add_argument("--serve-rate", type=float, default=200.0)
    ap.add_argument("--serve-seconds", type=float, default=1.0)
    ap.add_argument("--serve-pool", type=int, default=48)
    ap.add_argument("--serve-steps-scale", type=float, default=0.1)
    return ap.parse_args()


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world <= 1:
        return None, 0, 1
    import torch
    import torch.distributed as dist

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    os.environ.setdefault("CUDA_VISIBLE_DEVICES", str(local))
    dist.init_process_group("nccl")
    return dist, rank, world


def shard(cases, rank, world):
    """Models are independent: balance by element count, no data-path collective."""
    order = sorted(range(len(cases)), key=lambda k: -cases[k][2])
    loads = [0] * world
    mine = []
    for k in order:
        r = min(range(world), key=lambda q: loads[q])
        loads[r] += cases[k][2]
        if r == rank:
            mine.append(k)
    return sorted(mine)


class ClockSampler:
    """Samples nvidia-smi clocks and throttle reasons while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL,
                                         text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        vis = os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0]
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9 or (vis.isdigit() and p[0] != vis):
                continue
            try:
                sm.append(float(p[1]))
                smax.append(float(p[2]))
            except ValueError:
                continue
            for n, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm.sort()
        return {"sm_mhz": sm[len(sm) // 2], "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def cpu_oracle_rate(cases, sample_steps, threads):
    """Oracle Newton iterations/s over the first `sample_steps` steps of every model."""
    from oracle.oracle import OracleModel

    def one(case):
        fsi, opts, _ = case
        o = OracleModel(fsi, opts)
        for _ in range(sample_steps):
            if not o.solve_next():
                break
        it = o.iterations()
        o.close()
        return it

    t0 = time.perf_counter()
    with ThreadPoolExecutor(max_workers=threads) as ex:
        iters = sum(ex.map(one, cases))
    dt = time.perf_counter() - t0
    return iters / dt, iters, dt


def served_leg(args):
    """Poisson request stream served with continuous batching; p50/p99 latency."""
    import numpy as np

    from fedem_gb300 import models
    from fedem_gb300.batch import Model, Server

    pool = models.served_pool_c5(args.serve_pool, seed=5, steps_scale=args.serve_steps_scale)
    mods = [Model(f, o) for f, o, _, _ in pool]
    rng = np.random.default_rng(55)
    n_req = max(1, int(round(args.serve_rate * args.serve_seconds)))
    arrivals = np.cumsum(rng.exponential(1.0 / args.serve_rate, n_req))
    pick = rng.integers(0, len(mods), n_req)
    srv = Server(budget_bytes=120e9, mixed=True, sweeps=args.sweeps, min_batch=8, max_wait=0.02)
    t0 = srv.now()
    ids, k, overlap = [], 0, 0
    while True:
        now = srv.now() - t0
        while k < n_req and arrivals[k] <= now:
            ids.append(srv.submit(mods[pick[k]]))
            k += 1
        srv.pump()
        st = srv.status()
        overlap = max(overlap, st["live_batches"])
        if k == n_req and st["pending"] == 0 and st["live_batches"] == 0:
            break
    recs = [srv.request(i) for i in ids]
    # latency from the scheduled arrival (a request submitted late, behind a
    # blocking admission, still counts from when it arrived)
    lat = np.array([r["finished"] - (t0 + a) for r, a in zip(recs, arrivals)])
    its = sum(r["iterations"] for r in recs)
    span = max(r["finished"] for r in recs) - t0
    failed = sum(1 for r in recs if r["state"] != 2)
    srv.close()
    return {"p50_latency_s": float(np.percentile(lat, 50)), "p99_latency_s": float(np.percentile(lat, 99)),
            "throughput": its / span, "unit": UNIT, "requests": n_req, "failed": failed,
            "arrival_rate_per_s": args.serve_rate, "arrival_window_s": args.serve_seconds,
            "max_concurrent_batches": overlap,
            "pool": f"{len(mods)} models, 1k-200k DOF log-uniform, 100-2000 steps log-uniform x "
                    f"{args.serve_steps_scale}"}


def run_reference(args, dist, rank, world):
    """The CPU oracle on a bounded sample of the same workload, all host threads."""
    from fedem_gb300 import models

    if rank != 0:
        return
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle")], check=True)
    cases = models.batch_c4(args.models, seed=4, steps=args.sim_steps)
    threads = os.cpu_count() or 1
    steps = max(1, args.cpu_sample_steps // 4)
    for _ in range(args.warmup):
        cpu_oracle_rate(cases[:8], 2, threads)
    rates, tot_it, tot_t = [], 0, 0.0
    for _ in range(args.steps):
        r, it, dt = cpu_oracle_rate(cases, steps, threads)
        rates.append(r)
        tot_it += it
        tot_t += dt
    value = tot_it / tot_t
    sample = f"all {args.models} models, first {steps} time steps each, per bench step"
    line = {"metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * tot_t / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded generator of the 256-model beam batch)",
            "config": {"workload": f"{args.models} beam models x {args.sim_steps} HHT steps (bounded sample)",
                       "sample": sample},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    dist, rank, world = dist_setup()
    if args.impl == "reference":
        run_reference(args, dist, rank, world)
        if dist:
            dist.destroy_process_group()
        return
    import numpy as np

    import fedem_gb300
    from fedem_gb300 import models
    from fedem_gb300.batch import Batch, Model

    fedem_gb300.load_library()
    cases_all = models.batch_c4(args.models, seed=4, steps=args.sim_steps)
    mine = shard(cases_all, rank, world)
    cases = [cases_all[k] for k in mine]
    t_setup = time.perf_counter()
    mods = [Model(f, o) for f, o, _ in cases]
    setup_s = time.perf_counter() - t_setup
    n_el = sum(m.nel for m in mods)

    # ---- device-resident timed runs (mixed precision, batched) ----------------------
    mixed = not args.fp64
    b = Batch(mods, mixed=mixed, sweeps=args.sweeps)
    b.snapshot()
    if args.timed_only:
        args.warmup, args.steps, args.no_extras = 0, 1, True
    for _ in range(args.warmup):
        b.restore()
        b.run(max_batched=200000)
    b.phase_timings(reset=True)
    clocks = ClockSampler()
    if dist:
        dist.barrier()
    clocks.start()
    iters, dev_s, wall_s, kernels, batched, tsteps = 0, 0.0, 0.0, 0, 0, 0
    failed = 0
    for _ in range(args.steps):
        b.restore()
        st = b.run(max_batched=200000)
        iters += st["newton_iterations"]
        tsteps += st["time_steps"]
        dev_s += st["device_us"] * 1e-6
        wall_s += st["wall_us"] * 1e-6
        kernels = st["kernels_per_iteration"]
        batched += st["batched_iterations"]
        failed += st["models_failed"]
    clocks_info = clocks.stop()
    if dist:
        import torch

        t = torch.tensor([dev_s, float(iters), float(tsteps)], dtype=torch.float64, device="cuda")
        tmax = t.clone()
        dist.all_reduce(tmax, op=dist.ReduceOp.MAX)
        dist.all_reduce(t, op=dist.ReduceOp.SUM)
        dev_s_max, iters_tot, tsteps_tot = float(tmax[0]), float(t[1]), float(t[2])
    else:
        dev_s_max, iters_tot, tsteps_tot = dev_s, float(iters), float(tsteps)
    value = iters_tot / dev_s_max
    nsamp, ms3, el_s = b.phase_timings()
    final_mixed = b.all_triads().copy()
    # the dominant kernel timed alone (every model factoring), after the timed runs
    fac_ms, fac_bytes = b.time_factor(reps=10) if mixed and not args.timed_only else (0.0, 0.0)
    b.close()

    # ---- e2e through the C ABI from host buffers ------------------------------------
    e2e_iters, e2e_s, h2d, d2h = 0, 0.0, 0, 0
    out = np.zeros(12 * sum(m.ntri for m in mods))
    for k in range(0 if args.timed_only else args.steps):
        t0 = time.perf_counter()
        be = Batch(mods, mixed=mixed, sweeps=args.sweeps)
        st = be.run()
        be.all_triads(out)
        e2e_s += time.perf_counter() - t0
        e2e_iters += st["newton_iterations"]
        h2d = st["h2d_bytes"]
        d2h = out.nbytes
        be.close()
    e2e_value = e2e_iters / e2e_s if e2e_s > 0 else None

    extras = {}
    if (not args.no_extras or args.error_only) and rank == 0 and mixed:
        # ---- accuracy of the mixed path against the plain FP64 path ------------------
        bf = Batch(mods, mixed=False)
        bf.run()
        final_fp64 = bf.all_triads().copy()
        bf.close()
        off, worst = 0, 0.0
        for m, (fsi, opts, n) in zip(mods, cases):
            nt = m.ntri
            a = final_mixed[off:off + 12 * nt].reshape(nt, 4, 3)[:, 3, :]
            c = final_fp64[off:off + 12 * nt].reshape(nt, 4, 3)[:, 3, :]
            x0 = np.stack([np.arange(nt) * 0.25, np.zeros(nt), np.zeros(nt)], 1)
            denom = max(np.abs(c - x0).max(), 1e-300)
            worst = max(worst, float(np.abs(a - c).max() / denom))
            off += 12 * nt
        extras["max_rel_disp_err_mixed_vs_fp64"] = worst
    if not args.no_extras and rank == 0:
        # ---- plain per-model FP64 GPU path on a sample --------------------------------
        idx = np.linspace(0, len(mods) - 1, min(args.plain_sample, len(mods))).astype(int)
        p_it, p_s, p_ts = 0, 0.0, 0
        for k in idx:
            bp = Batch([mods[k]], mixed=False)
            st = bp.run()
            p_it += st["newton_iterations"]
            p_ts += st["time_steps"]
            p_s += st["device_us"] * 1e-6
            bp.close()
        plain_rate = p_it / p_s
        extras["plain_fp64_per_model"] = {"value": plain_rate, "unit": UNIT, "time_steps_per_s": p_ts / p_s,
                                          "sample": f"{len(idx)} of {len(mods)} models run one at a time"}
        extras["speedup_vs_plain"] = value / plain_rate
        extras["speedup_vs_plain_time_steps"] = (tsteps_tot / dev_s_max) / (p_ts / p_s)
        # ---- CPU oracle on a bounded sample ---------------------------------------------
        subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle")], check=True)
        threads = os.cpu_count() or 1
        c_rate, c_it, c_dt = cpu_oracle_rate(cases, args.cpu_sample_steps, threads)
        extras["cpu_baseline"] = {"value": c_rate, "unit": UNIT, "cores": threads, "kind": "port",
                                  "sample": f"all {len(cases)} models, first {args.cpu_sample_steps} "
                                            f"time steps each ({c_it} Newton iterations, {c_dt:.1f} s)"}
        # ---- served: Poisson request stream with continuous batching ----------------------
        extras["served"] = served_leg(args)

    hbm_peak, peak_kind = measured_peaks()
    roof, roof_el = None, None
    if nsamp > 0 and ms3[0] > 0:
        achieved = el_s * ELEM_BYTES / (ms3[0] * 1e-3) / 1e9
        roof_el = {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                   "frac": achieved / hbm_peak, "traffic": None,
                   "kernel": "kElements (element pass after the increment)", "peak_source": peak_kind,
                   "note": "bound by the FP64 rate (FP64 pipe 84-88 % busy), not by HBM",
                   "bytes_per_element": ELEM_BYTES, "samples": nsamp}
    roof_fwd = None
    if nsamp > 0 and ms3[3] > 0:
        # one forward elimination of the refinement solve (sampled inside the run)
        fb = forward_bytes(mods, 4)
        t_fwd = ms3[3] * 1e-3 / nsamp
        achieved = fb / t_fwd / 1e9
        traffic = FORWARD_TRAFFIC_256 if len(mods) == 256 and args.models == 256 else None
        roof_fwd = {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                    "frac": achieved / hbm_peak, "traffic": traffic,
                    "kernel": "kForwardCascade<float> (forward elimination, all fronts)",
                    "algorithmic_bytes_per_launch": fb, "launch_ms": t_fwd * 1e3, "peak_source": peak_kind,
                    "samples": nsamp}
    if fac_ms > 0:
        # the dominant kernel: the factorisation fused with the first forward
        # elimination, every model factoring, timed alone on the engine stream
        achieved = fac_bytes / (fac_ms * 1e-3) / 1e9
        traffic = FACTOR_TRAFFIC_256 if len(mods) == 256 and args.models == 256 else None
        roof = {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                "frac": achieved / hbm_peak, "traffic": traffic,
                "kernel": "kFactorForwardCascade<float> (LDL^T of every front + first forward elimination)",
                "algorithmic_bytes_per_launch": fac_bytes, "launch_ms": fac_ms, "peak_source": peak_kind,
                "note": "latency-bound: the launch time is set by the dependency chains of the assembly "
                        "trees and each front's dependent memory round trips, not by bytes",
                "timing": "10 launches after the timed runs, CUDA events on the engine stream"}
    elif roof_fwd is not None:
        roof = roof_fwd
    elif roof_el is not None:
        roof = roof_el
    phases = None
    if nsamp > 0:
        phases = {"elements": ms3[0] / nsamp, "factor_and_first_forward": ms3[1] / nsamp,
                  "other_solve": ms3[2] / nsamp, "second_forward": ms3[3] / nsamp}
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": 1000.0 * dev_s_max / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64+f32" if mixed else "f64",
                "data": "synthetic (seeded generator of the 256-model beam batch)",
                "config": {"workload": f"{args.models} beam models (10-4000 elements, log-uniform) x "
                                       f"{args.sim_steps} HHT-alpha steps, batched " +
                                       (f"mixed precision (FP32 fronts + FP64 refinement, {args.sweeps} "
                                        f"solves/iteration)" if mixed else "plain FP64"),
                           "elements": n_el, "models_on_rank0": len(mods), "l2": "inputs larger than L2 "
                           "(element matrices and state of all models ~%.2f GB)" % (n_el * 5200 / 1e9),
                           "host_setup_s": setup_s},
                "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
                "time_steps_per_s": tsteps_tot / dev_s_max,
                "newton_iterations_per_time_step": iters_tot / max(tsteps_tot, 1.0),
                "gpu_launches": kernels * batched, "kernels_per_batched_iteration": kernels,
                "batched_iterations": batched, "models_failed": failed,
                "wall_s_timed": wall_s, "clocks": clocks_info, "roofline": roof,
                "roofline_elements": roof_el, "roofline_forward": roof_fwd, "phase_ms_per_iteration": phases}
        line.update(extras)
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
