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
e2e:   the same through the C ABI from host buffers, per step: model set-up
       from the text (host threads), upload (fgpu_batch_create), run, download
       of every triad position.
Also reported: the batched plain FP64 path, the plain per-model FP64 GPU path
on a sample of models, the mixed path's error against the FP64 path, the CPU
oracle over the whole workload (cpu_baseline, and every model's final state
compared with both GPU paths), phase rooflines, clocks, the served leg, and
two single-model legs run to their end times in FP64 and mixed precision with
the oracle beside them (parity of the final state and a one-thread CPU
baseline): the space-frame tower (2,000 steps) and the superelement chain
(4,000 steps).

--impl reference: the CPU oracle (restatement of the reference algorithm; the
reference itself does not build here) on the same workload and boundary: the
timed steps together are one full run of every model, set-up included, on all
host threads.
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
# DRAM bytes (read + write) of one launch on this workload (256 models): the
# mean of the first two Newton-iteration launches of each kernel captured by
# ncu on the first 128 of these models, scaled by the ratio of algorithmic
# bytes (fronts) or of elements (profiles/dram_traffic_beam_batch_128models.md);
# for the back substitution the refinement solve's launch
FACTOR_TRAFFIC_256 = 202.5e6
FORWARD_TRAFFIC_256 = 152.1e6
BACKWARD_TRAFFIC_256 = 137.4e6
# DRAM bytes per element of the element pass after the increment (same capture)
ELEM_TRAFFIC = 1238


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
    ap.add_argument("--no-extras", action="store_true", help="skip plain/error/cpu/served legs (profiling runs)")
    ap.add_argument("--timed-only", action="store_true", help="one timed run, no warm-up, e2e or extras (ncu)")
    ap.add_argument("--fp64", action="store_true", help="time the batched plain FP64 path instead of mixed")
    ap.add_argument("--error-only", action="store_true", help="of the extras, run only the mixed-vs-FP64 check")
    ap.add_argument("--no-oracle", action="store_true", help="skip the full CPU oracle run (parity + cpu_baseline)")
    ap.add_argument("--space-frame-steps", type=int, default=2000, help="time steps of the space-frame tower leg")
    ap.add_argument("--no-space-frame", action="store_true", help="skip the space-frame tower leg")
    ap.add_argument("--superelement-steps", type=int, default=4000, help="time steps of the superelement chain leg")
    ap.add_argument("--no-superelements", action="store_true", help="skip the superelement chain leg")
    ap.add_argument("--no-cantilever", action="store_true", help="skip the cantilever leg")
    ap.add_argument("--single-models-only", action="store_true",
                    help="run only the single-model legs (space frame, superelement chain) and print their JSON")
    ap.add_argument("--serve-rate", type=float, default=200.0)
    ap.add_argument("--serve-seconds", type=float, default=1.0)
    ap.add_argument("--serve-pool", type=int, default=48)
    ap.add_argument("--serve-steps-scale", type=float, default=0.1)
    ap.add_argument("--served-only", action="store_true",
                    help="run only the served leg (with the --serve-* parameters) and print its JSON")
    ap.add_argument("--serve-slot-reuse", type=float, default=0.0,
                    help="share of an engine's models finished before its slots are reused (0: never)")
    return ap.parse_args()


def rank_env():
    """(rank, world size, local rank) from the launcher's environment."""
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def dist_setup():
    """One process per GPU: the rank's device is LOCAL_RANK, selected in the
    solver library's own CUDA runtime (fgpu_set_device) before anything is
    created; the process group (for the timing max and the sums) is NCCL."""
    rank, world, local = rank_env()
    if world <= 1:
        return None, 0, 1, local
    import torch
    import torch.distributed as dist

    torch.cuda.set_device(local)
    dist.init_process_group("nccl")
    return dist, rank, world, local


def rank_device(local, lib=None):
    """Selects this rank's GPU in the solver library; returns (ordinal, PCI bus id)."""
    from fedem_gb300.batch import set_device

    return set_device(local, lib)


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


def workload_config(args, cases):
    """The `config` of both arms: the same workload and the same timing boundary."""
    n_el = sum(c[2] for c in cases)
    return {"workload": f"{args.models} beam models (10-4000 elements, log-uniform, +/-20 % properties) x "
                        f"{args.sim_steps} HHT-alpha steps (alpha -0.1, dt 1 ms, Newton tolerance 1e-8)",
            "models": args.models, "time_steps_per_model": args.sim_steps, "elements": n_el,
            "e2e_boundary": "model text and options in, final triad positions out: model set-up (parse, "
                            "element matrices, equation numbering, symbolic analysis) and the whole run inside "
                            "the timed region",
            "l2": "inputs larger than L2 (element matrices and state of all models ~%.2f GB)" % (n_el * 5200 / 1e9)}


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

    def stop(self, index=None):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        vis = os.environ.get("CUDA_VISIBLE_DEVICES", "").split(",")[0]
        if not vis.isdigit():
            vis = str(index if index is not None else 0)
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


def oracle_full_run(cases, threads):
    """The CPU oracle over the whole workload: every model from its text to its
    end time (set-up inside the timed region, as in the e2e legs), one model per
    host thread at a time, largest first.  Returns (seconds, Newton iterations,
    final triad positions per model, iterations per model)."""
    from oracle.oracle import OracleModel

    order = sorted(range(len(cases)), key=lambda k: -cases[k][2])
    urs, its, scale = [None] * len(cases), [0] * len(cases), [0.0] * len(cases)

    def one(k):
        o = OracleModel(cases[k][0], cases[k][1])
        o.run_all()
        urs[k] = o.triads().copy()
        its[k] = o.iterations()
        scale[k] = o.max_displacement()
        o.close()

    t0 = time.perf_counter()
    with ThreadPoolExecutor(max_workers=threads) as ex:
        list(ex.map(one, order))
    dt = time.perf_counter() - t0
    return dt, sum(its), urs, its, scale


def rel_disp_error(a, c, x0, scale=None):
    """max |a - c| over the triad positions / the displacement scale: the
    given one (the largest displacement over the run), else max |c - x0|."""
    import numpy as np

    denom = max(float(scale if scale is not None else np.abs(c - x0).max()), 1e-300)
    return float(np.abs(a - c).max()) / denom


def served_leg(args, share, compare_batched=True):
    """Poisson request stream served with continuous batching (slot reuse at
    `share`); p50/p99 latency from each request's arrival to its completion,
    throughput, and the same requests run as one batch for comparison.  A
    request's model set-up from its text (host threads) is inside its latency;
    requests for a model text already set up reuse it (the pool repeats
    models), as a service keeps the set-up of the models it has seen."""
    import numpy as np

    from fedem_gb300 import models
    from fedem_gb300.batch import Batch, Model, Server

    pool = models.served_pool_c5(args.serve_pool, seed=5, steps_scale=args.serve_steps_scale)
    rng = np.random.default_rng(55)
    n_req = max(1, int(round(args.serve_rate * args.serve_seconds)))
    arrivals = np.cumsum(rng.exponential(1.0 / args.serve_rate, n_req))
    pick = rng.integers(0, len(pool), n_req)
    srv = Server(budget_bytes=120e9, mixed=True, sweeps=args.sweeps, min_batch=8, max_wait=0.02)
    srv.slot_reuse(share)
    setup = ThreadPoolExecutor(max_workers=os.cpu_count() or 1)
    t0 = srv.now()
    futs, ids, k, overlap = [], {}, 0, 0
    cache = {}  # pool index -> model set-up (future)
    kept = []
    while True:
        now = srv.now() - t0
        while k < n_req and arrivals[k] <= now:
            q = int(pick[k])
            if q not in cache:
                f, o, _, _ = pool[q]
                cache[q] = setup.submit(Model, f, o)
            futs.append((k, cache[q]))
            k += 1
        # requests whose model is set up are submitted
        rest = []
        for q, fut in futs:
            if fut.done():
                m = fut.result()
                kept.append(m)
                ids[q] = srv.submit(m)
            else:
                rest.append((q, fut))
        futs = rest
        srv.pump()
        st = srv.status()
        overlap = max(overlap, st["live_batches"])
        if k == n_req and not futs and st["pending"] == 0 and st["live_batches"] == 0:
            break
    setup.shutdown()
    ids = [ids[q] for q in range(n_req)]
    recs = [srv.request(i) for i in ids]
    # latency from the scheduled arrival (set-up and any wait for admission included)
    lat = np.array([r["finished"] - (t0 + a) for r, a in zip(recs, arrivals)])
    its = sum(r["iterations"] for r in recs)
    span = max(r["finished"] for r in recs) - t0
    failed = sum(1 for r in recs if r["state"] != 2)
    rebatches = srv.slot_reuse()
    srv.close()
    out = {"p50_latency_s": float(np.percentile(lat, 50)), "p99_latency_s": float(np.percentile(lat, 99)),
           "throughput": its / span, "unit": UNIT, "requests": n_req, "failed": failed,
           "arrival_rate_per_s": args.serve_rate, "arrival_window_s": args.serve_seconds,
           "max_concurrent_batches": overlap, "slot_reuse_share": share,
           "engines_rebuilt_for_slot_reuse": rebatches, "distinct_models_set_up": len(cache),
           "latency_definition": "scheduled Poisson arrival -> completion; the request's model set-up from its "
                                 "text (host threads) and any wait for admission included",
           "pool": f"{len(pool)} models, 1k-200k DOF log-uniform, 100-2000 steps log-uniform x "
                   f"{args.serve_steps_scale}"}
    if compare_batched and not args.no_oracle:
        # the same requests on the CPU oracle, all host threads, one request per
        # thread at a time (set-up inside the timed region), as a like-for-like
        # CPU baseline of the served workload
        threads = os.cpu_count() or 1
        subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle")], check=True)
        reqs = [(pool[int(q)][0], pool[int(q)][1], pool[int(q)][2]) for q in pick]
        c_dt, c_its, _, _, _ = oracle_full_run(reqs, threads)
        out["cpu_baseline_same_requests"] = {
            "value": c_its / c_dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"the {n_req} served requests, each from its text to its end time ({c_its} Newton "
                      f"iterations, {c_dt:.1f} s), one request per thread at a time"}
    if compare_batched:
        # the same requests as one batch (all present at once): device throughput
        b = Batch(kept, mixed=True, sweeps=args.sweeps)
        st = b.run()
        out["batched_same_requests"] = {"value": st["newton_iterations"] / (st["device_us"] * 1e-6),
                                        "unit": UNIT, "note": "the served requests' models in one batch, device time"}
        b.close()
    for f in cache.values():
        f.result().close()
    return out


def factor_flops(model):
    """Factorisation flops of one model's fronts, sum over the columns j of L
    of c_j (c_j + 3), c_j the off-diagonal entries of column j (a front of nr
    rows and np pivots has c = nr - 1 - k at its pivot k)."""
    import numpy as np

    _, info = model.symbolic()
    tot = 0
    for npiv, nrow in info[:, :2].astype(np.int64):
        c = nrow - 1 - np.arange(npiv)
        tot += int((c * (c + 3)).sum())
    return tot


def single_model_oracle(fsi, opts):
    """The oracle over one model, single-threaded, set-up included.  Runs in a
    spawned process beside the GPU legs.  Returns (seconds, Newton iterations,
    final triad matrices, largest displacement over the run)."""
    from oracle.oracle import OracleModel

    t0 = time.perf_counter()
    o = OracleModel(fsi, opts)
    o.run_all()
    dt = time.perf_counter() - t0
    out = dt, o.iterations(), o.triads().copy(), o.max_displacement()
    o.close()
    return out


def single_model_workloads(args):
    """The single-model legs: (key, fsi, options, steps, description).
    cantilever: the reference's plain-method case, 20 beams, 1,000 steps.
    space-frame tower: 12 storeys x 4 x 4 bays, 1,164 pipes, 40 revolute
    joints, 40 spring/damper pairs, 10 kN at 2 Hz on the top floor, FP64.
    superelement chain: 16 Craig-Bampton parts (40 x 4 x 4 hexahedra reduced to
    2 triads + 30 modes, 42 x 42), 15 revolute joints, gravity, 500 N m at
    2 Hz, Rayleigh 1 % at 10 Hz, dt 0.5 ms; its matrix files are written to a
    temporary directory first."""
    import tempfile

    from fedem_gb300 import models

    out = []
    if not args.no_cantilever:
        fsi, opts = models.cantilever_c1()
        out.append(("cantilever", fsi, opts, 1000,
                    "cantilever pipe, 5 m, 20 Euler-Bernoulli beams (120 free DOFs), 1 kN tip step load, 1000 "
                    "HHT-alpha steps of 1 ms"))
    if not args.no_space_frame:
        fsi, opts = models.space_frame_c2(steps=args.space_frame_steps)
        out.append(("space_frame", fsi, opts, args.space_frame_steps,
                    "space-frame tower, 12 storeys x 4 x 4 bays, 1164 beams, 40 revolute joints, 40 spring/damper "
                    f"pairs, sinusoidal 10 kN top load at 2 Hz, {args.space_frame_steps} HHT-alpha steps of 1 ms"))
    if not args.no_superelements:
        d = tempfile.mkdtemp(prefix="fedem_parts_")
        fsi, opts, _ = models.superelement_chain_c3(d, steps=args.superelement_steps)
        out.append(("superelement_chain", fsi, opts, args.superelement_steps,
                    "superelement chain, 16 parts (2 x 0.2 x 0.2 m steel blocks, 40 x 4 x 4 hexahedra reduced to 2 "
                    "triads + 30 component modes, 42 x 42 K and M), 15 revolute joints, gravity + 500 N m "
                    f"harmonic torque at 2 Hz, Rayleigh 1 % at 10 Hz, {args.superelement_steps} HHT-alpha steps "
                    "of 0.5 ms"))
    return out


def start_single_oracles(args, workloads):
    """(pool, {key: pending result}) of the oracle runs of the single-model
    legs, each in its own spawned process (a fresh interpreter: safe beside
    this process's CUDA context), or (None, {}) with --no-oracle."""
    if args.no_oracle or not workloads:
        return None, {}
    import multiprocessing

    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle")], check=True)
    pool = multiprocessing.get_context("spawn").Pool(len(workloads))
    return pool, {key: pool.apply_async(single_model_oracle, (fsi, opts)) for key, fsi, opts, _, _ in workloads}


def single_model_leg(fsi, opts, steps, desc, pending=None):
    """One model per batch through its run: plain FP64 and mixed precision,
    device time of a full run after a short warm-up run, phase timings, the
    factorisation (timed alone) against the measured FP64 FMA rate, and, when
    `pending` (the oracle's run in a spawned process) is given, both final
    states against the oracle's and the oracle's time as the CPU baseline."""
    import numpy as np

    from fedem_gb300.batch import Batch, Model, measure_fp64_peak, measure_tf32_mma_peak

    m = Model(fsi, opts)
    flops = factor_flops(m)
    peak_tf, _ = measure_fp64_peak()
    peak_tf32, _ = measure_tf32_mma_peak()
    out = {"workload": desc, "equations": m.neq, "unit": UNIT,
           "factor_flops_per_factorisation": flops, "fp64_fma_peak_tflops": peak_tf,
           "fp64_peak_source": "measured (fgpu_measure_fp64_peak: 8 FMA chains per thread, 8 blocks per SM)",
           "tf32_mma_peak_tflops": peak_tf32,
           "tf32_peak_source": "measured (fgpu_measure_tf32_mma_peak: mma.sync m16n8k8, 8 fragments per warp, "
                               "8 blocks per SM)"}
    finals = {}
    for mixed in (False, True):
        b = Batch([m], mixed=mixed)
        b.snapshot()
        b.run(max_batched=64)  # warm-up: graph instantiation, first launches
        b.restore()
        b.phase_timings(reset=True)
        st = b.run()
        n, ms, _ = b.phase_timings()
        key = "mixed" if mixed else "fp64"
        finals[key] = b.triads(0).copy()
        its = b.info(0)["iterations"]
        if its != st["newton_iterations"]:
            raise RuntimeError("single-model run: iteration counts disagree")
        ph = (ms / max(n, 1)).tolist()
        leg = {"value": st["newton_iterations"] / (st["device_us"] * 1e-6),
               "time_steps_per_s": st["time_steps"] / (st["device_us"] * 1e-6),
               "newton_iterations": its, "batched_iterations": st["batched_iterations"],
               "kernels_per_batched_iteration": st["kernels_per_iteration"], "failed": st["models_failed"],
               "ms_per_iteration": st["device_us"] * 1e-3 / max(st["batched_iterations"], 1),
               "phase_ms_per_iteration": {"elements": ph[0], "factor_and_first_forward": ph[1],
                                          "other_solve": ph[2], "second_forward": ph[3],
                                          "back_substitution": ph[4]}}
        # the factorisation fused with the first forward elimination, timed alone
        # (10 launches, CUDA events on the engine stream) after the run
        f_ms, _ = b.time_factor(reps=10)
        leg["factor_ms"] = f_ms
        if not mixed:
            achieved = flops / (f_ms * 1e-3) / 1e12
            leg["roofline_factor"] = {"bound": "fp64", "achieved": achieved, "peak": peak_tf, "unit": "TFLOP/s",
                                      "frac": achieved / peak_tf, "traffic": None,
                                      "kernel": "kFactorForwardCascade<double> (+ kLargeFactorForward<double>)",
                                      "timing": "10 launches after the run, CUDA events on the engine stream"}
        else:
            leg["factor_gflops"] = flops / (f_ms * 1e-3) / 1e9
            # FP32 fronts: large fronts' trailing tiles are 3xTF32 mma.sync products
            # (three TF32 products per multiply-add), small fronts FP32 scalar
            eff = peak_tf32 / 3.0
            achieved = flops / (f_ms * 1e-3) / 1e12
            leg["roofline_factor"] = {"bound": "tensor", "achieved": achieved, "peak": eff, "unit": "TFLOP/s",
                                      "frac": achieved / eff, "traffic": None,
                                      "peak_definition": "measured mma.sync TF32 rate / 3 (3xTF32 split)",
                                      "kernel": "kFactorForwardCascade<float> (+ kLargeFactorForward<float>)",
                                      "timing": "10 launches after the run, CUDA events on the engine stream"}
        out[key] = leg
        b.close()
    if pending is not None:
        c_dt, c_it, c_ur, c_scale = pending.get()
        out["parity_vs_oracle"] = {
            "max_rel_disp_err_fp64": float(np.abs(finals["fp64"][:, :, 3] - c_ur[:, :, 3]).max() / c_scale),
            "max_rel_disp_err_mixed": float(np.abs(finals["mixed"][:, :, 3] - c_ur[:, :, 3]).max() / c_scale),
            "oracle_iterations": c_it, "fp64_iterations": out["fp64"]["newton_iterations"],
            "definition": "final triad positions: max |gpu - oracle| / the largest triad displacement over "
                          "the run (oracle)"}
        out["cpu_baseline"] = {"value": c_it / c_dt, "unit": UNIT, "cores": 1, "kind": "port",
                               "sample": f"the full run ({steps} steps, {c_it} Newton iterations, {c_dt:.1f} s), "
                                         "set-up included, one thread"}
    m.close()
    return out


def run_reference(args, dist, rank, world):
    """The reference arm: the CPU oracle (the FP64 restatement of the reference
    algorithm; the reference itself does not build here) on the same workload
    and config as the GPU arm, all host threads.  Bench step k advances every
    model through time steps [k w, (k + 1) w), w = ceil(steps / K), so the K
    timed steps together are exactly one full run of the workload; each model's
    set-up (parse, element matrices, skyline structure) is inside the first
    step, as model set-up is inside the GPU arm's e2e region."""
    import numpy as np

    from fedem_gb300 import models
    from oracle.oracle import OracleModel

    if rank != 0:
        return
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle")], check=True)
    cases = models.batch_c4(args.models, seed=4, steps=args.sim_steps)
    threads = os.cpu_count() or 1
    # untimed warm-up: a few steps of the smallest models
    small = sorted(range(len(cases)), key=lambda k: cases[k][2])[:min(8, len(cases))]
    for _ in range(args.warmup):
        def warm(k):
            o = OracleModel(cases[k][0], cases[k][1])
            for _ in range(3):
                o.solve_next()
            o.close()
        with ThreadPoolExecutor(max_workers=threads) as ex:
            list(ex.map(warm, small))
    K = max(1, args.steps)
    window = int(math.ceil(args.sim_steps / K))
    order = sorted(range(len(cases)), key=lambda k: -cases[k][2])
    objs = [None] * len(cases)
    live = [True] * len(cases)

    def advance(k):
        if not live[k]:
            return 0
        if objs[k] is None:
            objs[k] = OracleModel(cases[k][0], cases[k][1])
        o = objs[k]
        it0 = o.iterations()
        for _ in range(window):
            if not o.solve_next():
                live[k] = False
                break
        return o.iterations() - it0

    tot_it, tot_t = 0, 0.0
    with ThreadPoolExecutor(max_workers=threads) as ex:
        for _ in range(K):
            t0 = time.perf_counter()
            tot_it += sum(ex.map(advance, order))
            tot_t += time.perf_counter() - t0
    for o in objs:
        if o is not None:
            o.close()
    value = tot_it / tot_t
    sample = (f"all {args.models} models, {window} time steps of each per bench step: the {K} timed steps are "
              f"one full {args.sim_steps}-step run of the workload ({tot_it} Newton iterations, {tot_t:.1f} s), "
              f"model set-up inside the first step; {threads} host threads, one model per thread at a time")
    line = {"metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * tot_t / K,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded generator of the 256-model beam batch)",
            "config": workload_config(args, cases),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def backward_bytes(models, elem_bytes, refinement=False):
    """Algorithmic bytes of one back substitution over all fronts: the L block
    (nrow x npiv), the row list, the solution values of all rows gathered, the
    pivots' solution written in the solve precision and in FP64 (the
    refinement solve of the last sweep also reads the accumulated FP64
    solution and writes the increment: 16 more bytes per pivot)."""
    import numpy as np

    per_piv = elem_bytes + (24 if refinement else 8)
    total = 0
    for m in models:
        _, info = m.symbolic()
        npiv, nrow = info[:, 0].astype(np.int64), info[:, 1].astype(np.int64)
        total += int((elem_bytes * nrow * npiv + 4 * nrow + elem_bytes * nrow + per_piv * npiv).sum())
    return total


def main():
    args = parse()
    dist, rank, world, local = dist_setup()
    if args.impl == "reference":
        run_reference(args, dist, rank, world)
        if dist:
            dist.destroy_process_group()
        return
    import numpy as np

    import fedem_gb300
    from fedem_gb300 import models
    from fedem_gb300.batch import Batch, create_models

    want_single = rank == 0 and not args.timed_only
    lib = fedem_gb300.load_library()
    dev, bus = rank_device(local, lib)
    if args.served_only:
        out = {"served": served_leg(args, args.serve_slot_reuse)}
        print(json.dumps(out), flush=True)
        return
    if args.single_models_only:
        work = single_model_workloads(args)
        pool, pending = start_single_oracles(args, work)
        out = {key: single_model_leg(fsi, opts, steps, desc, pending.get(key))
               for key, fsi, opts, steps, desc in work}
        print(json.dumps(out), flush=True)
        if pool is not None:
            pool.close()
        return
    print(f"rank {rank}: solver device {dev} ({bus})", file=sys.stderr, flush=True)
    cases_all = models.batch_c4(args.models, seed=4, steps=args.sim_steps)
    mine = shard(cases_all, rank, world)
    cases = [cases_all[k] for k in mine]
    threads = os.cpu_count() or 1
    t_setup = time.perf_counter()
    mods = create_models(cases, threads)
    setup_s = time.perf_counter() - t_setup
    n_el = sum(m.nel for m in mods)

    # ---- device-resident timed runs (mixed precision, batched) ----------------------
    mixed = not args.fp64
    b = Batch(mods, mixed=mixed, sweeps=args.sweeps)
    if b.device() != dev:
        raise RuntimeError(f"batch on device {b.device()}, rank {rank} selected {dev}")
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
    clocks_info = clocks.stop(dev)
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
    nsamp, ms5, el_s = b.phase_timings()
    final_mixed = b.all_triads().copy()
    iters_mixed = [b.info(k)["iterations"] for k in range(len(mods))]
    # the dominant kernel timed alone (every model factoring), after the timed runs
    fac_ms, fac_bytes = b.time_factor(reps=10) if mixed and not args.timed_only else (0.0, 0.0)
    shape, probe_ms, _ = b.launch_shape()
    b.close()

    # ---- e2e through the C ABI from host buffers: set-up, upload, run, download --------
    e2e_iters, e2e_s, h2d, d2h = 0, 0.0, 0, 0
    out = np.zeros(12 * sum(m.ntri for m in mods))
    for k in range(0 if args.timed_only else args.steps):
        t0 = time.perf_counter()
        me = create_models(cases, threads)
        be = Batch(me, mixed=mixed, sweeps=args.sweeps)
        st = be.run()
        be.all_triads(out)
        e2e_s += time.perf_counter() - t0
        e2e_iters += st["newton_iterations"]
        h2d = st["h2d_bytes"]
        d2h = out.nbytes
        be.close()
        for m in me:
            m.close()
    e2e_value = e2e_iters / e2e_s if e2e_s > 0 else None

    extras = {}
    x0s = []
    for m in mods:
        nt = m.ntri
        x0s.append(np.stack([np.arange(nt) * 0.25, np.zeros(nt), np.zeros(nt)], 1))

    def split(flat):
        out_, off = [], 0
        for m in mods:
            out_.append(flat[off:off + 12 * m.ntri].reshape(m.ntri, 4, 3)[:, 3, :])
            off += 12 * m.ntri
        return out_

    if (not args.no_extras or args.error_only) and rank == 0 and mixed:
        # ---- the batched plain FP64 path: its throughput and the mixed path's error --------
        bf = Batch(mods, mixed=False)
        bf.snapshot()
        bf.run()
        final_fp64 = bf.all_triads().copy()
        iters_fp64 = [bf.info(k)["iterations"] for k in range(len(mods))]
        bf.restore()
        stf = bf.run()
        bf.close()
        extras["batched_fp64"] = {"value": stf["newton_iterations"] / (stf["device_us"] * 1e-6), "unit": UNIT,
                                  "note": "same batch, plain FP64 fronts and one solve per iteration, device time"}
        extras["speedup_mixed_vs_batched_fp64"] = value / extras["batched_fp64"]["value"]
        pm, pf = split(final_mixed), split(final_fp64)
        errs = [rel_disp_error(a, c, x0) for a, c, x0 in zip(pm, pf, x0s)]
        extras["max_rel_disp_err_mixed_vs_fp64"] = max(errs)
        if not args.no_oracle and not args.error_only:
            # ---- the CPU oracle over the whole workload: parity of every model + cpu_baseline
            subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle")], check=True)
            c_dt, c_it, c_urs, c_its, c_scale = oracle_full_run(cases, threads)
            e64 = [rel_disp_error(a, c[:, :, 3], x0, sc) for a, c, x0, sc in zip(pf, c_urs, x0s, c_scale)]
            emx = [rel_disp_error(a, c[:, :, 3], x0, sc) for a, c, x0, sc in zip(pm, c_urs, x0s, c_scale)]
            f64 = [rel_disp_error(a, c[:, :, 3], x0) for a, c, x0 in zip(pf, c_urs, x0s)]
            fmx = [rel_disp_error(a, c[:, :, 3], x0) for a, c, x0 in zip(pm, c_urs, x0s)]
            extras["parity_vs_oracle"] = {
                "models": len(mods),
                "max_rel_disp_err_fp64_vs_oracle": max(e64),
                "worst_model_fp64": int(np.argmax(e64)),
                "max_rel_disp_err_mixed_vs_oracle": max(emx),
                "worst_model_mixed": int(np.argmax(emx)),
                "models_fp64_over_1e-10": int(sum(e > 1e-10 for e in e64)),
                "models_mixed_over_1e-8": int(sum(e > 1e-8 for e in emx)),
                "models_fp64_iterations_differ": int(sum(a != c for a, c in zip(iters_fp64, c_its))),
                "models_mixed_iterations_differ": int(sum(a != c for a, c in zip(iters_mixed, c_its))),
                "definition": "final triad positions after all steps: max |gpu - oracle| / the model's largest "
                              "triad displacement over the run (oracle)",
                "final_state_normalised": {"max_fp64": max(f64), "max_mixed": max(fmx),
                                           "definition": "the same over max |oracle - x0| of the final state, "
                                                         "which is small for models that end near a zero of "
                                                         "their oscillation"},
                "per_model_rel_err_fp64": [float("%.3g" % e) for e in e64],
                "per_model_rel_err_mixed": [float("%.3g" % e) for e in emx]}
            extras["cpu_baseline"] = {"value": c_it / c_dt, "unit": UNIT, "cores": threads, "kind": "port",
                                      "sample": f"the full workload: all {len(cases)} models, all "
                                                f"{args.sim_steps} time steps, set-up included ({c_it} Newton "
                                                f"iterations, {c_dt:.1f} s), one model per thread"}
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
        # the single-model oracle runs start here, after the batch oracle leg
        # (whose timing they would otherwise share cores with), and run beside
        # the GPU legs
        work = single_model_workloads(args) if want_single else []
        pool, pending = start_single_oracles(args, work)
        # ---- served: Poisson request stream with continuous batching ----------------------
        extras["served"] = served_leg(args, args.serve_slot_reuse)
        extras["served_with_slot_reuse"] = served_leg(args, 0.25 if args.serve_slot_reuse == 0.0 else 0.0,
                                                      compare_batched=False)
        for key, fsi, opts, steps, desc in work:
            extras[key] = single_model_leg(fsi, opts, steps, desc, pending.get(key))
        if pool is not None:
            pool.close()

    hbm_peak, peak_kind = measured_peaks()
    roof, roof_el = None, None
    if nsamp > 0 and ms5[0] > 0:
        achieved = el_s * ELEM_BYTES / (ms5[0] * 1e-3) / 1e9
        # per launch: the measured DRAM bytes per element x the sampled launches' mean active elements
        roof_el = {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                   "frac": achieved / hbm_peak, "traffic": ELEM_TRAFFIC * el_s / nsamp,
                   "kernel": "kElements (element pass after the increment)", "peak_source": peak_kind,
                   "note": "bound by the FP64 rate (FP64 pipe 84-88 % busy), not by HBM; the phase is sampled with "
                               "the partial norms running beside it on a second stream",
                   "bytes_per_element": ELEM_BYTES, "traffic_bytes_per_element": ELEM_TRAFFIC,
                   "samples": nsamp}
    E = 4 if mixed else 8
    roof_fwd = None
    if nsamp > 0 and ms5[3] > 0:
        # one forward elimination of the refinement solve (sampled inside the run)
        fb = forward_bytes(mods, E)
        t_fwd = ms5[3] * 1e-3 / nsamp
        achieved = fb / t_fwd / 1e9
        traffic = FORWARD_TRAFFIC_256 if len(mods) == 256 and args.models == 256 else None
        roof_fwd = {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                    "frac": achieved / hbm_peak, "traffic": traffic,
                    "kernel": "kForwardCascade<float> (forward elimination, all fronts)",
                    "algorithmic_bytes_per_launch": fb, "launch_ms": t_fwd * 1e3, "peak_source": peak_kind,
                    "samples": nsamp}
    roof_bwd = None
    # the back substitution launched on its own: the refinement solve's (the
    # first solve's runs inside the factorisation's launch in batches without
    # large fronts); an FP64 batch of one solve per iteration has none
    if nsamp > 0 and ms5[4] > 0.05 * ms5[1]:
        bb = backward_bytes(mods, E, refinement=mixed)
        t_bwd = ms5[4] * 1e-3 / nsamp
        achieved = bb / t_bwd / 1e9
        traffic = BACKWARD_TRAFFIC_256 if len(mods) == 256 and args.models == 256 else None
        roof_bwd = {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                    "frac": achieved / hbm_peak, "traffic": traffic,
                    "kernel": "kBackwardQueue (back substitution of the refinement solve, all fronts)",
                    "algorithmic_bytes_per_launch": bb, "launch_ms": t_bwd * 1e3, "peak_source": peak_kind,
                    "note": "latency-bound like the factor: queue hand-offs along the assembly trees",
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
        phases = {"elements": ms5[0] / nsamp, "factor_and_first_forward": ms5[1] / nsamp,
                  "other_solve": ms5[2] / nsamp, "second_forward": ms5[3] / nsamp,
                  "back_substitution": ms5[4] / nsamp}
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": 1000.0 * dev_s_max / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64+f32" if mixed else "f64",
                "data": "synthetic (seeded generator of the 256-model beam batch)",
                "config": workload_config(args, cases_all),
                "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
                "time_steps_per_s": tsteps_tot / dev_s_max,
                "newton_iterations_per_time_step": iters_tot / max(tsteps_tot, 1.0),
                "gpu_launches": kernels * batched, "kernels_per_batched_iteration": kernels,
                "batched_iterations": batched, "models_failed": failed, "models_on_rank0": len(mods),
                "host_setup_s": setup_s, "host_threads": threads, "device": {"ordinal": dev, "pci_bus_id": bus},
                "wall_s_timed": wall_s, "clocks": clocks_info, "roofline": roof,
                "roofline_elements": roof_el, "roofline_forward": roof_fwd, "roofline_backward": roof_bwd,
                "phase_ms_per_iteration": phases,
                "launch_shape": dict(shape, probe_ms=probe_ms,
                                     how="autotuned before the first batched iteration: candidates timed on the "
                                         "batch's own fronts, the fastest kept; every candidate gives the same "
                                         "result bits"),
                "value_definition": "Newton iterations of all models / device time of the batched mixed run, "
                                    "state resident in HBM (restored device-to-device between steps)"}
        line.update(extras)
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
