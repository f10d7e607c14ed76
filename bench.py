#!/usr/bin/env python3
"""Benchmark: factor-of-safety solve throughput on the 192k-element 3D slope.

Workload (the 3D slope the headline metric is quoted on): 120x40x40 mapped
hex mesh, NGLL=3, 4.63M dofs, three lognormally perturbed layers, seeded
synthetic data; a factor-of-safety solve searches SRF on [1, 3] to 0.01 with
nl_maxiter = 2000.  Form measured: the mixed-precision batched serving form --
FP32 element matrices and FP32 PCG with FP64 iterative refinement, k = 8
concurrent SRF trials sharing every element apply as 8 right-hand sides, the
search is the bisection with its next probes run ahead in the batch (sg_fos with
k = 8).

A step is one pass of the hot path over one batch: one plastic iteration of
the 8 trials (FP64-refined linear solve to the reference tolerances, then the
stress / yield / body-load update of each trial).  A whole FOS solve on the
192k mesh runs for hours, so FOS solves/s = 1 / (plastic iterations per FOS
solve x seconds per plastic iteration): the seconds are measured on the 192k
mesh, the iteration count is measured in the same run by a complete search of
the same slope cut to 24 x 4 x 6 = 576 elements (the fos_measured leg), where
the search also runs to the end and is timed as is.  The plain FP64 line and
the CPU reference use the same counts for their own search (bisection, one
trial at a time): the GPU's plain bisection on the cut, and the oracle's
bisection on the cut (tests/golden/slope3d_cut_fos.json).

Arms: default (ours, CUDA library through the C ABI) or --impl reference
(the CPU oracle -- a restatement of the reference's serial Fortran path --
timed on a bounded sample on all host cores).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

METRIC = "FOS solves/sec + p50/p99 latency, mixed-prec batched vs plain FP64 GPU"
UNIT = "FOS solves/s"
NL_MAXITER = 2000
SRF_LO, SRF_HI, SRF_STEP = 1.0, 3.0, 0.01
GRID = int(round((SRF_HI - SRF_LO) / SRF_STEP))
BISECT_TRIALS = math.ceil(math.log2(GRID))   # 8 trials of a bisection on the 200-step grid
GOLDEN_PCG = os.path.join(ROOT, "tests", "golden", "slope3d_192k_pcg.json")


def pcg_count_ref():
    """FP64 PCG iterations per plastic iteration of the reference algorithm on
    the 192k mesh at the SRF of the benchmark's first trial: the oracle's own
    count on that mesh (warm-started plastic iterations after the first,
    tests/golden/slope3d_192k_pcg.json), else the plain FP64 GPU leg's count
    from an earlier run.  Both CPU arms scale their timed sample with it."""
    try:
        with open(GOLDEN_PCG) as f:
            g = json.load(f)
        return float(g["pcg_steady"]), "oracle on the 192k mesh (tests/golden/slope3d_192k_pcg.json)"
    except Exception:
        return 861.5, "plain FP64 GPU leg on the 192k mesh"


N_CG_REF, N_CG_SRC = pcg_count_ref()
K_TRIALS = 8
CPU_SAMPLE_ITERS = 200       # PCG iterations of the oracle's timed sample (about 10 s of CPU work)
CUT = dict(nx=24, ny=4, nz=6)   # the 576-element cut of the benchmark slope
GOLDEN_FOS = os.path.join(ROOT, "tests", "golden", "slope3d_cut_fos.json")


def workload_config(world: int, ne: int = 192000, neq: int = 4633520, nx: int = 120) -> dict:
    """The config object both arms print (one workload, one work model)."""
    return {"workload": f"slope3d_{ne // 1000}k factor-of-safety solve ({nx}x40x40 hex, NGLL=3, {neq} dof; "
                        f"SRF on [{SRF_LO:g}, {SRF_HI:g}] to {SRF_STEP:g}, nl_maxiter {NL_MAXITER})",
            "nelmt": ne, "neq": neq,
            "fos_model": "FOS solves/s = 1 / (plastic iterations per FOS solve x s per plastic iteration); "
                         "iterations counted by a complete search of the 576-element cut of the same slope",
            "l2": "inputs larger than L2 (FP32 element matrices 1.87 GB)", "parallelism": f"replicas{world}"}


def golden_fos():
    """The oracle's bisection on the cut (critical SRF, probes), or None."""
    try:
        with open(GOLDEN_FOS) as f:
            return json.load(f)
    except Exception:
        return None


def oracle_fos_iterations():
    """Trial plastic iterations of the oracle's bisection on the cut (the CPU
    reference's own search); the bisection upper bound when no record exists."""
    g = golden_fos()
    if g:
        return sum(p["nl_iter"] for p in g["probes"]), "oracle bisection on the 576-element cut"
    return BISECT_TRIALS * NL_MAXITER, "upper bound: 8 bisection trials x nl_maxiter"


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return p["hbm_gbs"], "measured"
    except Exception:
        return 6800.0, "fallback"


class Clocks:
    """nvidia-smi sampler for the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(device), f"--query-gpu={self.FIELDS}",
                                       "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                      stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

    def stop(self):
        if self.p is None:
            return None
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except Exception:
            self.p.kill()
        self.f.flush()
        self.f.seek(0)
        sm, smax, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for line in self.f.read().splitlines():
            c = [x.strip() for x in line.split(",")]
            if len(c) < 9:
                continue
            try:
                sm.append(float(c[1]))
                smax.append(float(c[2]))
            except ValueError:
                continue
            for n, v in zip(names, c[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        os.unlink(self.f.name)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def dist():
    """(rank, world, local_rank); torch.distributed only when launched by torchrun."""
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as td
        td.init_process_group("gloo")
    return rank, world, local


def barrier_max(x: float, world: int) -> float:
    if world <= 1:
        return x
    import torch
    import torch.distributed as td
    t = torch.tensor([x], dtype=torch.float64)
    td.all_reduce(t, op=td.ReduceOp.MAX)
    return float(t.item())


def barrier(world: int):
    if world > 1:
        import torch.distributed as td
        td.barrier()


# ---------------------------------------------------------------------------
# CPU oracle sample (the reference algorithm, serial, FP64)
# ---------------------------------------------------------------------------
def oracle_sample(n_cg: float = N_CG_REF, iters: int = 30):
    """Time the oracle on a bounded sample of the workload and scale it to one
    plastic iteration of one trial on the full 192k-element mesh:
    sample = the same slope geometry at 120x5x10 = 6,000 elements; `iters` PCG
    iterations (the reference EBE apply + vector ops) and one stress /
    yield / body-load pass, scaled linearly by element count."""
    import numpy as np
    from oracle.pyoracle import OracleModel, lib as olib
    from specfem3d_geotech_gb300 import meshgen
    full = dict(nelmt=192000, neq=4633520)
    mesh = meshgen.slope3d(nx=120, ny=5, nz=10)
    om = OracleModel(mesh)
    km, dp, ext = om.stiffness_bodyload()
    dinv = np.where(np.arange(om.neq + 1) > 0, 1.0 / np.where(dp == 0, 1, dp), 0.0)
    ge = np.ascontiguousarray(om.arrays()["gdof_elmt"].reshape(-1), np.int32)
    import ctypes
    u = np.zeros(om.neq + 1)
    it = ctypes.c_int(0)
    kflat = np.ascontiguousarray(km.reshape(-1))
    t0 = time.perf_counter()
    olib().orc_pcg_solver(om.neq, om.nelmt, kflat, u, ext, dinv, ge, iters, 1e-300, ctypes.byref(it))
    t_pcg = (time.perf_counter() - t0) / iters
    ym, nu = mesh.props[:, 1].copy(), mesh.props[:, 2].copy()
    phi, coh, psi = mesh.props[:, 3].copy(), mesh.props[:, 4].copy(), mesh.props[:, 5].copy()
    ev = np.zeros(om.nelmt * 27 * 6)
    st = np.zeros(om.nelmt * 27 * 6)
    bl = np.zeros(om.neq + 1)
    t0 = time.perf_counter()
    om.stress_update(u, ym, nu, phi, coh, psi, 1e-5, 0, 0, ev, st, bl)
    t_st = time.perf_counter() - t0
    se = full["nelmt"] / om.nelmt
    t_nl = n_cg * t_pcg * se + t_st * se
    return dict(t_pcg_sample=t_pcg, t_stress_sample=t_st, sample_nelmt=om.nelmt, sample_neq=om.neq,
                scale=se, t_plastic_iter_full=t_nl, n_cg=n_cg)


def _oracle_worker(q, n_cg):
    q.put(oracle_sample(n_cg))


def cpu_reference(procs: int, n_cg: float = N_CG_REF):
    """Independent trials on `procs` host cores (spawned processes)."""
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    ps = [ctx.Process(target=_oracle_worker, args=(q, n_cg)) for _ in range(procs)]
    for p in ps:
        p.start()
    res = [q.get() for _ in ps]
    for p in ps:
        p.join()
    rate = sum(1.0 / r["t_plastic_iter_full"] for r in res)   # trial plastic iterations / s
    return rate, res


def run_reference(args, rank, world):
    if rank != 0:
        return 0
    procs = max(1, min(os.cpu_count() or 1, 16))
    t0 = time.time()
    steps = []
    res = None
    for i in range(args.warmup + args.steps):
        r, res = cpu_reference(procs)
        if i >= args.warmup:
            steps.append(r)
    rate = statistics.median(steps)
    s_ref, s_src = oracle_fos_iterations()
    value = rate / s_ref
    sample = (f"oracle (serial FP64 restatement of the reference path) on a 6,000-element cut of the same slope "
              f"(120x5x10): 30 PCG iterations + 1 stress pass per process, scaled by element count to 192k "
              f"elements and to {N_CG_REF:g} PCG iterations per plastic iteration ({N_CG_SRC}); {procs} independent processes "
              f"(independent trials); {s_ref} trial plastic iterations per FOS solve ({s_src})")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1000.0 * (time.time() - t0) / max(1, args.steps + args.warmup),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": workload_config(world),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": procs, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "trial_plastic_iters_per_s": rate, "fos_plastic_iterations": s_ref, "per_process": res}
    print(json.dumps(line))
    return 0


# ---------------------------------------------------------------------------
# GPU legs
# ---------------------------------------------------------------------------
def apply_kernel_name(kr: int, nelmt: int) -> str:
    v = os.environ.get("SG_APPLY_VARIANT", "5")
    if v == "2" and kr in (8, 16):
        return f"k_apply_tc<{kr}>"
    if v == "4" or (v == "5" and nelmt < 100000):
        return f"k_apply_mf<{kr}>"
    if v in ("3", "5") and kr in (8, 16):
        return f"k_apply_lanes<{kr}>"
    return f"k_apply_sparse_tma<float,{kr}>"


PREC_STEPS = 2               # plastic iterations compared by the 192k precision check


def precision_192k(r64, x64, r32, x32):
    """Mixed batched vs plain FP64 GPU on the 192k mesh after the same plastic
    iterations at the same SRF (the full trials take hours there)."""
    import numpy as np
    d = np.linalg.norm(x32 - x64) / np.linalg.norm(x64)
    return {"plastic_iterations": PREC_STEPS, "srf": r64["srf"], "rel_l2_displacement": float(d),
            "rel_umax": abs(r32["umax"] - r64["umax"]) / abs(r64["umax"]),
            "pcg_iters_fp64": r64["cg_tot"], "inner_pcg_iters_mixed": r32["cg_tot"],
            "pcg_inflation": r32["cg_tot"] / max(1, r64["cg_tot"]), "refine_rounds_mixed": r32["refine_steps"],
            "tolerance": 1e-6, "within_tolerance": bool(d <= 1e-6)}


PREC_SRFS = (1.0, 1.2)       # whole trials of the cut compared field by field with the oracle


def start_oracle_trials():
    """Oracle trials of the cut at PREC_SRFS, started in spawned processes
    before the first GPU call; they run on the host cores meanwhile."""
    import concurrent.futures as cf
    import multiprocessing as mp
    import oracle_jobs
    ex = cf.ProcessPoolExecutor(max_workers=len(PREC_SRFS), mp_context=mp.get_context("spawn"))
    return ex, {s: ex.submit(oracle_jobs._trial, s) for s in PREC_SRFS}


def precision_vs_oracle(sg, ctx, futures):
    """Config-2 report against the FP64 oracle on the 576-element cut: the
    mixed batched form (k trials in one batch) for whole trials at SRF 1.0
    and 1.2 -- displacement L2, largest stress error, plastic-iteration
    counts -- and at the oracle's critical SRF and the grid point below it
    (the failing and the just-converging trial of its bisection), whose
    summaries the oracle run in tests/golden holds."""
    import numpy as np
    from specfem3d_geotech_gb300 import meshgen
    mesh = meshgen.slope3d(**CUT)
    g = golden_fos()
    srfs = list(PREC_SRFS)
    near = []
    if g:
        crit = g["critical_srf"]
        by = {round(p["srf"], 10): p for p in g["probes"]}
        for s in (round(crit - SRF_STEP, 10), round(crit, 10)):
            if s in by:
                near.append(by[s])
                srfs.append(s)
    m = sg.Model(mesh, precision=sg.PREC_MIXED, ctx=ctx)
    ctl = sg.make_control(cg_tol=1e-8, nl_tol=1e-4, cg_maxiter=5000, nl_maxiter=NL_MAXITER,
                          precision=sg.PREC_MIXED)
    res, x = m.trials(srfs, ctl, want_x=True)
    stress = [m.last_stress(t) for t in range(len(PREC_SRFS))]
    m.close()
    out = {"mesh": f"slope3d cut {mesh.nelmt} elements", "form": f"mixed, {len(srfs)} trials in one batch",
           "tolerance_displacement": 1e-6, "trials": []}
    for t, s in enumerate(PREC_SRFS):
        ro = futures[s].result()
        smax = float(np.abs(ro["stress"]).max())
        out["trials"].append({
            "srf": s, "nl_iter_gpu": res[t]["nl_iter"], "nl_iter_oracle": ro["nl_iter"],
            "rel_l2_displacement": float(np.linalg.norm(x[t] - ro["x"]) / np.linalg.norm(ro["x"])),
            "max_stress_error_rel": float(np.abs(stress[t] - ro["stress"]).max() / smax),
            "rel_umax": abs(res[t]["umax"] - ro["umax"]) / ro["umax"]})
    for j, p in enumerate(near):
        r = res[len(PREC_SRFS) + j]
        out["trials"].append({
            "srf": p["srf"], "nl_iter_gpu": r["nl_iter"], "nl_iter_oracle": p["nl_iter"],
            "failed_gpu": r["failed"], "failed_oracle": p["failed"],
            "rel_umax": abs(r["umax"] - p["umax"]) / p["umax"], "source": "oracle bisection record"})
    out["within_tolerance"] = all(t.get("rel_l2_displacement", 0.0) <= 1e-6 for t in out["trials"])
    out["same_iteration_counts"] = all(t["nl_iter_gpu"] == t["nl_iter_oracle"] for t in out["trials"])
    return out


def fos_measured(sg, ctx, k_mixed=K_TRIALS, extra_ks=()):
    """Complete factor-of-safety searches on the 576-element cut of the same
    slope (nl_maxiter 2000, SRF on [1, 3] to 0.01): the mixed batched form
    (k = 8, bisection probes run ahead in the batch) and the plain FP64 form (bisection, one trial at
    a time), each timed end to end, with the plastic iterations each ran."""
    from specfem3d_geotech_gb300 import meshgen
    mesh = meshgen.slope3d(**CUT)
    out = {"mesh": f"slope3d cut {CUT['nx']}x{CUT['ny']}x{CUT['nz']} = {mesh.nelmt} elements",
           "nl_maxiter": NL_MAXITER, "srf_grid": f"[{SRF_LO:g}, {SRF_HI:g}] step {SRF_STEP:g}"}
    forms = [("mixed_batched", sg.PREC_MIXED, k_mixed), ("plain_fp64", sg.PREC_FP64, 1)]
    forms += [(f"mixed_batched_k{kk}", sg.PREC_MIXED, kk) for kk in extra_ks if kk != k_mixed]
    for name, prec, k in forms:
        m = sg.Model(mesh, precision=prec, ctx=ctx)
        ctl = sg.make_control(cg_tol=1e-8, nl_tol=1e-4, cg_maxiter=5000, nl_maxiter=NL_MAXITER, precision=prec)
        t0 = time.perf_counter()
        fos, nt, nr = m.fos(ctl, SRF_LO, SRF_HI, SRF_STEP, k=k)
        t = time.perf_counter() - t0
        out[name] = {"fos": round(fos, 10), "k": k, "trials": nt, "plastic_iterations": m.fos_steps(),
                     "seconds": t, "fos_solves_per_s": 1.0 / t}
        m.close()
    g = golden_fos()
    if g:
        out["oracle"] = {"fos": g["critical_srf"], "trials": len(g["probes"]),
                         "plastic_iterations": sum(p["nl_iter"] for p in g["probes"]),
                         "seconds": g["oracle_seconds"], "source": "tests/golden/slope3d_cut_fos.json"}
    crit = {out["mixed_batched"]["fos"], out["plain_fp64"]["fos"]} | ({g["critical_srf"]} if g else set())
    out["same_critical_srf"] = len(crit) == 1
    out["fos_level_speedup"] = out["plain_fp64"]["seconds"] / out["mixed_batched"]["seconds"]
    return out


def admission_report(res, workers, budget):
    """From each request's timeline: the largest footprint sum that ran at
    once, and the requests that waited in the queue while a worker was idle
    (held back by the HBM budget, not by the worker count)."""
    iv = [(r["t_start"], r["t_done"], r["footprint"]) for r in res]
    peak = 0.0
    for t0, _, _ in iv:
        peak = max(peak, sum(f for a, b, f in iv if a <= t0 < b))
    held = 0
    for r in res:
        a, s = r["t_arrival"], r["t_start"]
        if s - a < 1e-3:
            continue
        # a worker was idle at some moment of the wait: just after the
        # arrival or just after another request finished (50 ms margin, so
        # that a request starting at that finish counts as taking the worker)
        for b in [a] + [y for _, y, _ in iv if a <= y]:
            t = b + 0.05
            if t < s and sum(1 for x, y, _ in iv if x <= t < y) < workers:
                held += 1
                break
    return {"budget_gb": budget / 1e9, "peak_running_footprint_gb": peak / 1e9,
            "held_by_budget_with_idle_worker": held}


def serving_leg(sg, args):
    """Config 4 as a bounded run: a seeded Poisson stream of FOS requests
    (random slopes, log-uniform mesh sizes, k = 4..16 concurrent trials) through
    the request loop, once in the mixed batched form (4 workers, continuous
    batching, admission by estimated HBM footprint within --serve-budget-gb)
    and once as plain FP64 one at a time (1 worker, bisection, k = 1) on the
    requests up to --serve-plain-max elements.  Both arms see the same
    requests and the same nl_maxiter."""
    import numpy as np
    from specfem3d_geotech_gb300 import meshgen
    rng = np.random.default_rng(4)
    n = args.serve
    sizes = np.exp(rng.uniform(math.log(args.serve_min), math.log(args.serve_max), n)).astype(int)
    meshes = [meshgen.random_slope(rng, int(sz)) for sz in sizes]
    ks = rng.integers(4, 17, n)
    arrivals = np.cumsum(rng.exponential(1.0 / args.serve_rate, n))
    budget = int(args.serve_budget_gb * 1e9)

    def run(prec, kof, workers, idx, budget_bytes):
        ctl = sg.make_control(cg_tol=1e-8, nl_tol=1e-4, cg_maxiter=5000, nl_maxiter=args.serve_nl, precision=prec)
        srv = sg.Server(0, budget_bytes, workers=workers)
        t0 = time.perf_counter()
        ids = []
        for i in idx:
            dt = arrivals[i] - (time.perf_counter() - t0)
            if dt > 0:
                time.sleep(dt)
            ids.append(srv.submit(meshes[i], ctl, lo=1.0, hi=3.0, step=0.01, k=kof(i)))
        res = []
        for i, r in zip(idx, ids):
            res.append(srv.wait(r, timeout=7200))
            # progress on stderr, so that a run cut short still leaves its finished requests
            print(json.dumps({"serving_request": i, "prec": int(prec), **{kk: res[-1][kk] for kk in (
                "nelmt", "fos", "ntrials", "status", "footprint", "t_arrival", "t_start", "t_done")}}),
                  file=sys.stderr, flush=True)
        wall = time.perf_counter() - t0
        st = srv.stats()
        srv.close()
        lat = [r["t_done"] - r["t_arrival"] for r in res]
        out = {"requests": len(res), "solves_per_s": len(res) / wall, "p50_s": st["p50_s"], "p99_s": st["p99_s"],
               "mean_s": float(np.mean(lat)), "peak_concurrent": st["peak_concurrent"],
               "trials": int(sum(r["ntrials"] for r in res)), "wall_s": wall,
               "ok": all(r["status"] == 0 for r in res),
               "admission": admission_report(res, workers, st["budget_bytes"])}
        return res, out

    allidx = list(range(n))
    rm, mixed = run(sg.PREC_MIXED, lambda i: int(ks[i]), 4, allidx, budget)
    pidx = [i for i in allidx if sizes[i] <= args.serve_plain_max]
    out = {"requests": n, "rate_per_s": args.serve_rate, "nelmt": [int(r["nelmt"]) for r in rm],
           "k": [int(k) for k in ks], "nl_maxiter": args.serve_nl,
           "srf_grid": "bisection on [1, 3] to 0.01 (mixed: k probes run ahead in one batch; plain: one at a time)",
           "mixed_batched": mixed, "fos_mixed": [r["fos"] for r in rm],
           "per_request_work": "each trial runs at most nl_maxiter plastic iterations; trials per request in "
                               "mixed_batched.trials"}
    if pidx:
        rp, plain = run(sg.PREC_FP64, lambda i: 1, 1, pidx, 0)
        sub = [rm[i] for i in pidx]
        # the same requests in the mixed arm's run: solves/s over that subset's own span
        same = sum(1 for a, b in zip(sub, rp) if a["fos"] == b["fos"])
        out["plain_fp64_one_at_a_time"] = plain
        out["plain_subset"] = f"{len(pidx)} requests of at most {args.serve_plain_max} elements"
        out["same_critical_srf"] = f"{same}/{len(pidx)}"
        out["fos_plain"] = [r["fos"] for r in rp]
        if len(pidx) == n:
            out["solves_per_s_ratio"] = mixed["solves_per_s"] / plain["solves_per_s"]
    return out


def plain_fp64(sg, ctx, mesh, srf0, args, want_x=False):
    """Plain FP64 one-at-a-time trial on the same mesh: trial plastic iterations/s
    and PCG iterations per plastic iteration of the reference algorithm (and,
    for the precision leg, the trial's first PREC_STEPS plastic iterations)."""
    m64 = sg.Model(mesh, precision=sg.PREC_FP64, ctx=ctx)
    c64 = sg.make_control(cg_tol=1e-8, nl_tol=1e-4, cg_maxiter=5000, nl_maxiter=NL_MAXITER)
    m64.batch_begin(c64, 1)
    m64.batch_add(srf0)
    m64.batch_step(1)
    b64 = m64.batch_poll(0)[1]
    n64 = max(1, args.steps // 2)
    ctx.mark(4)
    m64.batch_step(n64)
    ctx.mark(5)
    t64 = ctx.elapsed_ms(4, 5)
    a64 = m64.batch_poll(0)[1]
    m64.batch_end()
    px = None
    if want_x:
        cp = sg.make_control(cg_tol=1e-8, nl_tol=1e-4, cg_maxiter=5000, nl_maxiter=PREC_STEPS)
        (r, ), x = m64.trials([srf0], cp, want_x=True)
        px = (r, x[0])
    m64.close()
    steps64 = a64["nl_iter"] - b64["nl_iter"]
    return steps64 / (t64 / 1000.0), (a64["cg_tot"] - b64["cg_tot"]) / max(1, steps64), px


def excavation_leg(sg, ctx, args):
    """Config 3 at its full size: the 100 x 100 x 50 = 500k-element block, a
    20 x 20 m pit removed in 4 lifts of 5 m, overburden initial stress with
    K0 = 0.5, mixed form (one trial: FP32 operator, FP64 refinement),
    nl_maxiter bounded by --excavation-nl (the second lift, a 10 m vertical
    cut in c = 20 kPa, phi = 30 deg soil, is past its critical height and
    runs to nl_maxiter, as it fails in the reference)."""
    from specfem3d_geotech_gb300 import meshgen
    mesh = meshgen.excavation()
    t0 = time.perf_counter()
    m = sg.Model(mesh, precision=sg.PREC_MIXED, ctx=ctx)
    t_build = time.perf_counter() - t0
    ctl = sg.make_control(cg_tol=1e-8, nl_tol=1e-4, cg_maxiter=5000, nl_maxiter=args.excavation_nl,
                          precision=sg.PREC_MIXED)
    t0 = time.perf_counter()
    rows = m.excavation(ctl, 1, 50.0, 0.0, 0.5, [2, 3, 4, 5])
    t_run = time.perf_counter() - t0
    out = {"mesh": f"excavation 100x100x50 = {m.nelmt} elements, {m.neq} dof", "nl_maxiter": args.excavation_nl,
           "model_build_s": t_build, "stages_s": t_run, "hbm_bytes": ctx.hbm_used,
           "stages": [{"stage": int(r[0]), "inner_pcg_iterations": int(r[1]), "plastic_iterations": int(r[2]),
                       "uxmax": float(r[3]), "umax": float(r[4]), "fmax": float(r[5]), "failed": int(r[6])}
                      for r in rows]}
    m.close()
    return out


def end_to_end(sg, ctx, mesh, srf, k, args, s_mixed, world):
    """The same work through the public API from host buffers: mesh H2D,
    device model build, the k trials for e2e_steps plastic iterations and the
    k displacement vectors copied back (the drop-in's result, x)."""
    e2e_steps = max(3, args.steps)
    ctl = sg.make_control(cg_tol=1e-8, nl_tol=1e-4, cg_maxiter=5000, nl_maxiter=e2e_steps, precision=sg.PREC_MIXED)
    t0 = time.perf_counter()
    me = sg.Model(mesh, precision=sg.PREC_MIXED, ctx=ctx)
    _, x = me.trials(srf, ctl, want_x=True)
    t_e2e = time.perf_counter() - t0
    me.close()
    h2d = sum(a.nbytes for a in (mesh.x, mesh.y, mesh.z, mesh.conn, mesh.mat_id, mesh.props)) + \
        sum(b.nbytes for b in mesh.bc)
    value = world / (s_mixed * t_e2e / e2e_steps)
    return {"value": value, "unit": UNIT, "h2d_bytes_per_step": h2d / e2e_steps,
            "d2h_bytes_per_step": x.nbytes / e2e_steps, "seconds": t_e2e, "steps": e2e_steps,
            "includes": "mesh upload, device model build (stiffness), cold-start plastic iterations, x download"}


def _oracle_sweep_worker(q):
    from oracle.pyoracle import OracleModel
    from specfem3d_geotech_gb300 import meshgen
    m = meshgen.slope2d()
    om = OracleModel(m)
    t0 = time.perf_counter()
    rows = om.sweep(list(m.control.srf))
    q.put({"seconds": time.perf_counter() - t0, "trials": len(rows),
           "plastic_iterations": int(sum(r["nl_iter"] for r in rows)),
           "critical_srf": next((r["srf"] for r in rows if r["failed"]), None)})


def run_config0(args, rank):
    """The reference's own CPU-sized case (the 300-element plane-strain slope,
    SRF 1.00, 1.05, ... until the first failure, nl_maxiter 2000): the whole
    sweep timed on the GPU (FP64, the drop-in path) and by the oracle on one
    host core, started together (the oracle in a spawned process)."""
    if rank != 0:
        return 0
    import multiprocessing as mp
    ctxp = mp.get_context("spawn")
    q = ctxp.Queue()
    proc = ctxp.Process(target=_oracle_sweep_worker, args=(q,))
    proc.start()
    import specfem3d_geotech_gb300 as sg
    from specfem3d_geotech_gb300 import build, meshgen
    build.build()
    ctx = sg.Context(0)
    mesh = meshgen.slope2d()
    m = sg.Model(mesh, ctx=ctx)
    c = mesh.control
    ctl = sg.make_control(cg_tol=c.cg_tol, nl_tol=c.nl_tol, cg_maxiter=c.cg_maxiter, nl_maxiter=c.nl_maxiter)
    t0 = time.perf_counter()
    rows = m.sweep(list(c.srf), ctl)
    t_gpu = time.perf_counter() - t0
    m.close()
    cpu = q.get(timeout=3600)
    proc.join()
    out = {"config0_sweep": {
        "case": "300-element plane-strain slope (30x1x10 hex, NGLL=3), SRF 1.00:0.05 to the first failure, "
                "nl_maxiter 2000, FP64",
        "gpu_fp64": {"seconds": t_gpu, "trials": len(rows), "plastic_iterations": int(sum(r["nl_iter"] for r in rows)),
                     "critical_srf": next((r["srf"] for r in rows if r["failed"]), None)},
        "cpu_oracle_1core": cpu, "speedup": cpu["seconds"] / t_gpu}}
    print(json.dumps(out), flush=True)
    ctx.close()
    return 0


def run_ours(args, rank, world, local):
    import numpy as np
    # oracle trials for the precision report start before any GPU call
    oex, ofut = (None, None) if (args.no_fp64 or rank != 0) else start_oracle_trials()
    import specfem3d_geotech_gb300 as sg
    from specfem3d_geotech_gb300 import build, meshgen
    build.build()
    ctx = sg.Context(local)
    mesh = meshgen.slope3d(nx=args.nx, seed=1 + rank)
    k = args.k
    srf = [1.0 + 2.0 * (t + 1) / (k + 1) for t in range(k)]   # the first probes of a search on [1, 3]

    # ---- mixed-precision batched form, inputs resident -------------------
    model = sg.Model(mesh, precision=sg.PREC_MIXED, ctx=ctx)
    ctl = sg.make_control(cg_tol=1e-8, nl_tol=1e-4, cg_maxiter=5000, nl_maxiter=NL_MAXITER,
                          precision=sg.PREC_MIXED)
    model.batch_begin(ctl, k)
    for s in srf:
        model.batch_add(s)
    model.batch_step(args.warmup)
    before = [model.batch_poll(t)[1] for t in range(k)]
    clocks = Clocks(local)
    ctx.profile(True)
    barrier(world)
    step_ms = []
    ctx.mark(0)
    for _ in range(args.steps):
        ctx.mark(2)
        model.batch_step(1)
        ctx.mark(3)
        step_ms.append(ctx.elapsed_ms(2, 3))
    ctx.mark(1)
    t_ms = ctx.elapsed_ms(0, 1)
    prof = ctx.profile_read()
    ctx.profile(False)
    clk = clocks.stop()
    after = [model.batch_poll(t)[1] for t in range(k)]
    slot_steps = sum(a["nl_iter"] - b["nl_iter"] for a, b in zip(after, before))
    cg = sum(a["cg_tot"] - b["cg_tot"] for a, b in zip(after, before))
    model.batch_end()
    prec32 = None
    if not args.no_fp64:
        cp = sg.make_control(cg_tol=1e-8, nl_tol=1e-4, cg_maxiter=5000, nl_maxiter=PREC_STEPS,
                             precision=sg.PREC_MIXED)
        r, x = model.trials(srf, cp, want_x=True)
        prec32 = (r[0], x[0])
    t_max = barrier_max(t_ms, world)
    step_s = t_max / args.steps / 1000.0                      # seconds per batch plastic iteration
    rate_all = slot_steps / (t_max / 1000.0) * world          # trial plastic iterations / s, all ranks
    ne, neq = model.nelmt, model.neq
    model.close()

    # ---- plastic iterations per FOS solve: complete searches on the cut ----
    fosm = None if args.no_fos else fos_measured(sg, ctx, k, [int(v) for v in args.fos_extra_k.split(',') if v])
    if fosm:
        s_mixed = fosm["mixed_batched"]["plastic_iterations"]
        s_plain = fosm["plain_fp64"]["plastic_iterations"]
        count_src = "measured: complete searches on the 576-element cut in this run"
    else:
        s_mixed = BISECT_TRIALS * NL_MAXITER      # bound: every bisection decision waits a failure
        s_plain = BISECT_TRIALS * NL_MAXITER
        count_src = "upper bounds: 3 rounds x nl_maxiter (batched), 8 trials x nl_maxiter (bisection)"
    value = world / (s_mixed * step_s)

    # roofline of the dominant kernel: the batched FP32 element apply (k RHS)
    hbm, peak_kind = peaks()
    ks_nnz_unique = 2349                      # structurally non-zero unique entries of a symmetric GLL K_e
    bytes_elem = ks_nnz_unique * 4 + 27 * 4   # matrix + connectivity
    kr = 1 << (k - 1).bit_length()
    bytes_apply = ne * bytes_elem + 2 * (neq + 1) * kr * 4
    apply_ms = prof["apply_ms"] / max(1, prof["apply_launches"])
    achieved = bytes_apply / (apply_ms / 1000.0) / 1e9
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "apply_traffic.json")
    if os.path.exists(tpath):
        with open(tpath) as f:
            traffic = json.load(f).get("bytes_per_launch")

    precision = None
    if args.no_fp64:
        rate64, n_cg_ref = float("nan"), N_CG_REF
    else:
        rate64, n_cg_ref, prec64 = plain_fp64(sg, ctx, mesh, srf[0], args, want_x=True)
        rate64 *= world
        precision = {"vs_fp64_oracle_576": precision_vs_oracle(sg, ctx, ofut) if ofut else None,
                     "vs_fp64_gpu_192k": precision_192k(prec64[0], prec64[1], prec32[0], prec32[1])}
    value64 = rate64 / s_plain
    e2e = None if args.no_e2e else end_to_end(sg, ctx, mesh, srf, k, args, s_mixed, world)

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_max / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
        "config": workload_config(world, ne, neq, args.nx),
        "form": {"k_trials": k, "step": f"one plastic iteration of the {k}-trial batch",
                 "search": "sg_fos, k = 8: the bisection with its next probes run ahead in the batch"},
        "fos_plastic_iterations": {"mixed_batched": s_mixed, "plain_fp64": s_plain, "source": count_src},
        "trial_plastic_iters_per_s": rate_all,
        "pcg_iters_per_step": cg / max(1, args.steps),
        "latency": {"step_p50_ms": float(np.percentile(step_ms, 50)),
                    "step_p99_ms": float(np.percentile(step_ms, 99))},
        "fp64_plain": {"trial_plastic_iters_per_s": rate64, "value": value64,
                       "pcg_iters_per_plastic_iter": n_cg_ref,
                       "mixed_batched_over_plain_per_trial_iteration": rate_all / rate64 if rate64 == rate64 else None,
                       "mixed_batched_over_plain_fos": value / value64 if value64 == value64 else None},
        "fos_measured": fosm,
        "precision": precision,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                     "traffic": traffic, "kernel": apply_kernel_name(kr, ne),
                     "algorithmic_bytes_per_launch": bytes_apply, "avg_launch_ms": apply_ms,
                     "peak_source": peak_kind},
        "kernel_ms_per_pcg_iter": {"apply": apply_ms,
                                   "gather": prof["gather_ms"] / max(1, prof["apply_launches"]),
                                   "update": prof["update_ms"] / max(1, prof["apply_launches"]),
                                   "stress_per_step": prof["stress_ms"] / max(1, args.steps)},
        "gpu_launches": prof["launches"],
        "clocks": clk,
        "e2e": e2e,
    }
    if rank == 0 and args.serve > 0:
        line["serving"] = serving_leg(sg, args)
    if rank == 0 and args.excavation:
        line["excavation_500k"] = excavation_leg(sg, ctx, args)
    if rank == 0 and not args.no_cpu:
        t0 = time.time()
        r = oracle_sample(n_cg=N_CG_REF, iters=CPU_SAMPLE_ITERS)
        s_ref, s_src = oracle_fos_iterations()
        cpu_rate = 1.0 / r["t_plastic_iter_full"]
        line["cpu_baseline"] = {
            "value": cpu_rate / s_ref, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": (f"oracle on a 6,000-element cut of the same slope ({CPU_SAMPLE_ITERS} PCG iterations + "
                       f"1 stress pass, {time.time() - t0:.0f} s), scaled by element count to 192k elements and to "
                       f"{N_CG_REF:g} PCG iterations per plastic iteration ({N_CG_SRC}); {s_ref} trial plastic iterations per "
                       f"FOS solve ({s_src})")}
    if oex is not None:
        oex.shutdown(wait=False, cancel_futures=True)
    if rank == 0:
        print(json.dumps(line), flush=True)
    ctx.close()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--k", type=int, default=K_TRIALS)
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU oracle baseline")
    ap.add_argument("--no-fp64", action="store_true", help="skip the plain FP64 comparison and precision report")
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end leg")
    ap.add_argument("--no-fos", action="store_true", help="skip the complete searches on the 576-element cut")
    ap.add_argument("--fos-extra-k", default="", help="more batch sizes for the searches on the cut, e.g. 16")
    ap.add_argument("--nx", type=int, default=120, help="elements along x (120 = the 192k-element mesh)")
    ap.add_argument("--excavation", action="store_true", help="add the 500k-element staged excavation leg")
    ap.add_argument("--config0", action="store_true",
                    help="only time the 300-element slope's SRF sweep on the GPU and by the oracle on one core")
    ap.add_argument("--excavation-nl", type=int, default=50, help="nl_maxiter of the excavation leg")
    ap.add_argument("--serve", type=int, default=6, help="requests in the serving leg (0 = skip)")
    ap.add_argument("--serve-rate", type=float, default=50.0, help="Poisson arrival rate of the serving leg (1/s)")
    ap.add_argument("--serve-min", type=int, default=300, help="smallest request mesh (elements)")
    ap.add_argument("--serve-max", type=int, default=3000, help="largest request mesh (elements)")
    ap.add_argument("--serve-nl", type=int, default=100, help="nl_maxiter of the serving requests")
    ap.add_argument("--serve-budget-gb", type=float, default=0.0,
                    help="HBM budget of the mixed server (0 = 90%% of free memory)")
    ap.add_argument("--serve-plain-max", type=int, default=10 ** 9,
                    help="largest request (elements) also run by the plain FP64 arm")
    args = ap.parse_args()
    rank, world, local = dist()
    if args.impl == "reference":
        return run_reference(args, rank, world)
    if args.config0:
        return run_config0(args, rank)
    return run_ours(args, rank, world, local)


if __name__ == "__main__":
    sys.exit(main())
