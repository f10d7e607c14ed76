#!/usr/bin/env python3
"""Benchmark: factor-of-safety solve throughput on the 192k-element 3D slope.

Workload (the 3D slope the headline metric is quoted on): 120x40x40 mapped
hex mesh, NGLL=3, 4.63M dofs, three lognormally perturbed layers, seeded
synthetic data.  Form measured: the mixed-precision batched serving form --
FP32 element matrices and FP32 PCG with FP64 iterative refinement, k = 8
concurrent SRF trials sharing every element apply as 8 right-hand sides.

A step is one pass of the hot path over one batch: one plastic iteration of
all 8 trials (FP64-refined linear solve to the reference tolerances, then the
stress / yield / body-load update of each trial).  A full FOS solve on this
mesh runs for hours (failing trials run nl_maxiter = 2000 plastic iterations
of ~825 PCG iterations each), so FOS solves/s is derived from the measured
trial-plastic-iteration rate with a fixed work model: one FOS solve = 8
bisection trials x 2000 plastic iterations (an upper bound on the work, so
the figure is a lower bound on throughput).  Both arms use the same model,
so their ratio is the ratio of measured rates.

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

METRIC = "FOS solves/sec + p50/p99 latency, mixed-prec batched vs plain FP64 GPU"
UNIT = "FOS solves/s"
NL_MAXITER = 2000
FOS_TRIALS = 8               # bisection trials per FOS solve on [1,3] to 0.01
FOS_WORK = FOS_TRIALS * NL_MAXITER   # trial plastic iterations per FOS solve (upper bound)
N_CG_REF = 825               # PCG iterations per plastic iteration of the FP64 reference algorithm on this mesh
K_TRIALS = 8
CPU_SAMPLE_ITERS = 200       # PCG iterations of the oracle's timed sample (about 10 s of CPU work)


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
    sample = the same slope geometry at 120x5x10 = 6,000 elements; 30 PCG
    iterations (the reference EBE apply + vector ops) and one stress /
    yield / body-load pass, scaled linearly by element and dof counts."""
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
    nm = om.nmatblk
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


# ---------------------------------------------------------------------------
def run_reference(args, rank, world):
    if rank != 0:
        return 0
    procs = max(1, min(os.cpu_count() or 1, 16))
    t0 = time.time()
    steps = []
    rate = None
    res = None
    for i in range(args.warmup + args.steps):
        r, res = cpu_reference(procs)
        if i >= args.warmup:
            steps.append(r)
        rate = r
    rate = statistics.median(steps)
    value = rate / FOS_WORK
    sample = (f"oracle (serial FP64 restatement of the reference path) on a 6,000-element cut of the same slope "
              f"(120x5x10): 30 PCG iterations + 1 stress pass per process, scaled by element count to 192k "
              f"elements and to {N_CG_REF} PCG iterations per plastic iteration; {procs} independent processes")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1000.0 * (time.time() - t0) / max(1, args.steps + args.warmup),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "slope3d_192k FOS solve (120x40x40, NGLL=3, 4.63M dof)",
                       "fos_work_model": f"{FOS_TRIALS} trials x {NL_MAXITER} plastic iterations"},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": procs, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "trial_plastic_iters_per_s": rate, "per_process": res}
    print(json.dumps(line))
    return 0


def apply_kernel_name(kr: int, nelmt: int) -> str:
    v = os.environ.get("SG_APPLY_VARIANT", "5")
    if v == "2" and kr in (8, 16):
        return f"k_apply_tc<{kr}>"
    if v == "4" or (v == "5" and nelmt < 100000):
        return f"k_apply_mf<{kr}>"
    if v in ("3", "5") and kr in (8, 16):
        return f"k_apply_lanes<{kr}>"
    return f"k_apply_sparse_tma<float,{kr}>"


PREC_STEPS = 2               # plastic iterations compared by the precision leg


def precision_report(r64, x64, r32, x32):
    """Mixed batched vs plain FP64 after the same plastic iterations at the same SRF."""
    import numpy as np
    d = np.linalg.norm(x32 - x64) / np.linalg.norm(x64)
    return {"plastic_iterations": PREC_STEPS, "srf": r64["srf"], "rel_l2_displacement": float(d),
            "rel_umax": abs(r32["umax"] - r64["umax"]) / abs(r64["umax"]),
            "rel_fmax": abs(r32["fmax"] - r64["fmax"]) / max(abs(r64["fmax"]), 1e-300),
            "pcg_iters_fp64": r64["cg_tot"], "inner_pcg_iters_mixed": r32["cg_tot"],
            "pcg_inflation": r32["cg_tot"] / max(1, r64["cg_tot"]), "refine_rounds_mixed": r32["refine_steps"],
            "tolerance": 1e-6, "within_tolerance": bool(d <= 1e-6)}


def serving_leg(sg, args):
    """Config 4 scaled to a bounded run: a seeded Poisson stream of FOS requests
    (random slopes, log-uniform mesh sizes, k = 4..16 concurrent trials) through
    the request loop, once in the mixed batched form (4 workers, continuous
    batching) and once as plain FP64 one at a time (1 worker, bisection, k = 1).
    Both arms see the same requests and the same nl_maxiter."""
    import numpy as np
    from specfem3d_geotech_gb300 import meshgen
    rng = np.random.default_rng(4)
    n = args.serve
    sizes = np.exp(rng.uniform(math.log(args.serve_min), math.log(args.serve_max), n)).astype(int)
    meshes = [meshgen.random_slope(rng, int(sz)) for sz in sizes]
    ks = rng.integers(4, 17, n)
    arrivals = np.cumsum(rng.exponential(1.0 / args.serve_rate, n))

    def run(prec, kof, workers):
        ctl = sg.make_control(cg_tol=1e-8, nl_tol=1e-4, cg_maxiter=5000, nl_maxiter=args.serve_nl, precision=prec)
        srv = sg.Server(0, 0, workers=workers)
        t0 = time.perf_counter()
        ids = []
        for i, m in enumerate(meshes):
            dt = arrivals[i] - (time.perf_counter() - t0)
            if dt > 0:
                time.sleep(dt)
            ids.append(srv.submit(m, ctl, lo=1.0, hi=3.0, step=0.01, k=kof(i)))
        res = [srv.wait(r, timeout=7200) for r in ids]
        wall = time.perf_counter() - t0
        st = srv.stats()
        srv.close()
        lat = [r["t_done"] - r["t_arrival"] for r in res]
        return res, {"solves_per_s": len(res) / wall, "p50_s": st["p50_s"], "p99_s": st["p99_s"],
                     "mean_s": float(np.mean(lat)), "peak_concurrent": st["peak_concurrent"],
                     "trials": int(sum(r["ntrials"] for r in res)), "wall_s": wall,
                     "ok": all(r["status"] == 0 for r in res)}

    rm, mixed = run(sg.PREC_MIXED, lambda i: int(ks[i]), 4)
    rp, plain = run(sg.PREC_FP64, lambda i: 1, 1)
    same = sum(1 for a, b in zip(rm, rp) if a["fos"] == b["fos"])
    return {"requests": n, "rate_per_s": args.serve_rate, "nelmt": [int(r["nelmt"]) for r in rm],
            "k": [int(k) for k in ks], "nl_maxiter": args.serve_nl,
            "srf_grid": "k-section (mixed) / bisection (plain) on [1, 3] to 0.01",
            "mixed_batched": mixed, "plain_fp64_one_at_a_time": plain,
            "solves_per_s_ratio": mixed["solves_per_s"] / plain["solves_per_s"],
            "same_critical_srf": f"{same}/{n}", "fos_mixed": [r["fos"] for r in rm],
            "fos_plain": [r["fos"] for r in rp]}


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


def end_to_end(sg, ctx, mesh, ctl, srf, k, args, world):
    """The same work through the public API from host buffers: mesh H2D +
    device model build, the k trials for e2e_steps plastic iterations, result D2H."""
    e2e_steps = max(1, args.steps // 2)
    t0 = time.perf_counter()
    me = sg.Model(mesh, precision=sg.PREC_MIXED, ctx=ctx)
    me.batch_begin(ctl, k)
    for s in srf:
        me.batch_add(s)
    me.batch_step(e2e_steps)
    res = [me.batch_poll(t)[1] for t in range(k)]
    me.batch_end()
    t_e2e = time.perf_counter() - t0
    me.close()
    slot_steps = sum(r["nl_iter"] for r in res)
    h2d = sum(a.nbytes for a in (mesh.x, mesh.y, mesh.z, mesh.conn, mesh.mat_id, mesh.props)) + \
        sum(b.nbytes for b in mesh.bc)
    return (slot_steps / t_e2e) * world / FOS_WORK, h2d, t_e2e, e2e_steps


def run_ours(args, rank, world, local):
    import numpy as np
    import specfem3d_geotech_gb300 as sg
    from specfem3d_geotech_gb300 import build, meshgen
    build.build()
    ctx = sg.Context(local)
    mesh = meshgen.slope3d(nx=args.nx, seed=1 + rank)
    k = args.k
    srf = [1.0 + 2.0 * (t + 1) / (k + 1) for t in range(k)]   # first k-section round on [1, 3]

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
        # config-2 precision report: the same batch of k trials, first PREC_STEPS plastic iterations
        cp = sg.make_control(cg_tol=1e-8, nl_tol=1e-4, cg_maxiter=5000, nl_maxiter=PREC_STEPS,
                             precision=sg.PREC_MIXED)
        r, x = model.trials(srf, cp, want_x=True)
        prec32 = (r[0], x[0])
    t_max = barrier_max(t_ms, world)
    rate_all = slot_steps / (t_max / 1000.0) * world         # trial plastic iterations / s, all ranks
    value = rate_all / FOS_WORK
    ne, neq = model.nelmt, model.neq
    model.close()

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
        precision = precision_report(prec64[0], prec64[1], prec32[0], prec32[1])
    if args.no_e2e:
        e2e = None
    else:
        e2e_value, h2d, t_e2e, e2e_steps = end_to_end(sg, ctx, mesh, ctl, srf, k, args, world)
        e2e = {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d / e2e_steps,
               "d2h_bytes_per_step": k * 80 / e2e_steps, "seconds": t_e2e, "steps": e2e_steps}

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_max / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
        "config": {"workload": f"slope3d_{ne // 1000}k ({args.nx}x40x40 hex, NGLL=3, {neq} dof), mixed "
                               f"FP32/FP64-refined, {k} concurrent SRF trials", "nelmt": ne, "neq": neq,
                   "k_trials": k, "step": f"one plastic iteration of the {k}-trial batch",
                   "fos_work_model": f"{FOS_TRIALS} trials x {NL_MAXITER} plastic iterations per FOS solve",
                   "l2": "inputs larger than L2 (FP32 element matrices 1.87 GB)", "parallelism": f"replicas{world}"},
        "trial_plastic_iters_per_s": rate_all,
        "pcg_iters_per_step": cg / max(1, args.steps),
        "latency": {"step_p50_ms": float(np.percentile(step_ms, 50)),
                    "step_p99_ms": float(np.percentile(step_ms, 99))},
        "fp64_plain": {"trial_plastic_iters_per_s": rate64, "value": rate64 / FOS_WORK,
                       "pcg_iters_per_plastic_iter": n_cg_ref,
                       "mixed_batched_over_plain": rate_all / rate64 if rate64 == rate64 else None},
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
    if rank == 0 and not args.no_cpu:
        t0 = time.time()
        r = oracle_sample(n_cg=n_cg_ref, iters=CPU_SAMPLE_ITERS)
        cpu_rate = 1.0 / r["t_plastic_iter_full"]
        line["cpu_baseline"] = {
            "value": cpu_rate / FOS_WORK, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": (f"oracle on a 6,000-element cut of the same slope ({CPU_SAMPLE_ITERS} PCG iterations + "
                       f"1 stress pass, "
                       f"{time.time() - t0:.0f} s), scaled by element count to 192k elements and to "
                       f"{n_cg_ref:.0f} PCG iterations per plastic iteration")}
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
    ap.add_argument("--no-fp64", action="store_true", help="skip the plain FP64 comparison")
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end leg")
    ap.add_argument("--nx", type=int, default=120, help="elements along x (120 = the 192k-element mesh)")
    ap.add_argument("--serve", type=int, default=6, help="requests in the serving leg (0 = skip)")
    ap.add_argument("--serve-rate", type=float, default=50.0, help="Poisson arrival rate of the serving leg (1/s)")
    ap.add_argument("--serve-min", type=int, default=300, help="smallest request mesh (elements)")
    ap.add_argument("--serve-max", type=int, default=3000, help="largest request mesh (elements)")
    ap.add_argument("--serve-nl", type=int, default=100, help="nl_maxiter of the serving requests")
    args = ap.parse_args()
    rank, world, local = dist()
    if args.impl == "reference":
        return run_reference(args, rank, world)
    return run_ours(args, rank, world, local)


if __name__ == "__main__":
    sys.exit(main())
