"""Generate the committed golden fixtures under tests/golden/ with the CPU oracle.

The reference (Fortran) cannot be compiled on the build machines, so long
oracle runs whose results the GPU tests compare against are stored here as
small JSON files instead of being recomputed in every test session.

    python tests/golden/make_golden.py slope2d_sweep     # ~20-40 min, 1 core
    python tests/golden/make_golden.py slope2d_trials    # ~1 min
    python tests/golden/make_golden.py slope3d_cut_fos   # ~1 h, 1 core
    python tests/golden/make_golden.py deck_trials       # ~5 min, 1 core
    python tests/golden/make_golden.py slope3d_192k_pcg  # ~1 h, 1 core, 12 GB
    python tests/golden/make_golden.py excavation_decks  # the reference's excavation decks
    python tests/golden/make_golden.py water_deck_trials # validation3 / validation4, ~6 min

tests/golden/decks/ holds some of the reference's own input decks, copied
unchanged from its input/ folder: validation1 (the slope of its input
chapter, doc/chap3_input.tex:174-190), cubit_example (a CUBIT-meshed slope
with the same material), and the excavations excavation_1d (all-elastic, one
stage, overburden initial stress), excavation_2d (three stages, initial
stress by the SEM gravity solve) and excavation_2d_single (the same three
regions removed in one stage, nexcavid = 3), and validation3 / validation4
(a slope with a weak layer and a two-surface water table; validation4 adds
a pseudo-static load).
"""
from __future__ import annotations

import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle.pyoracle import OracleModel  # noqa: E402
from specfem3d_geotech_gb300 import meshgen  # noqa: E402


def slope2d_sweep():
    """The 300-element slope's SRF sweep 1.00:0.05:2.00 up to the first failure."""
    m = meshgen.slope2d()
    om = OracleModel(m)
    t0 = time.time()
    rows = []
    for s in m.control.srf:
        r = om.trial(s)
        r["seconds"] = time.time() - t0
        rows.append(r)
        print(json.dumps(r), flush=True)
        if r["failed"] or r["errcode"]:
            break
    crit = next((r["srf"] for r in rows if r["failed"]), None)
    out = dict(mesh="slope2d", nelmt=om.nelmt, neq=om.neq, control=m.control.__dict__, trials=rows,
               critical_srf=crit, oracle_seconds=time.time() - t0)
    with open(os.path.join(HERE, "slope2d_sweep.json"), "w") as f:
        json.dump(out, f, indent=1, default=list)


def slope2d_trials():
    """Per-trial summaries and per-NL-iteration PCG counts at SRF 1.0 and 1.1."""
    m = meshgen.slope2d()
    om = OracleModel(m)
    rows = []
    for s in (1.0, 1.1):
        r = om.trial(s, want_log=True)
        r["nl_cg"] = r["nl_cg"].tolist()
        rows.append(r)
    with open(os.path.join(HERE, "slope2d_trials.json"), "w") as f:
        json.dump(dict(mesh="slope2d", trials=rows), f, indent=1)


def slope3d_cut_fos():
    """Critical SRF of the 576-element cut of the layered 3D slope (the mesh of
    tests/test_gpu_config1.py) by the oracle's bisection on [1, 3] to 0.01 --
    the same probes as orc_fos_bisection -- with every probe's summary, so
    that the GPU's factor-of-safety searches and the near-critical trials of
    the precision report can be checked against it without an hour of CPU."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from oracle_jobs import SLOPE3D_CUT, slope3d_cut
    om = OracleModel(slope3d_cut())
    t0 = time.time()
    lo, hi, step = 1.0, 3.0, 0.01
    a, b = 0, int(round((hi - lo) / step))
    rows = []
    while b - a > 1:
        m = (a + b) // 2
        r = om.trial(lo + step * m, want_log=True)
        ue = r.pop("uerr_log")
        r.pop("nl_cg")
        r["uerr_last2"] = [float(v) for v in ue[-2:]]
        r["seconds"] = time.time() - t0
        rows.append(r)
        print(json.dumps(r), flush=True)
        if r["failed"]:
            b = m
        else:
            a = m
    out = dict(mesh="slope3d", cut=SLOPE3D_CUT, nelmt=om.nelmt, neq=om.neq, search="bisection on [1, 3] step 0.01",
               critical_srf=round(lo + step * b, 10), probes=rows, oracle_seconds=time.time() - t0)
    with open(os.path.join(HERE, "slope3d_cut_fos.json"), "w") as f:
        json.dump(out, f, indent=1)


def deck_trials(names=("validation1", "cubit_example"), srfs=(1.0, 1.5, 2.0), fname="deck_trials.json"):
    """The reference's validation1 and cubit_example decks read by the
    oracle's deck reader: trials at the decks' first three SRFs (1.0, 1.5,
    2.0) with their summaries and the last two uerr values, so that the GPU
    runs of the same decks can be compared with the oracle."""
    out = {}
    for name in names:
        om = OracleModel(deck=os.path.join(HERE, "decks", name + ".sem"))
        rows = []
        t0 = time.time()
        for s in srfs:
            r = om.trial(s, want_log=True)
            ue = r.pop("uerr_log")
            r.pop("nl_cg")
            r["uerr_last2"] = [float(v) for v in ue[-2:]]
            r["seconds"] = time.time() - t0
            rows.append(r)
            print(name, json.dumps(r), flush=True)
        out[name] = dict(nelmt=om.nelmt, neq=om.neq, control={k: (v.tolist() if hasattr(v, "tolist") else v)
                                                               for k, v in om.control().items()}, trials=rows)
    with open(os.path.join(HERE, fname), "w") as f:
        json.dump(out, f, indent=1)


def water_deck_trials():
    """validation3 and validation4 (water table; validation4 with its eqload
    line) as the reference runs them: the deck's SRF list reads as 1.0 alone
    (its ntstep= / sf= keys are not the reader's nsrf= / srf=)."""
    deck_trials(("validation3", "validation4"), (1.0,), "water_deck_trials.json")


def slope3d_192k_pcg():
    """PCG iterations per plastic iteration of the reference algorithm on the
    benchmark's own mesh (the 192k-element layered slope, seed 1) at the SRF
    of the benchmark's first trial, 1 + 2/9: the oracle's trial for three
    plastic iterations, warm-started as src/slope.F90:285-299 does.  The
    benchmark's CPU arms scale their timed sample with the mean of the
    iterations after the first (the first starts from zero)."""
    m = meshgen.slope3d(nx=120, seed=1)
    m.control.nl_maxiter = 3
    t0 = time.time()
    om = OracleModel(m)
    t_build = time.time() - t0
    r = om.trial(1.0 + 2.0 / 9.0, want_log=True)
    cg = [int(v) for v in r["nl_cg"]]
    out = dict(mesh="slope3d", nx=120, ny=40, nz=40, seed=1, nelmt=om.nelmt, neq=om.neq, srf=1.0 + 2.0 / 9.0,
               nl_iter=r["nl_iter"], pcg_per_plastic_iteration=cg,
               pcg_steady=sum(cg[1:]) / max(1, len(cg) - 1), oracle_build_seconds=t_build,
               oracle_seconds=time.time() - t0)
    print(json.dumps(out), flush=True)
    with open(os.path.join(HERE, "slope3d_192k_pcg.json"), "w") as f:
        json.dump(out, f, indent=1)


def excavation_decks():
    """The reference's excavation decks run by the oracle as the deck says
    (stress0 line, nexcav / nexcavid / excavid, ninc): the stage rows
    [stage, cg_tot, nl_tot, uxmax, umax, fmax, failed, errcode] and the time
    of each run, so that the GPU's sg_excavation on the same decks can be
    compared without the CPU time."""
    import specfem3d_geotech_gb300 as sg
    out = {}
    for name in ("excavation_1d", "excavation_2d", "excavation_2d_single"):
        deck = os.path.join(HERE, "decks", name + ".sem")
        d = sg.read_deck(deck)
        om = OracleModel(deck=deck)
        t0 = time.time()
        rows = om.excavation(int(d["s0_type"]), float(d["z0"]), float(d["s0"]), float(d["k0"]),
                             [int(v) for v in d["excavid"]], ninc=int(d["ninc"]),
                             nexcavid=[int(v) for v in d["nexcavid"]])
        out[name] = dict(nelmt=om.nelmt, neq=om.neq, s0_type=int(d["s0_type"]), nexcav=int(d["nexcav"]),
                         excavid=[int(v) for v in d["excavid"]], nexcavid=[int(v) for v in d["nexcavid"]],
                         ninc=int(d["ninc"]), stages=rows.tolist(), oracle_seconds=time.time() - t0)
        print(name, json.dumps(out[name]), flush=True)
        with open(os.path.join(HERE, "excavation_decks.json"), "w") as f:
            json.dump(out, f, indent=1)


if __name__ == "__main__":
    for name in sys.argv[1:]:
        globals()[name]()
