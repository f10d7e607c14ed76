"""The reference's own input decks on the GPU.

tests/golden/decks holds two decks copied unchanged from the reference's
input/ folder: validation1, the slope of its input chapter
(doc/chap3_input.tex:174-190), and cubit_example, a CUBIT-meshed slope with
the same soil (gamma 18.8, E 1e5, nu 0.3, phi 20, c 29).  Both are read by the
product's deck reader (sg_model_from_deck) and run on the device.

* FP64 trials at the decks' SRFs 1.0, 1.5 and 2.0 against the oracle's runs
  of the same decks (tests/golden/deck_trials.json, made by
  tests/golden/make_golden.py deck_trials): equal plastic-iteration counts,
  PCG totals within 1 %, displacement maxima within the trial tolerance.
* the water decks validation3 and validation4 (water table, weak layer,
  pseudo-static load) at the SRF their reader gives them;
* the reference's excavation decks (excavation_1d, excavation_2d and
  excavation_2d_single) through sg_excavation as the decks specify them,
  against the oracle's runs (tests/golden/excavation_decks.json);
* validation1's own SRF list (1.0 1.5 2.0 2.15 ... 2.20) through
  sg_srf_sweep, the way the reference runs the deck (src/slope.F90:244-443):
  every listed SRF converges, and the plastic iterations climb through the
  2.15-2.20 bracket the list was written around (the displacement curve's
  knee, from which the reference's manual reads the factor of safety).
"""
import json
import os

import numpy as np
import pytest

import specfem3d_geotech_gb300 as sg

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
DECKS = os.path.join(HERE, "golden", "decks")
TRIAL_TOL = 5e-8     # a whole FP64 trial (the oracle's own reordering noise floor is 4e-8)
# excavation_2d's third stage runs 172 plastic iterations to nl_tol = 1e-5; the
# oracle's own dot-product orders (sequential, pairwise, strided, reverse)
# spread its uxmax and umax there by 8.9e-8 (stage 1: 1.6e-8), so the
# excavation decks are compared at about twice that
EXC_TOL = 2e-7


@pytest.fixture(scope="module")
def oracle_runs():
    with open(os.path.join(HERE, "golden", "deck_trials.json")) as f:
        return json.load(f)


def _control(m, prec=sg.PREC_FP64):
    c = m.deck_control()
    return c, sg.make_control(cg_tol=c["cg_tol"], nl_tol=c["nl_tol"], cg_maxiter=c["cg_maxiter"],
                              nl_maxiter=c["nl_maxiter"], phinu=c["phinu"], allelastic=c["allelastic"],
                              precision=prec)


@pytest.mark.parametrize("name", ["validation1", "cubit_example"])
def test_deck_trials_match_oracle(ctx, oracle_runs, name):
    gold = oracle_runs[name]
    m = sg.Model(deck=os.path.join(DECKS, name + ".sem"), ctx=ctx)
    assert (m.nelmt, m.neq) == (gold["nelmt"], gold["neq"])
    _, ctl = _control(m)
    for ro in gold["trials"]:
        r = m.trials([ro["srf"]], ctl)[0]
        assert r["nl_iter"] == ro["nl_iter"] and r["converged"] == ro["converged"] == 1, (ro["srf"], r, ro)
        assert abs(r["cg_tot"] - ro["cg_tot"]) <= max(3, 0.01 * ro["cg_tot"]), (r["cg_tot"], ro["cg_tot"])
        for k in ("umax", "uxmax"):
            assert abs(r[k] - ro[k]) <= TRIAL_TOL * abs(ro[k]), (k, r[k], ro[k])
    m.close()


def test_validation1_srf_list_sweep(ctx):
    m = sg.Model(deck=os.path.join(DECKS, "validation1.sem"), ctx=ctx)
    c, ctl = _control(m)
    srf = [float(s) for s in c["srf"]]
    assert srf == [1.0, 1.5, 2.0, 2.15, 2.16, 2.17, 2.18, 2.19, 2.2]
    res = m.sweep(srf, ctl)
    assert len(res) == len(srf)
    assert all(r["converged"] == 1 and r["failed"] == 0 for r in res)
    nl = [r["nl_iter"] for r in res]
    um = [r["umax"] for r in res]
    assert all(b > a for a, b in zip(nl, nl[1:])), nl
    assert all(b > a for a, b in zip(um, um[1:])), um
    # the knee: the last step of the list costs several times the first step of the bracket
    assert nl[-1] > 3 * nl[3], nl
    m.close()


@pytest.fixture(scope="module")
def oracle_excavations():
    with open(os.path.join(HERE, "golden", "excavation_decks.json")) as f:
        return json.load(f)


@pytest.mark.parametrize("name", ["excavation_1d", "excavation_2d", "excavation_2d_single"])
def test_reference_excavation_decks_match_oracle(ctx, oracle_excavations, name):
    """The reference's excavation decks as they are written (stress0 line,
    nexcav / nexcavid / excavid, ninc, all-elastic flag) through the deck
    reader and sg_excavation, against the oracle's runs of the same decks
    (tests/golden/excavation_decks.json): the same stages, plastic-iteration
    totals and failure flags, PCG totals within 1 %, displacement maxima
    within EXC_TOL."""
    gold = oracle_excavations.get(name)
    if gold is None:
        pytest.skip(f"no oracle record for {name}")
    deck = os.path.join(DECKS, name + ".sem")
    d = sg.read_deck(deck)
    m = sg.Model(deck=deck, ctx=ctx)
    _, ctl = _control(m)
    rows = m.excavation(ctl, int(d["s0_type"]), float(d["z0"]), float(d["s0"]), float(d["k0"]),
                        [int(v) for v in d["excavid"]], nexcavid=[int(v) for v in d["nexcavid"]],
                        ninc=int(d["ninc"]))
    m.close()
    ro = np.array(gold["stages"])
    assert rows.shape == ro.shape
    assert np.array_equal(rows[:, 0], ro[:, 0])
    assert np.array_equal(rows[:, 2], ro[:, 2]), (rows[:, 2], ro[:, 2])   # plastic iterations
    assert np.array_equal(rows[:, 6], ro[:, 6])                           # failed flags
    assert np.all(np.abs(rows[:, 1] - ro[:, 1]) <= np.maximum(3, 0.01 * ro[:, 1])), (rows[:, 1], ro[:, 1])
    err = np.abs(rows[:, 3:5] - ro[:, 3:5]) / np.abs(ro[:, 3:5])
    assert err.max() <= EXC_TOL, err


@pytest.mark.parametrize("name", ["validation3", "validation4"])
def test_reference_water_decks_match_oracle(ctx, name):
    """The reference's validation3 (a slope with a weak layer, c = 0, and a
    two-surface water table on materials 2 and 3) and validation4 (the same
    with its eqload: line, eqkx = 0.1) read as the reference reads them, at
    the SRF the reader gives them (1.0: their ntstep= / sf= keys are not the
    reader's nsrf= / srf=): the pore pressure enters the stress block and the
    pseudo-static load the right-hand side on the device, and the trial
    equals the oracle's run of the same deck (tests/golden/water_deck_trials.json)."""
    with open(os.path.join(HERE, "golden", "water_deck_trials.json")) as f:
        gold = json.load(f).get(name)
    if gold is None:
        pytest.skip(f"no oracle record for {name}")
    m = sg.Model(deck=os.path.join(DECKS, name + ".sem"), ctx=ctx)
    assert (m.nelmt, m.neq) == (gold["nelmt"], gold["neq"])
    c, ctl = _control(m)
    assert list(c["srf"]) == [1.0]
    for ro in gold["trials"]:
        r = m.trials([ro["srf"]], ctl)[0]
        assert r["nl_iter"] == ro["nl_iter"] and r["converged"] == ro["converged"], (r, ro)
        assert abs(r["cg_tot"] - ro["cg_tot"]) <= max(3, 0.01 * ro["cg_tot"]), (r["cg_tot"], ro["cg_tot"])
        for k in ("umax", "uxmax"):
            assert abs(r[k] - ro[k]) <= TRIAL_TOL * abs(ro[k]), (k, r[k], ro[k])
    m.close()
