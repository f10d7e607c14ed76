"""GPU parity: the CUDA path through the C ABI against the CPU oracle.

Tolerances: a single FP64 PCG solve must match the oracle's displacement to
relative L2 <= 1e-8 (the PCG step tolerance); a whole plastic trial to 5e-8
with identical plastic-iteration counts, 2e-5 on stresses and 2e-3 on fmax.
These are about twice the oracle's own rounding noise floor: the oracle moves
by 5e-9 (one solve) and 4e-8 / 8.7e-6 / 8e-4 (a trial's x / stress / fmax)
when only the summation order of its dot products changes -- the stress
figure is a yield decision at a GLL point near F = 0 that flips with the
order (tests/test_oracle_kat.py::test_pcg_rounding_noise_floor and
test_trial_rounding_noise_floor) -- so tighter bounds would test rounding
order, not the algorithm.  The mixed FP32/FP64 refinement form must stay within
1e-6 of the FP64 result.  Integer outputs (node numbering, dof maps) must be
identical.
"""
import json
import os

import numpy as np
import pytest

import specfem3d_geotech_gb300 as sg
from oracle.pyoracle import OracleModel, pcg_solver as orc_pcg
from specfem3d_geotech_gb300 import meshgen

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-8
TRIAL_TOL = 5e-8
STRESS_TOL = 2e-5
FMAX_TOL = 2e-3
MIXED_TOL = 1e-6


@pytest.fixture(scope="module")
def slope():
    mesh = meshgen.slope2d()
    return mesh, OracleModel(mesh)


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def test_dropin_pcg_matches_oracle(ctx, slope):
    mesh, om = slope
    km, dp, ext = om.stiffness_bodyload()
    dinv = np.where(np.arange(om.neq + 1) > 0, 1.0 / np.where(dp == 0, 1, dp), 0.0)
    ge = om.arrays()["gdof_elmt"]
    u_ref = np.zeros(om.neq + 1)
    err_r, it_r = orc_pcg(om.neq, om.nelmt, km, u_ref, ext, dinv, ge, 5000, 1e-8)
    u = np.zeros(om.neq + 1)
    it, err, tag = sg.pcg_solver(om.neq, om.nelmt, km, u, ext, dinv, ge, 5000, 1e-8, ctx=ctx)
    assert err == 0 and err_r == 0 and tag == ""
    assert abs(it - it_r) <= 2
    assert rel(u, u_ref) <= FP64_TOL
    # warm start from a perturbed solution (src/solver.f90:38-46)
    u0 = u_ref * 0.9
    u1, u2 = u0.copy(), u0.copy()
    err_r, it_r = orc_pcg(om.neq, om.nelmt, km, u1, ext, dinv, ge, 5000, 1e-8)
    it, err, _ = sg.pcg_solver(om.neq, om.nelmt, km, u2, ext, dinv, ge, 5000, 1e-8, ctx=ctx)
    assert err == 0 and abs(it - it_r) <= 2 and rel(u2, u1) <= FP64_TOL


def test_dropin_nonconvergence_is_reported(ctx, slope):
    mesh, om = slope
    km, dp, ext = om.stiffness_bodyload()
    dinv = np.where(np.arange(om.neq + 1) > 0, 1.0 / np.where(dp == 0, 1, dp), 0.0)
    ge = om.arrays()["gdof_elmt"]
    u = np.zeros(om.neq + 1)
    it, err, tag = sg.pcg_solver(om.neq, om.nelmt, km, u, ext, dinv, ge, 3, 1e-8, ctx=ctx)
    assert err == sg.SG_ERR_NOCONV == -1
    assert tag.strip() == "ERROR: PCG solver doesn't converge!"
    assert it == 4  # the Fortran DO variable after cg_maxiter iterations


def test_dropin_rejects_bad_dof_map(ctx, slope):
    mesh, om = slope
    km, dp, ext = om.stiffness_bodyload()
    ge = om.arrays()["gdof_elmt"].copy()
    ge[0, 0] = om.neq + 5
    u = np.zeros(om.neq + 1)
    with pytest.raises(sg.SgError):
        sg.pcg_solver(om.neq, om.nelmt, km, u, ext, dp, ge, 10, 1e-8, ctx=ctx)


def test_model_mesh_and_stiffness_match_oracle(ctx, slope):
    mesh, om = slope
    m = sg.Model(mesh, ctx=ctx)
    a, b = m.arrays(), om.arrays()
    assert m.nnode == om.nnode and m.neq == om.neq
    for key in ("g_num", "gdof", "gdof_elmt"):
        assert np.array_equal(a[key], b[key]), key
    assert np.abs(a["g_coord"] - b["g_coord"]).max() <= 1e-12 * np.abs(b["g_coord"]).max()
    km, dp, ext = m.stiffness()
    kr, dr, er = om.stiffness_bodyload()
    assert np.abs(km - kr).max() <= 1e-12 * np.abs(kr).max()
    assert rel(dp, dr) <= 1e-13
    assert rel(ext, er) <= 1e-13


def test_trial_matches_oracle_fp64(ctx, slope):
    mesh, om = slope
    m = sg.Model(mesh, ctx=ctx)
    ctl = sg.make_control(cg_tol=1e-8, nl_tol=1e-4, cg_maxiter=5000, nl_maxiter=2000)
    for srf in (1.0, 1.1):
        (r,), x = m.trials([srf], ctl, want_x=True)
        ro = om.trial(srf, want_x=True, want_stress=True)
        assert r["nl_iter"] == ro["nl_iter"] and r["converged"] == ro["converged"] == 1
        assert abs(r["cg_tot"] - ro["cg_tot"]) <= max(3, 0.01 * ro["cg_tot"])
        assert rel(x[0], ro["x"]) <= TRIAL_TOL
        st = m.last_stress(0)
        assert np.abs(st - ro["stress"]).max() <= STRESS_TOL * np.abs(ro["stress"]).max()
        for key in ("uxmax", "umax"):
            assert abs(r[key] - ro[key]) <= TRIAL_TOL * abs(ro[key]), key
        assert abs(r["fmax"] - ro["fmax"]) <= FMAX_TOL * abs(ro["fmax"])


def test_golden_sweep_prefix(ctx):
    """The first trials of the committed 300-element sweep are reproduced."""
    path = os.path.join(os.path.dirname(__file__), "golden", "slope2d_sweep.json")
    with open(path) as f:
        gold = json.load(f)
    m = sg.Model(meshgen.slope2d(), ctx=ctx)
    ctl = sg.make_control(cg_tol=1e-8, nl_tol=1e-4, cg_maxiter=5000, nl_maxiter=2000)
    for g in gold["trials"][:3]:
        r = m.trials([g["srf"]], ctl)[0]
        assert r["nl_iter"] == g["nl_iter"]
        assert abs(r["umax"] - g["umax"]) <= TRIAL_TOL * g["umax"]


def test_deterministic_bitwise(ctx, slope):
    mesh, _ = slope
    m = sg.Model(mesh, ctx=ctx)
    ctl = sg.make_control()
    _, x1 = m.trials([1.05], ctl, want_x=True)
    _, x2 = m.trials([1.05], ctl, want_x=True)
    assert np.array_equal(x1, x2)


def test_batched_trials_equal_single(ctx, slope):
    mesh, _ = slope
    m = sg.Model(mesh, ctx=ctx)
    ctl = sg.make_control()
    srfs = [1.0, 1.05, 1.1]
    res, xb = m.trials(srfs, ctl, want_x=True)
    for t, s in enumerate(srfs):
        (r1,), x1 = m.trials([s], ctl, want_x=True)
        assert res[t]["nl_iter"] == r1["nl_iter"]
        assert rel(xb[t], x1[0]) <= TRIAL_TOL


def test_mixed_precision_within_tolerance(ctx, slope):
    mesh, om = slope
    m64 = sg.Model(mesh, ctx=ctx)
    m32 = sg.Model(mesh, precision=sg.PREC_MIXED, ctx=ctx)
    c64 = sg.make_control()
    c32 = sg.make_control(precision=sg.PREC_MIXED)
    (r64,), x64 = m64.trials([1.0], c64, want_x=True)
    s64 = m64.last_stress(0)
    (r32,), x32 = m32.trials([1.0], c32, want_x=True)
    s32 = m32.last_stress(0)
    assert r32["nl_iter"] == r64["nl_iter"]
    assert rel(x32[0], x64[0]) <= MIXED_TOL
    # converged stress state (stored at convergence, src/slope.F90:377-381)
    serr = np.abs(s32 - s64).max() / np.abs(s64).max()
    print(f"mixed vs FP64: displacement {rel(x32[0], x64[0]):.2e}, stress {serr:.2e}")
    assert serr <= 1e-5
    assert r32["refine_steps"] >= r32["nl_iter"]


def test_confined_column_exact_on_gpu(ctx):
    E, nu, gam, H = 1e5, 0.3, 20.0, 4.0
    mesh = meshgen.column(n=4, H=H, E=E, nu=nu, gam=gam)
    m = sg.Model(mesh, ctx=ctx)
    ctl = sg.make_control(cg_tol=1e-14, nl_maxiter=10, allelastic=1)
    (r,), x = m.trials([1.0], ctl, want_x=True)
    a = m.arrays()
    Mmod = E * (1 - nu) / ((1 + nu) * (1 - 2 * nu))
    z = a["g_coord"][:, 2]
    g = a["gdof"][:, 2]
    uz = np.where(g > 0, x[0][g], 0.0)
    ex = -gam * (H * z - z * z / 2) / Mmod
    assert np.abs(uz - ex).max() <= 1e-9 * np.abs(ex).max()


def test_excavation_matches_oracle(ctx):
    mesh = meshgen.excavation(nx=6, ny=6, nz=4, L=12.0, H=8.0, pit=4.0, lifts=2, lift_h=2.0)
    om = OracleModel(mesh)
    om.set_control(1e-8, 5000, 1e-4, 200)
    ro = om.excavation(1, 8.0, 0.0, 0.5, [2, 3])
    m = sg.Model(mesh, ctx=ctx)
    ctl = sg.make_control(cg_tol=1e-8, nl_tol=1e-4, cg_maxiter=5000, nl_maxiter=200)
    r = m.excavation(ctl, 1, 8.0, 0.0, 0.5, [2, 3])
    assert r.shape == ro.shape
    assert np.array_equal(r[:, 2], ro[:, 2])            # plastic iterations per stage
    assert np.allclose(r[:, 3:5], ro[:, 3:5], rtol=1e-8)  # uxmax, umax


def test_tma_apply_matches_register_staged(ctx, slope, tmp_path):
    """The TMA-pipelined element apply gives bitwise the same trial as the
    register-staged one (same arithmetic, different data movement)."""
    import subprocess
    import sys
    mesh, _ = slope
    m = sg.Model(mesh, ctx=ctx)
    _, x1 = m.trials([1.05], sg.make_control(), want_x=True)
    out = tmp_path / "x0.npy"
    code = ("import sys; sys.path.insert(0, %r); import numpy as np; import specfem3d_geotech_gb300 as sg;"
            "from specfem3d_geotech_gb300 import meshgen; m = sg.Model(meshgen.slope2d());"
            "_, x = m.trials([1.05], sg.make_control(), want_x=True); np.save(%r, x)") % (
        os.path.dirname(os.path.dirname(os.path.abspath(__file__))), str(out))
    env = dict(os.environ, SG_APPLY_VARIANT="0")
    subprocess.run([sys.executable, "-c", code], check=True, env=env, timeout=300)
    assert np.array_equal(np.load(out), x1)


def test_continuous_batching_slot_refill(ctx, slope):
    """A trial started in a slot freed by a finished trial gives the same
    result as the trial run alone; so does a trial that ran in the mix."""
    mesh, _ = slope
    m = sg.Model(mesh, ctx=ctx)
    ctl = sg.make_control()
    alone = {s: m.trials([s], ctl)[0] for s in (1.0, 1.1, 1.05)}
    m.batch_begin(ctl, 2)
    a = m.batch_add(1.0)
    b = m.batch_add(1.1)
    c_started = False
    res = {}
    for _ in range(5000):
        nlive = m.batch_step(1)
        for slot in (a, b):
            state, r = m.batch_poll(slot)
            if state == 2 and r["srf"] not in res:
                res[r["srf"]] = r
                m.batch_release(slot)
                if not c_started:
                    m.batch_add(1.05)   # refills the freed slot while the other trial runs
                    c_started = True
        if nlive == 0 and c_started and len(res) == 3:
            break
        if nlive == 0 and len(res) >= 2 and not c_started:
            break
    m.batch_end()
    assert set(res) == {1.0, 1.1, 1.05}
    for s, r in res.items():
        assert r["nl_iter"] == alone[s]["nl_iter"]
        assert abs(r["umax"] - alone[s]["umax"]) <= TRIAL_TOL * alone[s]["umax"]


def test_sweep_critical_srf_matches_golden(ctx):
    """The slope3d SRF sweep 1.00:0.05:2.00 on the 300-element slope stops at the
    oracle's critical SRF (1.35) with the oracle's plastic-iteration counts."""
    path = os.path.join(os.path.dirname(__file__), "golden", "slope2d_sweep.json")
    with open(path) as f:
        gold = json.load(f)
    mesh = meshgen.slope2d()
    m = sg.Model(mesh, ctx=ctx)
    res = m.sweep(list(mesh.control.srf), sg.make_control())
    assert [r["srf"] for r in res] == [g["srf"] for g in gold["trials"]]
    assert res[-1]["failed"] == 1 and res[-1]["srf"] == gold["critical_srf"]
    for r, g in zip(res, gold["trials"]):
        assert r["nl_iter"] == g["nl_iter"] and r["failed"] == g["failed"]
        if not g["failed"]:
            assert abs(r["umax"] - g["umax"]) <= TRIAL_TOL * g["umax"]


def test_fos_mixed_batched_matches_oracle_critical_srf(ctx):
    """Mixed precision, a refilled batch of 8 concurrent trials: the oracle's
    critical SRF; plain FP64 bisection finds the same."""
    mesh = meshgen.slope2d()
    m = sg.Model(mesh, precision=sg.PREC_MIXED, ctx=ctx)
    fos, ntrials, nrounds = m.fos(sg.make_control(precision=sg.PREC_MIXED), lo=1.0, hi=2.0, step=0.05, k=8)
    assert abs(fos - 1.35) < 1e-12
    assert ntrials >= 2 and nrounds >= 1
    m64 = sg.Model(mesh, ctx=ctx)
    fos64, nt64, _ = m64.fos(sg.make_control(), lo=1.0, hi=2.0, step=0.05, k=1)
    assert abs(fos64 - 1.35) < 1e-12 and nt64 <= 5


def test_tensor_core_apply_matches_simt(ctx, tmp_path):
    """The tcgen05 batched apply (3xTF32, TMEM accumulators) reproduces the SIMT
    FP32 apply's trials to the mixed-precision tolerance, 8 trials per batch."""
    import subprocess
    import sys
    srfs = [1.0, 1.02, 1.05, 1.1, 1.15, 1.2, 1.25, 1.3]
    mesh = meshgen.slope2d()
    m = sg.Model(mesh, precision=sg.PREC_MIXED, ctx=ctx)
    ctl = sg.make_control(precision=sg.PREC_MIXED)
    res1, x1 = m.trials(srfs, ctl, want_x=True)
    out = tmp_path / "tc.npz"
    code = ("import sys; sys.path.insert(0, %r); import numpy as np; import specfem3d_geotech_gb300 as sg;"
            "from specfem3d_geotech_gb300 import meshgen; m = sg.Model(meshgen.slope2d(), precision=sg.PREC_MIXED);"
            "r, x = m.trials(%r, sg.make_control(precision=sg.PREC_MIXED), want_x=True);"
            "np.savez(%r, x=x, nl=np.array([t['nl_iter'] for t in r]))") % (
        os.path.dirname(os.path.dirname(os.path.abspath(__file__))), srfs, str(out))
    env = dict(os.environ, SG_APPLY_VARIANT="2")
    subprocess.run([sys.executable, "-c", code], check=True, env=env, timeout=600)
    d = np.load(out)
    assert [r["nl_iter"] for r in res1] == d["nl"].tolist()
    for t in range(len(srfs)):
        assert rel(d["x"][t], x1[t]) <= MIXED_TOL


def _variant_trials(variant, srfs, out, var="SG_APPLY_VARIANT", extra=None):
    import subprocess
    import sys
    code = ("import sys; sys.path.insert(0, %r); import numpy as np; import specfem3d_geotech_gb300 as sg;"
            "from specfem3d_geotech_gb300 import meshgen; m = sg.Model(meshgen.slope2d(), precision=sg.PREC_MIXED);"
            "r, x = m.trials(%r, sg.make_control(precision=sg.PREC_MIXED), want_x=True);"
            "np.savez(%r, x=x, nl=np.array([t['nl_iter'] for t in r]), cg=np.array([t['cg_tot'] for t in r]))") % (
        os.path.dirname(os.path.dirname(os.path.abspath(__file__))), srfs, str(out))
    env = dict(os.environ)
    env.update(extra or {})
    env[var] = str(variant)
    subprocess.run([sys.executable, "-c", code], check=True, env=env, timeout=600)
    return np.load(out)


@pytest.mark.parametrize("k", [8, 16])
def test_lane_apply_matches_node_lane_apply(tmp_path, k):
    """The lane-per-(element, trial) FP32 apply (sums in storage order) gives
    the node-lane TMA apply's trials to the mixed-precision tolerance, with the
    same plastic-iteration counts, for 8 and 16 trials per batch; two runs of
    it are bitwise equal."""
    srfs = [1.0 + 0.02 * t for t in range(k)]
    a = _variant_trials(1, srfs, tmp_path / "v1.npz")
    b = _variant_trials(3, srfs, tmp_path / "v3.npz")
    c = _variant_trials(3, srfs, tmp_path / "v3b.npz")
    assert a["nl"].tolist() == b["nl"].tolist()
    for t in range(k):
        assert rel(b["x"][t], a["x"][t]) <= MIXED_TOL
    assert np.array_equal(b["x"], c["x"]) and np.array_equal(b["cg"], c["cg"])


@pytest.mark.parametrize("k", [8, 16])
def test_fused_two_kernel_iteration_matches_three_kernels(tmp_path, k):
    """The FP32 PCG step as two kernels (the lane apply forms the direction,
    k_pcg_gather_update does the gather, the vector update and the next
    step's dots) against the three-kernel step: the same trials to the
    mixed-precision tolerance and plastic-iteration counts; reruns bitwise."""
    srfs = [1.0 + 0.02 * t for t in range(k)]
    env3 = {"SG_APPLY_VARIANT": "3"}
    a = _variant_trials(0, srfs, tmp_path / "f0.npz", var="SG_FUSED", extra=env3)
    b = _variant_trials(1, srfs, tmp_path / "f1.npz", var="SG_FUSED", extra=env3)
    c = _variant_trials(1, srfs, tmp_path / "f1b.npz", var="SG_FUSED", extra=env3)
    assert a["nl"].tolist() == b["nl"].tolist()
    for t in range(k):
        assert rel(b["x"][t], a["x"][t]) <= MIXED_TOL
    assert np.array_equal(b["x"], c["x"]) and np.array_equal(b["cg"], c["cg"])


def test_row_gather_matches_staged_gather(tmp_path):
    """The row-cooperative FP32 gather (coalesced 16-byte pieces, no shared
    memory) gives the staged gather's trials to the mixed-precision tolerance
    with the same plastic-iteration counts; two runs of it are bitwise equal."""
    srfs = [1.0 + 0.03 * t for t in range(8)]
    a = _variant_trials(0, srfs, tmp_path / "g0.npz", var="SG_GATHER_VARIANT")
    b = _variant_trials(1, srfs, tmp_path / "g1.npz", var="SG_GATHER_VARIANT")
    c = _variant_trials(1, srfs, tmp_path / "g1b.npz", var="SG_GATHER_VARIANT")
    assert a["nl"].tolist() == b["nl"].tolist()
    for t in range(len(srfs)):
        assert rel(b["x"][t], a["x"][t]) <= MIXED_TOL
    assert np.array_equal(b["x"], c["x"]) and np.array_equal(b["cg"], c["cg"])


def test_mixed_batch_of_eight_equals_single_trials(ctx, slope):
    """Eight mixed-precision trials in one batch (lane apply, row gather and
    16-byte update for 8 right-hand sides; columns finish at different PCG
    iterations) give each trial's single-trial result (node-lane apply, staged
    gather, scalar update) to the mixed-precision tolerance."""
    mesh, _ = slope
    m = sg.Model(mesh, precision=sg.PREC_MIXED, ctx=ctx)
    ctl = sg.make_control(precision=sg.PREC_MIXED)
    srfs = [1.0, 1.04, 1.08, 1.12, 1.16, 1.2, 1.24, 1.28]
    res, xb = m.trials(srfs, ctl, want_x=True)
    for t in (0, 3, 7):
        (r1,), x1 = m.trials([srfs[t]], ctl, want_x=True)
        assert res[t]["nl_iter"] == r1["nl_iter"]
        assert rel(xb[t], x1[0]) <= MIXED_TOL


@pytest.mark.parametrize("k", [1, 2, 8, 16])
def test_matrix_free_fp32_operator_matches_stored(tmp_path, k):
    """The matrix-free FP32 operator (stress fluxes at the GLL points from
    J^-1 and C, no stored element matrix) drives the mixed solve to the same
    trials as the stored FP32 matrices, to the mixed-precision tolerance, with
    the same plastic-iteration counts; two runs of it are bitwise equal.  All
    probes stay below the critical SRF 1.35 (a failing trial's displacement
    grows without bound and is not comparable)."""
    srfs = [1.0 + 0.02 * t for t in range(k)]
    a = _variant_trials(3, srfs, tmp_path / "st.npz")
    b = _variant_trials(4, srfs, tmp_path / "mf.npz")
    c = _variant_trials(4, srfs, tmp_path / "mf2.npz")
    assert a["nl"].tolist() == b["nl"].tolist()
    for t in range(k):
        assert rel(b["x"][t], a["x"][t]) <= MIXED_TOL
    assert np.array_equal(b["x"], c["x"]) and np.array_equal(b["cg"], c["cg"])


def test_graph_replay_bitwise_equal_to_eager(ctx, slope):
    """On small meshes each chunk of PCG iterations is replayed as a captured
    CUDA graph; with profiling on the same chunk runs as eager launches.  Both
    give bitwise the same trial (the graph holds exactly the eager launches)."""
    mesh, _ = slope
    m = sg.Model(mesh, precision=sg.PREC_MIXED, ctx=ctx)
    ctl = sg.make_control(precision=sg.PREC_MIXED)
    srfs = [1.0, 1.1, 1.2]
    r_graph, x_graph = m.trials(srfs, ctl, want_x=True)
    ctx.profile(True)
    try:
        r_eager, x_eager = m.trials(srfs, ctl, want_x=True)
    finally:
        ctx.profile(False)
    assert np.array_equal(x_graph, x_eager)
    assert [r["cg_tot"] for r in r_graph] == [r["cg_tot"] for r in r_eager]


@pytest.mark.parametrize("k", [1, 8, 16])
def test_matrix_free_line_form_bitwise_equals_point_form(tmp_path, k):
    """The line form of the matrix-free apply (xi terms kept in registers)
    does the point form's arithmetic in the same order: bitwise equal trials."""
    srfs = [1.0 + 0.02 * t for t in range(k)]
    os.environ.pop("SG_MF_POINTS", None)
    a = _variant_trials(4, srfs, tmp_path / "lines.npz")
    try:
        os.environ["SG_MF_POINTS"] = "1"
        b = _variant_trials(4, srfs, tmp_path / "points.npz")
    finally:
        os.environ.pop("SG_MF_POINTS", None)
    assert np.array_equal(a["x"], b["x"]) and np.array_equal(a["cg"], b["cg"])


def test_pseudo_static_load_matches_oracle(ctx, tmp_path):
    """sg_model_set_eqload builds the load of src/preprocess.f90:137-143 (the
    deck's eqload: line gives the same model), and a plastic trial under it
    matches the oracle's."""
    mesh = meshgen.slope2d()
    om = OracleModel(mesh)
    om.set_eqload(0.05, 0.0, 0.0)
    _, _, ext_o = om.stiffness_bodyload()
    m = sg.Model(mesh, ctx=ctx)
    m.set_eqload(0.05, 0.0, 0.0)
    _, _, ext = m.stiffness(want_k=False)
    assert rel(ext, ext_o) <= 1e-12
    # the same factors through the deck reader
    deck = meshgen.write_deck(mesh, str(tmp_path))
    with open(deck, "a") as f:
        f.write("eqload: eqkx=0.05, eqky=0.0, eqkz=0.0\n")
    md = sg.Model(None, deck=deck, ctx=ctx)
    _, _, ext_d = md.stiffness(want_k=False)
    assert np.array_equal(ext_d, ext)
    ctl = sg.make_control(cg_tol=1e-8, nl_tol=1e-4, cg_maxiter=5000, nl_maxiter=2000)
    (r,), x = m.trials([1.0], ctl, want_x=True)
    ro = om.trial(1.0, want_x=True)
    assert r["nl_iter"] == ro["nl_iter"] and r["failed"] == ro["failed"]
    assert rel(x[0], ro["x"]) <= TRIAL_TOL


def test_nodal_stress_matches_oracle(ctx, slope):
    """The device's valency-averaged nodal stress (src/slope.F90:419-437) is
    bitwise the oracle's average of the same element stresses, and within the
    stress tolerance of the oracle's own trial."""
    mesh, om = slope
    m = sg.Model(mesh, ctx=ctx)
    (r,), x = m.trials([1.0], sg.make_control(), want_x=True)
    st = m.last_stress(0)
    ns = m.nodal_stress(0)
    assert np.array_equal(ns, om.nodal_stress(st))
    ro = om.trial(1.0, want_x=True, want_stress=True)
    ns_o = om.nodal_stress(ro["stress"])
    assert np.abs(ns - ns_o).max() <= STRESS_TOL * np.abs(ns_o).max()
    u = m.nodal_displacement(x[0])
    assert u.shape == (m.nnode, 3) and abs(np.abs(u).max() - r["uxmax"]) <= 1e-12 * r["uxmax"]


def test_excavation_fields_match_oracle(ctx):
    """The last stage's nodal fields of the excavation driver
    (src/excavation.F90:597-661): von Mises effective plastic strain averaged
    over the intact valency and the smallest point safety factor per node."""
    mesh = meshgen.excavation(nx=6, ny=6, nz=4, L=12.0, H=8.0, pit=4.0, lifts=2, lift_h=2.0)
    om = OracleModel(mesh)
    om.set_control(1e-8, 5000, 1e-4, 200)
    ro, vm_o, sf_o = om.excavation(1, 8.0, 0.0, 0.5, [2, 3], want_fields=True)
    m = sg.Model(mesh, ctx=ctx)
    ctl = sg.make_control(cg_tol=1e-8, nl_tol=1e-4, cg_maxiter=5000, nl_maxiter=200)
    r = m.excavation(ctl, 1, 8.0, 0.0, 0.5, [2, 3])
    vm, sf = m.excavation_fields()
    assert r.shape == ro.shape
    outside = sf_o == 1e32                       # nodes of removed elements only
    assert np.array_equal(sf == 1e32, outside) and outside.sum() > 0
    np.testing.assert_allclose(sf[~outside], sf_o[~outside], rtol=1e-5)
    scale = max(np.abs(vm_o).max(), 1e-300)
    assert np.abs(vm - vm_o).max() <= STRESS_TOL * scale


@pytest.mark.parametrize("k", [1, 2, 4, 8])
def test_persistent_pcg_matches_separate_kernels(tmp_path, k):
    """On small meshes the FP32 PCG iterations run as one persistent
    cooperative kernel (grid barriers between apply, gather and update; every
    block recomputes alpha and beta from the partials in a fixed order).  Its
    trials equal those of the separate kernels to the mixed tolerance with the
    same plastic-iteration counts, and two runs are bitwise equal."""
    srfs = [1.0 + 0.03 * t for t in range(k)]
    a = _variant_trials(0, srfs, tmp_path / "sep.npz", var="SG_PERSIST")
    b = _variant_trials(1, srfs, tmp_path / "per.npz", var="SG_PERSIST")
    c = _variant_trials(1, srfs, tmp_path / "per2.npz", var="SG_PERSIST")
    assert a["nl"].tolist() == b["nl"].tolist()
    for t in range(k):
        assert rel(b["x"][t], a["x"][t]) <= MIXED_TOL
    assert np.array_equal(b["x"], c["x"]) and np.array_equal(b["cg"], c["cg"])


def _ws(tmp_path, text, name="ws.txt"):
    p = tmp_path / name
    p.write_text(text)
    return str(p)


def test_water_pressure_matches_oracle(ctx, tmp_path):
    """compute_pressure on the device (k_mark_submerged + k_water_pressure)
    against the oracle for the line kinds, the first-surface rule and a meshed
    surface; the deck's water: line gives the same field; a meshed surface off
    the origin plane is the reference's error."""
    slope2d = meshgen.slope2d(srf=(1.0,))
    slope2d.props = np.vstack([slope2d.props, slope2d.props])
    xc = slope2d.x[slope2d.conn - 1].mean(axis=1)
    slope2d.mat_id = np.where(xc < 14.0, 2, 1).astype(np.int32)
    box = meshgen.box(nx=3, ny=2, nz=3, L=3.0, W=2.0, zbot=-3.0, ztop=0.0)
    top = [(i + 3 * (j + 2 * 2) + 1, meshgen.FACE_ZMAX) for j in range(2) for i in range(3)]
    cases = [
        (slope2d, [2], "2\n0\n1 0.0 10.0 2.0\n1\n1 0.0 20.0 3.0 7.0\n"),
        (box, [1], "1\n2\n%d\n" % len(top) + "".join("%d %d\n" % f for f in top)),
    ]
    for n, (mesh, ids, text) in enumerate(cases):
        path = _ws(tmp_path, text, f"ws{n}.txt")
        om = OracleModel(mesh)
        om.set_water(ids, path)
        m = sg.Model(mesh, ctx=ctx)
        assert m.pore_pressure() is None
        m.set_water(ids, path)
        wp_o, sub_o = om.pore_pressure()
        wp = m.pore_pressure()
        assert (wp_o > 0).sum() > 0
        np.testing.assert_allclose(wp, wp_o, rtol=1e-13, atol=1e-12)
        assert np.array_equal(wp[~sub_o], np.zeros((~sub_o).sum()))
    mesh, ids, text = cases[0]
    mesh.water = (tuple(ids), text)
    deck = meshgen.write_deck(mesh, str(tmp_path / "deck"))
    md = sg.Model(None, deck=deck, ctx=ctx)
    od = OracleModel(deck=deck)
    np.testing.assert_allclose(md.pore_pressure(), od.pore_pressure()[0], rtol=1e-13, atol=1e-12)
    high = meshgen.box(nx=2, ny=2, nz=2, L=2.0, W=2.0, zbot=0.0, ztop=5.0)
    faces = [(i + 2 * (j + 2) + 1, meshgen.FACE_ZMAX) for j in range(2) for i in range(2)]
    path = _ws(tmp_path, "1\n2\n4\n" + "".join("%d %d\n" % f for f in faces), "high.txt")
    mh = sg.Model(high, ctx=ctx)
    with pytest.raises(sg.SgError, match="free surface cannot be determined"):
        mh.set_water([1], path)
    assert mh.pore_pressure() is None


def test_water_trial_matches_oracle(ctx, tmp_path):
    """A plastic slope trial under a water table (pore pressure added to the
    effective stress after the stored stress, src/slope.F90:334-341) matches
    the oracle's, in FP64 and in the mixed form."""
    mesh = meshgen.slope2d(srf=(1.0,))
    path = _ws(tmp_path, "1\n0\n1 0.0 20.0 6.0\n")
    om = OracleModel(mesh)
    om.set_water([1], path)
    ro = om.trial(1.0, want_x=True, want_stress=True)
    assert ro["converged"] == 1
    ctl = sg.make_control(cg_tol=1e-8, nl_tol=1e-4, cg_maxiter=5000, nl_maxiter=2000)
    m = sg.Model(mesh, ctx=ctx)
    m.set_water([1], path)
    (r,), x = m.trials([1.0], ctl, want_x=True)
    assert r["nl_iter"] == ro["nl_iter"] and r["converged"] == 1
    assert rel(x[0], ro["x"]) <= TRIAL_TOL
    st = m.last_stress(0)
    assert np.abs(st - ro["stress"]).max() <= STRESS_TOL * np.abs(ro["stress"]).max()
    assert abs(r["fmax"] - ro["fmax"]) <= FMAX_TOL * abs(ro["fmax"])
    mm = sg.Model(mesh, ctx=ctx, precision=sg.PREC_MIXED)
    mm.set_water([1], path)
    ctl32 = sg.make_control(cg_tol=1e-8, nl_tol=1e-4, cg_maxiter=5000, nl_maxiter=2000, precision=sg.PREC_MIXED)
    (rm,), xm = mm.trials([1.0], ctl32, want_x=True)
    assert rm["nl_iter"] == ro["nl_iter"]
    assert rel(xm[0], ro["x"]) <= MIXED_TOL
    # removing the pressure gives the dry trial back
    m.set_pore_pressure(None)
    (rd,), xd = m.trials([1.0], ctl, want_x=True)
    rdo = OracleModel(mesh).trial(1.0, want_x=True)
    assert rd["nl_iter"] == rdo["nl_iter"] and rel(xd[0], rdo["x"]) <= TRIAL_TOL


def test_water_excavation_matches_oracle(ctx, tmp_path):
    """Staged excavation under a water table (pore pressure added before the
    stored stress, src/excavation.F90:566-576)."""
    mesh = meshgen.excavation(nx=6, ny=6, nz=4, L=12.0, H=8.0, pit=4.0, lifts=2, lift_h=2.0)
    path = _ws(tmp_path, "1\n0\n1 0.0 12.0 5.0\n")
    om = OracleModel(mesh)
    om.set_control(1e-8, 5000, 1e-4, 200)
    om.set_water([1], path)
    ro = om.excavation(1, 8.0, 0.0, 0.5, [2, 3])
    m = sg.Model(mesh, ctx=ctx)
    m.set_water([1], path)
    ctl = sg.make_control(cg_tol=1e-8, nl_tol=1e-4, cg_maxiter=5000, nl_maxiter=200)
    r = m.excavation(ctl, 1, 8.0, 0.0, 0.5, [2, 3])
    assert r.shape == ro.shape
    assert ro[1, 2] > 2                                  # the water changes the second stage
    assert np.array_equal(r[:, 2], ro[:, 2])
    assert np.allclose(r[:, 3:5], ro[:, 3:5], rtol=1e-8)


def _stress_inputs(mesh, om, srf):
    from oracle.pyoracle import dt_viscoplas, strength_reduction
    gam, ym, nu, phi, coh, psi = (mesh.props[:, i] for i in range(6))
    _, cohf, nuf, phif, psif = strength_reduction(srf, coh, nu, phi, psi)
    dt = dt_viscoplas(nuf, phif, ym)
    a = om.arrays()
    km, dp, ext = om.stiffness_bodyload()
    dpi = np.zeros_like(dp)
    dpi[1:] = 1.0 / dp[1:]
    x = np.zeros(om.neq + 1)
    orc_pcg(om.neq, om.nelmt, km, x, ext, dpi, a["gdof_elmt"], 5000, 1e-8)
    return dict(props=(ym, nuf, phif, cohf, psif), dt=dt, a=a, x=x, km=km, dpi=dpi, ext=ext)


def _gpu_pass(om, I, x, conv, last, ev, st, bl, **kw):
    a = I["a"]
    return sg.stress_bodyload(om.neq, om.nelmt, om.nnode, a["g_coord"], a["g_num"] + 1, a["gdof_elmt"], a["mat_id"],
                              *I["props"], I["dt"], conv, last, x, ev, st, bl, **kw)


# One pass of the stress block from identical inputs.  Most points agree to
# rounding (1e-13), but points in axisymmetric states sit on the Lode corner,
# sin(3 theta) = -3 sqrt(3) J3 / (2 J2^1.5) = +-1, where theta = asin(s)/3 has an
# infinite derivative: a rounding delta ~ 1e-16 in s moves theta by
# sqrt(2 delta)/3 ~ 5e-9 and with it the point's flow direction.  That is the
# reference algorithm's own sensitivity, so the bounds are sqrt(eps)-scale: max
# norms 1e-7 of the field's maximum (observed 2.2e-9), L2 norms 1e-9 (observed
# 1.5e-10).
PASS_MAX_TOL = 1e-7
PASS_L2_TOL = 1e-9


def test_stress_dropin_matches_oracle_passes(ctx):
    """sg_stress_bodyload against the oracle's pass of src/slope.F90:311-383 on
    the same inputs: three plastic passes from the same state, then the
    finalising pass that stores the stress; a repeated call (cached mesh) is
    bitwise equal."""
    mesh = meshgen.slope2d(srf=(1.0,))
    om = OracleModel(mesh)
    I = _stress_inputs(mesh, om, 1.3)
    nst = om.nelmt * 27 * 6
    ev, st, bl = np.zeros(nst), np.zeros(nst), np.zeros(om.neq + 1)
    x = I["x"].copy()
    for it in range(4):
        last = it == 3
        evg, stg, blg = ev.copy(), st.copy(), bl.copy()
        fg = _gpu_pass(om, I, x, False, last, evg, stg, blg)
        ev2, st2, bl2 = ev.copy(), st.copy(), bl.copy()
        fg2 = _gpu_pass(om, I, x, False, last, ev2, st2, bl2)
        assert fg2 == fg and np.array_equal(ev2, evg) and np.array_equal(st2, stg) and np.array_equal(bl2, blg)
        fo = om.stress_update(x, *I["props"], I["dt"], 0, int(last), ev, st, bl)
        print(f"pass {it}: fmax {abs(fg - fo) / fo:.2e} evpt max {np.abs(evg - ev).max() / np.abs(ev).max():.2e} "
              f"l2 {rel(evg, ev):.2e} bodyload {rel(blg, bl):.2e}")
        assert fo > 0 and abs(fg - fo) <= 1e-12 * fo
        assert np.abs(evg - ev).max() <= PASS_MAX_TOL * np.abs(ev).max() and rel(evg, ev) <= PASS_L2_TOL
        assert rel(blg, bl) <= PASS_L2_TOL and blg[0] == 0.0
        if last:
            assert np.abs(stg - st.reshape(-1)).max() <= PASS_MAX_TOL * np.abs(st).max()
        else:
            load = I["ext"] + bl
            load[0] = 0.0
            orc_pcg(om.neq, om.nelmt, I["km"], x, load, I["dpi"], I["a"]["gdof_elmt"], 5000, 1e-8)
            x[0] = 0.0


def test_host_loop_with_gpu_dropins_matches_oracle_trial(ctx):
    """The reference's plastic loop on the host around the two GPU drop-ins
    (sg_pcg_solve, sg_stress_bodyload) gives the oracle's trial."""
    from dropin_loop import host_trial
    mesh = meshgen.slope2d(srf=(1.0,))
    om = OracleModel(mesh)
    a = om.arrays()

    def pcg(neq, nelmt, km, x, load, dpi, ge, maxit, tol):
        it, err, _ = sg.pcg_solver(neq, nelmt, km, x, load, dpi, ge, maxit, tol, ctx=ctx)
        return err, it

    def stress_pass(x, ym, nuf, phif, cohf, psif, dt, conv, last, ev, st, bl):
        return sg.stress_bodyload(om.neq, om.nelmt, om.nnode, a["g_coord"], a["g_num"] + 1, a["gdof_elmt"],
                                  a["mat_id"], ym, nuf, phif, cohf, psif, dt, conv, last, x, ev, st, bl, ctx=ctx)

    r = host_trial(om, mesh, 1.0, pcg, stress_pass)
    ro = om.trial(1.0, want_x=True, want_stress=True)
    assert r["nl_iter"] == ro["nl_iter"] and r["converged"] == 1
    assert rel(r["x"], ro["x"]) <= TRIAL_TOL
    assert np.abs(r["stress"] - ro["stress"].reshape(-1)).max() <= STRESS_TOL * np.abs(ro["stress"]).max()
    assert abs(r["fmax"] - ro["fmax"]) <= FMAX_TOL * abs(ro["fmax"])


def test_stress_dropin_excavation_form(ctx, tmp_path):
    """The excavation form over an element list (elmt_intact), with a water
    table: pressure before the stored stress, vmeps/scf accumulated in list
    order when finalising (src/excavation.F90:546-616)."""
    mesh = meshgen.excavation(nx=6, ny=6, nz=4, L=12.0, H=8.0, pit=4.0, lifts=2, lift_h=2.0)
    om = OracleModel(mesh)
    om.set_water([1], _ws(tmp_path, "1\n0\n1 0.0 12.0 5.0\n"))
    wp = om.pore_pressure()[0]
    I = _stress_inputs(mesh, om, 1.0)
    elist = np.flatnonzero(mesh.mat_id != 3) + 1            # the removed lifts' material stays out
    assert 0 < elist.size < om.nelmt
    nst = om.nelmt * 27 * 6
    rng = np.random.default_rng(3)
    st0 = -50.0 * rng.random(nst)                            # a stored (initial) stress
    x = 3.0 * I["x"]
    for last in (False, True):
        ev, st, bl = np.zeros(nst), st0.copy(), np.zeros(om.neq + 1)
        vm, sf = np.zeros(om.nnode), np.full(om.nnode, 1e32)
        fo = om.stress_update(x, *I["props"], I["dt"], 0, int(last), ev, st, bl, elist=elist, form=1, vmeps=vm,
                              scf=sf)
        evg, stg, blg = np.zeros(nst), st0.copy(), np.zeros(om.neq + 1)
        vmg, sfg = np.zeros(om.nnode), np.full(om.nnode, 1e32)
        fg = _gpu_pass(om, I, x, False, last, evg, stg, blg, elmt_list=elist, wpressure=wp, form=1, vmeps=vmg,
                       scf=sfg)
        assert fo > 0 and abs(fg - fo) <= 1e-12 * fo
        assert np.abs(evg - ev).max() <= PASS_MAX_TOL * np.abs(ev).max() and rel(evg, ev) <= PASS_L2_TOL
        assert np.abs(stg - st).max() <= PASS_MAX_TOL * np.abs(st).max()
        if last:
            assert np.array_equal(blg, np.zeros_like(blg))
            touched = sf < 1e32
            assert np.array_equal(sfg < 1e32, touched) and (~touched).any()
            np.testing.assert_allclose(sfg[touched], sf[touched], rtol=1e-9)
            assert np.abs(vmg - vm).max() <= PASS_MAX_TOL * np.abs(vm).max()
        else:
            assert rel(blg, bl) <= PASS_L2_TOL
