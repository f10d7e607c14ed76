"""Known-answer checks that pin the CPU oracle (no GPU).

The reference ships no tests or golden outputs and cannot be compiled here,
so the oracle is pinned by analytic answers: the NGLL=3 GLL tables, the
element matrix's rigid-body null space and symmetry, the exact confined
gravity column, the exact stress of an affine displacement on distorted
elements, the overburden closed form, stress invariants at the Lode corners
and Mohr-Coulomb yield values computed by hand.
"""
import json
import math
import os

import numpy as np
import pytest

from oracle import pyoracle
from oracle.pyoracle import OracleModel
from specfem3d_geotech_gb300 import meshgen

L = pyoracle.lib()


def tables():
    w = np.zeros(27)
    dl = np.zeros(3 * 27 * 27)
    ds = np.zeros(3 * 8 * 27)
    gn = np.zeros(8, np.int32)
    fc = np.zeros(54, np.int32)
    L.orc_tables(w, dl, ds, gn, fc)
    return w, dl.reshape(3, 27, 27), ds.reshape(3, 8, 27), gn, fc.reshape(6, 9)


def test_gll_weights_and_derivatives():
    w, dl, ds, gn, fc = tables()
    w1 = np.array([1 / 3, 4 / 3, 1 / 3])
    ref = np.einsum("k,j,i->kji", w1, w1, w1).reshape(-1)
    assert np.allclose(w, ref, rtol=0, atol=1e-15)
    assert abs(w.sum() - 8.0) < 1e-14  # volume of the reference cube
    # derivative of the Lagrange basis sums to zero (partition of unity)
    assert np.abs(dl.sum(axis=2)).max() < 1e-14
    # d/dxi of the hex8 shape functions sums to zero at every GLL point
    assert np.abs(ds.sum(axis=1)).max() < 1e-14
    assert gn.tolist() == [0, 2, 8, 6, 18, 20, 26, 24]
    # Exodus faces: 1 y-min, 2 x-max, 3 y-max, 4 x-min, 5 z-min, 6 z-max
    assert fc[4].tolist() == list(range(9)) and fc[5].tolist() == list(range(18, 27))
    assert fc[3].tolist() == [0, 3, 6, 9, 12, 15, 18, 21, 24]


def test_cmat_closed_form():
    c = np.zeros(36)
    E, nu = 1e5, 0.3
    L.orc_cmat(E, nu, c)
    c = c.reshape(6, 6)
    lam = E * nu / ((1 + nu) * (1 - 2 * nu))
    mu = E / (2 * (1 + nu))
    ref = np.zeros((6, 6))
    ref[:3, :3] = lam
    ref[np.arange(3), np.arange(3)] = lam + 2 * mu
    ref[np.arange(3, 6), np.arange(3, 6)] = mu
    assert np.allclose(c, ref, rtol=1e-14)


def inv(s):
    out = np.zeros(3)
    L.orc_stress_invariant(np.asarray(s, np.float64), out)
    return out


def test_stress_invariants_corners():
    # hydrostatic: J2 clamped to 1e-12, theta = asin(0)/3 = 0
    sigm, dsbar, th = inv([-5, -5, -5, 0, 0, 0])
    assert sigm == -5 and abs(dsbar - math.sqrt(3e-12)) < 1e-18 and th == 0.0
    # one principal stress above two equal ones: sin(3 theta) = -1, theta = -30 deg
    # (tension positive, Smith & Griffiths' convention)
    sigm, dsbar, th = inv([-10, -20, -20, 0, 0, 0])
    assert abs(sigm + 50 / 3) < 1e-12
    assert abs(dsbar - 10.0) < 1e-12
    assert abs(th + math.pi / 6) < 1e-7
    # one principal stress below two equal ones: theta = +30 deg
    sigm, dsbar, th = inv([-20, -10, -10, 0, 0, 0])
    assert abs(th - math.pi / 6) < 1e-7
    # pure shear: theta = 0
    sigm, dsbar, th = inv([0, 0, 0, 7, 0, 0])
    assert abs(th) < 1e-12 and abs(dsbar - math.sqrt(3) * 7) < 1e-12


def test_mohr_coulomb_hand_values():
    phi, c = 30.0, 10.0
    sigm, dsbar, th = -20.0, 15.0, 0.1
    f = L.orc_mohcouf(phi, c, sigm, dsbar, th)
    sp, cp = math.sin(math.radians(phi)), math.cos(math.radians(phi))
    ref = sp * sigm + dsbar * (math.cos(th) / math.sqrt(3) - math.sin(th) * sp / 3) - c * cp
    assert abs(f - ref) < 1e-12
    # potential derivatives: smooth branch and corner branch (|sin theta| > 0.49)
    dq = np.zeros(3)
    L.orc_mohcouq(0.0, 12.0, 0.2, dq)
    assert dq[0] == 0.0 and dq[1] > 0 and dq[2] != 0.0
    L.orc_mohcouq(10.0, 12.0, math.asin(0.5) + 1e-3, dq)
    sq3 = math.sqrt(3)
    sps = math.sin(math.radians(10.0))
    assert dq[2] == 0.0
    assert abs(dq[1] - (sq3 * 0.5 - sps * 0.5 / sq3) * sq3 * 0.5 / 12.0) < 1e-15
    m = np.zeros(108)
    L.orc_formm(np.array([-3.0, -2.0, -1.0, 0.5, 0.2, -0.1]), m)
    m = m.reshape(3, 6, 6)
    for a in m:
        assert np.allclose(a, a.T, atol=0)


def test_element_matrix_rigid_body_and_symmetry():
    mesh = meshgen.slope2d()
    om = OracleModel(mesh)
    km, dp, ext = om.stiffness_bodyload()
    arr = om.arrays()
    K = km[7].T  # [row, col]
    coords = arr["g_coord"][arr["g_num"][7]]
    scale = np.abs(K).max()
    assert np.abs(K - K.T).max() <= 1e-12 * scale
    modes = []
    for d in range(3):
        v = np.zeros((27, 3)); v[:, d] = 1; modes.append(v.reshape(-1))
    for a, b in ((0, 1), (1, 2), (2, 0)):
        v = np.zeros((27, 3)); v[:, a] = -coords[:, b]; v[:, b] = coords[:, a]; modes.append(v.reshape(-1))
    for v in modes:
        assert np.abs(K @ v).max() <= 1e-10 * scale * np.abs(v).max()
    ev = np.linalg.eigvalsh(0.5 * (K + K.T))
    assert ev.min() >= -1e-10 * scale
    assert (ev > 1e-8 * scale).sum() == 81 - 6
    # GLL structural zeros: nodes differing in all three lattice indices
    n, m = 0, 26
    assert np.all(K[3 * n:3 * n + 3, 3 * m:3 * m + 3] == 0.0)


def test_confined_gravity_column_exact():
    """1x1xn column, laterally confined, base fixed: u_z(z) = -g(Hz - z^2/2)/M."""
    E, nu, gam, H, n = 1e5, 0.3, 20.0, 4.0, 4
    mesh = meshgen.column(n=n, H=H, E=E, nu=nu, gam=gam)
    om = OracleModel(mesh)
    r = om.trial(1.0, want_x=True, want_stress=True)
    assert r["errcode"] == 0
    arr = om.arrays()
    M = E * (1 - nu) / ((1 + nu) * (1 - 2 * nu))
    z = arr["g_coord"][:, 2]
    uz_exact = -gam * (H * z - z * z / 2) / M
    g = arr["gdof"][:, 2]
    uz = np.where(g > 0, r["x"][g], 0.0)
    assert np.abs(uz - uz_exact).max() <= 1e-9 * np.abs(uz_exact).max()
    szz = r["stress"][..., 2]
    zp = arr["g_coord"][arr["g_num"], 2]
    assert np.abs(szz - (-gam * (H - zp))).max() <= 1e-8 * gam * H


def test_golden_trials_reproduce():
    """The committed oracle fixture for the 300-element slope is reproduced."""
    path = os.path.join(os.path.dirname(__file__), "golden", "slope2d_trials.json")
    if not os.path.exists(path):
        pytest.skip("fixture not generated")
    with open(path) as f:
        gold = json.load(f)
    om = OracleModel(meshgen.slope2d())
    g = gold["trials"][0]
    r = om.trial(g["srf"], want_log=True)
    assert r["nl_iter"] == g["nl_iter"] and r["cg_tot"] == g["cg_tot"]
    assert r["nl_cg"].tolist() == g["nl_cg"]
    assert abs(r["umax"] - g["umax"]) <= 1e-12 * g["umax"]


def test_golden_sweep_bracket():
    path = os.path.join(os.path.dirname(__file__), "golden", "slope2d_sweep.json")
    if not os.path.exists(path):
        pytest.skip("fixture not generated")
    with open(path) as f:
        gold = json.load(f)
    rows = gold["trials"]
    assert rows[-1]["failed"] == 1 and all(r["failed"] == 0 for r in rows[:-1])
    assert gold["critical_srf"] == rows[-1]["srf"]
    # plastic iterations grow towards failure
    nl = [r["nl_iter"] for r in rows[:-1]]
    assert nl == sorted(nl)


def test_pcg_rounding_noise_floor():
    """Summation order alone moves a cg_tol = 1e-8 PCG solve by ~5e-9 (relative L2).

    This bounds how closely any reimplementation can match the reference in
    FP64: the GPU parity tests use 1e-8, not a tighter figure.
    """
    om = OracleModel(meshgen.slope2d())
    km, dp, ext = om.stiffness_bodyload()
    dinv = np.where(np.arange(om.neq + 1) > 0, 1.0 / np.where(dp == 0, 1, dp), 0.0)
    ge = om.arrays()["gdof_elmt"]
    sol = []
    try:
        for order in (0, 1):
            L.orc_set_dot_order(order)
            u = np.zeros(om.neq + 1)
            err, it = pyoracle.pcg_solver(om.neq, om.nelmt, km, u, ext, dinv, ge, 5000, 1e-8)
            assert err == 0
            sol.append((u, it))
    finally:
        L.orc_set_dot_order(0)
    d = np.linalg.norm(sol[0][0] - sol[1][0]) / np.linalg.norm(sol[0][0])
    assert 1e-10 < d < 1e-8
    assert abs(sol[0][1] - sol[1][1]) <= 2


def test_trial_rounding_noise_floor():
    """How far rounding alone moves a plastic trial: only the dot-product
    summation order of the oracle changes (sequential, pairwise, strided
    partial sums, reverse).  At SRF 1.0 (12 plastic iterations) x moves by
    ~2e-8 and stress by < 1e-6; at SRF 1.1 (22 plastic iterations) some orders
    flip the yield decision of a GLL point near F = 0 and move the converged
    stress by 8.7e-6 (fmax by up to 8e-4) while x stays within 4e-8."""
    om = OracleModel(meshgen.slope2d())
    try:
        for srf, orders, ds_max in ((1.0, (1, 2, 3), 1e-6), (1.1, (1, 3, 128, 164), 1e-5)):
            L.orc_set_dot_order(0)
            a = om.trial(srf, want_x=True, want_stress=True)
            spread = []
            for order in orders:
                L.orc_set_dot_order(order)
                b = om.trial(srf, want_x=True, want_stress=True)
                assert a["nl_iter"] == b["nl_iter"]
                dx = np.linalg.norm(a["x"] - b["x"]) / np.linalg.norm(a["x"])
                assert 1e-10 < dx < 5e-8
                spread.append(np.abs(a["stress"] - b["stress"]).max() / np.abs(a["stress"]).max())
            assert max(spread) < ds_max
            if srf == 1.1:
                assert max(spread) > 5e-6     # the yield-flip mode is reached by some orders
    finally:
        L.orc_set_dot_order(0)

def _node_dofs(om):
    """(x, y, z) dof numbers of every element node with all three dofs free."""
    ge = np.asarray(om.arrays()["gdof_elmt"]).reshape(om.nelmt, 27, 3)
    rows = {tuple(r) for r in ge.reshape(-1, 3).tolist() if min(r) > 0}
    return np.array(sorted(rows))


def test_pseudo_static_load_known_answer():
    """The pseudo-static load of src/preprocess.f90:137-143 puts eqk * gamma *
    w detJ on each node and direction, beside the gravity load -gamma * w detJ
    on the z dof: on every fully free node the x, y and z loads are -eqkx,
    -eqky and (1 - eqkz) times the gravity-only z load."""
    mesh = meshgen.slope2d()
    _, _, g0 = OracleModel(mesh).stiffness_bodyload()
    om = OracleModel(mesh)
    om.set_eqload(0.1, 0.05, 0.02)
    _, _, g1 = om.stiffness_bodyload()
    dofs = _node_dofs(om)
    gz = g0[dofs[:, 2]]
    assert np.all(gz < 0)
    np.testing.assert_allclose(g1[dofs[:, 0]], -0.1 * gz, rtol=1e-12)
    np.testing.assert_allclose(g1[dofs[:, 1]], -0.05 * gz, rtol=1e-12)
    np.testing.assert_allclose(g1[dofs[:, 2]], 0.98 * gz, rtol=1e-12)
    assert np.all(g0[dofs[:, 0]] == 0) and np.all(g0[dofs[:, 1]] == 0)


def _free_distorted_box(seed=11):
    """2x2x2 box with its interior and top nodes moved (valid, non-parallelepiped
    elements) and no constraints, so every node carries three free dofs."""
    mesh = meshgen.box(nx=2, ny=2, nz=2, L=2.0, W=2.0, zbot=0.0, ztop=2.0,
                       props=(20.0, 1e5, 0.3, 30.0, 1e9, 0.0))
    rng = np.random.default_rng(seed)
    move = mesh.z > 0.5
    for a in (mesh.x, mesh.y, mesh.z):
        a[move] += rng.uniform(-0.15, 0.15, move.sum())
    mesh.bc = [np.zeros((0, 2), np.int32) for _ in range(3)]
    return mesh


def _affine_x(om, A, b):
    a = om.arrays()
    x = np.zeros(om.neq + 1)
    u = a["g_coord"] @ A.T + b
    x[a["gdof"].reshape(-1)] = u.reshape(-1)
    return x


def test_affine_displacement_gives_exact_elastic_stress():
    """u = A X + b: a trilinear-mapped 27-node element reproduces it exactly,
    so every GLL point of every (distorted) element has the strain sym(A) in
    the reference's order (xx yy zz, engineering xy yz zx) and sigma = C eps
    (src/postprocess.f90:40-79, src/preprocess.f90:12-68)."""
    mesh = _free_distorted_box()
    om = OracleModel(mesh)
    assert om.neq == 3 * om.nnode
    rng = np.random.default_rng(5)
    A = 1e-3 * rng.standard_normal((3, 3))
    x = _affine_x(om, A, np.array([0.1, -0.2, 0.05]))
    eps = np.array([A[0, 0], A[1, 1], A[2, 2], A[0, 1] + A[1, 0], A[1, 2] + A[2, 1], A[2, 0] + A[0, 2]])
    E, nu = 1e5, 0.3
    f = E / ((1 + nu) * (1 - 2 * nu))
    C = np.zeros((6, 6))
    C[:3, :3] = f * nu
    np.fill_diagonal(C[:3, :3], f * (1 - nu))
    C[3:, 3:] = np.eye(3) * E / (2 * (1 + nu))
    sig = C @ eps
    st = np.zeros(om.nelmt * 27 * 6)
    L.orc_elastic_stress(om.h, x, st)
    np.testing.assert_allclose(st.reshape(-1, 6), np.broadcast_to(sig, (om.nelmt * 27, 6)),
                               rtol=0, atol=1e-10 * np.abs(sig).max())
    # the plastic block stores the same stress when nothing yields (c = 1e9):
    # no plastic strain, no body load, fmax = 0
    ev, st2, bl = np.zeros_like(st), np.zeros_like(st), np.zeros(om.neq + 1)
    p = mesh.props[0]
    fmax = om.stress_update(x, [p[1]], [p[2]], [p[3]], [p[4]], [p[5]], 1e-5, 1, 1, ev, st2, bl)
    assert fmax == 0.0 and not ev.any() and not bl.any()
    np.testing.assert_allclose(st2, st, rtol=0, atol=1e-12 * np.abs(sig).max())


def test_overburden_stress_closed_form():
    """sigma_zz = p0 - gamma |z - z0|, sigma_xx = sigma_yy = k0 sigma_zz at each
    GLL point's node (src/postprocess.f90:10-33)."""
    mesh = meshgen.excavation(nx=4, ny=4, nz=3, L=8.0, H=6.0, pit=4.0, lifts=1, lift_h=2.0)
    om = OracleModel(mesh)
    a = om.arrays()
    st = np.zeros(om.nelmt * 27 * 6)
    L.orc_overburden_stress(om.h, 6.0, -5.0, 0.5, st)
    z = a["g_coord"][a["g_num"], 2]                              # (nelmt, 27)
    gam = mesh.props[a["mat_id"] - 1, 0][:, None]
    szz = -5.0 - gam * np.abs(z - 6.0)
    st = st.reshape(om.nelmt, 27, 6)
    assert np.array_equal(st[..., 2], szz)
    assert np.array_equal(st[..., 0], 0.5 * szz) and np.array_equal(st[..., 1], 0.5 * szz)
    assert not st[..., 3:].any()


def test_strength_reduction_and_time_step_closed_form():
    """c/SRF, atan(tan(phi)/SRF), atan(tan(psi)/SRF); the phi-nu correction of
    Zheng et al. (2005) only where sin(phif) < 1 - 2 nu; dt = 4 (1+nu)(1-2nu) /
    (E (1 - 2nu + sin^2 phif)) minimised over blocks
    (src/plastic_library.f90:17-88)."""
    from oracle.pyoracle import dt_viscoplas, strength_reduction
    coh = np.array([10.0, 25.0, 5.0])
    nu = np.array([0.3, 0.45, 0.2])
    phi = np.array([20.0, 30.0, 40.0])
    psi = np.array([0.0, 10.0, 5.0])
    ym = np.array([1e5, 5e4, 2e5])
    srf = 1.6
    d = math.pi / 180.0
    ist, cohf, nuf, phif, psif = strength_reduction(srf, coh, nu, phi, psi)
    assert ist == 0 and np.array_equal(nuf, nu)
    np.testing.assert_allclose(cohf, coh / srf, rtol=1e-15)
    np.testing.assert_allclose(phif, np.degrees(np.arctan(np.tan(phi * d) / srf)), rtol=1e-14)
    np.testing.assert_allclose(psif, np.degrees(np.arctan(np.tan(psi * d) / srf)), rtol=1e-14, atol=1e-15)
    # unit SRF leaves everything unchanged
    ist1, c1, n1, p1, q1 = strength_reduction(1.0, coh, nu, phi, psi)
    assert ist1 == 0 and np.array_equal(c1, coh) and np.array_equal(p1, phi) and np.array_equal(q1, psi)
    # phi-nu correction: blocks 0 and 2 have sin(phif) < 1 - 2 nu and are corrected,
    # block 1 (nu = 0.45, 1 - 2 nu = 0.1) is not
    ist2, _, nu2, phif2, _ = strength_reduction(srf, coh, nu, phi, psi, phinu=1)
    assert ist2 == 1 and nu2[1] == nu[1] and nu2[0] != nu[0] and nu2[2] != nu[2]
    for b in range(3):
        om2 = 1 - 2 * nu[b]
        snf = math.sin(phif2[b] * d)
        if snf < om2:
            beta = max(math.sin(phi[b] * d) / om2, 1.0 + 1e-12)
            assert abs(nu2[b] - 0.5 * (1 - snf / beta)) <= 1e-15
        else:
            assert nu2[b] == nu[b]
    assert ist2 == int(any(math.sin(phif2[b] * d) < 1 - 2 * nu[b] for b in range(3)))
    dt = dt_viscoplas(nuf, phif, ym)
    ref = min(4 * (1 + nuf[b]) * (1 - 2 * nuf[b]) / (ym[b] * (1 - 2 * nuf[b] + math.sin(phif[b] * d) ** 2))
              for b in range(3))
    assert abs(dt - ref) <= 1e-15 * ref


def test_reference_excavation_1d_deck_uplift_closed_form():
    """The reference's own excavation_1d deck (tests/golden/decks): a 20 x 100
    x 40 m block with its sides held normal and its base fixed, all-elastic,
    overburden initial stress from z0 = 40 (gamma = 1, E = 1e4, nu = 0.2), and
    the top 20 m (material 2) removed in one stage.  The release load is the
    overburden on the new surface, gamma * 20, and the laterally confined
    20 m column left below heaves by gamma * h * H / M with the constrained
    modulus M = E (1 - nu) / ((1 + nu)(1 - 2 nu)): 20 * 20 / 11111.1 =
    0.036 m.  The oracle, reading the deck as the reference does, gives it."""
    import specfem3d_geotech_gb300 as sg
    deck = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "decks", "excavation_1d.sem")
    d = sg.read_deck(deck)
    om = OracleModel(deck=deck)
    rows = om.excavation(int(d["s0_type"]), float(d["z0"]), float(d["s0"]), float(d["k0"]),
                         [int(v) for v in d["excavid"]], ninc=int(d["ninc"]),
                         nexcavid=[int(v) for v in d["nexcavid"]])
    E, nu, gam, h, H = 1e4, 0.2, 1.0, 20.0, 20.0
    M = E * (1 - nu) / ((1 + nu) * (1 - 2 * nu))
    exact = gam * h * H / M
    assert rows.shape == (1, 8) and rows[0, 6] == 0
    assert abs(rows[0, 4] - exact) <= 1e-9 * exact, (rows[0, 4], exact)
