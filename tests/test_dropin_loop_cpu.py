"""The reference's plastic loop (src/slope.F90:280-392) written out on the
host around the two drop-in routines -- pcg_solver and the stress / body-load
block -- reproduces the oracle's own trial bit for bit.  This pins the
oracle's single-pass entry (orc_stress_update) that the GPU drop-in
sg_stress_bodyload is checked against."""
import numpy as np

from dropin_loop import host_trial
from oracle.pyoracle import OracleModel, dt_viscoplas, pcg_solver, strength_reduction
from specfem3d_geotech_gb300 import meshgen


def test_host_loop_equals_oracle_trial():
    mesh = meshgen.slope2d(srf=(1.0,))
    om = OracleModel(mesh)
    r = host_trial(om, mesh, 1.0, pcg_solver, om.stress_update)
    ro = om.trial(1.0, want_x=True, want_stress=True)
    assert r["nl_iter"] == ro["nl_iter"] and r["converged"] == ro["converged"] == 1
    assert np.array_equal(r["x"], ro["x"])
    assert np.array_equal(r["stress"], ro["stress"].reshape(-1))
    assert r["fmax"] == ro["fmax"]


def test_element_list_and_forms():
    """An explicit list of all elements in order is the default pass; the
    excavation form adds vmeps/scf when finalising and, without a water table,
    leaves the stress state as the slope form does."""
    mesh = meshgen.slope2d(srf=(1.0,))
    om = OracleModel(mesh)
    gam, ym, nu, phi, coh, psi = (mesh.props[:, i] for i in range(6))
    _, cohf, nuf, phif, psif = strength_reduction(1.3, coh, nu, phi, psi)
    dt = dt_viscoplas(nuf, phif, ym)
    km, dp, ext = om.stiffness_bodyload()
    dpi = np.zeros_like(dp)
    dpi[1:] = 1.0 / dp[1:]
    x = np.zeros(om.neq + 1)
    c = mesh.control
    pcg_solver(om.neq, om.nelmt, km, x, ext, dpi, om.arrays()["gdof_elmt"], c.cg_maxiter, c.cg_tol)
    nst = om.nelmt * 27 * 6
    outs = []
    for elist, form in ((None, 0), (np.arange(1, om.nelmt + 1), 0), (None, 1)):
        ev, st, bl = np.zeros(nst), np.zeros(nst), np.zeros(om.neq + 1)
        vm, sf = np.zeros(om.nnode), np.full(om.nnode, 1e32)
        f1 = om.stress_update(x, ym, nuf, phif, cohf, psif, dt, 0, 0, ev, st, bl, elist=elist, form=form)
        f2 = om.stress_update(x, ym, nuf, phif, cohf, psif, dt, 0, 1, ev, st, bl, elist=elist, form=form,
                              vmeps=vm, scf=sf)
        outs.append((f1, f2, ev, st, bl, vm, sf))
    for o in outs[1:]:
        for a, b in zip(outs[0][:5], o[:5]):
            assert np.array_equal(a, b)
    assert outs[0][1] > 0.0 and (outs[0][2] != 0).any()
    assert np.array_equal(outs[0][5], np.zeros(om.nnode))     # slope form: untouched
    assert (outs[2][5] > 0).any() and (outs[2][6] < 1e32).all()  # excavation form: accumulated
