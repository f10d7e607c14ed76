"""slope3d's plastic loop for one SRF (src/slope.F90:244-392) written out on
the host around two callables: the pcg_solver contract and the stress /
body-load block.  The tests run it with the oracle's routines and with the
GPU drop-ins (sg_pcg_solve, sg_stress_bodyload)."""
import numpy as np

from oracle.pyoracle import dt_viscoplas, strength_reduction


def host_trial(om, mesh, srf, pcg, stress_pass):
    """slope3d's body for one SRF with the solve and the stress block as callables."""
    c = mesh.control
    gam, ym, nu, phi, coh, psi = (mesh.props[:, i] for i in range(6))
    _, cohf, nuf, phif, psif = strength_reduction(srf, coh, nu, phi, psi)
    dt = dt_viscoplas(nuf, phif, ym)
    km, dp, ext = om.stiffness_bodyload()
    dpi = np.zeros_like(dp)
    dpi[1:] = 1.0 / dp[1:]
    n1 = om.neq + 1
    x, oldx, bodyload = np.zeros(n1), np.zeros(n1), np.zeros(n1)
    nst = om.nelmt * 27 * 6
    evpt, stress = np.zeros(nst), np.zeros(nst)
    ge = om.arrays()["gdof_elmt"]
    for nl_iter in range(1, c.nl_maxiter + 1):
        load = ext + bodyload
        load[0] = 0.0
        err, _ = pcg(om.neq, om.nelmt, km, x, load, dpi, ge, c.cg_maxiter, c.cg_tol)
        assert err == 0
        x[0] = 0.0
        uerr = np.abs(x - oldx).max() / np.abs(x).max()
        oldx = x.copy()
        conv = uerr <= c.nl_tol
        last = conv or nl_iter == c.nl_maxiter
        fmax = stress_pass(x, ym, nuf, phif, cohf, psif, dt, conv, last, evpt, stress, bodyload)
        if last:
            break
    return dict(nl_iter=nl_iter, converged=int(conv), x=x, stress=stress, fmax=fmax)
