"""ctypes wrapper of the CPU oracle (oracle/sg_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()``
and by the CPU-baseline leg of ``bench.py``, always as the checker.  The
product never imports this module.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libsg_oracle.so")
_lib = None

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (a few seconds)."""
    src = os.path.join(_HERE, "sg_oracle.cpp")
    if force or not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(_LIB_PATH)
        vp, i, d = C.c_void_p, C.c_int, C.c_double
        L.orc_model_from_hex8.restype = vp
        L.orc_model_from_hex8.argtypes = [i, _dp, _dp, _dp, i, _ip, _ip, i, _dp, _ip, _ip]
        L.orc_model_from_deck.restype = vp
        L.orc_model_from_deck.argtypes = [C.c_char_p]
        L.orc_free.argtypes = [vp]
        L.orc_set_dot_order.argtypes = [i]
        L.orc_model_sizes.argtypes = [vp, _ip]
        L.orc_model_arrays.argtypes = [vp, vp, vp, vp, vp, vp]
        L.orc_model_control.argtypes = [vp, _dp, _ip, vp]
        L.orc_set_control.argtypes = [vp, d, i, d, i, i, i]
        L.orc_stiffness_bodyload.argtypes = [vp, _dp, _dp, _dp]
        L.orc_set_eqload.argtypes = [vp, d, d, d]
        L.orc_set_water.restype = i
        L.orc_set_water.argtypes = [vp, _ip, i, C.c_char_p, C.c_char_p]
        L.orc_pore_pressure.restype = i
        L.orc_pore_pressure.argtypes = [vp, vp, vp]
        L.orc_nodal_stress.argtypes = [vp, _dp, _dp]
        L.orc_principal_stress.argtypes = [i, _dp, _dp, _dp, _dp]
        L.orc_pcg_solver.restype = i
        L.orc_pcg_solver.argtypes = [i, i, _dp, _dp, _dp, _dp, _ip, i, d, C.POINTER(C.c_int)]
        L.orc_pcg_solver_gpu_order.restype = i
        L.orc_pcg_solver_gpu_order.argtypes = [i, i, _dp, _dp, _dp, _dp, _ip, i, d, C.POINTER(C.c_int)]
        L.orc_ebe_apply.argtypes = [i, i, _dp, _dp, _ip, _dp]
        L.orc_stress_update.restype = d
        L.orc_stress_update.argtypes = [vp, vp, i, i, _dp, _dp, _dp, _dp, _dp, _dp, d, i, i, _dp, _dp, _dp, vp,
                                        vp]
        L.orc_elastic_stress.argtypes = [vp, _dp, _dp]
        L.orc_overburden_stress.argtypes = [vp, d, d, d, _dp]
        L.orc_strength_reduction.restype = i
        L.orc_strength_reduction.argtypes = [d, i, i, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp]
        L.orc_dt_viscoplas.restype = d
        L.orc_dt_viscoplas.argtypes = [i, _dp, _dp, _dp]
        L.orc_slope_trial.argtypes = [vp, d, _dp, vp, vp, vp]
        L.orc_last_uerr_log.restype = i
        L.orc_last_uerr_log.argtypes = [vp, vp]
        L.orc_slope_sweep.restype = i
        L.orc_slope_sweep.argtypes = [vp, i, _dp, _dp]
        L.orc_fos_bisection.restype = d
        L.orc_fos_bisection.argtypes = [vp, d, d, d, C.POINTER(C.c_int)]
        L.orc_tables.argtypes = [_dp, _dp, _dp, _ip, _ip]
        L.orc_cmat.argtypes = [d, d, _dp]
        L.orc_stress_invariant.argtypes = [_dp, _dp]
        L.orc_mohcouf.restype = d
        L.orc_mohcouf.argtypes = [d, d, d, d, d]
        L.orc_mohcouq.argtypes = [d, d, d, _dp]
        L.orc_formm.argtypes = [_dp, _dp]
        L.orc_excavation.restype = i
        L.orc_excavation.argtypes = [vp, i, d, d, d, i, _ip, _ip, i, d, _dp, vp, vp, vp]
        _lib = L
    return _lib


TRIAL_KEYS = ("srf", "cg_tot", "nl_iter", "converged", "failed", "uxmax", "umax", "fmax", "uerr", "errcode")


class OracleModel:
    """A spectral mesh held by the oracle (hex2spec + apply_bc done in C++)."""

    def __init__(self, mesh=None, deck: str | None = None):
        L = lib()
        if deck is not None:
            self.h = L.orc_model_from_deck(deck.encode())
            if not self.h:
                raise FileNotFoundError(deck)
        else:
            bc_counts = np.array([b.shape[0] for b in mesh.bc], np.int32)
            bc_pairs = np.ascontiguousarray(np.concatenate(mesh.bc).astype(np.int32).reshape(-1))
            self.h = L.orc_model_from_hex8(
                mesh.nnode8, np.ascontiguousarray(mesh.x, np.float64), np.ascontiguousarray(mesh.y, np.float64),
                np.ascontiguousarray(mesh.z, np.float64), mesh.nelmt,
                np.ascontiguousarray(mesh.conn.reshape(-1), np.int32),
                np.ascontiguousarray(mesh.mat_id, np.int32), mesh.props.shape[0],
                np.ascontiguousarray(mesh.props.reshape(-1), np.float64), bc_counts, bc_pairs)
            c = mesh.control
            L.orc_set_control(self.h, c.cg_tol, c.cg_maxiter, c.nl_tol, c.nl_maxiter, c.phinu, c.allelastic)
        s = np.zeros(5, np.int32)
        L.orc_model_sizes(self.h, s)
        self.nnode, self.nelmt, self.neq, self.nmatblk, self.nsrf = (int(v) for v in s)

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_free(self.h)
            self.h = None

    def nodal_stress(self, stress_elmt):
        """Valency-averaged nodal stress [nnode][6] (src/slope.F90:419-437)."""
        st = np.ascontiguousarray(stress_elmt, np.float64).reshape(-1)
        out = np.zeros(6 * self.nnode)
        lib().orc_nodal_stress(self.h, st, out)
        return out.reshape(-1, 6)

    def set_eqload(self, eqkx, eqky, eqkz):
        """Pseudo-static earthquake load factors (src/preprocess.f90:137-143)."""
        lib().orc_set_eqload(self.h, eqkx, eqky, eqkz)

    def set_water(self, water_ids, wsfile: str):
        """Water table from a water-surface file and the water material IDs
        (src/compute_pressure.f90:10-186); raises RuntimeError with the
        reference's message when the pressure cannot be computed."""
        ids = np.ascontiguousarray(np.asarray(water_ids, np.int32).reshape(-1))
        tag = C.create_string_buffer(251)
        st = lib().orc_set_water(self.h, ids if ids.size else np.zeros(1, np.int32), int(ids.size),
                                 str(wsfile).encode(), tag)
        if st != 0:
            raise RuntimeError(tag.value.decode().strip())

    def pore_pressure(self):
        """(wpressure[nnode], submerged[nnode]) of the water table, or None."""
        wp = np.zeros(self.nnode)
        sub = np.zeros(self.nnode, np.int32)
        if lib().orc_pore_pressure(self.h, wp.ctypes.data, sub.ctypes.data) != 0:
            return None
        return wp, sub.astype(bool)

    def stress_update(self, x, ymf, nuf, phif, cohf, psif, dt, nl_isconv, last, evpt, stress, bodyload,
                      elist=None, form=0, vmeps=None, scf=None):
        """One pass of the stress / yield / flow / body-load block
        (src/slope.F90:311-383, src/excavation.F90:546-616); evpt, stress,
        bodyload (and vmeps, scf) are float64 arrays updated in place.
        Returns fmax."""
        el = None if elist is None else np.ascontiguousarray(elist, np.int32)
        f = lambda a: np.ascontiguousarray(a, np.float64)
        return lib().orc_stress_update(
            self.h, None if el is None else el.ctypes.data, 0 if el is None else int(el.size), int(form), f(x),
            f(ymf), f(nuf), f(phif), f(cohf), f(psif), float(dt), int(nl_isconv), int(last), evpt, stress, bodyload,
            None if vmeps is None else vmeps.ctypes.data, None if scf is None else scf.ctypes.data)

    def set_control(self, cg_tol, cg_maxiter, nl_tol, nl_maxiter, phinu=0, allelastic=0):
        lib().orc_set_control(self.h, cg_tol, cg_maxiter, nl_tol, nl_maxiter, phinu, allelastic)

    def control(self):
        dc = np.zeros(2)
        ic = np.zeros(4, np.int32)
        srf = np.zeros(max(self.nsrf, 1))
        lib().orc_model_control(self.h, dc, ic, srf.ctypes.data)
        return dict(cg_tol=dc[0], nl_tol=dc[1], cg_maxiter=int(ic[0]), nl_maxiter=int(ic[1]),
                    phinu=int(ic[2]), allelastic=int(ic[3]), srf=srf[: self.nsrf])

    def arrays(self):
        g_coord = np.zeros(3 * self.nnode)
        g_num = np.zeros(27 * self.nelmt, np.int32)
        gdof = np.zeros(3 * self.nnode, np.int32)
        gdof_elmt = np.zeros(81 * self.nelmt, np.int32)
        mat_id = np.zeros(self.nelmt, np.int32)
        lib().orc_model_arrays(self.h, g_coord.ctypes.data, g_num.ctypes.data, gdof.ctypes.data,
                               gdof_elmt.ctypes.data, mat_id.ctypes.data)
        return dict(g_coord=g_coord.reshape(-1, 3), g_num=g_num.reshape(-1, 27), gdof=gdof.reshape(-1, 3),
                    gdof_elmt=gdof_elmt.reshape(-1, 81), mat_id=mat_id)

    def stiffness_bodyload(self):
        km = np.zeros(81 * 81 * self.nelmt)
        dp = np.zeros(self.neq + 1)
        ext = np.zeros(self.neq + 1)
        lib().orc_stiffness_bodyload(self.h, km, dp, ext)
        return km.reshape(self.nelmt, 81, 81), dp, ext  # km[e, col, row]

    def trial(self, srf: float, want_x: bool = False, want_stress: bool = False, want_log: bool = False):
        res = np.zeros(10)
        x = np.zeros(self.neq + 1) if want_x else None
        st = np.zeros(6 * 27 * self.nelmt) if want_stress else None
        nl = np.zeros(self.control()["nl_maxiter"] + 1, np.int32) if want_log else None
        lib().orc_slope_trial(self.h, float(srf), res, None if x is None else x.ctypes.data,
                              None if st is None else st.ctypes.data, None if nl is None else nl.ctypes.data)
        out = dict(zip(TRIAL_KEYS, res.tolist()))
        for k in ("cg_tot", "nl_iter", "converged", "failed", "errcode"):
            out[k] = int(out[k])
        if want_x:
            out["x"] = x
        if want_stress:
            out["stress"] = st.reshape(self.nelmt, 27, 6)
        if want_log:
            out["nl_cg"] = nl[: out["nl_iter"]]
            n = lib().orc_last_uerr_log(self.h, None)
            ue = np.zeros(max(n, 1))
            lib().orc_last_uerr_log(self.h, ue.ctypes.data)
            out["uerr_log"] = ue[:n]
        return out

    def sweep(self, srf):
        srf = np.ascontiguousarray(srf, np.float64)
        res = np.zeros(10 * len(srf))
        n = lib().orc_slope_sweep(self.h, len(srf), srf, res)
        return [dict(zip(TRIAL_KEYS, r)) for r in res.reshape(-1, 10)[:n].tolist()]

    def fos_bisection(self, lo=1.0, hi=3.0, step=0.01):
        nt = C.c_int(0)
        v = lib().orc_fos_bisection(self.h, lo, hi, step, C.byref(nt))
        return v, nt.value

    def excavation(self, s0_type, z0, s0, k0, excavid, ninc=1, srf=1.0, nexcavid=None, want_fields=False):
        """Stage results [stage, cg_tot, nl_tot, uxmax, umax, fmax, failed, errcode]; with
        want_fields also the last stage's nodal vmeps and scf (src/excavation.F90:597-661)."""
        excavid = np.ascontiguousarray(excavid, np.int32)
        nexcav = len(excavid) if nexcavid is None else len(nexcavid)
        nexcavid = np.ones(nexcav, np.int32) if nexcavid is None else np.ascontiguousarray(nexcavid, np.int32)
        res = np.zeros(8 * nexcav)
        vm = np.zeros(self.nnode) if want_fields else None
        sf = np.zeros(self.nnode) if want_fields else None
        n = lib().orc_excavation(self.h, s0_type, z0, s0, k0, nexcav, nexcavid, excavid, ninc, srf, res, None,
                                 None if vm is None else vm.ctypes.data, None if sf is None else sf.ctypes.data)
        if n == -2:
            raise ValueError("excavation stage list passes the end of excavid")
        if want_fields:
            return res.reshape(-1, 8)[:n], vm, sf
        return res.reshape(-1, 8)[:n]


def pcg_solver(neq, nelmt, k, u, f, dprecon, gdof_elmt, cg_maxiter, cg_tol):
    """The reference pcg_solver contract; u is updated in place."""
    it = C.c_int(0)
    err = lib().orc_pcg_solver(neq, nelmt, np.ascontiguousarray(k, np.float64).reshape(-1), u,
                               np.ascontiguousarray(f, np.float64), np.ascontiguousarray(dprecon, np.float64),
                               np.ascontiguousarray(gdof_elmt, np.int32).reshape(-1), cg_maxiter, cg_tol,
                               C.byref(it))
    return err, it.value


def pcg_solver_gpu_order(neq, nelmt, k, u, f, dprecon, gdof_elmt, cg_maxiter, cg_tol):
    """pcg_solver evaluated in the GPU drop-in's order (fused multiply-adds,
    node-by-node gather, grid-shaped dot products); u is updated in place."""
    it = C.c_int(0)
    err = lib().orc_pcg_solver_gpu_order(neq, nelmt, np.ascontiguousarray(k, np.float64).reshape(-1), u,
                                         np.ascontiguousarray(f, np.float64),
                                         np.ascontiguousarray(dprecon, np.float64),
                                         np.ascontiguousarray(gdof_elmt, np.int32).reshape(-1), cg_maxiter, cg_tol,
                                         C.byref(it))
    return err, it.value


def strength_reduction(srf, coh, nu, phi, psi, phinu=0):
    """src/plastic_library.f90:42-88: (istat, cohf, nuf, phif, psif)."""
    f = lambda a: np.ascontiguousarray(a, np.float64)
    n = len(coh)
    cohf, nuf, phif, psif = (np.zeros(n) for _ in range(4))
    ist = lib().orc_strength_reduction(float(srf), int(phinu), n, f(coh), f(nu), f(phi), f(psi), cohf, nuf, phif,
                                       psif)
    return ist, cohf, nuf, phif, psif


def dt_viscoplas(nuf, phif, ym):
    """src/plastic_library.f90:17-39."""
    f = lambda a: np.ascontiguousarray(a, np.float64)
    return lib().orc_dt_viscoplas(len(nuf), f(nuf), f(phif), f(ym))


def principal_stress(stress_global):
    """Oracle of src/postprocess.f90:146-183: (psigma[n][3], taumax[n], nsigma[n])."""
    st = np.ascontiguousarray(stress_global, np.float64).reshape(-1)
    n = st.size // 6
    ps, tm, ns = np.zeros(3 * n), np.zeros(n), np.zeros(n)
    lib().orc_principal_stress(n, st, ps, tm, ns)
    return ps.reshape(n, 3), tm, ns
