"""GB300 solve path of SPECFEM3D_GEOTECH behind a C ABI.

The product is the CUDA library ``_lib/libsg.so`` (sources in ``csrc/``,
declarations in ``include/sg_solver.h``).  This package is a thin ctypes
mirror of that ABI for Python callers and tests:

* :func:`pcg_solver` -- the reference's ``pcg_solver`` contract
  (src/solver.f90:14-79): same arguments, ``u`` updated in place, returns
  ``(cg_iter, errcode, errtag)`` with errcode 0 / -1 like the Fortran.
* :class:`Model` -- a device-resident spectral model built from a hex8 mesh
  or a ``.sem`` deck, with slope3d trials, SRF sweeps, factor-of-safety
  search and staged excavation.

There is no CPU fallback: if the library cannot be loaded or no CUDA device
is present the calls raise.
"""
from __future__ import annotations

import ctypes as C
import math
import os
from typing import Optional, Sequence

import numpy as np

from . import meshgen  # noqa: F401

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libsg.so")
ERRTAG_LEN = 250

SG_OK, SG_ERR_NOCONV, SG_ERR_TIMEOUT, SG_ERR_OOM, SG_ERR_BADARG, SG_ERR_CUDA, SG_ERR_NODEVICE = 0, -1, -2, -3, -4, -5, -6
PREC_FP64, PREC_MIXED = 0, 1

EXPORTED = (
    "sg_create", "sg_create_status", "sg_destroy", "sg_last_error", "sg_hbm_used", "sg_pcg_solve",
    "sg_model_from_hex8", "sg_model_from_deck", "sg_model_free", "sg_model_info", "sg_model_arrays",
    "sg_model_control", "sg_model_stiffness", "sg_model_set_eqload", "sg_model_set_water", "sg_model_set_pore_pressure",
    "sg_model_pore_pressure", "sg_nodal_stress", "sg_excavation_fields",
    "sg_principal_stress", "sg_write_summary_header", "sg_write_summary_row", "sg_write_ensight_case", "sg_write_ensight_geo",
    "sg_write_ensight_var", "sg_srf_trials", "sg_last_stress", "sg_srf_sweep", "sg_fos", "sg_fos_steps",
    "sg_excavation", "sg_profile_enable", "sg_profile_read", "sg_batch_begin", "sg_batch_add", "sg_batch_step",
    "sg_batch_poll", "sg_batch_release", "sg_batch_end", "sg_timer_mark", "sg_timer_ms", "sg_pcg_solve_noalloc", "sg_stress_bodyload", "sg_mesh_from_deck", "sg_mesh_free", "sg_mesh_info",
    "sg_mesh_arrays", "sg_mesh_control",
    "sg_server_create", "sg_server_submit", "sg_server_submit_excavation", "sg_server_stages", "sg_server_wait", "sg_server_stats", "sg_server_destroy",
)


class SgError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[{code}] {msg}")
        self.code = code


class Control(C.Structure):
    """sg_control (include/sg_solver.h)."""

    _fields_ = [("cg_tol", C.c_double), ("nl_tol", C.c_double), ("cg_maxiter", C.c_int), ("nl_maxiter", C.c_int),
                ("phinu", C.c_int), ("allelastic", C.c_int), ("precision", C.c_int), ("reserved", C.c_int),
                ("refine_rtol", C.c_double), ("inner_rtol", C.c_double)]


class FosResult(C.Structure):
    """sg_fos_result (include/sg_solver.h)."""

    _fields_ = [("id", C.c_int), ("status", C.c_int), ("fos", C.c_double), ("ntrials", C.c_int),
                ("nrounds", C.c_int), ("nelmt", C.c_int), ("neq", C.c_int), ("footprint", C.c_double),
                ("hbm_bytes", C.c_double), ("t_arrival", C.c_double), ("t_start", C.c_double),
                ("t_done", C.c_double), ("kind", C.c_int), ("nstage", C.c_int)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class TrialResult(C.Structure):
    """sg_trial_result (include/sg_solver.h)."""

    _fields_ = [("srf", C.c_double), ("cg_tot", C.c_int), ("nl_iter", C.c_int), ("converged", C.c_int),
                ("failed", C.c_int), ("uxmax", C.c_double), ("umax", C.c_double), ("fmax", C.c_double),
                ("uerr", C.c_double), ("errcode", C.c_int), ("refine_steps", C.c_int), ("seconds", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


_lib = None


def lib(path: Optional[str] = None):
    """Load libsg.so (built by ``build.build()``); raises if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise OSError(f"{path} not built: run specfem3d_geotech_gb300.build.build()")
    L = C.CDLL(path)
    vp, i, d, sz = C.c_void_p, C.c_int, C.c_double, C.c_size_t
    L.sg_create.restype = vp
    L.sg_create.argtypes = [i, sz]
    L.sg_create_status.restype = i
    L.sg_destroy.argtypes = [vp]
    L.sg_last_error.restype = C.c_char_p
    L.sg_last_error.argtypes = [vp]
    L.sg_hbm_used.restype = sz
    L.sg_hbm_used.argtypes = [vp]
    L.sg_pcg_solve.restype = i
    L.sg_pcg_solve.argtypes = [vp, i, i, i, vp, vp, vp, vp, vp, i, d, C.POINTER(C.c_int), C.c_char_p]
    L.sg_pcg_solve_noalloc.restype = i
    L.sg_pcg_solve_noalloc.argtypes = [i, i, i, vp, vp, vp, vp, vp, i, d, C.POINTER(C.c_int), C.c_char_p]
    L.sg_mesh_from_deck.restype = vp
    L.sg_mesh_from_deck.argtypes = [C.c_char_p, C.c_char_p]
    L.sg_mesh_free.argtypes = [vp]
    L.sg_mesh_info.restype = i
    L.sg_mesh_info.argtypes = [vp, vp]
    L.sg_mesh_arrays.restype = i
    L.sg_mesh_arrays.argtypes = [vp, vp, vp, vp, vp, vp, vp]
    L.sg_mesh_control.restype = i
    L.sg_mesh_control.argtypes = [vp, vp, vp, vp, vp, vp, vp]
    L.sg_stress_bodyload.restype = i
    L.sg_stress_bodyload.argtypes = [vp, i, i, i, vp, vp, vp, vp, i, vp, vp, vp, vp, vp, d, i, i, vp, i, vp, i, vp,
                                     vp, vp, vp, vp, vp, C.POINTER(C.c_double), C.c_char_p]
    L.sg_model_from_hex8.restype = vp
    L.sg_model_from_hex8.argtypes = [vp, i, vp, vp, vp, i, vp, vp, i, vp, vp, vp, i, C.c_char_p]
    L.sg_model_from_deck.restype = vp
    L.sg_model_from_deck.argtypes = [vp, C.c_char_p, i, C.c_char_p]
    L.sg_model_free.argtypes = [vp]
    L.sg_model_info.restype = i
    L.sg_model_info.argtypes = [vp, vp]
    L.sg_model_arrays.restype = i
    L.sg_model_arrays.argtypes = [vp, vp, vp, vp, vp]
    L.sg_model_control.restype = i
    L.sg_model_control.argtypes = [vp, vp, vp, vp]
    L.sg_model_stiffness.restype = i
    L.sg_model_stiffness.argtypes = [vp, vp, vp, vp]
    L.sg_srf_trials.restype = i
    L.sg_srf_trials.argtypes = [vp, C.POINTER(Control), i, vp, vp, vp]
    L.sg_excavation_fields.restype = i
    L.sg_excavation_fields.argtypes = [vp, vp, vp]
    L.sg_nodal_stress.restype = i
    L.sg_nodal_stress.argtypes = [vp, i, vp]
    L.sg_principal_stress.restype = i
    L.sg_principal_stress.argtypes = [i, vp, vp, vp, vp]
    L.sg_write_summary_header.restype = i
    L.sg_write_summary_header.argtypes = [C.c_char_p, C.POINTER(Control), i]
    L.sg_write_summary_row.restype = i
    L.sg_write_summary_row.argtypes = [C.c_char_p, C.POINTER(TrialResult)]
    L.sg_write_ensight_case.restype = i
    L.sg_write_ensight_case.argtypes = [C.c_char_p, C.c_char_p, i, vp, i]
    L.sg_write_ensight_geo.restype = i
    L.sg_write_ensight_geo.argtypes = [C.c_char_p, i, vp, i, vp]
    L.sg_write_ensight_var.restype = i
    L.sg_write_ensight_var.argtypes = [C.c_char_p, C.c_char_p, i, i, vp]
    L.sg_model_set_eqload.restype = i
    L.sg_model_set_eqload.argtypes = [vp, d, d, d]
    L.sg_model_set_water.restype = i
    L.sg_model_set_water.argtypes = [vp, C.c_char_p, vp, i, C.c_char_p]
    L.sg_model_set_pore_pressure.restype = i
    L.sg_model_set_pore_pressure.argtypes = [vp, vp]
    L.sg_model_pore_pressure.restype = i
    L.sg_model_pore_pressure.argtypes = [vp, vp]
    L.sg_last_stress.restype = i
    L.sg_last_stress.argtypes = [vp, i, vp]
    L.sg_srf_sweep.restype = i
    L.sg_srf_sweep.argtypes = [vp, C.POINTER(Control), i, vp, vp, C.POINTER(C.c_int)]
    L.sg_fos.restype = i
    L.sg_fos.argtypes = [vp, C.POINTER(Control), d, d, d, i, C.POINTER(C.c_double), C.POINTER(C.c_int),
                         C.POINTER(C.c_int)]
    L.sg_fos_steps.restype = i
    L.sg_fos_steps.argtypes = [vp, C.POINTER(C.c_longlong)]
    L.sg_excavation.restype = i
    L.sg_excavation.argtypes = [vp, C.POINTER(Control), i, d, d, d, i, vp, vp, i, d, vp, C.POINTER(C.c_int)]
    L.sg_profile_enable.restype = i
    L.sg_profile_enable.argtypes = [vp, i]
    L.sg_profile_read.restype = i
    L.sg_profile_read.argtypes = [vp, vp, vp]
    L.sg_batch_begin.restype = i
    L.sg_batch_begin.argtypes = [vp, C.POINTER(Control), i]
    L.sg_batch_add.restype = i
    L.sg_batch_add.argtypes = [vp, d, C.POINTER(C.c_int)]
    L.sg_batch_step.restype = i
    L.sg_batch_step.argtypes = [vp, i, C.POINTER(C.c_int)]
    L.sg_batch_poll.restype = i
    L.sg_batch_poll.argtypes = [vp, i, C.POINTER(TrialResult), C.POINTER(C.c_int)]
    L.sg_batch_release.restype = i
    L.sg_batch_release.argtypes = [vp, i]
    L.sg_batch_end.restype = i
    L.sg_batch_end.argtypes = [vp]
    L.sg_server_create.restype = vp
    L.sg_server_create.argtypes = [i, sz, i]
    L.sg_server_submit.restype = i
    L.sg_server_submit.argtypes = [vp, i, vp, vp, vp, i, vp, vp, i, vp, vp, vp, C.POINTER(Control), d, d, d, i,
                                   C.POINTER(C.c_int)]
    L.sg_server_submit_excavation.restype = i
    L.sg_server_submit_excavation.argtypes = [vp, i, vp, vp, vp, i, vp, vp, i, vp, vp, vp, C.POINTER(Control), i, d,
                                              d, d, i, vp, vp, i, d, C.POINTER(C.c_int)]
    L.sg_server_stages.restype = i
    L.sg_server_stages.argtypes = [vp, i, vp]
    L.sg_server_wait.restype = i
    L.sg_server_wait.argtypes = [vp, i, d, C.POINTER(FosResult)]
    L.sg_server_stats.restype = i
    L.sg_server_stats.argtypes = [vp, vp]
    L.sg_server_destroy.argtypes = [vp]
    L.sg_timer_mark.restype = i
    L.sg_timer_mark.argtypes = [vp, i]
    L.sg_timer_ms.restype = d
    L.sg_timer_ms.argtypes = [vp, i, i]
    _lib = L
    return L


def _ptr(a: np.ndarray):
    return a.ctypes.data


class Context:
    """sg_ctx: one CUDA device, one stream, the device memory of its models."""

    def __init__(self, device: int = 0, hbm_budget: int = 0):
        L = lib()
        self.h = L.sg_create(device, hbm_budget)
        if not self.h:
            raise SgError(L.sg_create_status(), "sg_create: no usable CUDA device")

    def close(self):
        if getattr(self, "h", None):
            lib().sg_destroy(self.h)
            self.h = None

    __del__ = close

    @property
    def last_error(self) -> str:
        return lib().sg_last_error(self.h).decode()

    @property
    def hbm_used(self) -> int:
        return int(lib().sg_hbm_used(self.h))

    def mark(self, i: int):
        """Record CUDA event `i` on the context's stream."""
        lib().sg_timer_mark(self.h, i)

    def elapsed_ms(self, a: int, b: int) -> float:
        return float(lib().sg_timer_ms(self.h, a, b))

    def profile(self, on: bool = True):
        lib().sg_profile_enable(self.h, 1 if on else 0)

    def profile_read(self):
        ms = np.zeros(8)
        cnt = np.zeros(4, np.int64)
        lib().sg_profile_read(self.h, _ptr(ms), _ptr(cnt))
        return dict(total_ms=ms[0], apply_ms=ms[1], gather_ms=ms[2], update_ms=ms[3], stress_ms=ms[4],
                    stiffness_ms=ms[5], apply_launches=int(cnt[0]), launches=int(cnt[1]), pcg_iters=int(cnt[2]),
                    refine_residuals=int(cnt[3]))


_default_ctx: Optional[Context] = None


def default_context() -> Context:
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = Context(0)
    return _default_ctx


def pcg_solver(neq: int, nelmt: int, k: np.ndarray, u: np.ndarray, f: np.ndarray, dprecon: np.ndarray,
               gdof_elmt: np.ndarray, cg_maxiter: int, cg_tol: float, ctx: Optional[Context] = None):
    """Drop-in for ``pcg_solver(neq,nelmt,k,u,f,dprecon,gdof_elmt,cg_iter,errcode,errtag)``.

    ``k`` holds the reference's k(81,81,nelmt) (element e's column-major block
    at ``k[e]`` when shaped (nelmt, 81, 81) as [e, col, row]); ``u`` (neq+1,
    float64, C-contiguous) is updated in place; ``gdof_elmt`` is (nelmt, 81)
    int32 with 0 for constrained dofs.  Returns ``(cg_iter, errcode, errtag)``.
    """
    ctx = ctx or default_context()
    if u.dtype != np.float64 or not u.flags.c_contiguous or u.shape[0] != neq + 1:
        raise ValueError("u must be a C-contiguous float64 array of length neq+1")
    k = np.ascontiguousarray(k, np.float64)
    f = np.ascontiguousarray(f, np.float64)
    dprecon = np.ascontiguousarray(dprecon, np.float64)
    ge = np.ascontiguousarray(gdof_elmt, np.int32)
    it = C.c_int(0)
    tag = C.create_string_buffer(ERRTAG_LEN + 1)
    err = lib().sg_pcg_solve(ctx.h, neq, nelmt, 81, _ptr(k), _ptr(u), _ptr(f), _ptr(dprecon), _ptr(ge), cg_maxiter,
                             cg_tol, C.byref(it), tag)
    if err not in (SG_OK, SG_ERR_NOCONV):
        raise SgError(err, tag.value.decode().strip() or ctx.last_error)
    return it.value, err, tag.value.decode().rstrip()


def stress_bodyload(neq: int, nelmt: int, nnode: int, g_coord, g_num, gdof_elmt, mat_id, ym_blk, nuf_blk, phif_blk,
                    cohf_blk, psif_blk, dt: float, nl_isconv: bool, last: bool, x, evpt: np.ndarray,
                    stress_elmt: np.ndarray, bodyload: np.ndarray, elmt_list=None, wpressure=None, form: int = 0,
                    vmeps: Optional[np.ndarray] = None, scf: Optional[np.ndarray] = None,
                    ctx: Optional[Context] = None) -> float:
    """Drop-in for the stress / yield / flow / body-load block of the plastic
    loops (src/slope.F90:311-383, src/excavation.F90:546-616), on the GPU.

    Reference layout and 1-based ids: ``g_num`` (nelmt, 27) nodes 1..nnode,
    ``gdof_elmt`` (nelmt, 81), ``mat_id`` 1..nmatblk, ``elmt_list`` 1-based
    (None: all elements).  ``evpt`` and ``stress_elmt`` (nelmt*27*6),
    ``bodyload`` (neq+1) and, in the excavation form (``form=1``) when
    ``last``, ``vmeps``/``scf`` (nnode) are float64 arrays updated in place.
    Returns fmax.
    """
    ctx = ctx or default_context()
    for name, a in (("evpt", evpt), ("stress_elmt", stress_elmt), ("bodyload", bodyload), ("vmeps", vmeps),
                    ("scf", scf)):
        if a is not None and (a.dtype != np.float64 or not a.flags.c_contiguous):
            raise ValueError(f"{name} must be a C-contiguous float64 array")
    f = lambda a: np.ascontiguousarray(a, np.float64)
    i32 = lambda a: np.ascontiguousarray(a, np.int32)
    gc, gn, ge, mi = f(g_coord), i32(g_num), i32(gdof_elmt), i32(mat_id)
    props = [f(a) for a in (ym_blk, nuf_blk, phif_blk, cohf_blk, psif_blk)]
    xv = f(x)
    el = None if elmt_list is None else i32(elmt_list)
    wp = None if wpressure is None else f(wpressure)
    fm = C.c_double(0)
    tag = C.create_string_buffer(ERRTAG_LEN + 1)
    err = lib().sg_stress_bodyload(
        ctx.h, neq, nelmt, nnode, _ptr(gc), _ptr(gn), _ptr(ge), _ptr(mi), len(props[0]), *(_ptr(a) for a in props),
        float(dt), int(bool(nl_isconv)), int(bool(last)), None if el is None else _ptr(el),
        0 if el is None else int(el.size), None if wp is None else _ptr(wp), int(form), _ptr(xv), _ptr(evpt),
        _ptr(stress_elmt), _ptr(bodyload), None if vmeps is None else _ptr(vmeps), None if scf is None else _ptr(scf),
        C.byref(fm), tag)
    if err:
        raise SgError(err, tag.value.decode().strip() or ctx.last_error)
    return fm.value


def read_deck(path: str) -> dict:
    """Read a .sem / .psem deck and build the spectral mesh on the host (no GPU).

    Returns the reference's arrays -- ``g_coord`` (nnode, 3), ``g_num``
    (nelmt, 27) 0-based, ``gdof`` (nnode, 3), ``gdof_elmt`` (nelmt, 81),
    ``mat_id`` (1-based), ``props`` (nmatblk, 6) -- and the control values;
    raises :class:`SgError` with the reader's errtag on a bad deck.
    """
    L = lib()
    tag = C.create_string_buffer(ERRTAG_LEN + 1)
    h = L.sg_mesh_from_deck(str(path).encode(), tag)
    if not h:
        raise SgError(SG_ERR_BADARG, tag.value.decode().strip())
    try:
        info = np.zeros(8, np.int32)
        L.sg_mesh_info(h, _ptr(info))
        nnode, nelmt, neq, nmat, nsrf, nexcav, iswater, nwmat = (int(v) for v in info)
        out = dict(nnode=nnode, nelmt=nelmt, neq=neq, nmatblk=nmat, iswater=iswater,
                   g_coord=np.zeros((nnode, 3)), g_num=np.zeros((nelmt, 27), np.int32),
                   gdof=np.zeros((nnode, 3), np.int32), gdof_elmt=np.zeros((nelmt, 81), np.int32),
                   mat_id=np.zeros(nelmt, np.int32), props=np.zeros((nmat, 6)))
        L.sg_mesh_arrays(h, *(_ptr(out[k]) for k in ("g_coord", "g_num", "gdof", "gdof_elmt", "mat_id", "props")))
        dctl, ictl, srf = np.zeros(8), np.zeros(8, np.int32), np.zeros(max(nsrf, 1))
        nexid = np.zeros(max(nexcav, 1), np.int32)
        wids = np.zeros(max(nwmat, 1), np.int32)
        L.sg_mesh_control(h, _ptr(dctl), _ptr(ictl), _ptr(srf), _ptr(nexid), None, _ptr(wids))
        exid = np.zeros(max(int(nexid[:nexcav].sum()), 1), np.int32)
        L.sg_mesh_control(h, None, None, None, None, _ptr(exid), None)
        out.update(cg_tol=dctl[0], nl_tol=dctl[1], z0=dctl[2], s0=dctl[3], k0=dctl[4], eqk=tuple(dctl[5:8]),
                   cg_maxiter=int(ictl[0]), nl_maxiter=int(ictl[1]), phinu=int(ictl[2]), allelastic=int(ictl[3]),
                   nexcav=int(ictl[4]), ninc=int(ictl[5]), s0_type=int(ictl[6]), iseqload=int(ictl[7]),
                   srf=srf[:nsrf].copy(), nexcavid=nexid[:nexcav].copy(),
                   excavid=exid[:int(nexid[:nexcav].sum())].copy(), water_ids=wids[:nwmat].copy())
        return out
    finally:
        L.sg_mesh_free(h)


def pcg_solver_noalloc(neq: int, nelmt: int, k: np.ndarray, u: np.ndarray, f: np.ndarray, dprecon: np.ndarray,
                       gdof_elmt: np.ndarray, cg_maxiter: int, cg_tol: float):
    """:func:`pcg_solver` without any device allocation (sg_pcg_solve_noalloc).

    For callers that cannot allocate device memory: everything the solve
    needs on the GPU lives in the library's fixed 64 MiB static device array,
    so there is no context and no cudaMalloc.  Larger problems raise
    :class:`SgError` with SG_ERR_BADARG.  Calls must not overlap on the GPU.
    Returns ``(cg_iter, errcode, errtag)`` like :func:`pcg_solver`.
    """
    if u.dtype != np.float64 or not u.flags.c_contiguous or u.shape[0] != neq + 1:
        raise ValueError("u must be a C-contiguous float64 array of length neq+1")
    k = np.ascontiguousarray(k, np.float64)
    f = np.ascontiguousarray(f, np.float64)
    dprecon = np.ascontiguousarray(dprecon, np.float64)
    ge = np.ascontiguousarray(gdof_elmt, np.int32)
    it = C.c_int(0)
    tag = C.create_string_buffer(ERRTAG_LEN + 1)
    err = lib().sg_pcg_solve_noalloc(neq, nelmt, 81, _ptr(k), _ptr(u), _ptr(f), _ptr(dprecon), _ptr(ge),
                                     cg_maxiter, cg_tol, C.byref(it), tag)
    if err not in (SG_OK, SG_ERR_NOCONV):
        raise SgError(err, tag.value.decode().strip())
    return it.value, err, tag.value.decode().rstrip()


def make_control(cg_tol=1e-8, nl_tol=1e-4, cg_maxiter=5000, nl_maxiter=2000, phinu=0, allelastic=0,
                 precision=PREC_FP64, refine_rtol=1e-10, inner_rtol=1e-3) -> Control:
    return Control(cg_tol, nl_tol, cg_maxiter, nl_maxiter, phinu, allelastic, precision, 0, refine_rtol, inner_rtol)


class Model:
    """A spectral model resident on the device (sg_model)."""

    def __init__(self, mesh=None, deck: Optional[str] = None, precision: int = PREC_FP64,
                 ctx: Optional[Context] = None):
        self.ctx = ctx or default_context()
        self.precision = precision
        L = lib()
        tag = C.create_string_buffer(ERRTAG_LEN + 1)
        if deck is not None:
            self.h = L.sg_model_from_deck(self.ctx.h, deck.encode(), precision, tag)
            self.mesh = None
        else:
            self.mesh = mesh
            self._keep = [np.ascontiguousarray(mesh.x, np.float64), np.ascontiguousarray(mesh.y, np.float64),
                          np.ascontiguousarray(mesh.z, np.float64),
                          np.ascontiguousarray(mesh.conn.reshape(-1), np.int32),
                          np.ascontiguousarray(mesh.mat_id, np.int32),
                          np.ascontiguousarray(mesh.props.reshape(-1), np.float64),
                          np.array([b.shape[0] for b in mesh.bc], np.int32),
                          np.ascontiguousarray(np.concatenate(mesh.bc).reshape(-1), np.int32)]
            x, y, z, conn, mid, props, cnt, pairs = self._keep
            self.h = L.sg_model_from_hex8(self.ctx.h, mesh.nnode8, _ptr(x), _ptr(y), _ptr(z), mesh.nelmt, _ptr(conn),
                                          _ptr(mid), mesh.props.shape[0], _ptr(props), _ptr(cnt), _ptr(pairs),
                                          precision, tag)
        if not self.h:
            raise SgError(SG_ERR_BADARG, tag.value.decode().strip() or self.ctx.last_error)
        info = np.zeros(8, np.int32)
        L.sg_model_info(self.h, _ptr(info))
        self.nnode, self.nelmt, self.neq, self.nmatblk, self.nsrf, self.ngroups = (int(v) for v in info[:6])

    def close(self):
        if getattr(self, "h", None):
            lib().sg_model_free(self.h)
            self.h = None

    __del__ = close

    def arrays(self):
        g_coord = np.zeros(3 * self.nnode)
        g_num = np.zeros(27 * self.nelmt, np.int32)
        gdof = np.zeros(3 * self.nnode, np.int32)
        ge = np.zeros(81 * self.nelmt, np.int32)
        lib().sg_model_arrays(self.h, _ptr(g_coord), _ptr(g_num), _ptr(gdof), _ptr(ge))
        return dict(g_coord=g_coord.reshape(-1, 3), g_num=g_num.reshape(-1, 27), gdof=gdof.reshape(-1, 3),
                    gdof_elmt=ge.reshape(-1, 81))

    def deck_control(self):
        d = np.zeros(2)
        i = np.zeros(6, np.int32)
        srf = np.zeros(max(self.nsrf, 1))
        lib().sg_model_control(self.h, _ptr(d), _ptr(i), _ptr(srf))
        return dict(cg_tol=d[0], nl_tol=d[1], cg_maxiter=int(i[0]), nl_maxiter=int(i[1]), phinu=int(i[2]),
                    allelastic=int(i[3]), nexcav=int(i[4]), ninc=int(i[5]), srf=srf[: self.nsrf])

    def stiffness(self, want_k: bool = True):
        """(storekm[e, col, row], dprecon before inversion, extload) as built on the device."""
        km = np.zeros(81 * 81 * self.nelmt) if want_k else None
        dp = np.zeros(self.neq + 1)
        ext = np.zeros(self.neq + 1)
        st = lib().sg_model_stiffness(self.h, _ptr(km) if want_k else None, _ptr(dp), _ptr(ext))
        if st:
            raise SgError(st, self.ctx.last_error)
        return (km.reshape(self.nelmt, 81, 81) if want_k else None), dp, ext

    def excavation_fields(self):
        """(vmeps[nnode], scf[nnode]) of the last excavation stage."""
        vm, sf = np.zeros(self.nnode), np.zeros(self.nnode)
        st = lib().sg_excavation_fields(self.h, _ptr(vm), _ptr(sf))
        if st:
            raise SgError(st, "sg_excavation_fields")
        return vm, sf

    def nodal_stress(self, trial: int = 0):
        """Valency-averaged nodal stress [nnode][6] of a trial of the last batch."""
        out = np.zeros(6 * self.nnode)
        st = lib().sg_nodal_stress(self.h, trial, _ptr(out))
        if st:
            raise SgError(st, "sg_nodal_stress")
        return out.reshape(-1, 6)

    def nodal_displacement(self, x: np.ndarray):
        """nodalu[nnode][3] from a solution x(0:neq) (src/slope.F90:400-407)."""
        gdof = self.arrays()["gdof"]
        return np.where(gdof > 0, np.asarray(x)[gdof], 0.0)

    def set_eqload(self, eqkx: float, eqky: float, eqkz: float):
        """Pseudo-static earthquake load factors (the deck's eqload: line)."""
        st = lib().sg_model_set_eqload(self.h, eqkx, eqky, eqkz)
        if st:
            raise SgError(st, self.ctx.last_error)

    def set_water(self, water_ids: Sequence[int], wsfile: str):
        """Water table: the water materials (1-based IDs) and a water-surface file
        (the deck's water: line); the pore pressure is computed on the device."""
        ids = np.ascontiguousarray(np.asarray(water_ids, np.int32).reshape(-1))
        tag = C.create_string_buffer(ERRTAG_LEN + 1)
        st = lib().sg_model_set_water(self.h, str(wsfile).encode(), _ptr(ids) if ids.size else None,
                                      int(ids.size), tag)
        if st:
            raise SgError(st, tag.value.decode().strip())

    def set_pore_pressure(self, wpressure):
        """Pore pressure per node (nnode values); None removes it."""
        if wpressure is None:
            st = lib().sg_model_set_pore_pressure(self.h, None)
        else:
            wp = np.ascontiguousarray(wpressure, np.float64).reshape(-1)
            if wp.size != self.nnode:
                raise ValueError("wpressure needs one value per node")
            st = lib().sg_model_set_pore_pressure(self.h, _ptr(wp))
        if st:
            raise SgError(st, self.ctx.last_error)

    def pore_pressure(self):
        """Pore pressure per node, or None when no water table is set."""
        out = np.zeros(self.nnode)
        st = lib().sg_model_pore_pressure(self.h, _ptr(out))
        return None if st else out

    def trials(self, srf: Sequence[float], ctl: Control, want_x: bool = False):
        srf = np.ascontiguousarray(srf, np.float64)
        k = len(srf)
        res = (TrialResult * k)()
        x = np.zeros(k * (self.neq + 1)) if want_x else None
        st = lib().sg_srf_trials(self.h, C.byref(ctl), k, _ptr(srf), C.cast(res, C.c_void_p),
                                 _ptr(x) if want_x else None)
        if st not in (SG_OK, SG_ERR_NOCONV):
            raise SgError(st, self.ctx.last_error)
        out = [r.as_dict() for r in res]
        if want_x:
            return out, x.reshape(k, self.neq + 1)
        return out

    def last_stress(self, trial: int = 0):
        s = np.zeros(self.nelmt * 27 * 6)
        st = lib().sg_last_stress(self.h, trial, _ptr(s))
        if st:
            raise SgError(st, "sg_last_stress")
        return s.reshape(self.nelmt, 27, 6)

    def sweep(self, srf: Sequence[float], ctl: Control):
        srf = np.ascontiguousarray(srf, np.float64)
        res = (TrialResult * len(srf))()
        n = C.c_int(0)
        st = lib().sg_srf_sweep(self.h, C.byref(ctl), len(srf), _ptr(srf), C.cast(res, C.c_void_p), C.byref(n))
        if st not in (SG_OK, SG_ERR_NOCONV):
            raise SgError(st, self.ctx.last_error)
        return [res[i].as_dict() for i in range(n.value)]

    def fos(self, ctl: Control, lo: float = 1.0, hi: float = 3.0, step: float = 0.01, k: int = 1):
        v = C.c_double(0)
        nt = C.c_int(0)
        nr = C.c_int(0)
        st = lib().sg_fos(self.h, C.byref(ctl), lo, hi, step, k, C.byref(v), C.byref(nt), C.byref(nr))
        if st:
            raise SgError(st, self.ctx.last_error)
        return v.value, nt.value, nr.value

    def fos_steps(self) -> int:
        """Plastic iterations of the last fos(): batch iterations for k > 1,
        trial iterations summed over the bisection's trials for k = 1."""
        n = C.c_longlong(0)
        st = lib().sg_fos_steps(self.h, C.byref(n))
        if st:
            raise SgError(st, "sg_fos_steps")
        return int(n.value)

    # ---- continuous batching -------------------------------------------
    def batch_begin(self, ctl: Control, kmax: int):
        self._batch_ctl = ctl
        st = lib().sg_batch_begin(self.h, C.byref(ctl), kmax)
        if st:
            raise SgError(st, self.ctx.last_error)

    def batch_add(self, srf: float) -> int:
        slot = C.c_int(-1)
        st = lib().sg_batch_add(self.h, srf, C.byref(slot))
        if st:
            raise SgError(st, self.ctx.last_error)
        return slot.value

    def batch_step(self, nsteps: int = 1) -> int:
        n = C.c_int(0)
        st = lib().sg_batch_step(self.h, nsteps, C.byref(n))
        if st not in (SG_OK, SG_ERR_NOCONV):
            raise SgError(st, self.ctx.last_error)
        return n.value

    def batch_poll(self, slot: int):
        r = TrialResult()
        state = C.c_int(0)
        st = lib().sg_batch_poll(self.h, slot, C.byref(r), C.byref(state))
        if st:
            raise SgError(st, "sg_batch_poll")
        return state.value, r.as_dict()

    def batch_release(self, slot: int):
        st = lib().sg_batch_release(self.h, slot)
        if st:
            raise SgError(st, "sg_batch_release")

    def batch_end(self):
        lib().sg_batch_end(self.h)

    def excavation(self, ctl: Control, s0_type: int, z0: float, s0: float, k0: float, excavid: Sequence[int],
                   nexcavid: Optional[Sequence[int]] = None, ninc: int = 1, srf: float = 1.0):
        excavid = np.ascontiguousarray(excavid, np.int32)
        nexcavid = np.ones(len(excavid), np.int32) if nexcavid is None else np.ascontiguousarray(nexcavid, np.int32)
        if int(nexcavid.sum()) != excavid.size:
            raise ValueError("excavid must list sum(nexcavid) material ids")
        res = np.zeros(8 * len(nexcavid))
        n = C.c_int(0)
        st = lib().sg_excavation(self.h, C.byref(ctl), s0_type, z0, s0, k0, len(nexcavid), _ptr(nexcavid),
                                 _ptr(excavid), ninc, srf, _ptr(res), C.byref(n))
        if st:
            raise SgError(st, self.ctx.last_error)
        return res.reshape(-1, 8)[: n.value]


class Server:
    """sg_server: a request loop of factor-of-safety and staged-excavation solves
    (see include/sg_solver.h)."""

    def __init__(self, device: int = 0, hbm_budget: int = 0, workers: int = 4):
        self.h = lib().sg_server_create(device, hbm_budget, workers)
        if not self.h:
            raise SgError(SG_ERR_NODEVICE, "sg_server_create failed")
        self._keep = {}

    @staticmethod
    def _mesh_arrays(mesh):
        return [np.ascontiguousarray(mesh.x, np.float64), np.ascontiguousarray(mesh.y, np.float64),
                np.ascontiguousarray(mesh.z, np.float64), np.ascontiguousarray(mesh.conn.reshape(-1), np.int32),
                np.ascontiguousarray(mesh.mat_id, np.int32), np.ascontiguousarray(mesh.props.reshape(-1), np.float64),
                np.array([b.shape[0] for b in mesh.bc], np.int32),
                np.ascontiguousarray(np.concatenate(mesh.bc).reshape(-1), np.int32)]

    def submit(self, mesh, ctl: Control, lo: float = 1.0, hi: float = 3.0, step: float = 0.01, k: int = 8) -> int:
        x, y, z, conn, mid, props, cnt, pairs = self._mesh_arrays(mesh)
        rid = C.c_int(0)
        st = lib().sg_server_submit(self.h, mesh.nnode8, _ptr(x), _ptr(y), _ptr(z), mesh.nelmt, _ptr(conn), _ptr(mid),
                                    mesh.props.shape[0], _ptr(props), _ptr(cnt), _ptr(pairs), C.byref(ctl), lo, hi,
                                    step, k, C.byref(rid))
        if st:
            raise SgError(st, "sg_server_submit")
        return rid.value

    def submit_excavation(self, mesh, ctl: Control, s0_type: int, z0: float, s0: float, k0: float,
                          excavid: Sequence[int], ninc: int = 1, srf: float = 1.0,
                          nexcavid: Optional[Sequence[int]] = None) -> int:
        """Queue a staged-excavation request (sg_excavation on its own model)."""
        x, y, z, conn, mid, props, cnt, pairs = self._mesh_arrays(mesh)
        exid = np.ascontiguousarray(excavid, np.int32)
        nexid = np.ascontiguousarray(np.ones(exid.size) if nexcavid is None else nexcavid, np.int32)
        rid = C.c_int(0)
        st = lib().sg_server_submit_excavation(
            self.h, mesh.nnode8, _ptr(x), _ptr(y), _ptr(z), mesh.nelmt, _ptr(conn), _ptr(mid), mesh.props.shape[0],
            _ptr(props), _ptr(cnt), _ptr(pairs), C.byref(ctl), s0_type, z0, s0, k0, int(nexid.size), _ptr(nexid),
            _ptr(exid), ninc, srf, C.byref(rid))
        if st:
            raise SgError(st, "sg_server_submit_excavation")
        return rid.value

    def wait(self, rid: int, timeout: float = 3600.0):
        r = FosResult()
        st = lib().sg_server_wait(self.h, rid, timeout, C.byref(r))
        if st:
            raise SgError(st, "sg_server_wait")
        out = r.as_dict()
        if r.kind == 1:
            rows = np.zeros(8 * max(r.nstage, 1))
            lib().sg_server_stages(self.h, rid, _ptr(rows))
            out["stages"] = rows[:8 * r.nstage].reshape(-1, 8)
        return out

    def stats(self):
        o = np.zeros(6)
        lib().sg_server_stats(self.h, _ptr(o))
        return dict(completed=int(o[0]), p50_s=o[1], p99_s=o[2], solves_per_s=o[3], peak_concurrent=int(o[4]),
                    budget_bytes=o[5])

    def close(self):
        if getattr(self, "h", None):
            lib().sg_server_destroy(self.h)
            self.h = None

    __del__ = close


def write_summary(path: str, ctl: Control, results, nsrf: Optional[int] = None):
    """Summary file of a slope run (header, then one row per trial result dict)."""
    st = lib().sg_write_summary_header(path.encode(), C.byref(ctl), len(results) if nsrf is None else nsrf)
    if st:
        raise SgError(st, "sg_write_summary_header")
    for r in results:
        tr = TrialResult()
        for name, _ in TrialResult._fields_:
            if name in r:
                setattr(tr, name, r[name])
        st = lib().sg_write_summary_row(path.encode(), C.byref(tr))
        if st:
            raise SgError(st, "sg_write_summary_row")


def write_ensight(out_dir: str, head: str, g_coord: np.ndarray, g_num: np.ndarray, times, steps):
    """EnSight Gold output of a slope run: <head>.case, <head>.geo and, for each
    step (nodalu[nnode][3], stress_global[nnode][6] or None), <head>_stepNN.dis/.sig."""
    os.makedirs(out_dir, exist_ok=True)
    times = np.ascontiguousarray(times, np.float64)
    nt = len(times)
    tw = int(math.ceil(math.log10(nt + 1.0)))
    L = lib()

    def chk(st, what):
        if st:
            raise SgError(st, what)

    chk(L.sg_write_ensight_case(os.path.join(out_dir, head + ".case").encode(), head.encode(), nt, _ptr(times), 1),
        "sg_write_ensight_case")
    gc = np.ascontiguousarray(g_coord, np.float64).reshape(-1)
    gn = np.ascontiguousarray(g_num, np.int32).reshape(-1)
    chk(L.sg_write_ensight_geo(os.path.join(out_dir, head + ".geo").encode(), gc.size // 3, _ptr(gc), gn.size // 27,
                               _ptr(gn)), "sg_write_ensight_geo")
    for i, (u, sig) in enumerate(steps):
        stem = os.path.join(out_dir, f"{head}_step{i + 1:0{tw}d}")
        u = np.ascontiguousarray(u, np.float64).reshape(-1)
        chk(L.sg_write_ensight_var((stem + ".dis").encode(), b"Displacement field", 3, u.size // 3, _ptr(u)),
            "sg_write_ensight_var")
        if sig is not None:
            sg_ = np.ascontiguousarray(sig, np.float64).reshape(-1)
            chk(L.sg_write_ensight_var((stem + ".sig").encode(), b"Effective stress tensor", 6, sg_.size // 6,
                                       _ptr(sg_)), "sg_write_ensight_var")


def principal_stress(stress_global: np.ndarray):
    """(psigma[n][3] ascending, taumax[n], nsigma[n]) from nodal stresses [n][6]."""
    st = np.ascontiguousarray(stress_global, np.float64).reshape(-1)
    n = st.size // 6
    ps, tm, ns = np.zeros(3 * n), np.zeros(n), np.zeros(n)
    r = lib().sg_principal_stress(n, _ptr(st), _ptr(ps), _ptr(tm), _ptr(ns))
    if r:
        raise SgError(r, "sg_principal_stress")
    return ps.reshape(n, 3), tm, ns
