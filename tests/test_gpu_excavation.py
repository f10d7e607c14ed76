"""GPU parity of the staged-excavation driver's options (src/excavation.F90)
against the oracle, on a 6 x 6 x 4 block with a 4 x 4 m pit in 2 m lifts:

* initial stress by the SEM gravity solve (stress0 type 0,
  src/excavation.F90:182-238), which also runs the elastic-stress routine
  (src/postprocess.f90:40-79);
* load increments (ninc = 2, src/excavation.F90:509-641);
* unequal removal counts per stage, with the reference's stage index
  id0 = (stage-1)*nexcavid(stage)+1 (src/excavation.F90:339): counts [2, 1]
  remove lifts 2 and 3 in stage 1 and lift 3 again in stage 2 (lift 4 stays);
  counts whose index passes the end of excavid are refused;
* the elastic stress field itself, through an all-elastic trial of the
  layered 3D slope cut.

Stage rows are [stage, cg_tot, nl_tot, uxmax, umax, fmax, failed, errcode];
plastic-iteration totals and failure flags must be equal, and displacements
within 1e-8 for stages that converge. A stage that fails has run nl_maxiter
plastic iterations of a growing mechanism, which amplifies rounding: the
oracle's own dot-product order variants (sequential, pairwise, strided,
reverse, 5-way) spread its umax over 0.0518-0.0525 (1.3 %) and its fmax over
95-112 on the failing stage of the unequal-count case, so failed stages are
compared at 2e-2.
"""
import numpy as np
import pytest

import specfem3d_geotech_gb300 as sg
from oracle.pyoracle import OracleModel
from oracle_jobs import slope3d_cut
from specfem3d_geotech_gb300 import meshgen

pytestmark = pytest.mark.gpu

DISP_TOL = 1e-8
FAILED_DISP_TOL = 2e-2


def _mesh(lifts=2):
    return meshgen.excavation(nx=6, ny=6, nz=4, L=12.0, H=8.0, pit=4.0, lifts=lifts, lift_h=2.0)


def _both(ctx, lifts, s0_type, excavid, nexcavid=None, ninc=1):
    mesh = _mesh(lifts)
    om = OracleModel(mesh)
    om.set_control(1e-8, 5000, 1e-4, 200)
    ro = om.excavation(s0_type, 8.0, 0.0, 0.5, excavid, ninc=ninc, nexcavid=nexcavid)
    m = sg.Model(mesh, ctx=ctx)
    ctl = sg.make_control(cg_tol=1e-8, nl_tol=1e-4, cg_maxiter=5000, nl_maxiter=200)
    r = m.excavation(ctl, s0_type, 8.0, 0.0, 0.5, excavid, nexcavid=nexcavid, ninc=ninc)
    return r, ro


def _same(r, ro):
    assert r.shape == ro.shape and r.shape[0] >= 1
    assert np.array_equal(r[:, 0], ro[:, 0])
    assert np.array_equal(r[:, 2], ro[:, 2]), (r[:, 2], ro[:, 2])      # plastic iterations per stage
    assert np.array_equal(r[:, 6], ro[:, 6])                           # failed flags
    ok = ro[:, 6] == 0
    assert np.allclose(r[ok, 3:5], ro[ok, 3:5], rtol=DISP_TOL, atol=0)   # uxmax, umax
    assert np.allclose(r[~ok, 3:5], ro[~ok, 3:5], rtol=FAILED_DISP_TOL, atol=0)


def test_sem_gravity_initial_stress(ctx):
    r, ro = _both(ctx, 2, 0, [2, 3])
    _same(r, ro)


def test_load_increments(ctx):
    r, ro = _both(ctx, 2, 1, [2, 3], ninc=2)
    _same(r, ro)
    r1, _ = _both(ctx, 2, 1, [2, 3], ninc=1)
    assert not np.array_equal(r[:, 1], r1[:, 1])     # the increments change the solves


def test_unequal_stage_counts_keep_the_reference_index(ctx):
    r, ro = _both(ctx, 3, 1, [2, 3, 4], nexcavid=[2, 1])
    _same(r, ro)
    assert r.shape[0] == 2


def test_stage_index_past_excavid_is_refused(ctx):
    mesh = _mesh(3)
    m = sg.Model(mesh, ctx=ctx)
    ctl = sg.make_control(cg_tol=1e-8, nl_tol=1e-4, cg_maxiter=5000, nl_maxiter=200)
    with pytest.raises(sg.SgError) as e:
        m.excavation(ctl, 1, 8.0, 0.0, 0.5, [2, 3, 4], nexcavid=[1, 2])
    assert e.value.code == sg.SG_ERR_BADARG
    with pytest.raises(ValueError):
        OracleModel(mesh).excavation(1, 8.0, 0.0, 0.5, [2, 3, 4], nexcavid=[1, 2])


def test_elastic_stress_field_matches_oracle(ctx):
    mesh = slope3d_cut()
    om = OracleModel(mesh)
    om.set_control(1e-10, 5000, 1e-4, 10, 0, 1)
    ro = om.trial(1.0, want_x=True, want_stress=True)
    m = sg.Model(mesh, ctx=ctx)
    (r,), x = m.trials([1.0], sg.make_control(cg_tol=1e-10, nl_maxiter=10, allelastic=1), want_x=True)
    assert r["nl_iter"] == ro["nl_iter"] == 1
    assert np.linalg.norm(x[0] - ro["x"]) <= 1e-8 * np.linalg.norm(ro["x"])
    st = m.last_stress(0)
    assert np.abs(st - ro["stress"]).max() <= 1e-7 * np.abs(ro["stress"]).max()
