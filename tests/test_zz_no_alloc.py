"""sg_pcg_solve_noalloc: the pcg_solver drop-in for callers that cannot
allocate device memory (their process owns the GPU memory through its own
pool, or must not call cudaMalloc).  It is checked against the existing
entry point, sg_pcg_solve, on two calls in a row: the second call must not
see anything the first one left in the shared static scratch array.

This file is collected last on purpose (tests/test_zz_*), so that a run that
stops at the first failure has already run every other test.
"""
import numpy as np
import pytest

import specfem3d_geotech_gb300 as sg
from oracle.pyoracle import OracleModel
from specfem3d_geotech_gb300 import meshgen

FP64_TOL = 1e-8   # the tolerance of the drop-in parity tests


def _inputs():
    om = OracleModel(meshgen.slope2d())
    km, dp, ext = om.stiffness_bodyload()
    dinv = np.where(np.arange(om.neq + 1) > 0, 1.0 / np.where(dp == 0, 1, dp), 0.0)
    return om.neq, om.nelmt, km, ext, dinv, om.arrays()["gdof_elmt"]


@pytest.mark.gpu
def test_noalloc_matches_pcg_solve_on_two_calls(built_lib):
    neq, nelmt, km, ext, dinv, ge = _inputs()
    u_ref = np.zeros(neq + 1)
    it_ref, err_ref, _ = sg.pcg_solver(neq, nelmt, km, u_ref, ext, dinv, ge, 5000, 1e-8)
    assert err_ref == 0
    rel = lambda a, b: np.linalg.norm(a - b) / np.linalg.norm(b)  # noqa: E731
    outs = []
    for _ in range(2):
        u = np.zeros(neq + 1)
        it, err, tag = sg.pcg_solver_noalloc(neq, nelmt, km, u, ext, dinv, ge, 5000, 1e-8)
        assert err == 0 and tag == ""
        assert abs(it - it_ref) <= 2
        assert rel(u, u_ref) <= FP64_TOL
        # same gather groups and reduction order as sg_pcg_solve: in practice bitwise equal
        assert it == it_ref and np.array_equal(u, u_ref)
        outs.append((it, u))
    # the second call starts from a clean state: identical to the first
    assert outs[0][0] == outs[1][0]
    assert np.array_equal(outs[0][1], outs[1][1])
    # a warm start after those calls still matches the existing entry point
    u0 = 0.9 * u_ref
    u1, u2 = u0.copy(), u0.copy()
    it1, e1, _ = sg.pcg_solver(neq, nelmt, km, u1, ext, dinv, ge, 5000, 1e-8)
    it2, e2, _ = sg.pcg_solver_noalloc(neq, nelmt, km, u2, ext, dinv, ge, 5000, 1e-8)
    assert e1 == e2 == 0 and abs(it1 - it2) <= 2 and rel(u2, u1) <= FP64_TOL


@pytest.mark.gpu
def test_noalloc_takes_no_device_memory(built_lib):
    """The defining claim: after the first call on the device, later calls
    leave the device's free memory unchanged (nothing is allocated, nothing
    is cached by the call)."""
    torch = pytest.importorskip("torch")
    neq, nelmt, km, ext, dinv, ge = _inputs()
    u = np.zeros(neq + 1)
    sg.pcg_solver_noalloc(neq, nelmt, km, u, ext, dinv, ge, 5000, 1e-8)
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(3):
        u = np.zeros(neq + 1)
        _, err, _ = sg.pcg_solver_noalloc(neq, nelmt, km, u, ext, dinv, ge, 5000, 1e-8)
        assert err == 0
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0


def test_noalloc_rejects_problems_beyond_its_scratch(built_lib):
    """Sizes beyond the 64 MiB static array are refused before any device work."""
    nelmt, neq = 2000, 10
    k = np.zeros((nelmt, 81, 81))
    ge = np.zeros((nelmt, 81), np.int32)
    u = np.zeros(neq + 1)
    with pytest.raises(sg.SgError) as e:
        sg.pcg_solver_noalloc(neq, nelmt, k, u, np.zeros(neq + 1), np.zeros(neq + 1), ge, 10, 1e-8)
    assert e.value.code == sg.SG_ERR_BADARG
    assert "64 MiB" in str(e.value)


def test_noalloc_rejects_a_dof_map_that_is_not_a_node_numbering(built_lib):
    """Two slots whose smallest free dof is the same must carry the same three
    dofs (they are one node); otherwise the call is refused before any device
    work."""
    nelmt, neq = 2, 6
    ge = np.zeros((nelmt, 81), np.int32)
    ge[0, 0:3] = [1, 2, 3]
    ge[1, 0:3] = [1, 4, 5]     # same smallest dof 1, different triple
    u = np.zeros(neq + 1)
    with pytest.raises(sg.SgError) as e:
        sg.pcg_solver_noalloc(neq, nelmt, np.zeros((nelmt, 81, 81)), u, np.zeros(neq + 1), np.zeros(neq + 1), ge,
                              10, 1e-8)
    assert e.value.code == sg.SG_ERR_BADARG
    assert "dof triples" in str(e.value)
