"""Output writers on the host (no GPU): the EnSight Gold C-binary geometry,
per-node variables and case file of src/semgeotech.F90:126-312 and
src/visual.f90, and the summary file of src/slope.F90:213-220,409-416, read
back and checked field by field on the 300-element slope mesh."""
import math
import os

import numpy as np

import specfem3d_geotech_gb300 as sg
from oracle.pyoracle import OracleModel
from specfem3d_geotech_gb300 import meshgen


def _rec(b, off):
    return b[off:off + 80].decode().rstrip(), off + 80


def _i32(b, off):
    return int(np.frombuffer(b[off:off + 4], np.int32)[0]), off + 4


def test_ensight_geometry_and_variables(tmp_path):
    om = OracleModel(meshgen.slope2d())
    a = om.arrays()
    g_coord, g_num = a["g_coord"], a["g_num"]
    nnode, nelmt = g_coord.shape[0], g_num.shape[0]
    rng = np.random.default_rng(0)
    u = rng.standard_normal((nnode, 3))
    sig = rng.standard_normal((nnode, 6))
    times = [1.0, 1.05, 1.1]
    sg.write_ensight(str(tmp_path), "slope", g_coord, g_num, times, [(u, sig), (u, None), (u, sig)])
    # geometry
    b = open(tmp_path / "slope.geo", "rb").read()
    off = 0
    recs = []
    for _ in range(6):
        r, off = _rec(b, off)
        recs.append(r)
    assert recs == ["C Binary", "Created by write_ensight Routine", "semfem3d", "node id off",
                    "element id off", "part"]
    npart, off = _i32(b, off)
    r1, off = _rec(b, off)
    r2, off = _rec(b, off)
    nn, off = _i32(b, off)
    assert (npart, r1, r2, nn) == (1, "unstructured meshes", "coordinates", nnode)
    xyz = np.frombuffer(b[off:off + 12 * nnode], np.float32).reshape(3, nnode)
    off += 12 * nnode
    np.testing.assert_array_equal(xyz, g_coord.T.astype(np.float32))
    et, off = _rec(b, off)
    ncell, off = _i32(b, off)
    assert et == "hexa8" and ncell == 8 * nelmt
    cells = np.frombuffer(b[off:off + 32 * ncell], np.int32).reshape(ncell, 8)
    assert off + 32 * ncell == len(b)
    # first sub-cell of element 0: sequential corners 0,1,3,4,9,10,12,13 in
    # the Exodus order 1,2,4,3,5,6,8,7, 1-based
    np.testing.assert_array_equal(cells[0], g_num[0][[0, 1, 4, 3, 9, 10, 13, 12]] + 1)
    # last sub-cell of the last element: corners 13,14,16,17,22,23,25,26
    np.testing.assert_array_equal(cells[-1], g_num[-1][[13, 14, 17, 16, 22, 23, 26, 25]] + 1)
    # every node is used by some cell
    assert set(np.unique(cells)) == set(range(1, nnode + 1))
    # per-node variables: description, part, coordinates, components one after the other
    tw = int(math.ceil(math.log10(len(times) + 1.0)))
    for step, (name, ncomp, arr) in enumerate([("dis", 3, u), ("sig", 6, sig)]):
        b = open(tmp_path / f"slope_step{1:0{tw}d}.{name}", "rb").read()
        d, off = _rec(b, 0)
        p, off = _rec(b, off)
        npart, off = _i32(b, off)
        c, off = _rec(b, off)
        assert (p, npart, c) == ("part", 1, "coordinates")
        assert d == ("Displacement field" if name == "dis" else "Effective stress tensor")
        vals = np.frombuffer(b[off:], np.float32).reshape(ncomp, nnode)
        np.testing.assert_array_equal(vals, arr.T.astype(np.float32))
    assert not os.path.exists(tmp_path / f"slope_step{2:0{tw}d}.sig")
    # case file
    case = open(tmp_path / "slope.case").read().splitlines()
    assert case[0] == "FORMAT" and case[1] == "type:  ensight gold"
    assert "model:    slope.geo" in case
    assert any(l.startswith("vector per node:") and l.endswith("slope_step*.dis") for l in case)
    assert any(l.startswith("tensor symm per node:") and l.endswith("slope_step*.sig") for l in case)
    i = case.index([l for l in case if l.startswith("time values:")][0])
    assert case[i] == "time values:  0.10000E+01"
    assert case[i + 1] == " 0.10500E+01" and case[i + 2] == " 0.11000E+01"
    assert "number of steps:         3" in case


def test_summary_file(tmp_path):
    ctl = sg.make_control(cg_tol=1e-8, nl_tol=1e-4, cg_maxiter=5000, nl_maxiter=2000)
    rows = [dict(srf=1.0, cg_tot=2606, nl_iter=12, uxmax=0.0123, umax=0.0234, fmax=1.5e-3),
            dict(srf=1.05, cg_tot=3100, nl_iter=15, uxmax=0.0141, umax=0.0266, fmax=2.5e-3)]
    path = str(tmp_path / "slope_summary")
    sg.write_summary(path, ctl, rows, nsrf=21)
    lines = open(path).read().splitlines()
    assert lines[1].strip() == "Result summary produced by SPECFEM3D_GEOTECH"
    assert lines[3].strip() == "CG_MAXITER, CG_TOL, NL_MAXITER, NL_TOL"
    f = lines[4].split()
    assert int(f[0]) == 5000 and float(f[1]) == 1e-8 and int(f[2]) == 2000 and float(f[3]) == 1e-4
    assert lines[5].strip() == "Number of SRFs" and int(lines[6]) == 21
    assert lines[7].strip() == "SRF, CGITER, NLITER, UXMAX, UMAX, fmax"
    for r, l in zip(rows, lines[8:]):
        f = l.split()
        assert float(f[0]) == r["srf"] and int(f[1]) == r["cg_tot"] and int(f[2]) == r["nl_iter"]
        assert [float(v) for v in f[3:]] == [r["uxmax"], r["umax"], r["fmax"]]


def test_principal_stress_matches_oracle():
    """Principal stresses (ascending), maximum shear and normal stress per node
    (src/postprocess.f90:146-183) against the oracle, including hydrostatic
    states (J2 clamp) and the Lode corners; and the exact eigenvalues of the
    stress tensor."""
    from oracle import pyoracle
    rng = np.random.default_rng(1)
    st = rng.standard_normal((500, 6)) * 50.0
    st[0] = [-10, -10, -10, 0, 0, 0]          # hydrostatic
    st[1] = [-30, -10, -10, 0, 0, 0]          # Lode corner
    st[2] = [-10, -30, -30, 0, 0, 0]
    ps, tm, ns = sg.principal_stress(st)
    po, to, no = pyoracle.principal_stress(st)
    np.testing.assert_allclose(ps, po, rtol=1e-12, atol=1e-9)
    np.testing.assert_allclose(tm, to, rtol=1e-12, atol=1e-9)
    np.testing.assert_allclose(ns, no, rtol=1e-12, atol=1e-9)
    assert np.all(np.diff(ps, axis=1) >= 0)
    for k in range(3, 50):
        s = st[k]
        T = np.array([[s[0], s[3], s[5]], [s[3], s[1], s[4]], [s[5], s[4], s[2]]])
        np.testing.assert_allclose(ps[k], np.linalg.eigvalsh(T), rtol=1e-9, atol=1e-9)
