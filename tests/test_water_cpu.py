"""Water table (src/compute_pressure.f90:10-186) in the oracle: known answers.

The pore pressure of a submerged node under a surface is 9.81 (z_s - z); the
first surface of the file that covers a node decides it; nodes of dry
materials stay at 0.  A meshed surface (kind 2) keeps the reference's plane
offset D = det[xf1 xf2 xf3] in z = -(A x + B y + D)/C: exact for faces on a
plane through the origin, "free surface cannot be determined" otherwise.
"""
import numpy as np
import pytest

from oracle.pyoracle import OracleModel
from specfem3d_geotech_gb300 import meshgen

GAMW = 9.81


def _coords(om):
    return om.arrays()["g_coord"].reshape(-1, 3)


def _write(tmp_path, text, name="ws.txt"):
    p = tmp_path / name
    p.write_text(text)
    return str(p)


def test_horizontal_table(tmp_path):
    mesh = meshgen.slope2d(srf=(1.0,))
    om = OracleModel(mesh)
    om.set_water([1], _write(tmp_path, "1\n0\n1 0.0 20.0 4.0\n"))
    wp, sub = om.pore_pressure()
    z = _coords(om)[:, 2]
    assert sub.all()
    expect = np.where(z < 4.0, GAMW * (4.0 - z), 0.0)
    assert np.array_equal(wp, expect)
    assert (wp > 0).sum() > 0 and (wp == 0).sum() > 0


def test_dry_materials_stay_dry(tmp_path):
    mesh = meshgen.slope2d(srf=(1.0,))
    mesh.props = np.vstack([mesh.props, mesh.props])
    xc = mesh.x[mesh.conn - 1].mean(axis=1)
    mesh.mat_id = np.where(xc < 10.0, 2, 1).astype(np.int32)  # toe side is the water material
    om = OracleModel(mesh)
    om.set_water([2], _write(tmp_path, "1\n0\n1 0.0 20.0 20.0\n"))
    wp, sub = om.pore_pressure()
    g = om.arrays()
    gnum = g["g_num"].reshape(-1, 27)
    wet = np.zeros(om.nnode, bool)
    wet[gnum[mesh.mat_id == 2].reshape(-1)] = True
    assert np.array_equal(sub, wet)
    z = _coords(om)[:, 2]
    assert np.array_equal(wp, np.where(wet, GAMW * (20.0 - z), 0.0))


def test_inclined_table(tmp_path):
    mesh = meshgen.slope2d(srf=(1.0,))
    om = OracleModel(mesh)
    om.set_water([1], _write(tmp_path, "1\n1\n1 0.0 20.0 3.0 7.0\n"))
    wp, _ = om.pore_pressure()
    c = _coords(om)
    zs = 3.0 + (7.0 - 3.0) * (c[:, 0] - 0.0) / (20.0 - 0.0)
    covered = c[:, 2] <= 7.0
    expect = np.where(covered & (zs > c[:, 2]), GAMW * (zs - c[:, 2]), 0.0)
    assert np.array_equal(wp, expect)


def test_first_covering_surface_decides(tmp_path):
    mesh = meshgen.slope2d(srf=(1.0,))
    om = OracleModel(mesh)
    om.set_water([1], _write(tmp_path, "2\n0\n1 0.0 10.0 2.0\n0\n1 0.0 20.0 6.0\n"))
    wp, _ = om.pore_pressure()
    c = _coords(om)
    first = (c[:, 0] <= 10.0) & (c[:, 2] <= 2.0)
    second = ~first & (c[:, 2] <= 6.0)
    expect = np.where(first, GAMW * (2.0 - c[:, 2]), np.where(second, GAMW * (6.0 - c[:, 2]), 0.0))
    # z == 2 under the first surface: z1 > z fails, so 0 (the node is covered, the search stops)
    expect[first & (c[:, 2] == 2.0)] = 0.0
    assert np.array_equal(wp, expect)


def _top_faces(nx, ny, nz):
    k = nz - 1
    return [(i + nx * (j + ny * k) + 1, meshgen.FACE_ZMAX) for j in range(ny) for i in range(nx)]


def test_meshed_surface_on_origin_plane(tmp_path):
    mesh = meshgen.box(nx=3, ny=2, nz=3, L=3.0, W=2.0, zbot=-3.0, ztop=0.0)
    faces = _top_faces(3, 2, 3)
    text = "1\n2\n%d\n" % len(faces) + "".join("%d %d\n" % f for f in faces)
    om = OracleModel(mesh)
    om.set_water([1], _write(tmp_path, text))
    wp, _ = om.pore_pressure()
    z = _coords(om)[:, 2]
    assert np.array_equal(wp, np.where(z < 0.0, GAMW * (0.0 - z), 0.0))


def test_meshed_surface_off_origin_is_an_error(tmp_path):
    mesh = meshgen.box(nx=2, ny=2, nz=2, L=2.0, W=2.0, zbot=0.0, ztop=5.0)
    faces = _top_faces(2, 2, 2)
    text = "1\n2\n%d\n" % len(faces) + "".join("%d %d\n" % f for f in faces)
    om = OracleModel(mesh)
    with pytest.raises(RuntimeError, match="free surface cannot be determined"):
        om.set_water([1], _write(tmp_path, text))


def test_deck_water_line(tmp_path):
    mesh = meshgen.slope2d(srf=(1.0,))
    mesh.water = ((1,), "1\n0\n1 0.0 20.0 4.0\n")
    deck = meshgen.write_deck(mesh, str(tmp_path / "deck"))
    od = OracleModel(deck=deck)
    om = OracleModel(mesh)
    om.set_water([1], _write(tmp_path, mesh.water[1]))
    wp_d, sub_d = od.pore_pressure()
    wp, sub = om.pore_pressure()
    assert np.array_equal(wp_d, wp) and np.array_equal(sub_d, sub)


def test_pore_pressure_weakens_the_slope(tmp_path):
    """Pore pressure reduces the mean effective compression, so at the same
    SRF the wet slope is further past yield (larger fmax) after the same two
    plastic iterations, and its displacement grows more."""
    mesh = meshgen.slope2d(srf=(1.0,))
    dry = OracleModel(mesh)
    wet = OracleModel(mesh)
    wet.set_water([1], _write(tmp_path, "1\n0\n1 0.0 20.0 6.0\n"))
    for om in (dry, wet):
        om.set_control(1e-8, 5000, 1e-4, 2)
    r_dry = dry.trial(1.2)
    r_wet = wet.trial(1.2)
    assert r_wet["fmax"] > r_dry["fmax"]
    assert r_wet["umax"] > r_dry["umax"]


def test_inclined_table_given_right_to_left(tmp_path):
    """rx1 > rx2: the covered range is [min, max] and z interpolates from rx1."""
    mesh = meshgen.slope2d(srf=(1.0,))
    om = OracleModel(mesh)
    om.set_water([1], _write(tmp_path, "1\n1\n1 20.0 0.0 7.0 3.0\n"))
    wp, _ = om.pore_pressure()
    c = _coords(om)
    zs = 7.0 + (3.0 - 7.0) * (c[:, 0] - 20.0) / (0.0 - 20.0)
    covered = c[:, 2] <= 7.0
    assert np.array_equal(wp, np.where(covered & (zs > c[:, 2]), GAMW * (zs - c[:, 2]), 0.0))


def test_vertical_meshed_face_takes_its_top(tmp_path):
    """A vertical face (C = 0 in the plane equation) sets the surface at the
    face's highest corner; its bounding box in x is a single plane."""
    mesh = meshgen.box(nx=2, ny=2, nz=2, L=2.0, W=2.0, zbot=0.0, ztop=2.0)
    faces = [(i + 2 * (j + 2 * k) + 1, meshgen.FACE_XMAX) for k in range(2) for j in range(2) for i in (1,)]
    om = OracleModel(mesh)
    om.set_water([1], _write(tmp_path, "1\n2\n%d\n" % len(faces) + "".join("%d %d\n" % f for f in faces)))
    wp, _ = om.pore_pressure()
    c = _coords(om)
    on_plane = c[:, 0] == 2.0
    # the first face (lower element) covers the plane's nodes up to its top z = 1; the
    # upper element's face covers the rest with top z = 2
    ztop = np.where(c[:, 2] <= 1.0, 1.0, 2.0)
    assert np.array_equal(wp, np.where(on_plane, GAMW * (ztop - c[:, 2]), 0.0))


def test_reference_validation3_deck_water_table():
    """The reference's own validation3 deck (tests/golden/decks): its water
    file holds two surfaces -- a horizontal table z = 6.1 over 42.7 <= x <= 50
    first, then an inclined one from (0, 12.2) to (42.7, 6.1) -- and materials
    2 and 3 are the water materials.  Read as the reference reads the deck,
    every node of those materials has 9.81 (z_s(x) - z) where it lies under
    the surface and 0 above it, and the nodes of material 1 stay dry."""
    import os
    deck = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "decks", "validation3.sem")
    om = OracleModel(deck=deck)
    wp, sub = om.pore_pressure()
    a = om.arrays()
    c = a["g_coord"].reshape(-1, 3)
    x, z = c[:, 0], c[:, 2]
    gnum = a["g_num"].reshape(-1, 27)
    wet = np.zeros(om.nnode, bool)
    wet[gnum[np.isin(a["mat_id"], [2, 3])].reshape(-1)] = True
    assert np.array_equal(sub, wet)
    zs = np.where(x >= 42.7, 6.1, 12.2 + (6.1 - 12.2) * x / 42.7)
    expect = np.where(wet, np.maximum(GAMW * (zs - z), 0.0), 0.0)
    assert np.abs(wp - expect).max() <= 1e-12 * np.abs(expect).max()
    assert (wp > 0).sum() > 1000 and wp.max() > 100.0
