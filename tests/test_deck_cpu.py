"""The product's host deck reader and mesh builder (sg_mesh_from_deck: the
code sg_model_from_deck runs before it uploads) against the oracle's, on CPU.

Node numbering (get_global's merge), face constraints and node-major dof
numbering are integer work and must be identical; coordinates are copied,
so bitwise too.  Control values, the SRF list, the excavation lists, the
stress0 and eqload lines and the water IDs are read as the reference reads
them (src/read_input.f90:13-619); bad decks fail with its messages.
"""
import numpy as np
import pytest

import specfem3d_geotech_gb300 as sg
from oracle.pyoracle import OracleModel
from specfem3d_geotech_gb300 import meshgen


def _same_mesh(r, om):
    a = om.arrays()
    assert (r["nnode"], r["nelmt"], r["neq"]) == (om.nnode, om.nelmt, om.neq)
    for k in ("g_coord", "g_num", "gdof", "gdof_elmt", "mat_id"):
        assert np.array_equal(r[k], a[k]), k
    c = om.control()
    for k in ("cg_tol", "nl_tol", "cg_maxiter", "nl_maxiter", "phinu", "allelastic"):
        assert r[k] == c[k], k
    assert np.array_equal(r["srf"], c["srf"])


@pytest.mark.parametrize("name", ["slope2d", "slope3d", "excavation", "box"])
def test_deck_matches_oracle(tmp_path, name):
    mesh = {
        "slope2d": lambda: meshgen.slope2d(),
        "slope3d": lambda: meshgen.slope3d(nx=6, ny=3, nz=3),
        "excavation": lambda: meshgen.excavation(nx=6, ny=6, nz=4, L=12.0, H=8.0, pit=4.0, lifts=2, lift_h=2.0),
        "box": lambda: meshgen.box(nx=3, ny=2, nz=2),
    }[name]()
    deck = meshgen.write_deck(mesh, str(tmp_path))
    r = sg.read_deck(deck)
    _same_mesh(r, OracleModel(deck=deck))
    assert np.array_equal(r["props"], mesh.props)
    c = mesh.control
    assert r["nexcav"] == c.nexcav and np.array_equal(r["excavid"], np.array(c.excavid, np.int32))
    if c.nexcav:
        assert np.array_equal(r["nexcavid"], np.ones(c.nexcav, np.int32)) and r["ninc"] == c.ninc
    if mesh.stress0 is not None:
        t, z0, s0, k0 = mesh.stress0
        assert (r["s0_type"], r["z0"], r["s0"], r["k0"]) == (t, z0, s0, k0)
    else:
        assert r["s0_type"] == -1


def test_optional_lines(tmp_path):
    """eqload: and water: lines and the material list's water IDs."""
    mesh = meshgen.slope2d(srf=(1.0, 1.2))
    mesh.water = ((1,), "1\n0\n1 0.0 20.0 4.0\n")
    deck = meshgen.write_deck(mesh, str(tmp_path))
    with open(deck, "a") as f:
        f.write("eqload: eqkx=0.1, eqky=0.0, eqkz=-0.05\n")
    r = sg.read_deck(deck)
    assert r["iswater"] == 1 and np.array_equal(r["water_ids"], [1])
    assert r["iseqload"] == 1 and r["eqk"] == (0.1, 0.0, -0.05)
    assert np.array_equal(r["srf"], [1.0, 1.2])
    _same_mesh(r, OracleModel(deck=deck))


def _err(path):
    with pytest.raises(sg.SgError) as e:
        sg.read_deck(path)
    return str(e.value)


def test_bad_decks(tmp_path):
    mesh = meshgen.slope2d(srf=(1.0,))
    deck = meshgen.write_deck(mesh, str(tmp_path))
    text = open(deck).read()
    assert "cannot be opened" in _err(str(tmp_path / "missing.sem"))
    bad = tmp_path / "dup.sem"
    bad.write_text(text + "eqload: eqkx=0.1\neqload: eqkx=0.2\n")
    assert "copy of line type eqload: not permitted" in _err(str(bad))
    bad = tmp_path / "token.sem"
    bad.write_text(text + "gravity: g=9.81\n")
    assert 'invalid line type: "gravity:"' in _err(str(bad))
    bad = tmp_path / "water.sem"
    bad.write_text(text + "water: wsfile='ws'\n")     # no water IDs after the material blocks
    assert "water IDs cannot be read from material list" in _err(str(bad))
    # boundary-condition types the reference rejects, with its messages (src/apply_bc.f90:36-60)
    bcfile = tmp_path / "slope2d_ssbcux"
    good_bc = bcfile.read_text()
    for head, msg in (("2 0.5", "nonzero displacement BC not implemented"),
                      ("0 0.0", "nodal displacement BC not implemented"),
                      ("1 0.0", "edge displacement BC not implemented"),
                      ("7 0.0", "undefined displacement BC type")):
        bcfile.write_text(head + "\n" + good_bc.split("\n", 1)[1])
        assert msg in _err(deck), head
    bcfile.write_text(good_bc)
    bad = tmp_path / "nocontrol.sem"
    bad.write_text("\n".join(l for l in text.splitlines() if not l.startswith("control:")) + "\n")
    assert 'cannot read control information! make sure the line with "control:" token is correct' in _err(str(bad))
    bad = tmp_path / "method.sem"
    bad.write_text(text.replace("method='sem'", "method='xyz'"))
    assert "wrong value for method" in _err(str(bad))
    bad.write_text(text.replace("method='sem'", "method='fem'"))
    assert "not supported by this solver" in _err(str(bad))


def test_method_defaults_to_sem(tmp_path):
    """method='sem' is the reference's default (src/read_input.f90:87); a
    preinfo line without the key, or with a blank value, reads the same deck."""
    mesh = meshgen.slope2d(srf=(1.0, 1.5))
    deck = meshgen.write_deck(mesh, str(tmp_path))
    text = open(deck).read()
    assert "method='sem'" in text
    a = sg.read_deck(deck)
    for variant, repl in (("nomethod", ""), ("blank", "method=''")):
        d = tmp_path / (variant + ".sem")
        t = text.replace("method='sem', ", repl + (", " if repl else "")) if "method='sem', " in text \
            else text.replace("method='sem'", repl)
        assert ("method='sem'" not in t)
        d.write_text(t)
        b = sg.read_deck(str(d))
        for k in ("g_coord", "g_num", "gdof", "gdof_elmt", "mat_id", "props", "srf"):
            assert np.array_equal(a[k], b[k]), (variant, k)


def test_tolerance_merge_of_duplicate_nodes(tmp_path):
    """get_global merges points within 1e-10 |xmax - xmin| of each other
    (src/mesh_spec.f90:146-262).  Here the mesh is big enough for the threaded
    merge (several sorted chunks), and every third element refers to its own
    jittered copies of its corner nodes.  Node numbering, coordinates and dof
    maps equal the oracle's sequential merge."""
    mesh = meshgen.box(nx=20, ny=20, nz=14, L=20.0, W=20.0, zbot=0.0, ztop=14.0)
    rng = np.random.default_rng(7)
    tol = 1e-10 * 20.0
    x, y, z = list(mesh.x), list(mesh.y), list(mesh.z)
    conn = mesh.conn.copy()
    for e in range(0, mesh.nelmt, 3):
        for g in range(8):
            n = conn[e, g] - 1
            j = rng.uniform(-0.3, 0.3, 3) * tol
            x.append(mesh.x[n] + j[0]); y.append(mesh.y[n] + j[1]); z.append(mesh.z[n] + j[2])
            conn[e, g] = len(x)
    mesh.x, mesh.y, mesh.z, mesh.conn = np.array(x), np.array(y), np.array(z), conn
    assert mesh.nelmt * 27 >= 2 * 65536
    deck = meshgen.write_deck(mesh, str(tmp_path))
    r = sg.read_deck(deck)
    _same_mesh(r, OracleModel(deck=deck))
    assert r["nnode"] == 41 * 41 * 29                 # the copies merged away


def test_psem_deck_reads_its_unpartitioned_inputs(tmp_path):
    """A .psem deck names nproc, part_path and a ghost file for the MPI build;
    the single-GPU reader ignores them and reads the same input files."""
    mesh = meshgen.slope2d(srf=(1.0, 1.5))
    deck = meshgen.write_deck(mesh, str(tmp_path))
    text = open(deck).read()
    text = text.replace("preinfo: ", "preinfo: nproc=4, part_path='./partition', ")
    text = text.replace("idfile='slope2d_material_id'", "idfile='slope2d_material_id', gfile='slope2d_ghost'")
    assert "nproc=4" in text and "gfile=" in text
    psem = tmp_path / "slope2d.psem"
    psem.write_text(text)
    a, b = sg.read_deck(deck), sg.read_deck(str(psem))
    for k in ("g_coord", "g_num", "gdof", "gdof_elmt", "mat_id", "props", "srf"):
        assert np.array_equal(a[k], b[k]), k


@pytest.mark.parametrize("name", ["validation1", "cubit_example", "excavation_1d", "excavation_2d",
                                  "excavation_2d_single", "validation3", "validation4"])
def test_reference_decks_read_like_the_oracle(name):
    """Some of the reference's own decks (tests/golden/decks, copied from its
    input/ folder): CUBIT-exported coordinates, connectivity and side-set
    boundary files are merged and numbered exactly as the oracle does, and
    the excavation decks' stress0 and stage lines are read as the reference
    reads them (the stress0 line's usek0 key is read and unused, as in the
    reference)."""
    import os
    deck = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "decks", name + ".sem")
    r = sg.read_deck(deck)
    _same_mesh(r, OracleModel(deck=deck))
    assert r["nelmt"] == {"validation1": 1670, "cubit_example": 1690, "excavation_1d": 640, "excavation_2d": 1000,
                          "excavation_2d_single": 1000, "validation3": 1800, "validation4": 1800}[name]
    if name in ("validation3", "validation4"):
        # the water table (wsfile, water materials 2 and 3) and validation4's eqload line
        assert r["iswater"] == 1 and list(r["water_ids"]) == [2, 3]
        assert (r["iseqload"], r["eqk"]) == ((1, (0.1, 0.0, 0.0)) if name == "validation4" else (0, (0.0, 0.0, 0.0)))
    if name.startswith("excavation"):
        stage = {"excavation_1d": (1, [2], [1], 1, 40.0), "excavation_2d": (0, [2, 3, 4], [1, 1, 1], 1, 0.0),
                 "excavation_2d_single": (0, [2, 3, 4], [3], 1, 0.0)}[name]
        assert (r["s0_type"], list(r["excavid"]), list(r["nexcavid"]), r["ninc"], r["z0"]) == stage
        assert r["k0"] == 0.5
