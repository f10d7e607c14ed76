"""Synthetic slope and excavation meshes in the reference's input contract.

The reference reads an 8-node hexahedral mesh (Exodus/CUBIT corner order),
material ids, a material list and face-constraint lists from a ``.sem`` deck
(src/read_input.f90:13-619, src/apply_bc.f90:7-143) and expands it to 27-node
spectral elements (src/mesh_spec.f90:17-143).  The benchmark workloads have no
public dataset, so this module builds seeded synthetic meshes with the shapes,
sizes and property distributions of the workloads the solver is measured on:

* ``slope2d``   300-element plane-strain 45 degree slope (30x1x10), one material.
* ``slope3d``   192k-element 3D slope, 1:2 face, three layers, per-element
                lognormal (+-10 % ~ 1 sigma) properties (120x40x40).
* ``excavation`` 500k-element block with a 20x20 m pit removed in four 5 m lifts.
* ``random_slope`` per-request slope meshes for the serving stream.

Everything is returned as a :class:`Hex8Mesh`; :func:`write_deck` writes it out
as a reference-format deck directory.
"""
from __future__ import annotations

import dataclasses
import math
import os
from typing import List, Optional, Tuple

import numpy as np

# Exodus face ids used by the reference (src/element.f90:48-141):
# 1 = y-min, 2 = x-max, 3 = y-max, 4 = x-min, 5 = z-min, 6 = z-max.
FACE_YMIN, FACE_XMAX, FACE_YMAX, FACE_XMIN, FACE_ZMIN, FACE_ZMAX = 1, 2, 3, 4, 5, 6


@dataclasses.dataclass
class Control:
    """Control-line values of a deck (src/read_input.f90:321-378)."""

    cg_tol: float = 1e-8
    cg_maxiter: int = 5000
    nl_tol: float = 1e-4
    nl_maxiter: int = 2000
    srf: Tuple[float, ...] = (1.0,)
    phinu: int = 0
    allelastic: int = 0
    nexcav: int = 0
    excavid: Tuple[int, ...] = ()
    ninc: int = 1


@dataclasses.dataclass
class Hex8Mesh:
    """An 8-node hex mesh plus materials and constraints, reference layout.

    ``conn`` is (nelmt, 8) 1-based Exodus corner order, ``mat_id`` is 1-based,
    ``props`` is (nmatblk, 6) with columns gamma, E, nu, phi, c, psi (the
    material-list column order of src/read_input.f90:563-595), and ``bc[d]`` is an
    (n, 2) array of (element 1-based, face 1..6) pairs fixing dof d = x, y, z.
    """

    x: np.ndarray
    y: np.ndarray
    z: np.ndarray
    conn: np.ndarray
    mat_id: np.ndarray
    props: np.ndarray
    bc: List[np.ndarray]
    control: Control
    name: str = "mesh"
    stress0: Optional[Tuple[int, float, float, float]] = None  # (type, z0, s0, k0)
    # water table: (1-based water material IDs, text of the water-surface file)
    water: Optional[Tuple[Tuple[int, ...], str]] = None

    @property
    def nelmt(self) -> int:
        return int(self.conn.shape[0])

    @property
    def nnode8(self) -> int:
        return int(self.x.shape[0])


def _structured(nx: int, ny: int, nz: int, xs: np.ndarray, ys: np.ndarray,
                ztop_fn, zbot: float = 0.0):
    """Mapped structured hex mesh: columns from zbot to ztop(x, y)."""
    X, Y = np.meshgrid(xs, ys, indexing="xy")            # (ny+1, nx+1)
    ZT = ztop_fn(X, Y)
    t = np.arange(nz + 1, dtype=np.float64) / nz          # (nz+1,)
    # node (i, j, k) -> i + (nx+1)*(j + (ny+1)*k)
    x = np.broadcast_to(X[None], (nz + 1, ny + 1, nx + 1)).reshape(-1).copy()
    y = np.broadcast_to(Y[None], (nz + 1, ny + 1, nx + 1)).reshape(-1).copy()
    z = (zbot + (ZT[None] - zbot) * t[:, None, None]).reshape(-1)
    i, j, k = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    i, j, k = (a.transpose(2, 1, 0).reshape(-1) for a in (i, j, k))  # element e = i + nx*(j + ny*k)

    def nid(ii, jj, kk):
        return ii + (nx + 1) * (jj + (ny + 1) * kk)

    conn = np.stack([nid(i, j, k), nid(i + 1, j, k), nid(i + 1, j + 1, k), nid(i, j + 1, k),
                     nid(i, j, k + 1), nid(i + 1, j, k + 1), nid(i + 1, j + 1, k + 1),
                     nid(i, j + 1, k + 1)], axis=1).astype(np.int32) + 1
    return x, y, z, conn, (i, j, k)


def _box_bcs(ijk, nx, ny, nz) -> List[np.ndarray]:
    """Bottom fixed in x, y, z; x-faces ux = 0; y-faces uy = 0."""
    i, j, k = ijk
    e = np.arange(i.size, dtype=np.int32) + 1
    bot = np.stack([e[k == 0], np.full((k == 0).sum(), FACE_ZMIN, np.int32)], 1)
    xmin = np.stack([e[i == 0], np.full((i == 0).sum(), FACE_XMIN, np.int32)], 1)
    xmax = np.stack([e[i == nx - 1], np.full((i == nx - 1).sum(), FACE_XMAX, np.int32)], 1)
    ymin = np.stack([e[j == 0], np.full((j == 0).sum(), FACE_YMIN, np.int32)], 1)
    ymax = np.stack([e[j == ny - 1], np.full((j == ny - 1).sum(), FACE_YMAX, np.int32)], 1)
    ux = np.concatenate([bot, xmin, xmax]).astype(np.int32)
    uy = np.concatenate([bot, ymin, ymax]).astype(np.int32)
    uz = bot.astype(np.int32)
    return [ux, uy, uz]


def slope2d(srf: Optional[Tuple[float, ...]] = None) -> Hex8Mesh:
    """300-element plane-strain 45 degree slope extruded one element thick.

    x in [0, 20] m; surface 5 m for x < 10, rising linearly to 10 m at x = 15,
    10 m beyond; y in [0, 1]; 30x1x10 mapped elements.  E = 1e5 kPa, nu = 0.3,
    c = 10 kPa, phi = 20 deg, psi = 0, gamma = 20 kN/m^3.
    """
    nx, ny, nz = 30, 1, 10
    xs = np.linspace(0.0, 20.0, nx + 1)
    ys = np.linspace(0.0, 1.0, ny + 1)

    def ztop(X, Y):
        return np.clip(5.0 + (X - 10.0), 5.0, 10.0)

    x, y, z, conn, ijk = _structured(nx, ny, nz, xs, ys, ztop)
    props = np.array([[20.0, 1e5, 0.3, 20.0, 10.0, 0.0]])
    if srf is None:
        srf = tuple(round(1.0 + 0.05 * i, 10) for i in range(21))
    ctl = Control(cg_tol=1e-8, cg_maxiter=5000, nl_tol=1e-4, nl_maxiter=2000, srf=tuple(srf))
    return Hex8Mesh(x, y, z, conn, np.ones(conn.shape[0], np.int32), props,
                    _box_bcs(ijk, nx, ny, nz), ctl, name="slope2d")


def slope3d(nx: int = 120, ny: int = 40, nz: int = 40, seed: int = 1,
            sigma: float = math.log(1.1)) -> Hex8Mesh:
    """3D layered slope: 60x20x30 m, 1:2 face 10 m high along x.

    The ground is 20 m high for x <= 20, rises at 1:2 to 30 m at x = 40 (the
    embankment forms the upper block) and stays at 30 m beyond.  Three
    horizontal layers by element-centroid height (z < 10, 10..20, >= 20) take
    E = {2e5, 1e5, 5e4} kPa, c = {30, 15, 8} kPa, phi = {32, 25, 18} deg from
    the bottom up; nu = 0.3, gamma = 19 kN/m^3, psi = 0.  Each element is its
    own material block with E, c and phi scaled by exp(sigma * N(0,1)).
    """
    xs = np.linspace(0.0, 60.0, nx + 1)
    ys = np.linspace(0.0, 20.0, ny + 1)

    def ztop(X, Y):
        return np.clip(20.0 + 0.5 * (X - 20.0), 20.0, 30.0)

    x, y, z, conn, ijk = _structured(nx, ny, nz, xs, ys, ztop)
    zc = z[conn - 1].mean(axis=1)
    layer = np.where(zc < 10.0, 0, np.where(zc < 20.0, 1, 2))
    E = np.array([2e5, 1e5, 5e4])[layer]
    c = np.array([30.0, 15.0, 8.0])[layer]
    phi = np.array([32.0, 25.0, 18.0])[layer]
    rng = np.random.default_rng(seed)
    g = rng.standard_normal((3, conn.shape[0]))
    E = E * np.exp(sigma * g[0])
    c = c * np.exp(sigma * g[1])
    phi = phi * np.exp(sigma * g[2])
    ne = conn.shape[0]
    props = np.stack([np.full(ne, 19.0), E, np.full(ne, 0.3), phi, c, np.zeros(ne)], 1)
    ctl = Control(cg_tol=1e-8, cg_maxiter=5000, nl_tol=1e-4, nl_maxiter=2000, srf=(1.0,))
    return Hex8Mesh(x, y, z, conn, np.arange(1, ne + 1, dtype=np.int32), props,
                    _box_bcs(ijk, nx, ny, nz), ctl, name=f"slope3d_{nx}x{ny}x{nz}")


def excavation(nx: int = 100, ny: int = 100, nz: int = 50, L: float = 100.0,
               H: float = 50.0, pit: float = 20.0, lifts: int = 4, lift_h: float = 5.0) -> Hex8Mesh:
    """Staged pit excavation: a pit x pit m hole removed in `lifts` lifts.

    Material 1 is the ground; materials 2..lifts+1 are the lifts from the top
    down (identical properties: E = 2e5 kPa, nu = 0.25, c = 20 kPa,
    phi = 30 deg, psi = 0, gamma = 20).  Initial stress: overburden with
    K0 = 0.5 from the free surface z0 = H (stress0 type 1).
    """
    xs = np.linspace(0.0, L, nx + 1)
    ys = np.linspace(0.0, L, ny + 1)
    x, y, z, conn, ijk = _structured(nx, ny, nz, xs, ys, lambda X, Y: np.full_like(X, H))
    cen = np.stack([a[conn - 1].mean(axis=1) for a in (x, y, z)], 1)
    mat = np.ones(conn.shape[0], np.int32)
    inpit = (np.abs(cen[:, 0] - L / 2) < pit / 2) & (np.abs(cen[:, 1] - L / 2) < pit / 2)
    for s in range(lifts):
        ztop, zbot = H - s * lift_h, H - (s + 1) * lift_h
        sel = inpit & (cen[:, 2] < ztop) & (cen[:, 2] > zbot)
        mat[sel] = s + 2
    props = np.tile(np.array([[20.0, 2e5, 0.25, 30.0, 20.0, 0.0]]), (lifts + 1, 1))
    ctl = Control(cg_tol=1e-8, cg_maxiter=5000, nl_tol=1e-4, nl_maxiter=2000, srf=(1.0,),
                  nexcav=lifts, excavid=tuple(range(2, lifts + 2)), ninc=1)
    return Hex8Mesh(x, y, z, conn, mat, props, _box_bcs(ijk, nx, ny, nz), ctl,
                    name=f"excavation_{nx}x{ny}x{nz}", stress0=(1, H, 0.0, 0.5))


def random_slope(rng: np.random.Generator, nelmt_target: int) -> Hex8Mesh:
    """One serving request: slope angle U[20,50] deg, height U[5,20] m,
    1..3 layers with c ~ U[5,40] kPa, phi ~ U[15,35] deg (E = 1e5, nu = 0.3,
    gamma = 20, psi = 0).  Domain: 2H level ground at the toe, the slope, 2H
    level crest; depth H below the toe; width H."""
    beta = math.radians(rng.uniform(20.0, 50.0))
    H = rng.uniform(5.0, 20.0)
    nlay = int(rng.integers(1, 4))
    run = H / math.tan(beta)
    Lx, Ly, Hz = 4.0 * H + run, H, 2.0 * H
    # element counts proportional to the box dimensions
    s = (nelmt_target / (Lx * Ly * Hz)) ** (1.0 / 3.0)
    nx, ny, nz = (max(2, int(round(Lx * s))), max(1, int(round(Ly * s))), max(2, int(round(Hz * s))))
    xs = np.linspace(0.0, Lx, nx + 1)
    ys = np.linspace(0.0, Ly, ny + 1)
    x0 = 2.0 * H

    def ztop(X, Y):
        return H + np.clip((X - x0) * math.tan(beta), 0.0, H)

    x, y, z, conn, ijk = _structured(nx, ny, nz, xs, ys, ztop)
    zc = z[conn - 1].mean(axis=1)
    bounds = np.sort(rng.uniform(0.2, 1.8, nlay - 1)) * H
    layer = np.searchsorted(bounds, zc)
    c = rng.uniform(5.0, 40.0, nlay)
    phi = rng.uniform(15.0, 35.0, nlay)
    props = np.stack([np.full(nlay, 20.0), np.full(nlay, 1e5), np.full(nlay, 0.3), phi, c,
                      np.zeros(nlay)], 1)
    ctl = Control(cg_tol=1e-8, cg_maxiter=5000, nl_tol=1e-4, nl_maxiter=2000, srf=(1.0,))
    return Hex8Mesh(x, y, z, conn, (layer + 1).astype(np.int32), props, _box_bcs(ijk, nx, ny, nz),
                    ctl, name=f"req_{nx}x{ny}x{nz}")


def column(n: int = 4, H: float = 4.0, E: float = 1e5, nu: float = 0.3, gam: float = 20.0) -> Hex8Mesh:
    """Laterally confined 1x1xn gravity column (the analytic check case)."""
    x, y, z, conn, ijk = _structured(1, 1, n, np.array([0.0, 1.0]), np.array([0.0, 1.0]),
                                     lambda X, Y: np.full_like(X, H))
    props = np.array([[gam, E, nu, 30.0, 1e6, 0.0]])
    bc = _box_bcs(ijk, 1, 1, n)
    ctl = Control(cg_tol=1e-14, cg_maxiter=2000, nl_tol=1e-4, nl_maxiter=10, srf=(1.0,), allelastic=1)
    return Hex8Mesh(x, y, z, conn, np.ones(n, np.int32), props, bc, ctl, name="column")


def box(nx: int = 4, ny: int = 4, nz: int = 4, L: float = 4.0, W: float = 4.0, zbot: float = 0.0,
        ztop: float = 4.0, props=(20.0, 1e5, 0.3, 30.0, 10.0, 0.0)) -> Hex8Mesh:
    """Structured box [0, L] x [0, W] x [zbot, ztop] of nx*ny*nz elements
    (element e = i + nx*(j + ny*k), 1-based in conn order), bottom fixed,
    sides on rollers; one material (gamma, E, nu, phi, c, psi)."""
    x, y, z, conn, ijk = _structured(nx, ny, nz, np.linspace(0.0, L, nx + 1), np.linspace(0.0, W, ny + 1),
                                     lambda X, Y: np.full_like(X, ztop), zbot=zbot)
    ctl = Control(cg_tol=1e-8, cg_maxiter=5000, nl_tol=1e-4, nl_maxiter=200, srf=(1.0,))
    return Hex8Mesh(x, y, z, conn, np.ones(conn.shape[0], np.int32), np.array([props], np.float64),
                    _box_bcs(ijk, nx, ny, nz), ctl, name="box")


def write_deck(mesh: Hex8Mesh, directory: str, head: Optional[str] = None) -> str:
    """Write `mesh` as a reference-format serial deck (``<head>.sem`` + files)."""
    head = head or mesh.name
    os.makedirs(directory, exist_ok=True)

    def w(name, header, rows, fmt):
        with open(os.path.join(directory, f"{head}_{name}"), "w") as f:
            if header is not None:
                f.write(f"{header}\n")
            np.savetxt(f, rows, fmt=fmt)

    for nm, arr in (("coord_x", mesh.x), ("coord_y", mesh.y), ("coord_z", mesh.z)):
        w(nm, mesh.nnode8, arr, "%.17g")
    w("connectivity", mesh.nelmt, mesh.conn, "%d")
    w("material_id", mesh.nelmt, mesh.mat_id, "%d")
    with open(os.path.join(directory, f"{head}_material_list"), "w") as f:
        f.write("# material properties (id,domain,type,gamma,ym,nu,phi,coh,psi)\n")
        f.write(f"{mesh.props.shape[0]}\n")
        for i, p in enumerate(mesh.props):
            f.write(f"{i + 1}, 1, 0, " + ", ".join("%.17g" % v for v in p) + "\n")
        if mesh.water is not None:  # water IDs follow the blocks (src/read_input.f90:602-611)
            f.write(f"{len(mesh.water[0])}\n")
            for wid in mesh.water[0]:
                f.write(f"{wid}\n")
    if mesh.water is not None:
        with open(os.path.join(directory, f"{head}_water_surface"), "w") as f:
            f.write(mesh.water[1])
    for d, nm in enumerate(("ssbcux", "ssbcuy", "ssbcuz")):
        with open(os.path.join(directory, f"{head}_{nm}"), "w") as f:
            f.write("2 0.0\n")
            f.write(f"{mesh.bc[d].shape[0]}\n")
            np.savetxt(f, mesh.bc[d], fmt="%d")
    c = mesh.control
    lines = [
        "#pre information",
        "preinfo: method='sem', ngllx=3, nglly=3, ngllz=3, nenod=8, ngnode=8, inp_path='./input', out_path='./output/'",
        "#mesh information",
        f"mesh: xfile='{head}_coord_x', yfile='{head}_coord_y', zfile='{head}_coord_z', &",
        f"confile='{head}_connectivity', idfile='{head}_material_id'",
        "#boundary conditions",
        f"bc: uxfile='{head}_ssbcux', uyfile='{head}_ssbcuy', uzfile='{head}_ssbcuz'",
    ]
    if mesh.stress0 is not None:
        t, z0, s0, k0 = mesh.stress0
        lines += ["#initial stress", f"stress0: type={t}, z0={z0:g}, s0={s0:g}, k0={k0:g}"]
    lines += ["#material list", f"material: matfile='{head}_material_list'" +
              (", allelastic=1" if c.allelastic else "")]
    if mesh.water is not None:
        lines += ["#water table", f"water: wsfile='{head}_water_surface'"]
    ctl = (f"control: cg_tol={c.cg_tol:g}, cg_maxiter={c.cg_maxiter}, nl_tol={c.nl_tol:g}, "
           f"nl_maxiter={c.nl_maxiter}, nsrf={len(c.srf)}, srf=" + " ".join("%g" % s for s in c.srf))
    if c.nexcav:
        ctl += f", nexcav={c.nexcav}, excavid=" + " ".join(str(i) for i in c.excavid) + f", ninc={c.ninc}"
    if c.phinu:
        ctl += ", phinu=1"
    lines += ["#control parameters", ctl, "#save data options", "save: disp=1"]
    path = os.path.join(directory, f"{head}.sem")
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")
    return path
