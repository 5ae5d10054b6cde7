"""Seeded synthetic meshes written in the reference's own input formats.

The reference reads a command file (keywords parsed in
``SourceFiles/Solver/fioFile.cpp:69-462``) that names a mesh file in the
``.lis`` layout read by ``datModel::readdata`` (``SourceFiles/Solver/datModel.cpp:58-326``):

    title
    label line
    <2D|3D> <problem type>
    E nu rho KIc sig_ult
    numNode numEle
    <id x y z>                          x numNode
    <id algo n1..n4 | n1..n8>           x numEle   (algo 1 = PD, 2 = FE)
    ====Essential BCs====
    numEBC
    <numNode UX|UY|UZ value>            x numEBC
    <node ids>                          per EBC
    ====Natural BCs====
    numNBC  (<numEle value> headers, then 2 or 4 node ids per element)
    ====NO FAIL region====
    numNoFail  ids...
    ====pre-exist crack====
    numCrack   (2D: 2 points x 3 coords, 3D: 3 points x 3 coords)

Structured Q4 (2D) and Hex8 (3D) grids are generated with node index
``i + nx*(j + ny*k)`` (x fastest), holes are made by deleting elements and
then dropping orphan nodes (a node without element has zero volume, which
the reference divides by), and PD zones are element sets with algo type 1.

Coordinates are written with 17 significant digits so that the mesh read
back is bit-identical to the generated arrays.
"""
from __future__ import annotations

import dataclasses
import math
import os
from typing import Callable, List, Optional, Sequence, Tuple

import numpy as np

DOF_NAMES = ("UX", "UY", "UZ")


@dataclasses.dataclass
class EBC:
    dof: int                     # 0 = UX, 1 = UY, 2 = UZ
    value: float
    nodes: np.ndarray            # 1-based node ids
    velocity: Optional[float] = None   # VEBC velocity (command file)


@dataclasses.dataclass
class NBC:
    value: float
    elems: np.ndarray            # (numEle, 2|4) 1-based node ids
    velocity: Optional[float] = None


@dataclasses.dataclass
class Mesh:
    title: str
    dim: int
    protype: int                 # 1 plane stress, 2 plane strain (2D)
    E: float
    nu: float
    rho: float
    KIc: float
    sigult: float
    X: np.ndarray                # (N, 3)
    elems: np.ndarray            # (E, 4|8) 1-based
    algo: np.ndarray             # (E,) 1 PD, 2 FE
    ebcs: List[EBC]
    nbcs: List[NBC]
    nofail: np.ndarray           # 1-based ids
    cracks: List[np.ndarray]     # each (2,3) in 2D or (3,3) in 3D

    @property
    def n_node(self) -> int:
        return int(self.X.shape[0])

    @property
    def n_elem(self) -> int:
        return int(self.elems.shape[0])


def _fmt(v: float) -> str:
    return repr(float(v))


def write_lis(mesh: Mesh, path: str) -> None:
    """Write ``mesh`` in the ``.lis`` layout (``datModel.cpp:58-326``)."""
    lines: List[str] = []
    lines.append(mesh.title)
    lines.append("***" + mesh.title + "***")
    lines.append(f"{mesh.dim}D\t{mesh.protype}")
    lines.append("\t".join(_fmt(v) for v in (mesh.E, mesh.nu, mesh.rho, mesh.KIc, mesh.sigult)))
    lines.append(f"{mesh.n_node}\t{mesh.n_elem}")
    X = mesh.X
    for i in range(mesh.n_node):
        lines.append(f"{i + 1}\t{_fmt(X[i, 0])}\t{_fmt(X[i, 1])}\t{_fmt(X[i, 2])}")
    for e in range(mesh.n_elem):
        conn = " ".join(str(int(v)) for v in mesh.elems[e])
        lines.append(f"{e + 1}\t{int(mesh.algo[e])}\t{conn}")
    lines.append("=============================Essential BCs====================================")
    lines.append(str(len(mesh.ebcs)))
    for b in mesh.ebcs:
        lines.append(f"{len(b.nodes)}\t{DOF_NAMES[b.dof]}\t{_fmt(b.value)}")
    for b in mesh.ebcs:
        lines.append(" ".join(str(int(v)) for v in b.nodes))
    lines.append("=============================Natural BCs====================================")
    lines.append(str(len(mesh.nbcs)))
    for b in mesh.nbcs:
        lines.append(f"{len(b.elems)}\t{_fmt(b.value)}")
    for b in mesh.nbcs:
        for row in b.elems:
            lines.append(" ".join(str(int(v)) for v in row))
    lines.append("=============================NO FAIL region=================================")
    lines.append(str(len(mesh.nofail)))
    if len(mesh.nofail):
        lines.append(" ".join(str(int(v)) for v in mesh.nofail))
    lines.append("=============================pre-exist crack=================================")
    lines.append(str(len(mesh.cracks)))
    npt = 2 if mesh.dim == 2 else 3
    for c in mesh.cracks:
        lines.append("\t".join(_fmt(v) for v in np.asarray(c, dtype=np.float64)[:npt].ravel()))
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


def write_cmd(path: str, mesh_file: str, mesh: Mesh, *, solver: str, dt: float,
              nsteps: int, save: int, factor: float, nlf: float,
              newmark: Optional[Tuple[float, float]] = None, lumped: bool = True,
              fc: Optional[str] = None, precision: Optional[str] = None,
              extra: Sequence[str] = (), vtk: str = "BINARY", me: Optional[float] = None) -> None:
    """Write a command file with the reference's keywords (``fioFile.cpp:69-462``).

    ``fc`` is the text after the ``FC`` keyword; ``FC 3 s0 [seed] [pert]`` is the
    critical-stretch extension (the reference parses flag 3 but never acts on it).
    ``me`` is SETSOLVING's optional sixth value: crack-cut elements make the FE
    elements whose centres lie within me times the smallest element size PD.
    """
    setsolving = f"SETSOLVING {_fmt(dt)} {nsteps} {save} {_fmt(factor)} {_fmt(nlf)}"
    if me is not None:
        setsolving += f" {_fmt(me)}"
    out = [f"MSHFILE {mesh_file}", f"SOLVER {solver}", setsolving]
    if newmark is not None:
        out.append(f"NEWMARK ON {_fmt(newmark[0])} {_fmt(newmark[1])}")
    else:
        out.append("NEWMARK OFF")
    out.append("LUMPMASS " + ("ON" if lumped else "OFF"))
    for i, b in enumerate(mesh.ebcs):
        if b.velocity is not None:
            out.append(f"VEBC {i} {_fmt(b.velocity)}")
    for i, b in enumerate(mesh.nbcs):
        if b.velocity is not None:
            out.append(f"VNBC {i} {_fmt(b.velocity)}")
    if fc is not None:
        out.append(f"FC {fc}")
    if precision is not None:
        out.append(f"PRECISION {precision}")
    out.extend(extra)
    out.append(f"VTKFORMAT {vtk}")
    with open(path, "w") as f:
        f.write("\n".join(out) + "\n")


# --------------------------------------------------------------------------
# structured grids
# --------------------------------------------------------------------------

def _compact(X: np.ndarray, elems0: np.ndarray, algo: np.ndarray):
    """Drop orphan nodes; return (X, elems 1-based, algo, old->new map)."""
    used = np.zeros(X.shape[0], dtype=bool)
    used[elems0.ravel()] = True
    newid = -np.ones(X.shape[0], dtype=np.int64)
    newid[used] = np.arange(int(used.sum()))
    return X[used], newid[elems0] + 1, algo, newid


def grid2d(nx: int, ny: int, h: float, x0: float = 0.0, y0: float = 0.0):
    """Node coordinates and Q4 connectivity (0-based, CCW) of an nx x ny grid."""
    ii, jj = np.meshgrid(np.arange(nx), np.arange(ny), indexing="xy")
    X = np.zeros((nx * ny, 3))
    X[:, 0] = x0 + ii.ravel() * h
    X[:, 1] = y0 + jj.ravel() * h
    ei, ej = np.meshgrid(np.arange(nx - 1), np.arange(ny - 1), indexing="xy")
    ei = ei.ravel(); ej = ej.ravel()
    n0 = ei + nx * ej
    elems = np.stack([n0, n0 + 1, n0 + 1 + nx, n0 + nx], axis=1)
    centers = np.stack([x0 + (ei + 0.5) * h, y0 + (ej + 0.5) * h], axis=1)
    return X, elems, centers


def grid3d(nx: int, ny: int, nz: int, h: float):
    """Node coordinates and Hex8 connectivity (0-based) of an nx x ny x nz grid."""
    kk, jj, ii = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    X = np.stack([ii.ravel() * h, jj.ravel() * h, kk.ravel() * h], axis=1).astype(np.float64)
    ek, ej, ei = np.meshgrid(np.arange(nz - 1), np.arange(ny - 1), np.arange(nx - 1), indexing="ij")
    ei = ei.ravel(); ej = ej.ravel(); ek = ek.ravel()
    n0 = ei + nx * (ej + ny * ek)
    sxy = nx * ny
    bot = np.stack([n0, n0 + 1, n0 + 1 + nx, n0 + nx], axis=1)
    elems = np.concatenate([bot, bot + sxy], axis=1)
    centers = np.stack([(ei + 0.5) * h, (ej + 0.5) * h, (ek + 0.5) * h], axis=1)
    return X, elems, centers


def plate2d(nx: int, ny: int, h: float, *, pd_mask: Callable[[np.ndarray], np.ndarray],
            hole: Optional[Tuple[float, float, float]] = None,
            cracks: Sequence[np.ndarray] = (), title: str = "plate",
            material=(72e9, 0.22, 2440.0, 1.0e6, 1.0e8), protype: int = 1,
            top_velocity: Optional[float] = 0.05, top_value: float = 0.0) -> Mesh:
    """Plate of nx x ny nodes: bottom edge fixed (UX, UY), top edge UY driven."""
    X, elems, centers = grid2d(nx, ny, h)
    keep = np.ones(len(elems), dtype=bool)
    if hole is not None:
        cx, cy, r = hole
        keep &= (centers[:, 0] - cx) ** 2 + (centers[:, 1] - cy) ** 2 >= r * r
    elems, centers = elems[keep], centers[keep]
    algo = np.where(pd_mask(centers), 1, 2).astype(np.int64)
    Xc, el1, algo, newid = _compact(X, elems, algo)
    ids = np.arange(nx * ny)
    jrow = ids // nx
    bottom = newid[ids[jrow == 0]]; bottom = bottom[bottom >= 0] + 1
    top = newid[ids[jrow == ny - 1]]; top = top[top >= 0] + 1
    ebcs = [EBC(0, 0.0, bottom), EBC(1, 0.0, bottom),
            EBC(1, top_value, top, velocity=top_velocity)]
    E, nu, rho, KIc, sig = material
    return Mesh(title, 2, protype, E, nu, rho, KIc, sig, Xc, el1, algo, ebcs, [],
                np.zeros(0, dtype=np.int64), [np.asarray(c, dtype=np.float64) for c in cracks])


def box3d(nx: int, ny: int, nz: int, h: float, *, pd_mask: Callable[[np.ndarray], np.ndarray],
          hole: Optional[Tuple[float, float, float]] = None,
          cracks: Sequence[np.ndarray] = (), title: str = "box",
          material=(200e9, 0.3, 7850.0, 1.0e6, 1.0e8), x_velocity: Optional[float] = 0.1,
          pin_rigid: bool = False) -> Mesh:
    """Box of nx x ny x nz nodes pulled on both x faces (UX = -v, +v)."""
    X, elems, centers = grid3d(nx, ny, nz, h)
    keep = np.ones(len(elems), dtype=bool)
    if hole is not None:
        cx, cy, r = hole
        keep &= (centers[:, 0] - cx) ** 2 + (centers[:, 1] - cy) ** 2 >= r * r
    elems, centers = elems[keep], centers[keep]
    algo = np.where(pd_mask(centers), 1, 2).astype(np.int64)
    Xc, el1, algo, newid = _compact(X, elems, algo)
    ids = np.arange(nx * ny * nz)
    ix = ids % nx
    left = newid[ids[ix == 0]]; left = left[left >= 0] + 1
    right = newid[ids[ix == nx - 1]]; right = right[right >= 0] + 1
    vl = None if x_velocity is None else -x_velocity
    ebcs = [EBC(0, 0.0, left, velocity=vl), EBC(0, 0.0, right, velocity=x_velocity)]
    if pin_rigid:
        # fix UY/UZ on the x = 0 face so that the static problem is well posed
        ebcs.append(EBC(1, 0.0, left))
        ebcs.append(EBC(2, 0.0, left))
    E, nu, rho, KIc, sig = material
    return Mesh(title, 3, -1, E, nu, rho, KIc, sig, Xc, el1, algo, ebcs, [],
                np.zeros(0, dtype=np.int64), [np.asarray(c, dtype=np.float64) for c in cracks])


# --------------------------------------------------------------------------
# named workloads
# --------------------------------------------------------------------------

def plate_strip_crack(n: int = 101, L: float = 0.05, strip_frac: float = 0.4,
                      crack_len: float = 0.01, title: str = "plateStrip") -> Mesh:
    """n x n node square plate, central vertical PD strip, edge pre-crack in the strip.

    The strip covers the central ``strip_frac`` of the width (41 node columns for
    n = 101).  The crack starts a quarter element inside the strip's left
    edge, runs ``crack_len`` in +x at mid-height, and sits half an element above
    a node row so that no node lies on it.
    """
    h = L / (n - 1)
    ne = n - 1
    c0 = int(round(ne * (1.0 - strip_frac) / 2.0))
    c1 = ne - c0
    xs0 = c0 * h
    y_c = (ne // 2) * h + 0.5 * h

    def pd_mask(cent):
        return (cent[:, 0] > xs0) & (cent[:, 0] < c1 * h)

    crack = np.array([[xs0 + 0.25 * h, y_c, 0.0], [xs0 + 0.25 * h + crack_len, y_c, 0.0]])
    return plate2d(n, n, h, pd_mask=pd_mask, cracks=[crack], title=title)


def plate_edge_crack(n: int = 31, L: float = 0.03, a_frac: float = 0.41, pd_band: int = 0,
                     title: str = "plateEdge", KIc: float = 1.0e6, protype: int = 1) -> Mesh:
    """n x n node square FE plate with an edge pre-crack for FC 1 crack growth.

    The crack starts a quarter element inside the left edge and runs in +x to
    ``a_frac`` of the width, half an element above the middle node row.  Only
    the elements it cuts become PD at set-up (and, with ``pd_band`` > 0, the
    elements whose centres lie within ``pd_band`` elements of the crack line
    behind its tip); the PD region then grows with the crack.
    """
    h = L / (n - 1)
    ne = n - 1
    y_c = (ne // 2) * h + 0.5 * h
    x_tip = a_frac * L

    def pd_mask(cent):
        if pd_band <= 0:
            return np.zeros(len(cent), dtype=bool)
        return (np.abs(cent[:, 1] - y_c) < pd_band * h) & (cent[:, 0] < x_tip)

    crack = np.array([[0.25 * h, y_c, 0.0], [x_tip, y_c, 0.0]])
    return plate2d(n, n, h, pd_mask=pd_mask, cracks=[crack], title=title,
                   material=(72e9, 0.22, 2440.0, KIc, 1.0e8), protype=protype)


def split_triangles(mesh: Mesh, select: Optional[Callable[[np.ndarray], np.ndarray]] = None) -> Mesh:
    """Split the 2D quadrilaterals whose centres ``select`` accepts (all without
    it) into two 3-node triangles each, along alternating diagonals; a triangle
    is written as four node ids with the third repeated (the reference's
    pdfemEleTri3N records).  Element order: each split quad's two triangles in
    its place; algorithm types carry over."""
    X, el = mesh.X, mesh.elems
    cent = X[el - 1].mean(axis=1)
    pick = np.ones(len(el), dtype=bool) if select is None else np.asarray(select(cent), dtype=bool)
    rows, algo = [], []
    for e in range(len(el)):
        a, b, c, d = (int(v) for v in el[e])
        if not pick[e]:
            rows.append([a, b, c, d])
            algo.append(mesh.algo[e])
            continue
        if e % 2 == 0:
            rows += [[a, b, c, c], [a, c, d, d]]
        else:
            rows += [[a, b, d, d], [b, c, d, d]]
        algo += [mesh.algo[e], mesh.algo[e]]
    return dataclasses.replace(mesh, elems=np.array(rows, dtype=np.int64), algo=np.array(algo, dtype=np.int64))


def fc1_bench_case(n: int = 201, nsteps: int = 15):
    """FC 1 crack growth: n x n-node FE plate (30 mm), edge pre-crack to 0.41 W,
    K_Ic = 1 MPa m^0.5, top edge pulled 1e-6 m per load step, default FC 1
    (mr 6, dcf 1), reaction forces of the pulled edge; returns (mesh, write_case
    keywords).  At n = 201 the crack first grows at increment 5."""
    mesh = plate_edge_crack(n=n, KIc=1.0e6, title="pe201" if n == 201 else f"pe{n}")
    mesh.ebcs[2].velocity = 1e-6
    kw = dict(solver="QUASI-STATIC", dt=1.0, nsteps=nsteps, save=nsteps, factor=3.015, nlf=1.0, lumped=False,
              fc="1", extra=["RF 2", "SOLVE BICGSTAB 1e-10 20000"])
    return mesh, kw


def box_hole(nx: int = 121, ny: int = 61, nz: int = 21, h: float = 1e-3,
             radius: float = 8e-3, pd_x: int = 40, pd_y: int = 40,
             title: str = "boxHole") -> Mesh:
    """Hex8 box with a central cylindrical hole and a pd_x x pd_y element PD zone."""
    cx = (nx - 1) * h / 2.0
    cy = (ny - 1) * h / 2.0
    x0 = cx - pd_x * h / 2.0; x1 = cx + pd_x * h / 2.0
    y0 = cy - pd_y * h / 2.0; y1 = cy + pd_y * h / 2.0

    def pd_mask(cent):
        return (cent[:, 0] > x0) & (cent[:, 0] < x1) & (cent[:, 1] > y0) & (cent[:, 1] < y1)

    return box3d(nx, ny, nz, h, pd_mask=pd_mask, hole=(cx, cy, radius), title=title)


# Time steps are 0.8 x the stable central-difference step 2/sqrt(lambda_max(M^-1 K)),
# lambda_max from 200-300 power iterations (Rayleigh quotient, seed 0) on the
# FP64 internal force of each mesh: C1 8.99e-8 s, C2 1.69e-7 s.
def config_c1(n: int = 101, nsteps: int = 1000):
    """2D explicit: 101x101-node 50 mm plate, central PD strip, 10 mm edge pre-crack, FP64."""
    mesh = plate_strip_crack(n=n, L=0.05, title="plateStripC1")
    mesh.ebcs[2].velocity = 0.05
    h = 0.05 / (n - 1)
    dt = 0.8 * 8.99e-8 * (h / 5e-4)
    return mesh, dict(solver="DYNAMIC", dt=dt, nsteps=nsteps, save=max(1, nsteps), factor=3.015, nlf=1.0,
                      fc="3 1e-3", precision="FP64")


def config_c3(n: int = 401, nsteps: int = 50):
    """2D quasi-static: 401x401-node 200 mm plate (h = 0.5 mm), PD band over the middle 30% of the
    width, 40 mm (0.2 W) edge pre-crack, top edge pulled by 1e-6 m (dt * velocity; the reference's
    quasi-static rule applies it at the first increment and holds it), s0 = 1e-3, FP64."""
    L = 0.2 * (n - 1) / 400
    mesh = plate_strip_crack(n=n, L=L, strip_frac=0.3, crack_len=0.2 * L, title="plateStripC3")
    mesh.ebcs[2].velocity = 1e-6
    return mesh, dict(solver="QUASI-STATIC", dt=1.0, nsteps=nsteps, save=max(1, nsteps), factor=3.015, nlf=1.0,
                      fc="3 1e-3", precision="FP64")


def config_c2(nx: int = 121, ny: int = 61, nz: int = 21, nsteps: int = 5000, precision: str = "MIXED"):
    """3D explicit: 120x60x20 mm Hex8 box, 8 mm hole, 40x40 PD zone, s0 = 2e-3 +-5% per bond."""
    mesh = box_hole(nx=nx, ny=ny, nz=nz, h=1e-3, radius=8e-3, pd_x=40, pd_y=40, title="boxHoleC2")
    return mesh, dict(solver="DYNAMIC", dt=0.8 * 1.69e-7, nsteps=nsteps, save=max(1, nsteps), factor=3.015,
                      nlf=1.0, fc="3 2e-3 0 0.05", precision=precision)


def _segment_distance(p: np.ndarray, a: np.ndarray, b: np.ndarray) -> np.ndarray:
    ab = b - a
    t = np.clip(((p - a) @ ab) / (ab @ ab), 0.0, 1.0)
    return np.linalg.norm(p - (a + t[:, None] * ab), axis=1)


def config_c4(n_spec: int = 256, seed: int = 0, nsteps: int = 2000, precision: str = "MIXED",
              size_range: Tuple[int, int] = (60, 300), h: float = 5e-4, rho: float = 7850.0, nu: float = 0.25):
    """Batched 2D explicit: n_spec plates of uneven size, each with a hole or an edge pre-crack.

    Per specimen, from one seeded generator: node count uniform in
    [size_range[0]^2, size_range[1]^2] (square plate, side rounded), a central
    hole of radius 5-20 % of the width or an edge pre-crack at mid-height of
    length 5-40 % of the width (half an element above a node row), a PD zone
    of the elements within 10 h of the defect, E uniform in 50-210 GPa and s0
    uniform in 5e-4-3e-3.  Bottom edge fixed, top edge pulled at 0.05 m/s,
    dt = 0.8 x the stable step (the C1 estimate scaled by h and wave speed).
    Returns a list of (mesh, command keywords)."""
    rng = np.random.default_rng(seed)
    lo, hi = size_range
    c_ref = np.sqrt(72e9 / 2440.0)
    out = []
    for i in range(n_spec):
        count = int(rng.integers(lo * lo, hi * hi + 1))
        n = int(np.clip(round(np.sqrt(count)), lo, hi))
        W = (n - 1) * h
        E = float(rng.uniform(50e9, 210e9))
        s0 = float(rng.uniform(5e-4, 3e-3))
        use_hole = bool(rng.random() < 0.5)
        frac = float(rng.uniform(0.05, 0.20) if use_hole else rng.uniform(0.05, 0.40))
        cx = cy = W / 2.0
        cracks = []
        hole = None
        if use_hole:
            r = frac * W
            hole = (cx, cy, r)

            def pd_mask(cent, r=r):
                d = np.hypot(cent[:, 0] - cx, cent[:, 1] - cy)
                return d < r + 10.0 * h
        else:
            a = frac * W
            yc = (n - 1) // 2 * h + 0.5 * h
            p0 = np.array([0.25 * h, yc]); p1 = np.array([0.25 * h + a, yc])
            cracks = [np.array([[p0[0], p0[1], 0.0], [p1[0], p1[1], 0.0]])]

            def pd_mask(cent, p0=p0, p1=p1):
                return _segment_distance(cent[:, :2], p0, p1) < 10.0 * h
        mesh = plate2d(n, n, h, pd_mask=pd_mask, hole=hole, cracks=cracks, title=f"c4_{i:03d}",
                       material=(E, nu, rho, 1.0e6, 1.0e8), top_velocity=0.05)
        dt = 0.8 * 8.99e-8 * (h / 5e-4) * c_ref / np.sqrt(E / rho)
        out.append((mesh, dict(solver="DYNAMIC", dt=dt, nsteps=nsteps, save=max(1, nsteps), factor=3.015, nlf=1.0,
                               fc=f"3 {s0:.6e}", precision=precision)))
    return out


def penny_crack_box(nx: int = 201, ny: int = 101, nz: int = 41, h: float = 1e-3, radius_h: float = 10.0,
                    tilt_deg: float = 30.0, n_tri: int = 16, pd_frac: float = 0.05, title: str = "pennyBox") -> Mesh:
    """Hex8 box with an inclined penny crack (a fan of n_tri triangles, radius radius_h * h) at its centre,
    tilted by tilt_deg about the y axis, and a PD zone of the elements closest to the crack disk
    (pd_frac of all elements).  The crack centre sits at an element centre, so no node lies on it."""
    c = np.array([(nx - 1) * h / 2 + 0.5 * h, (ny - 1) * h / 2 + 0.5 * h, (nz - 1) * h / 2 + 0.5 * h])
    t = np.radians(tilt_deg)
    nrm = np.array([np.sin(t), 0.0, np.cos(t)])
    a1 = np.array([np.cos(t), 0.0, -np.sin(t)])
    a2 = np.array([0.0, 1.0, 0.0])
    r = radius_h * h
    th = np.linspace(0.0, 2 * np.pi, n_tri + 1)
    rim = [c + r * (np.cos(q) * a1 + np.sin(q) * a2) for q in th]
    cracks = [np.array([c, rim[j], rim[j + 1]]) for j in range(n_tri)]

    def disk_distance(p):
        d = p - c
        z = d @ nrm
        inplane = d - np.outer(z, nrm)
        rho = np.linalg.norm(inplane, axis=1)
        return np.hypot(z, np.maximum(rho - r, 0.0))

    n_el = (nx - 1) * (ny - 1) * (nz - 1)
    _, _, centers = grid3d(nx, ny, nz, h)
    dist = disk_distance(centers)
    k = min(n_el - 1, int(pd_frac * n_el))
    cut = np.partition(dist, k)[k]

    def pd_mask(cent):
        return disk_distance(cent) <= cut

    return box3d(nx, ny, nz, h, pd_mask=pd_mask, cracks=cracks, title=title)


def config_c5(nx: int = 201, ny: int = 101, nz: int = 41, nsteps: int = 200, dt_factor: float = 20.0,
              radius_h: float = 10.0, n_tri: int = 16):
    """3D implicit Newmark (beta 0.25, gamma 0.5): 200x100x40 Hex8 box, 5 % PD zone around an inclined penny
    crack of radius 10 h, x faces pulled at 0.1 m/s.  dt = dt_factor x 0.8 x the explicit stable step (the C2
    estimate at h = 1 mm): an implicit step much longer than an explicit one, so that K dominates K_N."""
    mesh = penny_crack_box(nx=nx, ny=ny, nz=nz, h=1e-3, radius_h=radius_h, n_tri=n_tri, title="pennyBoxC5")
    return mesh, dict(solver="DYNAMIC", dt=dt_factor * 0.8 * 1.69e-7, nsteps=nsteps, save=max(1, nsteps),
                      factor=3.015, nlf=1.0, newmark=(0.5, 0.25), precision="FP64")


CONFIGS = {"c1": config_c1, "c2": config_c2}


def write_case(mesh: Mesh, outdir: str, name: str, **cmd) -> str:
    """Write ``<name>.lis`` and ``<name>.in`` into outdir; return the command path."""
    os.makedirs(outdir, exist_ok=True)
    lis = os.path.join(outdir, name + ".lis")
    write_lis(mesh, lis)
    cmd_path = os.path.join(outdir, name + ".in")
    write_cmd(cmd_path, name + ".lis", mesh, **cmd)
    return cmd_path
