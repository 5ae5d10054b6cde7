"""Host set-up of a model for the oracle, independent of the product library.
Test infrastructure (the checker's own input path), not part of the product.

Restates, in Python/numpy:
  the mesh reader      datModel::readdata         SourceFiles/Solver/datModel.cpp:58-326
  the command reader   fioFiles::CMDfile/excuteCMD fioFile.cpp:54-462 (defaults datModel.cpp:17-52)
  pdsolve::setDatModel (pdsolve.cpp:114-151):
    DOF numbering       Setdof_Index             pdsolve.cpp:241-268
    volumes, min/max    setDeltaMaxMin_EleV_NV   :367-439 (element volumes of pdfemEle*::eleVolume)
    domain box, blocks  findDomainDimen, setBlock :153-195, :441-502
    PD/FE split, cracks initializePDE_FE, updatePDEbyCrack, b_eleIntersectCrack :504-822
    PDBEs, node types   updatePDBE, UpdateNodeType :1221-1440
    families            initialPDN_Fami          :1442-1568 (union rule)
    pre-crack bonds     updateBondstate, intersection, segmentPlaneIntersection :8910-9079, :1123-1210
and the prescribed-DOF arrays the oracle's explicit loop reads.  Floating-point
expressions that decide membership are evaluated in the reference's order
(elementwise numpy arithmetic, no fused multiply-add), so the arrays equal the
reference's set-up dumps bit for bit.

load(cmd_path) returns an object with the .array(name) / .info interface that
orc.Oracle reads.
"""
from __future__ import annotations

import math
import os
from types import SimpleNamespace

import numpy as np


class _Stream:
    """C++ stream semantics over a text: tok() is `>>`, getline() is std::getline."""

    def __init__(self, text: str):
        self.s, self.i = text, 0

    def tok(self) -> str:
        s, i, n = self.s, self.i, len(self.s)
        while i < n and s[i].isspace():
            i += 1
        j = i
        while j < n and not s[j].isspace():
            j += 1
        self.i = j
        if i == j:
            raise ValueError("unexpected end of mesh file")
        return s[i:j]

    def getline(self) -> str:
        j = self.s.find("\n", self.i)
        j = len(self.s) if j < 0 else j
        line, self.i = self.s[self.i:j], min(j + 1, len(self.s))
        return line


def read_mesh(path: str) -> SimpleNamespace:
    st = _Stream(open(path).read())
    m = SimpleNamespace()
    m.title = st.tok()
    st.getline(); st.getline()
    sdim = st.tok()
    m.protype = int(st.tok())
    m.E, m.nu, m.rho, m.KIc, m.sigult = (float(st.tok()) for _ in range(5))
    m.dim = {"2D": 2, "3D": 3}[sdim]
    m.n_node, m.n_elem = int(st.tok()), int(st.tok())
    X = np.zeros((m.n_node, 3))
    for _ in range(m.n_node):
        nid = int(st.tok())
        X[nid - 1] = [float(st.tok()) for _ in range(3)]
    m.X = X
    nen = 4 if m.dim == 2 else 8
    conn = -np.ones((m.n_elem, 8), dtype=np.int64)
    nn = np.zeros(m.n_elem, dtype=np.int64)
    algo = np.zeros(m.n_elem, dtype=np.int64)
    for e in range(m.n_elem):
        st.tok()
        algo[e] = int(st.tok())
        ids = [int(st.tok()) for _ in range(nen)]
        if m.dim == 3 and not (ids[2] != ids[3] and ids[4] != ids[5]):
            raise NotImplementedError("tetrahedral elements")
        k = 3 if m.dim == 2 and ids[3] == ids[2] else nen
        nn[e] = k
        conn[e, :k] = np.array(ids[:k]) - 1
    m.conn, m.elem_nn, m.algo = conn, nn, algo
    st.getline(); st.getline()
    nebc = int(st.tok())
    heads = [(int(st.tok()), st.tok(), float(st.tok())) for _ in range(nebc)]
    m.ebcs = []
    for cnt, sd, val in heads:
        nodes = np.array([int(st.tok()) - 1 for _ in range(cnt)], dtype=np.int64)
        m.ebcs.append(SimpleNamespace(dof={"UX": 0, "UY": 1, "UZ": 2}[sd], value=val, nodes=nodes,
                                      varying=False, velocity=0.0))
    st.getline(); st.getline()
    nnbc = int(st.tok())
    heads = [(int(st.tok()), float(st.tok())) for _ in range(nnbc)]
    tn = 2 if m.dim == 2 else 4
    m.nbcs = []
    for cnt, val in heads:
        el = [[int(st.tok()) - 1 for _ in range(tn)] for _ in range(cnt)]
        m.nbcs.append(SimpleNamespace(value=val, elems=el, varying=False, velocity=0.0))
    st.getline(); st.getline()
    nnf = int(st.tok())
    for _ in range(nnf):
        st.tok()
    st.getline(); st.getline()
    ncr = int(st.tok())
    npt = 3 if m.dim == 3 else 2
    m.cracks = [np.array([[float(st.tok()) for _ in range(3)] for _ in range(npt)]) for _ in range(ncr)]
    return m


def read_command(path: str):
    c = SimpleNamespace(solver=-1, dt=1.0, nsteps=1, factor=3.0, nlf=0.33, me=0.0, fail_flag=0, s0=0.0,
                        s0_seed=0, s0_pert=0.0, mr=6.0, dcf=1.0)
    mesh = None
    base = os.path.dirname(path) or "."
    for line in open(path):
        t = line.split()
        if not t or t[0].startswith("#"):
            continue
        k = t[0]
        if k == "MSHFILE":
            p = t[1] if os.path.exists(t[1]) or t[1].startswith("/") else os.path.join(base, t[1])
            mesh = read_mesh(p)
        elif k == "SOLVER":
            c.solver = {"DYNAMIC": 0, "STATIC": 1, "QUASI-STATIC": 2}[t[1]]
        elif k == "SETSOLVING" and len(t) >= 6:
            c.dt = 1.0 if c.solver == 2 else float(t[1])
            c.nsteps, c.factor, c.nlf = int(t[2]), float(t[4]), float(t[5])
            if len(t) > 6:
                c.me = float(t[6])
        elif k in ("EBC", "VEBC") and mesh is not None and len(t) >= 3:
            i = int(t[1])
            if 0 <= i < len(mesh.ebcs):
                if k == "VEBC":
                    mesh.ebcs[i].varying, mesh.ebcs[i].velocity = True, float(t[2])
                else:
                    mesh.ebcs[i].value = float(t[2])
        elif k in ("NBC", "VNBC") and mesh is not None and len(t) >= 3:
            i = int(t[1])
            if 0 <= i < len(mesh.nbcs):
                if k == "VNBC":
                    mesh.nbcs[i].varying, mesh.nbcs[i].velocity = True, float(t[2])
                else:
                    mesh.nbcs[i].value = float(t[2])
        elif k == "FC" and len(t) >= 2:
            f = int(t[1])
            c.fail_flag = f
            if f == 1 and len(t) > 3:
                c.mr, c.dcf = float(t[2]), float(t[3])
            if f == 3 and len(t) < 3:
                c.fail_flag = 0            # a bare FC 3 breaks nothing, as the reference
            elif f == 3:
                c.s0 = float(t[2])
                c.s0_seed = int(t[3]) if len(t) > 3 else 0
                c.s0_pert = float(t[4]) if len(t) > 4 else 0.0
    return mesh, c


def _det33(m):
    """pdfemEles::detMat33 order: wrapped diagonals minus anti-diagonals; m is (..., 3, 3)."""
    det = 0.0
    for i in range(3):
        a1 = 1.0
        a2 = 1.0
        for j in range(3):
            a1 = a1 * m[..., j, (i + j) % 3]
            a2 = a2 * m[..., j, (i - j + 3) % 3]
        det = det + a1 - a2
    return det


_KG = 1.0 / math.sqrt(3.0)
_PI = np.array([-1, 1, 1, -1, -1, 1, 1, -1], dtype=np.float64)
_QI = np.array([-1, -1, 1, 1, -1, -1, 1, 1], dtype=np.float64)
_RI = np.array([-1, -1, -1, -1, 1, 1, 1, 1], dtype=np.float64)


def _volumes(m):
    X, conn, nn = m.X, m.conn, m.elem_nn
    V = np.zeros(m.n_elem)
    if m.dim == 2:
        xN = X[np.where(conn >= 0, conn, 0)]                   # (E, 8, 3)
        one = np.ones(m.n_elem)

        def tri(a, b, c):
            mat = np.stack([np.stack([one, xN[:, a, 0], xN[:, a, 1]], -1),
                            np.stack([one, xN[:, b, 0], xN[:, b, 1]], -1),
                            np.stack([one, xN[:, c, 0], xN[:, c, 1]], -1)], 1)
            return 0.5 * np.abs(_det33(mat))
        a1 = tri(0, 1, 2)
        a2 = tri(2, 3, 0)
        return np.where(nn == 3, a1, a1 + a2)
    xN = X[conn]                                              # (E, 8, 3)
    g = (-_KG, _KG)
    for p in g:
        for q in g:
            for r in g:
                dN0 = 0.125 * _PI * (1 + q * _QI) * (1 + r * _RI)
                dN1 = 0.125 * _QI * (1 + p * _PI) * (1 + r * _RI)
                dN2 = 0.125 * _RI * (1 + p * _PI) * (1 + q * _QI)
                J = np.zeros((m.n_elem, 3, 3))
                for c in range(3):
                    for i in range(8):
                        J[:, 0, c] = J[:, 0, c] + dN0[i] * xN[:, i, c]
                        J[:, 1, c] = J[:, 1, c] + dN1[i] * xN[:, i, c]
                        J[:, 2, c] = J[:, 2, c] + dN2[i] * xN[:, i, c]
                V = V + _det33(J)
    return V


def _centres(m):
    X, conn, nn = m.X, m.conn, m.elem_nn
    c = np.zeros((m.n_elem, 3))
    if m.dim == 2:
        quad = nn == 4
        for j in range(4):
            c[quad] = c[quad] + X[conn[quad, j]] * 0.25
        tri = ~quad
        c[tri] = (X[conn[tri, 0]] + X[conn[tri, 1]] + X[conn[tri, 2]]) / 3.0
    else:
        for j in range(8):
            c = c + X[conn[:, j]] * 0.125
    return c


def _seg2d(a1, a2, b1, b2):
    """intersection (pdsolve.cpp:9058-9079); a1, a2 arrays (n, 2+), b1, b2 points."""
    out = ~((np.maximum(a1[:, 0], a2[:, 0]) < min(b1[0], b2[0])) |
            (np.maximum(a1[:, 1], a2[:, 1]) < min(b1[1], b2[1])) |
            (max(b1[0], b2[0]) < np.minimum(a1[:, 0], a2[:, 0])) |
            (max(b1[1], b2[1]) < np.minimum(a1[:, 1], a2[:, 1])))
    t1 = (((a1[:, 0] - b1[0]) * (b2[1] - b1[1]) - (a1[:, 1] - b1[1]) * (b2[0] - b1[0])) *
          ((a2[:, 0] - b1[0]) * (b2[1] - b1[1]) - (a2[:, 1] - b1[1]) * (b2[0] - b1[0])))
    t2 = (((b1[0] - a1[:, 0]) * (a2[:, 1] - a1[:, 1]) - (b1[1] - a1[:, 1]) * (a2[:, 0] - a1[:, 0])) *
          ((b2[0] - a1[:, 0]) * (a2[:, 1] - a1[:, 1]) - (b2[1] - a1[:, 1]) * (a2[:, 0] - a1[:, 0])))
    return out & ~(t1 > 0) & ~(t2 > 0)


def _cross(a, b):
    return np.stack([a[..., 1] * b[..., 2] - a[..., 2] * b[..., 1], a[..., 2] * b[..., 0] - a[..., 0] * b[..., 2],
                     a[..., 0] * b[..., 1] - a[..., 1] * b[..., 0]], -1)


def _seg_tri(p1, p2, t):
    """segmentPlaneIntersection (pdsolve.cpp:1123-1210); p1, p2 (n, 3), t (3, 3)."""
    nrm = _cross(t[1] - t[0], t[2] - t[0])
    v1, v2 = p1 - t[0], p2 - t[0]
    t1 = v1[:, 0] * nrm[0] + v1[:, 1] * nrm[1] + v1[:, 2] * nrm[2]
    t2 = v2[:, 0] * nrm[0] + v2[:, 1] * nrm[1] + v2[:, 2] * nrm[2]
    res = np.zeros(len(p1), dtype=bool)
    on = t1 * t2 == 0
    res[on] = True
    go = ~(t1 * t2 > 0) & ~on
    if go.any():
        w1, w2 = t[0] - p1[go], p2[go] - p1[go]
        d = (w1[:, 0] * nrm[0] + w1[:, 1] * nrm[1] + w1[:, 2] * nrm[2]) / \
            (w2[:, 0] * nrm[0] + w2[:, 1] * nrm[1] + w2[:, 2] * nrm[2])
        xs = p1[go] + d[:, None] * w2
        A = math.sqrt(nrm[0] * nrm[0] + nrm[1] * nrm[1] + nrm[2] * nrm[2])

        def area(a, b):
            n2 = _cross(a, b)
            return np.sqrt(n2[:, 0] * n2[:, 0] + n2[:, 1] * n2[:, 1] + n2[:, 2] * n2[:, 2])
        A0 = area(t[1] - xs, t[2] - xs)
        A1 = area(xs - t[0], np.broadcast_to(t[2] - t[0], xs.shape))
        A2 = area(np.broadcast_to(t[1] - t[0], xs.shape), xs - t[0])
        res[go] = ~(np.abs(A0 + A1 + A2 - A) > A * 1.0e-14)
    return res


def build(mesh, cmd) -> dict:
    m, c = mesh, cmd
    D, N, E = m.dim, m.n_node, m.n_elem
    active = np.ones((N, D), dtype=bool)
    for b in m.ebcs:
        active[b.nodes, b.dof] = False
    eq = -np.ones(N * D, dtype=np.int64)
    eq[active.reshape(-1)] = np.arange(int(active.sum()))
    vol_elem = _volumes(m)
    vol_node = np.zeros(N)
    for e in range(E):                                      # element order, as the reference adds
        k = m.elem_nn[e]
        vol_node[m.conn[e, :k]] += vol_elem[e] / k
    # C's pow (math.pow), as the reference: numpy's vectorised power may differ in the last bit
    min_delta = math.pow(float(vol_elem.min()), 1.0 / D)
    max_delta = math.pow(float(vol_elem.max()), 1.0 / D)
    lbc, rtc = m.X[0].copy(), m.X[0].copy()
    for j in range(D):
        lbc[j], rtc[j] = m.X[:, j].min(), m.X[:, j].max()
        lbc[j] = lbc[j] - 1.0e-14 * abs(lbc[j])
        rtc[j] = rtc[j] + 1.0e-14 * abs(rtc[j])
    bs = 2.5 * c.factor * min_delta
    nb = [int((rtc[i] - lbc[i]) / bs + 1) for i in range(3)]
    if D == 2:
        nb[2] = 1

    def bidx(x):
        ib = ((x - lbc) / bs).astype(np.int64)
        return ib, ib[..., 0] + ib[..., 1] * nb[0] + ib[..., 2] * nb[0] * nb[1]
    cen = _centres(m)
    _, eb = bidx(cen)
    nib, nbk = bidx(m.X)
    nblk = nb[0] * nb[1] * nb[2]
    block_elems = [[] for _ in range(nblk)]
    for e in range(E):
        block_elems[eb[e]].append(e)
    block_nodes = [[] for _ in range(nblk)]
    for k in range(N):
        block_nodes[nbk[k]].append(k)
    block_nodes = [np.array(b, dtype=np.int64) for b in block_nodes]

    def blocks_around(lo, hi):
        out = []
        for x in range(lo[0] - 1, hi[0] + 2):
            for y in range(lo[1] - 1, hi[1] + 2):
                for z in range(lo[2] - 1, hi[2] + 2):
                    if 0 <= x < nb[0] and 0 <= y < nb[1] and 0 <= z < nb[2]:
                        out.append(x + y * nb[0] + z * nb[0] * nb[1])
        return out

    def crack_range(cr):
        npt = D
        lo = [int((cr[:npt, k].min() - lbc[k]) / bs) for k in range(3)]
        hi = [int((cr[:npt, k].max() - lbc[k]) / bs) for k in range(3)]
        if D == 2:
            lo[2] = hi[2] = 0
        return lo, hi

    edges3 = [(0, 1), (1, 2), (2, 3), (3, 0), (4, 5), (5, 6), (6, 7), (7, 4), (0, 4), (1, 5), (2, 6), (3, 7)]

    def cut(e, cr):
        k = m.elem_nn[e]
        if D == 2:
            a = m.X[[m.conn[e, i] for i in range(k)]]
            b = m.X[[m.conn[e, (i + 1) % k] for i in range(k)]]
            return bool(_seg2d(a, b, cr[0], cr[1]).any())
        a = m.X[[m.conn[e, i] for i, _ in edges3]]
        b = m.X[[m.conn[e, j] for _, j in edges3]]
        return bool(_seg_tri(a, b, cr).any())
    algo = m.algo.copy()
    pde = [e for e in range(E) if algo[e] == 1]
    crack_elems = []
    for cr in m.cracks:
        old = len(crack_elems)
        lo, hi = crack_range(cr)
        for bi in blocks_around(lo, hi):
            for e in block_elems[bi]:
                if cut(e, cr) and e not in crack_elems:
                    crack_elems.append(e)
        new = crack_elems[old:]
        if not new:
            raise ValueError("a pre-existing crack cuts no element")
        cc = cen[new]
        mn, mx = cc.min(axis=0), cc.max(axis=0)
        blo = [int((mn[i] - lbc[i]) / bs) for i in range(3)]
        bhi = [int((mx[i] - lbc[i]) / bs) for i in range(3)]
        mf = c.me + 1e-15
        rsq = min_delta * min_delta * mf * mf
        for bi in blocks_around(blo, bhi):
            for e in block_elems[bi]:
                if algo[e] != 2:
                    continue
                d = cen[e] - cc
                dis = (d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]) + d[:, 2] * d[:, 2]
                if (dis < rsq).any():
                    algo[e] = 1
                    pde.append(e)
    fe = [e for e in range(E) if algo[e] == 2]
    # PDBEs: edges (2D) / faces (3D) of PD elements not shared by two of them
    lst = []
    for e in pde:
        cn = m.conn[e]
        if D == 2:
            k = m.elem_nn[e]
            for j in range(k):
                a, b = int(cn[j]), int(cn[(j + 1) % k])
                lst.append((a, b, 1, 0, 0) if a < b else (b, a, -1, 0, 0))
        else:
            faces = [(cn[0], cn[1], cn[2], cn[3]), (cn[4], cn[5], cn[6], cn[7]), (cn[0], cn[3], cn[7], cn[4]),
                     (cn[1], cn[2], cn[6], cn[5]), (cn[0], cn[4], cn[5], cn[1]), (cn[3], cn[7], cn[6], cn[2])]
            sgn = [-1, 1, -1, 1, -1, 1]
            for f, s in zip(faces, sgn):
                f = [int(v) for v in f]
                pos = f.index(min(f))
                lst.append((f[pos], f[(pos + 1) % 4], f[(pos + 2) % 4], f[(pos + 3) % 4], s))
    lst.sort(key=lambda r: r[0])                              # stable, by first node
    dead = [False] * len(lst)
    for i in range(len(lst)):
        if dead[i]:
            continue
        j = i + 1
        while j < len(lst) and lst[j][0] == lst[i][0]:
            if not dead[j]:
                same = lst[j][1] == lst[i][1] if D == 2 else lst[j][1:4] == lst[i][1:4]
                if same:
                    dead[i] = dead[j] = True
                    break
            j += 1
    pdbe = []
    for i, a in enumerate(lst):
        if dead[i]:
            continue
        if D == 2:
            pdbe.append([a[0], a[1], -1, -1] if a[2] == 1 else [a[1], a[0], -1, -1])
        else:
            pdbe.append([a[0], a[1], a[2], a[3]] if a[4] == 1 else [a[3], a[2], a[1], a[0]])
    node_type = np.zeros(N, dtype=np.int64)
    for e in pde:
        node_type[m.conn[e, :m.elem_nn[e]]] = 2
    for b in pdbe:
        node_type[b[:2 if D == 2 else 4]] = 1
    fam_node = np.nonzero(node_type)[0]
    fam_of = -np.ones(N, dtype=np.int64)
    fam_of[fam_node] = np.arange(len(fam_node))
    delta_node = np.array([c.factor * math.pow(float(v), 1.0 / D) for v in vol_node])
    fam_delta = delta_node[fam_node]
    fam_cdv = np.zeros(len(fam_node))
    for e in pde:
        k = m.elem_nn[e]
        dv = vol_elem[e]
        for a in m.conn[e, :k]:
            f = fam_of[a]
            fam_cdv[f] = fam_cdv[f] + dv / k
    # families: per block of family nodes, the candidates of the 27 blocks around it in scan order
    md = min_delta
    eps = md * md * 1.0e-16
    members = [None] * len(fam_node)
    by_block = {}
    for f, k in enumerate(fam_node):
        by_block.setdefault(int(nbk[k]), []).append(f)
    for bi, fams in by_block.items():
        ib = nib[fam_node[fams[0]]]
        cand = np.concatenate([block_nodes[b] for b in blocks_around(ib, ib)])
        xm = m.X[cand]
        dj2 = delta_node[cand] * delta_node[cand]
        for f in fams:
            k = fam_node[f]
            xk = m.X[k]
            d = xm - xk
            dist = (d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]) + d[:, 2] * d[:, 2]
            dk = fam_delta[f]
            keep = (dist > eps) & ((dist < (dk * dk + eps)) | (dist < (dj2 + eps)))
            members[f] = np.concatenate([[k], cand[keep]])
    fam_off = np.zeros(len(fam_node) + 1, dtype=np.int64)
    fam_off[1:] = np.cumsum([len(v) for v in members])
    fam_members = np.concatenate(members).astype(np.int64) if members else np.zeros(0, dtype=np.int64)
    bond_state = np.ones(len(fam_members), dtype=np.uint8)
    for cr in m.cracks:
        lo, hi = crack_range(cr)
        for bi in blocks_around(lo, hi):
            for node in block_nodes[bi]:
                f = fam_of[node]
                if f < 0:
                    continue
                q = np.arange(fam_off[f] + 1, fam_off[f + 1])
                q = q[bond_state[q] == 1]
                if not len(q):
                    continue
                k = fam_node[f]
                pk = np.broadcast_to(m.X[k], (len(q), 3))
                pm = m.X[fam_members[q]]
                hit = _seg_tri(pk, pm, cr) if D == 3 else _seg2d(pk, pm, cr[0], cr[1])
                bond_state[q[hit]] = 0
    u0 = np.zeros(N * D)
    bcflag = np.zeros(N, dtype=np.uint8)
    dtv = np.zeros(N * 3)
    for b in m.ebcs:
        u0[b.nodes * D + b.dof] = b.value
        if b.varying:
            bcflag[b.nodes] |= np.uint8(1 << b.dof)
            dtv[b.nodes * 3 + b.dof] = c.dt * b.velocity
    for i in range(D):
        bcflag[eq.reshape(N, D)[:, i] < 0] |= np.uint8(1 << (4 + i))
    material = np.array([m.E, m.nu, m.rho, m.KIc, m.sigult, c.nlf, c.factor, float(m.protype), c.dt,
                         float(c.nsteps), c.s0, float(c.s0_seed), c.s0_pert])
    geom = np.array([min_delta, max_delta, bs, *lbc, *rtc])
    return {"X": m.X.reshape(-1), "conn": m.conn.astype(np.int32).reshape(-1), "elem_nn": m.elem_nn.astype(np.int32),
            "fe_idx": np.array(fe, dtype=np.int32), "pde_idx": np.array(pde, dtype=np.int32),
            "eq": eq.astype(np.int32), "vol_node": vol_node, "vol_elem": vol_elem,
            "fam_off": fam_off, "fam_members": fam_members.astype(np.int32), "fam_horizon": fam_delta,
            "fam_cdv": fam_cdv, "pdbe": np.array(pdbe, dtype=np.int32).reshape(-1, 4),
            "node_type": node_type.astype(np.int32), "bond_state0": bond_state, "u0": u0, "bcflag": bcflag,
            "dtv": dtv, "material": material, "geom": geom,
            "csr_ia": np.zeros(0, dtype=np.int64), "csr_ja": np.zeros(0, dtype=np.int64)}


def csr_pattern(mesh, a: dict):
    """setCSRIndexes_gloStiffMat (pdsolve.cpp:959-1121): node k's rows hold the
    columns of its own family members and of the nodes of the FE elements
    around it, by node and then component; rows are the equations."""
    D, N = mesh.dim, mesh.n_node
    off, mem = a["fam_off"], a["fam_members"].astype(np.int64)
    nf = len(off) - 1
    rk = [np.repeat(mem[off[:-1]], np.diff(off))]
    rj = [mem]
    for e in a["fe_idx"]:
        nodes = mesh.conn[e, :mesh.elem_nn[e]]
        rk.append(np.repeat(nodes, len(nodes)))
        rj.append(np.tile(nodes, len(nodes)))
    pairs = np.unique(np.stack([np.concatenate(rk), np.concatenate(rj)], 1), axis=0) if nf or len(a["fe_idx"]) \
        else np.zeros((0, 2), dtype=np.int64)
    eq = a["eq"].astype(np.int64).reshape(N, D)
    cols = eq[pairs[:, 1]]                                     # (n_pairs, D), -1 where prescribed
    ia = np.zeros(int((eq >= 0).sum()) + 1, dtype=np.int64)
    ja = []
    start = np.searchsorted(pairs[:, 0], np.arange(N + 1))
    for k in range(N):
        c = cols[start[k]:start[k + 1]].reshape(-1)
        c = c[c >= 0]
        for d in range(D):
            r = eq[k, d]
            if r < 0:
                continue
            ja.append(c)
            ia[r + 1] = len(c)
    return np.cumsum(ia), (np.concatenate(ja) if ja else np.zeros(0, dtype=np.int64))


class HostModel:
    """The set-up arrays of a command file, with the interface orc.Oracle reads
    (the CSR pattern only with pattern=True: the explicit loop does not use it)."""

    def __init__(self, cmd_path: str, pattern: bool = False):
        mesh, cmd = read_command(cmd_path)
        self.mesh, self.cmd = mesh, cmd
        self.arrays = build(mesh, cmd)
        if pattern:
            self.arrays["csr_ia"], self.arrays["csr_ja"] = csr_pattern(mesh, self.arrays)
        a = self.arrays
        n_fam = len(a["fam_off"]) - 1
        self.info = SimpleNamespace(dim=mesh.dim, n_node=mesh.n_node, n_elem=mesh.n_elem,
                                    n_eq=int((a["eq"] >= 0).sum()), n_fam=n_fam, n_pdbe=len(a["pdbe"]),
                                    n_fe=len(a["fe_idx"]), n_bond=len(a["fam_members"]) - n_fam,
                                    fail_flag=cmd.fail_flag)
        self.dim = mesh.dim

    def array(self, name: str) -> np.ndarray:
        return self.arrays[name]


def load(cmd_path: str, pattern: bool = False) -> HostModel:
    return HostModel(cmd_path, pattern)
