"""Coarse-grid choice of the two-level BiCGStab (pdx method 8) on C3's loaded
increment (CPU analysis; test infrastructure, not part of the product).

The quasi-static stiffness of the 401x401-node strip plate has no mass term,
so BiCGStab with Jacobi needs about 1,850 iterations to a 1e-8 residual: its
smooth error modes converge slowly.  This script assembles the loaded
increment's K and f with the C restatement (FP64; the same matrix the GPU
assembles, pdsolve.cpp:6464-6590), builds the bilinear prolongation P of a
lattice coarse grid over the nodes' bounding box (per DOF component, as the
product does), and counts SciPy BiCGStab iterations to 1e-8 with Jacobi alone
and with Jacobi plus the exact Galerkin correction P (P^T K P)^-1 P^T
(additive, dense LU of the coarse matrix) for each coarse grid given.

    python oracle/twolevel_study.py [20x20 40x40 ...] [--no-jacobi] [--n 401]

--n sets the plate's nodes per side (the C3 configuration has 401).  Prints
one JSON line per preconditioner.
"""
from __future__ import annotations

import json
import os
import sys
import tempfile
import time

import numpy as np
import scipy.linalg as sla
import scipy.sparse as sp
import scipy.sparse.linalg as spla

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path[:0] = [HERE, os.path.join(os.path.dirname(HERE), "pdlsm-fem_mpi_gb300")]
import meshgen  # noqa: E402
import orc  # noqa: E402
import pdx  # noqa: E402


def prolongation2d(X: np.ndarray, eq: np.ndarray, cells, n: int) -> sp.csr_matrix:
    """Bilinear interpolation from the nodes of a grid of `cells` over the
    bounding box, per DOF component; empty coarse columns dropped."""
    D = 2
    lo, hi = X.min(axis=0), X.max(axis=0)
    u = (X[:, :2] - lo[:2]) / np.where(hi[:2] > lo[:2], hi[:2] - lo[:2], 1.0) * np.asarray(cells, float)
    ci = np.clip(np.floor(u).astype(np.int64), 0, np.asarray(cells) - 1)
    t = np.clip(u - ci, 0.0, 1.0)
    nxn = cells[0] + 1
    nc = (cells[0] + 1) * (cells[1] + 1) * D
    rows, cols, vals = [], [], []
    eqn = eq.reshape(-1, D)
    for corner in range(4):
        dx, dy = corner & 1, (corner >> 1) & 1
        w = np.where(dx, t[:, 0], 1 - t[:, 0]) * np.where(dy, t[:, 1], 1 - t[:, 1])
        node = (ci[:, 0] + dx) + nxn * (ci[:, 1] + dy)
        for i in range(D):
            e = eqn[:, i]
            ok = (e >= 0) & (w != 0)
            rows.append(e[ok]); cols.append(node[ok] * D + i); vals.append(w[ok])
    P = sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))), shape=(n, nc))
    keep = np.asarray((abs(P).sum(axis=0) > 0)).ravel()
    return P[:, keep].tocsr()


def main() -> None:
    argv = sys.argv[1:]
    nside = 401
    if "--n" in argv:
        i = argv.index("--n")
        nside = int(argv[i + 1])
        del argv[i:i + 2]
    args = [a for a in argv if not a.startswith("--")]
    cells_list = [tuple(int(c) for c in a.split("x")) for a in args] or [(20, 20)]
    d = tempfile.mkdtemp(prefix="pdx_twolevel_")
    mesh, kw = meshgen.config_c3(n=nside, nsteps=2)
    cmd = meshgen.write_case(mesh, d, "c3", **kw)
    host = pdx.Model(cmd, device=-1)
    o = orc.Oracle(host)
    eq = host.array("eq").reshape(-1)
    n = host.info.n_eq
    # the loaded increment: the prescribed DOFs at dt * v (quasi-static rule), the rest at 0
    u_all = host.array("u0").reshape(-1) + host.array("dtv").reshape(-1, 3)[:, :2].reshape(-1) * (eq < 0)
    ia, ja, K, f = o.assemble(u_all)
    A = sp.csr_matrix((K, ja, ia), shape=(n, n))
    dinv = 1.0 / A.diagonal()
    X = host.array("X").reshape(-1, 3)

    def run(M, name):
        its = [0]

        def cb(_):
            its[0] += 1
        t = time.time()
        x, info = spla.bicgstab(A, f, rtol=1e-8, maxiter=5000, M=M, callback=cb)
        res = float(np.linalg.norm(f - A @ x) / np.linalg.norm(f))
        print(json.dumps(dict(preconditioner=name, iterations=its[0], info=int(info), residual=res,
                              cpu_s=round(time.time() - t, 1))), flush=True)

    if "--no-jacobi" not in sys.argv:
        run(spla.LinearOperator((n, n), matvec=lambda r: dinv * r), "jacobi")
    for cells in cells_list:
        P = prolongation2d(X, eq, cells, n)
        lu = sla.lu_factor((P.T @ (A @ P)).toarray())
        M = spla.LinearOperator((n, n), matvec=lambda r, P=P, lu=lu: dinv * r + P @ sla.lu_solve(lu, P.T @ r))
        run(M, f"jacobi + galerkin {cells[0]}x{cells[1]} ({P.shape[1]} coarse DOFs)")


if __name__ == "__main__":
    main()
