"""Ceiling of a coarse correction on the C5 Newmark system (CPU analysis; test
infrastructure, not part of the product).

The learned two-level preconditioner (pdx_learned_*) adds a network's estimate
of the coarse error, P y(P^T r), to block-Jacobi inside flexible CG.  On the
same coarse grid the best such correction is the exact Galerkin one,
P (P^T A P)^-1 P^T r.  This script assembles the full C5 Newmark matrix
K_N = beta dt^2 K + M with the C restatement (FP64; the same matrix the GPU
assembles, pdsolve.cpp:6327-6397), builds the trilinear prolongation P of the
coarse grid the learned solver uses (25 x 12 x 5 cells), and counts
flexible-CG iterations to a 1e-8 relative residual for block-Jacobi alone and
for block-Jacobi plus the exact Galerkin correction, on the first Newmark
step's right-hand side and on random ones.  The ratio of the two iteration
counts bounds what any learned coarse correction on this grid can save.

    python oracle/galerkin_study.py [--size full|medium|small] [--random 2]

Prints one JSON line.  Full size needs about 15 GB of host memory.
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import tempfile
import time

import numpy as np
import scipy.linalg as sla
import scipy.sparse as sp

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path[:0] = [HERE, os.path.join(os.path.dirname(HERE), "pdlsm-fem_mpi_gb300")]
import meshgen  # noqa: E402
import orc  # noqa: E402
import pdx  # noqa: E402

SIZES = {"full": (201, 101, 41, (25, 12, 5)), "medium": (101, 51, 21, (12, 6, 3)), "small": (61, 31, 13, (8, 4, 2))}


def prolongation(X: np.ndarray, eq: np.ndarray, cells, n: int) -> sp.csr_matrix:
    """Trilinear interpolation from the nodes of a regular grid of `cells`
    over the bounding box, per DOF (the construction of the learned solver's
    coarse space)."""
    D = 3
    lo, hi = X.min(axis=0), X.max(axis=0)
    u = (X - lo) / np.where(hi > lo, hi - lo, 1.0) * np.asarray(cells, float)
    ci = np.clip(np.floor(u).astype(np.int64), 0, np.asarray(cells) - 1)
    t = np.clip(u - ci, 0.0, 1.0)
    nxn, nyn = cells[0] + 1, cells[1] + 1
    nc = (cells[0] + 1) * (cells[1] + 1) * (cells[2] + 1) * D
    rows, cols, vals = [], [], []
    eqn = eq.reshape(-1, D)
    for corner in range(8):
        dx, dy, dz = corner & 1, (corner >> 1) & 1, (corner >> 2) & 1
        w = np.where(dx, t[:, 0], 1 - t[:, 0]) * np.where(dy, t[:, 1], 1 - t[:, 1]) * np.where(dz, t[:, 2], 1 - t[:, 2])
        node = (ci[:, 0] + dx) + nxn * ((ci[:, 1] + dy) + nyn * (ci[:, 2] + dz))
        for i in range(D):
            e = eqn[:, i]
            ok = (e >= 0) & (w != 0)
            rows.append(e[ok]); cols.append(node[ok] * D + i); vals.append(w[ok])
    return sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))), shape=(n, nc))


def block_jacobi(A: sp.csr_matrix, bd: int = 3):
    """Inverses of the bd x bd diagonal blocks of consecutive rows (a last,
    shorter group takes the inverse of its own diagonal block)."""
    n = A.shape[0]
    nb = n // bd
    blocks = np.zeros((nb, bd, bd))
    idx = np.arange(nb) * bd
    for r in range(bd):
        for c in range(bd):
            blocks[:, r, c] = np.asarray(A[idx + r, idx + c]).ravel()
    inv = np.linalg.inv(blocks)
    tail = np.arange(nb * bd, n)
    tinv = np.linalg.inv(A[tail][:, tail].toarray()) if len(tail) else None

    def apply(r):
        z = np.empty_like(r)
        z[: nb * bd] = np.einsum("bij,bj->bi", inv, r[: nb * bd].reshape(nb, bd)).reshape(-1)
        if tinv is not None:
            z[nb * bd:] = tinv @ r[nb * bd:]
        return z
    return apply


def fcg(A, b, precond, rtol=1e-8, max_iter=2000):
    """Flexible CG keeping one direction (the plain method of the Newmark solves)."""
    x = np.zeros_like(b)
    r = b.copy()
    bn = np.linalg.norm(b)
    z = precond(r)
    p = z.copy()
    q = A @ p
    for it in range(1, max_iter + 1):
        pq = p @ q
        alpha = (r @ p) / pq
        x += alpha * p
        r -= alpha * q
        if np.linalg.norm(r) <= rtol * bn:
            return it, float(np.linalg.norm(b - A @ x) / bn)
        z = precond(r)
        beta = (z @ q) / pq
        p = z - beta * p
        q = A @ p
    return max_iter, float(np.linalg.norm(b - A @ x) / bn)


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--size", default="full", choices=list(SIZES))
    ap.add_argument("--random", type=int, default=2)
    args = ap.parse_args()
    nx, ny, nz, cells = SIZES[args.size]
    t0 = time.time()
    d = tempfile.mkdtemp(prefix="pdx_galerkin_")
    mesh, kw = meshgen.config_c5(nx=nx, ny=ny, nz=nz, nsteps=2)
    cmd = meshgen.write_case(mesh, d, "c5", **kw)
    host = pdx.Model(cmd, device=-1)
    o = orc.Oracle(host)
    info = host.info
    up = host.array("u0").reshape(-1).copy()
    up += host.array("dtv").reshape(-1) * (host.array("eq").reshape(-1) < 0)   # first step: prescribed advanced
    ia, ja, K, f = o.assemble(up)
    M = o.consistent_mass()
    beta = 0.25
    A = sp.csr_matrix((K * (beta * info.dt * info.dt) + M, ja, ia), shape=(info.n_eq, info.n_eq))
    del K, M
    t_asm = time.time() - t0
    X = host.array("X").reshape(-1, 3)
    P = prolongation(X, host.array("eq").reshape(-1), cells, info.n_eq)
    Ac = (P.T @ (A @ P)).toarray()
    lu = sla.lu_factor(Ac)
    bj = block_jacobi(A)

    def two_level(r):
        return bj(r) + P @ sla.lu_solve(lu, P.T @ r)

    rng = np.random.default_rng(0)
    rhs = [("newmark step 1", f)] + [(f"random {i}", rng.uniform(-1, 1, info.n_eq)) for i in range(args.random)]
    out = []
    for name, b in rhs:
        t = time.time()
        it_bj, res_bj = fcg(A, b, bj)
        t_bj = time.time() - t
        t = time.time()
        it_gk, res_gk = fcg(A, b, two_level)
        t_gk = time.time() - t
        out.append(dict(rhs=name, block_jacobi=it_bj, block_jacobi_galerkin=it_gk, ratio=it_bj / max(it_gk, 1),
                        residuals=[res_bj, res_gk], cpu_s=[round(t_bj, 1), round(t_gk, 1)]))
        print(json.dumps(out[-1]), flush=True)
    print(json.dumps({"study": "exact Galerkin coarse correction vs block-Jacobi flexible CG, C5 Newmark K_N",
                      "size": args.size, "n_eq": info.n_eq, "nnz": int(A.nnz), "coarse_cells": cells,
                      "coarse_dofs": int(P.shape[1]), "assembly_s": round(t_asm, 1), "solves": out}))


if __name__ == "__main__":
    main()
