"""Direct sparse solve used by the PARDISO stand-in of the reference build.

Reads (n, nnz, ia, ja, a, b) written by shim_impl.cpp (zero-based CSR, int64
indices, float64 values), solves with SciPy's SuperLU and writes x.
Test infrastructure only.
"""
import sys

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla


def main(inp: str, out: str) -> None:
    raw = open(inp, "rb").read()
    n, nnz = np.frombuffer(raw[:16], dtype=np.int64)
    off = 16
    ia = np.frombuffer(raw, dtype=np.int64, count=n + 1, offset=off); off += 8 * (n + 1)
    ja = np.frombuffer(raw, dtype=np.int64, count=nnz, offset=off); off += 8 * nnz
    a = np.frombuffer(raw, dtype=np.float64, count=nnz, offset=off); off += 8 * nnz
    b = np.frombuffer(raw, dtype=np.float64, count=n, offset=off)
    A = sp.csr_matrix((a, ja, ia), shape=(n, n))
    # PARDISO in the reference perturbs zero pivots (iparm[9] = 13,
    # calMatrixOperations.cpp:292): an empty row (a node whose bonds are all
    # broken) with a zero right-hand side then solves to 0.  SuperLU stops on
    # an exactly singular factor instead, so such rows get a unit diagonal,
    # which gives the same 0.
    empty = np.diff(A.indptr) == 0
    rowsum = np.asarray(abs(A).sum(axis=1)).ravel()
    empty |= rowsum == 0
    if empty.any():
        if np.any(b[empty] != 0):
            raise SystemExit("empty stiffness row with a nonzero load")
        A = A + sp.diags(empty.astype(np.float64))
    x = spla.splu(A.tocsc(), permc_spec="COLAMD").solve(b.copy())
    np.asarray(x, dtype=np.float64).tofile(out)


if __name__ == "__main__":
    main(sys.argv[1], sys.argv[2])
