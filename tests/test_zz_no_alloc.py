"""pdx_pcg_solve_noalloc: the allocation-free Jacobi PCG against pdx_solve_csr
(method 0) on the same system, twice in a row.  Collected last so that it
also runs after every other test of the session."""
import numpy as np
import pytest

import pdx
from conftest import rel


def spd_system(m: int, seed: int = 7):
    """5-point Laplacian on an m x m grid plus 0.05 I (SPD), CSR with sorted columns."""
    n = m * m
    rows, cols, vals = [], [], []
    for i in range(m):
        for j in range(m):
            r = i * m + j
            for di, dj in ((-1, 0), (0, -1), (0, 0), (0, 1), (1, 0)):
                ii, jj = i + di, j + dj
                if 0 <= ii < m and 0 <= jj < m:
                    rows.append(r)
                    cols.append(ii * m + jj)
                    vals.append(4.05 if (di, dj) == (0, 0) else -1.0)
    rows, cols, vals = np.array(rows), np.array(cols), np.array(vals)
    order = np.lexsort((cols, rows))
    rows, cols, vals = rows[order], cols[order], vals[order]
    ia = np.zeros(n + 1, dtype=np.int64)
    np.add.at(ia, rows + 1, 1)
    ia = np.cumsum(ia)
    b = np.random.default_rng(seed).standard_normal(n)
    return ia, cols.astype(np.int64), vals, b


@pytest.mark.gpu
def test_noalloc_pcg_matches_pcg_twice(built):
    torch = pytest.importorskip("torch")
    ia, ja, a, b = spd_system(64)
    n, nnz = len(b), len(a)
    x_ref, info_ref = pdx.solve_csr(ia, ja, a, b, method=0, rtol=1e-10, max_iter=5000)
    assert info_ref.converged
    dev = torch.device("cuda:0")
    d_ia = torch.from_numpy(ia).to(dev)
    d_ja = torch.from_numpy(ja.astype(np.int32)).to(dev)
    d_a = torch.from_numpy(a).to(dev)
    d_b = torch.from_numpy(b).to(dev)
    d_x = torch.empty(n, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream().cuda_stream
    for call in range(2):
        d_x.fill_(float("nan"))     # use_x0 = False: the solve zeroes x itself
        info, code = pdx.pcg_solve_noalloc(n, nnz, d_ia.data_ptr(), d_ja.data_ptr(), d_a.data_ptr(), d_b.data_ptr(),
                                           d_x.data_ptr(), rtol=1e-10, max_iter=5000, stream=stream)
        torch.cuda.synchronize()
        x = d_x.cpu().numpy()
        assert code == 0, call
        assert info.converged and info.rel_residual <= 1e-10, call
        assert info.iterations == info_ref.iterations, call
        # same kernels in the same order as pdx_solve_csr method 0
        assert rel(x, x_ref) < 1e-12, call
        assert np.linalg.norm(b - (np.add.reduceat(a * x[ja], ia[:-1]))) <= 1e-9 * np.linalg.norm(b)


def test_noalloc_rejects_oversize_before_any_launch(built):
    """The size check returns before any CUDA call, so the dummy device
    pointers are never touched; runs with and without a device."""
    big = 262144 + 1
    with pytest.raises(pdx.PdxError) as e:
        pdx.pcg_solve_noalloc(big, 10, 256, 256, 256, 256, 256)
    assert "exceeds the fixed work space" in str(e.value)
