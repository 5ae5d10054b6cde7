"""Learned two-level preconditioner: the network's gradients against the CPU
oracle (oracle/mlp_oracle.py, itself checked against finite differences), and
what the trained preconditioner gains over plain block-Jacobi flexible CG on
an implicit Newmark problem at the same true FP64 residual (1e-8)."""
import tempfile

import numpy as np
import pytest

import meshgen
import mlp_oracle
import pdx
from conftest import rel


def test_oracle_backward_matches_finite_differences():
    rng = np.random.default_rng(0)
    n, H, B = 7, 5, 3
    npar = H * n + H + H * H + H + n * H + n
    p = rng.standard_normal(npar) * 0.5
    X = rng.standard_normal((B, n))
    T = rng.standard_normal((B, n))
    w = rng.uniform(0.5, 1.5, B)
    _, g = mlp_oracle.loss_grad(p, n, H, X, T, w, bf16=False)
    eps = 1e-6
    fd = np.zeros(npar)
    for i in range(npar):
        dp = np.zeros(npar)
        dp[i] = eps
        fd[i] = (mlp_oracle.loss_grad(p + dp, n, H, X, T, w, bf16=False)[0] -
                 mlp_oracle.loss_grad(p - dp, n, H, X, T, w, bf16=False)[0]) / (2 * eps)
    assert rel(g, fd) < 1e-7


def test_bf16_rounding_is_nearest_even():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, -2.5, 3.0e-3], dtype=np.float32)
    r = mlp_oracle.to_bf16(x)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0 + 2 ** -6 and r[3] == -2.5
    assert abs(r[4] - 3.0e-3) <= 3.0e-3 * 2 ** -8


def small_newmark_case(dt_factor=20.0):
    d = tempfile.mkdtemp()
    mesh, kw = meshgen.config_c5(nx=41, ny=21, nz=11, nsteps=40, radius_h=3, dt_factor=dt_factor)
    return meshgen.write_case(mesh, d, "c5s", **kw)


@pytest.mark.gpu
def test_network_gradient_matches_oracle(built):
    H = 32
    n = (4 * 3 * 3) * 3
    with pdx.Model(small_newmark_case(), device=0) as m:
        m.learned_setup((3, 2, 2), hidden=H, seed=5, max_samples=8)
        p = m.mlp_params()
        assert p.size == H * n + H + H * H + H + n * H + n
        rng = np.random.default_rng(1)
        p = (rng.standard_normal(p.size) * 0.2).astype(np.float32)
        m.mlp_params(set_to=p)
        B = 16
        X = rng.standard_normal((B, n)).astype(np.float32)
        T = rng.standard_normal((B, n)).astype(np.float32)
        w = rng.uniform(0.5, 1.5, B).astype(np.float32)
        loss, g = m.mlp_loss_grad(X, T, w)
    lo, go = mlp_oracle.loss_grad(p.astype(np.float64), n, H, X, T, w.astype(np.float64), bf16=True)
    assert abs(loss - lo) <= 1e-3 * abs(lo)
    # BF16 operands, FP32 accumulation on the GPU; FP64 accumulation in the oracle
    assert rel(g, go) < 1e-2


@pytest.mark.gpu
def test_learned_preconditioner_gains_over_plain_fcg(built):
    cmd = small_newmark_case()
    its_plain, its_learned = [], []
    with pdx.Model(cmd, device=0) as a:
        a.newmark_init()
        for _ in range(15):
            a.newmark_step(4)
        for _ in range(5):
            i = a.newmark_step(4)
            assert i.converged and i.rel_residual <= 1e-8
            its_plain.append(i.iterations)
        ua = a.state()[0]
    with pdx.Model(cmd, device=0) as b:
        b.learned_setup((8, 4, 2), hidden=128, seed=0, max_samples=8192)
        b.newmark_init()
        for _ in range(15):
            b.newmark_step(4, collect=True)
        n_steps = b.learned_samples()
        b.learned_probe(20, seed=1)
        n_pairs = b.learned_samples()
        # tails near the tolerance are dropped: about half of each solve is kept
        assert n_steps > 200 and n_pairs > n_steps + 20 * 30
        loss = b.learned_train(epochs=100, lr=1e-3, seed=0)
        for _ in range(5):
            i = b.newmark_step(5)
            assert i.converged and i.rel_residual <= 1e-8
            its_learned.append(i.iterations)
        ub = b.state()[0]
    print(f"\ntrained on {n_pairs} pairs, final loss {loss:.3e}; iterations to 1e-8: "
          f"plain block-Jacobi FCG {its_plain}, learned {its_learned}")
    assert rel(ub, ua) < 1e-6
    assert sum(its_learned) < sum(its_plain)


@pytest.mark.gpu
def test_plain_solver_judges_and_replaces_a_bad_network(built):
    """Plain block-Jacobi flexible CG is the arbiter: with a network that only
    adds noise the learned solves are cut at the plain iteration count, and
    after two losses method 5 runs the plain method itself."""
    cmd = small_newmark_case()
    with pdx.Model(cmd, device=0) as b:
        b.learned_setup((8, 4, 2), hidden=32, seed=0, max_samples=4096)
        b.newmark_init()
        plain = [b.newmark_step(4, collect=True).iterations for _ in range(3)]
        b.learned_train(epochs=1, lr=1e-3, seed=0)
        assert b.learned_active()
        p = b.mlp_params()
        rng = np.random.default_rng(5)
        p = (rng.standard_normal(p.size) * 3.0).astype(np.float32)
        b.mlp_params(set_to=p)
        its = []
        for _ in range(4):
            i = b.newmark_step(5)
            assert i.converged and i.rel_residual <= 1e-8
            its.append(i.iterations)
        assert not b.learned_active()
        # once switched off, a method-5 step is a plain solve
        assert abs(its[-1] - np.mean(plain)) <= 20


def test_exact_galerkin_correction_bounds_the_learned_gain(built):
    """The learned network imitates a coarse solve on its grid; the exact
    Galerkin correction P (P^T A P)^-1 P^T on that grid is the best any such
    correction can do.  On the small C5 Newmark system (72,943 equations,
    8 x 4 x 2 coarse cells) it cuts block-Jacobi flexible-CG iterations to a
    1e-8 residual by less than 3x, so a learned coarse correction on this grid
    cannot reach a 3x faster solve (oracle/galerkin_study.py, CPU, FP64)."""
    import subprocess
    import sys
    import json
    from conftest import REPO
    r = subprocess.run([sys.executable, f"{REPO}/oracle/galerkin_study.py", "--size", "small", "--random", "0"],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    res = json.loads(r.stdout.strip().splitlines()[-1])
    s = res["solves"][0]
    print(f"\nsmall C5: block-Jacobi {s['block_jacobi']} its, with the exact Galerkin correction "
          f"{s['block_jacobi_galerkin']} its ({s['ratio']:.2f}x)")
    assert max(s["residuals"]) <= 1.01e-8
    assert 1.0 < s["ratio"] < 3.0


def test_exact_galerkin_correction_cuts_the_c3_bicgstab_iterations(built):
    """Pdx method 8 rests on this: C3's quasi-static stiffness has no mass
    term, so Jacobi BiCGStab's iterations are dominated by smooth error modes
    that a bilinear coarse grid captures.  On a 161 x 161-node strip plate
    (C3's geometry at 0.4 of its span) the exact Galerkin correction on a
    10 x 10-cell lattice cuts Jacobi BiCGStab's iterations to a 1e-8
    residual several-fold (oracle/twolevel_study.py, CPU, FP64)."""
    import subprocess
    import sys
    import json
    from conftest import REPO
    r = subprocess.run([sys.executable, f"{REPO}/oracle/twolevel_study.py", "10x10", "--n", "161"],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    rows = [json.loads(l) for l in r.stdout.strip().splitlines() if l.startswith("{")]
    jac = next(x for x in rows if x["preconditioner"] == "jacobi")
    gal = next(x for x in rows if x["preconditioner"].startswith("jacobi + galerkin"))
    print(f"\n161x161 C3 plate: Jacobi {jac['iterations']} its, with the Galerkin correction "
          f"{gal['iterations']} its")
    assert jac["info"] == 0 and gal["info"] == 0
    assert jac["residual"] <= 1.01e-8 and gal["residual"] <= 1.01e-8
    assert gal["iterations"] * 4 < jac["iterations"]
