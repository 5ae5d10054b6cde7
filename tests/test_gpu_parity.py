"""CUDA path against the oracle and the reference's FP64 goldens, through the
C ABI.  Tolerances: FP64 path 1e-10 relative L2 for displacement and stress
(the bar for the plain FP64 path), 1e-12 for single force/assembly
evaluations; broken-bond sets identical.  Mixed precision states its error."""
import os
import shutil
import tempfile

import numpy as np
import pytest

from conftest import case_cmd, golden, rel

import meshgen
import orc
import pdx

pytestmark = pytest.mark.gpu

CASES = [("p21", "p21_explicit"), ("b13", "b13_explicit")]
FP64_TOL = 1e-10


def bonds_only(m, arr):
    off = m.array("fam_off")
    keep = np.ones(len(m.array("bond_state0")), bool)
    keep[off[:-1]] = False
    return arr[keep]


@pytest.mark.parametrize("case,cmd", CASES)
def test_coefficients_match_oracle_and_reference(built, case, cmd):
    with pdx.Model(case_cmd(case, cmd), device=0, precision=0) as m:
        A, g, d, G = m.bond_coefficients()
        o = orc.Oracle(pdx.Model(case_cmd(case, cmd), device=-1))
        oA, og, od, oG = o.coeffs()
        gc = golden(case + "_coeffs")
        assert rel(A, gc["A"]) < 1e-13
        assert rel(g, og) < 1e-12 and rel(d, od) < 1e-12 and rel(G, oG) < 1e-12
        assert rel(g, gc["g"]) < 1e-12 and rel(d, gc["d"]) < 1e-12


@pytest.mark.parametrize("case,cmd", CASES)
def test_internal_force_fp64(built, case, cmd):
    gf = golden(case + "_force")
    with pdx.Model(case_cmd(case, cmd), device=0, precision=0) as m:
        f = m.internal_force(gf["u_all"])
    assert rel(f, gf["F"]) < 1e-12


@pytest.mark.parametrize("case,cmd", CASES)
def test_explicit_fp64_matches_reference(built, case, cmd):
    ge = golden(case + "_explicit")
    steps = list(ge["u_traj_steps"])
    with pdx.Model(case_cmd(case, cmd), device=0, precision=0) as m:
        m.explicit_init()
        done = 0
        worst = 0.0
        for i, s in enumerate(steps):
            m.explicit_advance(s + 1 - done)
            done = s + 1
            u, sig, phi, bs = m.state()
            worst = max(worst, rel(u, ge["u_traj"][i]))
        assert worst < FP64_TOL
        np.testing.assert_array_equal(bs, ge["bond_state_final"])
        np.testing.assert_allclose(phi, ge["phi_final"], rtol=0, atol=1e-15)
        assert rel(sig, ge["sigma_final"]) < FP64_TOL


@pytest.mark.parametrize("case,cmd", CASES)
def test_explicit_graph_path_equals_single_launches(built, case, cmd):
    """130 steps: the captured-graph path (64-step chunks) gives the same state as single launches."""
    with pdx.Model(case_cmd(case, cmd), device=0, precision=0) as a, \
            pdx.Model(case_cmd(case, cmd), device=0, precision=0) as b:
        a.explicit_init(); b.explicit_init()
        a.explicit_advance(130)
        for _ in range(130):
            b.explicit_advance(1)
        ua, _, _, sa = a.state()
        ub, _, _, sb = b.state()
    np.testing.assert_array_equal(ua, ub)
    np.testing.assert_array_equal(sa, sb)


@pytest.mark.parametrize("case,cmd", CASES)
def test_mixed_precision_error_is_stated(built, case, cmd):
    ge = golden(case + "_explicit")
    with pdx.Model(case_cmd(case, cmd), device=0, precision=1) as m:
        m.explicit_init()
        n = int(ge["u_traj_steps"][-1]) + 1
        m.explicit_advance(n)
        u, sig, phi, bs = m.state()
    err = rel(u, ge["u_traj"][-1])
    nb_diff = int((bs != ge["bond_state_final"]).sum())
    print(f"\n[{case}] mixed precision: displacement rel L2 error {err:.3e} vs FP64 reference, "
          f"{nb_diff} bond-state differences of {int((ge['bond_state_final'] == 0).sum())} broken")
    assert err < 1e-4
    assert nb_diff <= max(2, int(0.01 * (ge["bond_state_final"] == 0).sum()))


@pytest.mark.parametrize("case,cmd", CASES)
def test_stress_and_damage_match_oracle(built, case, cmd):
    """Nodal stress after step 15: the reference computes it before that
    step's failure pass (pdsolve.cpp:6062 before :6064), i.e. with the bond
    states left by step 14; damage uses the states after the pass."""
    host = pdx.Model(case_cmd(case, cmd), device=-1)
    o = orc.Oracle(host)
    _, bs14, _, _ = o.explicit(nsteps=14)
    u, bs, _, _ = o.explicit(nsteps=15)
    sig_o, _ = o.stress(u, bs14)
    _, phi_o = o.stress(u, bs)
    with pdx.Model(case_cmd(case, cmd), device=0, precision=0) as m:
        m.explicit_init()
        m.explicit_advance(16)
        ug, sg, phg, bsg = m.state()
    np.testing.assert_array_equal(bsg, bs)
    assert rel(ug, u) < FP64_TOL
    assert rel(phg, phi_o) < 1e-14
    assert rel(sg, sig_o) < FP64_TOL


@pytest.mark.parametrize("case,cmd,mode", [("p21", "p21s", 1), ("b13", "b13s", 1), ("p21", "p21_quasi", 2)])
def test_assembly_matches_reference(built, case, cmd, mode):
    host = pdx.Model(case_cmd(case, cmd), device=-1)
    o = orc.Oracle(host)
    v = host.array("u0").copy()
    with pdx.Model(case_cmd(case, cmd), device=0, precision=0) as m:
        ia, ja, a, f = m.assemble(mode, v)
    if mode == 1:
        vm = v.copy()
        vm[host.array("eq") >= 0] = 0.0
        oia, oja, oa, of = o.assemble(vm)
        gs = golden(case + "_static")
        np.testing.assert_array_equal(ia, gs["K_ia"])
        np.testing.assert_array_equal(ja, gs["K_ja"])
        assert rel(a, gs["K_a"]) < 1e-12
        assert rel(f, gs["F"]) < 1e-12
    else:
        oia, oja, oa, of = o.assemble(v)
        gq = golden(case + "_quasi")
        assert rel(a, gq["K_a_1"]) < 1e-12
        assert rel(f, gq["F_1"]) < 1e-12
    assert rel(a, oa) < 1e-12


@pytest.mark.parametrize("case", ["p21", "t21"])
def test_newmark_matrix_matches_reference(built, case):
    """K_N = beta dt^2 K + M and its load; t21 has triangles (consistent mass rho V / 12)."""
    gn = golden(case + "_newmark")
    host = pdx.Model(case_cmd(case, case + "_newmark"), device=-1)
    up = host.array("u0").reshape(-1).copy()
    up += host.array("dtv").reshape(-1, 3)[:, :2].reshape(-1) * (host.array("eq") < 0)
    with pdx.Model(case_cmd(case, case + "_newmark"), device=0, precision=0) as m:
        ia, ja, a, f = m.assemble(3, up)
    assert rel(a, gn["KN_a"]) < 1e-12
    assert rel(f, gn["FN"]) < 1e-12


@pytest.mark.parametrize("method", [0, 1, 2, 3, 6, 7])
def test_krylov_solves_reference_system(built, method):
    gs = golden("b13_static")
    x, info = pdx.solve_csr(gs["K_ia"], gs["K_ja"], gs["K_a"], gs["F"], method=method, rtol=1e-12,
                            max_iter=20000)
    ia, ja, a = gs["K_ia"], gs["K_ja"], gs["K_a"]
    r = gs["F"].copy()
    for i in range(len(ia) - 1):
        r[i] -= np.dot(a[ia[i]:ia[i + 1]], x[ja[ia[i]:ia[i + 1]]])
    true_res = np.linalg.norm(r) / np.linalg.norm(gs["F"])
    print(f"\nmethod {method}: {info.iterations} iterations, reported {info.rel_residual:.2e}, true {true_res:.2e}")
    if info.converged:
        assert true_res <= 1.01e-12
        assert info.method_used == method
        if method in (3, 7):
            # FP32 inner solves to 1e-4: a 1e-12 FP64 residual takes several refinement steps
            assert info.refinements >= 2
        # the reference's direct solve, in equation order; the system's 2-norm
        # condition number is 6.4e3, so a 1e-12 residual bounds the relative
        # error by 6.4e-9
        eq = pdx.Model(case_cmd("b13", "b13s"), device=-1).array("eq").reshape(-1)
        u_ref = np.zeros_like(x)
        u_ref[eq[eq >= 0]] = gs["u"].reshape(-1)[eq >= 0]
        assert rel(x, u_ref) < 1e-8
    else:
        # plain CG on the unsymmetric stiffness may stall; the drivers fall back to BiCGStab
        assert method in (0, 1, 3)


def _indefinite_convection_system(nx=40, seed=0):
    """A shifted, row-scaled 2D convection-diffusion matrix (unsymmetric and
    indefinite, as the stiffness of a cracked plate can be) with two empty
    rows and zero right-hand sides there (nodes with every bond broken)."""
    import scipy.sparse as sp
    rng = np.random.default_rng(seed)
    eye = sp.identity(nx)
    t = sp.diags([-1.0, 2.0, -1.0], [-1, 0, 1], (nx, nx))
    c = sp.diags([-1.0, 0.0, 1.0], [-1, 0, 1], (nx, nx))
    n = nx * nx
    a = sp.kron(eye, t) + sp.kron(t, eye) + 4.0 * (sp.kron(eye, c) + sp.kron(c, eye)) - 0.3 * sp.identity(n)
    a = (sp.diags(np.exp(rng.uniform(-2, 2, n))) @ a).tolil()
    empty = [5, 777]
    for i in empty:
        a[i, :] = 0.0
        a[:, i] = 0.0
    a = a.tocsr()
    a.sort_indices()
    b = rng.standard_normal(n)
    b[empty] = 0.0
    return a, b, empty


def test_gmres_solves_where_bicgstab_breaks_down(built):
    """GMRES(30) (method 6, the drivers' last fallback) solves the indefinite
    unsymmetric system on which Jacobi BiCGStab breaks down, and leaves the
    empty rows at zero; checked against a direct solve."""
    sps = pytest.importorskip("scipy.sparse")
    spla = pytest.importorskip("scipy.sparse.linalg")
    a, b, empty = _indefinite_convection_system()
    ia, ja = a.indptr.astype(np.int64), a.indices.astype(np.int64)
    _, info2 = pdx.solve_csr(ia, ja, a.data, b, method=2, rtol=1e-10, max_iter=3000)
    x, info6 = pdx.solve_csr(ia, ja, a.data, b, method=6, rtol=1e-10, max_iter=3000)
    d = a.diagonal()
    xd = spla.spsolve((a + sps.diags((d == 0).astype(float))).tocsc(), b)
    print(f"\nBiCGStab: converged {info2.converged}, residual {info2.rel_residual:.2e}; "
          f"GMRES: {info6.iterations} iterations, residual {info6.rel_residual:.2e}")
    assert not info2.converged
    assert info6.converged and info6.rel_residual <= 1e-10
    assert np.all(x[empty] == 0.0)
    assert np.linalg.norm(x - xd) / np.linalg.norm(xd) < 1e-8


def test_static_run_matches_reference_solution(built, tmp_path):
    gs = golden("b13_static")
    with pdx.Model(case_cmd("b13", "b13s"), device=0, precision=0) as m:
        m.run(str(tmp_path))
    path = os.path.join(tmp_path, "b13_static.vtk")
    assert os.path.exists(path)
    raw = open(path, "rb").read()
    i = raw.index(b"VECTORS U")
    j = raw.index(b"\n", i)
    n = len(gs["u"])
    U = np.frombuffer(raw, ">f4", 3 * n, j + 1).reshape(n, 3).astype(np.float64)
    assert rel(U, gs["u"]) < 1e-6   # float32 file, Krylov solve to 1e-8


def _text_lines_agree(mine: str, ref: str, rtol: float):
    """Same lines and tokens; numbers equal up to the printed precision (a
    last-digit difference where the FP64 states differ by ~1e-15 and the
    rounding boundary falls between them), or within 1e-9 of the largest
    number on the line (round-off noise such as 1e-23 beside 6e-6).
    Returns the number of differing lines."""
    a, b = mine.splitlines(), ref.splitlines()
    assert len(a) == len(b)
    differ = 0
    for la, lb in zip(a, b):
        if la == lb:
            continue
        differ += 1
        ta, tb = la.split(), lb.split()
        assert len(ta) == len(tb), (la, lb)
        scale = max(abs(float(y)) for y in tb)
        for x, y in zip(ta, tb):
            if x != y:
                fx, fy = float(x), float(y)
                assert abs(fx - fy) <= rtol * max(abs(fx), abs(fy)) + 1e-9 * scale, (la, lb)
    return differ


def test_ascii_results_match_reference_files(built, tmp_path):
    """VTKFORMAT ASCII: pdx_run writes the ASCII VTK file and the .sig and
    .disp text files at each save step, as the reference's own solver does
    (explicit, FC 2 with all candidates, 60 steps; the files of step 60 are
    the reference's, written by its pdfemSolver)."""
    gdir = os.path.join(os.path.dirname(__file__), "golden", "p21_ascii")
    with pdx.Model(case_cmd("p21", "p21_ascii"), device=0, precision=0) as m:
        m.run(str(tmp_path))
    for ext, rtol in (("vtk", 2e-4), ("sig", 2e-5), ("disp", 2e-4)):
        mine = open(os.path.join(tmp_path, f"p21_60.{ext}")).read()
        ref = open(os.path.join(gdir, f"p21_60.{ext}")).read()
        differ = _text_lines_agree(mine, ref, rtol)
        print(f"\n{ext}: {differ} of {len(ref.splitlines())} lines differ in the last digit")
        assert differ <= 0.01 * len(ref.splitlines())
    for n in (20, 40):
        for ext in ("vtk", "sig", "disp"):
            assert os.path.exists(os.path.join(tmp_path, f"p21_{n}.{ext}"))


def test_binary_vtk_matches_reference_file(built, tmp_path):
    """VTKFORMAT BINARY, same run: header, points and cells byte for byte as
    the reference's file; U, sigma and phi (big-endian float32) equal up to
    the float32 rounding of FP64 states that agree to ~1e-15."""
    src = os.path.join(os.path.dirname(__file__), "golden", "cases", "p21")
    text = open(os.path.join(src, "p21_ascii.in")).read().replace("VTKFORMAT ASCII", "VTKFORMAT BINARY")
    with open(os.path.join(tmp_path, "p21_bin.in"), "w") as f:
        f.write(text)
    shutil.copy(os.path.join(src, "p21_ascii.lis"), tmp_path)
    out = tmp_path / "out"
    out.mkdir()
    with pdx.Model(str(tmp_path / "p21_bin.in"), device=0, precision=0) as m:
        n = m.info.n_node
        m.run(str(out))
    mine = open(out / "p21_60.vtk", "rb").read()
    ref = open(os.path.join(os.path.dirname(__file__), "golden", "p21_ascii", "p21_60_binary.vtk"), "rb").read()
    assert len(mine) == len(ref)
    cut = ref.index(b"VECTORS U")
    assert mine[:cut] == ref[:cut]
    for key, count in ((b"VECTORS U", 3 * n), (b"TENSORS sigma", 9 * n), (b"LOOKUP_TABLE", n)):
        i, j = ref.index(key), mine.index(key)
        a = np.frombuffer(mine, ">f4", count, mine.index(b"\n", j) + 1).astype(np.float64)
        b = np.frombuffer(ref, ">f4", count, ref.index(b"\n", i) + 1).astype(np.float64)
        assert np.all(np.abs(a - b) <= 2.4e-7 * np.abs(b) + 1e-9 * np.abs(b).max()), key


@pytest.mark.parametrize("case,cmd", [("p21", "p21_explicit"), ("b13", "b13_explicit")])
def test_gpu_family_search_equals_host_and_reference(built, case, cmd):
    """A model with a device builds its families and CSR pattern on the GPU: the member lists
    (order included), offsets, pre-crack bond states and CSR pattern equal the
    host search's and the reference's set-up dump."""
    g = golden(case + "_setup")
    host = pdx.Model(case_cmd(case, cmd), device=-1)
    with pdx.Model(case_cmd(case, cmd), device=0) as dev:
        for name in ("fam_off", "fam_members", "bond_state0", "csr_ia", "csr_ja"):
            np.testing.assert_array_equal(dev.array(name), host.array(name))
        np.testing.assert_array_equal(dev.array("fam_members") + 1, g["fam_members"])
        np.testing.assert_array_equal(dev.array("fam_off"), g["fam_off"])


def test_gpu_family_search_full_size(built):
    """C2 (151,284 nodes, 31,584 families, 3.53M bonds, 59.4M nonzeros): GPU
    and host family lists and CSR pattern are identical; the set-up times are
    printed."""
    import time
    d = tempfile.mkdtemp()
    mesh, kw = meshgen.config_c2(nsteps=2)
    cmd = meshgen.write_case(mesh, d, "c2", **kw)
    t0 = time.perf_counter()
    host = pdx.Model(cmd, device=-1)
    t1 = time.perf_counter()
    with pdx.Model(cmd, device=0, verbose=2) as dev:
        t2 = time.perf_counter()
        for name in ("fam_off", "fam_members", "bond_state0", "csr_ia", "csr_ja"):
            np.testing.assert_array_equal(dev.array(name), host.array(name))
    print(f"\nC2 set-up: host-only model {t1 - t0:.2f} s, model with device {t2 - t1:.2f} s")


def test_step_host_equals_device_resident(built):
    cmd = case_cmd("b13", "b13_explicit")
    with pdx.Model(cmd, device=0, precision=0) as a, pdx.Model(cmd, device=0, precision=0) as b:
        a.explicit_init(); b.explicit_init()
        eq = a.array("eq")
        act = eq >= 0
        u0 = a.array("u0")
        un = np.zeros(a.info.n_eq); un[eq[act]] = u0[act]
        unm1 = un.copy()
        out = np.zeros_like(un)
        for _ in range(12):
            b.explicit_step_host(un, unm1, out)
            unm1, un = un, out.copy()
        a.explicit_advance(12)
        ua, _, _, sa = a.state()
        ub, _, _, sb = b.state()
    np.testing.assert_array_equal(ua.reshape(-1)[act], un[eq[act]])
    np.testing.assert_array_equal(sa, sb)


@pytest.mark.parametrize("precision", [0, 1])
def test_step_host_pinned_buffers_equal_device_resident(built, precision):
    """Page-locked host buffers take the in-place path (the load kernel reads
    them over the host link, the gather writes the result back); the states
    equal the device-resident run bit for bit, FP64 and mixed."""
    torch = pytest.importorskip("torch")
    cmd = case_cmd("b13", "b13_explicit")
    with pdx.Model(cmd, device=0, precision=precision) as a, pdx.Model(cmd, device=0, precision=precision) as b:
        a.explicit_init(); b.explicit_init()
        eq = a.array("eq")
        act = eq >= 0
        u0 = a.array("u0")
        bufs = [torch.zeros(a.info.n_eq, dtype=torch.float64, pin_memory=True).numpy() for _ in range(3)]
        un, unm1, out = bufs
        un[eq[act]] = u0[act]
        unm1[:] = un
        for _ in range(12):
            b.explicit_step_host(un, unm1, out)
            un, unm1, out = out, un, unm1
        a.explicit_advance(12)
        ua, _, _, sa = a.state()
        ub, _, _, sb = b.state()
    np.testing.assert_array_equal(ua.reshape(-1)[act], un[eq[act]])
    np.testing.assert_array_equal(ua, ub)
    np.testing.assert_array_equal(sa, sb)


def test_c1_full_size_fp64_parity(built):
    """Full 101x101 C1 plate, 200 explicit steps of the FP64 GPU path against the oracle."""
    d = tempfile.mkdtemp()
    mesh, kw = meshgen.config_c1(nsteps=200)
    cmd = meshgen.write_case(mesh, d, "c1", **kw)
    host = pdx.Model(cmd, device=-1)
    o = orc.Oracle(host)
    u_o, bs_o, _, nb = o.explicit(nsteps=199)
    with pdx.Model(cmd, device=0, precision=0) as m:
        m.explicit_init()
        m.explicit_advance(200)
        u, sig, phi, bs = m.state()
    assert rel(u, u_o) < FP64_TOL
    assert np.array_equal(bs, bs_o)


@pytest.mark.parametrize("lanes,fe_lanes", [(4, 1), (4, 2), (8, 4), (16, 8)])
def test_element_path_and_lane_counts_match_oracle(built, lanes, fe_lanes):
    """A jittered Hex8 box (no shared node stencils: FE-only nodes take the
    element path) against the oracle, FP64 and mixed, at several lane counts."""
    d = tempfile.mkdtemp()
    mesh = meshgen.box_hole(nx=13, ny=9, nz=5, h=1e-3, radius=2e-3, pd_x=8, pd_y=6)
    rng = np.random.default_rng(5)
    mesh.X[:, :3] += rng.uniform(-1e-4, 1e-4, mesh.X[:, :3].shape)
    cmd = meshgen.write_case(mesh, d, "jit", solver="DYNAMIC", dt=2e-8, nsteps=60, save=60, factor=3.015,
                             nlf=1.0, fc="3 2e-5 3 0.05")
    host = pdx.Model(cmd, device=-1)
    assert np.all(host.array("st_cls") == -1)
    o = orc.Oracle(host)
    u_o, bs_o, _, nb = o.explicit(nsteps=59)
    with pdx.Model(cmd, device=0, precision=0, lanes=lanes, fe_lanes=fe_lanes) as m:
        m.explicit_init()
        m.explicit_advance(60)
        u, _, _, bs = m.state()
    assert rel(u, u_o) < FP64_TOL
    assert np.array_equal(bs, bs_o)
    with pdx.Model(cmd, device=0, precision=1, lanes=lanes, fe_lanes=fe_lanes) as m:
        m.explicit_init()
        m.explicit_advance(60)
        u32, _, _, bs32 = m.state()
    assert rel(u32, u_o) < 1e-4
    assert int((bs32 != bs_o).sum()) <= max(2, int(0.01 * (bs_o == 0).sum()))


@pytest.mark.parametrize("method", [1, 2, 3, 6, 7, 8])
def test_quasi_static_increments_match_reference(built, method):
    """Three quasi-static increments, one pdx_quasi_step each, against the
    reference's direct-solve trajectory: the Krylov solves stop at a 1e-8 true
    residual, so the free displacements agree to the conditioning times that
    (errors relative to the last increment's free displacements)."""
    gq = golden("p21_quasi")
    with pdx.Model(case_cmd("p21", "p21_quasi"), device=0, precision=0) as m:
        # the reference records an increment before advancing the prescribed
        # DOFs and pdx_quasi_step returns after it: compare the free DOFs
        free = m.array("eq").reshape(-1) >= 0
        scale = np.linalg.norm(gq["u_traj"][-1].reshape(-1)[free])
        m.quasi_init()
        errs = []
        for i in range(3):
            info = m.quasi_step(method)
            assert info.converged and info.rel_residual <= 1e-8
            d = m.state()[0].reshape(-1)[free] - gq["u_traj"][i].reshape(-1)[free]
            errs.append(np.linalg.norm(d) / scale)
    print(f"\nmethod {method}: relative L2 error per increment {['%.1e' % e for e in errs]}")
    # GMRES stops at the first iteration whose residual is below 1e-8; the
    # other methods check every 10 iterations and end further below it
    assert max(errs) < (5e-6 if method == 6 else 1e-6)


@pytest.mark.parametrize("cmd", ["p21_fc2", "p21_fc2k"])
def test_fc2_principal_stress_breaking_matches_reference(built, cmd):
    """FC 2 after every explicit step (sigma_ult 3e7, Top-K 0 and 2) against the
    reference's own run: trajectory, broken-bond set, damage and stresses."""
    g = golden(cmd)
    steps = list(g["u_traj_steps"])
    with pdx.Model(case_cmd("p21", cmd), device=0, precision=0) as m:
        m.explicit_init()
        done, worst = 0, 0.0
        for i, s in enumerate(steps):
            m.explicit_advance(s + 1 - done)
            done = s + 1
            u, sig, phi, bs = m.state()
            worst = max(worst, rel(u, g["u_traj"][i]))
    broken = int((g["bond_state_final"] == 0).sum())
    print(f"\n[{cmd}] FP64: worst displacement error {worst:.2e}, {broken} broken bonds in the reference, "
          f"{int((bs != g['bond_state_final']).sum())} differences")
    np.testing.assert_array_equal(bs, g["bond_state_final"])
    assert worst < FP64_TOL
    np.testing.assert_allclose(phi, g["phi_final"], rtol=0, atol=1e-15)
    assert rel(sig, g["sigma_final"]) < FP64_TOL


def test_fc2_mixed_precision_error_is_stated(built):
    g = golden("p21_fc2")
    with pdx.Model(case_cmd("p21", "p21_fc2"), device=0, precision=1) as m:
        m.explicit_init()
        m.explicit_advance(int(g["u_traj_steps"][-1]) + 1)
        u, sig, phi, bs = m.state()
    err = rel(u, g["u_traj"][-1])
    nb_diff = int((bs != g["bond_state_final"]).sum())
    print(f"\n[p21_fc2] mixed precision: displacement rel L2 error {err:.3e}, {nb_diff} bond-state differences "
          f"of {int((g['bond_state_final'] == 0).sum())} broken")
    assert err < 1e-3
    assert nb_diff <= max(4, int(0.02 * (g["bond_state_final"] == 0).sum()))


def test_reaction_forces_match_reference(built, tmp_path):
    """RF 2 (the top edge): the per-step rows (U, RFx, RFy, RFz) of 61 explicit
    steps against the reference's calReacForc, through the API and in the
    RF.out file pdx_run writes."""
    g = golden("p21_rf")["rf_rows"]
    scale = np.abs(g[:, 2:5]).max()
    with pdx.Model(case_cmd("p21", "p21_rf"), device=0, precision=0) as m:
        m.explicit_init()
        m.explicit_advance(61)
        rows = m.reaction_forces()
        assert rows.shape == (61, 4)
        np.testing.assert_allclose(rows[:, 0], g[:, 1], rtol=1e-14, atol=0)
        assert np.abs(rows[:, 1:4] - g[:, 2:5]).max() <= 1e-10 * scale
        m.run(str(tmp_path))
    lines = open(tmp_path / "p21RF.out").read().splitlines()
    assert lines[0] == "Step\tU\tRFx\tRFy\tRFz" and len(lines) == 62
    last = [float(t) for t in lines[-1].split("\t")]
    assert last[0] == 60 and abs(last[3] - g[-1, 3]) <= 1e-5 * abs(g[-1, 3])


@pytest.mark.parametrize("method", [2, 8])
def test_fc2_in_newmark_steps_matches_reference(built, method):
    """FC 2 after every Newmark step (10 steps, sigma_ult 3e7), the reference
    solving K_N directly and this build with BiCGStab (method 2) or the
    two-level BiCGStab (method 8, its coarse inverse formed again whenever
    FC 2 has changed K) to 1e-13: displacement trajectory and the
    broken-bond set."""
    g = golden("p21_nmfc2")
    with pdx.Model(case_cmd("p21", "p21_nmfc2"), device=0, precision=0) as m:
        m.newmark_init()
        worst = 0.0
        for i in range(10):
            info = m.newmark_step(method)
            assert info.converged and info.method_used == method
            u, _, _, bs = m.state()
            worst = max(worst, rel(u, g["u_traj"][i]))
    print(f"\n[p21_nmfc2] worst displacement error {worst:.2e}, "
          f"{int((bs != g['bond_state_final']).sum())} bond differences of {int((g['bond_state_final'] == 0).sum())} broken")
    np.testing.assert_array_equal(bs, g["bond_state_final"])
    assert worst < 1e-9


def test_fc2_quasi_static_load_control_matches_reference(built):
    """Quasi-static FC 2 with Top-K 4 (20 increments): after an increment that
    cuts bonds the load holds, otherwise it steps by the ratio 1.001 sigma_ult /
    max sigma1 (capped by the BC velocity).  The state after every increment,
    the broken-bond set and the reaction forces against the reference."""
    g = golden("p21_qfc2")
    with pdx.Model(case_cmd("p21", "p21_qfc2"), device=0, precision=0) as m:
        m.quasi_init()
        worst = 0.0
        for i in range(20):
            info = m.quasi_step(2)
            assert info.converged
            u, _, _, bs = m.state()
            worst = max(worst, rel(u, g["u_after"][i]))
        rows = m.reaction_forces()
    rf = g["rf_rows"]
    print(f"\n[p21_qfc2] worst state error {worst:.2e}, {int((bs != g['bond_state_final']).sum())} bond differences "
          f"of {int((g['bond_state_final'] == 0).sum())} broken")
    np.testing.assert_array_equal(bs, g["bond_state_final"])
    assert worst < 1e-9
    assert rows.shape == (21, 4)
    assert np.abs(rows[1:, 1:4] - rf[:, 2:5]).max() <= 1e-8 * np.abs(rf[:, 2:5]).max()


def test_reading_the_state_between_quasi_increments_changes_nothing(built, tmp_path):
    """pdx_get_state applies the pending failure pass of an explicit run only:
    a quasi-static increment finishes its own pass, and its state (with the
    prescribed values already advanced for the next increment) must not be
    tested again.  Plate of 41 x 41 nodes, FC 3, three increments."""
    mesh, kw = meshgen.config_c3(n=41)
    cmd = meshgen.write_case(mesh, str(tmp_path), "q41", **kw)
    out = []
    for read_between in (False, True):
        with pdx.Model(cmd, device=0, precision=0) as m:
            m.quasi_init()
            for _ in range(3):
                m.quasi_step(2)
                if read_between:
                    m.state()
            out.append(m.state())
    np.testing.assert_array_equal(out[0][3], out[1][3])
    np.testing.assert_array_equal(out[0][0], out[1][0])
    assert int((out[1][3] == 0).sum()) == int((pdx.Model(cmd, device=-1).array("bond_state0") == 0).sum())
