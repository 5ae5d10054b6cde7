"""Node stencils of FE-only nodes (host set-up, CPU only): the assembled blocks
of a node's stencil class reproduce the element-by-element FE force of the
oracle at that node, and meshes without shared surroundings keep the
element path."""
import numpy as np
import pytest

from conftest import case_cmd, rel

import meshgen
import orc
import pdx


def stencil_force(m, u_all):
    d = m.dim
    S = 9 if d == 2 else 27
    feonly = m.array("feonly")
    cls = m.array("st_cls")
    nbr = m.array("st_nbr").reshape(-1, S)
    blk = m.array("st_blk").reshape(-1, S, d, d)
    u = u_all.reshape(-1, d)
    f = np.zeros((len(feonly), d))
    for i, k in enumerate(feonly):
        c = cls[i]
        assert c >= 0
        for s in range(S):
            j = nbr[i, s]
            if j >= 0:
                f[i] -= blk[c, s] @ u[j]
    return feonly, f


@pytest.mark.parametrize("case,cmd", [("p21", "p21_explicit"), ("b13", "b13_explicit")])
def test_stencil_rows_match_element_force(built, case, cmd):
    m = pdx.Model(case_cmd(case, cmd), device=-1)
    if not np.any(m.array("st_cls") >= 0):
        pytest.skip("stencils not used on this mesh")
    o = orc.Oracle(m)
    d = m.dim
    u = np.random.default_rng(3).standard_normal(m.info.n_node * d) * 1e-5
    f_ref = o.internal_force(u)
    feonly, f = stencil_force(m, u)
    eq = m.array("eq").reshape(-1, d)
    rows = eq[feonly]
    act = rows >= 0
    assert act.sum() > 0
    assert rel(f[act], f_ref[rows[act]]) < 1e-12
    # the classes are shared: far fewer classes than FE-only nodes
    assert len(np.unique(m.array("st_cls"))) * 8 <= len(feonly)


def test_jittered_mesh_keeps_element_path(built, tmp_path):
    mesh = meshgen.box_hole(nx=13, ny=9, nz=3, h=1e-3, radius=2e-3, pd_x=8, pd_y=6)
    rng = np.random.default_rng(5)
    mesh.X[:, :3] += rng.uniform(-1e-4, 1e-4, mesh.X[:, :3].shape)
    cmd = meshgen.write_case(mesh, str(tmp_path), "jit", solver="DYNAMIC", dt=1e-8, nsteps=2, save=1,
                             factor=3.015, nlf=1.0)
    m = pdx.Model(cmd, device=-1)
    assert np.all(m.array("st_cls") == -1)
