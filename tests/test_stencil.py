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


T2 = dict(X=16, Y=16, WX=18, WY=18)


def tile_decode(m):
    """The mixed step kernel's 2D lattice tiles, decoded on the host: the node
    of every staged site (-1 none), the node of every tile site and the site's
    class entry."""
    rows = m.array("tile_rows").reshape(-1, T2["WY"], 2)
    cls = m.array("tile_cls").astype(np.int32).reshape(len(rows), -1)
    mask = rows[:, :, 1].astype(np.uint32)
    staged = np.full((len(rows), T2["WY"], T2["WX"]), -1, np.int64)
    below = np.zeros(rows.shape[:2], np.int64)
    for x in range(T2["WX"]):
        bit = (mask >> x) & 1
        staged[:, :, x] = np.where(bit == 1, rows[:, :, 0] + below, -1)
        below += bit
    center = staged[:, 1:1 + T2["Y"], 1:1 + T2["X"]].reshape(len(rows), -1)
    return staged, center, cls


def tile_force(m, u):
    """Stencil sums of the tiled FE-only nodes through the tiles (staged
    neighbours by lattice offset, blocks from lat_blk), with the nodes."""
    staged, center, cls = tile_decode(m)
    have = cls >= 0
    lat = m.array("lat_blk").reshape(-1, 9, 2, 2).astype(np.float64)
    ut = np.where(staged[..., None] >= 0, u[np.maximum(staged, 0)], 0.0)
    tiles, sites = np.nonzero(have)
    y, x = np.divmod(sites, T2["X"])
    f = np.zeros((len(tiles), 2))
    for o in range(9):
        dx, dy = o % 3 - 1, o // 3 - 1
        f -= np.einsum("nij,nj->ni", lat[cls[tiles, sites] & 0x3FFF, o], ut[tiles, y + 1 + dy, x + 1 + dx])
    return center[have], cls[have], f


def stencil_force32(m, u, items):
    S = 9
    nbr = m.array("st_nbr").reshape(-1, S)[items]
    cls = m.array("st_cls")[items]
    blk32 = m.array("st_blk").reshape(-1, S, 2, 2).astype(np.float32).astype(np.float64)
    f = np.zeros((len(items), 2))
    for s_ in range(S):
        j = nbr[:, s_]
        ok = j >= 0
        f[ok] -= np.einsum("nij,nj->ni", blk32[cls[ok], s_], u[j[ok]])
    return f


@pytest.mark.parametrize("case", ["p21", "c4", "c1"])
def test_lattice_tiles_reproduce_stencils(built, case, tmp_path):
    """Every FE-only node of a 2D lattice mesh sits on exactly one tile site
    with its own stencil class, the tile stencil gives the per-node stencil
    sum, and the shadow bit marks every family member."""
    if case == "p21":
        cmd = case_cmd("p21", "p21_explicit")
    elif case == "c4":
        mesh, kw = meshgen.config_c4(n_spec=3, nsteps=2)[2]
        cmd = meshgen.write_case(mesh, str(tmp_path), "c4", **kw)
    else:
        mesh, kw = meshgen.config_c1(nsteps=2)
        cmd = meshgen.write_case(mesh, str(tmp_path), "c1", **kw)
    m = pdx.Model(cmd, device=-1)
    feonly = m.array("feonly")
    assert m.array_len("tile_rows") > 0, "lattice tiles not built"
    assert m.array_len("fe_rest") == 0
    nodes, cls, f_t = tile_force(m, np.random.default_rng(1).standard_normal((m.info.n_node, 2)))
    assert np.array_equal(np.sort(nodes), np.sort(feonly))
    pos = {int(k): i for i, k in enumerate(feonly)}
    items = np.array([pos[int(k)] for k in nodes])
    assert np.array_equal(cls & 0x3FFF, m.array("st_cls")[items])
    f_ref = stencil_force32(m, np.random.default_rng(1).standard_normal((m.info.n_node, 2)), items)
    assert rel(f_t, f_ref) < 1e-12
    need = np.zeros(m.info.n_node, bool)
    need[m.array("fam_members")] = True
    assert not np.any(need[nodes] & ((cls & 0x4000) == 0))


def test_3d_models_keep_per_node_stencils(built):
    m = pdx.Model(case_cmd("b13", "b13_explicit"), device=-1)
    assert m.array_len("tile_rows") == 0 and np.any(m.array("st_cls") >= 0)


def small_plate(tmp_path):
    """A 20 x 20-node plate whose PD band leaves a handful of FE-only nodes:
    no stencil classes, so no tiles."""
    for seed in range(50):
        mesh, kw = meshgen.config_c4(n_spec=1, size_range=(20, 20), nsteps=2, seed=seed)[0]
        p = meshgen.write_case(mesh, str(tmp_path), f"small{seed}", **kw)
        if pdx.Model(p, device=-1).array_len("tile_rows") == 0:
            return p
    raise AssertionError("no untiled small plate found")


def test_lattice_tiles_of_a_batch(built, tmp_path):
    """Batched models carry every specimen's tiles with node ids and classes
    shifted; the FE-only nodes of a specimen without tiles are listed for the
    per-node path."""
    paths = [meshgen.write_case(mesh, str(tmp_path), f"s{i}", **kw)
             for i, (mesh, kw) in enumerate(meshgen.config_c4(n_spec=3, size_range=(20, 40), nsteps=2))]
    paths.append(small_plate(tmp_path))
    b = pdx.Model.batch(paths, device=-1)
    feonly, rest = b.array("feonly"), b.array("fe_rest")
    assert len(rest) > 0
    u = np.random.default_rng(2).standard_normal((b.info.n_node, 2))
    nodes, cls, f_t = tile_force(b, u)
    assert np.array_equal(np.sort(np.concatenate([nodes, feonly[rest]])), np.sort(feonly))
    pos = {int(k): i for i, k in enumerate(feonly)}
    items = np.array([pos[int(k)] for k in nodes])
    assert np.array_equal(cls & 0x3FFF, b.array("st_cls")[items])
    assert rel(f_t, stencil_force32(b, u, items)) < 1e-12
