"""Batched models (pdx_batch_create): the merged host set-up is the
concatenation of the specimens' own set-ups (CPU), and a batched GPU run gives
every specimen exactly the fields and broken bonds of its single-model run."""
import tempfile

import numpy as np
import pytest

import meshgen
import pdx


def small_c4(n_spec=4, nsteps=60, precision="FP64", seed=0):
    d = tempfile.mkdtemp()
    specs = meshgen.config_c4(n_spec=n_spec, size_range=(20, 40), nsteps=nsteps, precision=precision, seed=seed)
    return [meshgen.write_case(m, d, f"s{i}", **kw) for i, (m, kw) in enumerate(specs)]


def test_batch_setup_is_concatenation(built):
    paths = small_c4()
    singles = [pdx.Model(p, device=-1) for p in paths]
    b = pdx.Model.batch(paths, device=-1)
    no, mo, eo = b.batch_offsets()
    assert b.info.n_node == sum(s.info.n_node for s in singles)
    assert b.info.n_bond == sum(s.info.n_bond for s in singles)
    assert b.info.n_eq == sum(s.info.n_eq for s in singles)
    assert np.array_equal(b.array("bond_state0"), np.concatenate([s.array("bond_state0") for s in singles]))
    fm, eq = b.array("fam_members"), b.array("eq")
    for i, s in enumerate(singles):
        assert np.array_equal(fm[mo[i]:mo[i + 1]], s.array("fam_members") + no[i])
        e = s.array("eq")
        eb = eq[no[i] * 2:no[i + 1] * 2]
        assert np.array_equal(eb[e >= 0], e[e >= 0] + eo[i])
        assert np.all(eb[e < 0] < 0)
        assert np.array_equal(b.array("u0")[no[i] * 2:no[i + 1] * 2], s.array("u0"))


def test_batch_rejects_mixed_dimensions(built, tmp_path):
    p2 = small_c4(n_spec=1)[0]
    mesh = meshgen.box_hole(nx=9, ny=7, nz=3, h=1e-3, radius=1.5e-3, pd_x=4, pd_y=4)
    p3 = meshgen.write_case(mesh, str(tmp_path), "b3", solver="DYNAMIC", dt=1e-8, nsteps=2, save=1, factor=3.015,
                            nlf=1.0, fc="3 1e-3")
    with pytest.raises(pdx.PdxError) as e:
        pdx.Model.batch([p2, p3], device=-1)
    assert e.value.code == 3


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [0, 1])
def test_batched_run_equals_single_runs(built, precision):
    nsteps = 80
    paths = small_c4(n_spec=5, nsteps=nsteps, seed=3)
    results = []
    for p in paths:
        with pdx.Model(p, device=0, precision=precision) as m:
            m.explicit_init()
            m.explicit_advance(nsteps)
            results.append(m.state())
    with pdx.Model.batch(paths, device=0, precision=precision) as b:
        b.explicit_init()
        b.explicit_advance(nsteps)
        u, sig, phi, bs = b.state()
        no, mo, eo = b.batch_offsets()
    nbroken = 0
    for i, (ui, si, pi, bi) in enumerate(results):
        np.testing.assert_array_equal(u[no[i]:no[i + 1]], ui)
        np.testing.assert_array_equal(bs[mo[i]:mo[i + 1]], bi)
        np.testing.assert_array_equal(phi[no[i]:no[i + 1]], pi)
        np.testing.assert_allclose(sig[no[i]:no[i + 1]], si, rtol=0, atol=1e-12 * max(1.0, np.abs(si).max()))
        nbroken += int((bi == 0).sum())
    assert nbroken > 0
