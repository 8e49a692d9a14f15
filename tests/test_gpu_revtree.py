"""ph_revtree (kdtree.F90:1851-2037) on the GPU against the oracle's revtree,
and the reference's own revtree test (test_kdtree.F90:57-135) on the GPU.

Nodes are matched by their particle range (inoderange identifies a node).
Nodes of at most 2048 particles are refitted with the reference's sequential
sums: centres, sizes, hmax and masses bit-exact against the oracle. Larger
nodes use blocked sums: centres and sizes to 1e-13 of the box size, masses
to n eps (the rounding of the reference's sequential sum of n equal masses:
1000 / 30000 summed 30000 times gives 999.99999999975). A density solve on the refitted tree then reproduces the oracle's
on its refitted tree (neighbour counts and hashes bit-exact, h to 1e-12).
"""
import numpy as np
import pytest

from known_answers import KA
from oracle import oracle as O
from phantom_gb300 import capi
from phantom_gb300 import setups as S

pytestmark = pytest.mark.gpu

SMALL = 2048
TOL = KA["kdtree_revtree_tol"]["value"]


def _by_range(rng_arr):
    return {(int(a), int(b)): k for k, (a, b) in enumerate(rng_arr) if a > 0}


def _moved(x, n, seed=5):
    rng = np.random.default_rng(seed)
    xm = x.copy()
    xm[:, :3] += 0.05 * n ** (-1 / 3) * rng.standard_normal((n, 3))
    xm[:, 3] *= 1.0 + 0.01 * rng.standard_normal(n)
    return xm


@pytest.mark.parametrize("name", ["random", "sedov", "grav"])
def test_revtree_matches_oracle(name):
    cfg, x, v, B = {"random": lambda: S.random_box(30000), "sedov": lambda: S.sedov(24),
                    "grav": lambda: S.gravity_cloud(20000)}[name]()
    n = len(x)
    o = O.Oracle(cfg, nthreads=8)
    o.set_particles(x, v, B)
    ctx = capi.Context(cfg)
    ctx.upload(x, v, B)
    o.maketree()
    xw, perm, _ = ctx.build_tree()
    assert np.array_equal(perm, o.get_tree()["inodeparts"])
    xm = _moved(xw, n)
    o.revtree(xm)
    ctx.revtree(xm)
    to, tg = o.get_tree(), ctx.nodes()
    mo, mg = _by_range(to["inoderange"]), _by_range(tg["inoderange"])
    assert set(mo) == set(mg)
    L = 1.0 if name != "grav" else 2.0
    for r, ko in mo.items():
        kg = mg[r]
        cnt = r[1] - r[0] + 1
        if cnt <= SMALL:
            assert np.array_equal(tg["xcen"][kg], to["xcen"][ko]), r
            assert tg["size"][kg] == to["size"][ko], r
            assert tg["mass"][kg] == to["mass"][ko], r
        else:
            assert np.abs(tg["xcen"][kg] - to["xcen"][ko]).max() <= 1.0e-13 * L, r
            assert abs(tg["size"][kg] - to["size"][ko]) <= 1.0e-13 * L, r
            assert abs(tg["mass"][kg] / to["mass"][ko] - 1.0) <= cnt * 2.3e-16, r
        assert tg["hmax"][kg] == to["hmax"][ko], r
    # density on the refitted tree
    o.densityiterate(1)
    do = o.get_density()
    xo, _, _ = o.get_particles()
    dg = ctx.densityiterate(1)
    assert np.array_equal(dg["nneigh"], do["nneigh"])
    assert np.array_equal(dg["neighhash"], do["neighhash"])
    assert np.abs(dg["xyzh"][:, 3] / xo[:, 3] - 1.0).max() < 1.0e-12


def test_revtree_known_answer_gpu():
    """test_kdtree.F90:57-135 on the GPU: revtree on the positions the tree
    was built from reproduces the built tree to the reference's tolerance."""
    cfg, x, v, _ = S.random_box(30000)
    ctx = capi.Context(cfg)
    ctx.upload(x, v)
    xw, _, _ = ctx.build_tree()
    t0 = ctx.nodes()
    ctx.revtree(xw)
    t1 = ctx.nodes()
    assert np.array_equal(t1["inoderange"], t0["inoderange"])
    assert np.array_equal(t1["isleaf"], t0["isleaf"])
    for k in ("xcen", "hmax", "mass"):
        assert (np.abs(t1[k] - t0[k]) <= TOL * np.maximum(np.abs(t0[k]), 1.0)).all(), k
    assert (t1["size"] + TOL >= t0["size"]).all()


def test_revtree_requires_a_tree():
    cfg, x, v, _ = S.random_box(1000)
    ctx = capi.Context(cfg)
    ctx.upload(x, v)
    with pytest.raises(capi.PhantomError) as e:
        ctx.revtree(x)
    assert e.value.code == 13
