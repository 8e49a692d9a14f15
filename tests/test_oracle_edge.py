"""Edge cases of the oracle itself (CPU): the reference behaviour the GPU edge
tests compare with.

* kdtree.F90:856-865: a node whose particles all land on one side of the
  pivot is split in the middle of its range; 12 coincident particles (more
  than minpart = 10) give a node of 12 with children of 6 and 6.
* kdtree.F90:167-179, 299-301: ncells = 2^(maxlevel+1) - 1 while the tree
  stays within the 2^k-indexed levels; with 6 particles the root is the
  only node.
* dens.F90:1443-1456: no h resolves 12 coincident particles (12 cnormk W(0)
  > hfact^3); the density iteration stops with its fatal error.
* force.F90:1293-1298: a pair at zero separation has no direction; with
  pairs and a group of 4 coincident the forces stay finite and the total
  force vanishes to rounding.
* step_leapfrog.f90:753-756: velocity iterations reaching maxits = 30 stop
  the step (an 11-particle self-gravitating set on its second step).
"""
import numpy as np
import pytest

from oracle import oracle as O
from phantom_gb300 import setups as S


@pytest.fixture(scope="module", autouse=True)
def _build():
    O.build()


def _coincident(cluster, n1d=12, seed=3):
    cfg, x, v, B = S.hydro_lattice(n1d)
    x = x.copy()
    n = len(x)
    rng = np.random.default_rng(seed)
    c0 = n // 2
    for k in rng.choice(c0 - 1, size=10, replace=False):
        x[k, :3] = x[k + 1, :3]
    x[c0:c0 + cluster, :3] = x[c0, :3]
    return cfg, x, v, B


def test_all_on_one_side_split_in_the_middle():
    cfg, x, v, B = _coincident(12)
    o = O.Oracle(cfg, nthreads=1)
    o.set_particles(x, v, B)
    o.maketree()
    t = o.get_tree()
    pos = x[t["inodeparts"] - 1, :3]
    found = 0
    for k in range(t["ncells"]):
        a, b = t["inoderange"][k]
        if a <= 0 or b - a + 1 != 12 or not np.all(pos[a - 1:b] == pos[a - 1]):
            continue
        kl, kr = t["left"][k] - 1, t["right"][k] - 1
        assert kl >= 0 and kr >= 0
        assert tuple(t["inoderange"][kl]) == (a, a + 5)
        assert tuple(t["inoderange"][kr]) == (a + 6, b)
        found += 1
    assert found == 1
    with pytest.raises(RuntimeError):
        o.set_particles(x, v, B)
        o.derivs(1, 0.0)


@pytest.mark.parametrize("n", [6, 11, 40, 12347])
def test_ncells_is_the_indexed_extent(n):
    cfg, x, v, B = S.random_box(n, seed=n)
    o = O.Oracle(cfg, nthreads=1)
    o.set_particles(x, v, B)
    o.maketree()
    o.densityiterate(1)
    st = o.get_density()["stats"]
    assert st["ncells"] == 2 ** (st["maxlevel"] + 1) - 1
    if n == 6:
        assert st["ncells"] == 1


def test_coincident_pairs_have_finite_forces():
    cfg, x, v, B = _coincident(4)
    o = O.Oracle(cfg, nthreads=4)
    o.set_particles(x, v, B)
    o.derivs(1, 0.0)
    f = o.get_force()["fxyzu"]
    assert np.isfinite(f).all()
    m = cfg["massoftype"]
    assert np.abs((m * f[:, :3]).sum(axis=0)).max() <= 1.0e-12 * (m * np.abs(f[:, :3]).sum())


def test_velocity_iterations_reaching_maxits_stop_the_step():
    cfg, x, v, B = S.random_box(11, seed=11, gravity=True)
    o = O.Oracle(cfg, nthreads=1)
    o.set_particles(x, v, B)
    dt = o.derivs(1, 0.0)
    dto, its, dterr = o.step(0.0, dt)
    assert its < 30
    with pytest.raises(RuntimeError, match="status 40"):
        o.step(dt, min(dto, dterr))
