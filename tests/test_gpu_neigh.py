"""Neighbour finding on the GPU against brute force (the reference's neigh
test, src/tests/test_neigh.f90): one density evaluation at the input h
(icall = 0) and, per particle, the neighbour count (self included, q_i^2 < 4,
periodic minimum image) against an O(N^2) count in numpy, integer-exact.

* random points in the unit box with random h (test_neigh.f90:31-120);
* 20 particles in a line along each axis (the pathological configurations
  of test_neigh.f90:397-433, where the reference checks that the tree has
  cells): the tree builds, and the counts are exact too.
"""
import numpy as np
import pytest

from phantom_gb300 import capi
from phantom_gb300 import setups as S

pytestmark = pytest.mark.gpu


def _brute(x, L=1.0, periodic=True):
    p = x[:, :3]
    d = p[:, None, :] - p[None, :, :]
    if periodic:
        d = np.where(np.abs(d) > 0.5 * L, d - L * np.sign(d), d)
    r2 = np.sum(d * d, axis=2)
    return np.sum(r2 * (1.0 / x[:, 3] ** 2)[:, None] < 4.0, axis=1)


def _gpu_counts(cfg, x):
    v = np.zeros((len(x), 4)); v[:, 3] = 1.0
    ctx = capi.Context(cfg)
    ctx.upload(x, v)
    xt, perm, ncells = ctx.build_tree()
    assert ncells > 0
    assert np.array_equal(np.sort(perm), np.arange(1, len(x) + 1))
    d = ctx.densityiterate(0)
    return d["nneigh"]


@pytest.mark.parametrize("seed", [24358, 7])
def test_random_points_counts_exact(seed):
    rng = np.random.Generator(np.random.PCG64(seed))
    n = 16 ** 3
    cfg = S.base_cfg(massoftype=1.0 / n, maxp=n, xmin=0.0, xmax=1.0, ymin=0.0, ymax=1.0, zmin=0.0, zmax=1.0)
    x = np.empty((n, 4))
    x[:, :3] = rng.uniform(0.0, 1.0, (n, 3))
    x[:, 3] = rng.uniform(0.01, 0.09, n)
    assert np.array_equal(_gpu_counts(cfg, x), _brute(x))


@pytest.mark.parametrize("axis", [0, 1, 2])
def test_particles_in_a_line(axis):
    n = 20
    psep = 1.0 / n
    cfg = S.base_cfg(massoftype=2.0, maxp=n, xmin=0.0, xmax=1.0, ymin=0.0, ymax=1.0, zmin=0.0, zmax=1.0)
    x = np.zeros((n, 4))
    x[:, axis] = np.arange(n) * psep
    x[:, 3] = cfg["hfact"] * psep
    assert np.array_equal(_gpu_counts(cfg, x), _brute(x))
