"""Edge cases of the particle sets against the oracle, through the C ABI.

* Small open sets: 6 particles (the root is the only leaf: 6 <= minpart),
  11 (one split) and 40, without and with self-gravity; a ragged set of
  12347 particles. Tree permutation, neighbour counts and neighbour-set
  hashes identical; h to 1e-12; forces, du/dt and the potential at the FP64
  bars; three leapfrog steps to 1e-10 with equal iteration counts. With
  6 particles every other particle is a neighbour (2h spans the set).
* Velocity iterations that do not converge: the 11-particle self-gravitating
  set collapses faster than the velocity corrector can follow at its dt;
  the reference stops with its fatal error once its reaches maxits = 30
  (step_leapfrog.f90:753-756); the oracle and the GPU stop at the same step
  (PH_ERR_TOLV).
* Periodic boundary placements (cross_boundary, boundary.f90): particles
  exactly on xmax (kept: only x > xmax wraps), on ymin, just outside zmax and
  xmin, on the far corner, and 0.4 box lengths beyond xmax. Wrapped
  positions identical to the oracle's, forces at the FP64 bars, three steps.
"""
import numpy as np
import pytest

from oracle import oracle as O
from phantom_gb300 import capi
from phantom_gb300 import setups as S

pytestmark = pytest.mark.gpu


def relmax(a, b):
    s = np.abs(b).max()
    return 0.0 if s == 0.0 else np.abs(a - b).max() / s


@pytest.fixture(scope="module", autouse=True)
def _build():
    O.build()
    capi.lib()


def _compare(cfg, x, v, B, nsteps=3):
    o = O.Oracle(cfg, nthreads=8)
    o.set_particles(x, v, B)
    ctx = capi.Context(cfg)
    ctx.upload(x, v, B)
    o.maketree()
    xw, perm, ncells = ctx.build_tree()
    t = o.get_tree()
    assert np.array_equal(perm, t["inodeparts"])
    assert ncells == t["ncells"]
    xo, _, _ = o.get_particles()
    assert np.array_equal(xw, xo)
    o.densityiterate(1)
    do = o.get_density()
    dg = ctx.densityiterate(1)
    assert np.array_equal(dg["nneigh"], do["nneigh"])
    assert np.array_equal(dg["neighhash"], do["neighhash"])
    xo, _, _ = o.get_particles()
    assert relmax(dg["xyzh"][:, 3], xo[:, 3]) < 1.0e-12
    # forces and steps from one derivs each (one density solve from the input h)
    o = O.Oracle(cfg, nthreads=8)
    o.set_particles(x, v, B)
    dto = o.derivs(1, 0.0)
    fo = o.get_force()
    ctx = capi.Context(cfg)
    ctx.upload(x, v, B)
    ctx.derivs(1, 0.0)
    fg = ctx.force(2, 0.0)
    for c in range(4):
        assert relmax(fg["fxyzu"][:, c], fo["fxyzu"][:, c]) < 1.0e-10, c
    assert abs(fg["dtcourant"] / fo["dtcourant"] - 1.0) < 1.0e-12
    assert abs(fg["dtforce"] / fo["dtforce"] - 1.0) < 1.0e-12
    if cfg["gravity"]:
        assert relmax(fg["poten"].astype(np.float64), fo["poten"].astype(np.float64)) < 1.0e-6
    tt, dt = 0.0, dto
    for _ in range(nsteps):
        dto, itso, dterro = o.step(tt, dt)
        _, itsg, _ = ctx.step(tt, dt)
        assert itso == itsg
        xo, vo, _ = o.get_particles()
        xg, vg, _ = ctx.download()
        assert relmax(xg, xo) < 1.0e-10
        assert relmax(vg[:, :3], vo[:, :3]) < 1.0e-10
        tt += dt
        dt = min(dto, dterro)
    return ctx


@pytest.mark.parametrize("n,gravity", [(6, False), (11, False), (40, False), (40, True), (12347, False),
                                       (12347, True)])
def test_small_and_ragged_open_sets(n, gravity):
    cfg, x, v, B = S.random_box(n, seed=n, gravity=gravity)
    ctx = _compare(cfg, x, v, B, nsteps=1 if n == 12347 else 3)
    if n == 6:
        nodes = ctx.nodes()
        assert len(nodes["isleaf"]) == 1 and nodes["isleaf"][0] == 1


def test_clustered_set_beyond_the_indexed_levels():
    """1000 particles in a cube of side 1e-3 inside 1000 spread over the box,
    maxp = 2000: the tree reaches below maxlevel_indexed = 10, where the
    reference numbers nodes from a counter (kdtree.F90:820-833), so ncells
    (2401) exceeds 2^11 - 1; the clump's h (1.2e-4) takes the exact neighbour
    tests instead of the FP32 pre-filter."""
    n = 2000
    cfg, x, v, B = S.random_box(n, seed=7)
    rng = np.random.default_rng(9)
    x = x.copy()
    x[:1000, :3] = rng.uniform(-0.5e-3, 0.5e-3, size=(1000, 3)) + 0.1234
    _compare(cfg, x, v, B, nsteps=1)


def test_velocity_iterations_not_converged_stop_like_the_reference():
    cfg, x, v, B = S.random_box(11, seed=11, gravity=True)
    o = O.Oracle(cfg, nthreads=1)
    o.set_particles(x, v, B)
    ctx = capi.Context(cfg)
    ctx.upload(x, v, B)
    dt = o.derivs(1, 0.0)
    ctx.derivs(1, 0.0)
    t = 0.0
    for k in range(20):
        try:
            dto, _, dterro = o.step(t, dt)
        except RuntimeError:
            with pytest.raises(capi.PhantomError) as e:
                ctx.step(t, dt)
            assert e.value.code == 10
            break
        ctx.step(t, dt)
        t += dt
        dt = min(dto, dterro)
    else:
        pytest.fail("the oracle's velocity iterations converged on every step")


def test_periodic_boundary_placements():
    cfg, x, v, B = S.hydro_lattice(12)
    x = x.copy()
    L = cfg["xmax"] - cfg["xmin"]
    x[0, 0] = cfg["xmax"]
    x[1, 1] = cfg["ymin"]
    x[2, 2] = cfg["zmax"] + 1.0e-3
    x[3, 0] = cfg["xmin"] - 1.0e-3
    x[4, :3] = [cfg["xmax"], cfg["ymax"], cfg["zmax"]]
    x[5, 0] = cfg["xmax"] + 0.4 * L
    _compare(cfg, x, v, B)
