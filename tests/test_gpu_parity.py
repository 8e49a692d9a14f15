"""GPU parity against the CPU oracle, through the C ABI.

Bars: tree permutation, per-particle neighbour counts and neighbour-set hashes
and all neighbour statistics are bit-exact; smoothing lengths agree to 1e-12
relative; gradh (stored in float32 as in the reference) to one float ulp;
accelerations, du/dt and dB/dt to 1e-10 of their maximum magnitude (FP64 path,
different summation order); timesteps to 1e-12; three leapfrog steps to 1e-10.
"""
import numpy as np
import pytest

from oracle import oracle as O
from phantom_gb300 import capi
from phantom_gb300 import setups as S

pytestmark = pytest.mark.gpu

WORKLOADS = {
    "lattice16": lambda: S.exact_lattice(16),
    "hydro24": lambda: S.hydro_lattice(24),
    "sedov32": lambda: S.sedov(32),
    "mhd24": lambda: S.mhd_vortex(24),
    "grav6k": lambda: S.gravity_cloud(6000),
}


def relmax(a, b):
    s = np.abs(b).max()
    return 0.0 if s == 0.0 else np.abs(a - b).max() / s


@pytest.fixture(scope="module", autouse=True)
def _build():
    O.build()
    capi.lib()


def _pair(name, nthreads=8):
    cfg, x, v, B = WORKLOADS[name]()
    o = O.Oracle(cfg, nthreads=nthreads)
    o.set_particles(x, v, B)
    ctx = capi.Context(cfg)
    ctx.upload(x, v, B)
    return cfg, (x, v, B), o, ctx


@pytest.mark.parametrize("name", list(WORKLOADS))
def test_tree_permutation_identical(name):
    _, _, o, ctx = _pair(name)
    o.maketree()
    t = o.get_tree()
    xw, perm, _ = ctx.build_tree()
    assert np.array_equal(perm, t["inodeparts"])
    xo, _, _ = o.get_particles()
    assert np.array_equal(xw, xo)  # periodic wrap identical


@pytest.mark.parametrize("name", list(WORKLOADS))
def test_density_parity(name):
    _, _, o, ctx = _pair(name)
    o.maketree(); o.densityiterate(1)
    do = o.get_density(); xo, _, _ = o.get_particles()
    ctx.build_tree()
    dg = ctx.densityiterate(1)
    assert np.array_equal(dg["nneigh"], do["nneigh"])
    assert np.array_equal(dg["neighhash"], do["neighhash"])
    for k in ("nneightry", "nneighact", "maxneightry", "maxneighact", "ncalc", "np", "ncalls_neigh",
              "ncells", "maxlevel", "minlevel"):
        assert dg["stats"][k] == do["stats"][k], k
    assert relmax(dg["xyzh"][:, 3], xo[:, 3]) < 1.0e-12
    gr = np.abs(dg["gradh"][:, 0].astype(np.float64) / do["gradh"][:, 0] - 1.0).max()
    assert gr <= 2.0 ** -23
    if do["divcurlB"].any():
        assert relmax(dg["divcurlB"].astype(np.float64), do["divcurlB"].astype(np.float64)) < 1.0e-5


@pytest.mark.parametrize("name", ["hydro24", "sedov32", "mhd24", "grav6k"])
def test_force_parity(name):
    _, (x, v, _), o, ctx = _pair(name)
    dto = o.derivs(1, 0.0)
    fo = o.get_force()
    dtg = ctx.derivs(1, 0.0)
    fg = ctx.force(2, 0.0)
    assert abs(dtg / dto - 1.0) < 1.0e-12
    for c in range(4):
        assert relmax(fg["fxyzu"][:, c], fo["fxyzu"][:, c]) < 1.0e-10, c
        assert relmax(fg["dBevol"][:, c], fo["dBevol"][:, c]) < 1.0e-10, c
    assert abs(fg["dtcourant"] / fo["dtcourant"] - 1.0) < 1.0e-12
    assert abs(fg["dtforce"] / fo["dtforce"] - 1.0) < 1.0e-12
    # div v relative to its largest value, or to a floor of 1e-9 v/h where the
    # flow is divergence free (the rotating cloud: div v is rounding noise)
    dvg, dvo = fg["divcurlv"].astype(np.float64), fo["divcurlv"].astype(np.float64)
    vscale = np.abs(v[:, :3]).max() / x[:, 3].min()
    assert np.abs(dvg - dvo).max() <= 1.0e-6 * max(np.abs(dvo).max(), 1.0e-9 * vscale)
    if name.startswith("grav"):
        # self-gravity: softened near field + tree far field, potential (float32)
        assert relmax(fg["poten"].astype(np.float64), fo["poten"].astype(np.float64)) < 1.0e-6


@pytest.mark.parametrize("name", ["hydro24", "sedov32", "mhd24", "grav6k"])
def test_leapfrog_steps_parity(name):
    cfg, _, o, ctx = _pair(name)
    dt = o.derivs(1, 0.0)
    ctx.derivs(1, 0.0)
    t = 0.0
    for _ in range(3):
        dto, itso, dterro = o.step(t, dt)
        dtg, itsg, dterrg = ctx.step(t, dt)
        assert itso == itsg
        assert abs(dtg / dto - 1.0) < 1.0e-10
        xo, vo, bo = o.get_particles()
        xg, vg, bg = ctx.download()
        assert relmax(xg, xo) < 1.0e-10
        assert relmax(vg[:, :3], vo[:, :3]) < 1.0e-10
        assert relmax(vg[:, 3], vo[:, 3]) < 1.0e-10
        if cfg["mhd"]:
            assert relmax(bg, bo) < 1.0e-10
        t += dt
        dt = min(dto, dterro)


def test_momentum_conservation_gpu():
    cfg, x, v, B = S.hydro_lattice(32)
    ctx = capi.Context(cfg)
    ctx.upload(x, v, B)
    ctx.derivs(1, 0.0)
    f = ctx.force(2, 0.0)["fxyzu"]
    m = cfg["massoftype"]
    assert np.abs((m * f[:, :3]).sum(axis=0)).max() < 1.0e-13 * (m * np.abs(f[:, :3]).sum())


def test_sedov_known_answer_gpu():
    """The reference's Sedov known-answer run (test_sedov.f90) through ph_step
    on the GPU: same step count, final state and conservation as the oracle."""
    import os
    import sys
    sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
    from known_answers import KA, sedov_known_answer_run
    cfg, x, v, B = S.sedov_test()
    o = O.Oracle(cfg, nthreads=8)
    o.set_particles(x, v, B)
    dto = o.derivs(1, 0.0)
    de_o, mom_o, n_o, xo, vo = sedov_known_answer_run((dto, o), cfg, x, v, B)
    ctx = capi.Context(cfg)
    ctx.upload(x, v, B)
    dtg = ctx.derivs(1, 0.0)
    de_g, mom_g, n_g, xg, vg = sedov_known_answer_run((dtg, ctx), cfg, x, v, B)
    assert n_g == n_o
    assert abs(de_g - de_o) < 1.0e-8
    assert mom_g < KA["sedov_momentum_tol"]["value"]
    assert relmax(xg, xo) < 1.0e-10
    assert relmax(vg, vo) < 1.0e-10


def test_periodic_self_gravity_parity():
    """Self-gravity in a periodic box: the far field's node separations and
    the near field's trial leaves take periodic images (node_sep codes, as
    getneigh_dual). Random particles in [-0.5, 0.5)^3, periodic, FP64 path
    against the oracle: accelerations to 1e-10, potential to 1e-6."""
    cfg, x, v, B = S.random_box(6000, seed=5, gravity=True)
    cfg = dict(cfg, periodic=1, xmin=-0.5, xmax=0.5, ymin=-0.5, ymax=0.5, zmin=-0.5, zmax=0.5)
    o = O.Oracle(cfg, nthreads=8)
    o.set_particles(x, v, B)
    o.derivs(1, 0.0)
    fo = o.get_force()
    ctx = capi.Context(cfg)
    ctx.upload(x, v, B)
    ctx.derivs(1, 0.0)
    fg = ctx.force(2, 0.0)
    for c in range(4):
        assert relmax(fg["fxyzu"][:, c], fo["fxyzu"][:, c]) < 1.0e-10, c
    assert relmax(fg["poten"].astype(np.float64), fo["poten"].astype(np.float64)) < 1.0e-6
