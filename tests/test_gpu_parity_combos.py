"""GPU parity against the oracle for physics and geometry combinations the
single-feature sets do not cover, through the C ABI, at the FP64 bars:
tree permutation, neighbour counts and neighbour-set hashes identical, h to
1e-12, accelerations, du/dt, dB/dt and dpsi/dt to 1e-10 of their maximum,
the potential to 1e-6, three leapfrog steps (x, v and B) to 1e-10 with equal
iteration counts; the precision form within 1e-5.

* a rectangular periodic box [0,1) x [0,0.5) x [0,0.25) (dxbound, dybound,
  dzbound all different: boundary.f90 wraps and get_sep's minimum image per
  axis), adiabatic hydro on a jittered 24 x 12 x 6 lattice;
* ideal MHD with self-gravity in open boundaries (the softened near field
  and the tree far field beside the Lorentz force and the cleaning): an
  isothermal cloud of 3000 particles with B = 0.2 z plus a random part;
* isothermal ideal MHD in a periodic box (P = c_s^2 rho beside the magnetic
  pressure, force.F90:2068-2168): the MHD vortex field with ieos = 1;
* adiabatic self-gravity in the rectangular periodic box (node separations
  and near-field trial leaves take each axis's own periodic image): 6000
  random particles;
* hfact 1.0 and 1.5 (about 30 and 107 neighbours), gamma 1.4, and opening
  angles 0.3 and 0.8 for the self-gravitating cloud;
* the runtime switches of the energy equation and the MHD terms, one derivs
  each: pdV or shock heating off, no conductivity and no quadratic
  viscosity, resistive heating off, no cleaning, other cleaning and
  resistivity strengths.
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


def rect_box():
    nx, ny, nz = 24, 12, 6
    dx = 1.0 / nx
    rng = np.random.Generator(np.random.PCG64(5))
    g = np.stack(np.meshgrid((np.arange(nx) + 0.5) * dx, (np.arange(ny) + 0.5) * dx, (np.arange(nz) + 0.5) * dx,
                             indexing="ij"), axis=-1).reshape(-1, 3)
    L = np.array([1.0, 0.5, 0.25])
    pos = np.mod(g + rng.normal(0.0, 0.05 * dx, size=g.shape), L)
    n = len(pos)
    x = np.empty((n, 4)); x[:, :3] = pos; x[:, 3] = 1.2 * dx
    v = np.empty((n, 4)); v[:, :3] = rng.uniform(-0.1, 0.1, size=(n, 3)); v[:, 3] = 1.0
    cfg = S.base_cfg(massoftype=float(L.prod()) / n, maxp=n, xmax=1.0, ymax=0.5, zmax=0.25)
    return cfg, x, v, np.zeros((n, 4))


def mhd_cloud():
    cfg, x, v, B = S.gravity_cloud(3000)
    n = len(x)
    rng = np.random.default_rng(43)
    cfg = dict(cfg, mhd=1)
    v = v.copy(); v[:, :3] += 0.1 * rng.standard_normal((n, 3))
    rho0 = 1.0 / (4.0 / 3.0 * np.pi)
    B = np.zeros((n, 4))
    B[:, 2] = 0.2 / rho0
    B[:, :3] += 0.05 / rho0 * rng.standard_normal((n, 3))
    B[:, 3] = 0.02 * rng.standard_normal(n)
    return cfg, x, v, B


def isothermal_mhd():
    cfg, x, v, B = S.mhd_vortex(16)
    cs = 0.3
    return dict(cfg, isothermal=1, ieos=1, polyk=cs * cs), x, v, B


def rect_box_gravity():
    n = 6000
    rng = np.random.Generator(np.random.PCG64(17))
    L = np.array([1.0, 0.5, 0.25])
    x = np.empty((n, 4)); x[:, :3] = rng.uniform(0.0, 1.0, size=(n, 3)) * L
    x[:, 3] = 1.2 * (float(L.prod()) / n) ** (1.0 / 3.0)
    v = np.zeros((n, 4)); v[:, :3] = 0.05 * rng.standard_normal((n, 3)); v[:, 3] = 1.0
    cfg = S.base_cfg(massoftype=1.0 / n, maxp=n, xmax=1.0, ymax=0.5, zmax=0.25, gravity=1)
    return cfg, x, v, np.zeros((n, 4))


def with_cfg(make, **kw):
    def f():
        cfg, x, v, B = make()
        return dict(cfg, **kw), x, v, B
    return f


SETS = {"rect_box": rect_box, "mhd_cloud": mhd_cloud, "isothermal_mhd": isothermal_mhd,
        "rect_box_gravity": rect_box_gravity,
        # about 30 and 107 neighbours: shorter and longer pair queues than hfact 1.2
        "hfact_1.0": lambda: S.hydro_lattice(16, hfact=1.0),
        "hfact_1.5": lambda: S.hydro_lattice(16, hfact=1.5),
        "gamma_1.4": with_cfg(lambda: S.hydro_lattice(16), gamma=1.4),
        # opening angles either side of the configuration's 0.5
        "theta_0.3": with_cfg(lambda: S.gravity_cloud(3000), tree_accuracy=0.3),
        "theta_0.8": with_cfg(lambda: S.gravity_cloud(3000), tree_accuracy=0.8)}


@pytest.mark.parametrize("name", list(SETS))
def test_fp64_parity(name):
    cfg, x, v, B = SETS[name]()
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
    # forces and steps from one derivs each
    o = O.Oracle(cfg, nthreads=8)
    o.set_particles(x, v, B)
    dto = o.derivs(1, 0.0)
    fo = o.get_force()
    ctx = capi.Context(cfg)
    ctx.upload(x, v, B)
    ctx.derivs(1, 0.0)
    fg = ctx.force(2, 0.0)
    for c in range(fo["fxyzu"].shape[1]):
        assert relmax(fg["fxyzu"][:, c], fo["fxyzu"][:, c]) < 1.0e-10, c
    if cfg["mhd"]:
        for c in range(4):
            assert relmax(fg["dBevol"][:, c], fo["dBevol"][:, c]) < 1.0e-10, c
    if cfg["gravity"]:
        assert relmax(fg["poten"].astype(np.float64), fo["poten"].astype(np.float64)) < 1.0e-6
    assert abs(fg["dtcourant"] / fo["dtcourant"] - 1.0) < 1.0e-12
    assert abs(fg["dtforce"] / fo["dtforce"] - 1.0) < 1.0e-12
    tt, dt = 0.0, dto
    for _ in range(3):
        dto, itso, dterro = o.step(tt, dt)
        _, itsg, _ = ctx.step(tt, dt)
        assert itso == itsg
        xo, vo, bo = o.get_particles()
        xg, vg, bg = ctx.download()
        assert relmax(xg, xo) < 1.0e-10
        assert relmax(vg[:, :3], vo[:, :3]) < 1.0e-10
        if cfg["mhd"]:
            assert relmax(bg, bo) < 1.0e-10
        tt += dt
        dt = min(dto, dterro)


@pytest.mark.parametrize("name", list(SETS))
def test_precision_form_within_bar(name):
    cfg, x, v, B = SETS[name]()
    tight = dict(cfg, tolh=1.0e-7)  # both forms converged: the bar is the pair arithmetic's
    o = O.Oracle(tight, nthreads=8)
    o.set_particles(x, v, B)
    o.derivs(1, 0.0)
    fo = o.get_force()
    ctx = capi.Context(tight, precision=capi.PH_PREC_MIXED)
    ctx.upload(x, v, B)
    ctx.derivs(1, 0.0)
    fg = ctx.force(2, 0.0)
    assert np.isfinite(fg["fxyzu"]).all()
    a_g, a_o = fg["fxyzu"][:, :3], fo["fxyzu"][:, :3]
    assert np.abs(a_g - a_o).max() <= 1.0e-5 * np.abs(a_o).max()


OPTIONS = [
    ("hydro", dict(ipdv_heating=0)),
    ("hydro", dict(ishock_heating=0)),
    ("hydro", dict(alphau=0.0, beta=0.0)),
    ("mhd", dict(iresistive_heating=0)),
    ("mhd", dict(psidecayfac=0.0)),
    ("mhd", dict(overcleanfac=2.0, alphaB=0.5)),
]


@pytest.mark.parametrize("base,opts", OPTIONS)
def test_runtime_options_match_oracle(base, opts):
    """The reference's runtime switches on the energy equation and the MHD
    terms (force.F90 finish_cell_and_store_results and the pair terms):
    pdV and shock heating off, no conductivity or quadratic viscosity,
    resistive heating off, no divergence cleaning, other cleaning and
    resistivity strengths. One derivs, FP64, at the parity bars."""
    cfg, x, v, B = S.hydro_lattice(16) if base == "hydro" else S.mhd_vortex(12)
    cfg = dict(cfg, **opts)
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
        if cfg["mhd"]:
            assert relmax(fg["dBevol"][:, c], fo["dBevol"][:, c]) < 1.0e-10, c
    assert abs(fg["dtcourant"] / fo["dtcourant"] - 1.0) < 1.0e-12
    assert abs(fg["dtforce"] / fo["dtforce"] - 1.0) < 1.0e-12
