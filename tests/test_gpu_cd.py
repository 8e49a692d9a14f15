"""Cullen & Dehnen viscosity switch on the GPU (nalpha = 3) against the
oracle, through the C ABI.

* The velocity-derivative pass: d(div v)/dt and dvdx(9) (float storage, as
  the reference) agree to 1e-6 of their largest magnitude (FP64 sums in a
  different order, rounded to float); a linear velocity field gives dvdx = A
  and d(div v)/dt = -tr(A A) on the GPU too.
* alphaloc (cons2prim) to 1e-6; forces with a per-particle alpha to 1e-10.
* Three leapfrog steps with the switch evolving alpha: positions and
  velocities to 1e-10, alpha to 1e-6.
* The mixed form with the switch stays within 1e-5 of the FP64 path.
"""
import numpy as np
import pytest

from oracle import oracle as O
from phantom_gb300 import capi
from phantom_gb300 import setups as S

pytestmark = pytest.mark.gpu

A = np.array([[0.3, -0.2, 0.1], [0.05, -0.4, 0.2], [0.1, 0.15, -0.25]])


def relmax(a, b):
    s = np.abs(b).max()
    return 0.0 if s == 0.0 else np.abs(a - b).max() / s


def _cd(cfg):
    return dict(cfg, nalpha=3, alpha=0.0, alphamax=1.0)


WL = {"sedov": lambda: S.sedov(16), "hydro": lambda: S.hydro_lattice(16), "mhd": lambda: S.mhd_vortex(12),
      "grav": lambda: S.gravity_cloud(5000)}


def _pair(name):
    cfg, x, v, B = WL[name]()
    cfg = _cd(cfg)
    o = O.Oracle(cfg, nthreads=8)
    o.set_particles(x, v, B)
    ctx = capi.Context(cfg)
    ctx.upload(x, v, B)
    return cfg, (x, v, B), o, ctx


def test_linear_field_known_answer_gpu():
    cfg, x, v, B = S.random_box(20000, seed=4)
    cfg = dict(_cd(cfg), tolh=1.0e-6)
    v = v.copy()
    v[:, :3] = x[:, :3] @ A.T
    ctx = capi.Context(cfg)
    ctx.upload(x, v)
    ctx.build_tree()
    ctx.densityiterate(1)
    a, d = ctx.get_alpha()
    assert np.abs(d - A.reshape(1, 9)).max() <= 2.0 ** -23 * np.abs(A).max()
    assert np.abs(a[:, 2] + np.trace(A @ A)).max() <= 2.0 ** -22 * abs(np.trace(A @ A))


@pytest.mark.parametrize("name", list(WL))
def test_switch_parity(name):
    cfg, (x, v, B), o, ctx = _pair(name)
    rng = np.random.default_rng(3)
    alpha = rng.uniform(0.0, 1.0, len(x)).astype(np.float32)
    o.set_alpha(alpha)
    ctx.set_alpha(alpha)
    o.derivs(1, 0.0)
    ctx.derivs(1, 0.0)
    ao, do = o.get_alpha()
    ag, dg = ctx.get_alpha()
    assert np.array_equal(ag[:, 0], alpha)
    assert relmax(ag[:, 2].astype(np.float64), ao[:, 2].astype(np.float64)) < 1.0e-6
    assert relmax(dg.astype(np.float64), do.astype(np.float64)) < 1.0e-6
    assert relmax(ag[:, 1].astype(np.float64), ao[:, 1].astype(np.float64)) < 1.0e-6
    fo = o.get_force()["fxyzu"]
    fg = ctx.force(2, 0.0)["fxyzu"]
    for c in range(4):
        assert relmax(fg[:, c], fo[:, c]) < 1.0e-10, c


@pytest.mark.parametrize("name", ["sedov", "mhd"])
def test_steps_with_switch_parity(name):
    cfg, (x, v, B), o, ctx = _pair(name)
    dto = o.derivs(1, 0.0)
    dtg = ctx.derivs(1, 0.0)
    o.alpha_initial()
    ctx.alpha_initial()
    t = 0.0
    dt = min(dto, dtg)
    for _ in range(3):
        o.step(t, dt)
        ctx.step(t, dt)
        t += dt
    xo, vo, Bo = o.get_particles()
    xg, vg, Bg = ctx.download()
    assert relmax(xg[:, :3], xo[:, :3]) < 1.0e-10
    assert relmax(vg, vo) < 1.0e-10
    ag, _ = ctx.get_alpha()
    ao, _ = o.get_alpha()
    assert relmax(ag[:, 0].astype(np.float64), ao[:, 0].astype(np.float64)) < 1.0e-6
    assert ag[:, 0].max() > 0.0


def test_mixed_form_with_switch():
    cfg, x, v, B = S.sedov(24)
    cfg = _cd(cfg)
    out = {}
    for prec in (capi.PH_PREC_FP64, capi.PH_PREC_MIXED):
        ctx = capi.Context(cfg, precision=prec)
        ctx.upload(x, v)
        ctx.set_alpha(np.full(len(x), 0.5, np.float32))
        ctx.derivs(1, 0.0)
        out[prec] = (ctx.force(2, 0.0)["fxyzu"], ctx.get_alpha()[0])
    fa, aa = out[capi.PH_PREC_FP64]
    fm, am = out[capi.PH_PREC_MIXED]
    s = np.abs(fa[:, :3]).max()
    assert np.abs(fm[:, :3] - fa[:, :3]).max() / s < 1.0e-5
    assert relmax(am[:, 1].astype(np.float64), aa[:, 1].astype(np.float64)) < 1.0e-3


def test_adjoint_runs_with_the_switch():
    # the adjoint of one derivs holds alpha fixed (its finite-difference check
    # is in test_gpu_adjoint.py); a zero cotangent gives zero gradients
    cfg, x, v, B = S.hydro_lattice(8)
    ctx = capi.Context(_cd(cfg))
    ctx.upload(x, v)
    gx, gv = ctx.adjoint(np.zeros((len(x), 4)))
    assert not gx.any() and not gv.any()


def test_rejects_other_nalpha():
    cfg, x, v, B = S.hydro_lattice(8)
    with pytest.raises(capi.PhantomError):
        capi.Context(dict(cfg, nalpha=2))
