"""The reference's derivshydro test (src/tests/test_derivs.f90:179-262, checks
check_hydro :1100-1126 and check_fxyzu :1164-1185) restated: a periodic cubic
lattice of 100^3 particles (psep = L/100), rho0 = 5, hfact = 1.2, tolh = 1e-5,
gamma = 5/3, dissipation off, the analytic velocity and thermal-energy fields
of set_velocity_and_energy. One derivs; the bars are the reference's:
h = h0 to 3.6e-4, div v (from the force loop under CONST_AV) against the
analytic divergence to 1e-3, the accelerations against -(gamma-1) grad u to
1e-3, du/dt / ((gamma-1) u) against -div v to 1e-3, gradh = 1.01948 to 1e-5.
And derivsav (test_derivs.f90:837-884): constant u = 4, alpha = 0.753,
With curl v on (phantomtest.f90:33 sets curlv; test_derivs.f90:1118-1121),
the three curl rows of divcurlv against the analytic curl to 1.5e-3, 1e-3,
1e-3.
the viscous accelerations against the continuum form c1 del^2 v + c2 grad
div v (av_coeffs, forceavx/y/z) to 5.7e-3 / 1.4e-2 / 1.3e-2.
And derivsmhd (test_derivs.f90:465-510): no pressure, the analytic B
field with B_ext: h to 3e-4, div B (symmetric, force loop) to 2e-3,
d(B/rho)/dt to 2e-3 / 2e-3 / 2e-2, the Lorentz force to 2.5e-2, div B and
curl B from the density loop to 1e-3 (the mixed form with its 1e-5 budget
added: the y force sits at 0.02499967 of its 0.025 bar in FP64).
The oracle (CPU), the GPU's FP64 path and its mixed form."""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
import derivs_fields as F  # noqa: E402

from phantom_gb300 import setups as S  # noqa: E402

XMIN, L = -0.5, 1.0


def _setup(curlv=0):
    cfg, x, v, B = S.exact_lattice(100, rho0=5.0)
    cfg = dict(cfg, alpha=0.0, alphau=0.0, alphaB=0.0, beta=0.0, curlv=curlv)
    vv, u = F.fields(x[:, :3], XMIN, L)
    v[:, :3] = vv
    v[:, 3] = u
    return cfg, x, v, B, u


def _check(cfg, x0, xo, fxyzu, divcurlv, gradh1, u):
    h0 = x0[0, 3]
    assert np.abs(xo[:, 3] / h0 - 1.0).max() <= 3.6e-4  # relative (stricter than the absolute-or-relative rule)
    pos = xo[:, :3]
    dcv = divcurlv.astype(np.float64).reshape(len(xo), -1)
    assert F.checkvalf(dcv[:, 0], F.divv(pos, XMIN, L), 1.0e-3) <= 1.0e-3
    if dcv.shape[1] == 4:  # curl v (test_derivs.f90:1118-1121, curlvfuncx/y/z :1466-1487)
        g = F.vgrad(pos, XMIN, L)
        curl = (g[:, 2, 1] - g[:, 1, 2], g[:, 0, 2] - g[:, 2, 0], g[:, 1, 0] - g[:, 0, 1])
        for k, tol in enumerate((1.5e-3, 1.0e-3, 1.0e-3)):
            assert F.checkvalf(dcv[:, 1 + k], curl[k], tol) <= tol, k
    fe = F.force(pos, XMIN, L, cfg["gamma"])
    for k in range(3):
        assert F.checkvalf(fxyzu[:, k], fe[:, k], 1.0e-3) <= 1.0e-3, k
    dudt = fxyzu[:, 3] / ((cfg["gamma"] - 1.0) * u)
    assert F.checkvalf(dudt, -F.divv(pos, XMIN, L), 1.0e-3) <= 1.0e-3
    assert F.checkvalf(gradh1.astype(np.float64), np.full(len(xo), 1.01948), 1.0e-5) <= 1.0e-5


@pytest.mark.parametrize("curlv", [0, 1])
def test_oracle_derivshydro_analytic(curlv):
    from oracle import oracle as O
    O.build()
    cfg, x, v, B, u = _setup(curlv)
    o = O.Oracle(cfg, nthreads=8)
    o.set_particles(x, v, B)
    o.derivs(1, 0.0)
    xo, _, _ = o.get_particles()
    f = o.get_force()
    d = o.get_density()
    _check(cfg, x, xo, f["fxyzu"], f["divcurlv"], d["gradh"][:, 0], u)


@pytest.mark.gpu
@pytest.mark.parametrize("curlv", [0, 1])
@pytest.mark.parametrize("mixed", [False, True])
def test_gpu_derivshydro_analytic(mixed, curlv):
    from phantom_gb300 import capi
    cfg, x, v, B, u = _setup(curlv)
    ctx = capi.Context(cfg, precision=capi.PH_PREC_MIXED if mixed else capi.PH_PREC_FP64)
    ctx.upload(x, v, B)
    ctx.build_tree()
    d = ctx.densityiterate(1)
    fo = ctx.force(1)
    _check(cfg, x, d["xyzh"], fo["fxyzu"], fo["divcurlv"], d["gradh"][:, 0], u)


AV_TOLS = (5.7e-3, 1.4e-2, 1.3e-2)


def _setup_av():
    """derivsav (test_derivs.f90:837-884): the same lattice and velocity
    field, constant u = 4, alpha = 0.753 (beta, alphau off)."""
    cfg, x, v, B = S.exact_lattice(100, rho0=5.0)
    cfg = dict(cfg, alpha=0.753, alphau=0.0, alphaB=0.0, beta=0.0)
    vv, _ = F.fields(x[:, :3], XMIN, L)
    v[:, :3] = vv
    v[:, 3] = 4.0
    return cfg, x, v, B


def _check_av(cfg, xo, fxyzu):
    fe = F.av_force(xo[:, :3], xo[:, 3], XMIN, L, cfg["gamma"], cfg["alpha"])
    for k in range(3):
        assert F.checkvalf(fxyzu[:, k], fe[:, k], AV_TOLS[k]) <= AV_TOLS[k], k


def test_oracle_derivsav_analytic():
    from oracle import oracle as O
    O.build()
    cfg, x, v, B = _setup_av()
    o = O.Oracle(cfg, nthreads=8)
    o.set_particles(x, v, B)
    o.derivs(1, 0.0)
    xo, _, _ = o.get_particles()
    _check_av(cfg, xo, o.get_force()["fxyzu"])


@pytest.mark.gpu
@pytest.mark.parametrize("mixed", [False, True])
def test_gpu_derivsav_analytic(mixed):
    from phantom_gb300 import capi
    cfg, x, v, B = _setup_av()
    ctx = capi.Context(cfg, precision=capi.PH_PREC_MIXED if mixed else capi.PH_PREC_FP64)
    ctx.upload(x, v, B)
    ctx.build_tree()
    d = ctx.densityiterate(1)
    fo = ctx.force(1)
    _check_av(cfg, d["xyzh"], fo["fxyzu"])


def _setup_mhd():
    """derivsmhd (test_derivs.f90:465-510): the same lattice and velocity
    field, no pressure (u = 0), B = B_ext + the analytic field as B/rho,
    psi = 0, dissipation off."""
    cfg, x, v, B = S.exact_lattice(100, rho0=5.0)
    cfg = dict(cfg, mhd=1, alpha=0.0, alphau=0.0, alphaB=0.0, beta=0.0, polyk=0.0)
    vv, _ = F.fields(x[:, :3], XMIN, L)
    v[:, :3] = vv
    v[:, 3] = 0.0
    Bf, _ = F.bfield(x[:, :3], XMIN, L)
    rho = cfg["massoftype"] * (cfg["hfact"] / x[:, 3]) ** 3
    Bevol = np.zeros((len(x), 4))
    Bevol[:, :3] = Bf / rho[:, None]
    return cfg, x, v, Bevol


def _check_mhd(cfg, x0, xo, fo, divcurlB, slack=0.0):
    """The reference's bars (+ slack: the mixed form's 1e-5 error budget)."""
    assert np.abs(xo[:, 3] / x0[0, 3] - 1.0).max() <= 3.0e-4
    rho = cfg["massoftype"] * (cfg["hfact"] / xo[:, 3]) ** 3
    divB, curlB, dBdt, fm = F.mhd_expected(xo[:, :3], rho, 5.0, XMIN, L)
    assert F.checkvalf(fo["divBsymm"].astype(np.float64), divB, 2.0e-3) <= 2.0e-3 + slack
    for k, tol in zip(range(3), (2.0e-3, 2.0e-3, 2.0e-2)):
        assert F.checkvalf(fo["dBevol"][:, k], dBdt[:, k], tol) <= tol + slack, k
    for k in range(3):
        assert F.checkvalf(fo["fxyzu"][:, k], fm[:, k], 2.5e-2) <= 2.5e-2 + slack, k
    dcb = divcurlB.astype(np.float64)
    assert F.checkvalf(dcb[:, 0], divB, 1.0e-3) <= 1.0e-3 + slack
    for k in range(3):
        assert F.checkvalf(dcb[:, 1 + k], curlB[:, k], 1.0e-3) <= 1.0e-3 + slack, k


def test_oracle_derivsmhd_analytic():
    from oracle import oracle as O
    O.build()
    cfg, x, v, B = _setup_mhd()
    o = O.Oracle(cfg, nthreads=8)
    o.set_particles(x, v, B)
    o.derivs(1, 0.0)
    xo, _, _ = o.get_particles()
    _check_mhd(cfg, x, xo, o.get_force(), o.get_density()["divcurlB"])


@pytest.mark.gpu
@pytest.mark.parametrize("mixed", [False, True])
def test_gpu_derivsmhd_analytic(mixed):
    from phantom_gb300 import capi
    cfg, x, v, B = _setup_mhd()
    ctx = capi.Context(cfg, precision=capi.PH_PREC_MIXED if mixed else capi.PH_PREC_FP64)
    ctx.upload(x, v, B)
    ctx.build_tree()
    d = ctx.densityiterate(1)
    fo = ctx.force(1)
    _check_mhd(cfg, x, d["xyzh"], fo, d["divcurlB"], slack=1.0e-5 if mixed else 0.0)
