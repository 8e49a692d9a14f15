"""Cullen & Dehnen viscosity switch in the oracle (nalpha = 3, the
reference's default build without CONST_AV).

Known answers: the exact-linear gradient estimate (dens.F90:866-1101)
reproduces a linear velocity field v = A x exactly, so dvdx = A to float
storage and, with zero accelerations, d(div v)/dt = -tr(A A) exactly;
alphaloc follows shock_capturing.f90:131-177 from those stored values; one
leapfrog step evolves alpha as step_leapfrog.f90:378-391 (alpha jumps up to
alphaloc, else decays at 0.1 c_s / h implicitly).
"""
import numpy as np

from oracle import oracle as O
from phantom_gb300 import setups as S

A = np.array([[0.3, -0.2, 0.1], [0.05, -0.4, 0.2], [0.1, 0.15, -0.25]])


def _linear(n=3000, seed=4):
    cfg, x, v, B = S.random_box(n, seed=seed)
    cfg = dict(cfg, nalpha=3, alpha=0.0, alphamax=1.0, tolh=1.0e-6)
    v = v.copy()
    v[:, :3] = x[:, :3] @ A.T
    return cfg, x, v


def test_linear_field_gradients_exact():
    cfg, x, v = _linear()
    o = O.Oracle(cfg, nthreads=4)
    o.set_particles(x, v)
    o.maketree()
    o.densityiterate(1)
    a, d = o.get_alpha()
    assert np.abs(d - A.reshape(1, 9)).max() <= 2.0 ** -24 * np.abs(A).max() * 2
    assert np.abs(a[:, 2] + np.trace(A @ A)).max() <= 2.0 ** -23 * abs(np.trace(A @ A))


def test_alphaloc_formula():
    cfg, x, v = _linear()
    o = O.Oracle(cfg, nthreads=4)
    o.set_particles(x, v)
    o.derivs(1, 0.0)
    a, d = o.get_alpha()
    xo, _, _ = o.get_particles()
    dv = d.astype(np.float64)
    divv = dv[:, 0] + dv[:, 4] + dv[:, 8]
    curl2 = (dv[:, 7] - dv[:, 5]) ** 2 + (dv[:, 2] - dv[:, 6]) ** 2 + (dv[:, 3] - dv[:, 1]) ** 2
    fac = np.maximum(-divv, 0.0) ** 2
    xi = np.where(fac + curl2 > 2.22e-16, fac / (fac + curl2), 1.0)
    cs = np.sqrt(cfg["gamma"] * (cfg["gamma"] - 1.0) * v[:, 3])
    src = 10.0 * xo[:, 3] ** 2 * xi * np.maximum(-a[:, 2].astype(np.float64), 0.0)
    want = np.clip(src / cs ** 2, cfg["alpha"], cfg["alphamax"])
    assert np.allclose(a[:, 1], want.astype(np.float32), rtol=2e-7, atol=0.0)
    assert (a[:, 1] > 0).any()


def test_step_evolves_alpha():
    cfg, x, v = _linear(2000)
    o = O.Oracle(cfg, nthreads=4)
    o.set_particles(x, v)
    rng = np.random.default_rng(2)
    o.set_alpha(rng.uniform(0.0, 0.05, len(x)).astype(np.float32))
    dt = o.derivs(1, 0.0)
    a0, _ = o.get_alpha()
    xo0, _, _ = o.get_particles()
    o.step(0.0, dt)
    a1, _ = o.get_alpha()
    xo1, _, _ = o.get_particles()  # h here is the density's h after the step
    # the update uses the predicted h, which is not returned: check the two branches
    up = a0[:, 0] < a0[:, 1]
    assert np.array_equal(a1[up, 0], a0[up, 1])
    dn = ~up
    assert (a1[dn, 0] <= a0[dn, 0]).all() and (a1[dn, 0] >= a0[dn, 1] - 1e-7).all()


def test_constant_alpha_build_unchanged():
    """nalpha = 0 (CONST_AV): alphaind is not touched and the forces use alpha."""
    cfg, x, v = _linear(1500)
    c0 = dict(cfg, nalpha=0, alpha=1.0)
    o = O.Oracle(c0, nthreads=4)
    o.set_particles(x, v)
    o.derivs(1, 0.0)
    a, d = o.get_alpha()
    assert not a.any() and not d.any()
