"""Individual timesteps (IND_TIMESTEPS) in the oracle.

* Known answer: the reference's Sedov test (src/tests/test_sedov.f90:88-193,
  its test build: individual timesteps, no CONST_AV, dtmax = tmax = 0.1)
  conserves total energy to the extracted tolerance and linear momentum to
  7e-15.
* When every particle sits in one bin the scheme is the global leapfrog
  with dt = dtmax / 2^nbinmax: the half kicks through twas (predictor
  twas - t, corrector dt then -(dt/2)) add to the global ones, so positions
  and velocities agree to rounding (1e-12).
* Invariants after every substep: bins within [0, nbinmax], the particles
  updated are those whose bin divides istepfrac, and time advances by
  dtmax / 2^nbinmax.
"""
import numpy as np
import pytest

from known_answers import KA
from oracle import oracle as O
from phantom_gb300 import setups as S


def _energy(o, m):
    xo, vo, _ = o.get_particles()
    return float(np.sum(0.5 * m * np.sum(vo[:, :3] ** 2, axis=1)) + np.sum(m * vo[:, 3])), vo


@pytest.mark.parametrize("nalpha", [3, 0])
def test_sedov_known_answer_individual_timesteps(nalpha):
    cfg, x, v, B = S.sedov_test(16)
    tmax = KA["sedov_tmax"]["value"]
    cfg = dict(cfg, ind_timesteps=1, dtmax=tmax, nalpha=nalpha, alpha=0.0 if nalpha else cfg["alpha"],
               alphamax=1.0)
    o = O.Oracle(cfg, nthreads=8)
    o.set_particles(x, v)
    o.derivs(1, 0.0)
    o.ind_init(0.0)
    m = cfg["massoftype"]
    e0, _ = _energy(o, m)
    t = 0.0
    while t < tmax * (1.0 - 1.0e-12):
        t, _ = o.ind_substep(t)
    e1, vo = _energy(o, m)
    assert abs(e1 / e0 - 1.0) <= KA["sedov_energy_tol"]["value"]
    assert np.abs(np.sum(m * vo[:, :3], axis=0)).max() <= KA["sedov_momentum_tol"]["value"]
    b, _, cnt = o.ind_state()
    assert len(np.unique(b)) > 1  # the blast spreads the particles over bins


def test_one_bin_is_the_global_leapfrog():
    cfg, x, v, B = S.hydro_lattice(10, vamp=0.01)
    cfg = dict(cfg, tolv=1.0e3, dtmax=2.0e-3)
    oi = O.Oracle(dict(cfg, ind_timesteps=1), nthreads=8)
    oi.set_particles(x, v)
    oi.derivs(1, 0.0)
    oi.ind_init(0.0)
    b, _, (nbinmax, _, _) = oi.ind_state()
    assert (b == nbinmax).all()
    dt = cfg["dtmax"] / 2 ** nbinmax
    og = O.Oracle(cfg, nthreads=8)
    og.set_particles(x, v)
    og.derivs(1, 0.0)
    t = 0.0
    for _ in range(4):
        t, na = oi.ind_substep(t)
        assert na == len(x)
        og.step(t - dt, dt)
        b, _, (nb, _, _) = oi.ind_state()
        if (b != nb).any() or nb != nbinmax:
            pytest.skip("bins changed during the comparison")
    xi, vi, _ = oi.get_particles()
    xg, vg, _ = og.get_particles()
    assert np.abs(xi[:, :3] - xg[:, :3]).max() < 1.0e-12
    assert np.abs(vi - vg).max() < 1.0e-12 * max(np.abs(vg).max(), 1.0)


def test_bin_invariants():
    cfg, x, v, B = S.sedov(12)
    cfg = dict(cfg, ind_timesteps=1, dtmax=0.02)
    o = O.Oracle(cfg, nthreads=8)
    o.set_particles(x, v)
    o.derivs(1, 0.0)
    o.ind_init(0.0)
    t = 0.0
    for _ in range(24):
        b0, _, (nbmax0, isf0, _) = o.ind_state()
        t_prev = t
        t, na = o.ind_substep(t)
        b, tw, (nbmax, isf, ibinnow) = o.ind_state()
        assert b.min() >= 0 and b.max() <= nbmax
        # the particles updated were those whose bin divided the step fraction
        want = int(np.sum((isf0 + 1) % (2 ** (nbmax0 - b0.astype(int))) == 0))
        assert na == want
        assert abs((t - t_prev) - cfg["dtmax"] / 2 ** nbmax0) <= 1e-12


def test_dt_too_small_stops_before_the_corrector():
    """dtmax = 2^34 x the particles' step: a bin above maxbins = 30; the
    substep stops with status 42 after derivs, before the corrector
    (step_leapfrog.f90:427-433)."""
    cfg, x, v, B = S.sedov(8)
    o0 = O.Oracle(cfg, nthreads=4)
    o0.set_particles(x, v)
    dt = o0.derivs(1, 0.0)
    cfg = dict(cfg, ind_timesteps=1, dtmax=dt * 2.0 ** 34)
    o = O.Oracle(cfg, nthreads=4)
    o.set_particles(x, v)
    o.derivs(1, 0.0)
    o.ind_init(0.0)
    with pytest.raises(RuntimeError, match="status 42"):
        o.ind_substep(0.0)
