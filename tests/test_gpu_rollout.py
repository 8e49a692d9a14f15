"""ph_rollout_adjoint: the adjoint through a checkpointed leapfrog rollout,
resident on the device, through the C ABI.

* The same rollout driven from the host (tests/pyphantom_autograd.py: numpy
  kicks and drifts, one ph_adjoint per force evaluation) gives the same loss
  and gradients (the device step predicts h before the h-rho solve, the host
  one starts from the last h; both converge to tolh = 1e-8).
* The reference's step sequence: the loss equals the oracle's rollout of the
  same steps (step_leapfrog.f90 with one corrector pass) to 1e-9.
* Against central finite differences of the FP64 oracle, for the benchmark's
  adjoint configuration at a test size: the hydro lattice with the
  reference's dissipation on (alpha = 1, beta = 2, alpha_u = 1), 16 steps,
  checkpoints every 4 steps, L = sum w . a_16 with w ~ N(0,1), gradients with
  respect to x, v and u of 64 random particles. With viscosity and
  conductivity on, L is only piecewise smooth (the viscosity switches on at
  v_ij . r_ij = 0, the conductivity signal speed is |P_i - P_j|^(1/2)), and
  over 16 steps a perturbation reaches many pairs: a difference quotient
  whose interval holds such a kink is not a derivative. The quotients are
  taken at eps = 1e-7; those that disagree with the quotient at 1e-6 by more
  than the bar are set aside (at least three quarters must remain), and the
  rest must agree with the adjoint to 1e-4 of the largest quotient (measured
  1.4e-5; with eps = 1e-6 screened against 1e-5 it is 2.0e-4, the 1e-6
  quotients of several components being moved by kinks while their 1e-7
  quotients agree with the adjoint to 1e-7 relative). The precision form's rollout
  (FP32 pair terms in the forward and in the adjoint) meets the same bar
  against the same FP64 quotients.
"""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))

from oracle import oracle as O
from phantom_gb300 import capi
from phantom_gb300 import setups as S

pytestmark = pytest.mark.gpu

TOL = 1.0e-4


def _setup(n1d):
    cfg, x, v, B = S.hydro_lattice(n1d)
    cfg = dict(cfg, tolh=1.0e-8, tolv=1.0e3)
    return cfg, x, v


def test_rollout_matches_host_harness_and_oracle():
    from pyphantom_autograd import Rollout
    cfg, x, v = _setup(10)
    n = len(x)
    rng = np.random.default_rng(3)
    w = np.zeros((n, 4)); w[:, :3] = rng.standard_normal((n, 3)); w[:, 3] = rng.standard_normal(n)
    dev = capi.Context(cfg)
    dev.upload(x, v)
    dt = 0.5 * dev.derivs(1, 0.0)
    K = 8
    dev.upload(x, v)
    L, gx, gv = dev.rollout_adjoint([dt] * K, w, ckpt=3)
    tm = dev.timings()
    assert tm[0] > 0.0 and tm[1] > 0.0 and tm[7] >= tm[0]
    ro = Rollout(dev, cfg, [dt] * K, ckpt=4)
    Lh, gxh, gvh = ro.loss_and_grad(x, v, w[:, :3])
    # the host harness weights the accelerations only: compare that part
    dev.upload(x, v)
    w3 = w.copy(); w3[:, 3] = 0.0
    L3, gx3, gv3 = dev.rollout_adjoint([dt] * K, w3, ckpt=4)
    assert abs(L3 / Lh - 1.0) < 1.0e-7
    assert np.abs(gx3 - gxh).max() <= 1.0e-6 * np.abs(gxh).max()
    assert np.abs(gv3 - gvh).max() <= 1.0e-6 * np.abs(gvh).max()
    # the checkpoint spacing does not change the result
    dev.upload(x, v)
    L3b, gx3b, gv3b = dev.rollout_adjoint([dt] * K, w3, ckpt=1)
    assert L3b == L3 and np.array_equal(gx3b, gx3) and np.array_equal(gv3b, gv3)
    # the loss is the oracle's rollout (with the reference's float32 gradh)
    o = O.Oracle(cfg, nthreads=8)
    o.set_particles(x, v)
    o.derivs(1, 0.0)
    t = 0.0
    for _ in range(K):
        o.step(t, dt)
        t += dt
    Lo = float(np.sum(w * o.get_force()["fxyzu"]))
    assert abs(L / Lo - 1.0) < 1.0e-9


def test_rollout_adjoint_matches_fd_with_dissipation():
    cfg, x, v = _setup(10)
    n = len(x)
    rng = np.random.default_rng(2024)
    w = np.zeros((n, 4)); w[:, :3] = rng.standard_normal((n, 3))
    dev = capi.Context(cfg)
    dev.upload(x, v)
    dt = 0.5 * dev.derivs(1, 0.0)
    K = 16
    dev.upload(x, v)
    L, gx, gv = dev.rollout_adjoint([dt] * K, w, ckpt=4)
    # the precision form's rollout and adjoint, against the same FP64 quotients
    # (FP32 density sums converge the h-rho solve to tolh = 1e-7 at best)
    dm = capi.Context(dict(cfg, tolh=1.0e-7), precision=capi.PH_PREC_MIXED)
    dm.upload(x, v)
    Lm, gxm, gvm = dm.rollout_adjoint([dt] * K, w, ckpt=4)
    assert abs(Lm / L - 1.0) < 1.0e-5
    o = O.Oracle(dict(cfg, f64_store=1), nthreads=os.cpu_count() or 1)

    def Lo(xx, vv):
        o.set_particles(xx, vv)
        o.derivs(1, 0.0)
        t = 0.0
        for _ in range(K):
            o.step(t, dt)
            t += dt
        return float(np.sum(w * o.get_force()["fxyzu"]))

    # the finite differences use the oracle with 1/Omega kept in FP64 (its
    # float32 storage would put rounding steps into a 1e-6 quotient), which
    # moves L by ~1e-7
    assert abs(Lo(x, v) / L - 1.0) < 1.0e-6
    idx = rng.choice(n, size=64, replace=False)

    def quotient(group, i, c, eps):
        if group == "x":
            ap = x.copy(); am = x.copy()
            ap[i, c] += eps; am[i, c] -= eps
            return (Lo(ap, v) - Lo(am, v)) / (2 * eps)
        ap = v.copy(); am = v.copy()
        ap[i, c] += eps; am[i, c] -= eps
        return (Lo(x, ap) - Lo(x, am)) / (2 * eps)

    for group, grads, comps in (("x", (gx, gxm), range(3)), ("v", (gv, gvm), range(3)), ("u", (gv, gvm), [3])):
        fd, fdc, ad, adm = [], [], [], []
        for i in idx:
            for c in comps:
                fd.append(quotient(group, i, c, 1.0e-7))
                fdc.append(quotient(group, i, c, 1.0e-6))
                ad.append(grads[0][i, c])
                adm.append(grads[1][i, c])
        fd, fdc, ad, adm = np.array(fd), np.array(fdc), np.array(ad), np.array(adm)
        scale = np.abs(fd).max()
        smooth = np.abs(fd - fdc) <= TOL * scale
        assert smooth.mean() >= 0.75, (group, smooth.mean())
        err = np.abs(ad[smooth] - fd[smooth]).max() / scale
        assert err <= TOL, (group, err)
        errm = np.abs(adm[smooth] - fd[smooth]).max() / scale
        assert errm <= TOL, ("mixed " + group, errm)


def test_rollout_refuses_unbuilt_physics():
    cfg, x, v, B = S.hydro_lattice(6)
    dev = capi.Context(dict(cfg, nalpha=3))
    dev.upload(x, v)
    with pytest.raises(capi.PhantomError) as e:
        dev.rollout_adjoint([1.0e-4] * 2, np.zeros((len(x), dev.vrows)))
    assert e.value.code == capi.PH_ERR_NOT_BUILT


def test_rollout_adjoint_mhd_matches_fd():
    """An MHD rollout (ph_rollout_adjoint_full): the 8^3 Orszag-Tang set with
    psi random and nonzero, dissipation and resistive heating on, 6 steps,
    checkpoints every 3, L = sum w . f_6 + sum wB . dBevol_6. The loss equals
    the oracle's rollout to 1e-6 and the gradients with respect to x, v, u,
    B/rho and psi of 12 particles match central differences of the FP64
    oracle at eps = 1e-7, screened against 1e-6."""
    cfg, x, v, B = S.mhd_vortex(8)
    cfg = dict(cfg, tolh=1.0e-8, tolv=1.0e3)
    n = len(x)
    rng = np.random.default_rng(37)
    B = B.copy()
    B[:, 3] = 0.05 * rng.standard_normal(n)
    w = rng.standard_normal((n, 4))
    wB = rng.standard_normal((n, 4))
    dev = capi.Context(cfg)
    dev.upload(x, v, B)
    dt = 0.5 * dev.derivs(1, 0.0)
    K = 6
    dev.upload(x, v, B)
    L, gx, gv, gb = dev.rollout_adjoint_full([dt] * K, w, wB, ckpt=3)
    # the checkpoint spacing does not change the result
    dev.upload(x, v, B)
    L1, gx1, gv1, gb1 = dev.rollout_adjoint_full([dt] * K, w, wB, ckpt=1)
    assert L1 == L and np.array_equal(gx1, gx) and np.array_equal(gv1, gv) and np.array_equal(gb1, gb)
    o = O.Oracle(dict(cfg, f64_store=1), nthreads=os.cpu_count() or 1)

    def Lo(xx, vv, bb):
        o.set_particles(xx, vv, bb)
        o.derivs(1, 0.0)
        t = 0.0
        for _ in range(K):
            o.step(t, dt)
            t += dt
        f = o.get_force()
        return float(np.sum(w * f["fxyzu"]) + np.sum(wB * f["dBevol"]))

    assert abs(Lo(x, v, B) / L - 1.0) < 1.0e-6
    idx = rng.choice(n, size=12, replace=False)
    arrs = {"x": x, "v": v, "u": v, "B": B, "psi": B}

    def quotient(group, i, c, eps):
        ap = arrs[group].copy(); am = arrs[group].copy()
        ap[i, c] += eps; am[i, c] -= eps
        if group == "x":
            return (Lo(ap, v, B) - Lo(am, v, B)) / (2 * eps)
        if group in ("B", "psi"):
            return (Lo(x, v, ap) - Lo(x, v, am)) / (2 * eps)
        return (Lo(x, ap, B) - Lo(x, am, B)) / (2 * eps)

    for group, grad, comps in (("x", gx, range(3)), ("v", gv, range(3)), ("u", gv, [3]), ("B", gb, range(3)),
                               ("psi", gb, [3])):
        fd, fdc, ad = [], [], []
        for i in idx:
            for c in comps:
                fd.append(quotient(group, i, c, 1.0e-7))
                fdc.append(quotient(group, i, c, 1.0e-6))
                ad.append(grad[i, c])
        fd, fdc, ad = np.array(fd), np.array(fdc), np.array(ad)
        scale = np.abs(fd).max()
        smooth = np.abs(fd - fdc) <= TOL * scale
        assert smooth.mean() >= 0.75, (group, smooth.mean())
        err = np.abs(ad[smooth] - fd[smooth]).max() / scale
        assert err <= TOL, (group, err)


def test_rollout_adjoint_self_gravity_matches_fd():
    """A self-gravitating rollout: the 1500-particle cloud (isothermal,
    viscosity on, tree_accuracy 0.5, random velocities added), 8 steps, checkpoints every 4,
    L = sum w . a_8. The loss equals the oracle's rollout (gradh and gradsoft
    in FP64) to 1e-6 and the gradients with respect to x and v of 16
    particles match central differences of the FP64 oracle at eps = 1e-7,
    screened against 1e-6 as for the hydro rollout (viscosity kinks; with a
    tree rebuilt every step a perturbation can also move a particle across a
    split plane or a node pair between the near and far field)."""
    cfg, x, v, B = S.gravity_cloud(1500)
    cfg = dict(cfg, tolh=1.0e-8, tolv=1.0e3)
    # random velocities on top of the rotation (under pure rotation every
    # pair sits on the viscosity's switch, v_ij . r_ij = 0)
    v = v.copy()
    v[:, :3] += 0.1 * np.random.default_rng(4).standard_normal((len(x), 3))
    n = len(x)
    rng = np.random.default_rng(31)
    dev = capi.Context(cfg)
    w = np.zeros((n, dev.vrows)); w[:, :3] = rng.standard_normal((n, 3))
    dev.upload(x, v)
    dt = 0.5 * dev.derivs(1, 0.0)
    K = 8
    dev.upload(x, v)
    L, gx, gv = dev.rollout_adjoint([dt] * K, w, ckpt=4)
    # the checkpoint spacing does not change the result
    dev.upload(x, v)
    L1, gx1, gv1 = dev.rollout_adjoint([dt] * K, w, ckpt=1)
    assert L1 == L and np.array_equal(gx1, gx) and np.array_equal(gv1, gv)
    o = O.Oracle(dict(cfg, f64_store=1), nthreads=os.cpu_count() or 1)

    def Lo(xx, vv):
        o.set_particles(xx, vv)
        o.derivs(1, 0.0)
        t = 0.0
        for _ in range(K):
            o.step(t, dt)
            t += dt
        return float(np.sum(w[:, :3] * o.get_force()["fxyzu"][:, :3]))

    assert abs(Lo(x, v) / L - 1.0) < 1.0e-6
    idx = rng.choice(n, size=16, replace=False)
    for group, arr, grad in (("x", x, gx), ("v", v, gv)):
        fd, fdc, ad = [], [], []
        for i in idx:
            for c in range(3):
                q = []
                for eps in (1.0e-7, 1.0e-6):
                    ap = arr.copy(); am = arr.copy()
                    ap[i, c] += eps; am[i, c] -= eps
                    if group == "x":
                        q.append((Lo(ap, v) - Lo(am, v)) / (2 * eps))
                    else:
                        q.append((Lo(x, ap) - Lo(x, am)) / (2 * eps))
                fd.append(q[0]); fdc.append(q[1])
                ad.append(grad[i, c])
        fd, fdc, ad = np.array(fd), np.array(fdc), np.array(ad)
        scale = np.abs(fd).max()
        smooth = np.abs(fd - fdc) <= TOL * scale
        assert smooth.mean() >= 0.75, (group, smooth.mean())
        err = np.abs(ad[smooth] - fd[smooth]).max() / scale
        assert err <= TOL, (group, err)
