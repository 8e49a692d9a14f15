"""Differentiation form: ph_adjoint against central finite differences of the
FP64 oracle (the reference's force on the reference's density solve).

The oracle runs with gradh kept in FP64 (f64_store; the reference's float32
storage of 1/Omega would put rounding steps into a 1e-6 difference quotient)
and tolh = 1e-8 (the converged h-rho solve that the adjoint differentiates).
Bar: |adjoint - FD| <= 1e-4 of the largest |FD| of the same variable group,
for the gradients with respect to x, v and u of
  * one derivs evaluation, L = sum w . a + s du/dt (artificial viscosity and
    conductivity on);
  * a 16-step leapfrog rollout with checkpoints every 4 steps, L = sum w . a_16,
    with the dissipation switches off: the viscosity term switches on at
    v_ij . r_ij = 0 and the conductivity signal speed is |P_i - P_j|^(1/2), so
    L is only piecewise smooth, and over 16 steps a 1e-6 perturbation reaches
    enough pairs that some cross a switch inside the difference interval
    (measured: 1e-3 scatter of the quotient between eps = 1e-5 and 1e-6,
    against 1e-8 agreement with the switches off).
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


def _setup(n1d=12):
    cfg, x, v, B = S.hydro_lattice(n1d)
    cfg = dict(cfg)
    cfg["tolh"] = 1.0e-8
    cfg["tolv"] = 1.0e3  # one velocity iteration per step (the reference's tolv > 1e2 branch)
    return cfg, x, v


def _oracle(cfg):
    c = dict(cfg)
    c["f64_store"] = 1
    return O.Oracle(c, nthreads=8)


def _check(name, adj, fd):
    scale = np.abs(fd).max()
    err = np.abs(adj - fd).max() / scale
    assert err <= TOL, (name, err, adj, fd)


def _check_screened(name, adj, fd, fd_coarse):
    """As _check, on the components where the difference quotient is locally
    smooth: the viscosity switch (v_ij . r_ij = 0) puts kinks into L, and a
    quotient whose interval holds one is not a derivative. Components whose
    quotients at eps and 10 eps disagree by more than the bar are set aside;
    at least three quarters must remain."""
    scale = np.abs(fd).max()
    smooth = np.abs(fd - fd_coarse) <= TOL * scale
    assert smooth.mean() >= 0.75, (name, smooth.mean())
    err = np.abs(adj[smooth] - fd[smooth]).max() / scale
    assert err <= TOL, (name, err)


@pytest.mark.parametrize("prec", [capi.PH_PREC_FP64, capi.PH_PREC_MIXED])
def test_adjoint_single_evaluation_matches_fd(prec):
    """The plain FP64 adjoint and the precision form's (FP32 pair terms on
    FP64 separations, Kahan sums) against the FP64 oracle's differences."""
    cfg, x, v = _setup()
    n = len(x)
    rng = np.random.default_rng(11)
    w4 = np.zeros((n, 4)); w4[:, :3] = rng.standard_normal((n, 3)); w4[:, 3] = rng.standard_normal(n)
    # FP32 density sums converge the h-rho solve to tolh = 1e-7 at best
    dev = capi.Context(dict(cfg, tolh=1.0e-7) if prec == capi.PH_PREC_MIXED else cfg, precision=prec)
    dev.upload(x, v)
    gx, gv = dev.adjoint(w4)
    o = _oracle(cfg)

    def L(xx, vv):
        o.set_particles(xx, vv)
        o.derivs(1, 0.0)
        return float(np.sum(w4 * o.get_force()["fxyzu"]))

    idx = rng.choice(n, size=24, replace=False)
    eps = 1.0e-6
    for group, arr, grad, comps in (("x", x, gx, range(3)), ("v", v, gv, range(3)), ("u", v, gv, [3])):
        fd, ad = [], []
        for i in idx:
            for c in comps:
                ap = arr.copy(); am = arr.copy()
                ap[i, c] += eps; am[i, c] -= eps
                if group == "x":
                    fd.append((L(ap, v) - L(am, v)) / (2 * eps))
                else:
                    fd.append((L(x, ap) - L(x, am)) / (2 * eps))
                ad.append(grad[i, c])
        _check(group, np.array(ad), np.array(fd))


def test_autograd_function_uses_the_adjoint():
    torch = pytest.importorskip("torch")
    from pyphantom_autograd import Derivs
    cfg, x, v = _setup(10)
    n = len(x)
    rng = np.random.default_rng(5)
    w = rng.standard_normal((n, 4)); w[:, 3] = 0.0
    dev = capi.Context(cfg)
    xt = torch.tensor(x, requires_grad=True)
    vt = torch.tensor(v, requires_grad=True)
    f = Derivs.apply(xt, vt, dev)
    (f * torch.from_numpy(w)).sum().backward()
    dev.upload(x, v)
    gx, gv = dev.adjoint(w)
    assert np.allclose(xt.grad.numpy(), gx, rtol=1e-12, atol=0.0)
    assert np.allclose(vt.grad.numpy(), gv, rtol=1e-12, atol=0.0)


def test_adjoint_rollout_with_checkpoints_matches_fd():
    from pyphantom_autograd import Rollout
    cfg, x, v = _setup(10)
    cfg.update(alpha=0.0, beta=0.0, alphau=0.0)
    n = len(x)
    rng = np.random.default_rng(7)
    w = rng.standard_normal((n, 3))
    dev = capi.Context(cfg)
    dev.upload(x, v)
    dt = 0.5 * dev.derivs(1, 0.0)
    K = 16
    ro = Rollout(dev, cfg, [dt] * K, ckpt=4)
    L, gx, gv = ro.loss_and_grad(x, v, w)
    o = _oracle(cfg)

    def Lo(xx, vv):
        o.set_particles(xx, vv)
        o.derivs(1, 0.0)
        t = 0.0
        for _ in range(K):
            o.step(t, dt)
            t += dt
        return float(np.sum(w * o.get_force()["fxyzu"][:, :3]))

    assert abs(Lo(x, v) / L - 1.0) < 1.0e-6  # the harness rollout is the reference's step sequence
    idx = rng.choice(n, size=6, replace=False)
    eps = 1.0e-6
    for group, arr, grad, comps in (("x", x, gx, range(3)), ("v", v, gv, range(3)), ("u", v, gv, [3])):
        fd, ad = [], []
        for i in idx:
            for c in comps:
                ap = arr.copy(); am = arr.copy()
                ap[i, c] += eps; am[i, c] -= eps
                if group == "x":
                    fd.append((Lo(ap, v) - Lo(am, v)) / (2 * eps))
                else:
                    fd.append((Lo(x, ap) - Lo(x, am)) / (2 * eps))
                ad.append(grad[i, c])
        _check("rollout " + group, np.array(ad), np.array(fd))


def test_adjoint_mhd_matches_fd():
    """Ideal MHD, accelerations: gradients with respect to x, v, u and B/rho
    (magnetic pressure and stress, v_A in the signal speed, the div B
    subtraction)."""
    cfg, x, v, B = S.mhd_vortex(8)
    cfg = dict(cfg)
    cfg["tolh"] = 1.0e-8
    n = len(x)
    rng = np.random.default_rng(13)
    w4 = np.zeros((n, 4)); w4[:, :3] = rng.standard_normal((n, 3))
    dev = capi.Context(cfg)
    dev.upload(x, v, B)
    gx, gv, gb = dev.adjoint(w4, with_B=True)
    o = _oracle(cfg)

    def L(xx, vv, bb):
        o.set_particles(xx, vv, bb)
        o.derivs(1, 0.0)
        return float(np.sum(w4 * o.get_force()["fxyzu"]))

    idx = rng.choice(n, size=16, replace=False)
    arrs = {"x": x, "v": v, "u": v, "B": B}

    def quotient(group, i, c, eps):
        ap = arrs[group].copy(); am = arrs[group].copy()
        ap[i, c] += eps; am[i, c] -= eps
        if group == "x":
            return (L(ap, v, B) - L(am, v, B)) / (2 * eps)
        if group == "B":
            return (L(x, v, ap) - L(x, v, am)) / (2 * eps)
        return (L(x, ap, B) - L(x, am, B)) / (2 * eps)

    for group, grad, comps in (("x", gx, range(3)), ("v", gv, range(3)), ("u", gv, [3]), ("B", gb, range(3))):
        fd, fdc, ad = [], [], []
        for i in idx:
            for c in comps:
                fd.append(quotient(group, i, c, 1.0e-6))
                fdc.append(quotient(group, i, c, 1.0e-5))
                ad.append(grad[i, c])
        _check_screened("mhd " + group, np.array(ad), np.array(fd), np.array(fdc))


@pytest.mark.parametrize("prec", [capi.PH_PREC_FP64, capi.PH_PREC_MIXED])
def test_adjoint_mhd_full_matches_fd(prec):
    """Ideal MHD with cotangents of every output of one derivs: the
    accelerations, du/dt with resistive heating on (the reference's default),
    d(B/rho)/dt and dpsi/dt (induction, artificial resistivity, psi cleaning,
    div B diffusion and decay: force.F90:1630-1671, 3107-3123), psi random and
    nonzero. Gradients with respect to x, v, u, B/rho and psi against
    screened central differences of the FP64 oracle (eps = 1e-6 against
    1e-5), in FP64 (measured about 1e-7 relative for each cotangent alone)
    and in the precision form."""
    cfg, x, v, B = S.mhd_vortex(8)
    cfg = dict(cfg, tolh=1.0e-8)
    n = len(x)
    rng = np.random.default_rng(29)
    B = B.copy()
    B[:, 3] = 0.05 * rng.standard_normal(n)
    w4 = rng.standard_normal((n, 4))
    wB = rng.standard_normal((n, 4))
    dev = capi.Context(dict(cfg, tolh=1.0e-7) if prec == capi.PH_PREC_MIXED else cfg, precision=prec)
    dev.upload(x, v, B)
    gx, gv, gb = dev.adjoint_full(w4, wB)
    o = _oracle(cfg)

    def L(xx, vv, bb):
        o.set_particles(xx, vv, bb)
        o.derivs(1, 0.0)
        f = o.get_force()
        return float(np.sum(w4 * f["fxyzu"]) + np.sum(wB * f["dBevol"]))

    idx = rng.choice(n, size=16, replace=False)
    arrs = {"x": x, "v": v, "u": v, "B": B, "psi": B}

    def quotient(group, i, c, eps):
        ap = arrs[group].copy(); am = arrs[group].copy()
        ap[i, c] += eps; am[i, c] -= eps
        if group == "x":
            return (L(ap, v, B) - L(am, v, B)) / (2 * eps)
        if group in ("B", "psi"):
            return (L(x, v, ap) - L(x, v, am)) / (2 * eps)
        return (L(x, ap, B) - L(x, am, B)) / (2 * eps)

    for group, grad, comps in (("x", gx, range(3)), ("v", gv, range(3)), ("u", gv, [3]), ("B", gb, range(3)),
                               ("psi", gb, [3])):
        fd, fdc, ad = [], [], []
        for i in idx:
            for c in comps:
                fd.append(quotient(group, i, c, 1.0e-6))
                fdc.append(quotient(group, i, c, 1.0e-5))
                ad.append(grad[i, c])
        _check_screened("mhd full " + group, np.array(ad), np.array(fd), np.array(fdc))


def test_adjoint_cullen_dehnen_matches_fd():
    """With the Cullen & Dehnen switch (nalpha = 3) the force uses alpha_i and
    alpha_j of alphaind(1,:), an input of one derivs: per-particle alpha set
    at random in [0, 1], gradients of L = sum w . a + s du/dt against the
    oracle's central differences with the same alpha."""
    cfg, x, v = _setup()
    cfg = dict(cfg, nalpha=3, alpha=0.0, alphamax=1.0)
    n = len(x)
    rng = np.random.default_rng(17)
    alpha = rng.uniform(0.0, 1.0, n).astype(np.float32)
    w4 = rng.standard_normal((n, 4))
    dev = capi.Context(cfg)
    dev.upload(x, v)
    dev.set_alpha(alpha)
    gx, gv = dev.adjoint(w4)
    o = _oracle(cfg)

    def L(xx, vv):
        o.set_particles(xx, vv)
        o.set_alpha(alpha)
        o.derivs(1, 0.0)
        return float(np.sum(w4 * o.get_force()["fxyzu"]))

    idx = rng.choice(n, size=16, replace=False)
    eps = 1.0e-6
    for group, arr, grad, comps in (("x", x, gx, range(3)), ("v", v, gv, range(3)), ("u", v, gv, [3])):
        fd, ad = [], []
        for i in idx:
            for c in comps:
                ap = arr.copy(); am = arr.copy()
                ap[i, c] += eps; am[i, c] -= eps
                if group == "x":
                    fd.append((L(ap, v) - L(am, v)) / (2 * eps))
                else:
                    fd.append((L(x, ap) - L(x, am)) / (2 * eps))
                ad.append(grad[i, c])
        _check("cd " + group, np.array(ad), np.array(fd))


def test_rollout_refuses_the_switch():
    from pyphantom_autograd import Rollout
    cfg, x, v = _setup(8)
    cfg = dict(cfg, nalpha=3, alpha=0.0)
    dev = capi.Context(cfg)
    with pytest.raises(NotImplementedError):
        Rollout(dev, cfg, [1.0e-3] * 4)


def _cloud(n, adiabatic=False):
    """The gravity cloud with random velocities added to its solid-body
    rotation: under pure rotation v_ij . r_ij vanishes (to rounding) for every
    pair, so every pair sits on the viscosity's switch, where a central
    difference averages the two one-sided slopes."""
    cfg, x, v, B = S.gravity_cloud(n)
    cfg = dict(cfg, tolh=1.0e-8)
    v = v.copy()
    v[:, :3] += 0.1 * np.random.default_rng(4).standard_normal((n, 3))
    if adiabatic:
        # the conductivity's signal speed is |v_ij . n| with self-gravity
        cfg.update(isothermal=0, ieos=2, gamma=5.0 / 3.0)
        v[:, 3] = 0.06 * (1.0 + 0.5 * np.random.default_rng(5).random(len(x)))
    return cfg, x, v


@pytest.mark.parametrize("adiabatic", [False, True])
@pytest.mark.parametrize("prec", [capi.PH_PREC_FP64, capi.PH_PREC_MIXED])
def test_adjoint_self_gravity_matches_fd(prec, adiabatic):
    """Self-gravity: the softened near field with its gradsoft term, the 1/r^2
    trial pairs outside both kernels and the far field (M2L sums of the node
    moments, their propagation and expansion), on a 2000-particle cloud
    (tree_accuracy 0.5: most of each particle's force comes from the far
    field). L = sum w . a (+ s du/dt adiabatic). Against central differences
    of the FP64 oracle at eps = 1e-6, screened against eps = 1e-5: a
    perturbation can move a particle across a node's split plane or flip a
    node pair between the near and far field, which puts a step into L."""
    cfg, x, v = _cloud(2000, adiabatic)
    n = len(x)
    rng = np.random.default_rng(17)
    w4 = np.zeros((n, 4)); w4[:, :3] = rng.standard_normal((n, 3))
    if adiabatic:
        w4[:, 3] = rng.standard_normal(n)
    dcfg = dict(cfg, tolh=1.0e-7) if prec == capi.PH_PREC_MIXED else cfg
    dev = capi.Context(dcfg, precision=prec)
    dev.upload(x, v)
    gx, gv = dev.adjoint(w4)
    o = _oracle(cfg)

    def L(xx, vv):
        o.set_particles(xx, vv)
        o.derivs(1, 0.0)
        return float(np.sum(w4 * o.get_force()["fxyzu"]))

    idx = rng.choice(n, size=24, replace=False)
    groups = [("x", x, gx, range(3)), ("v", v, gv, range(3))]
    if adiabatic:
        groups.append(("u", v, gv, [3]))
    for group, arr, grad, comps in groups:
        fd, fdc, ad = [], [], []
        for i in idx:
            for c in comps:
                q = []
                for eps in (1.0e-6, 1.0e-5):
                    ap = arr.copy(); am = arr.copy()
                    ap[i, c] += eps; am[i, c] -= eps
                    if group == "x":
                        q.append((L(ap, v) - L(am, v)) / (2 * eps))
                    else:
                        q.append((L(x, ap) - L(x, am)) / (2 * eps))
                fd.append(q[0]); fdc.append(q[1])
                ad.append(grad[i, c])
        _check_screened("grav " + group, np.array(ad), np.array(fd), np.array(fdc))


def test_adjoint_refuses_individual_timesteps():
    """With individual timesteps an evaluation re-computes the active
    particles' forces only (and walks the active cells only): ph_adjoint
    returns PH_ERR_NOT_BUILT rather than reading lists it did not build."""
    cfg, x, v, B = S.hydro_lattice(8)
    dev = capi.Context(dict(cfg, ind_timesteps=1, dtmax=1.0e-3))
    dev.upload(x, v, B)
    with pytest.raises(capi.PhantomError) as e:
        dev.adjoint(np.zeros((len(x), 4)))
    assert e.value.code == capi.PH_ERR_NOT_BUILT


def _fd_groups(L, arrs, grads, idx, eps=1.0e-6, coarse=1.0e-5):
    """Screened central differences of L(x, v, B) for the (group, arr key,
    component list) entries of grads."""
    x, v, B = arrs["x"], arrs["v"], arrs["B"]
    for group, key, grad, comps in grads:
        fd, fdc, ad = [], [], []
        for i in idx:
            for c in comps:
                q = []
                for e in (eps, coarse):
                    ap = arrs[key].copy(); am = arrs[key].copy()
                    ap[i, c] += e; am[i, c] -= e
                    args_p = {"x": (ap, v, B), "v": (x, ap, B), "B": (x, v, ap)}[key]
                    args_m = {"x": (am, v, B), "v": (x, am, B), "B": (x, v, am)}[key]
                    q.append((L(*args_p) - L(*args_m)) / (2 * e))
                fd.append(q[0]); fdc.append(q[1]); ad.append(grad[i, c])
        _check_screened(group, np.array(ad), np.array(fd), np.array(fdc))


def test_adjoint_mhd_self_gravity_matches_fd():
    """Ideal MHD and self-gravity together on a 1500-particle cloud
    (isothermal, B = 0.2 z plus a random part, psi random, random velocities
    on the rotation): cotangents of the accelerations, d(B/rho)/dt and
    dpsi/dt; gradients with respect to x, v, B/rho and psi against screened
    differences of the FP64 oracle."""
    cfg, x, v, B = S.gravity_cloud(1500)
    n = len(x)
    rng = np.random.default_rng(43)
    cfg = dict(cfg, tolh=1.0e-8, mhd=1)
    v = v.copy(); v[:, :3] += 0.1 * rng.standard_normal((n, 3))
    rho0 = 1.0 / (4.0 / 3.0 * np.pi)
    B = np.zeros((n, 4))
    B[:, 2] = 0.2 / rho0
    B[:, :3] += 0.05 / rho0 * rng.standard_normal((n, 3))
    B[:, 3] = 0.02 * rng.standard_normal(n)
    w4 = np.zeros((n, 4)); w4[:, :3] = rng.standard_normal((n, 3))
    wB = rng.standard_normal((n, 4))
    dev = capi.Context(cfg)
    dev.upload(x, v, B)
    gx, gv, gb = dev.adjoint_full(w4, wB)
    o = _oracle(cfg)

    def L(xx, vv, bb):
        o.set_particles(xx, vv, bb)
        o.derivs(1, 0.0)
        f = o.get_force()
        return float(np.sum(w4 * f["fxyzu"]) + np.sum(wB * f["dBevol"]))

    idx = rng.choice(n, size=12, replace=False)
    _fd_groups(L, {"x": x, "v": v, "B": B}, [("mhd+grav x", "x", gx, range(3)), ("mhd+grav v", "v", gv, range(3)),
                                           ("mhd+grav B", "B", gb, range(3)), ("mhd+grav psi", "B", gb, [3])], idx)


def test_adjoint_periodic_self_gravity_matches_fd():
    """Self-gravity in a periodic box (node separations and trial leaves take
    periodic images): 2000 random particles in [-0.5, 0.5)^3, adiabatic,
    random velocities; accelerations and du/dt weighted; gradients with
    respect to x, v and u against screened differences of the FP64 oracle."""
    cfg, x, v, B = S.random_box(2000, seed=5, gravity=True)
    cfg = dict(cfg, periodic=1, xmin=-0.5, xmax=0.5, ymin=-0.5, ymax=0.5, zmin=-0.5, zmax=0.5, tolh=1.0e-8)
    n = len(x)
    rng = np.random.default_rng(47)
    v = v.copy(); v[:, :3] = 0.3 * rng.standard_normal((n, 3))
    w4 = rng.standard_normal((n, 4))
    dev = capi.Context(cfg)
    dev.upload(x, v, B)
    gx, gv = dev.adjoint(w4)
    o = _oracle(cfg)

    def L(xx, vv, bb):
        o.set_particles(xx, vv, bb)
        o.derivs(1, 0.0)
        return float(np.sum(w4 * o.get_force()["fxyzu"]))

    idx = rng.choice(n, size=12, replace=False)
    _fd_groups(L, {"x": x, "v": v, "B": B}, [("periodic grav x", "x", gx, range(3)),
                                           ("periodic grav v", "v", gv, range(3)), ("periodic grav u", "v", gv, [3])],
               idx)


@pytest.mark.parametrize("prec", [capi.PH_PREC_FP64, capi.PH_PREC_MIXED])
@pytest.mark.parametrize("gravity", [False, True])
def test_adjoint_rectangular_periodic_box_matches_fd(prec, gravity):
    """The rectangular periodic box [0,1) x [0,0.5) x [0,0.25) (each axis its
    own periodic image; every particle within 2h of a z face): the hydro
    lattice of 24 x 12 x 6 particles, or 2000 random self-gravitating
    particles; accelerations and du/dt weighted; gradients with respect to x,
    v and u against screened differences of the FP64 oracle."""
    from test_gpu_parity_combos import rect_box
    if gravity:
        n = 2000
        rng0 = np.random.Generator(np.random.PCG64(19))
        L3 = np.array([1.0, 0.5, 0.25])
        x = np.empty((n, 4)); x[:, :3] = rng0.uniform(0.0, 1.0, size=(n, 3)) * L3
        x[:, 3] = 1.2 * (float(L3.prod()) / n) ** (1.0 / 3.0)
        v = np.zeros((n, 4)); v[:, 3] = 1.0
        B = np.zeros((n, 4))
        cfg = S.base_cfg(massoftype=1.0 / n, maxp=n, xmax=1.0, ymax=0.5, zmax=0.25, gravity=1)
    else:
        cfg, x, v, B = rect_box()
    n = len(x)
    rng = np.random.default_rng(53)
    v = v.copy(); v[:, :3] = 0.3 * rng.standard_normal((n, 3))
    cfg = dict(cfg, tolh=1.0e-8, tolv=1.0e3)
    w4 = rng.standard_normal((n, 4))
    dev = capi.Context(dict(cfg, tolh=1.0e-7) if prec == capi.PH_PREC_MIXED else cfg, precision=prec)
    dev.upload(x, v, B)
    gx, gv = dev.adjoint(w4)
    o = _oracle(cfg)

    def L(xx, vv, bb):
        o.set_particles(xx, vv, bb)
        o.derivs(1, 0.0)
        return float(np.sum(w4 * o.get_force()["fxyzu"]))

    idx = rng.choice(n, size=12, replace=False)
    _fd_groups(L, {"x": x, "v": v, "B": B}, [("rect x", "x", gx, range(3)), ("rect v", "v", gv, range(3)),
                                           ("rect u", "v", gv, [3])], idx)
