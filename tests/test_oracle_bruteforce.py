"""The oracle's density and pressure force against a brute-force numpy
restatement over all particle pairs (no tree, no trial lists, no position
cache): a check of the oracle's neighbour finding, periodic images and pair
sums that shares none of its code.

* density: at the oracle's converged h (tolh = 1e-8), rho_sum(h_i) =
  m cnormk h_i^-3 sum_j w(|r_ij| / h_i) (self included) equals
  rhoh(h_i) = m (hfact / h_i)^3 to 1e-7 (dens.F90:1486-1500, part.F90:779-817),
  and 1/Omega_i = 1 / (1 + h_i / (3 rho_i) d rho_sum / dh) matches the
  oracle's gradh to float32 storage (1e-6);
* force with the dissipation off (alpha = beta = alpha_u = 0): a_i =
  -sum_j m (P_i rho_i^-2 Omega_i^-1 grad W_ij(h_i) + P_j rho_j^-2 Omega_j^-1
  grad W_ij(h_j)) over pairs with q_i < 2 or q_j < 2, and du/dt_i =
  P_i rho_i^-2 sum_j m v_ij . grad W_ij(h_i) Omega_i^-1 (force.F90:1428-1741,
  2773-2900), with the oracle's float32 gradh, to 1e-12 of the largest
  value, and with artificial viscosity and conductivity on;
* self-gravity with no node well separated (tree_accuracy = 0): the softened
  near field over all pairs, to 1e-12.
Sets: a periodic jittered lattice of 8^3 with random velocities, and 600
random particles in open boundaries, both with u from 1 to 1.5.
"""
import numpy as np
import pytest

from oracle import oracle as O
from phantom_gb300 import setups as S

CNORMK = 1.0 / 3.1415926536  # kernel_cubic.f90:25 with the reference's pi (physcon.f90:23)


@pytest.fixture(scope="module", autouse=True)
def _build():
    O.build()


def w_kern(q):
    return np.where(q < 1.0, 1.0 - 1.5 * q * q + 0.75 * q ** 3, np.where(q < 2.0, 0.25 * (2.0 - q) ** 3, 0.0))


def dw_kern(q):
    return np.where(q < 1.0, q * (2.25 * q - 3.0), np.where(q < 2.0, -0.75 * (2.0 - q) ** 2, 0.0))


def _sets():
    # u varies between particles, so that the conductivity term is not zero
    cfg, x, v, B = S.hydro_lattice(8)
    rng = np.random.default_rng(31)
    v = v.copy(); v[:, 3] = 1.0 + 0.5 * rng.random(len(x))
    yield "lattice8", dict(cfg, tolh=1.0e-8, alpha=0.0, beta=0.0, alphau=0.0), x, v
    cfg, x, v, B = S.random_box(600, seed=23)
    rng = np.random.default_rng(29)
    v = v.copy(); v[:, :3] = 0.1 * rng.standard_normal((len(x), 3)); v[:, 3] = 1.0 + 0.5 * rng.random(len(x))
    yield "random600", dict(cfg, tolh=1.0e-8, alpha=0.0, beta=0.0, alphau=0.0), x, v


def _separations(cfg, x):
    d = x[:, None, :3] - x[None, :, :3]
    if cfg["periodic"]:
        L = np.array([cfg["xmax"] - cfg["xmin"], cfg["ymax"] - cfg["ymin"], cfg["zmax"] - cfg["zmin"]])
        d -= L * np.round(d / L)
    return d


@pytest.mark.parametrize("name,cfg,x,v", list(_sets()), ids=lambda a: a if isinstance(a, str) else "")
def test_density_and_pressure_force_against_all_pairs(name, cfg, x, v):
    o = O.Oracle(cfg, nthreads=4)
    o.set_particles(x, v)
    o.derivs(1, 0.0)
    xo, vo, _ = o.get_particles()
    gradh = o.get_density()["gradh"][:, 0].astype(np.float64)
    f = o.get_force()["fxyzu"]
    m, hfact, gamma = cfg["massoftype"], cfg["hfact"], cfg["gamma"]
    h = xo[:, 3]
    d = _separations(cfg, xo)
    r = np.sqrt((d * d).sum(axis=2))
    qi = r / h[:, None]
    # density and Omega at the converged h
    rho_sum = m * CNORMK / h ** 3 * w_kern(qi).sum(axis=1)
    rhoh = m * (hfact / h) ** 3
    assert np.abs(rho_sum / rhoh - 1.0).max() < 1.0e-7
    drhodh = m * CNORMK / h ** 4 * (-3.0 * w_kern(qi) - qi * dw_kern(qi)).sum(axis=1)
    omega = 1.0 + h / (3.0 * rhoh) * drhodh
    assert np.abs(gradh * omega - 1.0).max() < 1.0e-6
    # pressure force and pdV du/dt with the oracle's float32 gradh
    rho = rhoh
    P = (gamma - 1.0) * rho * vo[:, 3]
    pro2 = P / rho ** 2
    qj = r / h[None, :]
    with np.errstate(invalid="ignore", divide="ignore"):
        rhat = np.where(r[..., None] > 0.0, d / r[..., None], 0.0)
    gi = CNORMK / h[:, None] ** 4 * dw_kern(qi) * gradh[:, None]
    gj = CNORMK / h[None, :] ** 4 * dw_kern(qj) * gradh[None, :]
    pair = ((qi < 2.0) | (qj < 2.0)) & (r > 0.0)
    coef = np.where(pair, m * (pro2[:, None] * gi + pro2[None, :] * gj), 0.0)
    a = -(coef[..., None] * rhat).sum(axis=1)
    dv = vo[:, None, :3] - vo[None, :, :3]
    projv = (dv * rhat).sum(axis=2)
    dudt = pro2 * m * np.where(pair, projv * gi, 0.0).sum(axis=1)
    scale = np.abs(a).max()
    assert np.abs(f[:, :3] - a).max() <= 1.0e-12 * scale, name
    assert np.abs(f[:, 3] - dudt).max() <= 1.0e-12 * np.abs(dudt).max(), name


@pytest.mark.parametrize("name,cfg,x,v", list(_sets()), ids=lambda a: a if isinstance(a, str) else "")
def test_force_with_dissipation_against_all_pairs(name, cfg, x, v):
    """As above with artificial viscosity and conductivity on (alpha = 1,
    beta = 2, alpha_u = 1; force.F90:1478-1560, 1690-1741): per pair
    projv = v_ij . r_hat; for projv < 0 q_a = -rho_a^-1 vsig_a projv / 2 with
    vsig_a = max(alpha c_a - beta projv, 0); the pressure terms take
    P_a rho_a^-2 + q_a; du/dt adds the shock heating m q_i projv grad W_i and
    the conductivity vsig_u (u_i - u_j) (m alpha_u / (2 rho_i) grad W_i +
    m alpha_u / (2 rho_j) grad W_j), vsig_u = (2 |P_i - P_j| / (rho_i +
    rho_j))^(1/2)."""
    cfg = dict(cfg, alpha=1.0, beta=2.0, alphau=1.0)
    o = O.Oracle(cfg, nthreads=4)
    o.set_particles(x, v)
    o.derivs(1, 0.0)
    xo, vo, _ = o.get_particles()
    gradh = o.get_density()["gradh"][:, 0].astype(np.float64)
    f = o.get_force()["fxyzu"]
    m, hfact, gamma = cfg["massoftype"], cfg["hfact"], cfg["gamma"]
    h = xo[:, 3]
    d = _separations(cfg, xo)
    r = np.sqrt((d * d).sum(axis=2))
    qi, qj = r / h[:, None], r / h[None, :]
    rho = m * (hfact / h) ** 3
    u = vo[:, 3]
    P = (gamma - 1.0) * rho * u
    cs = np.sqrt(gamma * (gamma - 1.0) * u)
    pro2 = P / rho ** 2
    with np.errstate(invalid="ignore", divide="ignore"):
        rhat = np.where(r[..., None] > 0.0, d / r[..., None], 0.0)
    gi = CNORMK / h[:, None] ** 4 * dw_kern(qi) * gradh[:, None]
    gj = CNORMK / h[None, :] ** 4 * dw_kern(qj) * gradh[None, :]
    pair = ((qi < 2.0) | (qj < 2.0)) & (r > 0.0)
    projv = ((vo[:, None, :3] - vo[None, :, :3]) * rhat).sum(axis=2)
    vsi = np.maximum(cfg["alpha"] * cs[:, None] - cfg["beta"] * projv, 0.0)
    vsj = np.maximum(cfg["alpha"] * cs[None, :] - cfg["beta"] * projv, 0.0)
    neg = projv < 0.0
    qri = np.where(neg, -0.5 / rho[:, None] * vsi * projv, 0.0)
    qrj = np.where(neg, -0.5 / rho[None, :] * vsj * projv, 0.0)
    coef = np.where(pair, m * ((pro2[:, None] + qri) * gi + (pro2[None, :] + qrj) * gj), 0.0)
    a = -(coef[..., None] * rhat).sum(axis=1)
    pdv = pro2 * m * np.where(pair, projv * gi, 0.0).sum(axis=1)
    shock = np.where(pair, m * qri * projv * gi, 0.0).sum(axis=1)
    vsu = np.sqrt(np.abs(P[:, None] - P[None, :]) * 2.0 / (rho[:, None] + rho[None, :]))
    au = 0.5 * m * cfg["alphau"] / rho
    cond = np.where(pair, vsu * (u[:, None] - u[None, :]) * (au[:, None] * gi + au[None, :] * gj), 0.0).sum(axis=1)
    dudt = pdv + shock + cond
    assert np.abs(f[:, :3] - a).max() <= 1.0e-12 * np.abs(a).max(), name
    assert np.abs(f[:, 3] - dudt).max() <= 1.0e-12 * np.abs(dudt).max(), name


def fsoft_kern(q):
    q2 = q * q
    q4 = q2 * q2
    inner = q * (15.0 * q2 * q - 36.0 * q2 + 40.0) / 30.0
    with np.errstate(divide="ignore", invalid="ignore"):
        outer = (-5.0 * q4 * q2 + 36.0 * q4 * q - 90.0 * q4 + 80.0 * q2 * q - 2.0) / (30.0 * q2)
        far = 1.0 / q2
    return np.where(q < 1.0, inner, np.where(q < 2.0, outer, far))


def test_self_gravity_near_field_against_all_pairs():
    """Self-gravity with tree_accuracy = 0 (no node is well separated, so
    every pair is a near-field pair, kdtree.F90:1398-1420) against the direct
    sum: per pair m (f_i + f_j) / 2 along r_hat with f_a = fsoft(q_a) h_a^-2 +
    gradsoft_a grad W_a inside a's kernel and 1/r^2 outside (kernel_cubic.f90
    kernel_softening, force.F90:1303-1340, 1991-2053), with the oracle's
    float32 gradsoft and 1/Omega; pressure and dissipation off (isothermal,
    polyk = 0, alpha = beta = 0). 500 random particles in open boundaries;
    accelerations to 1e-12 of their maximum."""
    cfg, x, v, B = S.random_box(500, seed=37, gravity=True)
    cfg = dict(cfg, tolh=1.0e-8, tree_accuracy=0.0, isothermal=1, ieos=1, polyk=0.0, alpha=0.0, beta=0.0,
               alphau=0.0)
    rng = np.random.default_rng(41)
    v = v.copy(); v[:, :3] = 0.1 * rng.standard_normal((len(x), 3))
    o = O.Oracle(cfg, nthreads=4)
    o.set_particles(x, v)
    o.derivs(1, 0.0)
    xo, _, _ = o.get_particles()
    gh = o.get_density()["gradh"].astype(np.float64)
    f = o.get_force()["fxyzu"]
    m, h = cfg["massoftype"], xo[:, 3]
    d = _separations(cfg, xo)
    r = np.sqrt((d * d).sum(axis=2))
    qi, qj = r / h[:, None], r / h[None, :]
    with np.errstate(invalid="ignore", divide="ignore"):
        rhat = np.where(r[..., None] > 0.0, d / r[..., None], 0.0)
        inv_r2 = np.where(r > 0.0, 1.0 / (r * r), 0.0)
    gki = CNORMK / h[:, None] ** 4 * dw_kern(qi) * gh[:, 0][:, None]
    gkj = CNORMK / h[None, :] ** 4 * dw_kern(qj) * gh[:, 0][None, :]
    fi = np.where(qi < 2.0, fsoft_kern(qi) / h[:, None] ** 2 + gh[:, 1][:, None] * gki, inv_r2)
    fj = np.where(qj < 2.0, fsoft_kern(qj) / h[None, :] ** 2 + gh[:, 1][None, :] * gkj, inv_r2)
    off = r > 0.0
    a = -(np.where(off, 0.5 * m * (fi + fj), 0.0)[..., None] * rhat).sum(axis=1)
    assert np.abs(f[:, :3] - a).max() <= 1.0e-12 * np.abs(a).max()
