"""Seeded synthetic particle sets for the benchmark and parity workloads.

Each builder returns ``(cfg, xyzh, vxyzu, Bevol)`` with the arrays in the
reference layout (``xyzh(4,N)`` etc. stored row-per-particle, float64) and a
``cfg`` dict of the run-time switches that the C-ABI ``ph_params`` and the
oracle take.

Lattices follow ``set_unifdis('cubic')`` (src/setup/set_unifdis.f90:182-200):
particle (i,j,k) sits at ``xmin + (i-0.5)*dx`` with x varying fastest. The
Sedov deposition follows src/setup/setup_sedov.f90:119-135 (M4-kernel
weighted, renormalised to the blast energy). No public benchmark data exists
for this path; these seeded sets stand in for the reference's setups.
"""
from __future__ import annotations

import math

import numpy as np

PI = 3.1415926536  # physcon.f90:23
CNORMK = 1.0 / PI


def base_cfg(**kw) -> dict:
    """Defaults of the reference (options.f90:92-93, shock_capturing.f90:47-65,
    timestep.f90:52-62, eos.f90:1896-1898, kdtree.F90:46)."""
    cfg = dict(
        periodic=1, mhd=0, gravity=0, isothermal=0, ieos=2,
        ipdv_heating=1, ishock_heating=1, iresistive_heating=1, divB_hj_prepass=1,
        xmin=0.0, xmax=1.0, ymin=0.0, ymax=1.0, zmin=0.0, zmax=1.0,
        hfact=1.2, tolh=1.0e-4, massoftype=0.0,
        alpha=1.0, alphau=1.0, alphaB=1.0, beta=2.0,
        gamma=5.0 / 3.0, polyk=0.0,
        C_cour=0.3, C_force=0.25, tolv=1.0e-2, dtmax=1.0e29,
        psidecayfac=1.0, overcleanfac=1.0, tree_accuracy=0.5, maxp=0,
    )
    cfg.update(kw)
    return cfg


def cubic_lattice(n1d, lo=0.0, hi=1.0, jitter=0.0, seed=0):
    """Cubic lattice of n1d^3 points in [lo,hi)^3 with optional Gaussian jitter
    (sigma = jitter*dx), wrapped back into the box."""
    dx = (hi - lo) / n1d
    c = lo + (np.arange(n1d) + 0.5) * dx
    z, y, x = np.meshgrid(c, c, c, indexing="ij")
    pos = np.stack([x.ravel(), y.ravel(), z.ravel()], axis=1)
    if jitter > 0.0:
        rng = np.random.Generator(np.random.PCG64(seed))
        pos = pos + rng.normal(0.0, jitter * dx, size=pos.shape)
        L = hi - lo
        pos = lo + np.mod(pos - lo, L)
    return pos, dx


def hydro_lattice(n1d=64, jitter=0.05, seed=0, vseed=1, vamp=0.1, u0=1.0, rho0=1.0, hfact=1.2):
    """Plain FP64 adiabatic hydro workload: periodic unit cube, jittered cubic
    lattice, rho0=1, u0=1, gamma=5/3, velocities U[-vamp,vamp] per component,
    constant alpha_AV=1, beta=2, alpha_u=1."""
    pos, dx = cubic_lattice(n1d, 0.0, 1.0, jitter, seed)
    n = pos.shape[0]
    m = rho0 * 1.0 / n
    rng = np.random.Generator(np.random.PCG64(vseed))
    vel = rng.uniform(-vamp, vamp, size=(n, 3))
    xyzh = np.empty((n, 4)); xyzh[:, :3] = pos; xyzh[:, 3] = hfact * dx
    vxyzu = np.empty((n, 4)); vxyzu[:, :3] = vel; vxyzu[:, 3] = u0
    cfg = base_cfg(massoftype=m, hfact=hfact, maxp=n)
    return cfg, xyzh, vxyzu, np.zeros((n, 4))


def sedov(n1d=128, jitter=0.05, seed=0, ubg=1.0e-6, eblast=1.0, rho0=1.0, hfact=1.2):
    """Sedov blast: periodic [-0.5,0.5)^3, jittered lattice, blast energy
    deposited with M4 weights within 2*dx of the origin (hsmooth = dx) on top
    of a background u."""
    pos, dx = cubic_lattice(n1d, -0.5, 0.5, jitter, seed)
    n = pos.shape[0]
    m = rho0 / n
    hs = dx
    r2 = np.sum(pos * pos, axis=1)
    q = np.sqrt(r2) / hs
    w = np.where(q < 1.0, 0.75 * q ** 3 - 1.5 * q ** 2 + 1.0,
                 np.where(q < 2.0, 0.25 * (2.0 - q) ** 3, 0.0))
    uu = eblast * CNORMK * w / hs ** 3
    toten = np.sum(m * uu)
    u = ubg + uu * (eblast / toten)
    xyzh = np.empty((n, 4)); xyzh[:, :3] = pos; xyzh[:, 3] = hfact * dx
    vxyzu = np.zeros((n, 4)); vxyzu[:, 3] = u
    cfg = base_cfg(massoftype=m, hfact=hfact, maxp=n,
                   xmin=-0.5, xmax=0.5, ymin=-0.5, ymax=0.5, zmin=-0.5, zmax=0.5)
    return cfg, xyzh, vxyzu, np.zeros((n, 4))


def mhd_vortex(n1d=128, jitter=0.05, seed=0, hfact=1.2):
    """Ideal MHD Orszag-Tang-type 3D field with hyperbolic/parabolic cleaning:
    rho0=25/(36 pi), P0=5/(12 pi), v=(-sin 2pi y, sin 2pi x, 0.1 sin 2pi z),
    B=(-sin 2pi y, sin 4pi x, 0)/sqrt(4 pi), psi=0. Bevol stores B/rho."""
    pos, dx = cubic_lattice(n1d, 0.0, 1.0, jitter, seed)
    n = pos.shape[0]
    gamma = 5.0 / 3.0
    rho0 = 25.0 / (36.0 * math.pi)
    p0 = 5.0 / (12.0 * math.pi)
    m = rho0 / n
    x, y, z = pos[:, 0], pos[:, 1], pos[:, 2]
    tp = 2.0 * math.pi
    vxyzu = np.empty((n, 4))
    vxyzu[:, 0] = -np.sin(tp * y); vxyzu[:, 1] = np.sin(tp * x); vxyzu[:, 2] = 0.1 * np.sin(tp * z)
    vxyzu[:, 3] = p0 / ((gamma - 1.0) * rho0)
    B = np.zeros((n, 4))
    B[:, 0] = -np.sin(tp * y) / math.sqrt(4 * math.pi)
    B[:, 1] = np.sin(2 * tp * x) / math.sqrt(4 * math.pi)
    Bevol = B.copy(); Bevol[:, :3] /= rho0
    xyzh = np.empty((n, 4)); xyzh[:, :3] = pos; xyzh[:, 3] = hfact * dx
    cfg = base_cfg(massoftype=m, hfact=hfact, maxp=n, mhd=1, gamma=gamma)
    return cfg, xyzh, vxyzu, Bevol


def gravity_cloud(n=2 ** 21, seed=0, cs=0.2, omega=0.5, radius=1.0, hfact=1.2):
    """Self-gravitating isothermal cloud: n equal-mass particles uniformly
    random in a sphere of radius 1, total mass 1, G=1, c_s=0.2, solid-body
    rotation Omega about z, open boundaries, theta=0.5."""
    rng = np.random.Generator(np.random.PCG64(seed))
    pts = np.empty((0, 3))
    while pts.shape[0] < n:
        cand = rng.uniform(-radius, radius, size=(int(2.2 * n), 3))
        cand = cand[np.sum(cand * cand, axis=1) < radius * radius]
        pts = np.concatenate([pts, cand])[:n]
    m = 1.0 / n
    rho0 = 1.0 / (4.0 / 3.0 * math.pi * radius ** 3)
    h0 = hfact * (m / rho0) ** (1.0 / 3.0)
    xyzh = np.empty((n, 4)); xyzh[:, :3] = pts; xyzh[:, 3] = h0
    vxyzu = np.zeros((n, 4))
    vxyzu[:, 0] = -omega * pts[:, 1]; vxyzu[:, 1] = omega * pts[:, 0]
    cfg = base_cfg(massoftype=m, hfact=hfact, maxp=n, periodic=0, gravity=1, isothermal=1,
                   ieos=1, polyk=cs * cs, alphau=1.0,
                   xmin=-2.0, xmax=2.0, ymin=-2.0, ymax=2.0, zmin=-2.0, zmax=2.0)
    return cfg, xyzh, vxyzu, np.zeros((n, 4))


def exact_lattice(n1d=16, rho0=5.0, hfact=1.2, lo=-0.5, hi=0.5):
    """Unjittered cubic lattice as in the reference derivshydro test
    (src/tests/test_derivs.f90:128-177): periodic box, h = hfact*psep."""
    pos, dx = cubic_lattice(n1d, lo, hi, 0.0, 0)
    n = pos.shape[0]
    L = hi - lo
    m = rho0 * L ** 3 / n
    xyzh = np.empty((n, 4)); xyzh[:, :3] = pos; xyzh[:, 3] = hfact * (m / rho0) ** (1.0 / 3.0)
    vxyzu = np.zeros((n, 4)); vxyzu[:, 3] = 1.0
    cfg = base_cfg(massoftype=m, hfact=hfact, maxp=n, tolh=1.0e-5,
                   xmin=lo, xmax=hi, ymin=lo, ymax=hi, zmin=lo, zmax=hi)
    return cfg, xyzh, vxyzu, np.zeros((n, 4))


def sedov_test(n1d=16, hfact=1.2):
    """The reference's Sedov known-answer test (src/tests/test_sedov.f90:88-156):
    unjittered cubic lattice in the periodic [-0.5,0.5)^3 box, rho0 = 1,
    gamma = 5/3, u = 1 (the blast energy per unit mass) for particles within
    r_blast = 2 hfact psep of the origin and u = 0 elsewhere, v = 0,
    alpha = alpha_u = 1, beta = 2, tolh = 1e-5, tolv = 1e-3, C_cour = 0.1,
    C_force = 0.25, run to t = 0.1 with global timesteps."""
    pos, dx = cubic_lattice(n1d, -0.5, 0.5, 0.0, 0)
    n = pos.shape[0]
    m = 1.0 / n
    rblast = 2.0 * hfact * dx
    xyzh = np.empty((n, 4)); xyzh[:, :3] = pos; xyzh[:, 3] = hfact * dx
    vxyzu = np.zeros((n, 4))
    vxyzu[np.sum(pos * pos, axis=1) < rblast * rblast, 3] = 1.0
    cfg = base_cfg(massoftype=m, hfact=hfact, maxp=n, tolh=1.0e-5, tolv=1.0e-3, C_cour=0.1, C_force=0.25,
                   alphaB=0.0, xmin=-0.5, xmax=0.5, ymin=-0.5, ymax=0.5, zmin=-0.5, zmax=0.5, dtmax=0.1)
    return cfg, xyzh, vxyzu, np.zeros((n, 4))


WORKLOADS = {
    "hydro64": lambda: hydro_lattice(64),
    "sedov128": lambda: sedov(128),
    "mhd128": lambda: mhd_vortex(128),
    "cloud2m": lambda: gravity_cloud(2 ** 21),
}


def random_box(n=20000, seed=3, hfact=1.2, gravity=False):
    """Uniform random particles in [-0.5,0.5)^3 with h = hfact psep and
    m = 1000 / n, as the reference's revtree test sets them up
    (src/tests/test_kdtree.F90:60-69, set_unifdis('random'), at psep = n^(-1/3)
    rather than 1/100); open boundaries."""
    rng = np.random.Generator(np.random.PCG64(seed))
    pts = rng.uniform(-0.5, 0.5, size=(n, 3))
    psep = n ** (-1.0 / 3.0)
    xyzh = np.empty((n, 4)); xyzh[:, :3] = pts; xyzh[:, 3] = hfact * psep
    vxyzu = np.zeros((n, 4)); vxyzu[:, 3] = 1.0
    cfg = base_cfg(massoftype=1000.0 / n, hfact=hfact, maxp=n, periodic=0, gravity=1 if gravity else 0,
                   xmin=-1.0, xmax=1.0, ymin=-1.0, ymax=1.0, zmin=-1.0, zmax=1.0)
    return cfg, xyzh, vxyzu, np.zeros((n, 4))
