"""Analytic velocity and thermal-energy fields of the reference's derivs
tests and the derivatives they imply (src/tests/test_derivs.f90:1216-1242 vx,
vy, vz; :1246-1300 the velocity gradients; :1457 divvfunc; :1592 dudtfunc;
:1604 utherm; :1625-1660 the gradient of u; :1673-1707 forcefunc = -(gamma-1)
grad u), restated for a periodic box [xmin, xmin + L)^3, and the reference's
function check (utils_testsuite.f90:195-234: an element passes when its
absolute or its relative error is within the tolerance)."""
import numpy as np


def fields(x, xmin, L):
    """(v (N,3), u (N,)) of set_velocity_and_energy (test_derivs.f90:1029-1040)."""
    s = 2.0 * np.pi * (x - xmin) / L
    v = np.empty((len(x), 3))
    v[:, 0] = 0.5 / np.pi * L * np.sin(s[:, 0])
    v[:, 1] = 0.5 / np.pi * L * np.sin(s[:, 0]) - 0.5 / np.pi * L * np.sin(s[:, 2])
    v[:, 2] = 0.05 / np.pi * L * np.cos(2.0 * s[:, 1])
    u = 0.5 / np.pi * (3.0 + np.sin(s[:, 0]) + np.cos(s[:, 1]) + np.sin(s[:, 2]))
    return v, u


def divv(x, xmin, L):
    """dvx/dx + dvy/dy + dvz/dz."""
    s = 2.0 * np.pi * (x - xmin) / L
    return np.cos(s[:, 0])


def force(x, xmin, L, gamma):
    """-(gamma - 1) grad u."""
    s = 2.0 * np.pi * (x - xmin) / L
    g = np.empty((len(x), 3))
    g[:, 0] = 1.0 / L * np.cos(s[:, 0])
    g[:, 1] = -1.0 / L * np.sin(s[:, 1])
    g[:, 2] = 1.0 / L * np.cos(s[:, 2])
    return -(gamma - 1.0) * g


def checkvalf(x, exact, tol, smallval=1.0e-6):
    err = np.abs(x - exact)
    return float(np.where((np.abs(exact) > smallval) & (err > tol), err / np.maximum(np.abs(exact), smallval),
                          err).max())


AV_FACTOR = 124.0 / 105.0  # kernel_cubic.f90:30


def av_force(x, h, xmin, L, gamma, alpha, u=4.0):
    """Continuum form of the artificial-viscosity acceleration for the same
    velocity field with a constant u (test_derivs.f90:1714-1790 av_coeffs,
    forceavx/y/z): c1 del^2 v + c2 grad(div v), c1 = 0.1 fac, c2 = 0.2 fac,
    fac = alpha c_s h av_factor where div v < 0, else 0."""
    s = 2.0 * np.pi * (x - xmin) / L
    cs = np.sqrt(gamma * (gamma - 1.0) * u)
    fac = np.where(divv(x, xmin, L) < 0.0, alpha * cs * h * AV_FACTOR, 0.0)
    c1, c2 = 0.1 * fac, 0.2 * fac
    del2v = np.empty((len(x), 3))
    del2v[:, 0] = -2.0 * np.pi / L * np.sin(s[:, 0])
    del2v[:, 1] = -2.0 * np.pi / L * np.sin(s[:, 0]) + 2.0 * np.pi / L * np.sin(s[:, 2])
    del2v[:, 2] = -0.8 * np.pi / L * np.cos(2.0 * s[:, 1])
    graddivv = np.zeros((len(x), 3))
    graddivv[:, 0] = -2.0 * np.pi / L * np.sin(s[:, 0])
    return c1[:, None] * del2v + c2[:, None] * graddivv
