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


BEXT = (0.2, 0.3, 0.5)  # test_derivs.f90:476-478


def bfield(x, xmin, L):
    """B and its gradient dB[:, a, b] = dB_a/dx_b (test_derivs.f90:1947-2040)."""
    s = 2.0 * np.pi * (x - xmin) / L
    n = len(x)
    B = np.empty((n, 3))
    B[:, 0] = -5.0 / np.pi * L * np.cos(s[:, 2]) + BEXT[0] + 0.5 / np.pi * L * np.sin(s[:, 0])
    B[:, 1] = 5.0 / np.pi * L * np.sin(s[:, 0]) + BEXT[1]
    B[:, 2] = 15.0 / np.pi * L * np.cos(s[:, 1]) + BEXT[2]
    dB = np.zeros((n, 3, 3))
    dB[:, 0, 0] = np.cos(s[:, 0])
    dB[:, 0, 2] = 10.0 * np.sin(s[:, 2])
    dB[:, 1, 0] = 10.0 * np.cos(s[:, 0])
    dB[:, 2, 1] = -30.0 * np.sin(s[:, 1])
    return B, dB


def vgrad(x, xmin, L):
    """dv[:, a, b] = dv_a/dx_b of the velocity field (test_derivs.f90:1246-1300)."""
    s = 2.0 * np.pi * (x - xmin) / L
    dv = np.zeros((len(x), 3, 3))
    dv[:, 0, 0] = np.cos(s[:, 0])
    dv[:, 1, 0] = np.cos(s[:, 0])
    dv[:, 1, 2] = -np.cos(s[:, 2])
    dv[:, 2, 1] = -0.2 * np.sin(2.0 * s[:, 1])
    return dv


def mhd_expected(x, rho, rho0, xmin, L):
    """divB, curlB, d(B/rho)/dt = (B.grad) v / rho and the Lorentz force
    -(grad(B^2/2) - (B.grad)B) / rho0 (test_derivs.f90:2182-2340)."""
    B, dB = bfield(x, xmin, L)
    dv = vgrad(x, xmin, L)
    divB = dB[:, 0, 0] + dB[:, 1, 1] + dB[:, 2, 2]
    curlB = np.stack([dB[:, 2, 1] - dB[:, 1, 2], dB[:, 0, 2] - dB[:, 2, 0], dB[:, 1, 0] - dB[:, 0, 1]], axis=1)
    dBdt = np.einsum("nb,nab->na", B, dv) / rho[:, None]
    fiso = np.einsum("na,nab->nb", B, dB)      # grad(B^2/2)
    faniso = np.einsum("nb,nab->na", B, dB)    # (B.grad) B
    return divB, curlB, dBdt, -(fiso - faniso) / rho0
