"""The far-field mathematics of the oracle against exact point-mass sums: the
reference's Taylor-series test (src/tests/test_gravity.f90:97-220) restated.
compute_M2L of a distant node, expanded about a nearby centre
(expand_fgrav_in_taylor_series), against the exact force and potential:
(1) a point mass, evaluated off the centre; (2) a three-particle node with
its quadrupole, evaluated at the centre; (3) the same node, evaluated off
the centre. The bars are the reference's (relative, checkval1). The GPU far
field is tied to these routines by the parity and direct-summation tests."""
import numpy as np
import pytest

from oracle import oracle as O


@pytest.fixture(scope="module", autouse=True)
def _build():
    O.build()


def _rel(x, v):
    return abs(x - v) / abs(v) if abs(v) > 1.0e-6 else abs(x - v)


def _dx_dr(x1, x2):
    dx = np.asarray(x1, float) - np.asarray(x2, float)
    return dx, 1.0 / np.sqrt(dx @ dx)


def _check(f0, phi, fexact, phiexact, tols):
    for k in range(3):
        assert _rel(f0[k], fexact[k]) <= tols[k], (k, f0[k], fexact[k])
    assert _rel(phi, phiexact) <= tols[3], (phi, phiexact)


def test_point_mass_off_centre():
    totmass = 5.0
    xi, xj, x0 = np.array([0.05, -0.04, -0.05]), np.array([1.0, 1.0, 1.0]), np.zeros(3)
    dx, dr = _dx_dr(xi, xj)
    fexact, phiexact = -totmass * dr ** 3 * dx, -totmass * dr
    dx, dr = _dx_dr(x0, xj)
    fnode = O.m2l(dx, dr, totmass, np.zeros(6))
    f0, phi = O.taylor(fnode, xi - x0)
    _check(f0, phi, fexact, phiexact, (3.0e-4, 1.1e-4, 9.0e-5, 8.0e-4))


def _distant_node():
    totmass = 5.0
    xd = np.array([[1.03, 0.98, 1.01], [0.95, 1.01, 1.03], [0.99, 0.95, 0.95]])
    pm = totmass / 3.0
    xj = (pm * xd).sum(axis=0) / totmass
    q = np.zeros(6)
    for p in xd:
        d = p - xj
        q += pm * np.array([d[0] * d[0], d[0] * d[1], d[0] * d[2], d[1] * d[1], d[1] * d[2], d[2] * d[2]])
    return totmass, xd, pm, xj, q


def _exact(xi, xd, pm):
    f, phi = np.zeros(3), 0.0
    for p in xd:
        dx = xi - p
        dr = 1.0 / np.sqrt(dx @ dx)
        f -= dr ** 3 * dx
        phi -= dr
    return f * pm, phi * pm


def test_quadrupole_node_at_centre():
    totmass, xd, pm, xj, q = _distant_node()
    x0 = np.zeros(3)
    fexact, phiexact = _exact(x0, xd, pm)
    dx, dr = _dx_dr(x0, xj)
    f0, phi = O.taylor(O.m2l(dx, dr, totmass, q), np.zeros(3))
    _check(f0, phi, fexact, phiexact, (8.7e-5, 1.5e-6, 1.6e-5, 5.9e-6))


def test_quadrupole_node_off_centre():
    totmass, xd, pm, xj, q = _distant_node()
    x0, xi = np.zeros(3), np.array([0.05, 0.05, -0.05])
    fexact, phiexact = _exact(xi, xd, pm)
    dx, dr = _dx_dr(x0, xj)
    f0, phi = O.taylor(O.m2l(dx, dr, totmass, q), xi - x0)
    _check(f0, phi, fexact, phiexact, (1.3e-4, 1.4e-4, 3.2e-4, 9.7e-4))
