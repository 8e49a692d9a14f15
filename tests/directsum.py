"""Direct-summation self-gravity of SPH particles with kernel softening and
the gradsoft (grad-h) correction: a restatement of the reference's test
routine directsum_grav (src/tests/directsum.f90:48-194), G = 1, equal masses,
vectorised over j for each i. Returns the accelerations (N,3) and the total
potential energy. Also the reference's array check (utils_testsuite.f90:
473-518): an element passes when its absolute or its relative error is
within the tolerance."""
import numpy as np

CNORMK = 1.0 / np.pi


def _grkern(q):
    """grkern of the M4 cubic spline (kernel_cubic.f90)."""
    return np.where(q < 1.0, q * (2.25 * q - 3.0), np.where(q < 2.0, -0.75 * (2.0 - q) ** 2, 0.0))


def _softening(q2, q):
    """kernel_softening (kernel_cubic.f90:101-120): potential and force factor."""
    q4 = q2 * q2
    q6 = q4 * q2
    with np.errstate(divide="ignore", invalid="ignore"):
        pot = np.where(q < 1.0, q4 * q / 10.0 - 3.0 * q4 / 10.0 + 2.0 * q2 / 3.0 - 7.0 / 5.0,
                       np.where(q < 2.0, (q * (-q4 * q + 9.0 * q4 - 30.0 * q2 * q + 40.0 * q2 - 48.0) + 2.0) / (30.0 * q),
                                -1.0 / q))
        fs = np.where(q < 1.0, q * (15.0 * q2 * q - 36.0 * q2 + 40.0) / 30.0,
                      np.where(q < 2.0, (-5.0 * q6 + 36.0 * q4 * q - 90.0 * q4 + 80.0 * q2 * q - 2.0) / (30.0 * q2),
                               1.0 / q2))
    return pot, fs


def directsum_grav(xyzh, gradh, pmass):
    x = np.asarray(xyzh[:, :3], np.float64)
    h = np.asarray(xyzh[:, 3], np.float64)
    g1 = np.asarray(gradh[:, 0], np.float64)
    g2 = np.asarray(gradh[:, 1], np.float64)
    n = len(x)
    fgrav = np.zeros((n, 3))
    phitot = 0.0
    potensoft0 = -7.0 / 5.0
    for i in range(n):
        hi = h[i]
        hi1 = 1.0 / hi
        hi21 = hi1 * hi1
        hi41 = hi21 * hi21
        fgravi = np.zeros(3)
        sl = slice(i + 1, n)
        dx = x[i] - x[sl]
        hj = h[sl]
        hj1 = 1.0 / hj
        rij2 = np.sum(dx * dx, axis=1)
        rij = np.sqrt(rij2)
        rij1 = 1.0 / rij
        rij21 = rij1 * rij1
        dr = dx * rij1[:, None]
        hj21 = hj1 * hj1
        hj41 = hj21 * hj21
        fgravj = np.zeros_like(dx)
        q2i = rij2 * hi21
        q2j = rij2 * hj21
        ini = q2i < 4.0
        qi = np.sqrt(q2i)
        poti, fsi = _softening(q2i, qi)
        phii = np.where(ini, poti * hi1, -rij1)
        fmi = np.where(ini, fsi * hi21, rij21)
        dsofti = np.where(ini, 0.5 * (CNORMK * _grkern(qi) * hi41 * g1[i]) * g2[i], 0.0)
        fgravi -= np.sum(pmass * dsofti[:, None] * dr, axis=0)
        fgravj += pmass * dsofti[:, None] * dr
        inj = q2j < 4.0
        qj = np.sqrt(q2j)
        potj, fsj = _softening(q2j, qj)
        phij = np.where(inj, potj * hj1, -rij1)
        fmj = np.where(inj, fsj * hj21, rij21)
        dsoftj = np.where(inj, 0.5 * (CNORMK * _grkern(qj) * hj41 * g1[sl]) * g2[sl], 0.0)
        fgravi -= np.sum(pmass * dsoftj[:, None] * dr, axis=0)
        fgravj += pmass * dsoftj[:, None] * dr
        phiterm = 0.5 * (phii + phij)
        phitemp = np.sum(pmass * phiterm)
        phitot += np.sum(pmass * pmass * phiterm)
        fm = 0.5 * (fmi + fmj)
        fgravi -= np.sum(pmass * dr * fm[:, None], axis=0)
        fgrav[sl] += pmass * dr * fm[:, None] + fgravj
        fgrav[i] += fgravi
        phitot += pmass * phitemp + pmass * pmass * potensoft0 * hi1
    return fgrav, 0.5 * phitot


def checkval_array(x, xexact, tol, smallval=1.0e-6):
    """Largest error of utils_testsuite checkval_r8arr: the absolute error,
    divided by |exact| where that is above smallval and the absolute error
    is above tol."""
    err = np.abs(x - xexact)
    rel = np.where((np.abs(xexact) > smallval) & (err > tol), err / np.maximum(np.abs(xexact), smallval), err)
    return float(rel.max())
