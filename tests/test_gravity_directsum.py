"""Tree self-gravity against direct summation: the reference's gravity test
(src/tests/test_gravity.f90:228-420) restated. About 1000 equal-mass particles
random in a unit sphere, total mass 1, no pressure, no velocity, no
dissipation, tolh = 1e-5, tree_accuracy = 0.5. Forces from derivs against
directsum_grav per component (7.2e-3, 6e-3, 9.4e-3 with the reference's
absolute-or-relative rule), the total force m sum f to 2.5e-17 / 2.5e-17 /
2.9e-17, the potential energy sum poten against the direct sum's to 5.2e-4
and against -3/5 G M^2 / R to 3.6e-2. Run on the oracle (CPU) and on the
GPU's FP64 path; the mixed form meets the force and potential bars (its FP32
pair terms are not antisymmetric, so its total force is bounded by 1e-6 of
sum m |f| instead).
"""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
from directsum import checkval_array, directsum_grav  # noqa: E402

from phantom_gb300 import setups as S  # noqa: E402

TOLS = (7.2e-3, 6.0e-3, 9.4e-3)
FSUM = (2.5e-17, 2.5e-17, 2.9e-17)


def _cloud():
    cfg, x, v, B = S.gravity_cloud(1000, cs=0.0, omega=0.0)
    cfg = dict(cfg, alpha=0.0, alphau=0.0, alphaB=0.0, tolh=1.0e-5, tree_accuracy=0.5)
    return cfg, x, v, B


def _check(cfg, xyzh, gradh, f, poten, exact_fsum=True):
    m = cfg["massoftype"]
    fg, phitot = directsum_grav(xyzh, gradh, m)
    for k in range(3):
        assert checkval_array(f[:, k], fg[:, k], TOLS[k]) <= TOLS[k], k
    fsum = m * f[:, :3].sum(axis=0)
    if exact_fsum:
        for k in range(3):
            assert abs(fsum[k]) <= FSUM[k], (k, fsum)
    else:
        assert np.abs(fsum).max() <= 1.0e-6 * m * np.abs(f[:, :3]).sum()
    epot = float(np.sum(poten.astype(np.float64)))
    assert abs(epot / phitot - 1.0) <= 5.2e-4
    assert abs(epot / (-3.0 / 5.0) - 1.0) <= 3.6e-2


def test_oracle_gravity_against_direct_sum():
    from oracle import oracle as O
    O.build()
    cfg, x, v, B = _cloud()
    o = O.Oracle(cfg, nthreads=4)
    o.set_particles(x, v, B)
    o.derivs(1, 0.0)  # converge h as the reference's first get_derivs_global
    o.derivs(1, 0.0)
    xyzh, _, _ = o.get_particles()
    d = o.get_density()
    fo = o.get_force()
    _check(cfg, xyzh, d["gradh"], fo["fxyzu"], fo["poten"])


@pytest.mark.gpu
@pytest.mark.parametrize("mixed", [False, True])
def test_gpu_gravity_against_direct_sum(mixed):
    from phantom_gb300 import capi
    cfg, x, v, B = _cloud()
    ctx = capi.Context(cfg, precision=capi.PH_PREC_MIXED if mixed else capi.PH_PREC_FP64)
    ctx.upload(x, v, B)
    ctx.derivs(1, 0.0)
    ctx.build_tree()
    d = ctx.densityiterate(1)
    fo = ctx.force(2)
    _check(cfg, d["xyzh"], d["gradh"], fo["fxyzu"], fo["poten"], exact_fsum=not mixed)
