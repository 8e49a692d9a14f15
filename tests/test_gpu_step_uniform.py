"""The reference's step test (src/tests/test_step.F90:60-160) on the GPU: a
50^3 periodic cubic lattice in uniform motion v = (1, 1, 1) with no pressure
(u = 0, polyk = 0) and no dissipation, 10 leapfrog steps of dt = 0.2 (two
box crossings: the tree build wraps the particles every step). After every
step h = h0 to 3e-4 and the accelerations and du/dt are exactly zero (the
reference's bar is tiny(0.)). FP64 path and mixed form."""
import numpy as np
import pytest

from phantom_gb300 import capi
from phantom_gb300 import setups as S

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("mixed", [False, True])
def test_uniform_flow_exactly_force_free(mixed):
    cfg, x, v, B = S.exact_lattice(50, rho0=1.0)
    cfg = dict(cfg, alpha=0.0, alphau=0.0, alphaB=0.0, polyk=0.0, tolh=1.0e-5, dtmax=0.2)
    v[:, :3] = 1.0
    v[:, 3] = 0.0
    h0 = x[0, 3]
    ctx = capi.Context(cfg, precision=capi.PH_PREC_MIXED if mixed else capi.PH_PREC_FP64)
    ctx.upload(x, v, B)
    ctx.derivs(1, 0.0)
    n = len(x)
    t = 0.0
    for _ in range(10):
        ctx.step(t, 0.2)
        t += 0.2
        st = [np.zeros((n, 4)) for _ in range(5)] + [np.zeros(n, np.float32)]
        ctx.download_state(*st)
        xyzh, fxyzu = st[0], st[3]
        assert np.abs(xyzh[:, 3] / h0 - 1.0).max() <= 3.0e-4
        assert np.abs(fxyzu).max() <= np.finfo(np.float64).tiny
    # after two box crossings every particle is wrapped into the box
    xyzh = st[0]
    assert np.all((xyzh[:, :3] >= -0.5) & (xyzh[:, :3] < 0.5))
