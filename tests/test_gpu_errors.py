"""Failure reporting of the GPU path, injected on the host (no GPU fault):
NaN positions (kdtree.F90:391-393), impossible h tolerance (dens.F90:1443-1456,
bounded at 100 iterations), call order, capacity. Each returns a status code
and leaves the context usable."""
import numpy as np
import pytest

from phantom_gb300 import capi
from phantom_gb300 import setups as S

pytestmark = pytest.mark.gpu


def _ctx(n1d=10):
    cfg, x, v, B = S.hydro_lattice(n1d)
    ctx = capi.Context(cfg)
    return cfg, x, v, B, ctx


def test_nan_position_reported():
    cfg, x, v, B, ctx = _ctx()
    x = x.copy(); x[17, 1] = np.nan
    ctx.upload(x, v, B)
    with pytest.raises(capi.PhantomError) as e:
        ctx.build_tree()
    assert e.value.code == 3
    # the context still works after the error
    cfg2, x2, v2, B2 = S.hydro_lattice(10)
    ctx.upload(x2, v2, B2)
    ctx.derivs(1, 0.0)


def test_density_nonconvergence_reported():
    cfg, x, v, B, ctx = _ctx()
    ctx.set_params(dict(tolh=0.0))
    ctx.upload(x, v, B)
    ctx.build_tree()
    with pytest.raises(capi.PhantomError) as e:
        ctx.densityiterate(1)
    assert e.value.code == 7


def test_force_before_density_is_refused():
    cfg, x, v, B, ctx = _ctx()
    ctx.upload(x, v, B)
    with pytest.raises(capi.PhantomError) as e:
        ctx.force(1, 0.0)
    assert e.value.code == 13


def test_capacity_checked():
    cfg, x, v, B = S.hydro_lattice(8)
    ctx = capi.Context(cfg, maxp=100)
    with pytest.raises(capi.PhantomError) as e:
        ctx.upload(x, v, B)
    assert e.value.code == 12
