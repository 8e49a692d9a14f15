"""Mixed-precision form against the FP64 oracle.

The FP32 pair terms (on FP64 separations, Kahan-accumulated per particle)
must reproduce the FP64 accelerations, du/dt and dB/dt to within 1e-5 of
their maximum magnitude (the precision target of this form), smoothing
lengths to 1e-6 and three leapfrog steps to 1e-5.
"""
import numpy as np
import pytest

from oracle import oracle as O
from phantom_gb300 import capi
from phantom_gb300 import setups as S

pytestmark = pytest.mark.gpu

TOL = 1.0e-5


def relmax(a, b):
    s = np.abs(b).max()
    return 0.0 if s == 0.0 else np.abs(a - b).max() / s


@pytest.mark.parametrize("name,mk", [("hydro24", lambda: S.hydro_lattice(24)),
                                     ("sedov32", lambda: S.sedov(32)),
                                     ("mhd24", lambda: S.mhd_vortex(24)),
                                     ("grav6k", lambda: S.gravity_cloud(6000))])
def test_mixed_force_error(name, mk):
    cfg, x, v, B = mk()
    o = O.Oracle(cfg, nthreads=8)
    o.set_particles(x, v, B)
    o.derivs(1, 0.0)
    fo = o.get_force()
    xo, _, _ = o.get_particles()
    ctx = capi.Context(cfg, precision=capi.PH_PREC_MIXED)
    ctx.upload(x, v, B)
    ctx.derivs(1, 0.0)
    fg = ctx.force(2, 0.0)
    xg, _, _ = ctx.download()
    assert relmax(xg[:, 3], xo[:, 3]) < 1.0e-6
    for c in range(4):
        assert relmax(fg["fxyzu"][:, c], fo["fxyzu"][:, c]) < TOL, (name, c)
        if cfg["mhd"]:
            assert relmax(fg["dBevol"][:, c], fo["dBevol"][:, c]) < TOL, (name, c)


def test_mixed_steps_error():
    cfg, x, v, B = S.sedov(32)
    o = O.Oracle(cfg, nthreads=8)
    o.set_particles(x, v, B)
    dt = o.derivs(1, 0.0)
    ctx = capi.Context(cfg, precision=capi.PH_PREC_MIXED)
    ctx.upload(x, v, B)
    ctx.derivs(1, 0.0)
    t = 0.0
    for _ in range(3):
        dto, _, dterro = o.step(t, dt)
        ctx.step(t, dt)
        t += dt
        dt = min(dto, dterro)
    xo, vo, _ = o.get_particles()
    xg, vg, _ = ctx.download()
    assert relmax(xg[:, :3], xo[:, :3]) < TOL
    assert relmax(vg[:, :3], vo[:, :3]) < TOL
    assert relmax(vg[:, 3], vo[:, 3]) < TOL
