"""The ISOTHERMAL array layout through the C ABI: with maxvxyzu = 3 the caller
passes vxyzu(3,N) and fxyzu(3,N) (part.F90:465,516 with config.F90:50) and
gets the same numbers as a four-row caller, bit for bit.

* derivs, three leapfrog steps, state upload/download: the isothermal
  self-gravitating cloud, 3-row caller against 4-row caller;
* the adjoint: an isothermal hydro lattice, cotangent w(3,N) against w(4,N)
  with a zero u row;
* ph_conservation_noalloc on 3-row device arrays against ph_conservation;
* maxvxyzu = 3 without isothermal, or any other value, is PH_ERR_ARG.
"""
import ctypes as C

import numpy as np
import pytest

from phantom_gb300 import capi
from phantom_gb300 import setups as S

pytestmark = pytest.mark.gpu


def _pair(cfg, x, v, B=None):
    c4 = capi.Context(cfg)
    c4.upload(x, v, B)
    c3 = capi.Context(dict(cfg, maxvxyzu=3))
    c3.upload(x, np.ascontiguousarray(v[:, :3]), B)
    return c4, c3


def test_isothermal_rows_match_four_rows():
    cfg, x, v, B = S.gravity_cloud(3000)
    assert cfg["isothermal"] == 1
    c4, c3 = _pair(cfg, x, v, B)
    assert c3.vrows == 3
    d4 = c4.derivs(1, 0.0)
    d3 = c3.derivs(1, 0.0)
    assert d3 == d4
    f4 = c4.force(2)["fxyzu"]
    f3 = c3.force(2)["fxyzu"]
    assert f3.shape == (len(x), 3)
    assert np.array_equal(f3, f4[:, :3])
    t = 0.0
    for _ in range(3):
        dt = 0.5 * d4
        d4 = c4.step(t, dt)[0]
        d3 = c3.step(t, dt)[0]
        t += dt
    x4, v4, _ = c4.download()
    x3, v3, _ = c3.download()
    assert v3.shape == (len(x), 3)
    assert np.array_equal(x3, x4) and np.array_equal(v3, v4[:, :3])
    # state round trip in the 3-row layout
    n = len(x)
    st = [np.zeros((n, 4)), np.zeros((n, 3)), np.zeros((n, 4)), np.zeros((n, 3)), np.zeros((n, 4)),
          np.zeros(n, np.float32)]
    c3.download_state(*st)
    c3.upload_state(*st)
    back = [np.zeros_like(a) for a in st]
    c3.download_state(*back)
    for a, b in zip(st, back):
        assert np.array_equal(a, b)


def test_isothermal_rows_adjoint():
    cfg, x, v, B = S.hydro_lattice(8)
    cfg = dict(cfg, isothermal=1, ieos=1, polyk=1.0, tolh=1.0e-8)
    c4, c3 = _pair(cfg, x, v)
    rng = np.random.default_rng(3)
    w4 = np.zeros((len(x), 4)); w4[:, :3] = rng.standard_normal((len(x), 3))
    gx4, gv4 = c4.adjoint(w4)
    gx3, gv3 = c3.adjoint(np.ascontiguousarray(w4[:, :3]))
    assert gv3.shape == (len(x), 3)
    assert np.array_equal(gx3, gx4) and np.array_equal(gv3, gv4[:, :3])


def test_isothermal_rows_noalloc():
    torch = pytest.importorskip("torch")
    cfg, x, v, B = S.gravity_cloud(3000)
    c3 = capi.Context(dict(cfg, maxvxyzu=3))
    c3.upload(x, np.ascontiguousarray(v[:, :3]), B)
    c3.derivs(1, 0.0)
    ref = c3.conservation()
    n = len(x)
    st = [np.zeros((n, 4)), np.zeros((n, 3)), np.zeros((n, 4)), np.zeros((n, 3)), np.zeros((n, 4)),
          np.zeros(n, np.float32)]
    c3.download_state(*st)
    params = capi.make_params(dict(cfg, maxvxyzu=3, gravity=0))  # potential energy not compared here
    xyzh, vxyzu, fxyzu = (torch.from_numpy(a).cuda() for a in (st[0], st[1], st[3]))
    out = torch.zeros(8, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    rc = capi.lib().ph_conservation_noalloc(C.byref(params), n, C.c_void_p(xyzh.data_ptr()),
                                            C.c_void_p(vxyzu.data_ptr()), C.c_void_p(fxyzu.data_ptr()), None, None,
                                            C.c_void_p(out.data_ptr()),
                                            C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == 0
    torch.cuda.synchronize()
    got = out.cpu().numpy()
    # each sum against the sum of the magnitudes of its terms: the rotating
    # cloud's total momentum cancels to rounding level, so its own size is no
    # scale for the summation-order difference
    m = cfg["massoftype"]
    v, f = st[1][:, :3], st[3][:, :3]
    scale = np.zeros(8)
    scale[0:3] = m * np.abs(v).sum(axis=0)
    scale[3] = abs(ref[3])
    scale[7] = m * np.abs(v * f).sum()
    for k in (0, 1, 2, 3, 7):  # momentum, kinetic energy, the energy rate
        assert abs(got[k] - ref[k]) <= 1.0e-10 * max(scale[k], 1.0e-300), (k, got[k], ref[k])


def test_rows_argument_checks():
    cfg, x, v, B = S.sedov(8)
    for bad in (3, 2, 5):
        with pytest.raises(capi.PhantomError) as e:
            capi.Context(dict(cfg, maxvxyzu=bad))  # sedov is adiabatic: 3 rows need isothermal = 1
        assert e.value.code == 1
