"""ph_conservation_noalloc, the entry point that allocates nothing, against
ph_conservation on the same device state, through the C ABI.

Two calls in a row share the static scratch array: first a 72^3 hydro
lattice (1458 reduction blocks, more than the 1024-block grid of
ph_conservation, so the summation order differs), then a 24^3 MHD lattice
(54 blocks, rows left by the first call are stale). Each result must agree
with ph_conservation to 1e-10 of the sum of the magnitudes of its terms, the
bar the FP64 parity tests use. Collected last so that it also runs after the
other GPU tests in the same process.
"""
import ctypes as C

import numpy as np
import pytest

from phantom_gb300 import capi
from phantom_gb300 import setups as S

pytestmark = pytest.mark.gpu

TOL = 1.0e-10


def _device_state(setup):
    """Run derivs on a context; return its params, the caller-order state on
    the host and ph_conservation's sums of that state."""
    cfg, x, v, B = setup
    ctx = capi.Context(cfg)
    ctx.upload(x, v, B)
    ctx.derivs(1, 0.0)
    n = x.shape[0]
    xyzh, vxyzu, Bevol, fxyzu, dB = (np.zeros((n, 4)) for _ in range(5))
    divv = np.zeros(n, np.float32)
    ctx.download_state(xyzh, vxyzu, Bevol, fxyzu, dB, divv)
    ref = ctx.conservation()
    params = capi.make_params(cfg)
    del ctx
    return cfg, params, (xyzh, vxyzu, Bevol, fxyzu), ref


def _scale(cfg, ref, xyzh, vxyzu, Bevol, fxyzu):
    """Sum of |term| of each of the 8 sums (the size of their rounding error).
    The energies are sums of non-negative terms: their own value."""
    m = cfg["massoftype"]
    v, f = vxyzu[:, :3], fxyzu[:, :3]
    s = np.abs(ref).copy()
    s[0:3] = m * np.abs(v).sum(axis=0)
    s[7] = m * (np.abs((v * f).sum(axis=1)) + np.abs(fxyzu[:, 3])).sum()
    return np.maximum(s, 1.0e-300)


def _call_noalloc(torch, params, arrays, Bevol_used):
    L = capi.lib()
    xyzh, vxyzu, Bevol, fxyzu = (torch.from_numpy(a).cuda() for a in arrays)
    out = torch.zeros(8, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream().cuda_stream
    rc = L.ph_conservation_noalloc(C.byref(params), xyzh.shape[0], C.c_void_p(xyzh.data_ptr()),
                                   C.c_void_p(vxyzu.data_ptr()), C.c_void_p(fxyzu.data_ptr()),
                                   C.c_void_p(Bevol.data_ptr()) if Bevol_used else None, None,
                                   C.c_void_p(out.data_ptr()), C.c_void_p(stream))
    torch.cuda.synchronize()
    assert rc == 0, L.ph_strerror(rc).decode()
    return out.cpu().numpy()


def test_noalloc_matches_conservation_two_calls():
    torch = pytest.importorskip("torch")
    cases = [S.hydro_lattice(72), S.mhd_vortex(24)]
    for setup in cases:
        cfg, params, arrays, ref = _device_state(setup)
        got = _call_noalloc(torch, params, arrays, bool(cfg["mhd"]))
        err = np.abs(got - ref) / _scale(cfg, ref, *arrays)
        assert err.max() <= TOL, (cfg["mhd"], got, ref, err)


def test_noalloc_rejects_npart_above_limit():
    torch = pytest.importorskip("torch")
    L = capi.lib()
    cfg, _, _, _ = S.hydro_lattice(4)
    params = capi.make_params(cfg)
    buf = torch.zeros(16, dtype=torch.float64, device="cuda")
    p = C.c_void_p(buf.data_ptr())
    rc = L.ph_conservation_noalloc(C.byref(params), capi.PH_NOALLOC_MAX_PARTICLES + 1, p, p, p, None, None, p,
                                   None)
    assert rc == capi.PH_ERR_SCRATCH_LIMIT
    assert "static scratch limit" in L.ph_strerror(rc).decode()
