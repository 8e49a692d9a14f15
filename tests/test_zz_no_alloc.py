"""ph_conservation_noalloc, the entry point that allocates nothing, through
the C ABI.

Some callers cannot let this library allocate: host codes whose particle
arrays already live on the device in their own allocator, with no context of
this library, and which cannot take the device-wide synchronisation of
cudaMalloc/cudaFree in the middle of a step. ph_conservation_noalloc gives
them the momentum and energy sums of ph_conservation over their own device
arrays, with its scratch in a fixed array of the library's device image.

Checks, three calls in a row sharing that scratch array:

* a 72^3 hydro lattice (1458 reduction blocks, more than ph_conservation's
  1024-block grid, so the summation order differs);
* a 24^3 MHD lattice (54 blocks: rows left by the first call are stale);
* a self-gravitating cloud of 3000 particles with its potential energy read
  from the caller's float32 poten array.

Each result must agree with ph_conservation and with an independent numpy
FP64 evaluation of the same sums on the downloaded arrays, to 1e-10 of the
sum of the magnitudes of each sum's terms (the FP64 parity bar; the two
device reductions differ in order only, numpy in order and in the kernel's
arithmetic). Collected last so that it also runs after the other GPU tests
in the same process; it passes alone as well.
"""
import ctypes as C

import numpy as np
import pytest

from phantom_gb300 import capi
from phantom_gb300 import setups as S

pytestmark = pytest.mark.gpu

TOL = 1.0e-10


def energies_numpy(cfg, xyzh, vxyzu, fxyzu, Bevol, poten):
    """The eight sums of ph_conservation in FP64 with numpy, restating
    compute_energies (src/main/energies.f90): momentum m v (:297-299),
    kinetic energy 0.5 m v^2 (:288, :307, halved at :676), thermal energy m u
    (:433), magnetic energy 0.5 m B^2/rho = 0.5 m rho |B/rho|^2 (halved at
    :677), potential energy sum poten (:356), and the energy rate
    sum m (v . a + du/dt). Dead particles (h <= 0) are skipped. Returns the
    sums and the sum of |term| of each (the scale of its rounding error)."""
    m = cfg["massoftype"]
    live = xyzh[:, 3] > 0.0
    v, f = vxyzu[live, :3], fxyzu[live, :3]
    iso = bool(cfg["isothermal"])
    out = np.zeros(8)
    scale = np.zeros(8)
    out[0:3] = (m * v).sum(axis=0)
    scale[0:3] = (m * np.abs(v)).sum(axis=0)
    out[3] = (0.5 * m * (v * v).sum(axis=1)).sum()
    scale[3] = out[3]
    if not iso:
        out[4] = (m * vxyzu[live, 3]).sum()
        scale[4] = np.abs(m * vxyzu[live, 3]).sum()
    if cfg["mhd"]:
        rho = m * (cfg["hfact"] / np.abs(xyzh[live, 3])) ** 3  # rhoh, part.F90:779-785
        b = Bevol[live, :3]
        out[5] = (0.5 * m * rho * (b * b).sum(axis=1)).sum()
        scale[5] = out[5]
    if cfg["gravity"]:
        pt = poten[live].astype(np.float64)
        out[6] = pt.sum()
        scale[6] = np.abs(pt).sum()
    rate = m * ((v * f).sum(axis=1) + (0.0 if iso else fxyzu[live, 3]))
    out[7] = rate.sum()
    scale[7] = (m * (np.abs(v * f).sum(axis=1) + (0.0 if iso else np.abs(fxyzu[live, 3])))).sum()
    return out, np.maximum(scale, 1.0e-300)


def _device_state(setup):
    """Run derivs on a context; return its config, params, the caller-order
    state on the host and ph_conservation's sums of that state."""
    cfg, x, v, B = setup
    ctx = capi.Context(cfg)
    ctx.upload(x, v, B)
    ctx.derivs(1, 0.0)
    n = x.shape[0]
    xyzh, vxyzu, Bevol, fxyzu, dB = (np.zeros((n, 4)) for _ in range(5))
    divv = np.zeros(n, np.float32)
    ctx.download_state(xyzh, vxyzu, Bevol, fxyzu, dB, divv)
    poten = ctx.force(2, 0.0)["poten"] if cfg["gravity"] else None
    ref = ctx.conservation()
    params = capi.make_params(cfg)
    ctx.close()
    return cfg, params, (xyzh, vxyzu, Bevol, fxyzu, poten), ref


def _call_noalloc(torch, cfg, params, arrays):
    L = capi.lib()
    xyzh, vxyzu, Bevol, fxyzu, poten = arrays
    d = [torch.from_numpy(a).cuda() for a in (xyzh, vxyzu, Bevol, fxyzu)]
    dp = torch.from_numpy(poten).cuda() if poten is not None else None
    out = torch.full((8,), float("nan"), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream().cuda_stream
    rc = L.ph_conservation_noalloc(C.byref(params), xyzh.shape[0], C.c_void_p(d[0].data_ptr()),
                                   C.c_void_p(d[1].data_ptr()), C.c_void_p(d[3].data_ptr()),
                                   C.c_void_p(d[2].data_ptr()) if cfg["mhd"] else None,
                                   C.c_void_p(dp.data_ptr()) if dp is not None else None,
                                   C.c_void_p(out.data_ptr()), C.c_void_p(stream))
    torch.cuda.synchronize()
    assert rc == 0, L.ph_strerror(rc).decode()
    return out.cpu().numpy()


def test_noalloc_matches_conservation_and_numpy():
    torch = pytest.importorskip("torch")
    cases = [S.hydro_lattice(72), S.mhd_vortex(24), S.gravity_cloud(3000)]
    for setup in cases:
        cfg, params, arrays, ref = _device_state(setup)
        got = _call_noalloc(torch, cfg, params, arrays)
        xyzh, vxyzu, Bevol, fxyzu, poten = arrays
        want, scale = energies_numpy(cfg, xyzh, vxyzu, fxyzu, Bevol, poten)
        tag = (cfg["mhd"], cfg["gravity"])
        assert (np.abs(got - ref) / scale).max() <= TOL, (tag, got, ref)
        assert (np.abs(got - want) / scale).max() <= TOL, (tag, got, want)
        assert (np.abs(ref - want) / scale).max() <= TOL, (tag, ref, want)
        if cfg["gravity"]:
            assert want[6] < 0.0 and got[6] != 0.0  # the potential energy was read


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
