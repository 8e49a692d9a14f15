"""curl v (params.curlv, config.F90:166,384: ndivcurlv = 4) through the C ABI
against the oracle.

divcurlv(4,N): row 1 div v from the force loop (force.F90:2999), rows 2-4 the
curl of v from the density's velocity-gradient sums (dens.F90:758-802,
919-923) with the velocities the density is evaluated with. Checks on the
jittered hydro lattice 24^3 with random velocities:

* one derivs, FP64: every row within 2e-7 of the largest |value| of its row
  (float32 outputs of FP64 sums that differ only in summation order);
  precision form: div v within 1e-5, the curl rows within 5e-4. The
  velocity-gradient sums are made with the h of the last Newton iterate
  (store_results keeps the pre-update h), which is within tolh = 1e-4 of the
  root; FP32 density sums can end a cell's iteration one pass earlier or
  later than FP64, so for a few particles that h, and the curl with it,
  differs at the tolh level (measured 1.2e-4 on one particle of 13824, the
  others within 3e-7) while the final h agrees to 1e-6;
* three steps (ph_step, which predicts h from row 1): positions and
  velocities within the FP64 parity bar (1e-10 of the largest) and the curl
  rows as above, so the curl rows follow the step's predicted velocities;
* the state round trip: ph_download_state and ph_upload_state carry the
  four rows, and a context without curlv keeps the one-row layout.
"""
import numpy as np
import pytest

from oracle import oracle as O
from phantom_gb300 import capi
from phantom_gb300 import setups as S

pytestmark = pytest.mark.gpu


def _cfg():
    cfg, x, v, B = S.hydro_lattice(24)
    return dict(cfg, curlv=1), x, v


def _rows_close(g, o, tol, tol_curl=None):
    assert g.shape == o.shape == (len(g), 4)
    for k in range(4):
        t = tol if k == 0 or tol_curl is None else tol_curl
        scale = np.abs(o[:, k]).max()
        assert scale > 0.0
        assert np.abs(g[:, k].astype(np.float64) - o[:, k]).max() <= t * scale, (k, t)


@pytest.mark.parametrize("prec", [capi.PH_PREC_FP64, capi.PH_PREC_MIXED])
def test_curlv_derivs_matches_oracle(prec):
    cfg, x, v = _cfg()
    o = O.Oracle(cfg, nthreads=8)
    o.set_particles(x, v)
    o.derivs(1, 0.0)
    od = o.get_force()["divcurlv"]
    dev = capi.Context(cfg, precision=prec)
    dev.upload(x, v)
    dev.derivs(1, 0.0)
    n = len(x)
    xo, vo, fo = np.empty((n, 4)), np.empty((n, 4)), np.empty((n, 4))
    gd = dev.divcurlv_array()
    dev.download_state(xo, vo, None, fo, None, gd)
    if prec == capi.PH_PREC_FP64:
        _rows_close(gd, od, 2.0e-7)
    else:
        _rows_close(gd, od, 1.0e-5, 5.0e-4)
    # ph_force returns the same four rows (row 1 recomputed by the force loop)
    f = dev.force(2, 0.0)
    assert np.array_equal(f["divcurlv"], gd)


def test_curlv_steps_match_oracle():
    cfg, x, v = _cfg()
    o = O.Oracle(cfg, nthreads=8)
    o.set_particles(x, v)
    dev = capi.Context(cfg)
    dev.upload(x, v)
    dt = 0.5 * min(o.derivs(1, 0.0), dev.derivs(1, 0.0))
    t = 0.0
    for _ in range(3):
        o.step(t, dt)
        dev.step(t, dt)
        t += dt
    n = len(x)
    xo, vo, fo = np.empty((n, 4)), np.empty((n, 4)), np.empty((n, 4))
    gd = dev.divcurlv_array()
    dev.download_state(xo, vo, None, fo, None, gd)
    ox, ov, _ = o.get_particles()
    assert np.abs(xo - ox).max() <= 1.0e-10 * np.abs(ox).max()
    assert np.abs(vo - ov).max() <= 1.0e-10 * np.abs(ov).max()
    _rows_close(gd, o.get_force()["divcurlv"], 2.0e-7)


def test_curlv_state_round_trip():
    cfg, x, v = _cfg()
    dev = capi.Context(cfg)
    dev.upload(x, v)
    dev.derivs(1, 0.0)
    n = len(x)
    xo, vo, fo = np.empty((n, 4)), np.empty((n, 4)), np.empty((n, 4))
    gd = dev.divcurlv_array()
    dev.download_state(xo, vo, None, fo, None, gd)
    dev2 = capi.Context(cfg)
    dev2.upload_state(xo, vo, None, fo, None, gd)
    back = dev2.divcurlv_array()
    dev2.download_state(np.empty((n, 4)), np.empty((n, 4)), None, np.empty((n, 4)), None, back)
    assert np.array_equal(back, gd)
    # without curlv the layout stays one row
    dev3 = capi.Context(dict(cfg, curlv=0))
    dev3.upload(x, v)
    dev3.derivs(1, 0.0)
    one = dev3.divcurlv_array()
    assert one.shape == (n,)
    dev3.download_state(np.empty((n, 4)), np.empty((n, 4)), None, np.empty((n, 4)), None, one)
    assert np.array_equal(one, gd[:, 0])
