"""The symmetric FP64 force loop (each unordered neighbour pair evaluated once,
its terms added to both particles' sums) against the per-side loop that
evaluates every pair from each of its particles as the reference's
compute_forces does (force.F90:914-2060), through the C ABI.

Bars: accelerations, du/dt, dB/dt and dpsi/dt within 1e-12 of their largest
magnitude (the two loops differ in summation order and in the rounding of
the terms seen from j only); timesteps within 1e-12; the same neighbour pair
work halved; results bit-identical between runs and between warps per block
(fixed summation order). The FP64 parity tests against the oracle run on the
symmetric loop (it is the default for FP64 without self-gravity).
"""
import numpy as np
import pytest

from phantom_gb300 import capi
from phantom_gb300 import setups as S

pytestmark = pytest.mark.gpu


def _iso_hydro():
    cfg, x, v, B = S.hydro_lattice(20)
    return dict(cfg, isothermal=1, ieos=1, polyk=0.5), x, v, B


SETS = {
    "hydro24": lambda: S.hydro_lattice(24),
    "sedov32": lambda: S.sedov(32),
    "mhd24": lambda: S.mhd_vortex(24),
    "iso_hydro20": _iso_hydro,
    "hydro20_leaf6": lambda: (dict(S.hydro_lattice(20)[0], minpart=6),) + S.hydro_lattice(20)[1:],
    "sedov24_leaf16": lambda: (dict(S.sedov(24)[0], minpart=16),) + S.sedov(24)[1:],
}


def relmax(a, b):
    s = np.abs(b).max()
    return 0.0 if s == 0.0 else float(np.abs(a - b).max() / s)


def _force(cfg, x, v, B, sym, warps=4):
    ctx = capi.Context(cfg)
    ctx.set_tune(force_sym=1 if sym else 0, force_warps=warps)
    assert ctx.tune()["force_sym"] == (1 if sym else 0)
    ctx.upload(x, v, B)
    ctx.derivs(1, 0.0)
    out = ctx.force(2, 0.0)
    out["pairs"] = int(ctx.work_counters()[2])
    ctx.close()
    return out


@pytest.mark.parametrize("name", list(SETS))
def test_symmetric_matches_per_side(name):
    cfg, x, v, B = SETS[name]()
    a = _force(cfg, x, v, B, True)
    b = _force(cfg, x, v, B, False)
    for c in range(4):
        assert relmax(a["fxyzu"][:, c], b["fxyzu"][:, c]) < 1.0e-12, c
        assert relmax(a["dBevol"][:, c], b["dBevol"][:, c]) < 1.0e-12, c
    assert abs(a["dtcourant"] / b["dtcourant"] - 1.0) < 1.0e-12
    assert abs(a["dtforce"] / b["dtforce"] - 1.0) < 1.0e-12
    dvs, dvp = a["divcurlv"].astype(np.float64), b["divcurlv"].astype(np.float64)
    assert np.abs(dvs - dvp).max() <= 1.0e-6 * max(np.abs(dvp).max(), 1.0e-30)
    if cfg["mhd"]:
        assert relmax(a["divBsymm"].astype(np.float64), b["divBsymm"].astype(np.float64)) < 1.0e-6
    # each unordered pair once: a little over half the (i, trial j) tests
    assert a["pairs"] < 0.62 * b["pairs"], (a["pairs"], b["pairs"])


@pytest.mark.parametrize("name", ["sedov32", "mhd24"])
def test_symmetric_is_deterministic(name):
    cfg, x, v, B = SETS[name]()
    a = _force(cfg, x, v, B, True, warps=4)
    b = _force(cfg, x, v, B, True, warps=4)
    c = _force(cfg, x, v, B, True, warps=1)
    for k in ("fxyzu", "dBevol", "divcurlv"):
        assert np.array_equal(a[k], b[k]), k
        assert np.array_equal(a[k], c[k]), k


def test_symmetric_steps_match_per_side():
    cfg, x, v, B = S.sedov(24)
    res = []
    for sym in (True, False):
        ctx = capi.Context(cfg)
        ctx.set_tune(force_sym=1 if sym else 0)
        ctx.upload(x, v, B)
        dt = ctx.derivs(1, 0.0)
        t = 0.0
        its = []
        for _ in range(4):
            dtn, it, dterr = ctx.step(t, dt)
            its.append(it)
            t += dt
            dt = min(dtn, dterr)
        res.append((ctx.download(), its))
        ctx.close()
    (xa, va, _), ia = res[0]
    (xb, vb, _), ib = res[1]
    assert ia == ib
    assert relmax(xa, xb) < 1.0e-12 and relmax(va, vb) < 1.0e-11


@pytest.mark.parametrize("name", ["hydro24", "sedov32", "iso_hydro20", "hydro20_leaf6", "sedov24_leaf16"])
def test_symmetric_adjoint_matches_per_side(name):
    """The adjoint's pass over the pairs on the symmetric lists (each
    unordered pair's two ordered reverse terms evaluated once, both sides
    kept, j's share gathered in list order) against the per-side pass (each
    pair reversed from both of its particles): gradients with respect to x,
    v and u within 1e-11 of their largest magnitude (summation order only),
    and bit-identical between runs."""
    cfg, x, v, B = SETS[name]()
    cfg = dict(cfg, tolh=1.0e-8)
    n = len(x)
    rng = np.random.default_rng(41)
    w = rng.standard_normal((n, 4))
    out = {}
    for sym in (1, 0):
        ctx = capi.Context(cfg)
        ctx.set_tune(force_sym=sym)
        ctx.upload(x, v, B)
        out[sym] = ctx.adjoint(w)
        if sym:
            ctx.upload(x, v, B)
            again = ctx.adjoint(w)
            assert all(np.array_equal(a, b) for a, b in zip(again, out[sym]))
    for a, b in zip(out[1], out[0]):
        assert relmax(a, b) <= 1.0e-11, (name, relmax(a, b))
