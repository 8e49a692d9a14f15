"""Leaf size and launch configuration (ph_autotune, ph_set_tune).

* Warps per block (1, 2 or 4) regroup leaf cells into blocks and change no
  arithmetic: every output is bit-identical across configurations.
* A leaf size other than the reference's minpart = 10 builds a different
  tree; the GPU path reproduces the oracle built with the same leaf size
  (tree permutation, neighbour counts and hashes bit-exact, h to 1e-12,
  accelerations to 1e-10, as in the default-leaf parity tests).
* ph_autotune leaves the context as after the upload: a derivs after tuning
  equals one on a fresh context with the chosen configuration.
"""
import numpy as np
import pytest

from oracle import oracle as O
from phantom_gb300 import capi
from phantom_gb300 import setups as S

pytestmark = pytest.mark.gpu


def relmax(a, b):
    s = np.abs(b).max()
    return 0.0 if s == 0.0 else np.abs(a - b).max() / s


def _derivs(ctx, x, v, B=None):
    ctx.upload(x, v, B)
    ctx.derivs(1, 0.0)
    f = ctx.force(2, 0.0)
    d = ctx.densityiterate(1)  # a re-solve from the converged h: outputs of the same state
    return f, d


@pytest.mark.parametrize("prec", [capi.PH_PREC_FP64, capi.PH_PREC_MIXED])
def test_warps_per_block_change_no_bit(prec):
    cfg, x, v, B = S.sedov(24)
    ref = None
    for dw, fw, ww in [(4, 4, 2), (1, 1, 1), (2, 4, 4), (4, 2, 1)]:
        ctx = capi.Context(cfg, precision=prec)
        ctx.set_tune(dens_warps=dw, force_warps=fw, walk_warps=ww)
        t = ctx.tune()
        assert (t["dens_warps"], t["force_warps"], t["walk_warps"]) == (dw, fw, ww)
        f, d = _derivs(ctx, x, v)
        ctx.close()
        if ref is None:
            ref = (f, d)
            continue
        assert np.array_equal(f["fxyzu"], ref[0]["fxyzu"])
        assert np.array_equal(f["divcurlv"], ref[0]["divcurlv"])
        assert np.array_equal(d["xyzh"], ref[1]["xyzh"])
        assert np.array_equal(d["neighhash"], ref[1]["neighhash"])


@pytest.mark.parametrize("minpart", [6, 16])
@pytest.mark.parametrize("name", ["sedov", "mhd", "grav"])
def test_leaf_size_parity_with_oracle(minpart, name):
    cfg, x, v, B = {"sedov": lambda: S.sedov(24), "mhd": lambda: S.mhd_vortex(16),
                    "grav": lambda: S.gravity_cloud(5000)}[name]()
    cfg = dict(cfg)
    cfg["minpart"] = minpart
    o = O.Oracle(cfg, nthreads=8)
    o.set_particles(x, v, B)
    ctx = capi.Context(cfg)
    assert ctx.tune()["minpart"] == minpart
    ctx.upload(x, v, B)
    o.maketree()
    t = o.get_tree()
    leaves = t["inoderange"][t["leaf_is_active"] > 0]
    assert (leaves[:, 1] - leaves[:, 0] + 1).max() <= minpart
    _, perm, _ = ctx.build_tree()
    assert np.array_equal(perm, t["inodeparts"])
    o.densityiterate(1)
    do = o.get_density()
    xo, _, _ = o.get_particles()
    dg = ctx.densityiterate(1)
    assert np.array_equal(dg["nneigh"], do["nneigh"])
    assert np.array_equal(dg["neighhash"], do["neighhash"])
    assert dg["stats"]["nneightry"] == do["stats"]["nneightry"]
    assert relmax(dg["xyzh"][:, 3], xo[:, 3]) < 1.0e-12
    o.set_particles(x, v, B)
    ctx.upload(x, v, B)
    o.derivs(1, 0.0)
    fo = o.get_force()
    ctx.derivs(1, 0.0)
    fg = ctx.force(2, 0.0)
    for c in range(4):
        assert relmax(fg["fxyzu"][:, c], fo["fxyzu"][:, c]) < 1.0e-10, c


def test_autotune_restores_state_and_keeps_results():
    cfg, x, v, B = S.sedov(32)
    ctx = capi.Context(cfg, precision=capi.PH_PREC_MIXED)
    ctx.upload(x, v)
    t = ctx.autotune()
    assert t["minpart"] == 10
    for k in ("dens_warps", "force_warps", "walk_warps"):
        assert t[k] in (1, 2, 4)
    assert t["ms_before"] > 0.0 and t["ms_after"] > 0.0
    dt_tuned = ctx.derivs(1, 0.0)  # straight after tuning: the uploaded state
    f_tuned = ctx.force(2, 0.0)
    fresh = capi.Context(cfg, precision=capi.PH_PREC_MIXED)
    fresh.upload(x, v)
    assert fresh.derivs(1, 0.0) == dt_tuned
    assert np.array_equal(fresh.force(2, 0.0)["fxyzu"], f_tuned["fxyzu"])


def test_autotune_leaf_size_on_request():
    cfg, x, v, B = S.sedov(24)
    ctx = capi.Context(cfg, precision=capi.PH_PREC_MIXED)
    ctx.upload(x, v)
    t = ctx.autotune(leaf=True)
    assert t["minpart"] in (6, 8, 10, 12, 16)
    # the chosen leaf size is the one the context now builds with
    o = O.Oracle(dict(cfg, minpart=t["minpart"]), nthreads=8)
    o.set_particles(x, v)
    o.maketree()
    _, perm, _ = ctx.build_tree()
    assert np.array_equal(perm, o.get_tree()["inodeparts"])


def test_set_tune_rejects_out_of_range():
    cfg, x, v, B = S.sedov(12)
    ctx = capi.Context(cfg)
    for bad in (dict(dens_warps=0), dict(force_warps=8), dict(walk_warps=3), dict(minpart=1), dict(minpart=17)):
        with pytest.raises(capi.PhantomError) as e:
            ctx.set_tune(**bad)
        assert e.value.code == 1
    with pytest.raises(capi.PhantomError):
        capi.Context(dict(cfg, minpart=20))
