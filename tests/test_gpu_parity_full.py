"""GPU parity against the CPU oracle at the benchmark sizes, through the C ABI.

The four particle sets of the benchmark at their full sizes:

* hydro 64^3 = 262,144 particles (adiabatic, alpha=1, beta=2, alpha_u=1):
  one density + force evaluation, then 10 leapfrog steps;
* Sedov 128^3 = 2,097,152 particles (h varies by > 10x across the blast);
* ideal MHD 128^3 with hyperbolic/parabolic cleaning;
* the self-gravitating isothermal cloud of 2^21 particles (tree gravity,
  theta = 0.5, quadrupoles, adaptive softening).

Bars (the same as the small-set parity tests): tree permutation
(inodeparts) and periodic wrap identical; per-particle neighbour counts and
neighbour-set hashes identical; every neighbour statistic equal; h within
1e-12 relative; gradh (float32) within one float ulp; accelerations, du/dt,
dB/dt and dpsi/dt within 1e-10 of their largest magnitude; the potential
(float32) within 1e-6; dtcourant and dtforce within 1e-12; leapfrog steps
with the same velocity-iteration counts and positions, velocities and B
within 1e-10. At these sizes the tree has nodes of more than 2048 particles,
whose centre-of-mass sums are blocked on the GPU, and far deeper trees than
the small sets reach.

The mixed-precision form is compared with the FP64 oracle too: accelerations
and du/dt within 1e-5 of their largest magnitude. The h-rho solve stops at
the reference's tolh = 1e-4; a particle whose stopping test lies within the
FP32 rounding of the density sums stops one Newton-Raphson step apart in the
two forms, which moves h inside the tolerance band. The bar therefore holds
over all particles with the solve converged to tolh = 1e-7 in both, and at
tolh = 1e-4 for every particle outside the neighbourhood of such a particle
(their number is reported and bounded).

The oracle runs with OpenMP over leaf cells on every host core; its results
do not depend on the thread count.
"""
import os

import numpy as np
import pytest

from oracle import oracle as O
from phantom_gb300 import capi
from phantom_gb300 import setups as S

pytestmark = pytest.mark.gpu

CONFIGS = {
    "hydro64": (lambda: S.hydro_lattice(64), 10),
    "sedov128": (lambda: S.sedov(128), 1),
    "mhd128": (lambda: S.mhd_vortex(128), 1),
    "cloud2m": (lambda: S.gravity_cloud(2 ** 21), 1),
}
NTHREADS = os.cpu_count() or 1
_cache = {}


def relmax(a, b):
    s = np.abs(b).max()
    return 0.0 if s == 0.0 else float(np.abs(a - b).max() / s)


@pytest.fixture(scope="module", autouse=True)
def _build():
    O.build()
    capi.lib()


def _run(name):
    """Oracle and GPU FP64 results of one set: tree, density with neighbour
    diagnostics, one derivs, then the set's leapfrog steps."""
    if name in _cache:
        return _cache[name]
    _cache.clear()  # one full-size set in memory at a time
    mk, nsteps = CONFIGS[name]
    cfg, x, v, B = mk()
    r = {"cfg": cfg, "x": x, "v": v, "B": B, "nsteps": nsteps}
    o = O.Oracle(cfg, nthreads=NTHREADS)
    o.set_particles(x, v, B)
    o.maketree()
    r["o_perm"] = o.get_tree()["inodeparts"]
    o.densityiterate(1)
    r["o_dens"] = o.get_density()
    r["o_x"] = o.get_particles()[0]
    ctx = capi.Context(cfg)
    ctx.upload(x, v, B)
    xw, perm, _ = ctx.build_tree()
    r["g_perm"], r["g_xwrap"] = perm, xw
    r["g_dens"] = ctx.densityiterate(1)
    # one derivs (tree, density, force), then the leapfrog steps
    dto = o.derivs(1, 0.0)
    r["o_force"] = o.get_force()
    r["o_h"] = o.get_particles()[0][:, 3].copy()
    dtg = ctx.derivs(1, 0.0)
    r["g_force"] = ctx.force(2, 0.0)
    r["dt"] = (dto, dtg)
    # the mixed form through the same calls from the same input
    cm = capi.Context(cfg, precision=capi.PH_PREC_MIXED)
    cm.upload(x, v, B)
    cm.build_tree()
    cm.densityiterate(1, outputs=False)
    cm.derivs(1, 0.0)
    r["m_force"] = cm.force(2, 0.0)["fxyzu"]
    r["m_h"] = cm.download()[0][:, 3].copy()
    cm.close()
    steps = []
    t, dt = 0.0, dto
    for _ in range(nsteps):
        dto_n, itso, dterro = o.step(t, dt)
        dtg_n, itsg, dterrg = ctx.step(t, dt)
        xo, vo, bo = o.get_particles()
        xg, vg, bg = ctx.download()
        steps.append(dict(o=(dto_n, itso, dterro), g=(dtg_n, itsg, dterrg),
                          ex=relmax(xg, xo), ev=relmax(vg[:, :3], vo[:, :3]),
                          eu=relmax(vg[:, 3], vo[:, 3]) if vo[:, 3].any() else 0.0,
                          eb=relmax(bg, bo) if cfg["mhd"] else 0.0))
        t += dt
        dt = min(dto_n, dterro)
    r["steps"] = steps
    o.close()
    ctx.close()
    _cache[name] = r
    return r


@pytest.mark.parametrize("name", list(CONFIGS))
def test_full_tree_and_neighbours(name):
    r = _run(name)
    assert np.array_equal(r["g_perm"], r["o_perm"])
    assert np.array_equal(r["g_xwrap"][:, :3], r["o_x"][:, :3])  # periodic wrap identical
    dg, do = r["g_dens"], r["o_dens"]
    assert np.array_equal(dg["nneigh"], do["nneigh"])
    assert np.array_equal(dg["neighhash"], do["neighhash"])
    for k in ("nneightry", "nneighact", "maxneightry", "maxneighact", "ncalc", "np", "ncalls_neigh",
              "ncells", "maxlevel", "minlevel"):
        assert dg["stats"][k] == do["stats"][k], k
    assert relmax(dg["xyzh"][:, 3], r["o_x"][:, 3]) < 1.0e-12
    gr = np.abs(dg["gradh"][:, 0].astype(np.float64) / do["gradh"][:, 0] - 1.0).max()
    assert gr <= 2.0 ** -23
    if do["divcurlB"].any():
        assert relmax(dg["divcurlB"].astype(np.float64), do["divcurlB"].astype(np.float64)) < 1.0e-5


@pytest.mark.parametrize("name", list(CONFIGS))
def test_full_force(name):
    r = _run(name)
    fo, fg = r["o_force"], r["g_force"]
    dto, dtg = r["dt"]
    assert abs(dtg / dto - 1.0) < 1.0e-12
    for c in range(4):
        assert relmax(fg["fxyzu"][:, c], fo["fxyzu"][:, c]) < 1.0e-10, c
        assert relmax(fg["dBevol"][:, c], fo["dBevol"][:, c]) < 1.0e-10, c
    assert abs(fg["dtcourant"] / fo["dtcourant"] - 1.0) < 1.0e-12
    assert abs(fg["dtforce"] / fo["dtforce"] - 1.0) < 1.0e-12
    if r["cfg"]["gravity"]:
        assert relmax(fg["poten"].astype(np.float64), fo["poten"].astype(np.float64)) < 1.0e-6
    m = r["cfg"]["massoftype"]
    tg = (m * fg["fxyzu"][:, :3]).sum(axis=0)
    to = (m * fo["fxyzu"][:, :3]).sum(axis=0)
    scale = m * np.abs(fo["fxyzu"][:, :3]).sum()
    # total force: the same as the oracle's; for hydro the pair terms are
    # antisymmetric, so it vanishes to rounding (with MHD the div B source-term
    # subtraction, force.F90:2942-2957, and with gravity the far field's
    # truncation are not momentum conserving in the reference either)
    assert np.abs(tg - to).max() < 1.0e-10 * scale
    if not (r["cfg"]["gravity"] or r["cfg"]["mhd"]):
        assert np.abs(tg).max() < 1.0e-12 * scale


@pytest.mark.parametrize("name", list(CONFIGS))
def test_full_leapfrog_steps(name):
    r = _run(name)
    assert len(r["steps"]) == r["nsteps"]
    for k, s in enumerate(r["steps"]):
        (dto, itso, _), (dtg, itsg, _) = s["o"], s["g"]
        assert itso == itsg, k
        assert abs(dtg / dto - 1.0) < 1.0e-10, k
        for key in ("ex", "ev", "eu", "eb"):
            assert s[key] < 1.0e-10, (k, key, s[key])


def _mixed_forces(cfg, x, v, B):
    ctx = capi.Context(cfg, precision=capi.PH_PREC_MIXED)
    ctx.upload(x, v, B)
    ctx.derivs(1, 0.0)
    f = ctx.force(2, 0.0)["fxyzu"]
    ctx.close()
    return f


@pytest.mark.parametrize("name", list(CONFIGS))
def test_full_mixed_against_oracle(name):
    r = _run(name)
    cfg, x, v, B = r["cfg"], r["x"], r["v"], r["B"]
    fo = r["o_force"]["fxyzu"]
    ho, hm, fm = r["o_h"], r["m_h"], r["m_force"]
    ncomp = 4 if not cfg["isothermal"] else 3
    err = np.array([relmax(fm[:, c], fo[:, c]) for c in range(ncomp)])
    # particles whose h-rho solve stopped one iteration apart in the two forms
    flipped = np.abs(hm / ho - 1.0) > 1.0e-6
    nflip = int(flipped.sum())
    assert nflip <= 1.0e-4 * len(x), nflip
    if nflip == 0:
        assert err.max() < 1.0e-5, err
        return
    # the bar over the particles not affected by a flipped h (a flipped
    # particle moves the forces of every particle within 2 h of it) ...
    from scipy.spatial import cKDTree
    box = None
    if cfg["periodic"]:
        box = np.array([cfg["xmax"] - cfg["xmin"], cfg["ymax"] - cfg["ymin"], cfg["zmax"] - cfg["zmin"]])
        lo = np.array([cfg["xmin"], cfg["ymin"], cfg["zmin"]])
        pos = np.mod(r["o_x"][:, :3] - lo, box)
    else:
        pos = r["o_x"][:, :3]
    tree = cKDTree(pos, boxsize=box)
    hmax = float(ho.max())
    near = np.zeros(len(x), bool)
    for k in np.nonzero(flipped)[0]:
        cand = np.asarray(tree.query_ball_point(pos[k], 2.0 * max(ho[k], hmax) * 1.01), dtype=np.int64)
        d = pos[cand] - pos[k]
        if box is not None:
            d -= box * np.round(d / box)
        r = np.sqrt((d * d).sum(axis=1))
        near[cand[r < 2.0 * np.maximum(ho[k], ho[cand]) * 1.01]] = True
    keep = ~near
    for c in range(ncomp):
        s = np.abs(fo[:, c]).max()
        assert np.abs(fm[keep, c] - fo[keep, c]).max() < 1.0e-5 * s, c
    # ... and over all particles with the solve converged in both forms
    tight = dict(cfg, tolh=1.0e-7)
    o = O.Oracle(tight, nthreads=NTHREADS)
    o.set_particles(x, v, B)
    o.derivs(1, 0.0)
    fo7 = o.get_force()["fxyzu"]
    o.close()
    fm7 = _mixed_forces(tight, x, v, B)
    err7 = np.array([relmax(fm7[:, c], fo7[:, c]) for c in range(ncomp)])
    assert err7.max() < 1.0e-5, err7
