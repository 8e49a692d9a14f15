"""Individual timesteps (ind_timesteps = 1) on the GPU against the oracle,
through the C ABI.

* Substep parity (FP64 path): over 24 substeps of a Sedov blast (the bins
  spread over several levels) the bins, nbinmax, istepfrac, ibinnow and the
  number of particles updated agree exactly with the oracle; twas and the
  time to 1e-14 of dtmax; positions and velocities to 1e-9 of their scale
  (the FP64 pair sums in another order, the GPU's fused multiply-adds in the
  kicks). Without and with the Cullen & Dehnen switch; ideal MHD and
  self-gravity over 16 substeps (B to 1e-9 as well).
* Known answer: the reference's Sedov test (test_sedov.f90:88-193, individual
  timesteps, dtmax = tmax = 0.1) conserves total energy to the extracted
  tolerance and linear momentum to 7e-15 on the GPU's FP64 path; the mixed
  form conserves energy to the same tolerance and momentum to 1e-5 of
  sum m |v| (its FP32 pair terms are not exactly antisymmetric).
* One bin: with every particle in one bin a substep is the global leapfrog
  step (ph_step) to 1e-12.
* The mixed form over the same substeps: bins agree for at least 99% of the
  particles and positions stay within 1e-5 of the FP64 path.
"""
import numpy as np
import pytest

from known_answers import KA
from oracle import oracle as O
from phantom_gb300 import capi
from phantom_gb300 import setups as S

pytestmark = pytest.mark.gpu


def _scale(a):
    return max(float(np.abs(a).max()), 1.0e-300)


def _start(cfg, x, v, B=None, precision=capi.PH_PREC_FP64):
    ctx = capi.Context(cfg, precision=precision)
    ctx.upload(x, v, B)
    ctx.derivs(1, 0.0)
    if cfg.get("nalpha", 0) >= 2:
        ctx.alpha_initial()
    ctx.ind_init(0.0)
    return ctx


def _sedov_ind(n1d=12, nalpha=0):
    cfg, x, v, B = S.sedov(n1d)
    cfg = dict(cfg, ind_timesteps=1, dtmax=0.02)
    if nalpha:
        cfg.update(nalpha=3, alpha=0.0, alphamax=1.0)
    return cfg, x, v


def _parity(cfg, x, v, B=None, nsub=24):
    o = O.Oracle(cfg, nthreads=8)
    o.set_particles(x, v, B)
    o.derivs(1, 0.0)
    if cfg.get("nalpha", 0):
        o.alpha_initial()
    o.ind_init(0.0)
    ctx = _start(cfg, x, v, B)
    b_o, tw_o, c_o = o.ind_state()
    b_g, tw_g, c_g = ctx.ind_state()
    assert c_g == c_o and (b_g == b_o).all()
    t_o = t_g = 0.0
    seen = set()
    for k in range(nsub):
        t_o, na_o = o.ind_substep(t_o)
        t_g, na_g = ctx.ind_substep(t_g)
        b_o, tw_o, c_o = o.ind_state()
        b_g, tw_g, c_g = ctx.ind_state()
        assert na_g == na_o, k
        assert c_g == c_o, k
        assert (b_g == b_o).all(), (k, int(np.sum(b_g != b_o)))
        assert abs(t_g - t_o) <= 1.0e-14 * cfg["dtmax"], k
        assert np.abs(tw_g - tw_o).max() <= 1.0e-14 * cfg["dtmax"], k
        seen.update(np.unique(b_g).tolist())
    xo, vo, Bo = o.get_particles()
    xg, vg, Bg = ctx.download()
    assert np.abs(xg[:, :3] - xo[:, :3]).max() <= 1.0e-9 * _scale(xo[:, :3])
    assert np.abs(xg[:, 3] - xo[:, 3]).max() <= 1.0e-9 * _scale(xo[:, 3])
    assert np.abs(vg - vo).max() <= 1.0e-9 * _scale(vo)
    if cfg["mhd"]:
        assert np.abs(Bg - Bo).max() <= 1.0e-9 * _scale(Bo)
    assert len(seen) > 1  # several bins were in use


@pytest.mark.parametrize("nalpha", [0, 3])
def test_substeps_match_oracle(nalpha):
    cfg, x, v = _sedov_ind(12, nalpha)
    _parity(cfg, x, v)


@pytest.mark.parametrize("name", ["mhd", "grav"])
def test_substeps_match_oracle_mhd_gravity(name):
    """Ideal MHD with cleaning (B and psi kicked through twas) and
    self-gravity (far field on every leaf, near field on the active cells),
    dtmax = 16 x the first global step: bins over three levels."""
    cfg, x, v, B = S.mhd_vortex(10) if name == "mhd" else S.gravity_cloud(3000)
    c0 = capi.Context(cfg)
    c0.upload(x, v, B)
    dt = c0.derivs(1, 0.0)
    c0.close()
    _parity(dict(cfg, ind_timesteps=1, dtmax=16.0 * dt), x, v, B, nsub=16)


@pytest.mark.parametrize("precision", [capi.PH_PREC_FP64, capi.PH_PREC_MIXED])
@pytest.mark.parametrize("nalpha", [0, 3])
def test_sedov_known_answer_gpu(precision, nalpha):
    cfg, x, v, B = S.sedov_test(16)
    tmax = KA["sedov_tmax"]["value"]
    cfg = dict(cfg, ind_timesteps=1, dtmax=tmax, nalpha=nalpha, alpha=0.0 if nalpha else cfg["alpha"],
               alphamax=1.0)
    ctx = _start(cfg, x, v, precision=precision)
    m = cfg["massoftype"]

    def energy():
        _, vv, _ = ctx.download()
        return float(np.sum(0.5 * m * np.sum(vv[:, :3] ** 2, axis=1)) + np.sum(m * vv[:, 3])), vv

    e0, _ = energy()
    t = 0.0
    nsub = 0
    while t < tmax * (1.0 - 1.0e-12):
        t, _ = ctx.ind_substep(t)
        nsub += 1
        assert nsub < 100000
    e1, vv = energy()
    assert abs(e1 / e0 - 1.0) <= KA["sedov_energy_tol"]["value"]
    mom = np.abs(np.sum(m * vv[:, :3], axis=0)).max()
    if precision == capi.PH_PREC_FP64:
        assert mom <= KA["sedov_momentum_tol"]["value"]
    else:
        # FP32 pair terms are not exactly antisymmetric: the precision form's
        # 1e-5 per-term bound, on the momentum scale sum m |v|
        assert mom <= 1.0e-5 * float(np.sum(m * np.linalg.norm(vv[:, :3], axis=1)))
    b, _, _ = ctx.ind_state()
    assert len(np.unique(b)) > 1


def test_one_bin_is_the_global_leapfrog_gpu():
    cfg, x, v, B = S.hydro_lattice(10, vamp=0.01)
    cfg = dict(cfg, tolv=1.0e3, dtmax=2.0e-3)
    ci = _start(dict(cfg, ind_timesteps=1), x, v)
    b, _, (nbinmax, _, _) = ci.ind_state()
    assert (b == nbinmax).all()
    dt = cfg["dtmax"] / 2 ** nbinmax
    cg = capi.Context(cfg)
    cg.upload(x, v)
    cg.derivs(1, 0.0)
    t = 0.0
    for _ in range(4):
        t, na = ci.ind_substep(t)
        assert na == len(x)
        cg.step(t - dt, dt)
        b, _, (nb, _, _) = ci.ind_state()
        if (b != nb).any() or nb != nbinmax:
            pytest.skip("bins changed during the comparison")
    xi, vi, _ = ci.download()
    xg, vg, _ = cg.download()
    assert np.abs(xi[:, :3] - xg[:, :3]).max() < 1.0e-12
    assert np.abs(vi - vg).max() < 1.0e-12 * max(np.abs(vg).max(), 1.0)


def test_mixed_substeps_track_fp64():
    cfg, x, v = _sedov_ind(12)
    c64 = _start(cfg, x, v)
    c32 = _start(cfg, x, v, precision=capi.PH_PREC_MIXED)
    t64 = t32 = 0.0
    for _ in range(16):
        t64, _ = c64.ind_substep(t64)
        t32, _ = c32.ind_substep(t32)
    b64, _, _ = c64.ind_state()
    b32, _, _ = c32.ind_state()
    assert np.mean(b64 == b32) >= 0.99
    x64, _, _ = c64.download()
    x32, _, _ = c32.download()
    assert np.abs(x32[:, :3] - x64[:, :3]).max() <= 1.0e-5 * _scale(x64[:, :3])


def test_ind_entry_points_reject_global_timesteps():
    cfg, x, v, B = S.sedov(8)
    ctx = capi.Context(cfg)
    ctx.upload(x, v)
    ctx.derivs(1, 0.0)
    with pytest.raises(capi.PhantomError) as e:
        ctx.ind_init(0.0)
    assert e.value.code == 1  # PH_ERR_ARG


def test_dt_too_small_stops_before_the_corrector():
    """A timestep below dtmax / 2^30 (step_leapfrog.f90:427-433, fatal before
    the corrector): dtmax = 2^34 x the particles' step. The GPU refuses the
    substep with PH_ERR_IND_DT and leaves the velocities uncorrected; the
    oracle stops with its status 42."""
    cfg, x, v, B = S.sedov(8)
    c0 = capi.Context(cfg)
    c0.upload(x, v)
    dt = c0.derivs(1, 0.0)
    c0.close()
    cfg = dict(cfg, ind_timesteps=1, dtmax=dt * 2.0 ** 34)
    ctx = _start(cfg, x, v)
    with pytest.raises(capi.PhantomError) as e:
        ctx.ind_substep(0.0)
    assert e.value.code == capi.PH_ERR_IND_DT
    o = O.Oracle(cfg, nthreads=4)
    o.set_particles(x, v)
    o.derivs(1, 0.0)
    o.ind_init(0.0)
    with pytest.raises(RuntimeError, match="status 42"):
        o.ind_substep(0.0)


def test_substeps_match_oracle_rectangular_box():
    """Individual timesteps in the rectangular periodic box [0,1) x [0,0.5) x
    [0,0.25) (each axis its own periodic image), with a hot spot (u up to 21)
    that spreads the bins; dtmax = 16 x the first global step."""
    from test_gpu_parity_combos import rect_box
    cfg, x, v, B = rect_box()
    v = v.copy()
    r2 = (x[:, 0] - 0.5) ** 2 + (x[:, 1] - 0.25) ** 2 + (x[:, 2] - 0.125) ** 2
    v[:, 3] = 1.0 + 20.0 * np.exp(-r2 / 0.1 ** 2)
    c0 = capi.Context(cfg)
    c0.upload(x, v, B)
    dt = c0.derivs(1, 0.0)
    c0.close()
    _parity(dict(cfg, ind_timesteps=1, dtmax=16.0 * dt), x, v, B, nsub=16)
