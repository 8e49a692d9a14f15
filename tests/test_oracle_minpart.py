"""The oracle's leaf size (minpart, a compile-time constant of the reference,
config.F90:113): leaves hold at most minpart particles, the default is the
reference's 10, and the physics does not depend on it beyond rounding (the
neighbour sets are the same; only the trial lists and summation order change)."""
import numpy as np
import pytest

from oracle import oracle as O
from phantom_gb300 import setups as S


def _run(cfg, x, v, minpart):
    c = dict(cfg)
    if minpart is not None:
        c["minpart"] = minpart
    o = O.Oracle(c, nthreads=4)
    o.set_particles(x, v)
    o.maketree()
    t = o.get_tree()
    o.densityiterate(1)
    d = o.get_density()
    xo, _, _ = o.get_particles()
    o.set_particles(x, v)
    o.derivs(1, 0.0)
    return t, d, xo, o.get_force()


def test_default_is_the_reference_leaf_size():
    cfg, x, v, _ = S.hydro_lattice(10)
    t0, d0, x0, f0 = _run(cfg, x, v, None)
    t1, d1, x1, f1 = _run(cfg, x, v, 10)
    assert np.array_equal(t0["inodeparts"], t1["inodeparts"])
    assert np.array_equal(f0["fxyzu"], f1["fxyzu"])


@pytest.mark.parametrize("minpart", [4, 6, 16])
def test_leaf_size_changes_only_rounding(minpart):
    cfg, x, v, _ = S.hydro_lattice(10)
    t0, d0, x0, f0 = _run(cfg, x, v, 10)
    t1, d1, x1, f1 = _run(cfg, x, v, minpart)
    leaves = t1["inoderange"][t1["leaf_is_active"] > 0]
    assert (leaves[:, 1] - leaves[:, 0] + 1).max() <= minpart
    assert np.array_equal(d1["nneigh"], d0["nneigh"])
    assert np.array_equal(d1["neighhash"], d0["neighhash"])
    assert np.abs(x1[:, 3] / x0[:, 3] - 1.0).max() < 1.0e-12
    s = np.abs(f0["fxyzu"][:, :3]).max()
    assert np.abs(f1["fxyzu"][:, :3] - f0["fxyzu"][:, :3]).max() / s < 1.0e-10


def test_invalid_leaf_size_rejected():
    cfg, x, v, _ = S.hydro_lattice(4)
    for bad in (1, 17):
        with pytest.raises(ValueError):
            O.Oracle(dict(cfg, minpart=bad))
