"""A GPU run started from a Phantom full dump (phantom_gb300.dumpfile):
derivs on the state read back matches the oracle's on the same state, and
the GPU state after a step, written as a dump and read again, restarts with
the same forces (h and u as the dump stores them)."""
import numpy as np
import pytest

from oracle import oracle as O
from phantom_gb300 import capi
from phantom_gb300 import dumpfile as D
from phantom_gb300 import setups as S

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["sedov", "mhd"])
def test_run_from_dump_matches_oracle(name, tmp_path):
    cfg, x, v, B = {"sedov": lambda: S.sedov(16), "mhd": lambda: S.mhd_vortex(12)}[name]()
    p = str(tmp_path / "start_00000")
    D.write_fulldump(p, cfg, 0.0, x, v, B)
    c2, t, x2, v2, B2 = D.read_fulldump(p, cfg)
    ctx = capi.Context(c2)
    ctx.upload(x2, v2, B2)
    ctx.derivs(1, 0.0)
    fg = ctx.force(2, 0.0)["fxyzu"]
    o = O.Oracle(c2, nthreads=8)
    o.set_particles(x2, v2, B2)
    o.derivs(1, 0.0)
    fo = o.get_force()["fxyzu"]
    for c in range(4):
        s = np.abs(fo[:, c]).max()
        assert s == 0.0 or np.abs(fg[:, c] - fo[:, c]).max() / s < 1.0e-10, c
    # a step on the GPU, written and read back, restarts with the same forces
    dt = ctx.derivs(1, 0.0)
    ctx.step(0.0, dt)
    xs, vs, Bs = ctx.download()
    q = str(tmp_path / "next_00001")
    D.write_fulldump(q, c2, dt, xs, vs, Bs)
    c3, t3, x3, v3, B3 = D.read_fulldump(q, cfg)
    assert t3 == dt
    assert np.array_equal(x3[:, :3], xs[:, :3]) and np.array_equal(v3, vs)
    assert np.array_equal(x3[:, 3], xs[:, 3].astype(np.float32).astype(np.float64))
