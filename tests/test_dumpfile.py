"""The dump format (phantom_gb300/dumpfile.py) against the fixture that the
reference's own reader parsed (tests/golden/make_dump_golden.py):

* the writer reproduces the committed dump byte for byte;
* our reader finds in it what the reference's reader found (file id, header
  quantities by tag, block lengths, array names, counts and values);
* round trips of every data type, single-precision files, iorig (int*4)
  arrays, and the rejection of files that are not tagged Phantom dumps;
* a full dump restarts a run: the oracle's derivs on the state read back
  equals derivs on the state written (h as real*4, B through rho(h)).
"""
import json
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))

from make_dump_golden import golden_dump  # noqa: E402
from phantom_gb300 import dumpfile as D  # noqa: E402

FIX = os.path.join(HERE, "golden", "mhd_vortex4_00000")
REF = json.load(open(FIX + ".json"))


def test_writer_reproduces_fixture_bytes(tmp_path):
    p = str(tmp_path / "d_00000")
    golden_dump(p)
    assert open(p, "rb").read() == open(FIX, "rb").read()


def test_reader_agrees_with_reference_reader():
    d = D.read(FIX)
    assert d.fileid.strip() == REF["desc"]
    for k, v in REF["quantities"].items():
        got = d.get(k, all_values=True)
        assert np.allclose(np.asarray(got if len(got) > 1 else got[0]), v, rtol=0, atol=0), k
    for k, v in REF["units"].items():
        assert d.get(k) == v
    assert d.get("nparttot") == REF["part_numbers"]["nparttot"]
    assert d.get("npartoftype", all_values=True) == REF["part_numbers"]["npartoftype"]
    assert len(d.blocks) == len(REF["blocks"])
    for (length, arrs), rb in zip(d.blocks, REF["blocks"]):
        assert length == rb["dim"]
        assert len(arrs.get("int8", [])) == rb["nintdb"]
        assert len(arrs.get("real", [])) == rb["ndouble"]
        assert len(arrs.get("real4", [])) == rb["nsingle"]
        ours = {k: a for t in ("int8", "real", "real4") for k, a in arrs.get(t, [])}
        assert set(ours) == set(rb["data"])
        for k, a in ours.items():
            assert np.array_equal(a.astype(np.float64), np.asarray(rb["data"][k])), k


def test_round_trip_every_type_and_single_precision(tmp_path):
    n = 7
    rng = np.random.default_rng(1)
    hdr = {t: [] for t in D.TYPES}
    hdr["int"] = [("a", 3), ("b", -4)]
    hdr["int1"] = [("c", 5)]
    hdr["int2"] = [("d", -300)]
    hdr["int4"] = [("e", 70000)]
    hdr["int8"] = [("f", 2 ** 40)]
    hdr["real"] = [("g", 0.125), ("g", 0.5)]
    hdr["real4"] = [("h", 1.5)]
    hdr["real8"] = [("udist", 3.0e10)]
    arrs = {"int1": [("i1", np.arange(n, dtype=np.int8))], "int4": [("iorig", np.arange(n, dtype=np.int32) + 1)],
            "int8": [("i8", np.arange(n, dtype=np.int64) * 2 ** 33)],
            "real": [("x", rng.standard_normal(n))], "real4": [("h", rng.random(n).astype(np.float32))]}
    d = D.Dump("FT:test", hdr, [(n, arrs), (0, {})])
    p = str(tmp_path / "rt")
    D.write(p, d)
    r = D.read(p)
    assert r.fileid == "FT:test"
    for t in D.TYPES:
        assert [k for k, _ in r.header[t]] == [k for k, _ in hdr[t]]
        assert np.allclose([v for _, v in r.header[t]], [v for _, v in hdr[t]])
    assert r.get("g", all_values=True) == [0.125, 0.5]
    for t, lst in arrs.items():
        for (k, a), (k2, b) in zip(lst, r.blocks[0][1][t]):
            assert k == k2 and np.array_equal(a, b)
    # 4-byte default reals (the reference's singleprec files)
    q = str(tmp_path / "sp")
    D.write(q, d, singleprec=True)
    s = D.read(q)
    assert s.real == "<f4" and s.get("g", all_values=True) == [0.125, 0.5]
    assert s.get("udist") == 3.0e10  # real*8 stays double
    assert np.array_equal(s.blocks[0][1]["real"][0][1], arrs["real"][0][1].astype(np.float32))


def test_rejects_what_is_not_a_tagged_dump(tmp_path):
    p = str(tmp_path / "bad")
    open(p, "wb").write(b"\x00" * 64)
    with pytest.raises(D.DumpError):
        D.read(p)
    raw = bytearray(open(FIX, "rb").read())
    raw[4:8] = np.array([12345], "<i4").tobytes()  # int1 of the magic record
    open(p, "wb").write(bytes(raw))
    with pytest.raises(D.DumpError, match="endian"):
        D.read(p)


def test_restart_from_dump_reproduces_derivs(tmp_path):
    from oracle import oracle as O
    from phantom_gb300 import setups as S
    cfg, x, v, B = S.mhd_vortex(6)
    p = str(tmp_path / "r_00000")
    iorig = np.arange(1, len(x) + 1, dtype=np.int32)
    D.write_fulldump(p, cfg, 0.0, x, v, B, iorig=iorig)
    # the dump carries the header parameters; the rest come from the input
    # file on a restart, here cfg without the keys the dump carries
    carried = ("hfact", "tolh", "C_cour", "C_force", "alpha", "alphau", "alphaB", "massoftype", "gamma",
               "xmin", "xmax", "ymin", "ymax", "zmin", "zmax", "ieos", "polyk", "mhd", "periodic", "isothermal")
    infile = {k: val for k, val in cfg.items() if k not in carried}
    c2, t, x2, v2, B2 = D.read_fulldump(p, infile)
    assert D.read(p).arrays(1)["iorig"].tolist() == iorig.tolist()
    for k in carried:
        assert c2[k] == cfg[k] or abs(c2[k] - cfg[k]) <= 1e-15 * abs(cfg[k]), k
    # h went through real*4 and B through rho(h): both runs start from the dump's state
    o1 = O.Oracle(cfg, nthreads=4)
    o1.set_particles(x2, v2, B2)
    o1.derivs(1, 0.0)
    o2 = O.Oracle(c2, nthreads=4)
    o2.set_particles(x2, v2, B2)
    o2.derivs(1, 0.0)
    assert np.array_equal(o2.get_force()["fxyzu"], o1.get_force()["fxyzu"])
    assert np.abs(x2[:, 3] / x[:, 3] - 1.0).max() <= 2.0 ** -24


def test_alpha_array_round_trip(tmp_path):
    from phantom_gb300 import setups as S
    cfg, x, v, B = S.hydro_lattice(6)
    alpha = np.linspace(0.0, 1.0, len(x)).astype(np.float32)
    p = str(tmp_path / "a_00000")
    D.write_fulldump(p, dict(cfg, nalpha=3), 0.0, x, v, alpha=alpha)
    *_, a2 = D.read_fulldump(p, cfg, with_alpha=True)
    assert np.array_equal(a2, alpha)
    q = str(tmp_path / "n_00000")
    D.write_fulldump(q, cfg, 0.0, x, v)
    assert D.read_fulldump(q, cfg, with_alpha=True)[-1] is None
