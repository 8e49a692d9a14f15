"""Phantom's native dump format (utils_dumpfiles.f90, readwrite_dumps.f90):
reader and writer, so that runs of this library start from reference dumps
and write dumps that the reference's tools (phantom, splash, sarracen) read.

The format is Fortran unformatted sequential I/O: every record is framed by
its length in bytes as a 4-byte integer before and after. A file holds

* a magic record (open_dumpfile_w, utils_dumpfiles.f90:1111-1139): int*4
  060769, the default real 60878., int*4 060878, the format version (1) and
  int*4 690706; the size of the real tells single- from double-precision
  files, the integers tell the byte order;
* the file id, 100 characters; 'F' first for a full dump, 'T' second for the
  tagged format (fileident, readwrite_dumps_common.f90:32-69);
* the header (write_header, utils_dumpfiles.f90:1502-1605): for each of the 8
  data types (integer, int*1, int*2, int*4, int*8, real, real*4, real*8) a
  record with the count, and when non-zero a record of 16-character tags and
  a record of values;
* the number of array blocks, then per block a record of the block's array
  length (int*8) and its 8 per-type array counts (write_block_header,
  utils_dumpfiles.f90:1980-1991);
* the arrays, block by block, and within a block type by type, each as a
  16-character tag record and a data record (write_array_*).

Full dumps (write_fulldump, readwrite_dumps.f90:45-340) put the particle
arrays in block 1 (x, y, z, vx, vy, vz, u as real; h as real*4; alpha,
divv, poten as real*4; iorig as int*4) and the MHD arrays in block 4 (Bx, By,
Bz, psi as real; divB, curlB as real*4); the header carries the run
parameters by tag (fill_header, readwrite_dumps_common.f90:261-390).
Little-endian files with 8-byte default reals and 4-byte default integers
are written; both real sizes are read.
"""
from __future__ import annotations

import datetime
import math

import numpy as np

LENTAG = 16     # utils_dumpfiles.f90:14
LENID = 100     # utils_dumpfiles.f90:15
IVERSION = 1    # utils_dumpfiles.f90:17
INT1, INT2 = 60769, 60878          # utils_dumpfiles.f90:19 (060769, 060878)
INT1O, INT2O = 690706, 780806      # utils_dumpfiles.f90:20
MAXTYPES = 30   # part.F90 maxtypes (npartoftype header length)

# the 8 data types of the format, in file order (utils_dumpfiles.f90:22-30)
TYPES = ("int", "int1", "int2", "int4", "int8", "real", "real4", "real8")
_DT = {"int": "<i4", "int1": "<i1", "int2": "<i2", "int4": "<i4", "int8": "<i8",
       "real": "<f8", "real4": "<f4", "real8": "<f8"}


class DumpError(ValueError):
    pass


# ------------------------------------------------------------------ records
def _write_record(f, payload: bytes):
    n = np.array([len(payload)], "<i4").tobytes()
    f.write(n)
    f.write(payload)
    f.write(n)


def _read_record(f) -> bytes:
    head = f.read(4)
    if len(head) < 4:
        raise DumpError("unexpected end of file")
    n = int(np.frombuffer(head, "<i4")[0])
    if n < 0:
        raise DumpError("bad record length (byte order?)")
    data = f.read(n)
    tail = f.read(4)
    if len(data) < n or len(tail) < 4 or int(np.frombuffer(tail, "<i4")[0]) != n:
        raise DumpError("inconsistent record framing")
    return data


def _tag(s: str) -> bytes:
    b = s.encode("ascii")[:LENTAG]
    return b + b" " * (LENTAG - len(b))


def _tags(data: bytes) -> list[str]:
    if len(data) % LENTAG:
        raise DumpError("tag record length")
    return [data[k:k + LENTAG].decode("ascii").strip() for k in range(0, len(data), LENTAG)]


# ------------------------------------------------------------------ generic file
class Dump:
    """A dump file's content: the file id, the header as a list of
    (tag, value) per data type (tags may repeat: arrays in the header such as
    npartoftype are consecutive entries with one tag), and the blocks, each
    a (length, {type: [(tag, array)]}) pair in file order."""

    def __init__(self, fileid: str = "", header=None, blocks=None, real="real"):
        self.fileid = fileid
        self.header = header if header is not None else {t: [] for t in TYPES}
        self.blocks = blocks if blocks is not None else []
        self.real = real  # dtype of the default real: '<f8' or '<f4' files

    # header access (extract, utils_dumpfiles.f90)
    def get(self, tag: str, default=None, all_values: bool = False):
        for t in TYPES:
            vals = [v for (k, v) in self.header[t] if k == tag]
            if vals:
                return vals if all_values else vals[0]
        return default

    def arrays(self, block: int = 1) -> dict:
        """{tag: array} of a block (1-based, as the reference numbers them)."""
        if block > len(self.blocks):
            return {}
        out = {}
        for t in TYPES:
            for tag, a in self.blocks[block - 1][1].get(t, []):
                out[tag] = a
        return out


def write(path: str, d: Dump, singleprec: bool = False):
    """Write d (open_dumpfile_w, write_header, write_block_header,
    write_array). singleprec writes the default reals (header and arrays) as
    real*4, as the reference's singleprec option does."""
    dt = dict(_DT, real="<f4" if singleprec else "<f8")
    with open(path, "wb") as f:
        _write_record(f, np.array([INT1], "<i4").tobytes() + np.array([float(INT2)], dt["real"]).tobytes()
                      + np.array([INT2, IVERSION, INT1O], "<i4").tobytes())
        fid = d.fileid.encode("ascii")[:LENID]
        _write_record(f, fid + b" " * (LENID - len(fid)))
        for t in TYPES:
            entries = d.header.get(t, [])
            _write_record(f, np.array([len(entries)], "<i4").tobytes())
            if entries:
                _write_record(f, b"".join(_tag(k) for k, _ in entries))
                _write_record(f, np.array([v for _, v in entries], dt[t]).tobytes())
        _write_record(f, np.array([len(d.blocks)], "<i4").tobytes())
        for length, arrs in d.blocks:
            nums = [len(arrs.get(t, [])) for t in TYPES]
            _write_record(f, np.array([length], "<i8").tobytes() + np.array(nums, "<i4").tobytes())
        for length, arrs in d.blocks:
            for t in TYPES:
                for tag, a in arrs.get(t, []):
                    a = np.ascontiguousarray(a, dt[t])
                    if a.shape != (length,):
                        raise DumpError(f"array {tag}: shape {a.shape}, block length {length}")
                    _write_record(f, _tag(tag))
                    _write_record(f, a.tobytes())


def read(path: str) -> Dump:
    """Read any tagged dump (open_dumpfile_r, read_header, read_block_header,
    read_array): 8-byte or 4-byte default reals, little endian."""
    with open(path, "rb") as f:
        magic = _read_record(f)
        if len(magic) == 24:
            real = "<f8"
            i1 = int(np.frombuffer(magic[:4], "<i4")[0])
            i2, iv, i3 = (int(v) for v in np.frombuffer(magic[12:24], "<i4"))
        elif len(magic) == 20:
            real = "<f4"
            i1 = int(np.frombuffer(magic[:4], "<i4")[0])
            i2, iv, i3 = (int(v) for v in np.frombuffer(magic[8:20], "<i4"))
        else:
            raise DumpError("not a Phantom dump (magic record)")
        if i1 not in (INT1, INT1O):
            raise DumpError("wrong endian?")            # ierr_endian
        if iv == INT1O:
            iv = 0
        if iv > IVERSION:
            raise DumpError("file format version newer than this reader")
        if i2 not in (INT2, INT2O):
            raise DumpError("default real size wrong")  # ierr_realsize
        if i3 != INT1O:
            raise DumpError("default int size wrong")   # ierr_intsize
        fileid = _read_record(f).decode("ascii").rstrip()
        if len(fileid) < 2 or fileid[1] != "T":
            raise DumpError("untagged (pre-2016) dump: not supported")
        dt = dict(_DT, real=real)
        header = {}
        for t in TYPES:
            n = int(np.frombuffer(_read_record(f), "<i4")[0])
            if n > 0:
                tags = _tags(_read_record(f))
                vals = np.frombuffer(_read_record(f), dt[t])
                if len(tags) != n or len(vals) != n:
                    raise DumpError(f"header section {t}: {n} entries expected")
                header[t] = [(k, v.item()) for k, v in zip(tags, vals)]
            else:
                header[t] = []
        nblocks = int(np.frombuffer(_read_record(f), "<i4")[0])
        heads = []
        for _ in range(nblocks):
            r = _read_record(f)
            heads.append((int(np.frombuffer(r[:8], "<i8")[0]), [int(v) for v in np.frombuffer(r[8:40], "<i4")]))
        blocks = []
        for length, nums in heads:
            arrs = {}
            for t, cnt in zip(TYPES, nums):
                lst = []
                for _ in range(cnt):
                    tag = _tags(_read_record(f))[0]
                    a = np.frombuffer(_read_record(f), dt[t]).copy()
                    if a.shape != (length,):
                        raise DumpError(f"array {tag}: {a.size} values, block length {length}")
                    lst.append((tag, a))
                if lst:
                    arrs[t] = lst
            blocks.append((length, arrs))
    return Dump(fileid, header, blocks, real)


# ------------------------------------------------------------------ full dumps of this path
def fileident(mhd: bool, gravity: bool, when: datetime.datetime | None = None) -> str:
    """fileident('FT','Phantom') (readwrite_dumps_common.f90:32-69)."""
    when = when or datetime.datetime.now()
    extra = "+grav" if gravity else ""
    kind = f"(mhd+clean{extra})  " if mhd else f"(hydro{extra})"
    return f"FT:Phantom:phantom_gb300:0000000 {kind}: {when:%d/%m/%Y %H:%M:%S}.0"


def rhoh(h, m, hfact):
    """part.F90:779: rho = m (hfact / |h|)^3."""
    return m * (hfact / np.abs(h)) ** 3


def write_fulldump(path: str, cfg: dict, t: float, xyzh, vxyzu, Bevol=None, divcurlv=None, poten=None,
                   iorig=None, divcurlB=None, dtmax: float | None = None, rhozero: float = 0.0, alpha=None):
    """A full dump of the particle state, laid out as write_fulldump
    (readwrite_dumps.f90:45-340) with the header tags of fill_header
    (readwrite_dumps_common.f90:261-390) that this path's parameters cover.
    B is written as B = rho Bevol (the reference's Bxyz). alpha (alphaind(1,:),
    float) is written when given, as the reference does with the viscosity
    switch (readwrite_dumps.f90:258)."""
    xyzh = np.asarray(xyzh, np.float64)
    vxyzu = np.asarray(vxyzu, np.float64)
    n = xyzh.shape[0]
    mhd = bool(cfg.get("mhd", 0))
    gravity = bool(cfg.get("gravity", 0))
    isothermal = bool(cfg.get("isothermal", 0))
    m = float(cfg["massoftype"])
    npartoftype = [n] + [0] * (MAXTYPES - 1)
    hdr = {t: [] for t in TYPES}
    hi = hdr["int"]
    hi += [("nparttot", n), ("ntypes", MAXTYPES)] + [("npartoftype", v) for v in npartoftype]
    hi += [("nblocks", 1), ("nptmass", 0), ("ndustlarge", 0), ("ndustsmall", 0), ("idust", 7),
           ("idtmax_n", 1), ("idtmax_frac", 0), ("idumpfile", 0), ("majorv", 2025), ("minorv", 0),
           ("microv", 0), ("iexternalforce", 0), ("ieos", int(cfg.get("ieos", 2))), ("isink", 0)]
    h8 = hdr["int8"]
    h8 += [("nparttot", n), ("ntypes", MAXTYPES)] + [("npartoftype", v) for v in npartoftype]
    hr = hdr["real"]
    gamma = float(cfg.get("gamma", 5.0 / 3.0))
    # write_headeropts_eos (eos.f90:1690-1711)
    hr += [("gamma", gamma), ("RK2", 1.5 * float(cfg.get("polyk", 0.0))), ("polyk2", 0.0),
           ("qfacdisc", 0.75), ("qfacdisc2", 0.75), ("cs_min", 0.0)]
    hr += [("time", float(t)), ("dtmax", float(dtmax if dtmax is not None else cfg.get("dtmax", 0.0))),
           ("rhozero", float(rhozero)), ("hfact", float(cfg["hfact"])), ("tolh", float(cfg["tolh"])),
           ("C_cour", float(cfg["C_cour"])), ("C_force", float(cfg["C_force"])), ("alpha", float(cfg["alpha"])),
           ("alphau", float(cfg["alphau"])), ("alphaB", float(cfg.get("alphaB", 0.0)))]
    hr += [("massoftype", m)] + [("massoftype", 0.0)] * (MAXTYPES - 1)
    hr += [("Bextx", 0.0), ("Bexty", 0.0), ("Bextz", 0.0), ("dum", 0.0)]
    if cfg.get("periodic", 0):
        hr += [(k, float(cfg[k])) for k in ("xmin", "xmax", "ymin", "ymax", "zmin", "zmax")]
    hr += [("get_conserv", 1.0), ("mtot_in", 0.0), ("etot_in", 0.0), ("angtot_in", 0.0), ("totmom_in", 0.0),
           ("mdust_in", 0.0)]
    hdr["real8"] += [("udist", 1.0), ("umass", 1.0), ("utime", 1.0), ("umagfd", 1.0)]
    # block 1: hydro (write order of write_fulldump, grouped by type on disk)
    real = [("x", xyzh[:, 0]), ("y", xyzh[:, 1]), ("z", xyzh[:, 2]),
            ("vx", vxyzu[:, 0]), ("vy", vxyzu[:, 1]), ("vz", vxyzu[:, 2])]
    if not isothermal:
        real.append(("u", vxyzu[:, 3]))
    real4 = [("h", xyzh[:, 3].astype(np.float32))]
    if alpha is not None:
        real4.append(("alpha", np.asarray(alpha, np.float32)))
    if divcurlv is not None:
        # all ndivcurlv rows under divcurlv_label (part.F90:100-101,
        # readwrite_dumps.f90:259): divv, and curlvx, curlvy, curlvz with curl v
        dcv = np.asarray(divcurlv, np.float32).reshape(n, -1)
        for k, tag in enumerate(("divv", "curlvx", "curlvy", "curlvz")[:dcv.shape[1]]):
            real4.append((tag, dcv[:, k]))
    if gravity and poten is not None:
        real4.append(("poten", np.asarray(poten, np.float32)))
    b1 = {"real": real, "real4": real4}
    if iorig is not None:
        b1["int4"] = [("iorig", np.asarray(iorig, np.int32))]
    blocks = [(n, b1), (0, {})]
    if mhd:
        Bevol = np.asarray(Bevol, np.float64)
        rho = rhoh(xyzh[:, 3], m, float(cfg["hfact"]))
        b4 = {"real": [("Bx", Bevol[:, 0] * rho), ("By", Bevol[:, 1] * rho), ("Bz", Bevol[:, 2] * rho),
                       ("psi", Bevol[:, 3])]}
        if divcurlB is not None:
            dB = np.asarray(divcurlB, np.float32).reshape(n, 4)
            b4["real4"] = [("divB", dB[:, 0]), ("curlBx", dB[:, 1]), ("curlBy", dB[:, 2]), ("curlBz", dB[:, 3])]
        blocks += [(0, {}), (n, b4)]
    write(path, Dump(fileident(mhd, gravity), hdr, blocks))


def read_fulldump(path: str, cfg: dict | None = None, with_alpha: bool = False):
    """Particle state of a full dump (read_dump, readwrite_dumps.f90): returns
    (cfg, t, xyzh, vxyzu, Bevol) with cfg holding the dump's run parameters
    over those of the given cfg, and with_alpha the 'alpha' array too (None
    when absent). Only gas particles (the first type) are read; Bevol = B / rho."""
    d = read(path)
    if d.fileid[:1] != "F":
        raise DumpError("not a full dump")
    c = dict(cfg or {})
    for k in ("hfact", "tolh", "C_cour", "C_force", "alpha", "alphau", "alphaB", "dtmax", "gamma"):
        v = d.get(k)
        if v is not None:
            c[k] = float(v)
    for k in ("xmin", "xmax", "ymin", "ymax", "zmin", "zmax"):
        v = d.get(k)
        if v is not None:
            c[k] = float(v)
            c["periodic"] = 1
    ieos = d.get("ieos")
    if ieos is not None:
        c["ieos"] = int(ieos)
    rk2 = d.get("RK2")
    if rk2 is not None:
        c["polyk"] = 2.0 / 3.0 * float(rk2)  # read_headeropts_eos, eos.f90:1729
    c["massoftype"] = float(d.get("massoftype"))
    t = float(d.get("time", 0.0))
    a1 = d.arrays(1)
    n = d.blocks[0][0]
    ngas = int(d.get("npartoftype", n)) if d.get("npartoftype") is not None else n
    xyzh = np.empty((ngas, 4))
    for k, key in enumerate(("x", "y", "z")):
        xyzh[:, k] = a1[key][:ngas]
    xyzh[:, 3] = a1["h"][:ngas].astype(np.float64)
    vxyzu = np.zeros((ngas, 4))
    for k, key in enumerate(("vx", "vy", "vz", "u")):
        if key in a1:
            vxyzu[:, k] = a1[key][:ngas]
    c["isothermal"] = 0 if "u" in a1 else 1
    Bevol = np.zeros((ngas, 4))
    a4 = d.arrays(4)
    if "Bx" in a4:
        rho = rhoh(xyzh[:, 3], c["massoftype"], c["hfact"])
        for k, key in enumerate(("Bx", "By", "Bz")):
            Bevol[:, k] = a4[key][:ngas] / rho
        if "psi" in a4:
            Bevol[:, 3] = a4["psi"][:ngas]
        c["mhd"] = 1
    c["maxp"] = max(int(c.get("maxp", 0)), ngas)
    if not math.isfinite(c["massoftype"]) or c["massoftype"] <= 0.0:
        raise DumpError("massoftype missing or not positive")
    if with_alpha:
        alpha = a1["alpha"][:ngas].astype(np.float32) if "alpha" in a1 else None
        return c, t, xyzh, vxyzu, Bevol, alpha
    return c, t, xyzh, vxyzu, Bevol
