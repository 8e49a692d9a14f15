"""Golden fixture of the dump format: a small full dump written by
phantom_gb300.dumpfile (fixed date stamp, so the bytes are reproducible) and
what the reference's own Python reader (scripts/readPhantomDump.py) parses
from it: file id, header quantities, block array counts and names, and the
array values. Run where the reference sources are present:

    python tests/golden/make_dump_golden.py /path/to/phantom

The reader predates NumPy 2 (int() of a one-element array); it is run
unmodified with int shadowed in its module namespace.
"""
from __future__ import annotations

import builtins
import datetime
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from phantom_gb300 import dumpfile as D  # noqa: E402
from phantom_gb300 import setups as S  # noqa: E402

STAMP = datetime.datetime(2025, 1, 1, 12, 0, 0)


def golden_dump(path: str):
    """MHD vortex 4^3 at t = 0.25 with div v, as a full dump."""
    cfg, x, v, B = S.mhd_vortex(4)
    divv = np.linspace(-1.0, 1.0, len(x)).astype(np.float32)
    orig = D.fileident
    D.fileident = lambda mhd, grav, when=None: orig(mhd, grav, STAMP)
    try:
        D.write_fulldump(path, cfg, 0.25, x, v, B, divcurlv=divv)
    finally:
        D.fileident = orig
    return cfg, x, v, B, divv


def main(root: str):
    sys.path.insert(0, os.path.join(root, "scripts"))
    import readPhantomDump as R
    R.int = lambda a: builtins.int(np.asarray(a).reshape(-1)[0]) if isinstance(a, np.ndarray) else builtins.int(a)
    path = os.path.join(HERE, "mhd_vortex4_00000")
    golden_dump(path)
    d = R.read_dump(path)
    out = {
        "source": "scripts/readPhantomDump.py read_dump on mhd_vortex4_00000",
        "desc": d["desc"],
        "part_numbers": {k: np.asarray(v).tolist() for k, v in d["part_numbers"].items()},
        "part_numbers_long": {k: np.asarray(v).tolist() for k, v in d["part_numbers_long"].items()},
        "quantities": {k: np.asarray(v).tolist() for k, v in d["quantities"].items()},
        "units": {k: float(v) for k, v in d["units"].items()},
        "blocks": [{"dim": int(b["dim"]), "nintdb": int(b["nintdb"]), "ndouble": int(b["ndouble"]),
                    "nsingle": int(b["nsingle"]),
                    "data": {k: np.asarray(a, np.float64).tolist() for k, a in b["data"].items()}}
                   for b in d["blocks"]],
    }
    with open(os.path.join(HERE, "mhd_vortex4_00000.json"), "w") as f:
        json.dump(out, f, indent=0, sort_keys=True)
        f.write("\n")
    print(path)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        raise SystemExit(f"usage: python {os.path.basename(__file__)} <path of the reference source tree>")
    main(sys.argv[1])
