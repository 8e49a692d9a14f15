"""Extract the known-answer constants of the reference's own tests for this
path into reference_known_answers.json (run where the reference sources are
present; the JSON is committed, nothing at test time reads the sources).

Each entry keeps the file and line it was read from. The values are parsed
from the Fortran source text with a pattern per entry; a pattern that no
longer matches makes the script fail rather than write a stale value.

    python tests/golden/make_golden.py /path/to/phantom
"""
from __future__ import annotations

import json
import os
import re
import sys

# (key, file, pattern with one group per value, converters, meaning)
ENTRIES = [
    ("derivshydro_tolh", "src/tests/test_derivs.f90", r"^\s*tolh\s*=\s*([0-9.eEdD+-]+)\s*!\s*BEWARE", [float],
     "tolh of the derivs tests (the neighbour counts depend on it)"),
    ("derivshydro_realneigh_formula", "src/tests/test_derivs.f90",
     r"realneigh\s*=\s*(4\./3\.\*pi\*\(hfact\*radkern\)\*\*3)", [str],
     "expected neighbours on the exact lattice: int(4/3 pi (2 hfact)^3)"),
    ("derivshydro_mean_nneigh_tol", "src/tests/test_derivs.f90",
     r"checkval\(actualmean,real\(int\(realneigh\)\),([0-9.eEdD+-]+),", [float],
     "tolerance of the mean neighbour number"),
    ("derivshydro_gradh", "src/tests/test_derivs.f90",
     r"checkval\(n,gradh\(1,1:n\),([0-9.eEdD+-]+),([0-9.eEdD+-]+),", [float, float],
     "gradh (1/Omega) on the exact lattice and its relative tolerance"),
    ("sedov_npart_per_side", "src/tests/test_sedov.f90", r"^\s*npart\s*=\s*([0-9]+)\s*$", [int],
     "lattice particles per side of the Sedov test"),
    ("sedov_tmax", "src/tests/test_sedov.f90", r"^\s*tmax\s*=\s*([0-9.eEdD+-]+)", [float], "end time"),
    ("sedov_C_cour", "src/tests/test_sedov.f90", r"^\s*C_cour\s*=\s*([0-9.eEdD+-]+)", [float], "Courant factor"),
    ("sedov_C_force", "src/tests/test_sedov.f90", r"^\s*C_force\s*=\s*([0-9.eEdD+-]+)", [float], "force timestep factor"),
    ("sedov_tolv", "src/tests/test_sedov.f90", r"^\s*tolv\s*=\s*([0-9.eEdD+-]+)", [float], "velocity iteration tolerance"),
    ("sedov_tolh", "src/tests/test_sedov.f90", r"^\s*tolh\s*=\s*([0-9.eEdD+-]+)", [float], "h-rho tolerance"),
    ("sedov_energy_tol", "src/tests/test_sedov.f90", r"checkval\(etotend,etot_in,([0-9.eEdD+-]+),", [float],
     "total energy conservation tolerance (reference test build)"),
    ("sedov_momentum_tol", "src/tests/test_sedov.f90", r"checkval\(momtotend,totmom_in,([0-9.eEdD+-]+),", [float],
     "linear momentum tolerance"),
    ("kdtree_revtree_tol", "src/tests/test_kdtree.F90", r"^\s*tol\s*=\s*([0-9.eEdD+-]+)\s*$", [float],
     "relative tolerance of revtree against maketree on the same positions (x0, hmax, mass, quads)"),
    ("kdtree_revtree_psep", "src/tests/test_kdtree.F90", r"^\s*psep\s*=\s*(1\./100\.)", [str],
     "particle spacing of the random distribution of the revtree test"),
    ("sedov_test_setup_flags", "build/Makefile_setups", r"^ifeq \(\$\(SETUP\), (test)\)", [str],
     "the reference's test build (its options follow in the Makefile: no CONST_AV)"),
]


def fnum(s: str) -> float:
    return float(s.replace("d", "e").replace("D", "e"))


def main(root: str) -> None:
    out = {}
    for key, rel, pat, conv, meaning in ENTRIES:
        path = os.path.join(root, rel)
        lines = open(path, encoding="utf-8", errors="replace").read().splitlines()
        rx = re.compile(pat)
        for no, ln in enumerate(lines, 1):
            m = rx.search(ln)
            if m:
                vals = [fnum(g) if c is float else (int(g) if c is int else g) for g, c in zip(m.groups(), conv)]
                out[key] = {"value": vals[0] if len(vals) == 1 else vals, "source": f"{rel}:{no}",
                            "meaning": meaning}
                break
        else:
            raise SystemExit(f"pattern for {key} not found in {rel}")
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_known_answers.json")
    with open(dst, "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)
        f.write("\n")
    print(dst)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        raise SystemExit(f"usage: python {os.path.basename(__file__)} <path of the reference source tree>")
    main(sys.argv[1])
