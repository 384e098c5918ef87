"""Generates the golden fixtures under tests/golden/ from the reference project.

Run as `python tests/golden/make_golden.py <path of the reference project>`
(or with the path in the environment variable MCFD_REFERENCE).  Two sources:

1. Known-answer tests of the reference's C++ test suite, transcribed below
   with their file:line.  The script re-reads each cited line and checks that
   every number of the transcription appears there, so a typo fails loudly.
   The C++ reference cannot be built here (Eigen, MPI, CGNS are absent), so
   the C++ KATs are used as published data.
2. Roe and Lax-Friedrichs (Rusanov) normal-frame fluxes computed by importing
   the reference's own Python prototype (python/riemann.py:405-476) on
   seeded random states.  These are the only reference implementations of the
   two solvers.

Output: tests/golden/riemann_kat.json, tests/golden/python_fluxes.json.
"""
from __future__ import annotations

import json
import os
import re
import sys
from pathlib import Path

import numpy as np

def _reference_path() -> Path:
    """The reference checkout: the first argument, else $MCFD_REFERENCE."""
    if len(sys.argv) > 1:
        return Path(sys.argv[1])
    if os.environ.get("MCFD_REFERENCE"):
        return Path(os.environ["MCFD_REFERENCE"])
    sys.exit("usage: make_golden.py <path of the reference project> (or set MCFD_REFERENCE)")


REFERENCE = _reference_path() if __name__ == "__main__" else Path(os.environ.get("MCFD_REFERENCE", "."))
OUT = Path(__file__).resolve().parent

# ----------------------------------------------------------------------------
# (1) C++ KATs.  Each case: solver, dimension, left/right primitive, expected
# primitive state on the t axis (flux = GetFlux(expected)), comparison.
#   "near": |actual/expected - 1| <= eps, expected == 0 requires actual == 0
#           (test/riemann/euler/exact.cpp:20-26)
#   "ratio": |a - e| / max(|a|, |e|) <= eps per component
#           (test/riemann/euler/hllc.cpp:12-14, 23-27)
V_L, V_R, W_L3, W_R3 = 1.5, 2.5, 1.5, 0.5  # exact.cpp:135, 230-231
HW_L, HW_R = 3.5, 4.5                      # hllc.cpp:108

EXACT = "test/riemann/euler/exact.cpp"
HLLC = "test/riemann/euler/hllc.cpp"
AUSM = "test/riemann/euler/ausm.cpp"

SOD_STAR = [0.426319, 0.927453, 0.303130]
CASES = [
    # --- Exact 1D (exact.cpp:54-85)
    dict(src=EXACT, line=54, solver="exact", dim=1, left=[1.0, 0.0, 1.0], right=[0.125, 0.0, 0.1],
         expect=[0.426319, +0.927453, 0.303130], cmp="near", eps=[1e-4] * 3),
    dict(src=EXACT, line=54, solver="exact", dim=1, left=[0.125, 0.0, 0.1], right=[1.0, 0.0, 1.0],
         expect=[0.426319, -0.927453, 0.303130], cmp="near", eps=[1e-4] * 3),
    dict(src=EXACT, line=61, solver="exact", dim=1, left=[5.99924, 19.5975, 460.894],
         right=[5.99242, 6.19633, 46.0950], expect=[5.99924, 19.5975, 460.894], cmp="near", eps=[1e-4] * 3),
    dict(src=EXACT, line=66, solver="exact", dim=1, left=[1.0, 0.0, 1000], right=[1.0, 0.0, 0.01],
         expect=[0.575062, 19.59745, 460.8938], cmp="near", eps=[1e-4] * 3),
    dict(src=EXACT, line=71, solver="exact", dim=1, left=[1.0, 0.0, 0.01], right=[1.0, 0.0, 100],
         expect=[0.575113, -6.196328, 46.09504], cmp="near", eps=[1e-4] * 3),
    dict(src=EXACT, line=76, solver="exact", dim=1, left=[1.0, -2.0, 0.4], right=[1.0, +2.0, 0.4],
         expect=[0.21852, 0.0, 0.001894], cmp="near", eps=[1e-4] * 3),
    dict(src=EXACT, line=81, solver="exact", dim=1, left=[1.0, -4.0, 0.4], right=[1.0, +4.0, 0.4],
         expect=[0.0, 0.0, 0.0], cmp="near", eps=[1e-4] * 3),
    # --- Exact 3D (exact.cpp:251-275): v, w passive
    dict(src=EXACT, line=251, solver="exact", dim=3, left=[1.000, 0.0, V_L, W_L3, 1.0],
         right=[0.125, 0.0, V_R, W_R3, 0.1], expect=[0.426319, +0.927453, V_L, W_L3, 0.303130],
         cmp="near", eps=[1e-4] * 5),
    dict(src=EXACT, line=259, solver="exact", dim=3, left=[5.99924, 19.59750, V_L, W_L3, 460.894],
         right=[5.99242, -6.19633, V_R, W_R3, 46.0950], expect=[5.99924, 19.5975, V_L, W_L3, 460.894],
         cmp="near", eps=[1e-4] * 5),
    dict(src=EXACT, line=265, solver="exact", dim=3, left=[1.0, 0.0, V_L, W_L3, 1e+3],
         right=[1.0, 0.0, V_R, W_R3, 1e-2], expect=[0.575062, 19.59745, V_L, W_L3, 460.8938],
         cmp="near", eps=[1e-4] * 5),
    dict(src=EXACT, line=271, solver="exact", dim=3, left=[1.0, 0.0, V_L, W_L3, 1e-2],
         right=[1.0, 0.0, V_R, W_R3, 1e+2], expect=[0.575113, -6.196328, V_R, W_R3, 46.09504],
         cmp="near", eps=[1e-4] * 5),
    # --- HLLC 1D and 3D (hllc.cpp:45-66, 127-152)
    dict(src=HLLC, line=45, solver="hllc", dim=1, left=[1.0, 0.0, 1.0], right=[0.125, 0.0, 0.1],
         expect=[0.426319, +0.927453, 0.303130], cmp="ratio", eps=[0.05, 0.25, 0.05]),
    dict(src=HLLC, line=52, solver="hllc", dim=1, left=[5.99924, 19.5975, 460.894],
         right=[5.99242, 6.19633, 46.0950], expect=[5.99924, 19.5975, 460.894],
         cmp="ratio", eps=[0.05, 0.25, 0.05]),
    dict(src=HLLC, line=57, solver="hllc", dim=1, left=[1.0, 0.0, 1000], right=[1.0, 0.0, 0.01],
         expect=[0.575062, 19.59745, 460.8938], cmp="ratio", eps=[0.05, 0.25, 0.05]),
    dict(src=HLLC, line=62, solver="hllc", dim=1, left=[1.0, 0.0, 0.01], right=[1.0, 0.0, 100],
         expect=[0.575113, -6.196328, 46.09504], cmp="ratio", eps=[0.05, 0.25, 0.05]),
    dict(src=HLLC, line=127, solver="hllc", dim=3, left=[1.000, 0.0, 1.5, 3.5, 1.0],
         right=[0.125, 0.0, 2.5, 4.5, 0.1], expect=[0.426319, +0.927453, 1.5, 3.5, 0.303130],
         cmp="ratio", eps=[0.05, 0.25, 0.02, 0.02, 0.05]),
    dict(src=HLLC, line=135, solver="hllc", dim=3, left=[5.99924, 19.5975, 1.5, 3.5, 460.894],
         right=[5.99242, 6.19633, 2.5, 4.5, 46.0950], expect=[5.99924, 19.5975, 1.5, 3.5, 460.894],
         cmp="ratio", eps=[0.05, 0.25, 0.02, 0.02, 0.05]),
    dict(src=HLLC, line=141, solver="hllc", dim=3, left=[1.0, 0.0, 1.5, 3.5, 1e+3],
         right=[1.0, 0.0, 2.5, 4.5, 1e-2], expect=[0.575062, 19.59745, 1.5, 3.5, 460.8938],
         cmp="ratio", eps=[0.05, 0.25, 0.02, 0.02, 0.05]),
    dict(src=HLLC, line=147, solver="hllc", dim=3, left=[1.0, 0.0, 1.5, 3.5, 1e-2],
         right=[1.0, 0.0, 2.5, 4.5, 1e+2], expect=[0.575113, -6.196328, 2.5, 4.5, 46.09504],
         cmp="ratio", eps=[0.05, 0.25, 0.02, 0.02, 0.05]),
    # --- AUSM 1D (ausm.cpp:45-61): mass 0.34, momentum 0.27, energy 0.19
    dict(src=AUSM, line=45, solver="ausm", dim=1, left=[1.0, 0.0, 1.0], right=[0.125, 0.0, 0.1],
         expect=[0.426319, +0.927453, 0.303130], cmp="ratio", eps=[0.34, 0.27, 0.19]),
    dict(src=AUSM, line=52, solver="ausm", dim=1, left=[5.99924, 19.5975, 460.894],
         right=[5.99242, 6.19633, 46.0950], expect=[5.99924, 19.5975, 460.894],
         cmp="ratio", eps=[0.34, 0.27, 0.19]),
    dict(src=AUSM, line=57, solver="ausm", dim=1, left=[1.0, 0.0, 1000], right=[1.0, 0.0, 0.01],
         expect=[0.575062, 19.59745, 460.8938], cmp="ratio", eps=[0.34, 0.27, 0.19]),
]

# Vacuum KATs (exact.cpp:86-127 right vacuum, 1D; 293-340 left vacuum, 3D):
# expected flux = GetFlux(state) with an absolute tolerance.
VACUUM = [
    # right vacuum, left = (1.4, u_L, 1.0), right = (0, 100, 0); a_L = 1
    dict(src=EXACT, line=92, dim=1, left=[1.4, -6.0, 1.0], right=[0.0, 100.0, 0.0], expect="right", atol=0.0),
    dict(src=EXACT, line=99, dim=1, left=[1.4, -5.0, 1.0], right=[0.0, 100.0, 0.0], expect="right", atol=1e-18),
    dict(src=EXACT, line=106, dim=1, left=[1.4, -4.0, 1.0], right=[0.0, 100.0, 0.0],
         expect=[1.4 * 6.0 ** -5, 6.0 ** -1, 6.0 ** -7], atol=1e-19),
    dict(src=EXACT, line=115, dim=1, left=[1.4, 1.0, 1.0], right=[0.0, 100.0, 0.0], expect="left", atol=1e-14),
    dict(src=EXACT, line=121, dim=1, left=[1.4, 2.0, 1.0], right=[0.0, 100.0, 0.0], expect="left", atol=1e-14),
    # left vacuum, left = (0, -100, -50, -20, 0), right = (1.4, u_R, 50, 20, 1.0)
    dict(src=EXACT, line=304, dim=3, left=[0.0, -100.0, -50.0, -20.0, 0.0], right=[1.4, 6.0, 50.0, 20.0, 1.0],
         expect="left", atol=0.0),
    dict(src=EXACT, line=312, dim=3, left=[0.0, -100.0, -50.0, -20.0, 0.0], right=[1.4, 5.0, 50.0, 20.0, 1.0],
         expect="left", atol=1e-18),
    dict(src=EXACT, line=320, dim=3, left=[0.0, -100.0, -50.0, -20.0, 0.0], right=[1.4, 4.0, 50.0, 20.0, 1.0],
         expect=[1.4 * 6.0 ** -5, -(6.0 ** -1), 50.0, 20.0, 6.0 ** -7], atol=1e-16),
]


def _numbers(text: str) -> list[float]:
    out = []
    for tok in re.findall(r"[-+]?\d+\.?\d*(?:e[-+]?\d+)?", text):
        try:
            out.append(float(tok))
        except ValueError:
            pass
    return out


def verify_transcription() -> None:
    """Every number of a case's expected state must occur within +-12 lines
    of the cited line of the reference test file."""
    for case in CASES:
        lines = (REFERENCE / case["src"]).read_text().splitlines()
        lo, hi = max(0, case["line"] - 12), min(len(lines), case["line"] + 12)
        found = set(abs(x) for x in _numbers("\n".join(lines[lo:hi])))
        for x in case["left"] + case["right"] + case["expect"]:
            if x in (V_L, V_R, W_L3, W_R3, HW_L, HW_R, 0.0):
                continue
            if abs(x) not in found:
                raise SystemExit(f"transcription check failed: {x} not near {case['src']}:{case['line']}")


def python_fluxes(n: int = 64, seed: int = 20240603) -> dict:
    sys.path.insert(0, str(REFERENCE / "python"))
    import riemann  # noqa: E402  (the reference's own prototype)
    rng = np.random.default_rng(seed)
    out = {"source": "python/riemann.py:405-476 (Roe, LaxFriedrichs), gamma = 1.4",
           "seed": seed, "cases": []}
    roe, lf = riemann.Roe(1.4), riemann.LaxFriedrichs(1.4)
    eq = roe.equation()
    for i in range(n):
        rho = rng.uniform(0.1, 2.0, 2)
        u = rng.uniform(-2.0, 2.0, 2)
        p = rng.uniform(0.05, 3.0, 2)
        if i % 8 == 0:  # a few near-equal states
            rho[1], u[1], p[1] = rho[0] * 1.001, u[0], p[0] * 0.999
        ul = eq.primitive_to_conservative(rho[0], u[0], p[0])
        ur = eq.primitive_to_conservative(rho[1], u[1], p[1])
        out["cases"].append({
            "left": [float(rho[0]), float(u[0]), float(p[0])],
            "right": [float(rho[1]), float(u[1]), float(p[1])],
            "roe": [float(v) for v in roe.get_upwind_flux(ul, ur)],
            "lax_friedrichs": [float(v) for v in lf.get_upwind_flux(ul, ur)],
        })
    return out


def main() -> None:
    if not REFERENCE.exists():
        raise SystemExit(f"reference project not found at {REFERENCE}")
    verify_transcription()
    kat = {"gamma": 1.4, "cases": CASES, "vacuum": VACUUM}
    (OUT / "riemann_kat.json").write_text(json.dumps(kat, indent=1))
    (OUT / "python_fluxes.json").write_text(json.dumps(python_fluxes(), indent=1))
    print("wrote", OUT / "riemann_kat.json", OUT / "python_fluxes.json")


if __name__ == "__main__":
    main()
