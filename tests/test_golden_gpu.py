"""CUDA path (through the C ABI) against the golden vectors of the reference
scripts: same initial fields, k = 1 and 10 PT iterations, every field within
1e-11 of the field's max-norm."""
import math

import numpy as np
import pytest

import oracle
import sphericalstokes_gb300 as S
from test_golden import CASES, load, relerr

pytestmark = pytest.mark.gpu


def library_params(case, g):
    sc = eval(str(g["scalars_json"]))
    geom, bc = CASES[case]
    if geom == "spherical":
        x1, x2, x3 = g["coord_R_i"], g["coord_θ_i"], g["coord_φ_i"]
        p = S.default_params("spherical", bc="diapir" if bc == 0 else "free_slip", rheology="tau_power",
                             l1=sc["lr"], l2=sc["lθ"], l3=sc["lφ"], l_ref=sc["lr"], r=sc["r"], sh=sc.get("sh", 0.0))
    elif geom == "cylindrical":
        x1, x2, x3 = g["coord_R_i"], g["coord_θ_i"], g["coord_Z_i"]
        p = S.default_params("cylindrical", l1=sc["lr"], l2=sc["lθ"], l3=sc["lz"], l_ref=sc["lr"], r=sc["r"],
                             sh=sc["sh"], relax=sc["relax"], switch_err=0.0)
    else:
        x1, x2, x3 = g["coord_X_i"], g["coord_Y_i"], g["coord_Z_i"]
        p = S.default_params("cartesian", l1=sc["lx"], l2=sc["ly"], l3=sc["lz"], l_ref=sc["lx"], sh=sc["sh"],
                             relax=sc["relax"])
    S.set_params(p, n1=len(x1), n2=len(x2), n3=len(x3), c1=0.5 * (x1[0] + x1[-1]), c2=0.5 * (x2[0] + x2[-1]),
                 c3=0.5 * (x3[0] + x3[-1]), vpdt=sc["vpdt"], dmp=sc["dmp"], g=sc["g"], tau_C=sc["τ_C"],
                 n_exp=sc["n_exp"], init="none")
    return p


@pytest.mark.parametrize("case", list(CASES))
def test_library_matches_golden(case):
    g = load(case)
    geom = CASES[case][0]
    p = library_params(case, g)
    with S.Solver(p) as sv:
        for f, a in oracle.golden_fields(g, geom, "in_").items():
            sv.set(f, a)
        done = 0
        for k in (1, 10):
            sv.step(k - done)
            done = k
            ref = oracle.golden_fields(g, geom, f"k{k}_")
            bad = {}
            for f, r in ref.items():
                e = relerr(sv.get(f), r)
                if not e < 1e-11:
                    bad[f] = e
            assert not bad, (k, bad)
