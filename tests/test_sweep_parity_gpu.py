"""The timed kernel against the oracle: FP32 correction sweeps of the mixed-precision
solve (``sph_sweep``: the fused TMA sweep k_fused_tma<G,1> plus the boundary stages it
leaves to the BC launch) compared with the FP64 oracle's restatement of the same sweep
(``orc_sph_corr_sweep`` / ``orc_cc_corr_sweep``: compute_P! with rP, compute_V! with rV
in place of -ρg, the homogeneous BC set; SphericalStokes_diapir.jl:209-241, :308-329,
:61-99 and the cylindrical / Cartesian scripts' kernels).

Both start from the same correction problem: the one the library prepares from the
FP64 state (FP64 residual in rP/rV, frozen η and ηSM), read back through
``sph_corr_get`` after its FP32 rounding, optionally with a random initial correction
written through ``sph_corr_set`` so that every term of the update is active from the
first sweep.  Errors are max-norm differences relative to the max-norm of the field's
group (δP; the three δV components together; the six δτ components together).
Tolerance: 2e-4 for the FP32 sweeps against FP64 (the FP32 arithmetic and its fast
division, accumulated over up to 100 sweeps).
"""
import math
import os

import numpy as np
import pytest

import oracle
import sphericalstokes_gb300 as S

pytestmark = pytest.mark.gpu

TOL = 2e-4
STATE = ("dP", "dV1", "dV2", "dV3", "dTAU11", "dTAU22", "dTAU33", "dTAU12", "dTAU13", "dTAU23")
GROUPS = {"P": ("dP",), "V": ("dV1", "dV2", "dV3"), "TAU": ("dTAU11", "dTAU22", "dTAU33", "dTAU12", "dTAU13", "dTAU23")}
ORACLE_NAME = {"dP": "P", "dV1": "V1", "dV2": "V2", "dV3": "V3", "dTAU11": "TAU11", "dTAU22": "TAU22", "dTAU33": "TAU33",
               "dTAU12": "TAU12", "dTAU13": "TAU13", "dTAU23": "TAU23"}


def case_params(geometry, n, bc):
    if geometry == "spherical":
        return S.sector_params(n, bc=bc, rheology="edot_power_relax", n_exp=3.0, relax=0.5, edot_bg=0.25,
                               sig_bc=(0.0, 0.5, -0.5), incl_linear=1, precision="mixed")
    return S.default_params(geometry, n1=n[0], n2=n[1], n3=n[2], rheology="linear", precision="mixed")


def oracle_state(p):
    return oracle.Sph.from_params(p) if p.geometry == 0 else oracle.CC.from_params(p)


def run_case(p, k, random_start, seed=0, setup=None):
    """k GPU correction sweeps and the oracle's from the same start; returns the group errors.
    setup(solver): called before the correction problem is prepared (e.g. to set a field)."""
    rng = np.random.default_rng(seed)
    with S.Solver(p) as sv:
        if setup:
            setup(sv)
        if random_start:
            for f in STATE:
                a = sv.corr_get(f)
                sv.corr_set(f, 1e-2 * rng.standard_normal(a.shape))
        start = {f: sv.corr_get(f) for f in STATE + ("ETA", "ETA_SM", "rP", "rV1", "rV2", "rV3")}
        sv.sweep(k)
        got = {f: sv.corr_get(f) for f in STATE}
    o = oracle_state(p)
    for f in STATE:
        o.field(ORACLE_NAME[f])[:] = start[f]
    o.field("ETA")[:] = start["ETA"]
    o.field("ETA_SM")[:] = start["ETA_SM"]
    o.corr_sweep(start["rP"], start["rV1"], start["rV2"], start["rV3"], k)
    err = {}
    for g, fs in GROUPS.items():
        scale = max(float(np.abs(o.field(ORACLE_NAME[f])).max()) for f in fs)
        diff = max(float(np.abs(got[f] - o.field(ORACLE_NAME[f])).max()) for f in fs)
        # a group the oracle leaves exactly zero (δP and δτ after one sweep from a zero correction
        # with rP = 0) must be exactly zero on the GPU too
        err[g] = diff / scale if scale > 0.0 else (0.0 if diff == 0.0 else float("inf"))
    assert any(float(np.abs(o.field(ORACLE_NAME[f])).max()) > 0.0 for f in STATE), "the case exercises nothing"
    return err


CASES = [("spherical", (17, 13, 11), "free_slip"), ("spherical", (17, 13, 11), "stress"),
         ("spherical", (15, 19, 9), "diapir"), ("cylindrical", (17, 13, 11), "diapir"),
         ("cartesian", (15, 13, 17), "diapir")]


@pytest.mark.parametrize("geometry,n,bc", CASES)
@pytest.mark.parametrize("k", [1, 10, 100])
def test_correction_sweeps_match_oracle(geometry, n, bc, k):
    err = run_case(case_params(geometry, n, bc), k, random_start=False)
    assert max(err.values()) < TOL, err


@pytest.mark.parametrize("geometry,n,bc", CASES)
@pytest.mark.parametrize("k", [1, 10])
def test_correction_sweeps_from_random_correction_match_oracle(geometry, n, bc, k):
    err = run_case(case_params(geometry, n, bc), k, random_start=True, seed=k)
    assert max(err.values()) < TOL, err


def test_correction_sweeps_63_cubed_match_oracle():
    """The 63^3 spherical sector of the CPU-runnable configuration (linear, free slip) and the
    n = 3 stress-BC workload at 63^3: several x3 chunks per block column."""
    p = S.sector_params(63, bc="free_slip", rheology="linear", precision="mixed")
    err = run_case(p, 10, random_start=True)
    assert max(err.values()) < TOL, err
    err = run_case(case_params("spherical", (63, 63, 63), "stress"), 20, random_start=False)
    assert max(err.values()) < TOL, err


def test_correction_sweeps_255_slab_match_oracle():
    """A 255 x 255 x 16 slab of the 255^3 workload (same spacing, the sector's centre planes):
    production x1/x2 extents, every traction face, several x3 chunks (chunk 4 forced)."""
    p = case_params("spherical", (255, 255, 16), "stress")
    S.set_params(p, l3=(math.pi / 2) * 15 / 254)
    os.environ["SPH_FUSED_CHUNK"] = "4"
    try:
        err = run_case(p, 10, random_start=True)
    finally:
        del os.environ["SPH_FUSED_CHUNK"]
    assert max(err.values()) < TOL, err

