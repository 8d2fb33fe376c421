"""GPU parity: the CUDA kernels (through the C ABI) against the FP64 oracle.

Tolerances are relative to each field's max-norm: 1e-12 for single kernels,
1e-9 for fixed-iteration trajectories (FMA contraction and the algebraic form
e/(e+GSDT) of 1/(1+GSDT/e) differ from the oracle at the last bits only).
"""
import math

import numpy as np
import pytest

import oracle
import sphericalstokes_gb300 as S

pytestmark = pytest.mark.gpu

FIELDS = ("P", "V1", "V2", "V3", "TAU11", "TAU22", "TAU33", "TAU12", "TAU13", "TAU23", "ETA", "ETA_SM", "DT_R", "TII")


def relerr(a, b):
    scale = max(np.abs(b).max(), 1e-300)
    return float(np.abs(a - b).max() / scale)


def randomize(o, sv, rng, fields=FIELDS + ("RHO", "ETA_INI")):
    for f in fields:
        a = o.field(f)
        if f.startswith("ETA") or f == "DT_R":
            a[:] = np.exp(rng.uniform(-2, 2, a.shape))
        elif f == "TII":
            a[:] = rng.uniform(0.1, 2.0, a.shape)
        else:
            a[:] = rng.standard_normal(a.shape)
        sv.set(f, a)


def compare(o, sv, fields, tol):
    bad = {}
    for f in fields:
        e = relerr(sv.get(f), o.field(f))
        if not e < tol:
            bad[f] = e
    assert not bad, bad


GRIDS = [(13, 9, 11), (8, 16, 7)]


@pytest.mark.parametrize("n", GRIDS)
@pytest.mark.parametrize("bc", ["diapir", "free_slip", "stress"])
def test_single_kernels_spherical(n, bc):
    p = S.default_params("spherical", n1=n[0], n2=n[1], n3=n[2], bc=bc, n_exp=3.0, sig_bc=(0.0, 0.5, -0.5))
    rng = np.random.default_rng(1)
    with S.Solver(p) as sv:
        o = oracle.Sph.from_params(p)
        randomize(o, sv, rng)
        sv.maxloc(); o.maxloc()
        compare(o, sv, ["ETA_SM"], 1e-15)
        randomize(o, sv, rng)
        sv.compute_P(); o.compute_P()
        compare(o, sv, ["P", "TAU11", "TAU22", "TAU33", "TAU12", "TAU13", "TAU23", "DT_R"], 1e-12)
        sv.power_law(); o.power_law()
        compare(o, sv, ["TII", "ETA"], 1e-12)
        sv.compute_V(); o.compute_V()
        compare(o, sv, ["V1", "V2", "V3"], 1e-12)
        sv.apply_bc(); o.apply_bc()
        compare(o, sv, ["V1", "V2", "V3"], 1e-12)


@pytest.mark.parametrize("k", [1, 10, 100])
def test_trajectory_spherical_diapir(k):
    # SphericalStokes_diapir.jl setup (n_exp = 5, r = 1000, lr = 6) on a small grid
    p = S.default_params("spherical", n1=17, n2=15, n3=13)
    with S.Solver(p) as sv:
        sv.step(k)
        o = oracle.Sph.from_params(p)
        o.iterate(k)
        compare(o, sv, FIELDS, 1e-9)


@pytest.mark.parametrize("k", [1, 50])
def test_trajectory_free_slip_plateau_bcs(k):
    p = S.sector_params((15, 13, 11), bc="free_slip", rheology="linear")
    with S.Solver(p) as sv:
        sv.step(k)
        o = oracle.Sph.from_params(p)
        o.iterate(k)
        compare(o, sv, ("P", "V1", "V2", "V3", "TAU11", "TAU12", "TAU13", "TAU23", "DT_R"), 1e-9)


@pytest.mark.parametrize("k", [1, 50])
def test_trajectory_stress_bc_strain_rate_law(k):
    p = S.sector_params((15, 13, 11), bc="stress", rheology="edot_power_relax", n_exp=3.0, relax=0.5,
                        edot_bg=0.25, sig_bc=(0.0, 0.5, -0.5), incl_linear=1)
    with S.Solver(p) as sv:
        sv.step(k)
        o = oracle.Sph.from_params(p)
        o.iterate(k)
        compare(o, sv, ("P", "V1", "V2", "V3", "TAU11", "TAU22", "TAU12", "TAU23", "ETA"), 1e-9)


def test_residual_matches_oracle():
    p = S.sector_params((15, 13, 11), bc="stress", rheology="edot_power_relax", n_exp=3.0, relax=0.5,
                        edot_bg=0.25, sig_bc=(0.0, 0.5, -0.5), incl_linear=1)
    with S.Solver(p) as sv:
        sv.step(30)
        r = sv.residual()
        o = oracle.Sph.from_params(p)
        o.iterate(30)
        ro = o.residual(f_scale=r["f_scale"])
    for key in ("mom1", "mom2", "mom3", "div", "vmax"):
        assert abs(r[key] - ro[key]) <= 1e-9 * max(abs(ro[key]), 1e-300), (key, r[key], ro[key])


def test_fp32_follows_fp64():
    p = S.sector_params((15, 13, 11), bc="free_slip", rheology="linear")
    with S.Solver(p) as a:
        a.step(50)
        ref = {f: a.get(f) for f in ("V1", "V2", "V3", "P")}
    set_p = S.sector_params((15, 13, 11), bc="free_slip", rheology="linear", precision="fp32")
    with S.Solver(set_p) as b:
        b.step(50)
        for f, r in ref.items():
            assert relerr(b.get(f), r) < 1e-4, f


def test_reference_criterion_solve_small():
    p = S.default_params("spherical", n1=15, n2=13, n3=11)
    with S.Solver(p) as sv:
        res = sv.solve(tol=5e-7, maxiter=20000, nout=100, criterion="reference")
    o = oracle.Sph.from_params(p)
    # replay the oracle for the same number of iterations and the same err sequence
    errs = []
    for it in range(1, res.iters + 1):
        if it % 100 == 0:
            o.equal3()
        o.iterate(1)
        if it % 100 == 0:
            errs.append(o.check_err())
    assert res.converged
    assert len(errs) == len(res.hist_err)
    np.testing.assert_allclose(res.hist_err, errs, rtol=1e-6)
    assert errs[-1] < 5e-7 and all(e >= 5e-7 for e in errs[:-1])


# ---------------------------------------------------------------------------
# fused FP32 sweep against the one-kernel-per-step FP32 path and the oracle
FUSED_CASES = [
    ("spherical", dict(bc="diapir", n_exp=3.0)),
    ("spherical", dict(bc="free_slip", rheology="linear")),
    ("spherical", dict(bc="stress", rheology="edot_power_relax", n_exp=3.0, relax=0.5, edot_bg=0.25,
                       sig_bc=(0.0, 0.5, -0.5), incl_linear=1)),
    ("cylindrical", dict(n_exp=3.0)),
    ("cartesian", dict(n_exp=3.0)),
]


def _params(geom, n, **kw):
    if geom == "spherical" and kw.get("bc") in ("free_slip", "stress"):
        return S.sector_params(n, **kw)
    return S.default_params(geom, n1=n[0], n2=n[1], n3=n[2], **kw)


@pytest.mark.parametrize("geom,kw", FUSED_CASES)
@pytest.mark.parametrize("n", [(37, 19, 13), (33, 9, 70)])
def test_fused_equals_simple_fp32(geom, kw, n):
    k = 30
    out = {}
    for variant in ("simple", "auto"):
        p = _params(geom, n, precision="fp32", kernels=variant, **kw)
        with S.Solver(p) as sv:
            sv.step(k)
            out[variant] = {f: sv.get(f) for f in ("P", "V1", "V2", "V3", "TAU11", "TAU12", "TAU13", "TAU23", "ETA")}
    for f in out["simple"]:
        # the same expressions, contracted into FMAs differently by the compiler in each
        # kernel: FP32 rounding differences, amplified by 30 nonlinear iterations
        assert relerr(out["auto"][f], out["simple"][f]) < 1e-5, f


def test_fused_fp32_tracks_fp64_oracle():
    p = S.default_params("spherical", n1=35, n2=17, n3=21, n_exp=3.0, precision="fp32")
    k = 40
    with S.Solver(p) as sv:
        sv.step(k)
        got = {f: sv.get(f) for f in ("P", "V1", "V2", "V3", "TAU11", "TAU12")}
    p.precision = 0
    o = oracle.Sph.from_params(p)
    o.iterate(k)
    for f, g in got.items():
        assert relerr(g, o.field(f)) < 2e-4, f


@pytest.mark.parametrize("passes", [2, 3])
def test_trajectory_wide_max_filter(passes):
    p = S.sector_params((15, 13, 11), bc="stress", rheology="edot_power_relax", n_exp=3.0, relax=0.5,
                        edot_bg=0.25, sig_bc=(0.0, 0.5, -0.5), incl_linear=1, etasm_passes=passes)
    with S.Solver(p) as sv:
        sv.step(40)
        o = oracle.Sph.from_params(p)
        o.iterate(40)
        compare(o, sv, ("P", "V1", "V2", "V3", "TAU11", "TAU12", "ETA", "ETA_SM"), 1e-9)


def test_sweep_graph_equals_plain_sweeps(monkeypatch):
    """the CUDA-graph replay of correction sweeps gives the sweeps' result"""
    from bench import workload_params
    out = []
    for graphs in ("0", "1"):
        monkeypatch.setenv("SPH_NO_GRAPHS", "1" if graphs == "0" else "0")
        with S.Solver(workload_params(31, "mixed")) as sv:
            sv.sweep(200)
            sv.sweep_apply()
            out.append({f: sv.get(f) for f in ("V1", "V2", "V3", "P")})
    for f in out[0]:
        assert relerr(out[1][f], out[0][f]) == 0.0, f


@pytest.mark.parametrize("n", [31, (40, 17, 23)])
def test_sweep_tma_equals_cp_async(monkeypatch, n):
    """the TMA-fed fused correction sweep computes what the cp.async one does (same
    expressions; FMA contraction may differ between the two kernels)"""
    from bench import workload_params
    out = []
    for tma in ("0", "1"):
        monkeypatch.setenv("SPH_NO_TMA", "1" if tma == "0" else "0")
        p = workload_params(31, "mixed") if n == 31 else S.sector_params(n, bc="stress", rheology="edot_power_relax", n_exp=3.0,
                                                                         relax=0.5, edot_bg=0.25, sig_bc=(0.0, 0.5, -0.5),
                                                                         incl_linear=1, precision="mixed")
        with S.Solver(p) as sv:
            sv.sweep(57)
            sv.sweep_apply()
            out.append({f: sv.get(f) for f in ("V1", "V2", "V3", "P")})
    for f in out[0]:
        assert relerr(out[1][f], out[0][f]) < 1e-5, f


def test_sweep_profile_equals_sweeps():
    """per-launch timed sweeps compute what the graph-replayed sweeps compute"""
    from bench import workload_params
    out, times = [], None
    for prof in (False, True):
        with S.Solver(workload_params(31, "mixed")) as sv:
            if prof:
                times = sv.sweep_profile(200)
            else:
                sv.sweep(200)
            sv.sweep_apply()
            out.append({f: sv.get(f) for f in ("V1", "V2", "V3", "P")})
    for f in out[0]:
        assert relerr(out[1][f], out[0][f]) == 0.0, f
    sweep_ms, kernel_ms = times
    assert 0.0 < kernel_ms <= sweep_ms


def test_mixed_solution_matches_fp64():
    """FP32 sweeps inside FP64 defect correction reach the FP64 PT solution: both to
    FP64 residual 1e-8, relative velocity difference <= 1e-6"""
    from bench import workload_params
    vel = {}
    for prec in ("fp64", "mixed"):
        with S.Solver(workload_params(23, prec, tuned=True)) as sv:
            if prec == "mixed":
                r = sv.solve(tol=1e-8, maxiter=400_000, nout=100, criterion="residual", inner_rtol=1e-2, max_outer=60,
                             inner_max=100_000, warm_tol=1e-5)
            else:
                r = sv.solve(tol=1e-8, maxiter=400_000, nout=500, criterion="residual")
            assert r.converged and r.residual < 1e-8, (prec, r.status, r.residual)
            vel[prec] = [sv.get(f) for f in ("V1", "V2", "V3")]
    vmax = max(np.abs(v).max() for v in vel["fp64"])
    err = max(np.abs(a - b).max() for a, b in zip(vel["mixed"], vel["fp64"])) / vmax
    assert err <= 1e-6, err


X2_CASES = [
    ("spherical", 31, dict(bc="stress", rheology="edot_power_relax", n_exp=3.0, relax=0.5, edot_bg=0.25,
                           sig_bc=(0.0, 0.5, -0.5), incl_linear=1)),
    ("spherical", (40, 17, 23), dict(bc="stress", rheology="edot_power_relax", n_exp=3.0, relax=0.5, edot_bg=0.25,
                                     sig_bc=(0.0, 0.5, -0.5), incl_linear=1)),
    ("spherical", (33, 9, 21), dict(bc="free_slip", rheology="linear")),
    ("cylindrical", (35, 11, 19), dict(rheology="linear")),
    ("cartesian", (31, 13, 17), dict(rheology="linear")),
]


@pytest.mark.parametrize("geom,n,kw", X2_CASES)
def test_sweep_two_points_per_thread_equals_one(monkeypatch, geom, n, kw):
    """the paired-arithmetic TMA sweep (two x1-adjacent points per thread) computes what the
    one-point-per-thread TMA sweep does, up to FP32 rounding of the fused multiply-adds"""
    out = []
    for x2 in ("0", "1"):
        monkeypatch.setenv("SPH_SWEEP_X2", x2)
        nn = (n, n, n) if isinstance(n, int) else n
        p = _params(geom, nn, precision="mixed", **kw)
        with S.Solver(p) as sv:
            sv.sweep(57)
            sv.sweep_apply()
            out.append({f: sv.get(f) for f in ("V1", "V2", "V3", "P")})
    for f in out[0]:
        assert relerr(out[1][f], out[0][f]) < 1e-5, f


def test_warm_start_graph_equals_plain_iterations(monkeypatch):
    """the mixed solve's FP32 warm start replayed from CUDA graphs gives what the iterations
    launched one by one give (same iterations, same solution)"""
    from bench import workload_params
    out = []
    for graphs in ("0", "1"):
        monkeypatch.setenv("SPH_NO_GRAPHS", "1" if graphs == "0" else "0")
        with S.Solver(workload_params(31, "mixed", tuned=True)) as sv:
            r = sv.solve(tol=1e-8, maxiter=6000, nout=100, criterion="residual", inner_rtol=1e-2, max_outer=3,
                         inner_max=2000, warm_tol=1e-5)
            out.append((r.iters, r.outer, r.residual, {f: sv.get(f) for f in ("V1", "V2", "V3", "P")}))
    assert out[0][:3] == out[1][:3]
    for f in out[0][3]:
        assert np.array_equal(out[1][3][f], out[0][3][f]), f


@pytest.mark.parametrize("geom,bc,n", [("spherical", "stress", (40, 17, 23)), ("spherical", "free_slip", 21),
                                       ("spherical", "diapir", (33, 12, 19)), ("cylindrical", "diapir", (19, 33, 12)),
                                       ("cartesian", "diapir", (35, 14, 27)), ("cylindrical", "stress", (23, 21, 17))])
def test_sweep_x1_ghosts_equal_bc_stage(monkeypatch, geom, bc, n):
    """the correction sweep writing the x1-face ghost velocities itself (and the BC launch
    skipping that stage) leaves exactly the state the separate BC stage leaves"""
    out = []
    for off in ("1", "0"):
        monkeypatch.setenv("SPH_NO_XGHOST", off)
        p = S.default_params(geom, n1=n if isinstance(n, int) else n[0], n2=n if isinstance(n, int) else n[1],
                             n3=n if isinstance(n, int) else n[2], n_exp=3.0, bc=bc, precision="mixed",
                             rheology="edot_power_relax" if bc == "stress" else "linear")
        with S.Solver(p) as sv:
            sv.sweep(38)
            sv.sweep_apply()
            out.append({f: sv.get(f) for f in ("V1", "V2", "V3", "P", "TAU12", "TAU23")})
    for f in out[0]:
        assert np.array_equal(out[1][f], out[0][f]), f
