"""Batched solves: the case generator (CPU) and, on the GPU, sph_batch_solve against the
same solves run one after another, and the autotuner's chunk choice against results."""
import numpy as np
import pytest

import sphericalstokes_gb300 as S
from sphericalstokes_gb300 import batch as B

FIELDS = ("P", "V1", "V2", "V3", "TAU11", "TAU12", "TAU13", "TAU23", "ETA")


def test_sweep_cases_follow_the_distribution():
    cases = B.sweep_cases(256, seed=0)
    assert len(cases) == 256
    assert [c.geometry for c in cases[:6]] == [0, 1, 2, 0, 1, 2]
    assert all(c.n1 in B.EDGES and c.n2 in B.EDGES and c.n3 in B.EDGES for c in cases)
    ns = [c.n_exp if c.rheology == S.RHEO["edot_power_relax"] else 1.0 for c in cases]
    assert set(ns) == {1.0, 2.0, 3.0, 4.0}
    ratios = np.array([1.0 / c.vr for c in cases])
    assert ratios.min() >= 1e-4 and ratios.max() <= 1e-1
    again = B.sweep_cases(256, seed=0)
    assert all(a.n1 == b.n1 and a.vr == b.vr and a.sig_bc[1] == b.sig_bc[1] and a.sh == b.sh for a, b in zip(cases, again))


def test_batch_step_cap():
    """the reference's CFL up to a viscosity ratio of 1e2, then CFL(1e2) sqrt(1e2/vr)"""
    ref = lambda vr: 1.0 / (2.0 + 4.5 * np.log10(vr))
    for vr in (1.5, 10.0, 99.0):
        assert B.capped_cfl(vr) == ref(vr)
    for vr in (1e3, 1e4):
        assert B.capped_cfl(vr) == pytest.approx(np.sqrt(100.0 / vr) / 11.0, rel=1e-15) and B.capped_cfl(vr) < ref(vr)
    for c, r in zip(B.sweep_cases(30, seed=0), B.sweep_cases(30, seed=0, step_cap=False)):
        contrast = c.vr * (2.0 if c.rheology == S.RHEO["edot_power_relax"] else 1.0)
        cfl = min(ref(c.vr), B.capped_cfl(contrast))
        if c.geometry == 0:
            assert c.vpdt == pytest.approx(r.vpdt * cfl / ref(c.vr), rel=1e-12)
        else:  # the library's own step, dr CFL, is set at create time for these
            assert r.vpdt == 0.0 and c.vpdt == pytest.approx(c.l1 / (c.n1 - 1) * cfl, rel=1e-12)


def _small_cases(precision):
    return [
        S.sector_params((23, 17, 15), bc="stress", rheology="edot_power_relax", n_exp=3.0, relax=0.5, edot_bg=0.25,
                        sig_bc=(0.0, 0.5, -0.5), incl_linear=1, precision=precision),
        S.default_params("cylindrical", n1=19, n2=15, n3=13, rheology="linear", bc="stress", sig_bc=(0.0, 0.3, -0.3),
                         incl_linear=1, precision=precision),
        S.default_params("cartesian", n1=17, n2=15, n3=19, rheology="linear", incl_linear=1, precision=precision),
        S.sector_params((31, 15, 21), bc="free_slip", rheology="linear", precision=precision),
    ]


@pytest.mark.gpu
@pytest.mark.parametrize("precision,crit", [("fp64", "reference"), ("mixed", "residual")])
def test_batch_equals_serial(precision, crit):
    """every solve of the batch computes exactly what it computes alone (own stream, deterministic kernels)"""
    cases = _small_cases(precision)
    if crit == "reference":
        opts = S.make_opts(tol=1e-30, maxiter=400, nout=100, criterion=crit)
    else:
        opts = S.make_opts(tol=1e-8, maxiter=20000, nout=100, criterion=crit, inner_rtol=1e-2, max_outer=4, inner_max=4000)
    serial, fields_s = [], []
    for p in cases:
        with S.Solver(p) as sv:
            serial.append(sv.solve(tol=opts.tol, maxiter=opts.maxiter, nout=opts.nout, criterion=crit, inner_rtol=opts.inner_rtol,
                                   max_outer=opts.max_outer, inner_max=opts.inner_max))
            fields_s.append({f: sv.get(f) for f in FIELDS})
    solvers = [S.Solver(p) for p in _small_cases(precision)]
    try:
        res = S.solve_batch(solvers, opts, threads=3)
        fields_b = [{f: sv.get(f) for f in FIELDS} for sv in solvers]
    finally:
        for sv in solvers:
            sv.close()
    for i, (a, b) in enumerate(zip(serial, res)):
        assert (a.status, a.iters, a.outer) == (b.status, b.iters, b.outer), i
        for f in FIELDS:
            np.testing.assert_array_equal(fields_b[i][f], fields_s[i][f], err_msg=f"case {i} {f}")


@pytest.mark.gpu
def test_autotuned_chunk_gives_the_same_sweeps():
    p = _small_cases("mixed")[0]
    out = []
    for tune in (False, True):
        with S.Solver(p) as sv:
            if tune:
                k, ms = sv.autotune(sweeps=6)
                assert 1 <= k <= p.n3 and ms > 0.0
            sv.sweep(57)
            sv.sweep_apply()
            out.append({f: sv.get(f) for f in ("V1", "V2", "V3", "P")})
    for f in out[0]:
        np.testing.assert_array_equal(out[1][f], out[0][f], err_msg=f)


@pytest.mark.gpu
def test_batch_rejects_a_context_twice():
    with S.Solver(_small_cases("fp64")[3]) as sv:
        with pytest.raises(S.SphError):
            S.solve_batch([sv, sv], S.make_opts(maxiter=10), threads=2)


def _lockstep_cases():
    """uneven grids of all three geometries, linear and power law, mixed precision"""
    return [
        S.sector_params((23, 17, 15), bc="stress", rheology="edot_power_relax", n_exp=3.0, relax=0.5, edot_bg=0.25,
                        sig_bc=(0.0, 0.5, -0.5), incl_linear=1, precision="mixed"),
        S.default_params("cylindrical", n1=19, n2=15, n3=13, rheology="linear", bc="stress", sig_bc=(0.0, 0.3, -0.3),
                         incl_linear=1, precision="mixed"),
        S.default_params("cartesian", n1=33, n2=15, n3=19, rheology="linear", incl_linear=1, precision="mixed"),
        S.sector_params((31, 15, 21), bc="free_slip", rheology="linear", precision="mixed"),
        S.sector_params((15, 41, 9), bc="diapir", rheology="linear", precision="mixed"),
    ]


@pytest.mark.gpu
def test_lockstep_batch_equals_serial_with_own_budgets_and_a_diverging_solve():
    """The lockstep batch (one launch per sweep over all solves' blocks, rounds replayed from a
    graph): per-solve budgets that end inside a round (a last, shorter chunk), a solve stopped by
    max_outer, and a solve whose state holds a NaN (diverges at its first check) — every solve's
    status, iteration count and fields equal those of the same solve alone."""
    budgets = [(20000, 4000, 30), (1250, 600, 30), (20000, 4000, 1), (777, 300, 30), (20000, 4000, 30)]
    opts = [S.make_opts(tol=1e-8, maxiter=m, nout=100, criterion="residual", inner_rtol=1e-2, max_outer=mo, inner_max=im)
            for m, im, mo in budgets]

    def plant(sv, i):
        if i == 4:
            v = sv.get("V2")
            v[5, 20, 4] = np.nan
            sv.set("V2", v)

    serial, fields_s = [], []
    for i, (p, o) in enumerate(zip(_lockstep_cases(), opts)):
        with S.Solver(p) as sv:
            plant(sv, i)
            serial.append(sv.solve(tol=o.tol, maxiter=o.maxiter, nout=o.nout, criterion="residual", inner_rtol=o.inner_rtol,
                                   max_outer=o.max_outer, inner_max=o.inner_max))
            fields_s.append({f: sv.get(f) for f in FIELDS})
    solvers = [S.Solver(p) for p in _lockstep_cases()]
    try:
        for i, sv in enumerate(solvers):
            plant(sv, i)
        res = S.solve_batch(solvers, opts)
        fields_b = [{f: sv.get(f) for f in FIELDS} for sv in solvers]
    finally:
        for sv in solvers:
            sv.close()
    assert len({r.seconds for r in res}) == 1  # one lockstep batch: the batch's wall time for every solve
    assert serial[4].status == S.SPH_ERR_DIVERGED and serial[2].outer == 1 and serial[1].iters <= 1250
    for i, (a, b) in enumerate(zip(serial, res)):
        assert (a.status, a.iters, a.outer) == (b.status, b.iters, b.outer), i
        if a.status != S.SPH_ERR_DIVERGED:
            assert a.residual == b.residual, i
            for f in FIELDS:
                np.testing.assert_array_equal(fields_b[i][f], fields_s[i][f], err_msg=f"case {i} {f}")
