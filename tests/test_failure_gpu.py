"""Failure detection, exercised without a GPU fault:

* a NaN written into the state from the host ends a solve with SPH_ERR_DIVERGED at its next
  check, for every precision and criterion (the reference stops on a NaN error,
  SphericalStokes_mxpu.jl:426; its diapir scripts keep iterating on NaN);
* a solve given too few iterations ends with SPH_ERR_NOT_CONVERGED and its history;
* the TMA sweeps' bounded wait, run out on a barrier that nothing completes (no copy in
  flight), is reported as SPH_ERR_CUDA, the context refuses further work, and a new
  context computes the same sweeps as one that never saw the time-out.
"""
import numpy as np
import pytest

import sphericalstokes_gb300 as S

pytestmark = pytest.mark.gpu


def small(precision, rheology="linear"):
    return S.sector_params((15, 13, 11), bc="stress", rheology=rheology, n_exp=3.0, relax=0.5, edot_bg=0.25,
                           sig_bc=(0.0, 0.5, -0.5), incl_linear=1, precision=precision)


def plant_nan(sv):
    v = sv.get("V1")
    v[7, 6, 5] = np.nan
    sv.set("V1", v)


@pytest.mark.parametrize("precision,criterion", [("fp64", "reference"), ("fp64", "residual"), ("fp32", "reference"),
                                                 ("fp32", "residual"), ("mixed", "residual")])
def test_nan_in_the_state_diverges(precision, criterion):
    with S.Solver(small(precision)) as sv:
        plant_nan(sv)
        r = sv.solve(tol=1e-8, maxiter=10_000, nout=100, criterion=criterion, warm_tol=0.0)
    assert r.status == S.SPH_ERR_DIVERGED, r
    assert r.iters <= 100  # stopped at the first check
    assert len(r.hist_err) >= 1 and np.isnan(r.hist_err[-1])


@pytest.mark.parametrize("precision,criterion", [("fp64", "reference"), ("fp64", "residual"), ("mixed", "residual")])
def test_too_few_iterations_is_not_converged(precision, criterion):
    with S.Solver(small(precision, "edot_power_relax")) as sv:
        r = sv.solve(tol=1e-12, maxiter=300, nout=100, criterion=criterion, inner_max=100, max_outer=2)
    assert r.status == S.SPH_ERR_NOT_CONVERGED, r
    assert r.iters <= 300 and np.all(np.isfinite(r.hist_err)) and r.hist_err[-1] > 1e-12


def test_bounded_wait_time_out_is_reported_and_fatal():
    lib = S.load_library()
    p = small("mixed")
    with S.Solver(p) as ref:
        ref.sweep(8)
        want = ref.corr_get("dV1")
    with S.Solver(p) as sv:
        sv.sweep(8)
        assert lib.sph_selftest_wait_timeout(sv._h) == S.SPH_ERR_CUDA
        assert b"bounded wait" in lib.sph_last_error()
        assert lib.sph_sweep(sv._h, 1) == S.SPH_ERR_CUDA  # refused: the context is unusable
        assert b"unusable" in lib.sph_last_error()
        with pytest.raises(S.SphError):
            sv.get("V1")
    with S.Solver(p) as fresh:  # a new context on the same device is unaffected
        fresh.sweep(8)
        got = fresh.corr_get("dV1")
    assert np.array_equal(got, want)
