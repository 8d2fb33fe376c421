"""Known answers of the discrete scheme (the pins that need no reference run):
an exact steady state, a fixed point, the n = 1 limit of the power law, the
mirror symmetry of the centred inclusion, and a converged small solve of the
linear free-slip sphere against the FP64 oracle at the same iteration count."""
import numpy as np
import pytest

import oracle
import sphericalstokes_gb300 as S

pytestmark = pytest.mark.gpu


def test_cartesian_simple_shear_is_steady():
    """VX = Y sh with uniform η and no buoyancy solves the Cartesian scheme exactly
    (CartesianStokes_diapir.jl:342 sets it as the initial state)"""
    p = S.default_params("cartesian", n1=15, n2=13, n3=11, rheology="linear", vr=1.0, rho0=0.0, rho_in=0.0)
    with S.Solver(p) as sv:
        v0 = sv.get("V1")
        sv.step(300)
        v1, v2, v3, P = sv.get("V1"), sv.get("V2"), sv.get("V3"), sv.get("P")
        res = sv.residual()
    scale = np.abs(v0).max()
    assert scale > 0
    assert np.abs(v1 - v0).max() <= 1e-12 * scale
    assert max(np.abs(v2).max(), np.abs(v3).max()) <= 1e-12 * scale
    assert np.abs(P).max() <= 1e-12 * scale
    assert res["err"] <= 1e-10


def test_uniform_sphere_without_forcing_stays_at_rest():
    """η, ρ uniform, g = 0 and no boundary shear: V = P = τ = 0 is a fixed point"""
    p = S.default_params("spherical", n1=15, n2=13, n3=11, vr=1.0, rho_in=0.0, rho0=0.0, g=0.0, sh=0.0)
    with S.Solver(p) as sv:
        sv.step(100)
        for f in ("P", "V1", "V2", "V3", "TAU11", "TAU12", "TAU13", "TAU23"):
            assert np.abs(sv.get(f)).max() == 0.0, f


def test_power_law_with_n_one_returns_the_initial_viscosity():
    """power_law! (SphericalStokes_diapir.jl:259-265) with n = 1: η = 2/(1/η_ini + 1/η_ini)"""
    p = S.default_params("spherical", n1=15, n2=13, n3=11, n_exp=1.0)
    with S.Solver(p) as sv:
        sv.step(20)
        eta, eta_ini = sv.get("ETA"), sv.get("ETA_INI")
    expect = 2.0 / (1.0 / eta_ini + 1.0 / (eta_ini * 1.0))
    np.testing.assert_array_equal(eta, expect)
    np.testing.assert_allclose(eta, eta_ini, rtol=4e-16, atol=0)


def test_centred_inclusion_is_mirror_symmetric():
    """the sector's inclusion is centred at θ = π/2, φ = 0: P, V_r mirror-symmetric, V_θ odd in θ, V_φ odd in φ"""
    p = S.sector_params((21, 19, 17), bc="free_slip", rheology="linear")
    with S.Solver(p) as sv:
        sv.step(300)
        P, V1, V2, V3 = sv.get("P"), sv.get("V1"), sv.get("V2"), sv.get("V3")
    tol = lambda a: 1e-10 * np.abs(a).max()
    assert np.abs(P - P[:, ::-1, :]).max() <= tol(P)
    assert np.abs(P - P[:, :, ::-1]).max() <= tol(P)
    assert np.abs(V1 - V1[:, ::-1, :]).max() <= tol(V1)
    assert np.abs(V1 - V1[:, :, ::-1]).max() <= tol(V1)
    assert np.abs(V2 + V2[:, ::-1, :]).max() <= tol(V2)
    assert np.abs(V3 + V3[:, :, ::-1]).max() <= tol(V3)
    assert np.abs(V1).max() > 0 and np.abs(V2).max() > 0 and np.abs(V3).max() > 0


def test_converged_linear_sphere_matches_the_oracle():
    """the linear free-slip sector (centred inclusion) on a small grid to FP64 residual 1e-8,
    then the oracle for the same number of iterations"""
    p = S.sector_params((19, 17, 15), bc="free_slip", rheology="linear")
    with S.Solver(p) as sv:
        res = sv.solve(tol=1e-8, maxiter=200000, nout=100, criterion="residual")
        got = {f: sv.get(f) for f in ("P", "V1", "V2", "V3", "TAU11", "TAU12", "TAU13", "TAU23")}
    assert res.converged and res.residual <= 1e-8
    o = oracle.Sph.from_params(p)
    o.iterate(res.iters)
    assert o.residual()["err"] <= 1.01e-8
    for f, a in got.items():
        b = o.field(f)
        assert np.abs(a - b).max() <= 1e-9 * np.abs(b).max(), f
