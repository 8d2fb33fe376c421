"""Adjoint of the FP64 residual: dot-product tests of the hand-written transposed
stencils against the forward residual (every velocity entry independent, and the
interior-unknown form with the BC program), and gradients of a surface-velocity
misfit with respect to log η and ρ against central finite differences."""
import numpy as np
import pytest

import sphericalstokes_gb300 as S
from sphericalstokes_gb300 import adjoint as A

pytestmark = pytest.mark.gpu
FIELDS = ("V1", "V2", "V3", "P")


def _rand(sv, rng):
    return {f: np.asfortranarray(rng.standard_normal(sv.dims(f))) for f in FIELDS}


def _apply_A(sv, u, bc: bool):
    """A u = R(u) - R(0) with the forward residual (linear viscosity), optionally after the BC program"""
    def R(state):
        for f in FIELDS:
            sv.set(f, state[f])
        if bc:
            sv.apply_bc()
        return A.residual_fields(sv)
    zero = {f: np.zeros(sv.dims(f), order="F") for f in FIELDS}
    r1, r0 = R(u), R(zero)
    return {f: r1[f] - r0[f] for f in FIELDS}


def _dot(a, b):
    return sum(float(np.sum(a[f] * b[f])) for f in FIELDS)


CASES = [
    ("spherical", dict(bc="free_slip"), (13, 11, 9)),
    ("spherical", dict(bc="stress", sig_bc=(0.0, 0.5, -0.5)), (13, 11, 9)),
    ("spherical", dict(bc="diapir"), (12, 10, 9)),
    ("cylindrical", dict(bc="stress", sig_bc=(0.0, 0.3, -0.3)), (11, 9, 10)),
    ("cartesian", dict(bc="diapir"), (10, 11, 9)),
]


def _params(geom, kw, n):
    if geom == "spherical" and kw.get("bc") in ("free_slip", "stress"):
        return S.sector_params(n, rheology="linear", vr=10.0, **kw)
    return S.default_params(geom, n1=n[0], n2=n[1], n3=n[2], rheology="linear", vr=10.0, **kw)


@pytest.mark.parametrize("geom,kw,n", CASES)
@pytest.mark.parametrize("bc", [False, True])
def test_vjp_is_the_transpose_of_the_residual(geom, kw, n, bc):
    rng = np.random.default_rng(7)
    with S.Solver(_params(geom, kw, n)) as sv:
        u = _rand(sv, rng)
        lam = _rand(sv, rng)
        Au = _apply_A(sv, u, bc)
        g = A.vjp(sv, lam, interior=bc)
    if bc:  # interior unknowns: A u does not depend on the boundary entries, Aᵀλ is zero there
        for f in ("V1", "V2", "V3"):
            u[f] = np.where(g[f] != 0.0, u[f], 0.0)
    lhs, rhs = _dot(lam, Au), _dot(g, u)
    scale = sum(float(np.sum(np.abs(lam[f] * Au[f]))) for f in FIELDS)
    assert abs(lhs - rhs) <= 1e-12 * scale, (lhs, rhs, scale)


def _converged(sv, tol=1e-12):
    r = sv.solve(tol=tol, maxiter=400_000, nout=200, criterion="residual")
    assert r.converged, (r.status, r.residual)
    return r


@pytest.mark.parametrize("bc", ["free_slip", "stress"])
def test_gradients_match_central_differences(bc):
    p = S.sector_params((13, 11, 9), rheology="linear", vr=10.0, bc=bc, sig_bc=(0.0, 0.5, -0.5))
    rng = np.random.default_rng(11)
    with S.Solver(p) as sv:
        _converged(sv)
        base = {f: sv.get(f) for f in ("V1", "V2", "V3", "P", "TAU11", "TAU22", "TAU33", "TAU12", "TAU13", "TAU23")}
        grad = A.gradient(sv, tol=1e-12)
        assert grad["info"].status == S.SPH_OK, (grad["info"].status, grad["info"].err)
        eta0, rho0 = sv.get("ETA"), sv.get("RHO")

        def J_at(eta=None, rho=None):
            for f, a in base.items():
                sv.set(f, a)
            sv.set("ETA", eta0 if eta is None else eta)
            sv.set("ETA_INI", eta0 if eta is None else eta)
            sv.set("RHO", rho0 if rho is None else rho)
            _converged(sv)
            return A.surface_misfit(sv)[0]

        eps = 1e-4
        for _ in range(3):
            d = np.asfortranarray(rng.standard_normal(eta0.shape))
            fd = (J_at(eta=eta0 * np.exp(eps * d)) - J_at(eta=eta0 * np.exp(-eps * d))) / (2 * eps)
            ad = float(np.sum(grad["dlogeta"] * d))
            assert abs(fd - ad) <= 1e-5 * abs(fd), (fd, ad)
        d = np.asfortranarray(rng.standard_normal(rho0.shape))
        fd = (J_at(rho=rho0 + eps * d) - J_at(rho=rho0 - eps * d)) / (2 * eps)
        ad = float(np.sum(grad["drho"] * d))
        assert abs(fd - ad) <= 1e-5 * abs(fd), (fd, ad)


def _law_params(n=(13, 11, 9)):
    return S.sector_params(n, bc="stress", rheology="edot_power_relax", n_exp=3.0, relax=0.5, edot_bg=0.25,
                           sig_bc=(0.0, 0.5, -0.5), incl_linear=1, vr=10.0)


def test_vjp_of_the_power_law_residual_is_its_transposed_jacobian():
    """nonlinear residual (η from the strain-rate law): ⟨λ, J v⟩ with J v by central differences"""
    rng = np.random.default_rng(3)
    with S.Solver(_law_params()) as sv:
        sv.step(300)  # a state with non-trivial strain rates
        u = {f: sv.get(f) for f in FIELDS}
        v = _rand(sv, rng)
        lam = _rand(sv, rng)
        scale = max(np.abs(u[f]).max() for f in FIELDS)
        eps = 1e-6 * scale

        def R(w):
            for f in FIELDS:
                sv.set(f, w[f])
            return A.residual_fields(sv)
        rp = R({f: u[f] + eps * v[f] for f in FIELDS})
        rm = R({f: u[f] - eps * v[f] for f in FIELDS})
        Jv = {f: (rp[f] - rm[f]) / (2 * eps) for f in FIELDS}
        R(u)
        g = A.vjp(sv, lam, interior=False)
    lhs, rhs = _dot(lam, Jv), _dot(g, v)
    scale = sum(float(np.sum(np.abs(lam[f] * Jv[f]))) for f in FIELDS)
    assert abs(lhs - rhs) <= 1e-6 * scale, (lhs, rhs, scale)


def test_power_law_gradients_match_central_differences():
    p = _law_params()
    rng = np.random.default_rng(5)
    with S.Solver(p) as sv:
        _converged(sv)
        base = {f: sv.get(f) for f in ("V1", "V2", "V3", "P", "TAU11", "TAU22", "TAU33", "TAU12", "TAU13", "TAU23", "ETA")}
        grad = A.gradient(sv, tol=1e-12)
        assert grad["info"].status == S.SPH_OK, (grad["info"].status, grad["info"].err)
        ei0, rho0 = sv.get("ETA_INI"), sv.get("RHO")

        def J_at(ei=None, rho=None, n=None):
            for f, a in base.items():
                sv.set(f, a)
            sv.set("ETA_INI", ei0 if ei is None else ei)
            sv.set("RHO", rho0 if rho is None else rho)
            S.set_params(p, n_exp=3.0 if n is None else n)
            sv.update_params(p)
            _converged(sv)
            return A.surface_misfit(sv)[0]

        eps = 1e-4
        for _ in range(2):
            d = np.asfortranarray(rng.standard_normal(ei0.shape))
            fd = (J_at(ei=ei0 * np.exp(eps * d)) - J_at(ei=ei0 * np.exp(-eps * d))) / (2 * eps)
            ad = float(np.sum(grad["dlogeta_ini"] * d))
            assert abs(fd - ad) <= 1e-5 * abs(fd), ("eta_ini", fd, ad)
        fd = (J_at(n=3.0 + eps) - J_at(n=3.0 - eps)) / (2 * eps)
        assert abs(fd - grad["dn"]) <= 1e-5 * abs(fd), ("n", fd, grad["dn"])
        d = np.asfortranarray(rng.standard_normal(rho0.shape))
        fd = (J_at(rho=rho0 + eps * d) - J_at(rho=rho0 - eps * d)) / (2 * eps)
        ad = float(np.sum(grad["drho"] * d))
        assert abs(fd - ad) <= 1e-5 * abs(fd), ("rho", fd, ad)


def test_fd_check_of_the_power_law_misfit():
    """adjoint.fd_check (the bench's gradient-check leg) on a small grid: the adjoint gradient along
    seeded random directions in (log η_ini per cell, n, ρ per cell) equals central differences"""
    with S.Solver(_law_params()) as sv:
        r = A.fd_check(sv, directions=3, seed=1)
    assert len(r["directions"]) == 3 and r["forward_solves"] == 2 + 2 * 3
    assert r["max_rel_diff"] <= 1e-5, r["directions"]
