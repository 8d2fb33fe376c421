"""Adjoint of the FP64 Stokes residual: gradients of an objective of the
converged velocities with respect to the per-cell viscosity and density.

With R(u; η, ρ) = 0 the discrete Stokes equations of the current state
(u = interior velocities and pressures), an objective J(u) has

    dJ/dη = -λᵀ ∂R/∂η,   dJ/dρ = -λᵀ ∂R/∂ρ,   where  (∂R/∂u)ᵀ λ = (∂J/∂u)ᵀ.

``sph_residual_vjp`` applies (∂R/∂u)ᵀ and the two contractions with the
hand-written transposed stencils; ``sph_adjoint_solve`` solves for λ with the
forward PT scheme's pseudo-steps on the transposed rows.  For the linear
rheology the viscosity is the parameter; for the strain-rate power law the
Jacobian includes η's dependence on V and the gradients are with respect to the
per-cell prefactor η_ini and the exponent n (``law_vjp``).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import SPH_ERR_DIVERGED, SPH_ERR_NOT_CONVERGED, SPH_OK, SolveInfo, Solver, _check, make_opts

_PD = C.POINTER(C.c_double)
VEL = ("V1", "V2", "V3")


def _ptr(a):
    return a.ctypes.data_as(_PD) if a is not None else None


def _empty(sv: Solver, name: str) -> np.ndarray:
    return np.zeros(sv.dims(name), dtype=np.float64, order="F")


def _fortran(a) -> np.ndarray | None:
    return None if a is None else np.asfortranarray(a, dtype=np.float64)


def residual_fields(sv: Solver) -> dict:
    """R_V (interior nodes) and R_P = div V of the current state, in the reference layout."""
    out = {f: _empty(sv, f) for f in VEL + ("P",)}
    _check(sv.lib, sv.lib.sph_residual_fields(sv._h, *[_ptr(out[f]) for f in VEL + ("P",)]), "sph_residual_fields")
    return out


def vjp(sv: Solver, lam: dict, interior: bool = True) -> dict:
    """(∂R/∂(V, P))ᵀ λ and the η, ρ contractions; ``interior``: with respect to the interior
    velocities (the BC program composed in), else to every velocity entry."""
    ins = [_fortran(lam.get(f)) for f in VEL + ("P",)]
    out = {f: _empty(sv, f) for f in VEL + ("P",)}
    out["ETA"] = _empty(sv, "P")
    out["RHO"] = _empty(sv, "P")
    _check(sv.lib, sv.lib.sph_residual_vjp(sv._h, *[_ptr(a) for a in ins], *[_ptr(out[f]) for f in VEL + ("P", "ETA", "RHO")],
                                           1 if interior else 0), "sph_residual_vjp")
    return out


def law_vjp(sv: Solver) -> tuple[np.ndarray, float]:
    """After :func:`vjp`: its η contraction through the viscosity law — per cell (∂R/∂η_ini)ᵀλ
    and the total (∂R/∂n)ᵀλ (``sph_residual_vjp_law``)."""
    g = _empty(sv, "P")
    gn = C.c_double()
    _check(sv.lib, sv.lib.sph_residual_vjp_law(sv._h, _ptr(g), C.byref(gn)), "sph_residual_vjp_law")
    return g, float(gn.value)


def adjoint_solve(sv: Solver, b: dict, tol: float = 1e-10, maxiter: int = 1_000_000, nout: int = 500, lam0: dict | None = None):
    """λ with (∂R/∂u)ᵀ λ = b (interior-unknown form); returns (λ, SolveInfo)."""
    bs = [_fortran(b.get(f)) for f in VEL + ("P",)]
    lam = {f: (np.array(lam0[f], dtype=np.float64, order="F", copy=True) if lam0 and f in lam0 else _empty(sv, f))
           for f in VEL + ("P",)}
    info = SolveInfo()
    o = make_opts(tol=tol, maxiter=maxiter, nout=nout)
    rc = sv.lib.sph_adjoint_solve(sv._h, *[_ptr(a) for a in bs], *[_ptr(lam[f]) for f in VEL + ("P",)], C.byref(o), C.byref(info))
    if rc not in (SPH_OK, SPH_ERR_NOT_CONVERGED, SPH_ERR_DIVERGED):
        _check(sv.lib, rc, "sph_adjoint_solve")
    return lam, info


def surface_misfit(sv: Solver, v_obs: np.ndarray | None = None) -> tuple[float, dict]:
    """J = 1/2 Σ (V_r - V_obs)² over the interior nodes of the outermost interior radial face
    (i = n1 - 1, θ and φ indices 1 .. n-2); returns J and ∂J/∂u."""
    V1 = sv.get("V1")
    n1 = V1.shape[0] - 1
    s = V1[n1 - 1, 1:-1, 1:-1]
    obs = 0.0 if v_obs is None else v_obs
    r = s - obs
    b = {"V1": np.zeros_like(V1)}
    b["V1"][n1 - 1, 1:-1, 1:-1] = r
    return 0.5 * float(np.sum(r * r)), b


def gradient(sv: Solver, objective=surface_misfit, tol: float = 1e-10, maxiter: int = 1_000_000) -> dict:
    """dJ/d(log η) and dJ/dρ per cell at the current (converged) state."""
    J, b = objective(sv)
    lam, info = adjoint_solve(sv, b, tol=tol, maxiter=maxiter)
    g = vjp(sv, lam, interior=True)
    g_ini, g_n = law_vjp(sv)
    eta, eta_ini = sv.get("ETA"), sv.get("ETA_INI")
    return {"J": J, "dlogeta": -eta * g["ETA"], "dlogeta_ini": -eta_ini * g_ini, "dn": -g_n, "drho": -g["RHO"],
            "lambda": lam, "info": info}
