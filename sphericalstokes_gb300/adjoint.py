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


STATE = ("V1", "V2", "V3", "P", "TAU11", "TAU22", "TAU33", "TAU12", "TAU13", "TAU23", "ETA")


def fd_check(sv: Solver, directions: int = 16, seed: int = 0, sigma: float = 0.1, eps: float = 1e-4, tol: float = 1e-12,
             maxiter: int = 2_000_000) -> dict:
    """The gradient check of a surface-velocity misfit for a power-law solve (strain-rate law):
    the observation is the surface V_r of a forward solve with log η_ini perturbed by a seeded
    Gaussian field of standard deviation ``sigma``; J = 1/2 Σ (V_r - V_obs)² at the unperturbed
    parameters.  The adjoint gradient with respect to (log η_ini per cell, n, ρ per cell) is
    compared with central differences of J along ``directions`` seeded random directions, each
    J from a forward solve converged to FP64 residual ``tol`` from the base state."""
    import time

    p = sv.params
    rng = np.random.default_rng(seed)
    ei0, rho0, n0 = sv.get("ETA_INI"), sv.get("RHO"), float(p.n_exp)
    t0 = time.perf_counter()
    solves = 0

    def converge():
        nonlocal solves
        r = sv.solve(tol=tol, maxiter=maxiter, nout=500, criterion="residual")
        solves += 1
        if not r.converged:
            raise RuntimeError(f"forward solve not converged: status {r.status}, residual {r.residual:.3e}")

    # the observation: a forward run with perturbed log η_ini
    sv.set("ETA_INI", ei0 * np.exp(sigma * rng.standard_normal(ei0.shape)))
    converge()
    v1 = sv.get("V1")
    v_obs = v1[v1.shape[0] - 2, 1:-1, 1:-1].copy()
    sv.set("ETA_INI", ei0)
    converge()
    base = {f: sv.get(f) for f in STATE}
    t_fwd = time.perf_counter()
    grad = gradient(sv, objective=lambda s: surface_misfit(s, v_obs), tol=1e-12, maxiter=maxiter)
    t_adj = time.perf_counter()
    if grad["info"].status != SPH_OK:
        raise RuntimeError(f"adjoint solve not converged: status {grad['info'].status}")

    def J_at(de, dn, dr, s):
        for f, a in base.items():
            sv.set(f, a)
        sv.set("ETA_INI", ei0 * np.exp(s * eps * de))
        sv.set("RHO", rho0 + s * eps * dr)
        p.n_exp = n0 + s * eps * dn
        sv.update_params(p)
        converge()
        return surface_misfit(sv, v_obs)[0]

    rows = []
    for _ in range(directions):
        de = np.asfortranarray(rng.standard_normal(ei0.shape))
        dr = np.asfortranarray(rng.standard_normal(rho0.shape))
        dn = float(rng.standard_normal())
        ad = float(np.sum(grad["dlogeta_ini"] * de)) + grad["dn"] * dn + float(np.sum(grad["drho"] * dr))
        fd = (J_at(de, dn, dr, 1.0) - J_at(de, dn, dr, -1.0)) / (2.0 * eps)
        rows.append({"fd": fd, "adjoint": ad, "rel_diff": abs(fd - ad) / max(abs(fd), 1e-300)})
    for f, a in base.items():  # back to the base state and parameters
        sv.set(f, a)
    p.n_exp = n0
    sv.update_params(p)
    return {"J": grad["J"], "directions": rows, "max_rel_diff": max(r["rel_diff"] for r in rows),
            "adjoint_iterations": int(grad["info"].iters), "forward_solves": solves,
            "seconds": {"forward": round(t_fwd - t0, 2), "adjoint": round(t_adj - t_fwd, 2),
                        "fd": round(time.perf_counter() - t_adj, 2)}}
