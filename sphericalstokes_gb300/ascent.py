"""Diapir ascent: Stokes solves alternating with explicit advection of the
density and viscosity fields, and the gradient of an objective of the final
velocities with respect to the initial fields by the adjoint through time with
checkpoint-and-recompute.

Per step t: fields F_t = (ρ_t, L_t), L = log η_ini (log η for the linear
rheology); u_t solves R(u_t; F_t) = 0; dt_t from the CFL number; F_{t+1} =
Adv(F_t; u_t, dt_t) (``sph_advect``, upwinding with a smoothed |v| so that
the step is differentiable).  The objective J depends on the last
solve's velocities.  Reverse sweep, from μ_T = 0:

    a_t  = (∂F_{t+1}/∂u_t)ᵀ μ_{t+1}            (sph_advect_vjp, then sph_bc_vjp)
    λ_t  : (∂R/∂u)ᵀ λ_t = ∂J/∂u_t + a_t        (sph_adjoint_solve)
    μ_t  = (∂F_{t+1}/∂F_t)ᵀ μ_{t+1} - (∂R/∂F_t)ᵀ λ_t

The fields are stored every ``checkpoint_every`` steps; a segment's states are
recomputed from its checkpoint during the reverse sweep.  The time steps and
smoothing scales are those of the forward run (their dependence on u is not
differentiated).
The scripts of the reference run a single time step, so this has no
counterpart there.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import RHEO, Solver, _check
from . import adjoint as A

_PD = C.POINTER(C.c_double)
STATE = ("V1", "V2", "V3", "P", "TAU11", "TAU22", "TAU33", "TAU12", "TAU13", "TAU23", "ETA")


def _law(sv: Solver) -> bool:
    return sv.params.rheology == RHEO["edot_power_relax"]


def set_fields(sv: Solver, F: tuple[np.ndarray, np.ndarray]) -> None:
    rho, L = F
    sv.set("RHO", rho)
    eta = np.exp(L)
    sv.set("ETA_INI", eta)
    if not _law(sv):
        sv.set("ETA", eta)


def get_fields(sv: Solver) -> tuple[np.ndarray, np.ndarray]:
    return sv.get("RHO"), np.log(sv.get("ETA_INI"))


def _ptrs(arrs):
    return (_PD * len(arrs))(*[a.ctypes.data_as(_PD) for a in arrs])


def advect(sv: Solver, F, dt: float, delta: float = 0.0):
    ins = [np.asfortranarray(a, dtype=np.float64) for a in F]
    outs = [np.zeros_like(a, order="F") for a in ins]
    _check(sv.lib, sv.lib.sph_advect(sv._h, float(dt), float(delta), len(ins), _ptrs(ins), _ptrs(outs)), "sph_advect")
    return tuple(outs)


def advect_vjp(sv: Solver, F, mu_new, dt: float, delta: float = 0.0):
    ins = [np.asfortranarray(a, dtype=np.float64) for a in F]
    mus = [np.asfortranarray(a, dtype=np.float64) for a in mu_new]
    outs = [np.zeros_like(a, order="F") for a in ins]
    av = {f: np.zeros(sv.dims(f), order="F") for f in A.VEL}
    _check(sv.lib, sv.lib.sph_advect_vjp(sv._h, float(dt), float(delta), len(ins), _ptrs(ins), _ptrs(mus), _ptrs(outs),
                                         *[av[f].ctypes.data_as(_PD) for f in A.VEL]), "sph_advect_vjp")
    return tuple(outs), av


def velocity_scale(sv: Solver) -> float:
    return max(float(np.abs(sv.get(f)).max()) for f in A.VEL)


def bc_vjp(sv: Solver, av: dict) -> dict:
    out = {f: np.array(av[f], dtype=np.float64, order="F", copy=True) for f in A.VEL}  # Fortran order: raw pointers follow
    _check(sv.lib, sv.lib.sph_bc_vjp(sv._h, *[out[f].ctypes.data_as(_PD) for f in A.VEL]), "sph_bc_vjp")
    return out


def cfl_dt(sv: Solver, cfl: float = 0.5) -> float:
    """dt with dt Σ_d |v_d| a_d <= cfl in every cell (cell-mean velocities, the advection's metric)."""
    p = sv.params
    V1, V2, V3 = sv.get("V1"), sv.get("V2"), sv.get("V3")
    v1, v2, v3 = 0.5 * (V1[:-1] + V1[1:]), 0.5 * (V2[:, :-1] + V2[:, 1:]), 0.5 * (V3[:, :, :-1] + V3[:, :, 1:])
    from .plateau import linspace
    x1, x2 = linspace(p.c1, p.l1, p.n1), linspace(p.c2, p.l2, p.n2)
    d1, d2, d3 = (p.n1 - 1) / p.l1, (p.n2 - 1) / p.l2, (p.n3 - 1) / p.l3
    a1 = d1
    a2 = d2 / x1[:, None, None] if p.geometry != 2 else d2
    a3 = d3 / (x1[:, None, None] * np.sin(x2)[None, :, None]) if p.geometry == 0 else d3
    rate = np.abs(v1) * a1 + np.abs(v2) * a2 + np.abs(v3) * a3
    return cfl / float(rate.max())


def _solve(sv: Solver, tol: float, maxiter: int):
    r = sv.solve(tol=tol, maxiter=maxiter, nout=200, criterion="residual", hist_cap=1)
    if not r.converged:
        raise RuntimeError(f"Stokes solve did not converge: status {r.status}, residual {r.residual:.3e}")
    return r


def forward(sv: Solver, F0, nsteps: int, objective=A.surface_misfit, dts=None, deltas=None, cfl: float = 0.5,
            checkpoint_every: int = 5, smooth: float = 0.05, tol: float = 1e-12, maxiter: int = 2_000_000) -> dict:
    """nsteps solve+advect steps from F0; returns J, the time steps, the |v| smoothing scales
    (``smooth`` × max|V| of each step unless given) and the checkpoints."""
    F = tuple(np.array(a, dtype=np.float64, order="F", copy=True) for a in F0)
    checkpoints, used, dl = {}, [], []
    J = None
    for t in range(nsteps):
        if t % checkpoint_every == 0:
            checkpoints[t] = tuple(np.array(a, order="F", copy=True) for a in F)
        set_fields(sv, F)
        _solve(sv, tol, maxiter)
        if t == nsteps - 1:
            J = objective(sv)[0]
        dt = dts[t] if dts is not None else cfl_dt(sv, cfl)
        delta = deltas[t] if deltas is not None else smooth * velocity_scale(sv)
        used.append(dt)
        dl.append(delta)
        F = advect(sv, F, dt, delta)
    return {"J": J, "dts": used, "deltas": dl, "checkpoints": checkpoints, "F_final": F}


def gradient(sv: Solver, F0, nsteps: int, objective=A.surface_misfit, dts=None, deltas=None, cfl: float = 0.5,
             checkpoint_every: int = 5, smooth: float = 0.05, tol: float = 1e-12, adj_tol: float = 1e-11,
             maxiter: int = 2_000_000) -> dict:
    """dJ/dρ_0 and dJ/dL_0 by the adjoint through time with checkpoint-and-recompute (time steps
    and smoothing scales of the forward run held fixed)."""
    fwd = forward(sv, F0, nsteps, objective, dts, deltas, cfl, checkpoint_every, smooth, tol, maxiter)
    dts, deltas = fwd["dts"], fwd["deltas"]
    mu = tuple(np.zeros_like(a, order="F") for a in F0)
    law = _law(sv)
    solves = {"forward": nsteps, "recompute": 0, "adjoint": 0}
    for s0 in sorted(fwd["checkpoints"], reverse=True):
        s1 = min(s0 + checkpoint_every, nsteps)
        F = fwd["checkpoints"][s0]
        seg = []
        for t in range(s0, s1):  # recompute the segment's states
            set_fields(sv, F)
            _solve(sv, tol, maxiter)
            solves["recompute"] += 1
            seg.append((F, {f: sv.get(f) for f in STATE}))
            F = advect(sv, F, dts[t], deltas[t])
        for t in reversed(range(s0, s1)):
            Ft, state = seg[t - s0]
            set_fields(sv, Ft)
            for f, a in state.items():
                sv.set(f, a)
            mu_old, av = advect_vjp(sv, Ft, mu, dts[t], deltas[t])
            b = bc_vjp(sv, av)
            if t == nsteps - 1:
                _, bj = objective(sv)
                for f, a in bj.items():
                    b[f] = b.get(f, 0.0) + a
            lam, info = A.adjoint_solve(sv, b, tol=adj_tol, maxiter=maxiter)
            solves["adjoint"] += 1
            if info.status != 0:
                raise RuntimeError(f"adjoint solve did not converge: status {info.status}, err {info.err:.3e}")
            g = A.vjp(sv, lam, interior=True)
            g_ini, _ = A.law_vjp(sv)
            eta_par = np.exp(Ft[1])
            gL = eta_par * (g_ini if law else g["ETA"])
            mu = (mu_old[0] - g["RHO"], mu_old[1] - gL)
    return {"J": fwd["J"], "drho0": mu[0], "dL0": mu[1], "dts": dts, "deltas": deltas, "solves": solves}
