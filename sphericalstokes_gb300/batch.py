"""Batched diapir solves: the parameter sweep of many independent small solves
(grid edge per axis from {31, 47, 63, 79, 95}, coordinate system cycled
spherical / cylindrical / Cartesian, power-law exponent n in {1, 2, 3, 4},
inclusion/matrix viscosity ratio log-uniform in [1e-4, 1e-1], far-field
stress ratio uniform in [0, 1]) and its runner over ``sph_batch_solve``.

Each case is one of the reference's diapir setups (SphericalStokes_diapir.jl,
CylindricalStokes_diapir.jl, CartesianStokes_diapir.jl) with the strain-rate
power law (linear for n = 1).

PT step of the batch (``step_cap``).  The reference's step, CFL = 1/(2 + 4.5 log10 vr)
of the grid spacing (CylindricalStokes_diapir.jl:250,322), was chosen for vr = 10^2.  A
velocity node between two cells whose ηSM differ by vr takes the mean of their steps
(compute_V!, SphericalStokes_diapir.jl:315-327), about vr/2 times the step that the
stiffer cell's pressure tolerates, so the local Courant number is CFL·sqrt(vr/2): 0.64
at vr = 10^2, 1.4 at 10^3 and 3.5 at 10^4.  Draws above 10^2 then diverge within a few
hundred iterations (plain FP64 PT as well as the mixed solve).  ``step_cap`` keeps the
local Courant number at the value the reference's choice has at vr = 10^2: the step is
at most CFL(10^2)·sqrt(10^2/c) of the spacing, c the viscosity contrast of the solve's
starting state (vr, or 2 vr under the strain-rate law, whose zero-strain-rate viscosity is
twice the linear one).  The PT step does not change the discrete equations, only how fast
(and whether) the iteration reaches their solution.  The stress ratio s sets the far-field normal
stresses (0, +s/2, -s/2) on the spherical sector and the cylindrical faces; the
Cartesian scheme has no deviatoric normal stresses to load, so there s is the
simple-shear rate of the script's own boundary condition.
"""
from __future__ import annotations

import math
import time

import numpy as np

from . import Solver, default_params, make_opts, sector_params, solve_batch

EDGES = (31, 47, 63, 79, 95)
GEOMETRIES = ("spherical", "cylindrical", "cartesian")


def capped_cfl(vr: float) -> float:
    """The reference's CFL = 1/(2 + 4.5 log10 vr), limited to CFL(10^2)·sqrt(10^2/vr) (module docstring)."""
    return min(1.0 / (2.0 + 4.5 * math.log10(vr)), (1.0 / 11.0) * math.sqrt(100.0 / vr))


def sweep_cases(count: int = 256, seed: int = 0, edges=EDGES, precision: str = "mixed", step_cap: bool = True) -> list:
    """Parameters of ``count`` solves drawn with numpy's PCG64 generator from ``seed``;
    ``step_cap``: the PT step from :func:`capped_cfl` instead of the reference's CFL."""
    rng = np.random.default_rng(seed)
    cases = []
    for i in range(count):
        n = tuple(int(x) for x in rng.choice(edges, size=3))
        geom = GEOMETRIES[i % 3]
        n_exp = int(rng.integers(1, 5))
        ratio = float(10.0 ** rng.uniform(-4.0, -1.0))
        s = float(rng.uniform(0.0, 1.0))
        rheo = dict(rheology="linear") if n_exp == 1 else dict(rheology="edot_power_relax", n_exp=float(n_exp), relax=0.5,
                                                                  edot_bg=1.0)
        if geom == "spherical":
            p = sector_params(n, bc="stress", sig_bc=(0.0, 0.5 * s, -0.5 * s), vr=1.0 / ratio, incl_linear=1,
                              precision=precision, **rheo)
        elif geom == "cylindrical":
            p = default_params("cylindrical", n1=n[0], n2=n[1], n3=n[2], bc="stress", sig_bc=(0.0, 0.5 * s, -0.5 * s),
                               vr=1.0 / ratio, incl_linear=1, precision=precision, **rheo)
        else:
            p = default_params("cartesian", n1=n[0], n2=n[1], n3=n[2], bc="diapir", sh=s, vr=1.0 / ratio, incl_linear=1,
                               precision=precision, **rheo)
        if step_cap:
            cfl = 1.0 / (2.0 + 4.5 * math.log10(p.vr))
            base = p.vpdt / cfl if p.vpdt > 0 else p.l1 / (p.n1 - 1)  # the spacing the reference's step scales
            # the strain-rate law starts from twice the linear viscosity (η_t = 2/(1/η_ini + 1/η_PL)
            # at zero strain rate) over the linear inclusion: the contrast is 2 vr
            contrast = p.vr * (2.0 if n_exp > 1 else 1.0)
            p.vpdt = base * min(cfl, capped_cfl(contrast))
        cases.append(p)
    return cases


def run(cases: list, opts, threads: int = 0, autotune: bool = True, serial: bool = False) -> dict:
    """Solve every case; with ``serial`` one after another on the calling thread, else
    concurrently through ``sph_batch_solve``.  Returns wall time, solves/s and the results."""
    solvers = [Solver(p) for p in cases]
    try:
        tuned = {}
        if autotune:
            for sv in solvers:
                key = (sv.params.geometry, sv.params.n1, sv.params.n2, sv.params.n3)
                if sv.params.precision == 2 and key not in tuned:
                    tuned[key] = sv.autotune()
        if isinstance(opts, list):
            ol = opts
        else:
            ol = [opts] * len(solvers)
        t0 = time.perf_counter()
        if serial:
            res = [sv.solve(tol=o.tol, maxiter=o.maxiter, nout=o.nout, criterion={0: "reference", 1: "residual", 2: "reference_plateau"}[o.criterion],
                            inner_rtol=o.inner_rtol, max_outer=o.max_outer, inner_max=o.inner_max, warm_tol=o.warm_tol,
                            hist_cap=1) for sv, o in zip(solvers, ol)]
        else:
            res = solve_batch(solvers, ol, threads=threads)
        wall = time.perf_counter() - t0
        return {"wall_s": wall, "solves_per_s": len(solvers) / wall, "results": res, "tuned": tuned}
    finally:
        for sv in solvers:
            sv.close()


__all__ = ["sweep_cases", "capped_cfl", "run", "make_opts", "EDGES", "GEOMETRIES"]
