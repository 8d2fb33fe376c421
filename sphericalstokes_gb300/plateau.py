"""Plateau driver: the continuation of scripts_plateau/SphericalStokes_plateau.jl
(SPH_3D_Plateau, :367-600) on the library's solver.

The script's physics per PT iteration is the spherical free-slip scheme with
the stress-based power law (library: ``bc="free_slip"``,
``rheology="tau_power"``); what the driver adds is
  * the non-dimensional parameter set (:370-439),
  * the layered initial ρ and η of ``initialize_geometry!`` (:120-167): sticky
    air over a crust with a plateau of elevation ``he`` and a crustal root
    ``hr`` joined by linear ramps over the transition zone ``dt``, over a
    lithospheric mantle and the mantle,
  * the continuation schedule (:485-522): eight solves of at most ``maxiter``
    iterations; steps 2-6 raise the crust viscosity (η re-initialised in place,
    η_ini = η, pseudo-step from the new viscosity ratio), steps 7 and 8 switch
    the power-law exponent,
  * the plateau's exit check (a NaN Vφ ratio is left out, :540-552) and the
    per-step output folders ``out_plateau_<it>`` (:554-583).
"""
from __future__ import annotations

import math
import os
from dataclasses import dataclass, field

import numpy as np

from . import Params, Solver, SolveResult, set_params


def linspace(c: float, l: float, n: int) -> np.ndarray:
    """The library's node coordinates c - l/2 .. c + l/2 (its linspace, the scripts' range(a, b, length=n))."""
    lo, hi = c - l / 2.0, c + l / 2.0
    x = lo + (hi - lo) * np.arange(n, dtype=np.float64) / (n - 1)
    x[-1] = hi
    return x


@dataclass
class PlateauSetup:
    """Dimensional inputs of SPH_3D_Plateau (SphericalStokes_plateau.jl:370-399) and the grid."""
    nr: int = 70
    nth: int = 5
    nph: int = 5
    dmp: float = 4.5
    eta_m: float = 1e20          # mantle viscosity [Pa s]
    eta_l: float = 1e22          # lithospheric mantle
    eta_c: tuple = (1e20, 5e20, 1e21, 3e21, 6e21, 1e22)  # crust, continuation steps 1-6
    eta_a: float = 5e18          # sticky air
    rho_m: float = 3300.0
    rho_l: float = 3300.0
    rho_c: float = 2800.0
    rho_a: float = 0.0
    h_m: float = 360e3           # mantle thickness [m]
    h_l: float = 87e3            # lithospheric mantle
    h_r: float = 28e3            # crustal root
    h_c: float = 35e3            # crust
    h_e: float = 5e3             # plateau elevation
    h_a: float = 50e3            # sticky air
    d_l: float = 700e3           # lowland extent
    d_t: float = 100e3           # transition zone
    d_h: float = 600e3           # highland extent
    g: float = 9.81
    n_exp: float = 1.0           # steps 1-6
    n_exp_pl: float = 3.0        # step 7
    n_exp_pl2: float = 6.0       # step 8
    tau_c: float = 24e6          # reference stress of the power law [Pa]
    r: float = 6371e3            # sphere radius [m]
    extra: dict = field(default_factory=dict)

    def scaled(self) -> dict:
        """Non-dimensional values (scales: model height, mantle viscosity, mantle density; :411-439)."""
        lr_d = self.h_m + self.h_l + self.h_r + self.h_c + self.h_e + self.h_a
        sl, se, sr = lr_d, self.eta_m, self.rho_m
        s = {"sl": sl, "se": se, "sr": sr, "lr": lr_d / sl,
             "lth": (self.d_l + self.d_t + self.d_h) / self.r, "lph": (self.d_l + self.d_t + self.d_h) / self.r,
             "rho_m": self.rho_m / sr, "rho_l": self.rho_l / sr, "rho_c": self.rho_c / sr, "rho_a": self.rho_a / sr,
             "eta_m": self.eta_m / se, "eta_l": self.eta_l / se, "eta_c": tuple(x / se for x in self.eta_c),
             "eta_a": self.eta_a / se, "r": self.r / sl, "h_m": self.h_m / sl, "h_l": self.h_l / sl,
             "h_r": self.h_r / sl, "h_c": self.h_c / sl, "h_e": self.h_e / sl, "h_a": self.h_a / sl,
             "d_l": self.d_l / sl, "d_t": self.d_t / sl, "d_h": self.d_h / sl,
             "g": self.g / se ** 2 * sr ** 2 * sl ** 3, "tau_c": self.tau_c / se ** 2 * sr * sl ** 2}
        return s

    def viscosity_ratio(self, step: int) -> float:
        s = self.scaled()
        ec = s["eta_c"][min(step, 6) - 1]
        vals = (s["eta_m"], s["eta_l"], ec, s["eta_a"])
        return max(vals) / min(vals)

    def params(self, precision: str = "fp64", **kw) -> Params:
        """Library parameters of continuation step 1: the grid of :447-452 (R from r - (hc+hr+hl+hm)
        to r + lr - (hc+hr+hl+hm), θ from π/2 - dl/r to π/2 + (dt+dh)/r, φ from -dl/r to (dt+dh)/r)."""
        from . import default_params

        s = self.scaled()
        H = s["h_c"] + s["h_r"] + s["h_l"] + s["h_m"]
        r1lo, r1hi = s["r"] - H, s["r"] + s["lr"] - H
        t_lo, t_hi = math.pi / 2.0 - s["d_l"] / s["r"], math.pi / 2.0 + (s["d_t"] + s["d_h"]) / s["r"]
        p_lo, p_hi = -s["d_l"] / s["r"], (s["d_t"] + s["d_h"]) / s["r"]
        p = default_params("spherical")
        set_params(p, precision=precision, bc="free_slip", rheology="tau_power", init="none",
                   n1=self.nr, n2=self.nth, n3=self.nph,
                   c1=0.5 * (r1lo + r1hi), l1=r1hi - r1lo, c2=0.5 * (t_lo + t_hi), l2=t_hi - t_lo,
                   c3=0.5 * (p_lo + p_hi), l3=p_hi - p_lo, l_ref=s["lr"], r=s["r"], dmp=self.dmp, g=s["g"],
                   tau_C=s["tau_c"], n_exp=self.n_exp, vr=self.viscosity_ratio(1), vpdt=0.0,
                   eta0=s["eta_m"], rho0=s["rho_m"], sh=0.0)
        set_params(p, **kw)
        return p

    def coordinates(self, p: Params) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
        """Cell-centre coordinate grids R, θ, φ (n1 x n2 x n3, Fortran order) of the library's grid."""
        x1, x2, x3 = linspace(p.c1, p.l1, p.n1), linspace(p.c2, p.l2, p.n2), linspace(p.c3, p.l3, p.n3)
        R, T, F = np.meshgrid(x1, x2, x3, indexing="ij")
        return np.asfortranarray(R), np.asfortranarray(T), np.asfortranarray(F)


def initialize_geometry(A: np.ndarray, R: np.ndarray, th: np.ndarray, ph: np.ndarray, r: float, he: float, hc: float,
                        hr: float, hl: float, dt: float, gl: float, gc: float, ga: float) -> np.ndarray:
    """``initialize_geometry!`` (SphericalStokes_plateau.jl:120-167) in place: the listed
    conditions applied in the script's order, each overwriting the cells it selects
    (lithosphere ``gl``, crust and root ``gc``, sticky air above the topography ``ga``)."""
    z = R - r                       # height above the reference radius
    y = (th - math.pi / 2.0) * r    # distance along θ from the domain's θ origin
    x = ph * r                      # distance along φ
    k = hr / dt
    e = he / dt
    A[z > -hc - hr - hl] = gl
    A[(z > -hc) & (y < 0)] = gc
    A[(z > -hc) & (x > 0)] = gc
    A[(z > -hc - hr) & (y >= dt) & (x <= -dt)] = gc
    A[(z > -hc + k * ph * r) & (y >= dt) & (x <= 0) & (x >= -dt)] = gc
    A[(z > -hc + k * (math.pi / 2.0 - th) * r) & (y >= 0) & (y <= dt) & (x <= -dt)] = gc
    A[(z > np.maximum(-hc + k * (math.pi / 2.0 - th) * r, -hc + k * ph * r)) & (y >= 0) & (y <= dt) & (x <= 0) & (x >= -dt)] = gc
    A[(z > 0) & (y < 0)] = ga
    A[(z > 0) & (x > 0)] = ga
    A[(z > he) & (y >= dt) & (x <= -dt)] = ga
    A[(z > -(e * ph * r)) & (y >= dt) & (x <= 0) & (x >= -dt)] = ga
    A[(z > -(e * (math.pi / 2.0 - th) * r)) & (y >= 0) & (y <= dt) & (x <= -dt)] = ga
    A[(z > np.minimum(-(e * (math.pi / 2.0 - th) * r), -(e * ph * r))) & (y >= 0) & (y <= dt) & (x <= 0) & (x >= -dt)] = ga
    return A


def initial_fields(setup: PlateauSetup, p: Params) -> tuple[np.ndarray, np.ndarray]:
    """ρ and η of step 1 (:484-485): ρm / ηm everywhere, then the layers."""
    s = setup.scaled()
    R, T, F = setup.coordinates(p)
    geo = dict(r=s["r"], he=s["h_e"], hc=s["h_c"], hr=s["h_r"], hl=s["h_l"], dt=s["d_t"])
    rho = initialize_geometry(np.full(R.shape, s["rho_m"], order="F"), R, T, F, gl=s["rho_l"], gc=s["rho_c"], ga=s["rho_a"], **geo)
    eta = initialize_geometry(np.full(R.shape, s["eta_m"], order="F"), R, T, F, gl=s["eta_l"], gc=s["eta_c"][0], ga=s["eta_a"], **geo)
    return rho, eta


def reset_crust_viscosity(setup: PlateauSetup, p: Params, eta: np.ndarray, step: int) -> np.ndarray:
    """Continuation steps 2-6 (:487-516): η re-initialised in place with the crust value of the step."""
    s = setup.scaled()
    R, T, F = setup.coordinates(p)
    return initialize_geometry(eta, R, T, F, r=s["r"], he=s["h_e"], hc=s["h_c"], hr=s["h_r"], hl=s["h_l"], dt=s["d_t"],
                               gl=s["eta_l"], gc=s["eta_c"][step - 1], ga=s["eta_a"])


def _phys_line(setup: PlateauSetup, step: int, n_exp: float, vr: float, dmp: float) -> str:
    """Save_phys of the plateau script (:28-35): 23 values, the scaled quantities under the _d names."""
    s = setup.scaled()
    vals = [s["sl"], s["se"], s["sr"], s["eta_m"], s["eta_l"], s["eta_c"][min(step, 6) - 1], s["eta_a"], s["rho_m"], s["rho_l"],
            s["rho_c"], s["rho_a"], s["h_m"], s["h_l"], s["h_r"], s["h_c"], s["h_e"], n_exp, s["tau_c"], vr, s["g"] * 1e15,
            s["r"], dmp]
    return "%d " % 1 + " ".join("%f" % v for v in vals)


def run(setup: PlateauSetup, precision: str = "fp64", steps: int = 8, maxiter: int = 200, nout: int = 10,
        tol: float = 5e-7, out_root: str | os.PathLike | None = None, solver: Solver | None = None) -> list[SolveResult]:
    """The continuation of :486-584 on one solver; returns the result of each step.  With
    ``out_root``, step ``it`` is written to ``out_root/out_plateau_<it>`` in the script's format."""
    p = setup.params(precision)
    own = solver is None
    sv = Solver(p) if own else solver
    try:
        rho, eta = initial_fields(setup, p)
        sv.set("RHO", rho)
        sv.set("ETA", eta)
        sv.set("ETA_INI", eta)
        results = []
        n_exp = setup.n_exp
        for it in range(1, steps + 1):
            if 2 <= it <= 6:
                eta = reset_crust_viscosity(setup, p, sv.get("ETA"), it)
                sv.set("ETA", eta)
                sv.set("ETA_INI", eta)
                set_params(p, vr=setup.viscosity_ratio(it), vpdt=0.0)
                sv.update_params(p)
            elif it in (7, 8):
                n_exp = setup.n_exp_pl if it == 7 else setup.n_exp_pl2
                set_params(p, n_exp=n_exp)
                sv.update_params(p)
            res = sv.solve(tol=tol, maxiter=maxiter, nout=nout, criterion="reference_plateau")
            results.append(res)
            if out_root is not None:
                d = os.path.join(os.fspath(out_root), f"out_plateau_{it}")
                sv.save(d, num=1, tol=tol * 1e7, runtime=0.0, result=res)
                with open(os.path.join(d, "1_phys.inf"), "w") as f:
                    f.write(_phys_line(setup, it, n_exp, setup.viscosity_ratio(it), setup.dmp))
        return results
    finally:
        if own:
            sv.close()


# ---------------------------------------------------------------------------
# Elliptical plateau on a curved shell (a larger plateau experiment built on the same
# solver): crust of 35 km outside and 70 km inside an elliptical plateau (semi-axes
# 12° x 6°) with a cos² taper over 2°, a seeded Gaussian random density perturbation,
# a power-law crust over a linear mantle; the topography load enters through a sticky-air
# layer above the reference surface, as in the reference plateau experiment.
@dataclass
class EllipsePlateau:
    nr: int = 511
    nth: int = 255
    nph: int = 255
    R_km: float = 6371.0
    depth_km: float = 200.0
    air_km: float = 20.0            # sticky-air layer above the reference surface
    extent_deg: float = 40.0        # θ and φ extent
    semi_deg: tuple = (12.0, 6.0)   # ellipse semi-axes along θ and φ
    taper_deg: float = 2.0
    crust_km: tuple = (35.0, 70.0)  # outside / inside the plateau
    rho_crust: float = 2800.0
    rho_mantle: float = 3300.0
    rho_air: float = 0.0
    drho_frac: float = 0.02         # amplitude of the random density perturbation
    corr_km: float = 20.0           # correlation length of the random field
    seed: int = 0
    n_exp: float = 3.0
    eta_ratio: float = 1e-2         # crust / mantle viscosity
    eta_air: float = 1e-3           # air / mantle viscosity
    dmp: float = 4.5
    # "sticky_air": an air layer of air_km above the reference surface carries the topography;
    # "free_surface": the domain ends at the reference surface, whose traction carries the load of
    # the plateau's isostatic topography h = (ρ_mantle - ρ_crust)/ρ_crust (h_crust - h_crust,outside)
    # (SPH_BC_FREE_SURFACE) with the stabilisation term θ Δt ρ_crust g V_r
    top: str = "sticky_air"
    fs_theta_dt: float = 0.5        # θ Δt of the stabilisation, in units of η_mantle / (ρ_mantle g depth)

    def params(self, precision: str = "mixed", **kw) -> Params:
        """Spherical shell r in [R - depth, R + air], scaled by the depth; stress-free
        mantle-scale units (η_mantle = 1, ρ_mantle = 1, g = 1)."""
        from . import default_params

        L = self.depth_km
        fs = self.top == "free_surface"
        r0, r1 = (self.R_km - self.depth_km) / L, (self.R_km + (0.0 if fs else self.air_km)) / L
        ext = math.radians(self.extent_deg)
        p = default_params("spherical")
        vr = 1.0 / (self.eta_ratio if fs else min(self.eta_ratio, self.eta_air))
        set_params(p, precision=precision, bc="free_surface" if fs else "free_slip", rheology="edot_power_relax",
                   n_exp=self.n_exp, relax=0.5, edot_bg=1.0, init="none", n1=self.nr, n2=self.nth, n3=self.nph,
                   c1=0.5 * (r0 + r1), l1=r1 - r0, c2=math.pi / 2, l2=ext, c3=0.0, l3=ext, l_ref=r1 - r0, r=self.R_km / L,
                   dmp=self.dmp, g=1.0, vr=vr, vpdt=0.0, eta0=1.0, rho0=1.0, sh=0.0, incl_linear=1,
                   fs_kappa=self.fs_theta_dt * self.rho_crust / self.rho_mantle if fs else 0.0)
        set_params(p, **kw)
        return p

    def crust_thickness_km(self, th: np.ndarray, ph: np.ndarray) -> np.ndarray:
        """35 km outside, 70 km inside the ellipse, cos² taper over ``taper_deg`` outside its edge
        (distance measured along the ray from the centre in the ellipse's own scaling)."""
        a, b = (math.radians(x) for x in self.semi_deg)
        dth, dph = th - math.pi / 2, ph
        e = np.sqrt((dth / a) ** 2 + (dph / b) ** 2)          # 1 on the ellipse
        rad = np.sqrt(dth ** 2 + dph ** 2)
        edge = np.where(e > 0, rad / np.maximum(e, 1e-300), a)  # ellipse radius along this ray
        dist = np.degrees(np.maximum(e - 1.0, 0.0) * edge)      # angular distance beyond the edge
        w = np.where(e <= 1.0, 1.0, np.where(dist < self.taper_deg, np.cos(0.5 * math.pi * dist / self.taper_deg) ** 2, 0.0))
        return self.crust_km[0] + (self.crust_km[1] - self.crust_km[0]) * w

    def random_field(self, shape: tuple, spacing_km: tuple) -> np.ndarray:
        """Seeded Gaussian random field (PCG64 white noise smoothed by a Gaussian kernel of
        ``corr_km``), scaled to max |f| = 1."""
        rng = np.random.default_rng(self.seed)
        f = rng.standard_normal(shape)
        F = np.fft.rfftn(f)
        k = [np.fft.fftfreq(n, d=h) for n, h in zip(shape[:-1], spacing_km[:-1])] + [np.fft.rfftfreq(shape[-1], d=spacing_km[-1])]
        K2 = sum(np.meshgrid(*[kk ** 2 for kk in k], indexing="ij"))
        F *= np.exp(-0.5 * (2 * math.pi) ** 2 * K2 * self.corr_km ** 2)
        g = np.fft.irfftn(F, s=shape, axes=tuple(range(len(shape))))
        return g / np.abs(g).max()

    def fields(self, p: Params) -> dict:
        """ρ, η_ini and the phase flag (1: linear mantle / air) in the reference layout."""
        L = self.depth_km
        x1, x2, x3 = linspace(p.c1, p.l1, p.n1), linspace(p.c2, p.l2, p.n2), linspace(p.c3, p.l3, p.n3)
        R, T, F = np.meshgrid(x1, x2, x3, indexing="ij")
        depth = (self.R_km / L - R) * L                       # km below the reference surface
        hc = self.crust_thickness_km(T, F)
        air, crust = depth < 0.0, (depth >= 0.0) & (depth < hc)
        rm = 1.0
        rho = np.full(R.shape, rm)
        rho[crust] = self.rho_crust / self.rho_mantle
        rho[air] = self.rho_air / self.rho_mantle
        mid = self.R_km - 0.5 * self.depth_km
        sp = (p.l1 * L / (p.n1 - 1), p.l2 * mid / (p.n2 - 1), p.l3 * mid / (p.n3 - 1))
        noise = self.random_field(R.shape, sp)
        rho = np.where(air, rho, rho * (1.0 + self.drho_frac * noise))
        eta = np.ones(R.shape)
        eta[crust] = self.eta_ratio
        eta[air] = self.eta_air
        phase = np.where(crust, 0.0, 1.0)
        out = {"RHO": np.asfortranarray(rho), "ETA_INI": np.asfortranarray(eta), "ETA": np.asfortranarray(eta),
               "PHASE": np.asfortranarray(phase)}
        if self.top == "free_surface":
            out["TOP_LOAD"] = np.asfortranarray(self.surface_load(p))
        return out

    def topography_km(self, th: np.ndarray, ph: np.ndarray) -> np.ndarray:
        """Isostatic (Airy) elevation of the plateau: h = (ρ_mantle - ρ_crust)/ρ_crust times the crust
        thickness in excess of the outside value."""
        excess = self.crust_thickness_km(th, ph) - self.crust_km[0]
        return (self.rho_mantle - self.rho_crust) / self.rho_crust * excess

    def surface_load(self, p: Params) -> np.ndarray:
        """SPH_FIELD_TOP_LOAD of the free-surface top: ρ_crust g h on the top cells (units ρ_mantle g depth),
        zero below."""
        x2, x3 = linspace(p.c2, p.l2, p.n2), linspace(p.c3, p.l3, p.n3)
        T, F = np.meshgrid(x2, x3, indexing="ij")
        q = np.zeros((p.n1, p.n2, p.n3), order="F")
        q[p.n1 - 1] = self.rho_crust / self.rho_mantle * self.topography_km(T, F) / self.depth_km
        return q


def ellipse_solver(setup: EllipsePlateau, precision: str = "mixed", **kw) -> Solver:
    """A solver holding the elliptical-plateau fields."""
    p = setup.params(precision, **kw)
    sv = Solver(p)
    for f, a in setup.fields(p).items():
        sv.set(f, a)
    return sv
