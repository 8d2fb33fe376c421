"""Elliptical plateau set-up: crust thickness with the cos² taper, the seeded random
density field, layering and phases (CPU); a mixed-precision solve on a reduced grid
reduces the FP64 residual (GPU)."""
import math

import numpy as np
import pytest

import sphericalstokes_gb300 as S
from sphericalstokes_gb300 import plateau as PL


def test_crust_thickness_ellipse_and_taper():
    e = PL.EllipsePlateau()
    c = math.pi / 2
    r = math.radians
    th = np.array([c, c + r(11.9), c + r(12.1), c + r(13.0), c + r(14.5), c, c])
    ph = np.array([0.0, 0.0, 0.0, 0.0, 0.0, r(5.9), r(8.5)])
    h = e.crust_thickness_km(th, ph)
    assert h[0] == 70.0 and h[1] == 70.0 and h[5] == 70.0      # inside
    assert 35.0 < h[3] < h[2] < 70.0                             # within the 2° taper, decreasing
    assert h[4] == 35.0 and h[6] == 35.0                         # beyond the taper
    assert h[2] == pytest.approx(35.0 + 35.0 * math.cos(0.5 * math.pi * 0.1 / 2.0) ** 2, rel=1e-12)


def test_random_field_is_seeded_and_smooth():
    e = PL.EllipsePlateau(seed=0)
    f1 = e.random_field((24, 20, 16), (5.0, 30.0, 30.0))
    f2 = PL.EllipsePlateau(seed=0).random_field((24, 20, 16), (5.0, 30.0, 30.0))
    f3 = PL.EllipsePlateau(seed=1).random_field((24, 20, 16), (5.0, 30.0, 30.0))
    np.testing.assert_array_equal(f1, f2)
    assert np.abs(f1 - f3).max() > 0.1
    assert np.abs(f1).max() == pytest.approx(1.0)
    # neighbours along the finely spaced axis are strongly correlated (correlation length 20 km >> 5 km)
    assert np.corrcoef(f1[:-1].ravel(), f1[1:].ravel())[0, 1] > 0.9


def test_fields_layering():
    e = PL.EllipsePlateau(nr=41, nth=21, nph=21)
    p = e.params()
    f = e.fields(p)
    rho, eta, phase = f["RHO"], f["ETA_INI"], f["PHASE"]
    assert rho.shape == (41, 21, 21)
    assert set(np.unique(eta)) == {1.0, e.eta_ratio, e.eta_air}
    crust = phase == 0
    assert crust.any() and (~crust).any()
    assert np.all(np.abs(rho[crust] / (e.rho_crust / e.rho_mantle) - 1.0) <= e.drho_frac + 1e-12)
    assert rho[-1].max() == 0.0   # sticky air at the top row
    # the plateau's crust is thicker: more crust cells in the centre column than at a corner column
    assert crust[:, 10, 10].sum() > crust[:, 0, 0].sum()


@pytest.mark.gpu
def test_mixed_solve_on_a_reduced_plateau_grid():
    e = PL.EllipsePlateau(nr=47, nth=31, nph=31)
    with PL.ellipse_solver(e, "mixed") as sv:
        r0 = sv.residual()["err"]
        res = sv.solve(tol=1e-8, maxiter=400000, nout=100, criterion="residual", inner_rtol=1e-2, max_outer=30, inner_max=20000)
        # a viscosity contrast of 1e3 (air / mantle) and n = 3: a bounded budget, an order of magnitude
        assert np.isfinite(res.residual) and res.residual < 0.1 * r0, (r0, res.residual, res.status)


def test_free_surface_fields_and_load():
    """top="free_surface": no air cells, the domain ends at the reference surface, and the top cells
    carry the isostatic load of the plateau (70 km crust inside: (3300-2800)/2800 x 35 km = 6.25 km of
    topography, ρ_crust g h in units of ρ_mantle g depth); outside the taper the load is zero"""
    e = PL.EllipsePlateau(nr=41, nth=21, nph=21, top="free_surface")
    p = e.params()
    assert p.bc == S.BC["free_surface"] and p.fs_kappa > 0.0
    assert abs((p.c1 + 0.5 * p.l1) - e.R_km / e.depth_km) < 1e-12
    f = e.fields(p)
    assert f["RHO"].min() > 0.5  # crust and mantle only
    q = f["TOP_LOAD"]
    assert np.all(q[:-1] == 0.0)
    peak = e.rho_crust / e.rho_mantle * (e.rho_mantle - e.rho_crust) / e.rho_crust * 35.0 / e.depth_km
    assert abs(q[-1, 10, 10] - peak) < 1e-12 and q[-1, 0, 0] == 0.0


@pytest.mark.gpu
def test_mixed_solve_on_a_reduced_free_surface_plateau():
    e = PL.EllipsePlateau(nr=47, nth=31, nph=31, top="free_surface")
    with PL.ellipse_solver(e, "mixed") as sv:
        r0 = sv.residual()["err"]
        res = sv.solve(tol=1e-8, maxiter=400000, nout=100, criterion="residual", inner_rtol=1e-2, max_outer=30, inner_max=20000)
        assert np.isfinite(res.residual) and res.residual < 0.1 * r0, (r0, res.residual, res.status)
        v = [sv.get(f) for f in ("V1", "V2", "V3")]
    assert all(np.isfinite(a).all() for a in v) and max(np.abs(a).max() for a in v) > 0.0
