"""Diapir ascent (solve + advection steps) and its adjoint through time with
checkpoint-and-recompute: the advection transpose by a dot-product test, and the
gradient of the final surface-velocity misfit with respect to the initial
density and log-viscosity fields against central finite differences."""
import numpy as np
import pytest

import sphericalstokes_gb300 as S
from sphericalstokes_gb300 import ascent as AS

pytestmark = pytest.mark.gpu


def _params():
    # grid off-centre from the inclusion: no symmetry plane where the cell-mean velocities
    # vanish and a perturbation would flip the upwind direction (not differentiable there)
    import math
    return S.sector_params((13, 11, 9), bc="free_slip", rheology="linear", vr=10.0, c2=math.pi / 2 + 0.11, c3=0.07)


def test_advection_transpose():
    rng = np.random.default_rng(2)
    with S.Solver(_params()) as sv:
        sv.step(200)
        shape = sv.dims("P")
        phi = (np.asfortranarray(rng.standard_normal(shape)), np.asfortranarray(rng.standard_normal(shape)))
        mu = (np.asfortranarray(rng.standard_normal(shape)), np.asfortranarray(rng.standard_normal(shape)))
        dt = 0.3 * AS.cfl_dt(sv)
        delta = 0.05 * AS.velocity_scale(sv)
        out = AS.advect(sv, phi, dt, delta)
        back, av = AS.advect_vjp(sv, phi, mu, dt, delta)
    lhs = sum(float(np.sum(m * o)) for m, o in zip(mu, out))
    rhs = sum(float(np.sum(b * f)) for b, f in zip(back, phi))
    assert abs(lhs - rhs) <= 1e-12 * sum(float(np.sum(np.abs(m * o))) for m, o in zip(mu, out))
    assert all(np.isfinite(a).all() for a in av.values())


def test_ascent_gradient_matches_central_differences():
    rng = np.random.default_rng(9)
    with S.Solver(_params()) as sv:
        F0 = AS.get_fields(sv)
        nsteps = 4
        g = AS.gradient(sv, F0, nsteps, checkpoint_every=2)
        assert g["solves"] == {"forward": 4, "recompute": 4, "adjoint": 4}

        def J(F):
            return AS.forward(sv, F, nsteps, dts=g["dts"], deltas=g["deltas"], checkpoint_every=2)["J"]

        eps = 1e-4
        for which in (1, 0):
            d = np.asfortranarray(rng.standard_normal(F0[which].shape))
            Fp = list(F0); Fm = list(F0)
            Fp[which] = F0[which] + eps * d
            Fm[which] = F0[which] - eps * d
            fd = (J(tuple(Fp)) - J(tuple(Fm))) / (2 * eps)
            ad = float(np.sum((g["dL0"] if which == 1 else g["drho0"]) * d))
            assert abs(fd - ad) <= 1e-5 * abs(fd), (which, fd, ad)
