"""CPU checks of the oracle's correction sweep (orc_sph_corr_sweep, orc_cc_corr_sweep),
the FP64 specification of the mixed-precision solve's FP32 sweep:

* known answer: from a zero correction with rP = 0, one sweep leaves δP = δτ = 0 and
  sets every interior velocity node to rV times the average DT_R of its two cells,
  DT_R = vpdt² / (KBDT + GSDT / (1 + GSDT/η)) (SphericalStokes_diapir.jl:225-226, :308-329);
* linearity: the sweep map (δ, rP, rV) -> δ' is linear (homogeneous BCs, frozen η), so
  scaling every input by α scales the output by α, and sums map to sums.
"""
import math

import numpy as np
import pytest

import oracle

STATE = ("P", "V1", "V2", "V3", "TAU11", "TAU22", "TAU33", "TAU12", "TAU13", "TAU23")


class P:
    """The attributes oracle.Sph.from_params / oracle.CC.from_params read, for a small case
    (built here: these CPU tests need no library)."""

    def __init__(self, geometry, n, bc):
        self.geometry = geometry
        self.n1, self.n2, self.n3 = n
        self.bc = bc
        self.rheology = 0
        self.init = 0
        self.dmp, self.vr, self.g, self.tau_C, self.n_exp, self.relax, self.edot_bg = 4.5, 1e3, 1.0, 1.0, 1.0, 0.5, 1.0
        self.sh, self.etasm_passes, self.rho0, self.eta0 = 0.3, 1, 0.0, 1.0
        self.sig_bc = (0.0, 0.5, -0.5)
        if geometry == 0:
            self.c1, self.c2, self.c3 = 1.0, math.pi / 2, 0.0
            self.l1, self.l2, self.l3 = 1.0, math.pi / 2, math.pi / 2
            self.r = 1.0
        else:
            self.c1, self.c2, self.c3 = (1000.0, 0.0, 0.0) if geometry == 1 else (0.0, 0.0, 0.0)
            self.l1, self.l2, self.l3 = (6.0, 0.006, 6.0) if geometry == 1 else (6.0, 6.0, 6.0)
            self.r = 1000.0 if geometry == 1 else 0.0
        self.l_ref = self.l1
        self.vpdt = self.l1 / (self.n1 - 1) / (2.0 + 4.5 * math.log10(self.vr))


def make(geometry, n, bc, rng):
    p = P(geometry, n, bc)
    o = oracle.Sph.from_params(p) if geometry == 0 else oracle.CC.from_params(p)
    eta = np.exp(rng.uniform(-1.0, 1.0, o.field("P").shape))
    o.field("ETA")[:] = eta
    o.field("ETA_SM")[:] = eta * np.exp(rng.uniform(0.0, 0.5, eta.shape))
    return p, o


CASES = [(0, (9, 8, 7), 0), (0, (9, 8, 7), 1), (0, (9, 8, 7), 2), (1, (9, 8, 7), 0), (2, (8, 9, 7), 0)]


@pytest.mark.parametrize("geometry,n,bc", CASES)
def test_one_sweep_from_zero_is_rv_times_step(geometry, n, bc):
    rng = np.random.default_rng(0)
    p, o = make(geometry, n, bc, rng)
    rV = [rng.standard_normal(o.field(f).shape) for f in ("V1", "V2", "V3")]
    o.corr_sweep(np.zeros(o.field("P").shape), *rV, k=1)
    for f in ("P", "TAU11", "TAU22", "TAU33", "TAU12", "TAU13", "TAU23"):
        assert np.abs(o.field(f)).max() == 0.0, f
    kbc = p.dmp * 2.0 * math.pi * p.vpdt / p.l_ref
    gsc = 4.0 * math.pi * p.vpdt / p.l_ref
    sm, e = o.field("ETA_SM"), o.field("ETA")
    dt = p.vpdt ** 2 / (kbc * sm + gsc * sm / (1.0 + gsc * sm / e))
    n1, n2, n3 = n
    exp1 = rV[0][1:n1, 1:n2 - 1, 1:n3 - 1] * 0.5 * (dt[0:n1 - 1, 1:n2 - 1, 1:n3 - 1] + dt[1:n1, 1:n2 - 1, 1:n3 - 1])
    exp2 = rV[1][1:n1 - 1, 1:n2, 1:n3 - 1] * 0.5 * (dt[1:n1 - 1, 0:n2 - 1, 1:n3 - 1] + dt[1:n1 - 1, 1:n2, 1:n3 - 1])
    exp3 = rV[2][1:n1 - 1, 1:n2 - 1, 1:n3] * 0.5 * (dt[1:n1 - 1, 1:n2 - 1, 0:n3 - 1] + dt[1:n1 - 1, 1:n2 - 1, 1:n3])
    np.testing.assert_allclose(o.field("V1")[1:n1, 1:n2 - 1, 1:n3 - 1], exp1, rtol=1e-13, atol=1e-15)
    np.testing.assert_allclose(o.field("V2")[1:n1 - 1, 1:n2, 1:n3 - 1], exp2, rtol=1e-13, atol=1e-15)
    np.testing.assert_allclose(o.field("V3")[1:n1 - 1, 1:n2 - 1, 1:n3], exp3, rtol=1e-13, atol=1e-15)


@pytest.mark.parametrize("geometry,n,bc", CASES)
def test_sweeps_are_linear(geometry, n, bc):
    def run(scale_a, scale_b, k=3):
        _, o = make(geometry, n, bc, np.random.default_rng(7))
        ra, rb = np.random.default_rng(11), np.random.default_rng(12)
        for f in STATE:
            sh = o.field(f).shape
            o.field(f)[:] = scale_a * ra.standard_normal(sh) + scale_b * rb.standard_normal(sh)
        rhs = []
        for f in ("P", "V1", "V2", "V3"):
            sh = o.field(f).shape
            rhs.append(scale_a * ra.standard_normal(sh) + scale_b * rb.standard_normal(sh))
        o.corr_sweep(*rhs, k=k)
        return {f: o.field(f).copy() for f in STATE}

    a, b, ab, a3 = run(1.0, 0.0), run(0.0, 1.0), run(1.0, 1.0), run(-2.5, 0.0)
    for f in STATE:
        s = max(np.abs(a[f]).max(), np.abs(b[f]).max(), 1e-300)
        assert np.abs(ab[f] - (a[f] + b[f])).max() <= 1e-12 * s, f
        assert np.abs(a3[f] + 2.5 * a[f]).max() <= 1e-12 * s, f
