"""The hand-written adjoint against a reference gradient: ``sph_residual_vjp`` and
``sph_residual_vjp_law`` compared with PyTorch autograd VJPs of the FP64 CPU restatement
of the residual (oracle/residual_torch.py, pinned to the C++ oracle's residual), on random
states of small spherical sectors.  Every velocity entry is an independent input (flags 0).

* linear viscosity: (∂R/∂(V, P))ᵀλ, (∂R/∂η)ᵀλ and (∂R/∂ρ)ᵀλ per cell, free-slip and
  far-field-stress boundaries;
* strain-rate power law: the full Jacobian (η's dependence on V included), (∂R/∂η)ᵀλ at
  η = η_t(V), and through the law (∂R/∂η_ini)ᵀλ per cell and (∂R/∂n)ᵀλ.

Agreement: max-norm difference ≤ 1e-10 of each output's max-norm.
"""
import numpy as np
import pytest

import sphericalstokes_gb300 as S
from sphericalstokes_gb300 import adjoint as A

torch = pytest.importorskip("torch")
from oracle import residual_torch as RT  # noqa: E402

pytestmark = pytest.mark.gpu
TOL = 1e-10
VEL = ("V1", "V2", "V3")


def _state(sv, rng, law):
    st = {}
    for f in VEL + ("P",):
        st[f] = np.asfortranarray(rng.standard_normal(sv.dims(f)))
    st["RHO"] = np.asfortranarray(rng.standard_normal(sv.dims("P")))
    st["ETA_INI" if law else "ETA"] = np.asfortranarray(np.exp(rng.uniform(-1.0, 1.0, sv.dims("P"))))
    for f, a in st.items():
        sv.set(f, a)
    if law:  # about a fifth of the cells linear (phase 1), the rest on the power law
        sv.set("PHASE", np.asfortranarray((rng.uniform(size=sv.dims("P")) < 0.2).astype(np.float64)))
    return st


def _close(got, want, what):
    scale = float(np.abs(want).max())
    assert scale > 0.0, what
    err = float(np.abs(got - want).max()) / scale
    assert err <= TOL, (what, err)


@pytest.mark.parametrize("bc", ["free_slip", "stress"])
def test_linear_vjp_equals_autograd(bc):
    p = S.sector_params((11, 9, 8), rheology="linear", vr=10.0, bc=bc, sig_bc=(0.0, 0.5, -0.5))
    rng = np.random.default_rng(21)
    with S.Solver(p) as sv:
        st = _state(sv, rng, law=False)
        lam = {f: np.asfortranarray(rng.standard_normal(sv.dims(f))) for f in VEL + ("P",)}
        g = A.vjp(sv, lam, interior=False)
    gr = RT.SphGrid(p)
    t = {f: RT.tensor(a, grad=True) for f, a in st.items()}
    R = RT.residual(gr, t["V1"], t["V2"], t["V3"], t["P"], t["ETA"], t["RHO"])
    L = sum((RT.tensor(lam[f]) * r).sum() for f, r in zip(VEL + ("P",), R))
    names = VEL + ("P", "ETA", "RHO")
    grads = torch.autograd.grad(L, [t[f] for f in names])
    for f, want in zip(names, grads):
        _close(g[f], want.numpy(), f)


def test_power_law_vjp_equals_autograd():
    p = S.sector_params((11, 9, 8), bc="stress", rheology="edot_power_relax", n_exp=3.0, relax=0.5, edot_bg=0.25,
                        sig_bc=(0.0, 0.5, -0.5), incl_linear=1, vr=10.0)
    rng = np.random.default_rng(22)
    with S.Solver(p) as sv:
        st = _state(sv, rng, law=True)
        phase = sv.get("PHASE") != 0.0
        assert phase.any() and not phase.all()
        lam = {f: np.asfortranarray(rng.standard_normal(sv.dims(f))) for f in VEL + ("P",)}
        g = A.vjp(sv, lam, interior=False)
        g_ini, g_n = A.law_vjp(sv)
    gr = RT.SphGrid(p)
    t = {f: RT.tensor(a, grad=True) for f, a in st.items()}
    n = torch.tensor(3.0, dtype=torch.float64, requires_grad=True)
    eta = RT.edot_law(gr, t["V1"], t["V2"], t["V3"], t["ETA_INI"], n, torch.from_numpy(np.ascontiguousarray(phase)))
    R = RT.residual(gr, t["V1"], t["V2"], t["V3"], t["P"], eta, t["RHO"])
    L = sum((RT.tensor(lam[f]) * r).sum() for f, r in zip(VEL + ("P",), R))
    leaves = [t[f] for f in VEL + ("P", "RHO", "ETA_INI")] + [n, eta]
    grads = torch.autograd.grad(L, leaves)
    for f, want in zip(VEL + ("P", "RHO"), grads[:5]):
        _close(g[f], want.numpy(), f)
    _close(g_ini, grads[5].numpy(), "ETA_INI")
    assert abs(g_n - float(grads[6])) <= TOL * abs(float(grads[6])), ("n", g_n, float(grads[6]))
    _close(g["ETA"], grads[7].numpy(), "ETA (at the law's viscosity)")
