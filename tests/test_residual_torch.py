"""CPU pin of the PyTorch restatement of the residual (oracle/residual_torch.py, the
autograd reference for the adjoint) against the C++ oracle's residual fields
(orc_sph_residual) on random states: linear viscosity and the strain-rate law, free-slip
and far-field-stress boundaries."""
import math
from types import SimpleNamespace

import numpy as np
import pytest

import oracle

torch = pytest.importorskip("torch")
from oracle import residual_torch as RT  # noqa: E402


def params(bc, rheology, n=(11, 9, 8)):
    return SimpleNamespace(geometry=0, bc=bc, rheology=rheology, init=1, n1=n[0], n2=n[1], n3=n[2], c1=1.0, c2=math.pi / 2,
                           c3=0.0, l1=1.0, l2=math.pi / 2, l3=math.pi / 2, l_ref=1.0, vpdt=0.01, dmp=4.5, g=1.0, tau_C=1.0,
                           n_exp=3.0, relax=0.5, edot_bg=0.25, r=1.0, sh=0.0, sig_bc=(0.0, 0.5, -0.5), eta0=1.0, vr=10.0,
                           rho0=0.0, rho_in=-1.0, radius=0.01, incl_linear=1, etasm_passes=1)


def random_state(p, seed):
    rng = np.random.default_rng(seed)
    o = oracle.Sph.from_params(p)
    for f in ("V1", "V2", "V3", "P"):
        o.field(f)[:] = rng.standard_normal(o.field(f).shape)
    o.field("ETA")[:] = np.exp(rng.uniform(-1, 1, o.field("ETA").shape))
    o.field("ETA_INI")[:] = np.exp(rng.uniform(-1, 1, o.field("ETA").shape))
    o.field("RHO")[:] = rng.standard_normal(o.field("RHO").shape)
    return o


@pytest.mark.parametrize("bc", [1, 2])
@pytest.mark.parametrize("rheology", [0, 3])
def test_torch_residual_equals_oracle_residual(bc, rheology):
    p = params(bc, rheology)
    o = random_state(p, 3)
    want = o.residual_fields()
    gr = RT.SphGrid(p)
    t = {f: RT.tensor(o.field(f)) for f in ("V1", "V2", "V3", "P", "ETA", "ETA_INI", "RHO")}
    if rheology == 3:
        eta = RT.edot_law(gr, t["V1"], t["V2"], t["V3"], t["ETA_INI"], torch.tensor(3.0, dtype=torch.float64),
                          torch.from_numpy(np.ascontiguousarray(o.phase != 0)))
    else:
        eta = t["ETA"]
    got = RT.residual(gr, t["V1"], t["V2"], t["V3"], t["P"], eta, t["RHO"])
    for f, g in zip(("V1", "V2", "V3", "P"), got):
        w = want[f]
        assert np.abs(g.detach().numpy() - w).max() <= 1e-12 * np.abs(w).max(), f
