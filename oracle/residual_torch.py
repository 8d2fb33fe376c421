"""ORACLE — test infrastructure only.

FP64 PyTorch (CPU) restatement of the spherical Stokes residual, written for
automatic differentiation: its autograd vector-Jacobian products are the
reference gradients that the library's hand-written VJP kernels
(``sph_residual_vjp``, ``sph_residual_vjp_law``) are checked against.  Only
``tests/`` import it; the product library never calls it.

The residual is that of the FP64 oracle (``orc_sph_residual`` in oracle.cpp),
i.e. the reference's compute_P!/compute_V! stencils with the stresses at
their viscous fixed point:

* strain rates with the spherical metric terms, SphericalStokes_diapir.jl:184-208;
* τ_ii = 2 η D_ii at cells, τ_ij = avg4(η) D_ij at edges (the fixed point of
  the stress update :218-238);
* momentum residual at interior velocity nodes, :267-307 (σ_ii = -P + τ_ii,
  the ρg body force);
* continuity R_P = ∇·V at every cell (:184-189);
* far-field normal-stress boundary (not in the reference): the boundary-cell
  pressure is slaved to the traction, P = τ_nn - σ_bc (the average of the two
  conditions on cells of both a θ and a φ face);
* strain-rate power law (not in the reference): η = η_t(V), the unrelaxed
  target 2/(1/η_ini + 1/(η_ini (ε̇_II/ε̇_bg)^((1-n)/n))), ε̇_II from the cell
  strain rates and the 4-edge averages of the engineering shear rates at the
  clamped interior cell, linear (phase) cells η = η_ini.

Arrays use the reference layout's shapes (``A[i, j, k]`` = Julia
``A[i+1, j+1, k+1]``): P, η, ρ (nr, nt, np); VR (nr+1, nt, np), Vθ
(nr, nt+1, np), Vφ (nr, nt, np+1).
"""
from __future__ import annotations

import torch


def _coords(c: float, l: float, n: int) -> torch.Tensor:
    lo, hi = c - l / 2.0, c + l / 2.0
    x = torch.tensor([lo + (hi - lo) * i / (n - 1) for i in range(n)], dtype=torch.float64)
    x[-1] = hi
    return x


class SphGrid:
    """Geometry and scalars of a spherical sector (the library's ``Params`` fields)."""

    def __init__(self, p):
        self.n = (p.n1, p.n2, p.n3)
        self.x1, self.x2 = _coords(p.c1, p.l1, p.n1), _coords(p.c2, p.l2, p.n2)
        self._dr, self._dt, self._dp = (p.n1 - 1) / p.l1, (p.n2 - 1) / p.l2, (p.n3 - 1) / p.l3
        self.g = p.g
        self.traction = p.bc == 2
        self.sig_t, self.sig_p = p.sig_bc[1], p.sig_bc[2]
        self.edot_bg = p.edot_bg


def strain_rates(gr: SphGrid, VR, Vt, Vp):
    """(DIVV, DRR, Dθθ, Dφφ) at cells and the engineering shear rates (E_Rθ, E_Rφ, E_θφ) at edges."""
    nr, nt, np_ = gr.n
    x1, x2 = gr.x1, gr.x2
    Rc = x1.view(-1, 1, 1)
    tc = x2.view(1, -1, 1)
    inv_sin, cot = 1.0 / torch.sin(tc), 1.0 / torch.tan(tc)
    avxa = (VR[:-1] + VR[1:]) * 0.5
    avya = (Vt[:, :-1] + Vt[:, 1:]) * 0.5
    d1 = (VR[1:] - VR[:-1]) * gr._dr
    d2 = (Vt[:, 1:] - Vt[:, :-1]) * gr._dt / Rc
    d3 = (Vp[:, :, 1:] - Vp[:, :, :-1]) * gr._dp / Rc * inv_sin
    div = d1 + d2 + d3 + 2.0 * avxa / Rc + avya / Rc * cot
    DRR = d1 - div / 3.0
    Dtt = d2 + avxa / Rc - div / 3.0
    Dpp = d3 + avxa / Rc + avya / Rc * cot - div / 3.0
    # τ_Rθ edges (nr-1, nt-1, np-2)
    aR = ((x1[:-1] + x1[1:]) * 0.5).view(-1, 1, 1)
    Ert = ((Vt[1:nr, 1:nt, 1:np_ - 1] - Vt[0:nr - 1, 1:nt, 1:np_ - 1]) * gr._dr
           + (VR[1:nr, 1:nt, 1:np_ - 1] - VR[1:nr, 0:nt - 1, 1:np_ - 1]) * gr._dt / aR
           - (Vt[0:nr - 1, 1:nt, 1:np_ - 1] + Vt[1:nr, 1:nt, 1:np_ - 1]) * 0.5 / aR)
    # τ_Rφ edges (nr-1, nt-2, np-1)
    aT = x2[1:nt - 1].view(1, -1, 1)
    Erp = ((Vp[1:nr, 1:nt - 1, 1:np_] - Vp[0:nr - 1, 1:nt - 1, 1:np_]) * gr._dr
           + (VR[1:nr, 1:nt - 1, 1:np_] - VR[1:nr, 1:nt - 1, 0:np_ - 1]) * gr._dp / aR / torch.sin(aT)
           - (Vp[0:nr - 1, 1:nt - 1, 1:np_] + Vp[1:nr, 1:nt - 1, 1:np_]) * 0.5 / aR)
    # τ_θφ edges (nr-2, nt-1, np-1)
    aR2 = x1[1:nr - 1].view(-1, 1, 1)
    aT2 = ((x2[:-1] + x2[1:]) * 0.5).view(1, -1, 1)
    Etp = ((Vp[1:nr - 1, 1:nt, 1:np_] - Vp[1:nr - 1, 0:nt - 1, 1:np_]) * gr._dt / aR2
           + (Vt[1:nr - 1, 1:nt, 1:np_] - Vt[1:nr - 1, 1:nt, 0:np_ - 1]) * gr._dp / aR2 / torch.sin(aT2)
           - (Vp[1:nr - 1, 0:nt - 1, 1:np_] + Vp[1:nr - 1, 1:nt, 1:np_]) * 0.5 / aR2 / torch.tan(aT2))
    return div, DRR, Dtt, Dpp, Ert, Erp, Etp


def edot_law(gr: SphGrid, VR, Vt, Vp, eta_ini, n_exp, phase):
    """Unrelaxed target η_t(V) of the strain-rate power law (linear cells: η_ini)."""
    nr, nt, np_ = gr.n
    _, DRR, Dtt, Dpp, Ert, Erp, Etp = strain_rates(gr, VR, Vt, Vp)
    DD = 0.5 * (DRR * DRR + Dtt * Dtt + Dpp * Dpp)
    ert = (Ert[0:nr - 2, 0:nt - 2] + Ert[0:nr - 2, 1:nt - 1] + Ert[1:nr - 1, 0:nt - 2] + Ert[1:nr - 1, 1:nt - 1]) * 0.25
    erp = (Erp[0:nr - 2, :, 0:np_ - 2] + Erp[0:nr - 2, :, 1:np_ - 1] + Erp[1:nr - 1, :, 0:np_ - 2] + Erp[1:nr - 1, :, 1:np_ - 1]) * 0.25
    etp = (Etp[:, 0:nt - 2, 0:np_ - 2] + Etp[:, 0:nt - 2, 1:np_ - 1] + Etp[:, 1:nt - 1, 0:np_ - 2] + Etp[:, 1:nt - 1, 1:np_ - 1]) * 0.25
    ed_int = torch.sqrt(DD[1:nr - 1, 1:nt - 1, 1:np_ - 1] + 0.25 * (ert * ert + erp * erp + etp * etp))
    ci = torch.clamp(torch.arange(nr) - 1, 0, nr - 3)
    cj = torch.clamp(torch.arange(nt) - 1, 0, nt - 3)
    ck = torch.clamp(torch.arange(np_) - 1, 0, np_ - 3)
    ed = ed_int[ci][:, cj][:, :, ck]  # boundary cells take the invariant of the clamped interior cell
    pl = eta_ini * torch.pow(ed / gr.edot_bg, (1.0 - n_exp) / n_exp)
    et = 2.0 / (1.0 / eta_ini + 1.0 / pl)
    return torch.where(phase, eta_ini, et)


def residual(gr: SphGrid, VR, Vt, Vp, P, eta, rho):
    """(R_VR, R_Vθ, R_Vφ, R_P): momentum residual at interior nodes (zero elsewhere, velocity
    shapes) and ∇·V at every cell, for the viscosity ``eta`` per cell."""
    nr, nt, np_ = gr.n
    x1, x2 = gr.x1, gr.x2
    div, DRR, Dtt, Dpp, Ert, Erp, Etp = strain_rates(gr, VR, Vt, Vp)
    E = eta
    tRR, ttt, tpp = 2.0 * E * DRR, 2.0 * E * Dtt, 2.0 * E * Dpp
    tRt = (E[0:nr - 1, 0:nt - 1, 1:np_ - 1] + E[0:nr - 1, 1:nt, 1:np_ - 1] + E[1:nr, 0:nt - 1, 1:np_ - 1]
           + E[1:nr, 1:nt, 1:np_ - 1]) * 0.25 * Ert
    tRp = (E[0:nr - 1, 1:nt - 1, 0:np_ - 1] + E[0:nr - 1, 1:nt - 1, 1:np_] + E[1:nr, 1:nt - 1, 0:np_ - 1]
           + E[1:nr, 1:nt - 1, 1:np_]) * 0.25 * Erp
    ttp = (E[1:nr - 1, 0:nt - 1, 0:np_ - 1] + E[1:nr - 1, 0:nt - 1, 1:np_] + E[1:nr - 1, 1:nt, 0:np_ - 1]
           + E[1:nr - 1, 1:nt, 1:np_]) * 0.25 * Etp
    if gr.traction:  # boundary-cell pressure from the traction condition
        j = torch.arange(nt).view(1, -1, 1)
        k = torch.arange(np_).view(1, 1, -1)
        bt = (j == 0) | (j == nt - 1)
        bp = (k == 0) | (k == np_ - 1)
        both = bt & bp
        Pt = ttt - gr.sig_t
        Pp = tpp - gr.sig_p
        P = torch.where(both, (Pt + Pp) / 2.0, torch.where(bt, Pt, torch.where(bp, Pp, P)))
    sRR, stt, spp = tRR - P, ttt - P, tpp - P
    rG = rho * gr.g
    R1 = torch.zeros((nr + 1, nt, np_), dtype=torch.float64)
    R2 = torch.zeros((nr, nt + 1, np_), dtype=torch.float64)
    R3 = torch.zeros((nr, nt, np_ + 1), dtype=torch.float64)
    # VR nodes (i0+1, j0+1, k0+1): i0 < nr-1, j0 < nt-2, k0 < np-2
    aR = ((x1[:-1] + x1[1:]) * 0.5).view(-1, 1, 1)
    aT = x2[1:nt - 1].view(1, -1, 1)
    m = (slice(0, nr - 1), slice(1, nt - 1), slice(1, np_ - 1))
    p_ = (slice(1, nr), slice(1, nt - 1), slice(1, np_ - 1))
    d = ((sRR[p_] - sRR[m]) * gr._dr
         + (tRt[0:nr - 1, 1:nt - 1, 0:np_ - 2] - tRt[0:nr - 1, 0:nt - 2, 0:np_ - 2]) * gr._dt / aR
         + (tRp[0:nr - 1, 0:nt - 2, 1:np_ - 1] - tRp[0:nr - 1, 0:nt - 2, 0:np_ - 2]) * gr._dp / aR / torch.sin(aT)
         + 2.0 * ((sRR[m] + sRR[p_]) * 0.5) / aR
         - (((stt[m] + stt[p_]) * 0.5) + ((spp[m] + spp[p_]) * 0.5)) / aR
         + ((tRt[0:nr - 1, 0:nt - 2, 0:np_ - 2] + tRt[0:nr - 1, 1:nt - 1, 0:np_ - 2]) * 0.5) / aR / torch.tan(aT)
         - (rG[m] + rG[p_]) * 0.5)
    R1 = R1.index_put((torch.arange(1, nr).view(-1, 1, 1), torch.arange(1, nt - 1).view(1, -1, 1),
                       torch.arange(1, np_ - 1).view(1, 1, -1)), d)
    # Vθ nodes: i0 < nr-2, j0 < nt-1, k0 < np-2
    aR = x1[1:nr - 1].view(-1, 1, 1)
    aT = ((x2[:-1] + x2[1:]) * 0.5).view(1, -1, 1)
    m = (slice(1, nr - 1), slice(0, nt - 1), slice(1, np_ - 1))
    p_ = (slice(1, nr - 1), slice(1, nt), slice(1, np_ - 1))
    d = ((tRt[1:nr - 1, 0:nt - 1, 0:np_ - 2] - tRt[0:nr - 2, 0:nt - 1, 0:np_ - 2]) * gr._dr
         + (stt[p_] - stt[m]) * gr._dt / aR
         + (ttp[0:nr - 2, 0:nt - 1, 1:np_ - 1] - ttp[0:nr - 2, 0:nt - 1, 0:np_ - 2]) * gr._dp / aR / torch.sin(aT)
         + 3.0 * ((tRt[0:nr - 2, 0:nt - 1, 0:np_ - 2] + tRt[1:nr - 1, 0:nt - 1, 0:np_ - 2]) * 0.5) / aR
         + (((stt[m] + stt[p_]) * 0.5) - ((spp[m] + spp[p_]) * 0.5)) / aR / torch.tan(aT))
    R2 = R2.index_put((torch.arange(1, nr - 1).view(-1, 1, 1), torch.arange(1, nt).view(1, -1, 1),
                       torch.arange(1, np_ - 1).view(1, 1, -1)), d)
    # Vφ nodes: i0 < nr-2, j0 < nt-2, k0 < np-1
    aR = x1[1:nr - 1].view(-1, 1, 1)
    aT = x2[1:nt - 1].view(1, -1, 1)
    d = ((tRp[1:nr - 1, 0:nt - 2, 0:np_ - 1] - tRp[0:nr - 2, 0:nt - 2, 0:np_ - 1]) * gr._dr
         + (ttp[0:nr - 2, 1:nt - 1, 0:np_ - 1] - ttp[0:nr - 2, 0:nt - 2, 0:np_ - 1]) * gr._dt / aR
         + (spp[1:nr - 1, 1:nt - 1, 1:np_] - spp[1:nr - 1, 1:nt - 1, 0:np_ - 1]) * gr._dp / aR / torch.sin(aT)
         + 3.0 * ((tRp[0:nr - 2, 0:nt - 2, 0:np_ - 1] + tRp[1:nr - 1, 0:nt - 2, 0:np_ - 1]) * 0.5) / aR
         + 2.0 * ((ttp[0:nr - 2, 0:nt - 2, 0:np_ - 1] + ttp[0:nr - 2, 1:nt - 1, 0:np_ - 1]) * 0.5) / aR / torch.tan(aT))
    R3 = R3.index_put((torch.arange(1, nr - 1).view(-1, 1, 1), torch.arange(1, nt - 1).view(1, -1, 1),
                       torch.arange(1, np_).view(1, 1, -1)), d)
    return R1, R2, R3, div


def tensor(a, grad: bool = False) -> torch.Tensor:
    """FP64 leaf tensor of a reference-layout numpy array."""
    import numpy as np

    t = torch.from_numpy(np.ascontiguousarray(np.asarray(a, dtype=np.float64)))
    return t.requires_grad_(grad)

