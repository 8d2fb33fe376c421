"""Free-surface-stabilised top boundary (SPH_BC_FREE_SURFACE, not in the reference; the
plateau's topography load without sticky air): on the top radial face the traction of a
surface load q(θ, φ) plus the stabilisation term κ V_r, zero shear traction, free slip on the
other faces.  The oracle (orc_sph_fs_pressure, the bc-3 branch of orc_sph_apply_bc) is the
specification.

* CPU: the oracle's known answer — a uniform load on a uniform, weightless fluid in a closed
  sector is carried by a uniform pressure: the PT iteration ends at P = q, V = 0.
* GPU: single kernels against the oracle (1e-12), FP64 trajectories (1e-9), the FP64 residual
  (1e-9), the FP32 correction sweep that the mixed solve times (2e-4, as for the other BC
  sets), and the known answer through FP64 PT iterations.
"""
import math
from types import SimpleNamespace

import numpy as np
import pytest

import oracle


def _load(shape, seed=0):
    """a smooth surface load on the top cells: a Gaussian bump of height 2 on a base of 0.5"""
    n1, n2, n3 = shape
    q = np.zeros(shape, order="F")
    jj, kk = np.meshgrid(np.arange(n2), np.arange(n3), indexing="ij")
    q[n1 - 1] = 0.5 + 2.0 * np.exp(-(((jj - 0.4 * n2) / (0.25 * n2)) ** 2 + ((kk - 0.6 * n3) / (0.3 * n3)) ** 2))
    return q


def test_oracle_uniform_load_is_carried_by_the_pressure():
    p = SimpleNamespace(geometry=0, bc=3, rheology=0, init=0, n1=13, n2=11, n3=9, c1=1.0, c2=math.pi / 2, c3=0.0, l1=1.0,
                        l2=math.pi / 2, l3=math.pi / 2, l_ref=1.0, vpdt=0.0, dmp=4.5, g=0.0, tau_C=1.0, n_exp=1.0, relax=0.5,
                        edot_bg=1.0, r=1.0, sh=0.0, sig_bc=(0.0, 0.0, 0.0), eta0=1.0, vr=10.0, rho0=0.0, rho_in=0.0, radius=0.01,
                        incl_linear=0, etasm_passes=1, fs_kappa=0.3)
    o = oracle.Sph.from_params(p)
    o.top_load[-1] = 2.5
    o.iterate(40000)
    assert np.abs(o.P - 2.5).max() < 1e-6
    assert max(np.abs(o.field(f)).max() for f in ("V1", "V2", "V3")) < 1e-7


# ---------------------------------------------------------------------------- GPU
def _params(S, n=(15, 13, 11), precision="fp64", rheology="linear", **kw):
    return S.sector_params(n, bc="free_surface", rheology=rheology, n_exp=3.0, relax=0.5, edot_bg=0.25, incl_linear=1,
                           fs_kappa=0.4, precision=precision, **kw)


@pytest.mark.gpu
def test_single_kernels_and_trajectory_match_oracle():
    import sphericalstokes_gb300 as S
    from test_parity_gpu import compare, randomize

    p = _params(S)
    rng = np.random.default_rng(3)
    with S.Solver(p) as sv:
        o = oracle.Sph.from_params(p)
        q = _load(o.P.shape)
        o.top_load[:] = q
        sv.set("TOP_LOAD", q)
        randomize(o, sv, rng)
        sv.compute_P(); o.compute_P()
        compare(o, sv, ["P", "TAU11", "TAU22", "TAU33", "TAU12", "TAU13", "TAU23", "DT_R"], 1e-12)
        sv.apply_bc(); o.apply_bc()
        compare(o, sv, ["V1", "V2", "V3"], 1e-12)
    for k in (1, 50):
        with S.Solver(p) as sv:
            sv.set("TOP_LOAD", q)
            sv.step(k)
            o = oracle.Sph.from_params(p)
            o.top_load[:] = q
            o.iterate(k)
            compare(o, sv, ("P", "V1", "V2", "V3", "TAU11", "TAU12", "TAU13", "TAU23", "DT_R"), 1e-9)


@pytest.mark.gpu
def test_residual_matches_oracle():
    import sphericalstokes_gb300 as S

    p = _params(S, rheology="edot_power_relax")
    with S.Solver(p) as sv:
        o = oracle.Sph.from_params(p)
        q = _load(o.P.shape)
        sv.set("TOP_LOAD", q)
        sv.step(30)
        r = sv.residual()
        o.top_load[:] = q
        o.iterate(30)
        ro = o.residual(f_scale=r["f_scale"])
    for key in ("mom1", "mom2", "mom3", "div", "vmax"):
        assert abs(r[key] - ro[key]) <= 1e-9 * max(abs(ro[key]), 1e-300), (key, r[key], ro[key])


@pytest.mark.gpu
@pytest.mark.parametrize("k,random_start", [(1, True), (10, True), (100, False)])
def test_correction_sweeps_match_oracle(k, random_start):
    import sphericalstokes_gb300 as S
    from test_sweep_parity_gpu import TOL, run_case

    p = _params(S, n=(17, 13, 11), precision="mixed", rheology="edot_power_relax")
    err = run_case(p, k, random_start=random_start, seed=k, setup=lambda sv: sv.set("TOP_LOAD", _load((17, 13, 11))))
    assert max(err.values()) < TOL, err


@pytest.mark.gpu
def test_uniform_load_is_carried_by_the_pressure():
    """the oracle's known answer on the GPU (FP64 PT iterations): P = q, V = 0"""
    import sphericalstokes_gb300 as S

    p = _params(S, n=(13, 11, 9), g=0.0, rho_in=0.0, vr=1.0)
    S.set_params(p, fs_kappa=0.3)
    with S.Solver(p) as sv:
        q = np.zeros(sv.dims("P"), order="F")
        q[-1] = 2.5
        sv.set("TOP_LOAD", q)
        sv.step(40000)
        P = sv.get("P")
        vmax = max(np.abs(sv.get(f)).max() for f in ("V1", "V2", "V3"))
    assert np.abs(P - 2.5).max() < 1e-6 and vmax < 1e-7
