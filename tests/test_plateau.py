"""Plateau driver (scripts_plateau/SphericalStokes_plateau.jl): scaling, the layered
initial fields of initialize_geometry! against the golden fixture made from the script
itself, and (GPU) the eight-step continuation against an oracle replay."""
import math
import re

import numpy as np
import pytest

import oracle
import sphericalstokes_gb300 as S
from sphericalstokes_gb300 import plateau as PL


@pytest.fixture(scope="module")
def golden():
    from pathlib import Path
    g = np.load(Path(__file__).parent / "golden" / "sph_plateau.npz", allow_pickle=True)
    return g, eval(str(g["scalars_json"]))


def test_scaling_matches_the_script(golden):
    _, sc = golden
    s = PL.PlateauSetup().scaled()
    pairs = {"lr": "lr", "lth": "lθ", "lph": "lφ", "r": "r", "h_m": "hm", "h_l": "hl", "h_r": "hr", "h_c": "hc", "h_e": "he",
             "h_a": "ha", "d_l": "dl", "d_t": "dt", "d_h": "dh", "g": "g", "tau_c": "τ_C", "rho_c": "ρc", "rho_a": "ρa",
             "eta_l": "ηl", "eta_a": "ηa"}
    for k, j in pairs.items():
        np.testing.assert_allclose(s[k], sc[j], rtol=1e-15, atol=0, err_msg=k)
    np.testing.assert_allclose(s["eta_c"], [sc["ηc"], sc["ηc_2"], sc["ηc_3"], sc["ηc_4"], sc["ηc_5"], sc["ηc_6"]], rtol=1e-15)
    assert PL.PlateauSetup().viscosity_ratio(1) == sc["vr"]


def test_grid_matches_the_script(golden):
    g, sc = golden
    setup = PL.PlateauSetup(nr=int(sc["nr"]), nth=int(sc["nθ"]), nph=int(sc["nφ"]))
    p = setup.params()
    for c, l, n, x in ((p.c1, p.l1, p.n1, g["coord_R_i"]), (p.c2, p.l2, p.n2, g["coord_θ_i"]), (p.c3, p.l3, p.n3, g["coord_φ_i"])):
        np.testing.assert_allclose(PL.linspace(c, l, n), x, rtol=1e-14, atol=1e-15)


def test_initialize_geometry_matches_golden(golden):
    g, sc = golden
    R, T, F = np.meshgrid(g["coord_R_i"], g["coord_θ_i"], g["coord_φ_i"], indexing="ij")
    geo = dict(r=sc["r"], he=sc["he"], hc=sc["hc"], hr=sc["hr"], hl=sc["hl"], dt=sc["dt"])
    rho = PL.initialize_geometry(np.full(R.shape, sc["ρm"]), R, T, F, gl=sc["ρl"], gc=sc["ρc"], ga=sc["ρa"], **geo)
    eta = PL.initialize_geometry(np.full(R.shape, sc["ηm"]), R, T, F, gl=sc["ηl"], gc=sc["ηc"], ga=sc["ηa"], **geo)
    np.testing.assert_array_equal(rho, g["in_ρ"])
    np.testing.assert_array_equal(eta, g["in_η"])
    assert {sc["ρc"], sc["ρa"]} <= set(np.unique(rho)) and {sc["ηl"], sc["ηa"]} <= set(np.unique(eta))  # every layer present


@pytest.mark.gpu
def test_continuation_matches_oracle_replay():
    # steps 1-7; step 8 (n = 6) overflows the stress power law on this unconverged small state
    # in the oracle as well (NaN), where the library stops the step with SPH_ERR_DIVERGED
    setup = PL.PlateauSetup(nr=16, nth=9, nph=8)
    steps, iters = 7, 30
    res = None
    p = setup.params()
    with S.Solver(p) as sv:
        res = PL.run(setup, steps=steps, maxiter=iters, nout=10, tol=1e-30, solver=sv)
        got = {f: sv.get(f) for f in ("P", "V1", "V2", "V3", "TAU11", "TAU12", "TAU23", "ETA", "ETA_INI")}
    assert [r.iters for r in res] == [iters] * steps

    q = setup.params()
    o = oracle.Sph.from_params(q)
    rho, eta = PL.initial_fields(setup, q)
    o.rho[:] = rho
    o.eta[:] = eta
    o.eta_ini[:] = eta
    for it in range(1, steps + 1):
        if 2 <= it <= 6:
            e = PL.reset_crust_viscosity(setup, q, o.eta.copy(order="F"), it)
            o.eta[:] = e
            o.eta_ini[:] = e
            o.prm.vpdt = q.l1 / (q.n1 - 1) / (2.0 + 4.5 * math.log10(setup.viscosity_ratio(it)))
        elif it == 7:
            o.prm.n_exp = setup.n_exp_pl
        elif it == 8:
            o.prm.n_exp = setup.n_exp_pl2
        o.iterate(iters)
    for f, a in got.items():
        b = o.field(f)
        assert np.abs(a - b).max() <= 1e-9 * max(np.abs(b).max(), 1e-300), f


@pytest.mark.gpu
def test_continuation_writes_the_script_output(tmp_path):
    setup = PL.PlateauSetup(nr=12, nth=7, nph=6)
    PL.run(setup, steps=2, maxiter=20, nout=10, tol=5e-7, out_root=tmp_path)  # iter > 20 never holds: 20 iterations
    for it in (1, 2):
        d = tmp_path / f"out_plateau_{it}"
        infos = [float(t) for t in re.split(r"[,\s]+", (d / "1_infos.inf").read_text().strip())]
        assert infos[4:] == [12, 7, 6, 5, 0]  # εnonl*1e7 and run time 0 printed with %d
        phys = [float(t) for t in (d / "1_phys.inf").read_text().split()]
        assert len(phys) == 23 and phys[0] == 1
        assert phys[6] == pytest.approx(setup.scaled()["eta_c"][it - 1])
        a = np.fromfile(d / "A_VR.bin", dtype="<f8")
        assert a.size == 13 * 7 * 6
