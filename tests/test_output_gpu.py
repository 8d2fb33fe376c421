"""sph_save: the scripts' output format (Save_infos, Save_phys, SaveArray of
SphericalStokes_diapir.jl:23-43, :461-485 and the cylindrical / Cartesian
analogues), read back the way the MATLAB visualisation reads it
(visu_diapir/visu_diapir.m: `load` of the .inf files, `fread(fid, 'double')`
+ `reshape` of the .bin files)."""
import re

import numpy as np
import pytest

import sphericalstokes_gb300 as S

pytestmark = pytest.mark.gpu


def _load_inf(path):
    """MATLAB `load` of a one-line ASCII file: numbers separated by blanks or commas"""
    return np.array([float(t) for t in re.split(r"[,\s]+", path.read_text().strip()) if t])


def _fread(path, shape):
    return np.fromfile(path, dtype="<f8").reshape(shape, order="F")


NAMES = {
    "spherical": (("R", "TH", "PH"), ("VR", "VTH", "VPH"), ("TAU_RR", "TAU_THTH", "TAU_PHPH", "TAU_RTH", "TAU_RPH", "TAU_THPH")),
    "cylindrical": (("R", "TH", "Z"), ("VR", "VTH", "VZ"), ("TAU_RR", "TAU_THTH", "TAU_ZZ", "TAU_RTH", "TAU_RZ", "TAU_THZ")),
    "cartesian": (("X3D", "Y3D", "Z3D"), ("VX", "VY", "VZ"), ("TAU_XX", "TAU_YY", "TAU_ZZ", "TAU_XY", "TAU_XZ", "TAU_YZ")),
}
FIELDS = ("V1", "V2", "V3", "TAU11", "TAU22", "TAU33", "TAU12", "TAU13", "TAU23")


@pytest.mark.parametrize("geom", ["spherical", "cylindrical", "cartesian"])
def test_save_reads_back_like_the_matlab_reader(tmp_path, geom):
    n = (15, 13, 11)
    p = S.default_params(geom, n1=n[0], n2=n[1], n3=n[2], n_exp=3.0)
    with S.Solver(p) as sv:
        res = sv.solve(tol=1e-30, maxiter=300, nout=100, criterion="reference")
        sv.save(tmp_path, num=1, tol=5e-7, runtime=12.6, result=res)
        got = {f: sv.get(f) for f in FIELDS + ("P", "ETA", "RHO", "TII")}

    infos = _load_inf(tmp_path / "1_infos.inf")
    assert infos.shape == (9,)
    assert infos[0] == 1 and tuple(infos[4:7]) == n
    np.testing.assert_allclose(infos[1:4], [p.l1, p.l2, p.l3], rtol=1e-6, atol=1e-6)
    assert infos[7] == 0.0 and infos[8] == 13.0  # %d of a Float64 in Julia's Printf: rounded, no decimals
    phys = _load_inf(tmp_path / "1_phys.inf")
    expect = [1, p.eta0, p.rho0, p.rho_in, p.n_exp, p.tau_C, p.vr, p.g, p.sh]
    expect += [p.radius, p.dmp] if geom == "cartesian" else [p.r, p.radius, p.dmp]
    np.testing.assert_allclose(phys, expect, rtol=1e-6, atol=1e-6)

    coords, vel, tau = NAMES[geom]
    X = _fread(tmp_path / f"A_{coords[0]}.bin", n)
    Y = _fread(tmp_path / f"A_{coords[1]}.bin", n)
    Z = _fread(tmp_path / f"A_{coords[2]}.bin", n)
    assert np.all(np.diff(X, axis=0) > 0) and np.all(np.diff(Y, axis=1) > 0) and np.all(np.diff(Z, axis=2) > 0)
    np.testing.assert_allclose(X[0, 0, 0], p.c1 - p.l1 / 2, rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(Z[0, 0, -1], p.c3 + p.l3 / 2, rtol=1e-12, atol=1e-12)
    for name, f in zip(vel + tau, FIELDS):
        a = got[f]
        np.testing.assert_array_equal(_fread(tmp_path / f"A_{name}.bin", a.shape), a)
    for name, f in (("P", "P"), ("ETAS", "ETA"), ("RHO", "RHO"), ("TII", "TII")):
        np.testing.assert_array_equal(_fread(tmp_path / f"A_{name}.bin", n), got[f])
    np.testing.assert_array_equal(np.fromfile(tmp_path / "A_err_evo.bin", dtype="<f8"), res.hist_err)
    np.testing.assert_array_equal(np.fromfile(tmp_path / "A_iter_evo.bin", dtype="<f8"), res.hist_iter.astype(float))

    if geom == "cylindrical":
        np.testing.assert_allclose(_fread(tmp_path / "A_RHOG.bin", n), got["RHO"] * p.g, rtol=0, atol=0)
        D = [_fread(tmp_path / f"A_{x}.bin", n) for x in ("D_RR", "D_THTH", "D_ZZ")]
        scale = max(np.abs(d).max() for d in D)
        assert np.abs(D[0] + D[1] + D[2]).max() <= 1e-12 * scale  # deviatoric
        divv = _fread(tmp_path / "A_DIVV.bin", n)
        assert np.isfinite(divv).all()
        for name, f in (("D_RTH", "TAU12"), ("D_RZ", "TAU13"), ("D_THZ", "TAU23")):
            assert _fread(tmp_path / f"A_{name}.bin", got[f].shape).shape == got[f].shape


def test_get_into_caller_array():
    """Solver.get(out=...) fills a caller's Fortran-ordered array with what get() returns,
    and refuses arrays of the wrong shape, type or order"""
    p = S.default_params("spherical", n1=15, n2=13, n3=11, n_exp=3.0)
    with S.Solver(p) as sv:
        sv.step(5)
        for f in ("V1", "P", "TAU12"):
            ref = sv.get(f)
            out = np.full(ref.shape, np.nan, order="F")
            assert sv.get(f, out=out) is out
            assert np.array_equal(out, ref)
        with pytest.raises(ValueError):
            sv.get("P", out=np.zeros(sv.dims("P")))  # C order
        with pytest.raises(ValueError):
            sv.get("P", out=np.zeros(sv.dims("V1"), order="F"))
