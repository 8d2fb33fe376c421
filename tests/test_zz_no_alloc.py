"""sph_check_err_noalloc: the reference's exit check (check_err! and the
maximum(abs.(.)) ratios, SphericalStokes_diapir.jl:332-344, :428-432) on
caller-owned device arrays, with its reduction slots in a static device array
instead of allocated memory.  Checked against the err history that sph_solve
computes with the reference criterion on the same iterates, on two calls in a
row (the second also shows that the shared slots were cleared)."""
import ctypes as C

import numpy as np
import pytest

import sphericalstokes_gb300 as S

pytestmark = pytest.mark.gpu


def _device(torch, a):
    """host field (Fortran order, the reference's layout) -> device copy with the same memory order"""
    return torch.from_numpy(np.ascontiguousarray(a.ravel(order="F"))).cuda()


def _check_err(lib, torch, new, old):
    m = len(new)
    vp = (C.c_void_p * m)(*[t.data_ptr() for t in new])
    op = (C.c_void_p * m)(*[t.data_ptr() for t in old])
    cnt = (C.c_int64 * m)(*[t.numel() for t in new])
    err = C.c_double(-1.0)
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = lib.sph_check_err_noalloc(m, vp, op, cnt, C.byref(err), stream)
    return rc, err.value


def test_check_err_noalloc_matches_solve_history():
    torch = pytest.importorskip("torch")
    lib = S.load_library()
    p = S.default_params("spherical", n1=31, n2=23, n3=19)
    with S.Solver(p) as sv:  # the existing entry point: err at iterations 100 and 200
        res = sv.solve(tol=1e-30, maxiter=200, nout=100, criterion="reference")
    assert list(res.hist_iter) == [100, 200]

    got = []
    with S.Solver(p) as sv:  # the same iterates, snapshots taken by the caller
        for _ in range(2):
            sv.step(99)
            old = [_device(torch, sv.get(f)) for f in ("V1", "V2", "V3")]
            sv.step(1)
            new = [_device(torch, sv.get(f)) for f in ("V1", "V2", "V3")]
            rc, err = _check_err(lib, torch, new, old)
            assert rc == S.SPH_OK, lib.sph_last_error().decode()
            got.append(err)
    assert got[1] < got[0]  # a stale slot from the first call would have kept the larger value
    np.testing.assert_allclose(got, res.hist_err, rtol=1e-12, atol=0.0)


def test_check_err_noalloc_rejects_more_arrays_than_its_scratch():
    torch = pytest.importorskip("torch")
    lib = S.load_library()
    a = torch.ones(16, dtype=torch.float64, device="cuda")
    rc, err = _check_err(lib, torch, [a] * 9, [a] * 9)
    assert rc == S.SPH_ERR_INVALID and err == -1.0
    assert "holds 1 to 8" in lib.sph_last_error().decode()
    rc, err = _check_err(lib, torch, [a] * 8, [a] * 8)  # at the maximum: fine, no change -> 0
    assert rc == S.SPH_OK and err == 0.0


def test_check_err_noalloc_propagates_nan():
    """A NaN in a snapshot makes err NaN, as Julia's maximum(abs.(.)) ratio does (a caller's
    isnan(err) divergence guard then fires), and a later call without NaN is finite again."""
    torch = pytest.importorskip("torch")
    lib = S.load_library()
    v = torch.linspace(1.0, 2.0, 1000, dtype=torch.float64, device="cuda")
    old = v.clone()
    old[123] = float("nan")
    rc, err = _check_err(lib, torch, [v, v], [v.clone(), old])
    assert rc == S.SPH_OK and np.isnan(err)
    rc, err = _check_err(lib, torch, [v], [v * 0.5])
    assert rc == S.SPH_OK and err == pytest.approx(0.5, rel=1e-15)
