"""C-ABI checks that need no GPU: the library loads, exports every symbol the
header declares, and its host-side entry points behave (no device work)."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

import sphericalstokes_gb300 as S

HEADER = Path(__file__).resolve().parent.parent / "include" / "sphstokes.h"


def declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\s*\*?\s*(sph_[a-z0-9_]+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_header_declares_entry_points():
    names = declared_functions()
    assert "sph_create" in names and "sph_solve" in names and "sph_step" in names
    assert len(names) >= 15


def test_library_exports_every_declared_symbol():
    lib = C.CDLL(str(S.LIB_PATH))
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_header():
    assert set(declared_functions()) <= set(S._SIGS)


def test_abi_version_and_strerror():
    lib = S.load_library()
    assert lib.sph_abi_version() == 2
    assert lib.sph_strerror(S.SPH_ERR_DIVERGED).decode().startswith("diverged")
    assert lib.sph_strerror(12345).decode() == "unknown status"


@pytest.mark.parametrize("geom,n_exp,rheo", [("spherical", 5.0, 1), ("cylindrical", 1.0, 2), ("cartesian", 5.0, 2)])
def test_params_default_follow_scripts(geom, n_exp, rheo):
    p = S.default_params(geom)
    assert (p.n1, p.n2, p.n3) == (207, 207, 207)
    assert p.n_exp == n_exp and p.rheology == rheo
    assert p.dmp == 4.5 and p.vr == 100.0 and p.rho_in == -10.0
    if geom == "spherical":
        assert p.c1 == 1000.0 and abs(p.l2 - 6.0 / 1000.0) < 1e-18 and p.l_ref == 6.0
    if geom == "cylindrical":
        assert p.n_exp_late == 5.0 and p.switch_err == 1e-5 and p.l3 == 6.0


def test_field_dims_match_reference_allocations():
    p = S.default_params("spherical", n1=11, n2=9, n3=7)
    assert S.field_dims(p, "P") == (11, 9, 7)
    assert S.field_dims(p, "VR") == (12, 9, 7)
    assert S.field_dims(p, "Vθ") == (11, 10, 7)
    assert S.field_dims(p, "Vφ") == (11, 9, 8)
    assert S.field_dims(p, "τ_Rθ") == (10, 8, 5)
    assert S.field_dims(p, "τ_Rφ") == (10, 7, 6)
    assert S.field_dims(p, "τ_θφ") == (9, 8, 6)


def test_invalid_params_rejected_without_device_work():
    lib = S.load_library()
    p = S.default_params("spherical", n1=3)
    h = C.c_void_p()
    assert lib.sph_create(C.byref(p), C.byref(h)) == S.SPH_ERR_INVALID
    assert b"5 cells" in lib.sph_last_error()
    p = S.default_params("spherical")
    p.abi_version = 99
    assert lib.sph_create(C.byref(p), C.byref(h)) == S.SPH_ERR_INVALID
    p = S.default_params("spherical", c2=0.1, l2=1.0)
    assert lib.sph_create(C.byref(p), C.byref(h)) == S.SPH_ERR_INVALID
    # 1024 x 1023 x 1023 cells: a box of 2^30 points, past the FP32 sweep's 32-bit byte offsets
    p = S.default_params("spherical", n1=1023, n2=1023, n3=1023, precision="mixed")
    assert lib.sph_create(C.byref(p), C.byref(h)) == S.SPH_ERR_INVALID
    assert b"FP32 sweep" in lib.sph_last_error()
    assert lib.sph_step(None, 1) == S.SPH_ERR_INVALID
    assert lib.sph_destroy(None) == 0


def test_sector_params():
    p = S.sector_params(63)
    assert p.c1 == 1.0 and abs(p.l2 - np.pi / 2) < 1e-15 and p.radius == 0.01 and p.rho_in == -1.0
    # PT step from the smallest spacing (r_min sin(θ_min) dφ)
    assert abs(p.vpdt - 0.5 * np.sin(np.pi / 4) * (np.pi / 2) / 62 / (2 + 4.5 * 3)) < 1e-15
