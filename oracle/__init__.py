"""ORACLE — test infrastructure only.

ctypes wrapper of ``oracle/_build/liboracle.so``, the FP64 CPU restatement of
the reference's PT kernels (``oracle/oracle.cpp``).  Only ``tests/``,
``__graft_entry__.smoke()`` and ``bench.py``'s CPU baseline / reference arm
use it, as the reference the GPU results are compared with; the product library never calls it.

Arrays are numpy float64 in the reference's layout: Fortran order, the sizes of
the scripts' ``@zeros`` calls, ``A[i,j,k]`` = Julia ``A[i+1,j+1,k+1]``.
"""
from __future__ import annotations

import ctypes as C
import math
from pathlib import Path

import numpy as np

_DIR = Path(__file__).resolve().parent
LIB_PATH = _DIR / "_build" / "liboracle.so"
PI = 3.141592653589793
_PD = C.POINTER(C.c_double)
_PU8 = C.POINTER(C.c_uint8)


class SphState(C.Structure):
    _fields_ = [("nr", C.c_int64), ("nt", C.c_int64), ("np", C.c_int64)] + [
        (n, _PD) for n in ("P", "VR", "Vt", "Vp", "VR_err", "Vt_err", "Vp_err", "tRR", "ttt", "tpp", "tRt", "tRp",
                           "ttp", "rho", "eta", "eta_ini", "etaSM", "DT_R", "tII", "R", "th", "ph")
    ] + [("phase", _PU8), ("eta_tmp", _PD)]


class SphParams(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("_dr", "_dt", "_dp", "dmp", "vpdt", "lr", "g", "tau_C", "n_exp", "r", "sh")] + [
        ("bc", C.c_int32), ("rheo", C.c_int32)] + [(n, C.c_double) for n in ("relax", "edot_bg", "sig_t", "sig_p")] + [
        ("passes", C.c_int32), ("pad_", C.c_int32), ("fs_kappa", C.c_double), ("top_load", _PD)]


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            from sphericalstokes_gb300.build import build_oracle
            build_oracle()
        L = C.CDLL(str(LIB_PATH))
        L.orc_sph_iterate.argtypes = [C.POINTER(SphState), C.POINTER(SphParams), C.c_int64]
        L.orc_sph_check_err.argtypes = [C.POINTER(SphState)]
        L.orc_sph_check_err.restype = C.c_double
        L.orc_sph_equal3.argtypes = [C.POINTER(SphState)]
        for n in ("orc_sph_compute_P", "orc_sph_power_law", "orc_sph_compute_V", "orc_sph_apply_bc"):
            getattr(L, n).argtypes = [C.POINTER(SphState), C.POINTER(SphParams)]
        L.orc_sph_compute_TII.argtypes = [C.POINTER(SphState)]
        L.orc_copy_BC.argtypes = [_PD, C.c_int64, C.c_int64, C.c_int64]
        L.orc_copy_boundary_faces.argtypes = [_PD, C.c_int64, C.c_int64, C.c_int64]
        L.orc_maxloc.argtypes = [_PD, _PD, C.c_int64, C.c_int64, C.c_int64]
        L.orc_sph_edot_law.argtypes = [C.POINTER(SphState), C.POINTER(SphParams), _PD, C.c_int32, _PD]
        L.orc_sph_scratch_size.argtypes = [C.c_int64] * 3
        L.orc_sph_scratch_size.restype = C.c_int64
        L.orc_sph_residual.argtypes = [C.POINTER(SphState), C.POINTER(SphParams), _PD, _PD, _PD, _PD, _PD, _PD]
        L.orc_sph_residual_scratch_size.argtypes = [C.c_int64] * 3
        L.orc_sph_residual_scratch_size.restype = C.c_int64
        L.orc_num_threads.restype = C.c_int32
        L.orc_set_num_threads.argtypes = [C.c_int32]
        _lib = L
    return _lib


def _ptr(a):
    return a.ctypes.data_as(_PD) if a is not None else None


def linspace(c: float, l: float, n: int) -> np.ndarray:
    """Node coordinates c - l/2 .. c + l/2 (the reference's range(a, b, length=n)); same formula as the library."""
    lo, hi = c - l / 2.0, c + l / 2.0
    x = np.array([lo + (hi - lo) * i / (n - 1) for i in range(n)], dtype=np.float64)
    x[-1] = hi
    return x


class Sph:
    """State of one spherical solve (SphericalStokes_diapir.jl:369-404) held in numpy arrays."""

    NAMES = {"P": "P", "V1": "VR", "V2": "Vt", "V3": "Vp", "TAU11": "tRR", "TAU22": "ttt", "TAU33": "tpp",
             "TAU12": "tRt", "TAU13": "tRp", "TAU23": "ttp", "ETA": "eta", "ETA_INI": "eta_ini", "ETA_SM": "etaSM",
             "DT_R": "DT_R", "TII": "tII", "RHO": "rho", "TOP_LOAD": "top_load"}

    def __init__(self, nr, nt, np_, *, r, c2, lr, lt, lp, l_ref, dmp, vpdt, g, tau_C, n_exp, sh, bc, rheo,
                 relax=0.5, edot_bg=1.0, sig_t=0.0, sig_p=0.0, c1=None, c3=0.0, passes=1, fs_kappa=0.0):
        self.n = (nr, nt, np_)
        c1 = r if c1 is None else c1
        z = lambda *s: np.zeros(s, dtype=np.float64, order="F")
        self.P = z(nr, nt, np_); self.VR = z(nr + 1, nt, np_); self.Vt = z(nr, nt + 1, np_); self.Vp = z(nr, nt, np_ + 1)
        self.VR_err = z(nr + 1, nt, np_); self.Vt_err = z(nr, nt + 1, np_); self.Vp_err = z(nr, nt, np_ + 1)
        self.tRR = z(nr, nt, np_); self.ttt = z(nr, nt, np_); self.tpp = z(nr, nt, np_)
        self.tRt = z(nr - 1, nt - 1, np_ - 2); self.tRp = z(nr - 1, nt - 2, np_ - 1); self.ttp = z(nr - 2, nt - 1, np_ - 1)
        self.rho = z(nr, nt, np_); self.eta = z(nr, nt, np_) + 1.0; self.eta_ini = z(nr, nt, np_)
        self.etaSM = z(nr, nt, np_); self.DT_R = z(nr, nt, np_); self.tII = z(nr, nt, np_)
        x1, x2, x3 = linspace(c1, lr, nr), linspace(c2, lt, nt), linspace(c3, lp, np_)
        self.x1, self.x2, self.x3 = x1, x2, x3
        self.R = np.asfortranarray(np.broadcast_to(x1[:, None, None], (nr, nt, np_)).copy())
        self.th = np.asfortranarray(np.broadcast_to(x2[None, :, None], (nr, nt, np_)).copy())
        self.ph = np.asfortranarray(np.broadcast_to(x3[None, None, :], (nr, nt, np_)).copy())
        self.phase = np.zeros((nr, nt, np_), dtype=np.uint8, order="F")
        self.eta_tmp = np.zeros(nr * nt * np_ + int(lib().orc_sph_scratch_size(nr, nt, np_)), dtype=np.float64)
        self.prm = SphParams(_dr=(nr - 1) / lr, _dt=(nt - 1) / lt, _dp=(np_ - 1) / lp, dmp=dmp, vpdt=vpdt, lr=l_ref,
                             g=g, tau_C=tau_C, n_exp=n_exp, r=r, sh=sh, bc=bc, rheo=rheo, relax=relax,
                             edot_bg=edot_bg, sig_t=sig_t, sig_p=sig_p, passes=passes, fs_kappa=fs_kappa)
        self.top_load = np.zeros((nr, nt, np_), dtype=np.float64, order="F")  # free-surface load (top layer read)
        self._sync()

    def _sync(self):
        s = SphState(nr=self.n[0], nt=self.n[1], np=self.n[2])
        for f, _ in SphState._fields_[3:-2]:
            setattr(s, f, _ptr(getattr(self, f)))
        s.phase = self.phase.ctypes.data_as(_PU8)
        s.eta_tmp = _ptr(self.eta_tmp)
        self.st = s
        self.prm.top_load = _ptr(self.top_load)

    @classmethod
    def from_params(cls, p) -> "Sph":
        """Oracle state for a library ``Params`` (spherical geometry), initialised like the library."""
        rheo = {0: 2, 1: 0, 3: 1}[p.rheology]
        o = cls(p.n1, p.n2, p.n3, r=p.r, c1=p.c1, c2=p.c2, c3=p.c3, lr=p.l1, lt=p.l2, lp=p.l3, l_ref=p.l_ref,
                dmp=p.dmp, vpdt=p.vpdt if p.vpdt > 0 else p.l1 / (p.n1 - 1) / (2.0 + 4.5 * math.log10(p.vr)),
                g=p.g, tau_C=p.tau_C, n_exp=p.n_exp, sh=p.sh, bc=p.bc, rheo=rheo, relax=p.relax,
                edot_bg=p.edot_bg, sig_t=p.sig_bc[1], sig_p=p.sig_bc[2], passes=max(1, p.etasm_passes),
                fs_kappa=getattr(p, "fs_kappa", 0.0))
        o.rho[:] = p.rho0
        o.eta[:] = p.eta0
        if p.init == 1:
            L = lib()
            L.orc_sph_init_inclusion.argtypes = [_PD, _PD, _PD, _PD, C.c_int64, C.c_int64, C.c_int64, C.c_double, C.c_double, C.c_double]
            L.orc_sph_init_velocity.argtypes = [_PD, _PD, C.c_int64, C.c_int64, C.c_int64, C.c_double, C.c_double]
            nr, nt, np_ = o.n
            L.orc_sph_init_inclusion(_ptr(o.rho), _ptr(o.R), _ptr(o.th), _ptr(o.ph), nr, nt, np_, p.r, p.radius, p.rho_in)
            L.orc_sph_init_inclusion(_ptr(o.eta), _ptr(o.R), _ptr(o.th), _ptr(o.ph), nr, nt, np_, p.r, p.radius, p.eta0 / p.vr)
            L.orc_sph_init_velocity(_ptr(o.Vp), _ptr(o.th), nr, nt, np_, p.sh, p.r)
            if p.incl_linear:
                o.phase[:] = (o.eta != p.eta0).astype(np.uint8)
        o.eta_ini[:] = o.eta
        return o

    @classmethod
    def from_golden(cls, g, bc: int) -> "Sph":
        """Oracle state from a golden file of a spherical script: its coordinates, scalars and initial fields."""
        sc = eval(str(g["scalars_json"]))
        x1, x2, x3 = g["coord_R_i"], g["coord_θ_i"], g["coord_φ_i"]
        nr, nt, np_ = len(x1), len(x2), len(x3)
        o = cls(nr, nt, np_, r=sc["r"], c1=0.5 * (x1[0] + x1[-1]), c2=0.5 * (x2[0] + x2[-1]), c3=0.5 * (x3[0] + x3[-1]),
                lr=sc["lr"], lt=sc["lθ"], lp=sc["lφ"], l_ref=sc["lr"], dmp=sc["dmp"], vpdt=sc["vpdt"], g=sc["g"],
                tau_C=sc["τ_C"], n_exp=sc["n_exp"], sh=sc.get("sh", 0.0), bc=bc, rheo=0)
        o.R[:] = x1[:, None, None]
        o.th[:] = x2[None, :, None]
        o.ph[:] = x3[None, None, :]
        for jn, canon in SCRIPT_NAMES["spherical"].items():
            o.field(canon)[:] = g["in_" + jn]
        return o

    def field(self, name: str) -> np.ndarray:
        return getattr(self, self.NAMES[name])

    # kernels
    def iterate(self, k: int = 1):
        lib().orc_sph_iterate(C.byref(self.st), C.byref(self.prm), int(k))

    def equal3(self):
        lib().orc_sph_equal3(C.byref(self.st))

    def check_err(self) -> float:
        return float(lib().orc_sph_check_err(C.byref(self.st)))

    def maxloc(self):
        nr, nt, np_ = self.n
        lib().orc_maxloc(_ptr(self.etaSM), _ptr(self.eta), nr, nt, np_)
        lib().orc_copy_BC(_ptr(self.etaSM), nr, nt, np_)
        for _ in range(self.prm.passes - 1):
            tmp = self.etaSM.copy(order="F")
            lib().orc_maxloc(_ptr(self.etaSM), _ptr(tmp), nr, nt, np_)
            lib().orc_copy_BC(_ptr(self.etaSM), nr, nt, np_)

    def compute_P(self):
        lib().orc_sph_compute_P(C.byref(self.st), C.byref(self.prm))
        if self.prm.bc == 2:
            L = lib()
            L.orc_sph_stress_pressure.argtypes = [_PD, _PD, _PD, C.c_int64, C.c_int64, C.c_int64, C.c_double, C.c_double]
            L.orc_sph_stress_pressure(_ptr(self.P), _ptr(self.ttt), _ptr(self.tpp), *self.n, self.prm.sig_t, self.prm.sig_p)
        if self.prm.bc == 3:
            L = lib()
            L.orc_sph_fs_pressure.argtypes = [_PD] * 4 + [C.c_int64] * 3 + [C.c_double]
            L.orc_sph_fs_pressure(_ptr(self.P), _ptr(self.tRR), _ptr(self.VR), _ptr(self.top_load), *self.n, self.prm.fs_kappa)

    def power_law(self):
        nr, nt, np_ = self.n
        L = lib()
        if self.prm.rheo == 0:
            L.orc_sph_compute_TII(C.byref(self.st))
            L.orc_copy_BC(_ptr(self.tII), nr, nt, np_)
            L.orc_sph_power_law(C.byref(self.st), C.byref(self.prm))
        elif self.prm.rheo == 1:
            out = np.zeros_like(self.eta)
            L.orc_sph_edot_law(C.byref(self.st), C.byref(self.prm), _ptr(out), 1, _ptr(self.eta_tmp))
            self.eta[:] = out

    def compute_V(self):
        lib().orc_sph_compute_V(C.byref(self.st), C.byref(self.prm))

    def apply_bc(self):
        lib().orc_sph_apply_bc(C.byref(self.st), C.byref(self.prm))

    def corr_sweep(self, rP, rV1, rV2, rV3, k: int = 1):
        """k correction sweeps of the mixed-precision solve (orc_sph_corr_sweep): the state holds the
        correction (δP, δV, δτ), η and ηSM are frozen, rP / rV are the right-hand sides (reference layouts)."""
        rhs = [np.asfortranarray(np.asarray(a, dtype=np.float64)) for a in (rP, rV1, rV2, rV3)]
        for a, f in zip(rhs, ("P", "V1", "V2", "V3")):
            if a.shape != self.field(f).shape:
                raise ValueError(f"right-hand side of {f}: shape {a.shape}, expected {self.field(f).shape}")
        L = lib()
        L.orc_sph_corr_sweep.argtypes = [C.POINTER(SphState), C.POINTER(SphParams), _PD, _PD, _PD, _PD, C.c_int64]
        L.orc_sph_corr_sweep(C.byref(self.st), C.byref(self.prm), *[_ptr(a) for a in rhs], int(k))

    def residual_fields(self) -> dict:
        """The residual's fields (orc_sph_residual): momentum rows rV1..rV3 (velocity shapes, zero
        outside the interior nodes) and rP = div V (cells)."""
        nr, nt, np_ = self.n
        scr = np.zeros(int(lib().orc_sph_residual_scratch_size(nr, nt, np_)), dtype=np.float64)
        out = np.zeros(5, dtype=np.float64)
        f = {k: np.zeros(self.field(k).shape, dtype=np.float64, order="F") for k in ("V1", "V2", "V3", "P")}
        lib().orc_sph_residual(C.byref(self.st), C.byref(self.prm), _ptr(out), _ptr(scr), _ptr(f["V1"]), _ptr(f["V2"]),
                               _ptr(f["V3"]), _ptr(f["P"]))
        return f

    def residual(self, f_scale: float | None = None) -> dict:
        nr, nt, np_ = self.n
        scr = np.zeros(int(lib().orc_sph_residual_scratch_size(nr, nt, np_)), dtype=np.float64)
        out = np.zeros(5, dtype=np.float64)
        lib().orc_sph_residual(C.byref(self.st), C.byref(self.prm), _ptr(out), _ptr(scr), None, None, None, None)
        fs = f_scale if f_scale is not None else max(np.abs(self.rho).max() * abs(self.prm.g), 1e-300)
        mom = out[:3].max() / fs
        cont = out[3] * (self.x1[-1] - self.x1[0]) / (out[4] if out[4] > 0 else 1.0)
        return {"mom1": out[0], "mom2": out[1], "mom3": out[2], "div": out[3], "vmax": out[4], "err": max(mom, cont)}


def set_threads(n: int):
    lib().orc_set_num_threads(int(n))


def num_threads() -> int:
    return int(lib().orc_num_threads())


# ---------------------------------------------------------------------------
# cylindrical / Cartesian scripts (oracle_cyl_cart.cpp)
class CCState(C.Structure):
    _fields_ = [("n1", C.c_int64), ("n2", C.c_int64), ("n3", C.c_int64)] + [
        (n, _PD) for n in ("P", "V1", "V2", "V3", "t11", "t22", "t33", "t12", "t13", "t23", "rho", "eta", "eta_ini",
                           "eta_pl", "etaSM", "DT_R", "tII", "x1", "x2", "x3")]


class CCParams(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("d1", "d2", "d3", "dmp", "vpdt", "lr", "g", "tau_C", "n_exp", "relax", "r", "sh")]


# reference array names of each script -> canonical field names
SCRIPT_NAMES = {
    "spherical": {"P": "P", "VR": "V1", "Vθ": "V2", "Vφ": "V3", "τ_RR": "TAU11", "τ_θθ": "TAU22", "τ_φφ": "TAU33",
                  "τ_Rθ": "TAU12", "τ_Rφ": "TAU13", "τ_θφ": "TAU23", "η": "ETA", "η_ini": "ETA_INI", "ηSM": "ETA_SM",
                  "DT_R": "DT_R", "τII": "TII", "ρ": "RHO"},
    "cylindrical": {"P": "P", "VR": "V1", "Vθ": "V2", "VZ": "V3", "τ_RR": "TAU11", "τ_θθ": "TAU22", "τ_ZZ": "TAU33",
                    "τ_Rθ": "TAU12", "τ_RZ": "TAU13", "τ_θZ": "TAU23", "η": "ETA", "η_INI": "ETA_INI", "ηSM": "ETA_SM",
                    "DT_R": "DT_R", "τII": "TII", "ρ": "RHO", "η_PL": "ETA_PL"},
    "cartesian": {"P": "P", "VX": "V1", "VY": "V2", "VZ": "V3", "τ_XX": "TAU11", "τ_YY": "TAU22", "τ_ZZ": "TAU33",
                  "τ_XY": "TAU12", "τ_XZ": "TAU13", "τ_YZ": "TAU23", "η": "ETA", "η_INI": "ETA_INI", "ηSM": "ETA_SM",
                  "DT_R": "DT_R", "τII": "TII", "ρ": "RHO", "η_PL": "ETA_PL"},
}
_CC_ATTR = {"P": "P", "V1": "V1", "V2": "V2", "V3": "V3", "TAU11": "t11", "TAU22": "t22", "TAU33": "t33", "TAU12": "t12",
            "TAU13": "t13", "TAU23": "t23", "RHO": "rho", "ETA": "eta", "ETA_INI": "eta_ini", "ETA_PL": "eta_pl",
            "ETA_SM": "etaSM", "DT_R": "DT_R", "TII": "tII"}


class CC:
    """State of one cylindrical or Cartesian diapir solve (numpy arrays, reference layout)."""

    def __init__(self, geometry: str, fields: dict, x1, x2, x3, *, d1, d2, d3, dmp, vpdt, lr, g, tau_C, n_exp, relax, r, sh):
        self.geometry = geometry
        self.arr = {k: np.asfortranarray(np.array(v, dtype=np.float64)) for k, v in fields.items()}
        self.x = [np.ascontiguousarray(np.array(a, dtype=np.float64)) for a in (x1, x2, x3)]
        n1, n2, n3 = self.arr["P"].shape
        st = CCState(n1=n1, n2=n2, n3=n3)
        for canon, attr in _CC_ATTR.items():
            setattr(st, attr, _ptr(self.arr[canon]))
        st.x1, st.x2, st.x3 = (_ptr(a) for a in self.x)
        self.st = st
        self.prm = CCParams(d1=d1, d2=d2, d3=d3, dmp=dmp, vpdt=vpdt, lr=lr, g=g, tau_C=tau_C, n_exp=n_exp, relax=relax, r=r, sh=sh)

    @classmethod
    def from_golden(cls, g, geometry: str) -> "CC":
        names = SCRIPT_NAMES[geometry]
        sc = eval(str(g["scalars_json"]))
        fields = {canon: g["in_" + jn] for jn, canon in names.items()}
        if geometry == "cylindrical":
            x1, x2, x3 = g["coord_R_i"], g["coord_θ_i"], g["coord_Z_i"]
            d = (sc["dr"], sc["dθ"], sc["dz"])
            lr = sc["lr"]
        else:
            x1, x2, x3 = g["coord_X_i"], g["coord_Y_i"], g["coord_Z_i"]
            d = (sc["dx"], sc["dy"], sc["dz"])
            lr = sc["lx"]
        return cls(geometry, fields, x1, x2, x3, d1=d[0], d2=d[1], d3=d[2], dmp=sc["dmp"], vpdt=sc["vpdt"], lr=lr,
                   g=sc["g"], tau_C=sc["τ_C"], n_exp=sc["n_exp"], relax=sc["relax"], r=sc.get("r", 0.0), sh=sc["sh"])

    @classmethod
    def from_params(cls, p) -> "CC":
        """Zero state of a library ``Params`` of cylindrical (1) or Cartesian (2) geometry: node
        coordinates c ± l/2, spacings l/(n-1), the scalars of the scripts."""
        geometry = {1: "cylindrical", 2: "cartesian"}[p.geometry]
        n1, n2, n3 = p.n1, p.n2, p.n3
        z = lambda *s: np.zeros(s, dtype=np.float64, order="F")
        fields = {f: z(n1, n2, n3) for f in ("P", "TAU11", "TAU22", "TAU33", "RHO", "ETA", "ETA_INI", "ETA_PL", "ETA_SM",
                                             "DT_R", "TII")}
        fields.update(V1=z(n1 + 1, n2, n3), V2=z(n1, n2 + 1, n3), V3=z(n1, n2, n3 + 1), TAU12=z(n1 - 1, n2 - 1, n3 - 2),
                      TAU13=z(n1 - 1, n2 - 2, n3 - 1), TAU23=z(n1 - 2, n2 - 1, n3 - 1))
        vpdt = p.vpdt if p.vpdt > 0 else p.l1 / (n1 - 1) / (2.0 + 4.5 * math.log10(p.vr))
        return cls(geometry, fields, linspace(p.c1, p.l1, n1), linspace(p.c2, p.l2, n2), linspace(p.c3, p.l3, n3),
                   d1=p.l1 / (n1 - 1), d2=p.l2 / (n2 - 1), d3=p.l3 / (n3 - 1), dmp=p.dmp, vpdt=vpdt, lr=p.l_ref, g=p.g,
                   tau_C=p.tau_C, n_exp=p.n_exp, relax=p.relax, r=p.r, sh=p.sh)

    def field(self, name: str) -> np.ndarray:
        return self.arr[name]

    def iterate(self, k: int = 1):
        fn = lib().orc_cyl_iterate if self.geometry == "cylindrical" else lib().orc_cart_iterate
        fn.argtypes = [C.POINTER(CCState), C.POINTER(CCParams), C.c_int64]
        fn(C.byref(self.st), C.byref(self.prm), int(k))

    def corr_sweep(self, rP, rV1, rV2, rV3, k: int = 1):
        """k correction sweeps of the mixed-precision solve (orc_cc_corr_sweep), as Sph.corr_sweep."""
        rhs = [np.asfortranarray(np.asarray(a, dtype=np.float64)) for a in (rP, rV1, rV2, rV3)]
        for a, f in zip(rhs, ("P", "V1", "V2", "V3")):
            if a.shape != self.arr[f].shape:
                raise ValueError(f"right-hand side of {f}: shape {a.shape}, expected {self.arr[f].shape}")
        L = lib()
        L.orc_cc_corr_sweep.argtypes = [C.c_int32, C.POINTER(CCState), C.POINTER(CCParams), _PD, _PD, _PD, _PD, C.c_int64]
        L.orc_cc_corr_sweep(1 if self.geometry == "cylindrical" else 2, C.byref(self.st), C.byref(self.prm),
                            *[_ptr(a) for a in rhs], int(k))


def golden_fields(g, geometry: str, prefix: str) -> dict:
    """canonical-name dict of the golden arrays with the given prefix ('in_' or 'k10_' ...)"""
    return {canon: g[prefix + jn] for jn, canon in SCRIPT_NAMES[geometry].items() if prefix + jn in g.files}
