"""sphericalstokes_gb300 — GB300 (sm_103a) pseudo-transient Stokes solver.

Host-side mirror of the solver surface of PTsolvers/SphericalStokes over the
C ABI of ``libsphstokes.so`` (``include/sphstokes.h``).  The reference scripts
run, per pseudo-transient (PT) iteration, ``maxloc!``, ``compute_P!``,
``compute_TII!``/``power_law!``, ``compute_V!`` and ``BC_R!``/``BC_θ!``/``BC_φ!``
(scripts_diapir/SphericalStokes_diapir.jl:413-425) on arrays they own; here a
:class:`Solver` owns the device arrays and exposes the same steps under the
same names, plus the whole loop (:meth:`Solver.step`, :meth:`Solver.solve`).

There is no CPU fallback: constructing a :class:`Solver` without the compiled
library or without a CUDA device raises.
"""
from __future__ import annotations

import ctypes as C
import math
import os
from dataclasses import dataclass
from pathlib import Path

import numpy as np

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "libsphstokes.so"

# enums of sphstokes.h
SPH_OK, SPH_ERR_INVALID, SPH_ERR_CUDA, SPH_ERR_NOT_CONVERGED, SPH_ERR_DIVERGED = 0, -1, -2, -3, -4
SPH_ERR_NOMEM, SPH_ERR_UNSUPPORTED, SPH_ERR_NO_DEVICE = -5, -6, -7
GEOM = {"spherical": 0, "cylindrical": 1, "cartesian": 2}
PREC = {"fp64": 0, "fp32": 1, "mixed": 2}
BC = {"diapir": 0, "free_slip": 1, "stress": 2, "free_surface": 3}
RHEO = {"linear": 0, "tau_power": 1, "tau_power_relax": 2, "edot_power_relax": 3}
INIT = {"none": 0, "inclusion": 1}
KERNELS_VARIANT = {"auto": 0, "simple": 1}
CRIT = {"reference": 0, "residual": 1, "reference_plateau": 2}
FIELDS = {
    "P": 0, "V1": 1, "V2": 2, "V3": 3, "TAU11": 4, "TAU22": 5, "TAU33": 6,
    "TAU12": 7, "TAU13": 8, "TAU23": 9, "ETA": 10, "ETA_INI": 11, "ETA_SM": 12,
    "DT_R": 13, "TII": 14, "RHO": 15, "PHASE": 16, "ETA_PL": 17, "TOP_LOAD": 18,
}
# the reference's array names (SphericalStokes_diapir.jl:381-399) -> field ids
ALIASES = {
    "VR": "V1", "Vθ": "V2", "Vφ": "V3", "VZ": "V3", "VX": "V1", "VY": "V2",
    "τ_RR": "TAU11", "τ_θθ": "TAU22", "τ_φφ": "TAU33", "τ_Rθ": "TAU12", "τ_Rφ": "TAU13", "τ_θφ": "TAU23",
    "η": "ETA", "η_ini": "ETA_INI", "ηSM": "ETA_SM", "τII": "TII", "ρ": "RHO",
}
KERNELS = {"maxloc": 0, "compute_P": 1, "rheology": 2, "compute_V": 3, "bc": 4}
# fields of the correction problem of the mixed-precision solve (sph_corr_field) and the
# reference-layout field whose size each one has
CORR_FIELDS = {
    "dP": (0, "P"), "dV1": (1, "V1"), "dV2": (2, "V2"), "dV3": (3, "V3"), "dTAU11": (4, "TAU11"), "dTAU22": (5, "TAU22"),
    "dTAU33": (6, "TAU33"), "dTAU12": (7, "TAU12"), "dTAU13": (8, "TAU13"), "dTAU23": (9, "TAU23"), "ETA": (10, "P"),
    "ETA_SM": (11, "P"), "rP": (12, "P"), "rV1": (13, "V1"), "rV2": (14, "V2"), "rV3": (15, "V3"),
}


class SphError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{msg} (status {code})")
        self.code = code


class Params(C.Structure):
    _fields_ = [
        ("abi_version", C.c_int32), ("geometry", C.c_int32), ("precision", C.c_int32), ("bc", C.c_int32),
        ("rheology", C.c_int32), ("init", C.c_int32), ("n1", C.c_int32), ("n2", C.c_int32), ("n3", C.c_int32),
        ("c1", C.c_double), ("c2", C.c_double), ("c3", C.c_double),
        ("l1", C.c_double), ("l2", C.c_double), ("l3", C.c_double),
        ("l_ref", C.c_double), ("vpdt", C.c_double), ("dmp", C.c_double), ("g", C.c_double),
        ("tau_C", C.c_double), ("n_exp", C.c_double), ("n_exp_late", C.c_double), ("switch_err", C.c_double),
        ("relax", C.c_double), ("edot_bg", C.c_double), ("r", C.c_double), ("sh", C.c_double),
        ("sig_bc", C.c_double * 3),
        ("eta0", C.c_double), ("vr", C.c_double), ("rho0", C.c_double), ("rho_in", C.c_double),
        ("radius", C.c_double), ("incl_linear", C.c_int32), ("kernels", C.c_int32),
        ("etasm_passes", C.c_int32), ("reserved_i", C.c_int32),
        ("fs_kappa", C.c_double), ("reserved", C.c_double * 7),
    ]


class SolveOpts(C.Structure):
    _fields_ = [
        ("criterion", C.c_int32), ("nout", C.c_int32), ("maxiter", C.c_int64), ("tol", C.c_double),
        ("inner_rtol", C.c_double), ("max_outer", C.c_int32), ("inner_max", C.c_int32),
        ("warm_tol", C.c_double), ("reserved", C.c_double * 6),
    ]


class SolveInfo(C.Structure):
    _fields_ = [
        ("iters", C.c_int64), ("outer", C.c_int32), ("status", C.c_int32), ("err", C.c_double),
        ("residual", C.c_double), ("seconds", C.c_double), ("nhist", C.c_int64),
        ("device_ms", C.c_double), ("sweep_ms", C.c_double), ("outer_ms", C.c_double),
        ("flags", C.c_int32), ("reserved_i", C.c_int32), ("reserved", C.c_double * 3),
    ]


SPH_SOLVE_WARM_ABANDONED = 1


# every symbol include/sphstokes.h declares, with its ctypes signature
_SIGS = {
    "sph_abi_version": ([], C.c_int),
    "sph_params_default": ([C.POINTER(Params), C.c_int32], C.c_int),
    "sph_field_dims": ([C.POINTER(Params), C.c_int32, C.POINTER(C.c_int64)], C.c_int),
    "sph_create": ([C.POINTER(Params), C.POINTER(C.c_void_p)], C.c_int),
    "sph_destroy": ([C.c_void_p], C.c_int),
    "sph_set_stream": ([C.c_void_p, C.c_void_p], C.c_int),
    "sph_set_field": ([C.c_void_p, C.c_int32, C.POINTER(C.c_double), C.c_int64], C.c_int),
    "sph_get_field": ([C.c_void_p, C.c_int32, C.POINTER(C.c_double), C.c_int64], C.c_int),
    "sph_update_params": ([C.c_void_p, C.POINTER(Params)], C.c_int),
    "sph_batch_solve": ([C.POINTER(C.c_void_p), C.c_int32, C.POINTER(SolveOpts), C.POINTER(SolveInfo), C.c_int32], C.c_int),
    "sph_autotune": ([C.c_void_p, C.c_int32, C.POINTER(C.c_int32), C.POINTER(C.c_double)], C.c_int),
    "sph_step": ([C.c_void_p, C.c_int64], C.c_int),
    "sph_solve": ([C.c_void_p, C.POINTER(SolveOpts), C.POINTER(SolveInfo), C.POINTER(C.c_int64),
                   C.POINTER(C.c_double), C.c_int64], C.c_int),
    "sph_residual": ([C.c_void_p, C.POINTER(C.c_double)], C.c_int),
    "sph_sweep": ([C.c_void_p, C.c_int64], C.c_int),
    "sph_sweep_apply": ([C.c_void_p], C.c_int),
    "sph_sweep_profile": ([C.c_void_p, C.c_int64, C.POINTER(C.c_double), C.POINTER(C.c_double)], C.c_int),
    "sph_run_kernel": ([C.c_void_p, C.c_int32], C.c_int),
    "sph_last_device_ms": ([C.c_void_p, C.POINTER(C.c_double)], C.c_int),
    "sph_strerror": ([C.c_int], C.c_char_p),
    "sph_last_error": ([], C.c_char_p),
    "sph_residual_fields": ([C.c_void_p] + [C.POINTER(C.c_double)] * 4, C.c_int),
    "sph_residual_vjp": ([C.c_void_p] + [C.POINTER(C.c_double)] * 10 + [C.c_int32], C.c_int),
    "sph_residual_vjp_law": ([C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double)], C.c_int),
    "sph_advect": ([C.c_void_p, C.c_double, C.c_double, C.c_int32, C.POINTER(C.POINTER(C.c_double)),
                    C.POINTER(C.POINTER(C.c_double))], C.c_int),
    "sph_advect_vjp": ([C.c_void_p, C.c_double, C.c_double, C.c_int32] + [C.POINTER(C.POINTER(C.c_double))] * 3
                       + [C.POINTER(C.c_double)] * 3, C.c_int),
    "sph_bc_vjp": ([C.c_void_p] + [C.POINTER(C.c_double)] * 3, C.c_int),
    "sph_adjoint_solve": ([C.c_void_p] + [C.POINTER(C.c_double)] * 8 + [C.POINTER(SolveOpts), C.POINTER(SolveInfo)], C.c_int),
    "sph_save": ([C.c_void_p, C.c_char_p, C.c_int32, C.c_double, C.c_double, C.POINTER(C.c_int64), C.POINTER(C.c_double),
                  C.c_int64], C.c_int),
    "sph_check_err_noalloc": ([C.c_int32, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p), C.POINTER(C.c_int64),
                               C.POINTER(C.c_double), C.c_void_p], C.c_int),
    "sph_corr_get": ([C.c_void_p, C.c_int32, C.POINTER(C.c_double), C.c_int64], C.c_int),
    "sph_corr_set": ([C.c_void_p, C.c_int32, C.POINTER(C.c_double), C.c_int64], C.c_int),
    "sph_selftest_wait_timeout": ([C.c_void_p], C.c_int),
    "sph_solve_history_ms": ([C.c_void_p, C.POINTER(C.c_double), C.c_int64, C.POINTER(C.c_int64)], C.c_int),
}

_lib = None


def load_library(path: str | os.PathLike | None = None) -> C.CDLL:
    """Load libsphstokes.so (built by ``__graft_entry__.build()``); raises if absent."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise SphError(SPH_ERR_NO_DEVICE, f"{p} is missing: build it with sphericalstokes_gb300.build.build_library()")
    lib = C.CDLL(str(p))
    for name, (args, res) in _SIGS.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    if path is None:
        _lib = lib
    return lib


def _check(lib, rc: int, what: str) -> int:
    if rc != SPH_OK:
        msg = lib.sph_last_error().decode() or lib.sph_strerror(rc).decode()
        raise SphError(rc, f"{what}: {msg}")
    return rc


def default_params(geometry: str = "spherical", **kw) -> Params:
    """Parameters of the reference script of ``geometry`` (diapir setup), updated by ``kw``.

    Keys accept the enum names of this module (e.g. ``precision="mixed"``,
    ``bc="free_slip"``, ``rheology="edot_power_relax"``).
    """
    lib = load_library()
    p = Params()
    _check(lib, lib.sph_params_default(C.byref(p), GEOM[geometry]), "sph_params_default")
    set_params(p, **kw)
    return p


def set_params(p: Params, **kw) -> Params:
    enums = {"geometry": GEOM, "precision": PREC, "bc": BC, "rheology": RHEO, "init": INIT, "kernels": KERNELS_VARIANT}
    for k, v in kw.items():
        if k in enums and isinstance(v, str):
            v = enums[k][v]
        if k == "sig_bc":
            for i, x in enumerate(v):
                p.sig_bc[i] = x
            continue
        if not hasattr(p, k):
            raise KeyError(k)
        setattr(p, k, v)
    return p


def field_dims(p: Params, field: str) -> tuple[int, int, int]:
    lib = load_library()
    d = (C.c_int64 * 3)()
    _check(lib, lib.sph_field_dims(C.byref(p), FIELDS[ALIASES.get(field, field)], d), "sph_field_dims")
    return int(d[0]), int(d[1]), int(d[2])


@dataclass
class SolveResult:
    status: int
    iters: int
    outer: int
    err: float
    residual: float
    seconds: float
    hist_iter: np.ndarray
    hist_err: np.ndarray
    device_ms: float = 0.0
    sweep_ms: float = 0.0
    outer_ms: float = 0.0
    flags: int = 0

    @property
    def warm_abandoned(self) -> bool:
        return bool(self.flags & SPH_SOLVE_WARM_ABANDONED)

    @property
    def converged(self) -> bool:
        return self.status == SPH_OK


class Solver:
    """One grid's device state and the PT loop over it (the body of ``SPH_3D_Inclusion``)."""

    def __init__(self, params: Params | None = None, **kw):
        self.lib = load_library()
        self.params = params if params is not None else default_params(kw.pop("geometry", "spherical"))
        set_params(self.params, **kw)
        h = C.c_void_p()
        _check(self.lib, self.lib.sph_create(C.byref(self.params), C.byref(h)), "sph_create")
        self._h = h

    # -- lifetime -------------------------------------------------------------
    def close(self):
        if getattr(self, "_h", None):
            self.lib.sph_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # -- fields -----------------------------------------------------------------
    def dims(self, name: str) -> tuple[int, int, int]:
        return field_dims(self.params, name)

    def get(self, name: str, out: np.ndarray | None = None) -> np.ndarray:
        """Field in the reference's layout: Fortran-ordered float64 array, A[i,j,k] = Julia A[i+1,j+1,k+1].

        ``out``: a Fortran-ordered float64 array of the field's shape to copy into (e.g. a view
        of pinned host memory, which the device writes at full link speed); a new array if None."""
        fid = FIELDS[ALIASES.get(name, name)]
        shp = self.dims(name)
        if out is None:
            out = np.zeros(shp, dtype=np.float64, order="F")
        elif out.shape != shp or out.dtype != np.float64 or not out.flags.f_contiguous or not out.flags.writeable:
            raise ValueError(f"{name}: out must be a writeable Fortran-ordered float64 array of shape {shp}")
        _check(self.lib, self.lib.sph_get_field(self._h, fid, out.ctypes.data_as(C.POINTER(C.c_double)), out.size), f"get {name}")
        return out

    def set(self, name: str, a) -> None:
        fid = FIELDS[ALIASES.get(name, name)]
        shp = self.dims(name)
        a = np.asfortranarray(np.asarray(a, dtype=np.float64))
        if a.shape != shp:
            raise ValueError(f"{name}: expected shape {shp}, got {a.shape}")
        _check(self.lib, self.lib.sph_set_field(self._h, fid, a.ctypes.data_as(C.POINTER(C.c_double)), a.size), f"set {name}")

    # -- the reference's kernels --------------------------------------------
    def maxloc(self):
        """maxloc!(ηSM, η) + copy_BC!(ηSM) (SphericalStokes_diapir.jl:414-415)."""
        _check(self.lib, self.lib.sph_run_kernel(self._h, KERNELS["maxloc"]), "maxloc")

    def compute_P(self):
        """compute_P! (SphericalStokes_diapir.jl:209-241)."""
        _check(self.lib, self.lib.sph_run_kernel(self._h, KERNELS["compute_P"]), "compute_P")

    def power_law(self):
        """compute_TII! + copy_BC!(τII) + power_law! (or the configured viscosity law)."""
        _check(self.lib, self.lib.sph_run_kernel(self._h, KERNELS["rheology"]), "rheology")

    def compute_V(self):
        """compute_V! (SphericalStokes_diapir.jl:308-329)."""
        _check(self.lib, self.lib.sph_run_kernel(self._h, KERNELS["compute_V"]), "compute_V")

    def apply_bc(self):
        """BC_R!, BC_θ!, BC_φ! (or the configured BC set) in call order."""
        _check(self.lib, self.lib.sph_run_kernel(self._h, KERNELS["bc"]), "bc")

    # -- loops --------------------------------------------------------------------
    def step(self, k: int = 1) -> float:
        """Exactly k PT iterations; returns their device time in ms (CUDA events)."""
        _check(self.lib, self.lib.sph_step(self._h, int(k)), "sph_step")
        ms = C.c_double()
        self.lib.sph_last_device_ms(self._h, C.byref(ms))
        return ms.value

    def solve(self, tol: float = 5e-7, maxiter: int = 100000, nout: int = 100, criterion: str = "reference",
              inner_rtol: float = 1e-3, max_outer: int = 50, inner_max: int = 200000, warm_tol: float = 0.0,
              hist_cap: int = 100000, raise_on_fail: bool = False) -> SolveResult:
        o = SolveOpts()
        o.criterion = CRIT[criterion]
        o.nout, o.maxiter, o.tol = nout, maxiter, tol
        o.inner_rtol, o.max_outer, o.inner_max, o.warm_tol = inner_rtol, max_outer, inner_max, warm_tol
        info = SolveInfo()
        hi = np.zeros(hist_cap, dtype=np.int64)
        he = np.zeros(hist_cap, dtype=np.float64)
        rc = self.lib.sph_solve(self._h, C.byref(o), C.byref(info), hi.ctypes.data_as(C.POINTER(C.c_int64)),
                                he.ctypes.data_as(C.POINTER(C.c_double)), hist_cap)
        if rc not in (SPH_OK, SPH_ERR_NOT_CONVERGED, SPH_ERR_DIVERGED) or (raise_on_fail and rc != SPH_OK):
            _check(self.lib, rc, "sph_solve")
        n = int(info.nhist)
        return SolveResult(int(info.status), int(info.iters), int(info.outer), float(info.err), float(info.residual),
                           float(info.seconds), hi[:n].copy(), he[:n].copy(), float(info.device_ms), float(info.sweep_ms),
                           float(info.outer_ms), int(info.flags))

    def history_ms(self) -> np.ndarray:
        """Wall-clock ms from the start of the last solve to each of its history entries."""
        n = C.c_int64()
        _check(self.lib, self.lib.sph_solve_history_ms(self._h, None, 0, C.byref(n)), "sph_solve_history_ms")
        out = np.zeros(int(n.value), dtype=np.float64)
        _check(self.lib, self.lib.sph_solve_history_ms(self._h, out.ctypes.data_as(C.POINTER(C.c_double)), len(out),
                                                       C.byref(n)), "sph_solve_history_ms")
        return out

    def autotune(self, sweeps: int = 20) -> tuple[int, float]:
        """Pick the fused sweep's x3 chunk length for this grid size; returns (chunk, ms per sweep)."""
        k, ms = C.c_int32(), C.c_double()
        _check(self.lib, self.lib.sph_autotune(self._h, int(sweeps), C.byref(k), C.byref(ms)), "sph_autotune")
        return int(k.value), float(ms.value)

    def update_params(self, p: Params) -> None:
        """Change scalar parameters between solves (``sph_update_params``); grid and model choices stay."""
        _check(self.lib, self.lib.sph_update_params(self._h, C.byref(p)), "sph_update_params")
        self.params = p

    def sweep(self, k: int) -> float:
        """k FP32 sweeps of the current defect-correction step (MIXED); returns their device time in ms."""
        _check(self.lib, self.lib.sph_sweep(self._h, int(k)), "sph_sweep")
        return self.last_device_ms()

    def save(self, folder: str | os.PathLike, num: int = 1, tol: float = 5e-7, runtime: float = 0.0,
             result: SolveResult | None = None) -> None:
        """Write the fields in the scripts' output format (``<num>_infos.inf``, ``<num>_phys.inf``,
        ``A_<name>.bin``) into ``folder``; ``result`` supplies err_evo / iter_evo."""
        hi = np.ascontiguousarray(result.hist_iter if result is not None else np.zeros(0), dtype=np.int64)
        he = np.ascontiguousarray(result.hist_err if result is not None else np.zeros(0), dtype=np.float64)
        _check(self.lib, self.lib.sph_save(self._h, os.fsencode(str(folder)), int(num), float(tol), float(runtime),
                                           hi.ctypes.data_as(C.POINTER(C.c_int64)), he.ctypes.data_as(C.POINTER(C.c_double)),
                                           len(hi)), "sph_save")

    def sweep_profile(self, k: int) -> tuple[float, float]:
        """k sweeps launched one at a time with events around each fused-kernel launch;
        returns (device ms of the k sweeps, summed device ms of the fused-kernel launches)."""
        sw, kn = C.c_double(), C.c_double()
        _check(self.lib, self.lib.sph_sweep_profile(self._h, int(k), C.byref(sw), C.byref(kn)), "sph_sweep_profile")
        return float(sw.value), float(kn.value)

    def sweep_apply(self) -> None:
        _check(self.lib, self.lib.sph_sweep_apply(self._h), "sph_sweep_apply")

    def corr_get(self, name: str) -> np.ndarray:
        """A field of the correction problem sph_sweep iterates (``CORR_FIELDS``), reference layout."""
        fid, like = CORR_FIELDS[name]
        out = np.zeros(self.dims(like), dtype=np.float64, order="F")
        _check(self.lib, self.lib.sph_corr_get(self._h, fid, out.ctypes.data_as(C.POINTER(C.c_double)), out.size),
               f"corr_get {name}")
        return out

    def corr_set(self, name: str, a) -> None:
        """Overwrite a field of the correction problem (stored as FP32)."""
        fid, like = CORR_FIELDS[name]
        a = np.asfortranarray(np.asarray(a, dtype=np.float64))
        if a.shape != self.dims(like):
            raise ValueError(f"{name}: expected shape {self.dims(like)}, got {a.shape}")
        _check(self.lib, self.lib.sph_corr_set(self._h, fid, a.ctypes.data_as(C.POINTER(C.c_double)), a.size),
               f"corr_set {name}")

    def residual(self) -> dict:
        out = (C.c_double * 7)()
        _check(self.lib, self.lib.sph_residual(self._h, out), "sph_residual")
        keys = ["mom1", "mom2", "mom3", "div", "vmax", "f_scale", "err"]
        return dict(zip(keys, list(out)))

    def last_device_ms(self) -> float:
        ms = C.c_double()
        self.lib.sph_last_device_ms(self._h, C.byref(ms))
        return ms.value


def teff_bytes(n1: int, n2: int, n3: int, word: int) -> float:
    """Effective bytes per PT iteration, A_eff = 26 nr nθ nφ sizeof(T) (SphericalStokes_diapir.jl:447)."""
    return 26.0 * n1 * n2 * n3 * word


def sector_params(n: int | tuple[int, int, int], **kw) -> Params:
    """Spherical sector of the benchmark configurations: r in [0.5, 1.5], θ in [π/4, 3π/4],
    φ in [-π/4, π/4], inclusion of radius 0.1 at (1, π/2, 0) (squared radius compared,
    as the reference does), radial gravity.  PT step from the smallest grid spacing."""
    n1, n2, n3 = (n, n, n) if isinstance(n, int) else n
    vr = kw.pop("vr", 1e3)
    p = default_params("spherical")
    cfl = 1.0 / (2.0 + 4.5 * math.log10(vr))
    hmin = min(1.0 / (n1 - 1), 0.5 * (math.pi / 2) / (n2 - 1), 0.5 * math.sin(math.pi / 4) * (math.pi / 2) / (n3 - 1))
    set_params(p, n1=n1, n2=n2, n3=n3, c1=1.0, c2=math.pi / 2, c3=0.0, l1=1.0, l2=math.pi / 2, l3=math.pi / 2,
               l_ref=1.0, r=1.0, radius=0.01, eta0=1.0, vr=vr, rho0=0.0, rho_in=-1.0, g=1.0, sh=0.0,
               vpdt=hmin * cfl, init="inclusion")
    set_params(p, **kw)
    return p


def make_opts(tol: float = 5e-7, maxiter: int = 100000, nout: int = 100, criterion: str = "reference",
              inner_rtol: float = 1e-3, max_outer: int = 50, inner_max: int = 200000, warm_tol: float = 0.0) -> SolveOpts:
    o = SolveOpts()
    o.criterion = CRIT[criterion]
    o.nout, o.maxiter, o.tol = nout, maxiter, tol
    o.inner_rtol, o.max_outer, o.inner_max, o.warm_tol = inner_rtol, max_outer, inner_max, warm_tol
    return o


def solve_batch(solvers: list, opts: list | SolveOpts, threads: int = 0) -> list[SolveResult]:
    """``sph_batch_solve``: every solver's PT solve, concurrently on the GPU (one stream each,
    ``threads`` host threads); ``opts`` one SolveOpts for all or one per solver."""
    lib = load_library()
    n = len(solvers)
    if isinstance(opts, SolveOpts):
        opts = [opts] * n
    ctxs = (C.c_void_p * n)(*[s._h for s in solvers])
    oa = (SolveOpts * n)(*opts)
    ia = (SolveInfo * n)()
    _check(lib, lib.sph_batch_solve(ctxs, n, oa, ia, int(threads)), "sph_batch_solve")
    empty_i, empty_e = np.zeros(0, dtype=np.int64), np.zeros(0)
    return [SolveResult(int(x.status), int(x.iters), int(x.outer), float(x.err), float(x.residual), float(x.seconds),
                        empty_i, empty_e, float(x.device_ms), float(x.sweep_ms), float(x.outer_ms), int(x.flags)) for x in ia]
