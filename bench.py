#!/usr/bin/env python3
"""Benchmark of the GB300 PT Stokes solver (one JSON line on stdout).

Workload (the headline configuration): spherical sector 255^3 cells,
r in [0.5, 1.5], θ in [π/4, 3π/4], φ in [-π/4, π/4]; n = 3 strain-rate power
law (η0 = 1, relaxation 0.5) with a linear inclusion (η = 1e-3, Δρ = -1,
radius 0.1 at the sector centre), radial gravity, far-field pure-shear normal
stresses σθθ = +0.5, σφφ = -0.5 on the lateral faces, free slip on the radial
faces.  Inputs are seeded synthetic fields of that shape (the reference has no
dataset).

* ``value``: T_eff (the reference's A_eff = 26·nr·nθ·nφ·sizeof(T) per PT
  iteration, SphericalStokes_diapir.jl:447, with sizeof(float) = 4) of the
  FP32 PT sweeps of the FP32+FP64 defect-correction solve, inputs resident in
  HBM, device time from CUDA events on the library's stream.  One "step" is
  one PT sweep.
* ``e2e``: the same metric through the C ABI with host buffers, per step of
  K sweeps: upload of the problem (ρ, η_ini, η, phase, V, P from pinned host
  memory), one defect-correction step of the mixed-precision solve (FP64
  residual, K FP32 sweeps, FP64 update and residual), download of V and P
  into pinned host memory.
* ``roofline``: the fused sweep kernel alone — A_eff per launch over its average
  launch duration, from CUDA event pairs around each launch on the library's
  stream (``sph_sweep_profile``, the same K sweeps launched one at a time).
* ``time_to_tol``: wall time to FP64 residual 1e-8 of the mixed solve and of
  plain FP64 PT on the same workload at ``--solve-n`` cells per axis (default
  63: plain FP64 PT at 255^3 runs for hours), with the relative velocity error
  of the mixed solution against the FP64 one.
* ``batch``: a seeded draw of small uneven solves (``--batch``, edges from
  ``--batch-edges``) through ``sph_batch_solve`` against the same solves one
  after another.
* ``plateau_511x255x255``: FP32 correction sweeps of the elliptical plateau
  set-up on its 511 x 255 x 255 grid (``--plateau-sweeps``).
* ``cpu_baseline``: the FP64 CPU oracle (restatement of the reference kernels)
  timed on the host cores on a bounded sample of the same workload.

``--impl reference`` times the reference's CPU implementation of the path (the
oracle port, all host threads) on the same workload and prints its line.
Multi-GPU (torchrun): every rank solves an independent replica (the path does
not shard); rank 0 prints the aggregate.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "T_eff GB/s and time-to-1e-8 at 255³ n=3: FP32+FP64-refine vs FP64 PT, 1 GB300"


def workload_params(n: int, precision: str, tuned: bool = False, dmp: float | None = None):
    """The n=3 spherical-sector workload.  ``tuned``: the PT parameters of the
    time-to-tolerance runs, the same for plain FP64 and for the mixed solve —
    two passes of the ηSM max filter, twice the reference pseudo-step, damping 3.
    ``dmp``: the damping (bulk/shear pseudo-modulus ratio ×2) instead of the set's."""
    import sphericalstokes_gb300 as S

    p = S.sector_params(n, bc="stress", rheology="edot_power_relax", n_exp=3.0, relax=0.5, edot_bg=0.25,
                        sig_bc=(0.0, 0.5, -0.5), incl_linear=1, precision=precision)
    if tuned:
        S.set_params(p, etasm_passes=2, vpdt=2.0 * p.vpdt, dmp=3.0)
    if dmp is not None:
        S.set_params(p, dmp=dmp)
    return p


def pt_parameters(p, n: int) -> str:
    """The PT parameters of a solve, stated against the reference's step."""
    import sphericalstokes_gb300 as S

    ref = S.sector_params(n).vpdt
    return (f"pseudo-step {p.vpdt / ref:g}x the reference's (CFL = 1/(2+4.5 log10 vr) of the smallest spacing), "
            f"dmp {p.dmp:g}, ηSM max filter {p.etasm_passes} pass(es)")


def workload_desc(n: int) -> str:
    return (f"spherical sector {n}^3, r∈[0.5,1.5] θ∈[π/4,3π/4] φ∈[-π/4,π/4], n=3 strain-rate power law "
            f"(relax 0.5) + linear inclusion η=1e-3 Δρ=-1 r=0.1, far-field σθθ=+0.5 σφφ=-0.5")


def workload_config(n: int) -> dict:
    """The ``config`` of both arms' lines (identical, so the two lines describe one workload)."""
    return {"workload": workload_desc(n), "n": n,
            "step": "one PT iteration over the workload's grid (T_eff from A_eff = 26 n^3 sizeof(T) per iteration)",
            "l2": "state > 1.7 GB per iteration at 255^3 > L2 (inputs larger than L2, no flush)", "parallelism": "replicas"}


def reference_params(n: int, m: int | None = None):
    """The parameters of the n=3 workload built without the library: the values of
    ``workload_params(n, "fp64")`` (spherical defaults of the diapir script with the sector
    geometry), m x3 planes at the same spacing about the sector's centre (all n when m is None)."""
    from types import SimpleNamespace

    m = n if m is None else m
    vr = 1e3
    cfl = 1.0 / (2.0 + 4.5 * math.log10(vr))
    hmin = min(1.0 / (n - 1), 0.5 * (math.pi / 2) / (n - 1), 0.5 * math.sin(math.pi / 4) * (math.pi / 2) / (n - 1))
    p = SimpleNamespace(geometry=0, bc=2, rheology=3, init=1, n1=n, n2=n, n3=m, c1=1.0, c2=math.pi / 2, c3=0.0,
                        l1=1.0, l2=math.pi / 2, l3=(math.pi / 2) * (m - 1) / (n - 1), l_ref=1.0, vpdt=hmin * cfl, dmp=4.5,
                        g=1.0, tau_C=1.0, n_exp=3.0, relax=0.5, edot_bg=0.25, r=1.0, sh=0.0, sig_bc=(0.0, 0.5, -0.5),
                        eta0=1.0, vr=vr, rho0=0.0, rho_in=-1.0, radius=0.01, incl_linear=1, etasm_passes=1)
    return p


def reference_workload(n: int, m: int | None = None):
    """(parameters, oracle state) of the workload for the oracle port of the reference's kernels."""
    import oracle

    p = reference_params(n, m)
    return p, oracle.Sph.from_params(p)


# ---------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int = 0):
        self.gpu = gpu_index
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits", "-lms", "200",
                                          "-i", str(self.gpu)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        busy = [x for x in sm if smax and x > 0.5 * max(smax)] or sm
        return {"sm_mhz": statistics.median(busy) if busy else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"hbm_gbs": d["hbm_gbs"], "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


# ---------------------------------------------------------------------------
def cpu_baseline(n: int, seconds: float = 15.0, threads: int | None = None) -> dict:
    """FP64 oracle PT iterations of the same workload on the host cores (bounded sample)."""
    import oracle
    import sphericalstokes_gb300 as S

    if threads:
        oracle.set_threads(threads)
    _, o = reference_workload(n)
    o.iterate(1)  # warm-up
    t0 = time.perf_counter()
    it = 0
    while True:
        o.iterate(1)
        it += 1
        if time.perf_counter() - t0 > seconds:
            break
    dt = (time.perf_counter() - t0) / it
    teff = S.teff_bytes(n, n, n, 8) / dt / 1e9
    return {"value": round(teff, 3), "unit": "GB/s", "cores": oracle.num_threads(), "kind": "port",
            "sample": f"{it} FP64 PT iterations of the {n}^3 workload ({dt * 1e3:.1f} ms each)"}


def linear_reference_params(n: int):
    """The linear case built without the library: the n^3 sector with linear viscosity and free slip
    on all faces (the reference's diapir step and inclusion), as ``linear_params`` gives the library."""
    p = reference_params(n)
    p.bc, p.rheology, p.n_exp, p.sig_bc = 1, 0, 1.0, (0.0, 0.0, 0.0)
    return p


def linear_params(n: int, precision: str):
    """The linear case for the library: the workload's sector with linear viscosity and free slip."""
    import sphericalstokes_gb300 as S

    p = workload_params(n, precision)
    S.set_params(p, bc="free_slip", rheology="linear", n_exp=1.0, sig_bc=(0.0, 0.0, 0.0))
    return p


def cpu_time_to_tol(n: int, tol: float = 1e-8, check: int = 1000, max_iters: int = 5_000_000) -> dict:
    """The linear 63^3-style case on the CPU: plain FP64 PT of the oracle port (all host threads) on the n^3 spherical
    sector, linear viscosity (inclusion 1e-3, Δρ = -1), free slip on all faces, the reference's PT
    step, iterated to FP64 residual `tol` (checked every `check` iterations)."""
    import oracle

    p = linear_reference_params(n)
    o = oracle.Sph.from_params(p)
    t0 = time.perf_counter()
    it, err, hist = 0, float("inf"), []
    while it < max_iters:
        o.iterate(check)
        it += check
        err = o.residual()["err"]
        hist.append([it, round(time.perf_counter() - t0, 2), err])
        if not (err == err) or err < tol:
            break
    return {"n": n, "tol": tol, "iterations": it, "seconds": round(time.perf_counter() - t0, 2), "residual": err,
            "converged": bool(err < tol), "cores": oracle.num_threads(), "history_every": max(1, len(hist) // 20),
            "curve_iter_s_residual": hist[:: max(1, len(hist) // 20)] + hist[-1:],
            "setup": "linear free-slip sector, inclusion η 1e-3 Δρ -1 r 0.1, reference PT step, residual every "
                     f"{check} iterations (the reference's Threads backend is absent: oracle port of its kernels)"}


def linear_time_to_tolerance(n: int, tol: float = 1e-8) -> dict:
    """The linear case on the GPU: the setup of ``cpu_time_to_tol`` (linear free-slip n^3 sector, the
    reference's PT step) to FP64 residual ``tol``, as plain FP64 PT and as the mixed solve."""
    import sphericalstokes_gb300 as S

    info: dict = {"n": n, "tol": tol, "setup": "linear free-slip sector, inclusion η 1e-3 Δρ -1 r 0.1, reference PT step"}
    for prec in ("fp64", "mixed"):
        p = linear_params(n, prec)
        with S.Solver(p) as sv:
            if prec == "fp64":
                r = sv.solve(tol=tol, maxiter=5_000_000, nout=1000, criterion="residual")
            else:
                r = sv.solve(tol=tol, maxiter=5_000_000, nout=100, criterion="residual", inner_rtol=1e-2, max_outer=200,
                             inner_max=300_000, warm_tol=0.0)
            info[prec] = {"seconds": round(r.seconds, 3), "iterations": r.iters, "residual": r.residual, "converged": r.converged}
            info[prec + "_V"] = [sv.get(f) for f in ("V1", "V2", "V3")]
    vmax = max(float(abs(v).max()) for v in info["fp64_V"])
    info["rel_velocity_error_mixed_vs_fp64"] = max(float(abs(a - b).max()) for a, b in zip(info.pop("mixed_V"), info.pop("fp64_V"))) / vmax
    if info["mixed"]["converged"] and info["fp64"]["converged"]:
        info["speedup_mixed_vs_fp64"] = round(info["fp64"]["seconds"] / info["mixed"]["seconds"], 2)
    return info


def run_reference(args) -> None:
    """The reference's CPU implementation of the path (the oracle port of its kernels, all host
    threads) on the same workload.  A step is one FP64 PT iteration over a sample of the grid:
    n x n x m cells with the workload's spacing (m x3 planes about the sector's centre), m
    chosen from one full-grid iteration so that the whole --steps/--warmup run takes about
    --ref-seconds."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import oracle

    n = args.n
    _, full = reference_workload(n)
    full.iterate(1)
    t0 = time.perf_counter()
    full.iterate(1)
    t_full = time.perf_counter() - t0
    del full
    nsteps = args.steps + args.warmup
    m = int(max(8, min(n, math.floor(n * args.ref_seconds / max(nsteps * t_full, 1e-9)))))
    _, o = reference_workload(n, m)  # same spacing, m x3 planes about the sector's centre
    for _ in range(args.warmup):
        o.iterate(1)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        o.iterate(1)
    dt = (time.perf_counter() - t0) / max(args.steps, 1)
    teff = 26.0 * n * n * m * 8 / dt / 1e9
    ms_full = dt * 1e3 * n / m  # the sample's time per cell over the whole grid
    sample = (f"{args.steps} FP64 PT iterations on {n}x{n}x{m} cells ({m} x3 planes of the {n}^3 workload at its spacing; "
              f"one full {n}^3 iteration took {t_full * 1e3:.0f} ms)")
    line = {
        "metric": METRIC, "value": round(teff, 3), "unit": "GB/s", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(dt * 1e3, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
        "config": workload_config(n),
        "ms_per_iteration": round(ms_full, 3), "word_bytes": 8,
        "cpu_baseline": {"value": round(teff, 3), "unit": "GB/s", "cores": oracle.num_threads(), "kind": "port", "sample": sample},
        "e2e": {"value": round(teff, 3), "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    if args.cpu_solve_n > 0:
        line["cpu_time_to_tol"] = cpu_time_to_tol(args.cpu_solve_n)
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
def _curve(ms: "np.ndarray", err: "np.ndarray", keep: int = 40) -> list:
    """(seconds, residual) pairs of a solve's history, at most ``keep`` of them (the last kept)."""
    import numpy as np

    idx = np.unique(np.linspace(0, len(ms) - 1, min(keep, len(ms))).astype(int)) if len(ms) else []
    return [[round(float(ms[i]) * 1e-3, 3), float(err[i])] for i in idx]


def _time_to(ms, err, level: float):
    """Seconds at the first history entry with residual <= level (None if never)."""
    for t, e in zip(ms, err):
        if e <= level:
            return float(t) * 1e-3
    return None


def time_to_tolerance(args) -> dict:
    """Mixed-precision solve to FP64 residual 1e-8 and plain FP64 PT from the same start with the same
    PT parameters.  Plain FP64 runs to 1e-8 or for --fp64-budget-s seconds (iterations from a short
    timed probe), with its residual history: the speed-up is taken at the residual both reached (1e-8
    when both converged), from their residual-against-time curves."""
    import numpy as np

    import sphericalstokes_gb300 as S

    n = args.solve_n
    info: dict = {"n": n, "tol": 1e-8}
    vel = {}
    p = workload_params(n, "mixed", tuned=args.tuned, dmp=args.dmp)
    info["pt_parameters"] = pt_parameters(p, n) + " (both solves)"
    with S.Solver(p) as sv:
        r = sv.solve(tol=1e-8, maxiter=args.max_sweeps, nout=100, criterion="residual", inner_rtol=args.inner_rtol,
                     max_outer=args.max_outer, inner_max=args.inner_max, warm_tol=args.warm_tol, hist_cap=1_000_000)
        ms_m = sv.history_ms()
        err_m = r.hist_err[:len(ms_m)]
        vel["mixed"] = [sv.get(f) for f in ("V1", "V2", "V3")]
    info["mixed"] = {"seconds": round(r.seconds, 3), "iterations": r.iters, "outer": r.outer, "residual": r.residual,
                     "converged": r.converged, "sweep_s": round(r.sweep_ms * 1e-3, 3), "outer_s": round(r.outer_ms * 1e-3, 3),
                     "curve_s_residual": _curve(ms_m, err_m)}
    p = workload_params(n, "fp64", tuned=args.tuned, dmp=args.dmp)
    nout = args.fp64_nout
    maxiter = args.fp64_maxiter
    if args.fp64_budget_s > 0:
        with S.Solver(p) as probe:  # FP64 ms per iteration (a separate state: the solve below starts fresh)
            probe.step(10)
            ms_it = probe.step(50) / 50
        maxiter = min(maxiter, max(nout, int(args.fp64_budget_s * 1e3 / ms_it) // nout * nout))
        info["fp64_budget_s"] = args.fp64_budget_s
    with S.Solver(p) as sv:
        r = sv.solve(tol=1e-8, maxiter=maxiter, nout=nout, criterion="residual", hist_cap=1_000_000)
        ms_f = sv.history_ms()
        err_f = r.hist_err[:len(ms_f)]
        vel["fp64"] = [sv.get(f) for f in ("V1", "V2", "V3")]
    info["fp64"] = {"seconds": round(r.seconds, 3), "iterations": r.iters, "residual": r.residual, "converged": r.converged,
                    "ms_per_iteration": round(r.device_ms / max(r.iters, 1), 4), "maxiter": maxiter,
                    "curve_s_residual": _curve(ms_f, err_f)}
    # the residual both solves reached: 1e-8 if plain FP64 converged, else its last (lowest) residual
    common = max(1e-8, float(np.nanmin(err_f)) if len(err_f) else 1.0)
    tm, tf = _time_to(ms_m, err_m, common), _time_to(ms_f, err_f, common)
    info["common_residual"] = common
    info["seconds_to_common_residual"] = {"mixed": tm, "fp64": tf}
    if tm and tf:
        info["speedup_mixed_vs_fp64"] = round(tf / tm, 2)
    vmax = max(float(np.abs(v).max()) for v in vel["fp64"])
    info["rel_velocity_error_mixed_vs_fp64"] = max(float(np.abs(a - b).max()) for a, b in zip(vel["mixed"], vel["fp64"])) / vmax
    info["rel_velocity_error_against"] = ("the converged FP64 solution" if info["fp64"]["converged"]
                                          else f"the last FP64 iterate (residual {info['fp64']['residual']:.2e})")
    return info


# ---------------------------------------------------------------------------
# replicas: every rank solves its own copy of the workload on its own GPU; the only
# communication is the barrier around the timed region and the max of the per-rank times
def replica_group(world: int):
    """The process group of the replicas (gloo on host memory), or None for one process."""
    if world <= 1:
        return None
    import torch.distributed as dist

    if not dist.is_initialized():
        dist.init_process_group("gloo")
    return dist


def replica_barrier(dist) -> None:
    if dist is not None:
        dist.barrier()


def replica_max(dist, x: float) -> float:
    """Max of x over the replicas (the slowest rank's time)."""
    if dist is None:
        return x
    import torch

    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def run_ours(args) -> None:
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if world > 1:
        os.environ["CUDA_VISIBLE_DEVICES"] = os.environ.get("LOCAL_RANK", "0")
    import numpy as np

    import sphericalstokes_gb300 as S

    dist = replica_group(world)

    def barrier():
        replica_barrier(dist)

    def max_over_ranks(x: float) -> float:
        return replica_max(dist, x)

    n = args.n
    word = 4
    aeff = S.teff_bytes(n, n, n, word)
    pk = peaks()
    out: dict = {}

    # --- device-resident sweeps of the mixed-precision solve (the hot path) ---
    p = workload_params(n, "mixed")
    with S.Solver(p) as sv:
        # bring the state to a realistic mid-solve iterate: a short mixed solve, then a fresh correction step
        if args.prep_sweeps > 0:
            sv.solve(tol=1e-8, maxiter=args.prep_sweeps, nout=100, criterion="residual", inner_rtol=1e-3, max_outer=2,
                     inner_max=args.prep_sweeps)
        sv.sweep(args.warmup)
        # nvidia-smi samples every 200 ms and the K timed sweeps last a few ms at the default K, so
        # the sampler runs over the same K-sweep block repeated for clock_load_s seconds before and
        # half that after the timed region: its samples are of this load, the timed block included
        clk = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
        clk.start()
        t_load = time.perf_counter()
        while time.perf_counter() - t_load < args.clock_load_s:
            sv.sweep(args.steps)
        barrier()
        ms = sv.sweep(args.steps)
        barrier()
        t_load = time.perf_counter()
        while time.perf_counter() - t_load < 0.5 * args.clock_load_s:
            sv.sweep(args.steps)
        clocks = clk.stop()
        ms_step = ms / max(args.steps, 1)
        ms_step_max = max_over_ranks(ms_step)
        # the same K sweeps once more, launched one at a time with an event pair around every
        # launch of the fused sweep kernel: its average launch duration for the roofline
        prof_sweep_ms, prof_kernel_ms = sv.sweep_profile(args.steps)
    value = aeff * world / (ms_step_max * 1e-3) / 1e9
    kernel_ms = prof_kernel_ms / max(args.steps, 1)
    launches_per_sweep = 1 + 2  # fused sweep (writes the x1-face ghosts) + the x2- and x3-face stages of the stress BC set
    out.update({"value": round(value, 3), "ms_per_step": round(ms_step_max, 5), "kernel_ms": kernel_ms,
                "kernel_share": prof_kernel_ms / prof_sweep_ms if prof_sweep_ms > 0 else None})

    # --- end to end through the C ABI with host buffers: upload the problem from pinned host
    # memory, K sweeps of the mixed-precision solve (sph_solve with maxiter = K), download V, P ---
    e2e = None
    solve_info = {}
    if not args.no_e2e:
        import torch

        p = workload_params(n, "mixed")
        with S.Solver(p) as sv0:  # the problem a caller holds in host memory
            host_in = {}
            for f in ("RHO", "ETA_INI", "ETA", "PHASE", "V1", "V2", "V3", "P"):
                a = sv0.get(f)
                t = torch.empty(a.shape[::-1], dtype=torch.float64).pin_memory()
                t.numpy()[...] = a.T  # C-order view of the Fortran-ordered field
                host_in[f] = (t, a.shape)
        h2d = sum(t.numel() * 8 for t, _ in host_in.values())
        outs = ("V1", "V2", "V3", "P")
        host_out = {}
        with S.Solver(workload_params(n, "mixed")) as sv0:
            for f in outs:  # pinned result buffers, as for the inputs
                host_out[f] = torch.empty(sv0.dims(f)[::-1], dtype=torch.float64).pin_memory()
        barrier()
        with S.Solver(workload_params(n, "mixed")) as sv:
            sv.solve(tol=1e-30, maxiter=args.warmup, nout=100, criterion="residual", inner_rtol=1e-30, max_outer=1,
                     inner_max=args.warmup)  # warm-up: graphs, TMA maps
            t0 = time.perf_counter()
            for f, (t, shp) in host_in.items():
                sv.set(f, t.numpy().T)
            t1 = time.perf_counter()  # sph_set_field returns after its copy and repack are done
            r = sv.solve(tol=1e-30, maxiter=args.steps, nout=100, criterion="residual", inner_rtol=1e-30, max_outer=1,
                         inner_max=args.steps)
            t2 = time.perf_counter()
            res = {f: sv.get(f, out=host_out[f].numpy().T) for f in outs}
            wall = time.perf_counter() - t0
            t_up, t_down = t1 - t0, t0 + wall - t2
        d2h = sum(a.nbytes for a in res.values())
        wall_max = max_over_ranks(wall)
        e2e_val = aeff * r.iters * world / wall_max / 1e9
        e2e = {"value": round(e2e_val, 3), "unit": "GB/s", "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
               "h2d_gbs": round(h2d / t_up / 1e9, 2), "d2h_gbs": round(d2h / t_down / 1e9, 2),
               "copy_share": round((t_up + t_down) / wall, 3),
               "step": f"upload 8 fields from pinned host memory, {r.iters} mixed-precision sweeps + FP64 residual, "
                       "download V and P into pinned host memory (one call chain); h2d_gbs / d2h_gbs: host-timed "
                       "rates of the field calls (one contiguous copy each plus the repack kernel into the padded box)"}

    if args.solve_n:
        solve_info = time_to_tolerance(args)
    linear_info = None
    if args.linear_solve_n:
        linear_info = linear_time_to_tolerance(args.linear_solve_n)
    adjoint_info = None
    if args.adjoint_n:
        from sphericalstokes_gb300 import adjoint as A

        with S.Solver(workload_params(args.adjoint_n, "fp64")) as sv:
            adjoint_info = A.fd_check(sv, directions=args.adjoint_dirs, seed=0)
        adjoint_info = {"n": args.adjoint_n, "objective": "1/2 sum (V_r - V_obs)^2 on the top interior face; V_obs from "
                        "a forward solve with log eta_ini + N(0, 0.1^2) per cell (seed 0)",
                        "parameters": "log eta_ini per cell, n, rho per cell; central differences eps 1e-4, forward solves "
                        "to FP64 residual 1e-12", **adjoint_info}
    # plain FP64 PT (one kernel per reference step) on the same workload: its time per iteration,
    # the per-iteration baseline of the mixed-precision solve's FP32 sweep
    fp64_info = None
    if args.fp64_iters > 0:
        with S.Solver(workload_params(n, "fp64")) as sv:
            sv.step(2)
            ms64 = sv.step(args.fp64_iters) / args.fp64_iters
        fp64_info = {"ms_per_iteration": round(ms64, 4), "iterations": args.fp64_iters,
                     "teff_gbs_fp64": round(S.teff_bytes(n, n, n, 8) / (ms64 * 1e-3) / 1e9, 2),
                     "fp32_sweep_speedup": round(ms64 / out["ms_per_step"], 2)}

    plateau_info = None
    if args.plateau_sweeps > 0:
        from sphericalstokes_gb300 import plateau as PL

        ep = PL.EllipsePlateau(top=args.plateau_top)
        with PL.ellipse_solver(ep, "mixed") as sv:
            sv.sweep(args.warmup)
            ms = sv.sweep(args.plateau_sweeps)
        r_solve = None
        if args.plateau_solve_sweeps > 0:  # a budget-bounded mixed solve from the initial state
            p0 = ep.params("mixed")
            step = args.plateau_step * p0.l1 / (p0.n1 - 1) / (2.0 + 4.5 * math.log10(p0.vr))  # x the library's dr CFL
            with PL.ellipse_solver(ep, "mixed", vpdt=step) as sv:
                r0 = sv.residual()["err"]
                r_solve = sv.solve(tol=1e-8, maxiter=args.plateau_solve_sweeps, nout=100, criterion="residual", inner_rtol=1e-2,
                                   max_outer=1000, inner_max=100_000, hist_cap=10_000)
                ms_hist = sv.history_ms()
        cells = ep.nr * ep.nth * ep.nph
        plateau_info = {"grid": [ep.nr, ep.nth, ep.nph], "sweeps": args.plateau_sweeps, "top": ep.top,
                        "ms_per_sweep": round(ms / args.plateau_sweeps, 4),
                        "teff_gbs": round(26 * cells * 4 / (ms / args.plateau_sweeps * 1e-3) / 1e9, 1),
                        "setup": ("elliptical plateau on a 40°x40° shell, 200 km deep, n=3 crust over linear mantle (ratio 1e-2), "
                                  "seeded ±2% density field; " +
                                  ("free-surface-stabilised top carrying the isostatic topography load" if ep.top == "free_surface"
                                   else "20 km sticky air") + "; FP32 correction sweeps")}
        if r_solve is not None:
            plateau_info["solve"] = {"sweeps": r_solve.iters, "outer": r_solve.outer, "seconds": round(r_solve.seconds, 2),
                                     "initial_residual": r0, "residual": r_solve.residual, "status": r_solve.status,
                                     "pt_step": f"{args.plateau_step:g} x the reference's (dr CFL), dmp {ep.dmp:g}",
                                     "curve_s_residual": _curve(ms_hist, r_solve.hist_err[:len(ms_hist)])}

    batch_info = None
    if args.batch > 0:
        from sphericalstokes_gb300 import batch as B

        edges = tuple(int(x) for x in args.batch_edges.split(","))
        cases = B.sweep_cases(args.batch, seed=0, edges=edges)
        bo = S.make_opts(tol=1e-8, maxiter=args.batch_budget, nout=100, criterion="residual", inner_rtol=1e-2, max_outer=30,
                         inner_max=args.batch_budget, warm_tol=0.0)
        rb = B.run(cases, bo, threads=args.batch_threads, autotune=bool(args.batch_autotune))
        # the serial reference: every stride-th case solved alone, one after another
        stride = max(1, args.batch // args.batch_serial) if args.batch_serial > 0 else 1
        sub = list(range(0, args.batch, stride))
        rs = B.run([cases[i] for i in sub], bo, serial=True, autotune=bool(args.batch_autotune))
        cells = [c.n1 * c.n2 * c.n3 for c in cases]

        def leg(r, idx):
            conv = [x for x in r["results"] if x.converged]
            work = sum(cells[i] * x.iters for i, x in zip(idx, r["results"]))  # cell sweeps done
            return {"solves": len(idx), "wall_s": round(r["wall_s"], 3), "converged": len(conv),
                    "converged_solves_per_s": round(len(conv) / r["wall_s"], 3),
                    "cell_sweeps_per_s": round(work / r["wall_s"], 1),
                    "teff_gbs": round(work * 26 * 4 / r["wall_s"] / 1e9, 1)}

        lb, ls = leg(rb, range(args.batch)), leg(rs, sub)
        same = all((rb["results"][i].status, rb["results"][i].iters, rb["results"][i].outer) == (b.status, b.iters, b.outer)
                   for i, b in zip(sub, rs["results"]))
        lockstep = len({x.seconds for x in rb["results"]}) == 1
        batch_info = {"solves": args.batch, "edges": list(edges), "budget_sweeps": args.batch_budget, "batch": lb, "serial": ls,
                      "speedup_vs_serial": (round(lb["converged_solves_per_s"] / ls["converged_solves_per_s"], 2)
                                            if ls["converged_solves_per_s"] > 0 else None),
                      "speedup_basis": "converged solves per second, batch (all solves) over serial (every "
                                       f"{stride}-th solve alone)",
                      "mode": "lockstep (one launch per sweep over all solves' blocks, graph-replayed rounds)" if lockstep
                              else "host threads, one stream per solve",
                      "batch_equals_serial_subset": same, "statuses": {str(k): sum(1 for x in rb["results"] if x.status == k)
                                                               for k in sorted({x.status for x in rb["results"]})},
                      "cases": "seed-0 draw: edge per axis from the list, geometry cycled sph/cyl/cart, n in 1..4, "
                               "viscosity ratio log-U[1e-4,1e-1], stress ratio U[0,1]; mixed precision to residual 1e-8 "
                               "or the sweep budget; PT step at most CFL(1e2)·sqrt(1e2/vr) of the spacing"
                               + ("; autotuned chunk per size" if args.batch_autotune else "")}

    if rank != 0:
        return
    line = {
        "metric": METRIC, "value": out["value"], "unit": "GB/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": out["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "precision": "FP32 sweeps inside FP64 defect correction (residual, update, norms in FP64)",
        "data": "synthetic",
        "config": workload_config(n),
        "ms_per_iteration": round(ms_step_max, 5), "word_bytes": word,
        "iteration": "one FP32 PT sweep of the FP32+FP64 defect-correction solve",
        "roofline": {"bound": "hbm", "kernel": "k_fused_tma (FP32 PT sweep, correction problem)",
                     "achieved": round(aeff / (out["kernel_ms"] * 1e-3) / 1e9, 3), "peak": pk["hbm_gbs"], "unit": "GB/s",
                     "frac": round(aeff / (out["kernel_ms"] * 1e-3) / 1e9 / pk["hbm_gbs"], 4),
                     "traffic": args.traffic, "peak_source": pk["source"],
                     "algorithmic_bytes_per_launch": aeff, "kernel_ms_per_launch": round(out["kernel_ms"], 5),
                     "kernel_share_of_sweep": round(out["kernel_share"], 4) if out["kernel_share"] else None},
        "clocks": clocks,
        "gpu_launches": args.steps * launches_per_sweep,
    }
    if e2e:
        line["e2e"] = e2e
    if solve_info:
        line["time_to_tol"] = solve_info
    if linear_info:
        line["linear_time_to_tol"] = linear_info
    if adjoint_info:
        line["adjoint_fd"] = adjoint_info
    if batch_info:
        line["batch"] = batch_info
    if plateau_info:
        line["plateau_511x255x255"] = plateau_info
    if fp64_info:
        line["fp64_pt"] = fp64_info
    if not args.no_cpu and world == 1:
        line["cpu_baseline"] = cpu_baseline(n, seconds=args.cpu_seconds)
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000, help="timed PT sweeps")
    ap.add_argument("--warmup", type=int, default=50, help="untimed PT sweeps before the timed region")
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--n", type=int, default=255, help="cells per axis")
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end measurement through host buffers")
    ap.add_argument("--solve-n", type=int, default=63,
                    help="time mixed vs plain FP64 PT to residual 1e-8 at this size (0: skip; 255 takes hours in FP64)")
    ap.add_argument("--fp64-maxiter", type=int, default=2_000_000)
    ap.add_argument("--fp64-budget-s", type=float, default=0.0,
                    help="cap plain FP64 PT of the time-to-tolerance leg at about this many seconds (0: run to 1e-8)")
    ap.add_argument("--fp64-nout", type=int, default=1000, help="FP64 residual checks every this many iterations")
    ap.add_argument("--fp64-iters", type=int, default=5,
                    help="plain FP64 PT iterations timed on the same workload (the FP32 sweep's per-iteration baseline; 0: skip)")
    ap.add_argument("--tuned", type=int, default=1,
                    help="time-to-tolerance PT parameters: 1 the tuned set (2 ηSM passes, 2x step, dmp 3), 0 the reference's")
    ap.add_argument("--dmp", type=float, default=None,
                    help="time-to-tolerance damping instead of the parameter set's (both solves)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--ref-seconds", type=float, default=90.0, help="target length of the --impl reference run")
    ap.add_argument("--adjoint-n", type=int, default=0,
                    help="adjoint gradient of the n^3 workload against central differences (0: skip)")
    ap.add_argument("--adjoint-dirs", type=int, default=16, help="seeded random directions of that check")
    ap.add_argument("--linear-solve-n", type=int, default=0,
                    help="the linear free-slip n^3 sector to residual 1e-8 on the GPU, FP64 PT and mixed (0: skip)")
    ap.add_argument("--cpu-solve-n", type=int, default=0,
                    help="--impl reference: also iterate the linear free-slip n^3 sector to residual 1e-8 on the CPU")
    ap.add_argument("--prep-sweeps", type=int, default=500)
    ap.add_argument("--max-sweeps", type=int, default=2_000_000)
    ap.add_argument("--inner-rtol", type=float, default=1e-2)
    ap.add_argument("--max-outer", type=int, default=60)
    ap.add_argument("--inner-max", type=int, default=200_000)
    ap.add_argument("--warm-tol", type=float, default=1e-3,
                    help="FP32 warm-start tolerance of the mixed solve (1e-3: shortest time at 63^3 among 1e-2 .. 1e-5)")
    ap.add_argument("--traffic", type=float, default=None,
                    help="DRAM bytes per launch of the fused sweep kernel, as an ncu capture of the same build measured "
                         "them (dram__bytes_read.sum + dram__bytes_write.sum); reported as roofline.traffic (null if absent)")
    ap.add_argument("--clock-load-s", type=float, default=1.0,
                    help="seconds of the same sweep load before (and half of it after) the timed region, so that the "
                         "200 ms clock sampler sees it")
    ap.add_argument("--batch", type=int, default=256, help="batched-solve leg: number of solves (0: skip)")
    ap.add_argument("--batch-edges", default="31,47",
                    help="grid edges the batched solves draw from (the full sweep: 31,47,63,79,95)")
    ap.add_argument("--batch-budget", type=int, default=100_000, help="sweep budget per batched solve")
    ap.add_argument("--batch-autotune", type=int, default=0, help="autotune the sweep chunk per grid size first")
    ap.add_argument("--batch-threads", type=int, default=16)
    ap.add_argument("--batch-serial", type=int, default=32,
                    help="solves of the serial reference (every batch/this-th case; 0: all)")
    ap.add_argument("--plateau-sweeps", type=int, default=200,
                    help="sweeps timed on the 511x255x255 elliptical-plateau grid (0: skip)")
    ap.add_argument("--plateau-top", default="free_surface", choices=["free_surface", "sticky_air"])
    ap.add_argument("--plateau-step", type=float, default=0.25,
                    help="PT step of the plateau solve, as a multiple of the reference's dr CFL")
    ap.add_argument("--plateau-solve-sweeps", type=int, default=0,
                    help="sweep budget of a mixed solve of the plateau from its initial state (0: skip)")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
