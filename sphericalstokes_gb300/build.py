"""Build the in-tree shared libraries.

* ``sphericalstokes_gb300/libsphstokes.so`` — the CUDA C-ABI library, compiled
  by nvcc for sm_103a only (``-gencode arch=compute_103a,code=sm_103a``).
* ``oracle/_build/liboracle.so`` — the FP64 CPU oracle (test infrastructure),
  compiled by g++ with OpenMP.

Both are plain ``nvcc``/``g++`` invocations (no cmake), a few seconds each,
and run the same on x86_64 and aarch64 hosts.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
LIB = PKG / "libsphstokes.so"
ORACLE_DIR = ROOT / "oracle"
ORACLE_LIB = ORACLE_DIR / "_build" / "liboracle.so"

NVCC_FLAGS = [
    "-gencode", "arch=compute_103a,code=sm_103a",
    "-O3", "-lineinfo", "-std=c++17",
    "-Xcompiler", "-fPIC", "-shared",
]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the sm_103a library cannot be built")


def _stale(target: Path, sources: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(s.stat().st_mtime > t for s in sources)


def build_library(force: bool = False, verbose: bool = False) -> Path:
    sources = sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cuh")) + [ROOT / "include" / "sphstokes.h"]
    if not force and not _stale(LIB, sources):
        return LIB
    cmd = [_nvcc(), *NVCC_FLAGS, f"-I{ROOT / 'include'}", "-o", str(LIB) + ".tmp", str(CSRC / "sphstokes.cu")]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("nvcc failed:\n" + res.stdout + res.stderr)
    if verbose:
        sys.stderr.write(res.stderr)
    os.replace(str(LIB) + ".tmp", LIB)
    return LIB


def build_oracle(force: bool = False) -> Path:
    sources = sorted(ORACLE_DIR.glob("*.cpp"))
    if not force and not _stale(ORACLE_LIB, sources):
        return ORACLE_LIB
    ORACLE_LIB.parent.mkdir(parents=True, exist_ok=True)
    cxx = shutil.which("g++") or "g++"
    cmd = [cxx, "-O2", "-std=c++17", "-fopenmp", "-fPIC", "-shared", "-ffp-contract=off",
           "-o", str(ORACLE_LIB) + ".tmp", *map(str, sources)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("g++ failed:\n" + res.stdout + res.stderr)
    os.replace(str(ORACLE_LIB) + ".tmp", ORACLE_LIB)
    return ORACLE_LIB


def build_all(force: bool = False) -> None:
    with ThreadPoolExecutor(max_workers=2) as ex:
        futs = [ex.submit(build_library, force), ex.submit(build_oracle, force)]
        for f in futs:
            f.result()


if __name__ == "__main__":
    build_all(force="--force" in sys.argv)
    print(LIB)
    print(ORACLE_LIB)
