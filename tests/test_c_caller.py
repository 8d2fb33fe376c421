"""The C ABI from a compiled C caller (tests/c_caller.c, built here with gcc against
include/sphstokes.h and the in-tree libsphstokes.so), not only through ctypes: without a
device it fails loudly at sph_create; on the GPU its pressure after k reference iterations
equals the Python mirror's bit for bit (same library, same kernels)."""
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

import sphericalstokes_gb300 as S

ROOT = Path(__file__).resolve().parent.parent
SRC = ROOT / "tests" / "c_caller.c"


def _build(tmp_path) -> Path:
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    exe = tmp_path / "c_caller"
    lib_dir = Path(S.LIB_PATH).parent
    cmd = [cc, "-std=c99", "-Wall", "-Wextra", "-Werror", f"-I{ROOT / 'include'}", "-o", str(exe), str(SRC),
           f"-L{lib_dir}", "-lsphstokes", f"-Wl,-rpath,{lib_dir}", "-lm"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    return exe


def _has_device() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def test_c_caller_builds_and_fails_loudly_without_a_device(tmp_path):
    exe = _build(tmp_path)
    if _has_device():
        pytest.skip("a CUDA device is present: the GPU test runs the program")
    res = subprocess.run([str(exe), "3"], capture_output=True, text=True, timeout=120)
    assert res.returncode == 1 and "sph_create" in res.stderr, (res.returncode, res.stdout, res.stderr)


@pytest.mark.gpu
def test_c_caller_equals_the_python_mirror(tmp_path):
    exe = _build(tmp_path)
    res = subprocess.run([str(exe), "10"], capture_output=True, text=True, timeout=300)
    assert res.returncode == 0, res.stderr
    tok = res.stdout.split()
    assert tok[0] == "P" and tok[3] == "residual"
    p = S.default_params("spherical", n1=15, n2=13, n3=11, precision="fp64")
    with S.Solver(p) as sv:
        sv.step(10)
        P = sv.get("P")
        r = sv.residual()
    assert float(tok[1]) == float(np.abs(P).max())
    assert float(tok[2]) == pytest.approx(float(P.ravel(order="F").sum()), rel=1e-12)  # C sums in order, numpy pairwise
    assert float(tok[4]) == r["err"]
