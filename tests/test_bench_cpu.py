"""bench.py's reference arm on CPU: its workload equals the library arm's, it never maps the
product library, and its line carries the same ``config`` as the library arm's."""
import json
import math
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))

import bench  # noqa: E402


KEYS = ("geometry", "bc", "rheology", "init", "n1", "n2", "n3", "c1", "c2", "c3", "l1", "l2", "l3", "l_ref", "vpdt", "dmp",
        "g", "tau_C", "n_exp", "relax", "edot_bg", "r", "sh", "eta0", "vr", "rho0", "rho_in", "radius", "incl_linear",
        "etasm_passes")


@pytest.mark.parametrize("n", [31, 255])
def test_reference_workload_equals_library_workload(n):
    lib = bench.workload_params(n, "fp64")
    ref = bench.reference_params(n)
    for k in KEYS:
        assert getattr(ref, k) == pytest.approx(getattr(lib, k), rel=1e-15, abs=0.0), k
    assert tuple(ref.sig_bc) == tuple(lib.sig_bc)


@pytest.mark.parametrize("n", [23, 63])
def test_linear_case_is_the_same_on_both_sides(n):
    """the linear free-slip case: the GPU leg's parameters equal those the oracle port iterates on the CPU"""
    lib = bench.linear_params(n, "fp64")
    ref = bench.linear_reference_params(n)
    for k in KEYS:
        assert getattr(ref, k) == pytest.approx(getattr(lib, k), rel=1e-15, abs=0.0), k
    assert tuple(ref.sig_bc) == tuple(lib.sig_bc) == (0.0, 0.0, 0.0)
    assert lib.bc == 1 and lib.rheology == 0


def test_reference_sample_keeps_the_spacing():
    full, _ = bench.reference_workload(31)
    sample, _ = bench.reference_workload(31, 9)
    assert sample.n3 == 9 and sample.vpdt == full.vpdt
    assert sample.l3 / (sample.n3 - 1) == pytest.approx(full.l3 / (full.n3 - 1), rel=1e-15)
    assert math.isclose(sample.c3, 0.0)


def test_reference_arm_does_not_map_the_product_library():
    code = ("import sys; sys.argv=['bench.py','--impl','reference','--n','23','--steps','2','--warmup','1',"
            "'--ref-seconds','0.5']; import bench; bench.main(); "
            "print('MAPPED', open('/proc/self/maps').read().count('libsphstokes'))")
    out = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr
    lines = out.stdout.strip().splitlines()
    line = json.loads(lines[0])
    assert lines[-1] == "MAPPED 0"
    assert line["impl"] == "reference" and line["config"] == bench.workload_config(23)
    assert line["cpu_baseline"]["kind"] == "port" and line["e2e"]["h2d_bytes_per_step"] == 0
    assert line["ms_per_iteration"] > 0 and line["word_bytes"] == 8


def test_time_to_and_curve_helpers():
    ms = [10.0, 20.0, 30.0, 40.0]
    err = [1.0, 0.5, 0.05, 0.001]
    assert bench._time_to(ms, err, 0.5) == pytest.approx(0.020)
    assert bench._time_to(ms, err, 0.01) == pytest.approx(0.040)
    assert bench._time_to(ms, err, 1e-9) is None
    c = bench._curve(ms, err, keep=3)
    assert c[0] == [0.01, 1.0] and c[-1] == [0.04, 0.001] and len(c) == 3


def test_pt_parameters_states_the_solve_s_own_values():
    p = bench.workload_params(63, "fp64", tuned=True)
    assert bench.pt_parameters(p, 63).startswith("pseudo-step 2x") and "dmp 3" in bench.pt_parameters(p, 63)
    q = bench.workload_params(63, "fp64", dmp=3.5)
    assert "pseudo-step 1x" in bench.pt_parameters(q, 63) and "dmp 3.5" in bench.pt_parameters(q, 63)
