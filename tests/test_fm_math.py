"""FP64 fast math of the column kernels (clm_fastmath.cuh), compiled for the
host with g++ (no a*b+c contraction outside the explicit fma calls) and
checked against libm and IEEE division: the table-driven exp and log within
about one ulp, the Newton-Raphson reciprocal within one ulp (special values
and magnitudes beyond 2^120 through the division itself)."""
import shutil
import subprocess
from pathlib import Path

import pytest

REPO = Path(__file__).resolve().parent.parent
SRC = REPO / "tests" / "native" / "fm_check.cpp"
CSRC = REPO / "climaland.jl_gb300" / "csrc"


@pytest.fixture(scope="module")
def results(tmp_path_factory):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    exe = tmp_path_factory.mktemp("fm") / "fm_check"
    subprocess.run([gxx, "-O2", "-std=c++17", "-ffp-contract=off", f"-I{CSRC}", str(SRC), "-o", str(exe)],
                   check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    return {line.split()[0]: float(line.split()[1]) for line in out.splitlines()}


@pytest.mark.parametrize("name,bound", [
    ("exp", 1.05), ("log", 1.05), ("rcp", 1.0), ("rcp_wide", 1.0), ("rcp_special", 0.0),
])
def test_fast_math_accuracy(results, name, bound):
    assert results[name] <= bound, (name, results[name], bound)
