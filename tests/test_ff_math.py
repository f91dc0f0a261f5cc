"""Double-float arithmetic of the mixed path (clm_ff.cuh), compiled for the
host with g++ (no a*b+c contraction) and checked against FP64: conversions,
add, mul, div, exp and log stay within 2^-44 relative (log: relative to
max(1, |log x|), the precision of a double-float of that size)."""
import shutil
import subprocess
from pathlib import Path

import pytest

REPO = Path(__file__).resolve().parent.parent
SRC = REPO / "tests" / "native" / "ff_check.cpp"
CSRC = REPO / "climaland.jl_gb300" / "csrc"


@pytest.fixture(scope="module")
def results(tmp_path_factory):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    exe = tmp_path_factory.mktemp("ff") / "ff_check"
    subprocess.run([gxx, "-O2", "-std=c++17", "-ffp-contract=off", f"-I{CSRC}", str(SRC), "-o", str(exe)],
                   check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    return {line.split()[0]: float(line.split()[1]) for line in out.splitlines()}


@pytest.mark.parametrize("name,bound", [
    ("roundtrip", 2.0 ** -47), ("add", 2.0 ** -46), ("mul", 2.0 ** -45), ("div", 2.0 ** -44),
    ("exp", 2.0 ** -44), ("log_abs", 2.0 ** -44),
])
def test_double_float_accuracy(results, name, bound):
    assert results[name] <= bound, (name, results[name], bound)
