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


@pytest.fixture(scope="module")
def closure_results(tmp_path_factory):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    exe = tmp_path_factory.mktemp("ffc") / "ff_closure_check"
    subprocess.run([gxx, "-O2", "-std=c++17", "-ffp-contract=off", f"-I{CSRC}", f"-I{REPO / 'include'}",
                    str(REPO / "tests" / "native" / "ff_closure_check.cpp"), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    return {ln.split()[0]: [float(x) for x in ln.split()[1:]] for ln in out.splitlines()}


@pytest.mark.parametrize("name", ["vg_unsaturated", "vg_saturated", "bc_unsaturated", "bc_saturated"])
def test_double_float_pressure_head_matches_fp64(closure_results, name):
    """psi_dpsi_ff against the FP64 closure at the same (pair-held) inputs,
    very dry states included: psi to 1e-11 of max(|psi|, 1 m), dpsi (float,
    for the Jacobian: its exponent is formed from the pairs' high words) to
    3e-5 relative; the saturated branch (S > 1) and van Genuchten's very
    dry branch (S^(-1/m) beyond e^80, in log space) stay in double-float;
    Brooks-Corey's very dry points, whose psi leaves the pair's range, go
    back to the FP64 closure."""
    e_psi, e_d, n_ff, n_back = closure_results[name]
    assert e_psi <= 1e-11 and e_d <= 3e-5, (name, e_psi, e_d)
    assert n_ff > 10000, (name, n_ff)
    if name != "bc_unsaturated":
        assert n_back <= 0.002 * n_ff, (name, n_ff, n_back)
