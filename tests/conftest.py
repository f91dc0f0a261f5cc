import os
import sys
from pathlib import Path

import pytest

REPO = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(REPO / "climaland.jl_gb300"))
sys.path.insert(0, str(REPO / "oracle"))
sys.path.insert(0, str(REPO))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: longer CPU test")


def pytest_terminal_summary(terminalreporter):
    """One line per parity test: columns, steps, the excused fraction (columns
    above the bar, within 10 x the oracle's own spread) and the largest
    errors."""
    gc = sys.modules.get("gpu_common")
    if gc is None or not getattr(gc, "SUMMARY", None):
        return
    tr = terminalreporter
    tr.write_sep("-", "parity against the oracle (excused: above the bar, within 10 x the oracle's spread)")
    for name, st in gc.SUMMARY:
        errs = " ".join(f"{k[:-len('_max_err_all')]}={v:.2e}" for k, v in st.items() if k.endswith("_max_err_all"))
        tr.write_line(f"{name}: {st['columns']} cols x {st.get('steps', '?')} steps, noise {st.get('noise')}, "
                      f"excused {st['excused']} ({100 * st['excused_frac']:.2f} %; oracle itself "
                      f"{100 * st.get('oracle_self_excused_frac', 0.0):.2f} %), "
                      f"err/spread max {st['excused_err_over_spread_max']:.2g}, "
                      f"re-measured {st.get('rechecked', 0)}, {errs}")
