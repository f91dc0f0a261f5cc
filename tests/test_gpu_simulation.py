"""LandSimulation (step!/solve!) on the GPU against the oracle."""
import numpy as np
import pytest

import oracle as O
from climaland_gb300 import _abi as A
from climaland_gb300 import simulation as SIM
from climaland_gb300 import soil as S
from gpu_common import require_gpu
from test_host_mirror import eh_model

pytestmark = pytest.mark.gpu


def test_land_simulation_solve_matches_oracle():
    require_gpu()
    m = eh_model(ncol=64)
    Y = m.initialize()
    z = m.domain.centers()
    Y["vartheta_l"][:] = 0.25 + 0.05 * (z + 0.5) ** 2
    rc = m.parameters.rho_c_ds + Y["vartheta_l"] * A.DEFAULT_EARTH["cp_l"] * A.DEFAULT_EARTH["rho_l"]
    Y["rho_e_int"][:] = rc * (280.0 + 2.0 * z - A.DEFAULT_EARTH["T_0"])
    sim = SIM.LandSimulation(0.0, 450.0 * 48, 450.0, m, Y)
    sim.step()
    sim.solve()
    assert abs(sim.t - 450.0 * 48) < 1e-9
    got = sim.Y
    sim.close()
    w = S.to_workload(m, Y, dt=450.0)
    st = w.copy_state()
    O.Oracle(w).step(st, 0.0, 450.0, 48)
    assert np.max(np.abs(got["vartheta_l"] - st[0])) < 1e-10
    assert np.max(np.abs(got["rho_e_int"] - st[2])) / np.max(np.abs(st[2])) < 1e-10
