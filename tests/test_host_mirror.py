"""The Python mirror of the reference interface (soil.py, simulation.py):
model/BC types translate into the C-ABI description the oracle and the
library consume (CPU only; the GPU run is in test_gpu_simulation.py)."""
import numpy as np

import oracle as O
from climaland_gb300 import _abi as A
from climaland_gb300 import parameters as PR
from climaland_gb300 import soil as S


def eh_model(ncol=4):
    p = PR.EnergyHydrologyParameters.from_composition(
        nu=0.495, nu_ss_om=0.0, nu_ss_quartz=1.0, nu_ss_gravel=0.0,
        hydrology_cm=PR.vanGenuchten(2.6, 2.0), K_sat=0.0443 / 3600 / 100, S_s=1e-3, theta_r=0.1)
    top = S.WaterHeatBC(water=S.WaterFluxBC(-1e-7),
                        heat=S.HeatFluxBC(S.Forcing(amp=150.0, omega=2 * np.pi / 86400)))
    return S.EnergyHydrology(parameters=p, domain=S.Column(zlim=(-1.0, 0.0), nelements=20, ncol=ncol),
                             boundary_conditions=dict(top=top, bottom=S.EnergyWaterFreeDrainage()))


def test_energy_hydrology_translation():
    m = eh_model()
    cfg = m.config()
    assert cfg.model == A.CLM_MODEL_ENERGY_HYDROLOGY and cfg.phase_change == 1
    assert (cfg.bc_top_water, cfg.bc_top_heat) == (A.CLM_BC_FLUX, A.CLM_BC_FLUX)
    assert (cfg.bc_bottom_water, cfg.bc_bottom_heat) == (A.CLM_BC_FREE_DRAINAGE,) * 2
    f = m.forcing()
    assert np.all(f[A.CLM_BC_TOP_WATER][A.CLM_F_BASE] == -1e-7)
    assert np.all(f[A.CLM_BC_TOP_HEAT][A.CLM_F_AMP] == 150.0)
    Y = m.initialize()
    Y["vartheta_l"][:] = 0.3
    rc = m.parameters.rho_c_ds + 0.3 * A.DEFAULT_EARTH["cp_l"] * A.DEFAULT_EARTH["rho_l"]
    Y["rho_e_int"][:] = rc * (285.0 - A.DEFAULT_EARTH["T_0"])
    w = S.to_workload(m, Y, dt=450.0)
    assert w.cfg.nlayers == 20 and w.ncells == 80
    st = w.copy_state()
    rc_, fl, it = O.Oracle(w).step(st, 0.0, 450.0, 10)
    assert rc_ == 0 and fl.max() == 0


def test_richards_translation_moisture_state():
    p = PR.RichardsParameters(nu=0.495, hydrology_cm=PR.vanGenuchten(2.6, 1.43),
                              K_sat=0.0443 / 3600 / 100, S_s=1e-3, theta_r=0.124)
    m = S.RichardsModel(parameters=p, domain=S.Column(zlim=(-1.5, 0.0), nelements=150),
                        boundary_conditions=dict(top=S.MoistureStateBC(0.494), bottom=S.FreeDrainage()))
    cfg = m.config()
    assert cfg.bc_top_water == A.CLM_BC_STATE and cfg.bc_bottom_water == A.CLM_BC_FREE_DRAINAGE
    assert m.forcing()[A.CLM_BC_TOP_WATER][A.CLM_F_BASE][0] == 0.494
    assert A.CLM_BC_BOTTOM_WATER not in m.forcing()


def test_column_geometry_matches_reference_centres():
    c = S.Column(zlim=(-10.0, 0.0), nelements=50)
    z = c.centers()
    zf = np.linspace(-10.0, 0.0, 51)
    assert np.allclose(z, 0.5 * (zf[1:] + zf[:-1]), atol=1e-14)
