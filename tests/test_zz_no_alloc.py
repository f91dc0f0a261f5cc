"""The allocation-free step (clm_step_eh_noalloc) against the handle path.

Callers whose device memory belongs to another allocator (a caching
allocator under a fixed budget), or who forbid allocation after start-up,
cannot let the library call cudaMalloc; this entry
point takes every buffer from the caller and keeps its working scratch in a
fixed array inside the library. The test drives it through the C ABI on
caller-owned device buffers for two calls in a row and compares each result
with the handle API's clm_step on the same workload, at the parity
tolerance of the other GPU tests (1e-10). This file is collected last so
that a failure here comes after every other test has run.
"""
import ctypes

import numpy as np
import pytest

from climaland_gb300 import _abi as A
from climaland_gb300 import device as D
from climaland_gb300 import workloads as WL

pytestmark = pytest.mark.gpu

TOL = 1e-10


@pytest.fixture
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _workload(brooks_corey=False):
    w = WL.energy_hydrology_c1(ncol=1000, nlayers=15, seed=7)
    w.params[A.CLM_P_K_SAT] = np.minimum(w.params[A.CLM_P_K_SAT], 1e-5)
    return WL.brooks_corey(w) if brooks_corey else w


@pytest.mark.parametrize("case", ["van_genuchten", "brooks_corey", "deepest_widest"])
def test_noalloc_matches_handle_path_two_calls(torch_cuda, case):
    torch = torch_cuda
    lib = D.load_library()
    nsteps = 6
    if case == "deepest_widest":
        # the documented maximum depth (32 layers: the largest shared-memory
        # request) on enough columns that the grid reaches the 1024-slot cap
        # of the fixed scratch array, so the last slot's scratch is used
        w = WL.energy_hydrology_c1(ncol=40000, nlayers=32, seed=11)
        w.params[A.CLM_P_K_SAT] = np.minimum(w.params[A.CLM_P_K_SAT], 1e-5)
        nsteps = 2
    else:
        w = _workload(case == "brooks_corey")
    # reference: the handle API, two calls
    with D.SoilColumns(w) as g:
        g.step(w.t0, w.dt, nsteps)
        ref1 = g.get_state()
        g.step(w.t0 + nsteps * w.dt, w.dt, nsteps)
        ref2 = g.get_state()
    # caller-owned device buffers in the reference layout
    dev = lambda a: torch.tensor(np.ascontiguousarray(a), dtype=torch.float64, device="cuda")
    z_lo, z_hi, prm = dev(w.z_lo), dev(w.z_hi), dev(w.params)
    forc = {s: dev(f) for s, f in w.forcing.items()}
    fptr = (ctypes.c_void_p * 4)(*[forc[s].data_ptr() if s in forc else None for s in range(4)])
    st = [dev(a) for a in w.copy_state()]
    flags = torch.zeros(w.ncol, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream()

    def call(t):
        return lib.clm_step_eh_noalloc(
            ctypes.byref(w.cfg), w.ncol, int(w.nlayers[0]), z_lo.data_ptr(), z_hi.data_ptr(),
            prm.data_ptr(), fptr, st[0].data_ptr(), st[1].data_ptr(), st[2].data_ptr(),
            st[3].data_ptr(), st[4].data_ptr(), flags.data_ptr(), t, w.dt, nsteps,
            ctypes.c_void_p(stream.cuda_stream))

    assert call(w.t0) == A.CLM_OK
    torch.cuda.synchronize()
    got1 = [x.cpu().numpy() for x in st]
    assert call(w.t0 + nsteps * w.dt) == A.CLM_OK
    torch.cuda.synchronize()
    got2 = [x.cpu().numpy() for x in st]
    # the calls allocate no device memory: repeated calls leave the device's
    # free memory unchanged (the driver may reserve memory of its own once,
    # e.g. local memory on a kernel's first launches, so the reading starts
    # after two calls)
    free = []
    t = w.t0 + 2 * nsteps * w.dt
    for _ in range(3):
        assert call(t) == A.CLM_OK
        torch.cuda.synchronize()
        free.append(torch.cuda.mem_get_info()[0])
        t += nsteps * w.dt
    assert free[0] == free[1] == free[2]
    for got, ref in ((got1, ref1), (got2, ref2)):
        assert np.max(np.abs(got[0] - ref[0])) <= TOL
        assert np.max(np.abs(got[1] - ref[1])) <= TOL
        assert np.max(np.abs(got[2] - ref[2])) / np.max(np.abs(ref[2])) <= TOL
        assert np.max(np.abs(got[3] - ref[3])) <= TOL * max(np.max(np.abs(ref[3])), 1.0)
        assert np.max(np.abs(got[4] - ref[4])) / max(np.max(np.abs(ref[4])), 1.0) <= TOL
    assert int(flags.max()) == 0


def test_noalloc_rejects_sizes_beyond_its_maximum(torch_cuda):
    lib = D.load_library()
    w = _workload()
    null = None
    for nl in (1, 33, 64):
        rc = lib.clm_step_eh_noalloc(ctypes.byref(w.cfg), w.ncol, nl, null, null, null, null,
                                     null, null, null, null, null, null, 0.0, w.dt, 1, null)
        assert rc == A.CLM_ERR_ARG


# configurations clm_create refuses (a boundary kind in a slot that does not
# admit it, Newton settings out of range; create=True) and the options this
# entry point does not carry (mixed path, learned guess, RichardsModel)
REFUSED = [
    ("bc_top_water", A.CLM_BC_FREE_DRAINAGE, True),
    ("bc_top_heat", A.CLM_BC_FREE_DRAINAGE, True),
    ("bc_top_water", A.CLM_BC_FLUX_ADVECTIVE, True),
    ("bc_bottom_water", A.CLM_BC_FLUX_ADVECTIVE, True),
    ("bc_bottom_heat", A.CLM_BC_FLUX_ADVECTIVE, True),
    ("bc_top_water", A.CLM_BC_PRECIP_RUNOFF, True),
    ("newton_mode", 7, True),
    ("max_iters", 0, True),
    ("max_iters", 1001, True),
    ("hydrology_cm", 5, True),
    ("precision", A.CLM_PREC_MIXED, False),
    ("learned_guess", 1, False),
    ("model", A.CLM_MODEL_RICHARDS, False),
]


@pytest.mark.parametrize("field,value,create", REFUSED)
def test_noalloc_rejects_configurations_clm_create_rejects(torch_cuda, field, value, create):
    lib = D.load_library()
    w = _workload()
    null = None
    cfg = A.ClmConfig.from_buffer_copy(w.cfg)
    setattr(cfg, field, value)
    rc = lib.clm_step_eh_noalloc(ctypes.byref(cfg), w.ncol, 15, null, null, null, null,
                                 null, null, null, null, null, null, 0.0, w.dt, 1, null)
    assert rc == A.CLM_ERR_ARG
    if create:  # the handle API refuses the same configuration
        h = A._H()
        assert lib.clm_create(ctypes.byref(cfg), ctypes.byref(h)) == A.CLM_ERR_ARG
        assert not h.value
