"""ctypes binding of libclimaland_cuda and a handle wrapper.

There is no CPU fallback: if the library is not built or no CUDA device is
present, the calls raise.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _abi as A

_LIB = None


class ClmError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{A.STATUS_NAMES.get(code, code)}: {msg}")
        self.code = code


def load_library(path=None) -> ctypes.CDLL:
    """Load (once) and bind the CUDA library."""
    global _LIB
    if _LIB is None or path is not None:
        p = path or A.library_path()
        if not p.exists():
            raise ClmError(A.CLM_ERR_STATE,
                           f"{p} is not built (run climaland.jl_gb300/build.py or __graft_entry__.build())")
        lib = A.bind(ctypes.CDLL(str(p)))
        if path is not None:
            return lib
        _LIB = lib
    return _LIB


def _c(a, dtype=np.float64):
    if a is None:
        return None
    return np.ascontiguousarray(a, dtype=dtype)


class SoilColumns:
    """One libclimaland_cuda handle holding a batch of soil columns on the GPU.

    Built from a `workloads.Workload` (or any object with the same fields).
    """

    def __init__(self, w, *, precision=None, newton_mode=None, max_iters=None,
                 newton_tol=None, energy_norm_scale=None, cols_per_cta=None, learned_guess=None,
                 schedule=None, graph=None, host_chunks=None, tol_regroup=None, lib=None):
        self.lib = lib or load_library()
        self.w = w
        cfg = A.ClmConfig.from_buffer_copy(w.cfg)
        if precision is not None:
            cfg.precision = precision
        if newton_mode is not None:
            cfg.newton_mode = newton_mode
        if max_iters is not None:
            cfg.max_iters = max_iters
        if newton_tol is not None:
            cfg.newton_tol = newton_tol
        if energy_norm_scale is not None:
            cfg.energy_norm_scale = energy_norm_scale
        if cols_per_cta is not None:
            cfg.cols_per_cta = cols_per_cta
        if learned_guess is not None:
            cfg.learned_guess = int(learned_guess)
        if tol_regroup is not None:
            cfg.tol_regroup = int(tol_regroup)  # enum clm_tol_schedule (a bool: tiles or regroup)
        if schedule is not None:
            cfg.schedule = int(schedule)
        if graph is not None:
            cfg.graph = int(bool(graph))
        if host_chunks is not None:
            cfg.host_chunks = int(host_chunks)
        self.cfg = cfg
        self.eh = cfg.model == A.CLM_MODEL_ENERGY_HYDROLOGY
        self.ncol = w.ncol
        self.ncells = w.ncells
        h = ctypes.c_void_p()
        rc = self.lib.clm_create(ctypes.byref(cfg), ctypes.byref(h))
        if rc != 0:
            raise ClmError(rc, "clm_create failed")
        self.h = h
        self._check(self.lib.clm_set_geometry(self.h, A.dptr(_c(w.z_lo)), A.dptr(_c(w.z_hi)),
                                              A.iptr(_c(w.offsets, np.int32))))
        if getattr(w, "z_faces", None) is not None:  # stretched columns
            self._check(self.lib.clm_set_faces(self.h, A.dptr(_c(w.z_faces))))
        prm = _c(w.params)
        self._check(self.lib.clm_set_params(self.h, A.dptr(prm), prm.shape[0]))
        for slot, f in w.forcing.items():
            f = _c(f)
            self._check(self.lib.clm_set_bc(self.h, int(slot), A.dptr(f), f.shape[0]))
        if getattr(w, "root", None) is not None:
            self.set_root_extraction(w.root)
        if getattr(w, "atmos", None) is not None:
            self.set_atmos(w.atmos, getattr(w, "atmos_params", None))
        self.set_state(w.vartheta_l, w.theta_i, w.rho_e_int, w.intF_w, w.intF_e)

    def set_root_extraction(self, root):
        """RootExtraction canopy values (CLM_RX_NFIELDS rows of ncol), or None
        to remove the source."""
        if root is None:
            self._check(self.lib.clm_set_root_extraction(self.h, None, 0))
            return
        r = _c(root)
        self._check(self.lib.clm_set_root_extraction(self.h, A.dptr(r), r.shape[0]))

    def set_atmos(self, drivers, params=None):
        """Drivers of the atmosphere-driven top boundary (CLM_AT_NFIELDS rows
        of ncol) and its constants (ClmAtmosParams; None: the defaults), or
        drivers None to remove them."""
        if drivers is None:
            self._check(self.lib.clm_set_atmos(self.h, None, None, 0))
            return
        d = _c(drivers)
        pp = ctypes.byref(params) if params is not None else None
        self._check(self.lib.clm_set_atmos(self.h, pp, A.dptr(d), d.shape[0]))

    def atmos_fluxes(self):
        """The boundary's diagnostics at the current state: (CLM_AF_NFIELDS, ncol)."""
        out = np.zeros((A.CLM_AF_NFIELDS, self.ncol))
        self._check(self.lib.clm_atmos_fluxes(self.h, A.dptr(out), A.CLM_AF_NFIELDS))
        return out

    # -- plumbing -----------------------------------------------------------
    def _check(self, rc):
        if rc != 0:
            msg = self.lib.clm_last_error(self.h)
            raise ClmError(rc, msg.decode() if msg else "")

    def close(self):
        if getattr(self, "h", None):
            self.lib.clm_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- state ----------------------------------------------------------------
    def set_state(self, v, ti=None, e=None, Fw=None, Fe=None):
        Fw = np.zeros(self.ncol) if Fw is None else Fw
        if self.eh and Fe is None:
            Fe = np.zeros(self.ncol)
        self._check(self.lib.clm_set_state(self.h, A.dptr(_c(v)), A.dptr(_c(ti) if self.eh else None),
                                           A.dptr(_c(e) if self.eh else None), A.dptr(_c(Fw)),
                                           A.dptr(_c(Fe) if self.eh else None)))

    def get_state(self, out=None):
        """State in the reference layout; `out` (5 arrays, e.g. pinned) is
        filled in place when given."""
        if out is not None:
            v, ti, e, Fw, Fe = out
        else:
            v = np.empty(self.ncells)
            Fw = np.empty(self.ncol)
            ti = e = Fe = None
            if self.eh:
                ti = np.empty(self.ncells)
                e = np.empty(self.ncells)
                Fe = np.empty(self.ncol)
        self._check(self.lib.clm_get_state(self.h, A.dptr(v), A.dptr(ti), A.dptr(e), A.dptr(Fw), A.dptr(Fe)))
        return v, ti, e, Fw, Fe

    def set_state_device(self, ptrs):
        self._check(self.lib.clm_set_state_device(self.h, *[ctypes.c_void_p(p) if p else None for p in ptrs]))

    def get_state_device(self, ptrs):
        self._check(self.lib.clm_get_state_device(self.h, *[ctypes.c_void_p(p) if p else None for p in ptrs]))

    # -- stepping -----------------------------------------------------------------
    def step_host(self, state, t, dt, nsteps=1):
        """clm_step_host: `state` (v, ti, e, Fw, Fe; float64 C-contiguous
        host arrays in the C ABI layout, pinned for overlap) is copied in,
        advanced and copied back in place, pipelined over column chunks."""
        v, ti, e, fw, fe = state
        for a in (v, ti, e, fw, fe):
            assert a is None or (a.dtype == np.float64 and a.flags.c_contiguous)
        self._check(self.lib.clm_step_host(self.h, A.dptr(v), A.dptr(ti), A.dptr(e), A.dptr(fw),
                                           A.dptr(fe), float(t), float(dt), int(nsteps)))

    def step(self, t, dt, nsteps=1):
        self._check(self.lib.clm_step(self.h, float(t), float(dt), int(nsteps)))

    def step_async(self, t, dt, nsteps=1):
        self._check(self.lib.clm_step_async(self.h, float(t), float(dt), int(nsteps)))

    def set_stream(self, stream_ptr):
        """Run on a caller-owned cudaStream_t (an int handle, e.g.
        torch.cuda.Stream().cuda_stream); None restores the handle's own."""
        self._check(self.lib.clm_set_stream(self.h, ctypes.c_void_p(stream_ptr) if stream_ptr else None))

    def sync(self):
        self._check(self.lib.clm_sync(self.h))

    def budgets(self):
        W = np.empty(self.ncol)
        E = np.empty(self.ncol)
        self._check(self.lib.clm_get_budgets(self.h, A.dptr(W), A.dptr(E)))
        return W, E

    def status(self):
        f = np.empty(self.ncol, np.uint32)
        it = np.empty(self.ncol, np.int32)
        self._check(self.lib.clm_get_status(self.h, A.uptr(f), A.iptr(it)))
        return f, it

    # -- learned Newton guess ---------------------------------------------------------
    def autotune(self, t, dt, probe_steps=4):
        """clm_autotune: time every launch configuration on probe_steps
        steps from the current state (which is restored) and keep the
        fastest. Returns the timed candidates as dicts."""
        table = (A.ClmTuneEntry * 16)()
        n = ctypes.c_int32(0)
        self._check(self.lib.clm_autotune(self.h, float(t), float(dt), int(probe_steps),
                                          ctypes.cast(table, ctypes.c_void_p), 16, ctypes.byref(n)))
        return [{k: getattr(table[i], k) for k, _ in A.ClmTuneEntry._fields_} for i in range(min(n.value, 16))]

    def launch_config(self):
        c, s, g = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
        self._check(self.lib.clm_get_launch_config(self.h, ctypes.byref(c), ctypes.byref(s), ctypes.byref(g)))
        return {"cols_per_cta": c.value, "schedule": s.value, "grid": g.value}

    def load_mlp(self, blob: bytes):
        buf = ctypes.create_string_buffer(bytes(blob), len(blob))
        self._check(self.lib.clm_load_mlp(self.h, buf, len(blob)))

    def features(self, t, dt, X_ptr):
        """Raw network inputs (ncol x 67 floats) into the device array X_ptr."""
        self._check(self.lib.clm_features(self.h, float(t), float(dt), ctypes.c_void_p(X_ptr)))

    # -- closures -----------------------------------------------------------------
    def update_aux(self, t):
        nc = self.ncells
        out = {k: np.zeros(nc) for k in ("K", "psi", "theta_l", "T", "kappa", "Tf")}
        bc = np.zeros(4 * self.ncol)
        self._check(self.lib.clm_update_aux(
            self.h, float(t), *[A.dptr(out[k]) for k in ("K", "psi", "theta_l", "T", "kappa", "Tf")],
            A.dptr(bc)))
        out["bc"] = bc.reshape(4, self.ncol)
        return out

    def _tend(self, fn, t):
        nc, ncol = self.ncells, self.ncol
        d = [np.zeros(nc), np.zeros(nc), np.zeros(nc), np.zeros(ncol), np.zeros(ncol)]
        self._check(fn(self.h, float(t), *[A.dptr(a) for a in d]))
        return d

    def exp_tendency(self, t):
        return self._tend(self.lib.clm_exp_tendency, t)

    def imp_tendency(self, t):
        return self._tend(self.lib.clm_imp_tendency, t)

    def jacobian(self, t, dtgamma):
        nc = self.ncells
        J = [np.zeros(3 * nc) for _ in range(3)]
        self._check(self.lib.clm_jacobian(self.h, float(t), float(dtgamma), *[A.dptr(a) for a in J]))
        return [a.reshape(nc, 3) for a in J]

    def solve(self, Wvv, Wev, Wee, fv, fe):
        nc = self.ncells
        dv = np.zeros(nc)
        de = np.zeros(nc)
        self._check(self.lib.clm_solve(self.h, A.dptr(_c(Wvv)), A.dptr(_c(Wev)), A.dptr(_c(Wee)),
                                       A.dptr(_c(fv)), A.dptr(_c(fe)), A.dptr(dv), A.dptr(de)))
        return dv, de
