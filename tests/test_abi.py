"""CPU checks of the C ABI: the library builds, loads without a GPU and
exports every function include/climaland_cuda.h declares; the ctypes
mirror agrees with the header; host-only entry points behave."""
import ctypes
import re
from pathlib import Path

import pytest

import oracle as O
from climaland_gb300 import _abi as A

REPO = Path(__file__).resolve().parent.parent
HEADER = REPO / "include" / "climaland_cuda.h"


def header_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[a-z_0-9]+\s*\*?\s*(clm_[a-z_0-9]+)\s*\(", text, flags=re.M)
    return sorted(set(names))


@pytest.fixture(scope="module")
def lib():
    import sys
    sys.path.insert(0, str(REPO / "climaland.jl_gb300"))
    import build as B
    path = B.build()
    return A.bind(ctypes.CDLL(str(path)))


def test_header_and_mirror_agree():
    assert header_functions() == sorted(A.declared_symbols())


def test_library_exports_every_declared_symbol(lib):
    for name in header_functions():
        assert hasattr(lib, name), name


def test_config_struct_size_matches(lib):
    # clm_config_default writes sizeof(clm_config) bytes; a larger guard
    # buffer catches a size mismatch between ctypes and C.
    buf = (ctypes.c_ubyte * (ctypes.sizeof(A.ClmConfig) + 64))()
    for i in range(len(buf)):
        buf[i] = 0xAB
    lib.clm_config_default(ctypes.cast(buf, ctypes.POINTER(A.ClmConfig)))
    tail = bytes(buf[ctypes.sizeof(A.ClmConfig):])
    assert tail == b"\xab" * 64
    c = A.ClmConfig.from_buffer_copy(bytes(buf[: ctypes.sizeof(A.ClmConfig)]))
    d = A.default_config()
    assert A.config_to_dict(c) == A.config_to_dict(d)


def test_forcing_hash_matches_oracle(lib):
    ol = O.lib()
    for seed in (0, 7, 4000):
        for c in (0, 1, 31, 1048575):
            for k in (0, 1, 23, 191):
                assert lib.clm_forcing_hash01(seed, c, k) == ol.clm_forcing_hash01(seed, c, k)


def test_version(lib):
    assert b"sm_103a" in lib.clm_version()


def test_create_rejects_bad_config_before_touching_the_device(lib):
    cfg = A.default_config()
    cfg.ncol = 0
    h = ctypes.c_void_p()
    assert lib.clm_create(ctypes.byref(cfg), ctypes.byref(h)) == A.CLM_ERR_ARG
    cfg.ncol = 10
    cfg.bc_top_water = A.CLM_BC_FREE_DRAINAGE
    assert lib.clm_create(ctypes.byref(cfg), ctypes.byref(h)) == A.CLM_ERR_ARG
    assert lib.clm_last_error(None) == b"null handle"


def test_guess_modes_match_the_header_and_are_checked(lib):
    import re
    text = (REPO / "include" / "climaland_cuda.h").read_text()
    body = re.search(r"enum clm_guess \{([^}]*)\}", text).group(1)
    vals = {k: int(v) for k, v in re.findall(r"(CLM_GUESS_\w+) = (\d+)", body)}
    assert vals == {"CLM_GUESS_NONE": A.CLM_GUESS_NONE, "CLM_GUESS_NETWORK": A.CLM_GUESS_NETWORK,
                    "CLM_GUESS_EXTRAPOLATE": A.CLM_GUESS_EXTRAPOLATE}
    h = ctypes.c_void_p()
    cfg = A.default_config()
    cfg.ncol = 10
    cfg.model = A.CLM_MODEL_ENERGY_HYDROLOGY
    cfg.learned_guess = A.CLM_GUESS_EXTRAPOLATE  # with fixed Newton: nothing to start
    assert lib.clm_create(ctypes.byref(cfg), ctypes.byref(h)) == A.CLM_ERR_ARG
    cfg.newton_mode = A.CLM_NEWTON_TOL
    cfg.learned_guess = 3
    assert lib.clm_create(ctypes.byref(cfg), ctypes.byref(h)) == A.CLM_ERR_ARG


def test_tolerance_schedules_match_the_header_and_are_checked(lib):
    """enum clm_tol_schedule in the header, the ctypes mirror and the Julia
    binding agree; the default is CLM_TOL_AUTO (clm_config_default and the
    mirror's default_config); values outside the enum are refused before
    the device is touched."""
    import re
    text = (REPO / "include" / "climaland_cuda.h").read_text()
    body = re.search(r"enum clm_tol_schedule \{([^}]*)\}", text).group(1)
    vals = {k: int(v) for k, v in re.findall(r"(CLM_TOL_\w+) = (\d+)", body)}
    assert vals == {"CLM_TOL_TILES": A.CLM_TOL_TILES, "CLM_TOL_REGROUP": A.CLM_TOL_REGROUP,
                    "CLM_TOL_SPLIT": A.CLM_TOL_SPLIT, "CLM_TOL_AUTO": A.CLM_TOL_AUTO}
    jl = (REPO / "climaland.jl_gb300" / "julia" / "ClimaLandGB300.jl").read_text()
    for k, v in vals.items():
        assert re.search(rf"const {k} = Int32\({v}\)", jl), k
    c = A.ClmConfig()
    lib.clm_config_default(ctypes.byref(c))
    assert c.tol_regroup == A.CLM_TOL_AUTO == A.default_config().tol_regroup
    h = ctypes.c_void_p()
    for bad in (-1, 4):
        cfg = A.default_config()
        cfg.ncol = 10
        cfg.newton_mode = A.CLM_NEWTON_TOL
        cfg.tol_regroup = bad
        assert lib.clm_create(ctypes.byref(cfg), ctypes.byref(h)) == A.CLM_ERR_ARG


def test_create_rejects_runoff_outside_richards(lib):
    # the precipitation/runoff top boundary is RichardsAtmosDrivenFluxBC: an
    # EnergyHydrology handle (whose atmosphere-driven boundary is
    # CLM_BC_ATMOS), the heat or bottom slots and unknown runoff kinds are
    # refused before any device work
    h = ctypes.c_void_p()
    cfg = A.default_config()
    cfg.ncol = 10
    cfg.nlayers = 5
    cfg.bc_top_water = A.CLM_BC_PRECIP_RUNOFF
    assert lib.clm_create(ctypes.byref(cfg), ctypes.byref(h)) == A.CLM_ERR_ARG  # EnergyHydrology
    cfg.model = A.CLM_MODEL_RICHARDS
    cfg.runoff = 7
    assert lib.clm_create(ctypes.byref(cfg), ctypes.byref(h)) == A.CLM_ERR_ARG
    cfg.runoff = A.CLM_RUNOFF_TOPMODEL
    cfg.bc_top_water = A.CLM_BC_FLUX
    cfg.bc_bottom_water = A.CLM_BC_PRECIP_RUNOFF
    assert lib.clm_create(ctypes.byref(cfg), ctypes.byref(h)) == A.CLM_ERR_ARG


def test_create_rejects_unknown_hydrology_closure(lib):
    h = ctypes.c_void_p()
    cfg = A.default_config()
    cfg.ncol = 10
    cfg.nlayers = 5
    cfg.hydrology_cm = 2
    assert lib.clm_create(ctypes.byref(cfg), ctypes.byref(h)) == A.CLM_ERR_ARG
    cfg.hydrology_cm = -1
    assert lib.clm_create(ctypes.byref(cfg), ctypes.byref(h)) == A.CLM_ERR_ARG


def test_julia_binding_config_matches_the_header_layout():
    # the Julia mirror of clm_config must list the ctypes fields in order
    # with the same widths (ccall passes the struct by reference)
    text = (REPO / "climaland.jl_gb300" / "julia" / "ClimaLandGB300.jl").read_text()
    body = re.search(r"mutable struct ClmConfig\n(.*?)\n\s*ClmConfig\(\) = new\(\)", text, re.S).group(1)
    fields = re.findall(r"^\s*([A-Za-z_0-9]+)::([A-Za-z0-9]+)", body, re.M)
    jl = {"Int32": ctypes.c_int32, "Int64": ctypes.c_int64, "UInt64": ctypes.c_uint64,
          "Float64": ctypes.c_double, "ClmEarthParams": A.ClmEarthParams}
    assert [n for n, _ in fields] == [n for n, _ in A.ClmConfig._fields_]
    for (n, t), (_, ct) in zip(fields, A.ClmConfig._fields_):
        assert ctypes.sizeof(jl[t]) == ctypes.sizeof(ct), n


def test_atmos_params_default_matches_the_mirror(lib):
    # clm_atmos_params_default writes exactly sizeof(ClmAtmosParams) bytes
    # and the Python twin holds the same values
    buf = (ctypes.c_ubyte * (ctypes.sizeof(A.ClmAtmosParams) + 64))()
    for i in range(len(buf)):
        buf[i] = 0xAB
    lib.clm_atmos_params_default(ctypes.cast(buf, ctypes.POINTER(A.ClmAtmosParams)))
    assert all(b == 0xAB for b in bytes(buf[ctypes.sizeof(A.ClmAtmosParams):]))
    a = A.ClmAtmosParams.from_buffer_copy(bytes(buf[: ctypes.sizeof(A.ClmAtmosParams)]))
    for k, v in A.DEFAULT_ATMOS.items():
        assert getattr(a, k) == v, k


def test_create_rejects_misplaced_atmos_boundary(lib):
    h = ctypes.c_void_p()
    for model, tw, th, runoff in ((A.CLM_MODEL_RICHARDS, A.CLM_BC_ATMOS, A.CLM_BC_ATMOS, 0),
                                  (A.CLM_MODEL_ENERGY_HYDROLOGY, A.CLM_BC_ATMOS, A.CLM_BC_FLUX, 0),
                                  (A.CLM_MODEL_ENERGY_HYDROLOGY, A.CLM_BC_FLUX, A.CLM_BC_ATMOS, 0),
                                  (A.CLM_MODEL_ENERGY_HYDROLOGY, A.CLM_BC_ATMOS, A.CLM_BC_ATMOS, 7)):
        cfg = A.default_config()
        cfg.model, cfg.ncol, cfg.nlayers = model, 4, 5
        cfg.bc_top_water, cfg.bc_top_heat, cfg.runoff = tw, th, runoff
        assert lib.clm_create(ctypes.byref(cfg), ctypes.byref(h)) == A.CLM_ERR_ARG
    cfg = A.default_config()
    cfg.ncol, cfg.nlayers = 4, 5
    cfg.bc_bottom_water = A.CLM_BC_ATMOS  # a top-only kind
    assert lib.clm_create(ctypes.byref(cfg), ctypes.byref(h)) == A.CLM_ERR_ARG


# ---- the Julia binding's ccall signatures against the header ------------------

def _header_prototypes():
    """{name: (return type, [argument types])} of every function the header
    declares (argument names dropped, whitespace normalised)."""
    text = (REPO / "include" / "climaland_cuda.h").read_text()
    text = re.sub(r"/\*.*?\*/", " ", text, flags=re.S)
    out = {}
    for m in re.finditer(r"\n\s*([A-Za-z_][A-Za-z0-9_ \*]*?)\b(clm_[a-z0-9_]+)\s*\(([^;{]*?)\)\s*;", text):
        ret = " ".join(m.group(1).split())
        args = [] if m.group(3).strip() in ("", "void") else [" ".join(a.split()) for a in m.group(3).split(",")]
        types = []
        for a in args:
            a = re.sub(r"\s*\*\s*", "* ", a).strip()
            parts = a.split()
            # drop the parameter name: the last token unless it is a type word
            if len(parts) > 1 and not parts[-1].endswith("*") and parts[-1] not in ("int", "double"):
                parts = parts[:-1]
            types.append(" ".join(parts).replace("* *", "**").replace(" *", "*"))
        out[m.group(2)] = (ret, types)
    return out


def _julia_ccalls():
    """[(name, return type, [argument types])] of every ccall in the binding."""
    text = (REPO / "climaland.jl_gb300" / "julia" / "ClimaLandGB300.jl").read_text()
    calls = []
    for m in re.finditer(r"ccall\(\(:(clm_[a-z0-9_]+),\s*libclm\),\s*([A-Za-z0-9_{}]+),\s*\(", text):
        i, depth, j = m.end(), 1, m.end()
        while depth:
            depth += {"(": 1, ")": -1}.get(text[j], 0)
            j += 1
        tup = text[i:j - 1]
        types, buf, d = [], "", 0
        for ch in tup:
            if ch == "," and d == 0:
                types.append(buf.strip())
                buf = ""
                continue
            d += {"{": 1, "}": -1}.get(ch, 0)
            buf += ch
        if buf.strip():
            types.append(buf.strip())
        calls.append((m.group(1), m.group(2), types))
    return calls


_C_TO_JULIA = {
    "int": {"Cint", "Int32"}, "void": {"Cvoid"}, "const char*": {"Cstring"}, "double": {"Float64"},
    "int32_t": {"Int32"}, "int64_t": {"Int64"}, "uint64_t": {"UInt64"},
    "clm_handle*": {"Ptr{Cvoid}"}, "const clm_handle*": {"Ptr{Cvoid}"}, "clm_handle**": {"Ref{Ptr{Cvoid}}"},
    "const clm_config*": {"Ref{ClmConfig}", "Ptr{ClmConfig}"}, "clm_config*": {"Ref{ClmConfig}"},
    "clm_atmos_params*": {"Ref{ClmAtmosParams}"},
    "const clm_atmos_params*": {"Ref{ClmAtmosParams}", "Ptr{ClmAtmosParams}"},
    "double*": {"Ptr{Float64}", "Ref{Float64}", "Ptr{Cvoid}"},
    "const double*": {"Ptr{Float64}", "Ref{Float64}", "Ptr{Cvoid}"},
    "int32_t*": {"Ptr{Int32}"}, "const int32_t*": {"Ptr{Int32}"}, "uint32_t*": {"Ptr{UInt32}"},
    "void*": {"Ptr{Cvoid}"}, "const void*": {"Ptr{Cvoid}"},
}


def test_julia_ccalls_match_the_header():
    """Every ccall of the Julia binding names a header function with the same
    number of arguments, and each Julia argument type is one that ccall
    converts to the header's C type (pointers of the right element type, or
    Ptr{Cvoid} for device memory; integer widths exact)."""
    protos = _header_prototypes()
    calls = _julia_ccalls()
    assert len(calls) >= 25
    wrapped = set()
    for name, ret, types in calls:
        assert name in protos, name
        cret, cargs = protos[name]
        assert ret in _C_TO_JULIA[cret], (name, ret, cret)
        assert len(types) == len(cargs), (name, types, cargs)
        for jt, ct in zip(types, cargs):
            assert jt in _C_TO_JULIA[ct], (name, jt, ct)
        wrapped.add(name)
    # the closure-level entry points a ClimaTimeSteppers host binds
    for name in ("clm_update_aux", "clm_exp_tendency", "clm_imp_tendency", "clm_jacobian", "clm_solve",
                 "clm_get_budgets", "clm_get_status", "clm_set_faces", "clm_step", "clm_set_state",
                 "clm_get_state", "clm_set_state_device"):
        assert name in wrapped, name


def test_julia_structs_match_the_header_offsets():
    """ClmConfig, ClmEarthParams and ClmAtmosParams: each Julia field at the C
    offset (natural alignment, as Julia lays out isbits fields)."""
    text = (REPO / "climaland.jl_gb300" / "julia" / "ClimaLandGB300.jl").read_text()
    size = {"Int32": 4, "Int64": 8, "UInt64": 8, "Float64": 8}
    layouts = {}

    def layout(name):
        if name in layouts:
            return layouts[name]
        body = re.search(r"(?:mutable )?struct %s\n(.*?)\n(?:\s*%s\(\) = new\(\)\n)?end" % (name, name), text, re.S).group(1)
        off, fields, align = 0, [], 1
        for fn, ft in re.findall(r"^\s*([A-Za-z_0-9]+)::([A-Za-z0-9]+)", body, re.M):
            sz, al = (size[ft], size[ft]) if ft in size else layout(ft)[1:3]
            off = (off + al - 1) // al * al
            fields.append((fn, off))
            off += sz
            align = max(align, al)
        total = (off + align - 1) // align * align
        layouts[name] = (fields, total, align)
        return layouts[name]

    for jname, cstruct in (("ClmConfig", A.ClmConfig), ("ClmEarthParams", A.ClmEarthParams),
                           ("ClmAtmosParams", A.ClmAtmosParams)):
        fields, total, _ = layout(jname)
        assert [f for f, _ in fields] == [f for f, _ in cstruct._fields_], jname
        for fn, off in fields:
            assert getattr(cstruct, fn).offset == off, (jname, fn)
        assert total == ctypes.sizeof(cstruct), jname
