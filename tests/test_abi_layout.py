"""The ctypes mirror of the C ABI against the headers themselves.

A C program compiled against include/poe2d.h and include/poe2d_surrogate.h
prints the size and field offsets of every public struct and the value of
every public constant; the Python binding (poe2d_gb300._lib, surrogate.py)
must agree with all of them, so a header change that the binding missed fails
here, on the CPU, instead of as wrong arguments on the GPU.
"""
import ctypes as C
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

STRUCTS = {
    "poe_grid": ("Grid", ["NX", "NZ", "dx", "dz", "dt"]),
    "poe_pml_params": ("PmlParams", ["npoints", "rcoef", "npower", "k_max", "alpha_max", "alpha_top_extra",
                                     "cp_max"]),
    "poe_source": ("Source", ["ix", "iz", "kind", "f0", "amplitude", "t_cut"]),
    "poe_receiver": ("Receiver", ["ix", "iz", "comp"]),
    "poe_biot_material": ("BiotMaterial", ["rho_s", "phi", "k_s", "k_frame", "mu_frame", "rho_f", "k_f", "eta",
                                           "kappa", "tortuosity"]),
    "poe_checkpoint_header": ("CheckpointHeader", ["magic", "version", "header_bytes", "NX", "NZ", "P", "R", "Wx",
                                                   "Hz", "plane", "steps", "nrec", "src_kind", "src_ix", "src_iz",
                                                   "f0", "amplitude", "t_cut", "dx", "dz", "dt", "reserved0",
                                                   "prof_hash", "coef_hash", "rec_hash", "payload_bytes",
                                                   "checksum", "reserved"]),
}

CONSTANTS = ["POE_OK", "POE_EINVAL", "POE_ECFL", "POE_ENONFINITE", "POE_ETIMEOUT", "POE_ECUDA", "POE_ENOMEM",
             "POE_EIO", "POE_ESTATE", "POE_SRC_REF_DGAUSS_P", "POE_SRC_RICKER_FZ", "POE_REC_NONE", "POE_REC_VX",
             "POE_REC_VZ", "POE_REC_P", "POE_CTX_FAST_STENCIL", "POE_CTX_NO_PALETTE", "POE_NCOEF", "POE_NFIELDS",
             "POE_ORDER_ROWS", "POE_ORDER_COLUMNS", "POE_ORDER_TILE_MAJOR", "POE_ORDER_BALANCED",
             "POE_AUTOTUNE_CANDIDATES", "POE_CHECKPOINT_VERSION", "POE_SPAN_NEVER", "POE_SPAN_ALWAYS",
             "POE_SPAN_AUTO", "POE_SG_MAP", "POE_SG_MAP_CH", "POE_SG_SCALARS", "POE_SG_SAMPLES", "POE_SG_CHANNELS"]
CONSTANTS += ["POE_C_RHO", "POE_C_RHOF", "POE_C_RSM", "POE_C_EOK", "POE_C_LAMBDAC", "POE_C_MU", "POE_C_ALPHA",
              "POE_C_RBM"]
CONSTANTS += ["POE_MAX_MATERIALS", "POE_MROW", "POE_M_CO", "POE_M_C1", "POE_M_C2", "POE_M_RHOF_EOK", "POE_M_RCO",
              "POE_M_RC1"]
CONSTANTS += ["POE_F_" + f.upper() for f in ("vx", "vz", "wx", "wz", "sxx", "szz", "sxz", "p", "g11", "g22",
                                              "xi1", "xi2")]


@pytest.fixture(scope="module")
def header_facts(tmp_path_factory):
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    d = tmp_path_factory.mktemp("abi")
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "poe2d.h"', '#include "poe2d_surrogate.h"',
             "int main(void) {"]
    for s, (_, fields) in STRUCTS.items():
        lines.append('printf("sizeof %s %%zu\\n", sizeof(%s));' % (s, s))
        for f in fields:
            lines.append('printf("offset %s.%s %%zu\\n", offsetof(%s, %s));' % (s, f, s, f))
    for k in CONSTANTS:
        lines.append('printf("const %s %%ld\\n", (long)%s);' % (k, k))
    lines += ["return 0;", "}"]
    src = d / "probe.c"
    src.write_text("\n".join(lines) + "\n")
    exe = d / "probe"
    subprocess.run([cc, "-std=c11", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), str(src), "-o",
                    str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    facts = {}
    for ln in out.splitlines():
        kind, name, val = ln.split()
        facts[(kind, name)] = int(val)
    return facts


def test_structs_match_ctypes(header_facts):
    from poe2d_gb300 import _lib as L
    for s, (py, fields) in STRUCTS.items():
        cls = getattr(L, py)
        assert [f[0] for f in cls._fields_] == fields, s
        assert C.sizeof(cls) == header_facts[("sizeof", s)], s
        for f in fields:
            assert getattr(cls, f).offset == header_facts[("offset", "%s.%s" % (s, f))], (s, f)


def test_constants_match_python(header_facts):
    from poe2d_gb300 import _lib as L
    from poe2d_gb300 import surrogate as S
    c = {k[1]: v for k, v in header_facts.items() if k[0] == "const"}
    status = ["POE_OK", "POE_EINVAL", "POE_ECFL", "POE_ENONFINITE", "POE_ETIMEOUT", "POE_ECUDA", "POE_ENOMEM",
              "POE_EIO", "POE_ESTATE"]
    for k in status:
        assert getattr(L, k) == c[k], k
    assert L.SRC_REF_DGAUSS_P == c["POE_SRC_REF_DGAUSS_P"] and L.SRC_RICKER_FZ == c["POE_SRC_RICKER_FZ"]
    assert (L.REC_NONE, L.REC_VX, L.REC_VZ, L.REC_P) == (c["POE_REC_NONE"], c["POE_REC_VX"], c["POE_REC_VZ"],
                                                         c["POE_REC_P"])
    assert L.CTX_FAST_STENCIL == c["POE_CTX_FAST_STENCIL"] and L.CTX_NO_PALETTE == c["POE_CTX_NO_PALETTE"]
    # coefficient planes and readable fields, in the binding's order
    assert len(L.COEFS) == c["POE_NCOEF"]
    for i, n in enumerate(["RHO", "RHOF", "RSM", "EOK", "LAMBDAC", "MU", "ALPHA", "RBM"]):
        assert c["POE_C_" + n] == i and L.COEFS[i] == n.lower(), n
    assert len(L.FIELDS) == c["POE_NFIELDS"]
    for i, f in enumerate(L.FIELDS):
        assert c["POE_F_" + f.upper()] == i, f
    assert (L.MAX_MATERIALS, L.MROW) == (c["POE_MAX_MATERIALS"], c["POE_MROW"])
    assert (L.M_CO, L.M_C1, L.M_C2, L.M_RHOF_EOK, L.M_RCO, L.M_RC1) == tuple(
        c["POE_M_" + k] for k in ("CO", "C1", "C2", "RHOF_EOK", "RCO", "RC1"))
    # Solver.tune documents 0 rows, 1 columns, 2 tile-major, 3 balanced
    assert (L.ORDER_ROWS, L.ORDER_COLUMNS, L.ORDER_TILE_MAJOR, L.ORDER_BALANCED) == (
        c["POE_ORDER_ROWS"], c["POE_ORDER_COLUMNS"], c["POE_ORDER_TILE_MAJOR"], c["POE_ORDER_BALANCED"]) == (0, 1, 2, 3)
    assert L.AUTOTUNE_CANDIDATES == c["POE_AUTOTUNE_CANDIDATES"] == 2 * 4 * 2 * 2
    assert (L.SPAN_NEVER, L.SPAN_ALWAYS, L.SPAN_AUTO) == (
        c["POE_SPAN_NEVER"], c["POE_SPAN_ALWAYS"], c["POE_SPAN_AUTO"]) == (0, 1, 2)
    assert L.CHECKPOINT_VERSION == c["POE_CHECKPOINT_VERSION"]
    assert (S.MAP, S.MAP_CH, S.SCALARS, S.SAMPLES, S.CHANNELS) == (
        c["POE_SG_MAP"], c["POE_SG_MAP_CH"], c["POE_SG_SCALARS"], c["POE_SG_SAMPLES"], c["POE_SG_CHANNELS"])


def _prototypes():
    import re
    out = {}
    for h in ("poe2d.h", "poe2d_surrogate.h"):
        t = open(os.path.join(ROOT, "include", h)).read()
        t = re.sub(r"/\*.*?\*/", "", t, flags=re.S)
        t = re.sub(r"//[^\n]*", "", t)
        for m in re.finditer(r"([A-Za-z_][\w\s\*]*?)\b(poe_\w+)\s*\(([^;{]*?)\)\s*;", t):
            args = [" ".join(a.split()) for a in m.group(3).split(",")]
            out[m.group(2)] = (" ".join(m.group(1).split()), [] if args == ["void"] else args)
    return out


def _ctype_of(decl):
    """The ctypes type a C parameter declaration binds to; for a pointer,
    the pointer type (c_void_p is accepted for any pointer as well)."""
    from poe2d_gb300 import _lib as L
    import re
    t = re.sub(r"\b(const)\b", " ", decl)
    stars = t.count("*")
    base = t.replace("*", " ").split()[0]
    scalars = {"int": C.c_int, "int32_t": C.c_int32, "int64_t": C.c_int64, "uint32_t": C.c_uint32,
               "uint64_t": C.c_uint64, "uint8_t": C.c_uint8, "float": C.c_float, "double": C.c_double,
               "char": C.c_char}
    structs = {s: getattr(L, py) for s, (py, _) in STRUCTS.items()}
    opaque = {"poe_ctx", "poe_batch", "poe_sg", "void"}
    if stars == 0:
        return scalars[base]
    if base in opaque:
        return C.c_void_p if stars == 1 else C.POINTER(C.c_void_p)
    assert stars == 1, decl
    return C.POINTER(structs[base] if base in structs else scalars[base])


def test_symbols_match_prototypes():
    """Every declared function is bound, with its return type and one ctypes
    argument per parameter of the same width and signedness."""
    from poe2d_gb300 import _lib as L
    protos = _prototypes()
    assert len(protos) >= 40
    assert set(protos) == set(L.SYMBOLS), (set(protos) ^ set(L.SYMBOLS))
    rets = {"int": C.c_int, "int32_t": C.c_int32, "void": None, "const char *": C.c_char_p}
    for name, (ret, args) in protos.items():
        res, argtypes = L.SYMBOLS[name]
        assert res is rets[ret], (name, ret, res)
        assert len(argtypes) == len(args), (name, args)
        for decl, got in zip(args, argtypes):
            want = _ctype_of(decl)
            if "*" in decl and got is C.c_void_p:
                continue
            assert got is want or got == want, (name, decl, got, want)
