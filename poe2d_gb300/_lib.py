"""ctypes binding of ``libpoe2d.so`` (the C ABI in include/poe2d.h).

There is no fallback: if the library is missing it is built from
``poe2d_gb300/csrc`` with nvcc, and if that fails the import of any solver
entry point raises.  Set-up functions (profiles, coefficients, tables) run on
the host and need no GPU; contexts need a CUDA device.
"""
from __future__ import annotations

import ctypes as C
import os

from . import build as _build

POE_OK, POE_EINVAL, POE_ECFL, POE_ENONFINITE, POE_ETIMEOUT, POE_ECUDA, POE_ENOMEM, POE_EIO, POE_ESTATE = range(9)
SRC_REF_DGAUSS_P, SRC_RICKER_FZ = 0, 1
REC_NONE, REC_VX, REC_VZ, REC_P = -1, 0, 1, 2
CTX_FAST_STENCIL = 1
CTX_NO_PALETTE = 2
MAX_MATERIALS, MROW = 64, 14
ORDER_ROWS, ORDER_COLUMNS, ORDER_TILE_MAJOR, ORDER_BALANCED = range(4)
AUTOTUNE_CANDIDATES = 32
SPAN_NEVER, SPAN_ALWAYS, SPAN_AUTO = range(3)
M_CO, M_C1, M_C2, M_RHOF_EOK, M_RCO, M_RC1 = range(8, 14)
FIELDS = ["vx", "vz", "wx", "wz", "sxx", "szz", "sxz", "p", "g11", "g22", "xi1", "xi2"]
COEFS = ["rho", "rhof", "rsm", "eok", "lambdac", "mu", "alpha", "rbm"]


class Grid(C.Structure):
    _fields_ = [("NX", C.c_int32), ("NZ", C.c_int32), ("dx", C.c_float), ("dz", C.c_float), ("dt", C.c_float)]


class PmlParams(C.Structure):
    _fields_ = [("npoints", C.c_int32), ("rcoef", C.c_float), ("npower", C.c_float), ("k_max", C.c_float),
                ("alpha_max", C.c_float), ("alpha_top_extra", C.c_double), ("cp_max", C.c_float)]


class Source(C.Structure):
    _fields_ = [("ix", C.c_int32), ("iz", C.c_int32), ("kind", C.c_int32), ("f0", C.c_float),
                ("amplitude", C.c_float), ("t_cut", C.c_double)]


class Receiver(C.Structure):
    _fields_ = [("ix", C.c_int32), ("iz", C.c_int32), ("comp", C.c_int32)]


class BiotMaterial(C.Structure):
    _fields_ = [(n, C.c_float) for n in ("rho_s", "phi", "k_s", "k_frame", "mu_frame",
                                         "rho_f", "k_f", "eta", "kappa", "tortuosity")]


class CheckpointHeader(C.Structure):
    """poe_checkpoint_header: the first bytes of a checkpoint image."""
    _fields_ = [("magic", C.c_char * 8), ("version", C.c_uint32), ("header_bytes", C.c_uint32),
                ("NX", C.c_int32), ("NZ", C.c_int32), ("P", C.c_int32), ("R", C.c_int32), ("Wx", C.c_int32),
                ("Hz", C.c_int32), ("plane", C.c_int64), ("steps", C.c_int64), ("nrec", C.c_int32),
                ("src_kind", C.c_int32), ("src_ix", C.c_int32), ("src_iz", C.c_int32), ("f0", C.c_float),
                ("amplitude", C.c_float), ("t_cut", C.c_double), ("dx", C.c_float), ("dz", C.c_float),
                ("dt", C.c_float), ("reserved0", C.c_int32), ("prof_hash", C.c_uint64), ("coef_hash", C.c_uint64),
                ("rec_hash", C.c_uint64), ("payload_bytes", C.c_int64), ("checksum", C.c_uint64),
                ("reserved", C.c_uint64 * 2)]


CHECKPOINT_VERSION = 2


class PoeError(RuntimeError):
    def __init__(self, status, msg=""):
        self.status = status
        super().__init__("poe2d status %d (%s)%s" % (status, _status_name(status), (": " + msg) if msg else ""))


_NAMES = {0: "ok", 1: "EINVAL", 2: "ECFL", 3: "ENONFINITE", 4: "ETIMEOUT", 5: "ECUDA", 6: "ENOMEM", 7: "EIO",
          8: "ESTATE"}


def _status_name(s):
    return _NAMES.get(s, "?")


_fp = C.POINTER(C.c_float)
_lib = None

SYMBOLS = {
    "poe_pml_build": (C.c_int, [C.POINTER(Grid), C.POINTER(PmlParams), _fp, _fp]),
    "poe_pml_defaults": (None, [C.POINTER(PmlParams), C.c_int32, C.c_float, C.c_float]),
    "poe_coeffs_from_medium": (C.c_int, [C.POINTER(Grid), _fp, _fp, _fp, _fp, _fp, C.c_int32, _fp]),
    "poe_coeffs_biot": (C.c_int, [C.c_int64, C.POINTER(BiotMaterial), C.c_int32, C.POINTER(C.c_uint8), _fp, _fp]),
    "poe_material_palette": (C.c_int, [_fp, C.c_int64, C.c_float, C.POINTER(C.c_uint8), _fp,
                                       C.POINTER(C.c_int32)]),
    "poe_check_courant": (C.c_int, [C.POINTER(Grid), C.c_float]),
    "poe_source_table": (C.c_int, [C.POINTER(Grid), C.POINTER(Source), C.c_int64, _fp, C.POINTER(C.c_int64)]),
    "poe_create": (C.c_int, [C.POINTER(Grid), _fp, _fp, _fp, C.c_void_p, C.c_uint32, C.POINTER(C.c_void_p)]),
    "poe_add_shot": (C.c_int, [C.c_void_p, C.POINTER(Source), C.POINTER(Receiver), C.c_int32,
                               C.POINTER(C.c_int32)]),
    "poe_run": (C.c_int, [C.c_void_p, C.c_int64]),
    "poe_sync": (C.c_int, [C.c_void_p]),
    "poe_get_traces": (C.c_int, [C.c_void_p, C.c_int32, _fp, C.c_int64]),
    "poe_get_field": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, _fp]),
    "poe_set_field": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, _fp]),
    "poe_get_derived_noalloc": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, _fp]),
    "poe_wait_limit_check": (C.c_int, [C.c_int32, C.c_int32, C.POINTER(C.c_int32)]),
    "poe_checkpoint_size": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_int64)]),
    "poe_checkpoint_save": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_int64]),
    "poe_checkpoint_load": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_int64]),
    "poe_checkpoint_info": (C.c_int, [C.c_void_p, C.c_int64, C.POINTER(CheckpointHeader)]),
    "poe_tune": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32]),
    "poe_tune_span": (C.c_int, [C.c_void_p, C.c_int32]),
    "poe_tune_tile": (C.c_int, [C.c_void_p, C.c_int32]),
    "poe_tuning": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                             C.POINTER(C.c_int32)]),
    "poe_batch_tune_span": (C.c_int, [C.c_void_p, C.c_int32]),
    "poe_autotune": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_int32), C.POINTER(C.c_int32), _fp]),
    "poe_steps_done": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_int64)]),
    "poe_reset_shot": (C.c_int, [C.c_void_p, C.c_int32]),
    "poe_check_finite": (C.c_int, [C.c_void_p, C.c_int32, C.c_float, _fp]),
    "poe_kernel_launches": (C.c_int, [C.c_void_p, C.POINTER(C.c_int64)]),
    "poe_last_error": (C.c_char_p, [C.c_void_p]),
    "poe_status_string": (C.c_char_p, [C.c_int]),
    "poe_destroy": (None, [C.c_void_p]),
    "poe_batch_create": (C.c_int, [C.POINTER(C.c_void_p), C.c_int32, C.c_void_p, C.POINTER(C.c_void_p)]),
    "poe_batch_run": (C.c_int, [C.c_void_p, C.POINTER(C.c_int64)]),
    "poe_batch_sync": (C.c_int, [C.c_void_p]),
    "poe_batch_launches": (C.c_int, [C.c_void_p, C.POINTER(C.c_int64)]),
    "poe_batch_last_error": (C.c_char_p, [C.c_void_p]),
    "poe_batch_destroy": (None, [C.c_void_p]),
    "poe_sg_gemm": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_int32,
                              C.c_float, C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_int32, C.c_int32,
                              C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p]),
    "poe_sg_create": (C.c_int, [C.c_int32, C.c_uint64, C.c_void_p, C.POINTER(C.c_void_p)]),
    "poe_sg_param_count": (C.c_int, [C.c_void_p, C.POINTER(C.c_int64)]),
    "poe_sg_get_params": (C.c_int, [C.c_void_p, _fp, C.c_int64]),
    "poe_sg_set_params": (C.c_int, [C.c_void_p, _fp, C.c_int64]),
    "poe_sg_get_grads": (C.c_int, [C.c_void_p, _fp, C.c_int64]),
    "poe_sg_forward": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p]),
    "poe_sg_loss_grad": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.POINTER(C.c_float)]),
    "poe_sg_adam": (C.c_int, [C.c_void_p, C.c_float]),
    "poe_sg_get_state": (C.c_int, [C.c_void_p, _fp, _fp, _fp, C.c_int64, C.POINTER(C.c_int32)]),
    "poe_sg_train_step": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_float,
                                    C.POINTER(C.c_float)]),
    "poe_sg_launches": (C.c_int, [C.c_void_p, C.POINTER(C.c_int64)]),
    "poe_sg_gather_rows": (C.c_int, [C.c_void_p, C.c_int64, C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p]),
    "poe_sg_last_error": (C.c_char_p, [C.c_void_p]),
    "poe_sg_destroy": (None, [C.c_void_p]),
    "poe_ref_receivers": (C.c_int32, [C.POINTER(Grid), C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32,
                                      C.c_int32, C.POINTER(Receiver), C.c_int32]),
}


def lib_path():
    return _build.LIB


def lib():
    """Load libpoe2d.so, building it first if needed; raises if unavailable."""
    global _lib
    if _lib is None:
        path = _build.LIB
        if not os.path.exists(path):
            _build.build()
        L = C.CDLL(path)
        for name, (res, args) in SYMBOLS.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def check(status, ctx=None):
    if status != POE_OK:
        msg = ""
        if ctx:
            m = lib().poe_last_error(ctx)
            msg = m.decode() if m else ""
        raise PoeError(status, msg)
