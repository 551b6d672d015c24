"""ctypes front end of the CPU oracle (test infrastructure only).

Loads ``oracle/_build/libpoe2d_oracle.so`` (the plain-C restatement in
``poe2d_oracle.c``) and, when it was built in a tree that has the reference
sources, ``oracle/_ref/libpoe2d_ref.so`` (the reference's own kernels and
set-up lines compiled for the host, see ``build_ref.sh``).

Only tests, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline and
reference legs use this module.  The product package never imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libpoe2d_oracle.so")
REF_PATH = os.path.join(HERE, "_ref", "libpoe2d_ref.so")

REFMIXED, F32, F64 = 0, 1, 2
SRC_P, SRC_FZ = 0, 1

FIELDS = ["vx", "vz", "wx", "wz", "sxx", "szz", "sxz", "p", "g11", "g22", "xi1", "xi2",
          "m_dx_sxx", "m_dz_sxx", "m_dx_s2", "m_dz_s2", "m_dx_sxz", "m_dz_sxz",
          "m_dx_vx1", "m_dx_vx2", "m_dz_vx", "m_dx_vz", "m_dz_vz1", "m_dz_vz2"]
FIELD_ID = {n: i for i, n in enumerate(FIELDS)}

_fp = C.POINTER(C.c_float)
_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)


def _f(a):
    return a.ctypes.data_as(_fp)


def build(quiet=True):
    """Compile the oracle with the Makefile beside this file."""
    out = subprocess.run(["make", "-C", HERE], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    if not quiet:
        print(out.stdout)


_lib = None
_ref = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        L.orc_pml_profiles.argtypes = [C.c_int, C.c_int, C.c_float, C.c_float, C.c_float, C.c_int,
                                       C.c_float, C.c_float, C.c_float, C.c_float, C.c_double,
                                       C.c_float, _fp, _fp]
        L.orc_pml_profiles.restype = None
        L.orc_coeffs_from_medium.argtypes = [C.c_int64, _fp, _fp, _fp, _fp, _fp, C.c_int, _fp]
        L.orc_coeffs_from_medium.restype = C.c_int
        L.orc_source_table.argtypes = [C.c_int, C.c_float, C.c_float, C.c_double, C.c_float,
                                       C.c_float, C.c_float, C.c_int64, _fp]
        L.orc_source_table.restype = C.c_int64
        L.orc_new.argtypes = [C.c_int, C.c_int, C.c_int, C.c_float, C.c_float, C.c_float, _fp, _fp, _fp]
        L.orc_new.restype = C.c_void_p
        L.orc_free.argtypes = [C.c_void_p]
        L.orc_set_source.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, _fp, C.c_int64]
        L.orc_set_receivers.argtypes = [C.c_void_p, C.c_int, _ip]
        L.orc_set_threads.argtypes = [C.c_void_p, C.c_int]
        L.orc_run.argtypes = [C.c_void_p, C.c_int64, _fp]
        L.orc_run.restype = C.c_int64
        L.orc_get_field.argtypes = [C.c_void_p, C.c_int, _fp]
        L.orc_get_field64.argtypes = [C.c_void_p, C.c_int, _dp]
        L.orc_set_field.argtypes = [C.c_void_p, C.c_int, _fp]
        L.orc_steps_done.argtypes = [C.c_void_p]
        L.orc_steps_done.restype = C.c_int64
        _lib = L
    return _lib


def ref_available():
    return os.path.exists(REF_PATH)


def ref():
    """The reference's own code compiled for the host (only where it was built)."""
    global _ref
    if _ref is None:
        R = C.CDLL(REF_PATH)
        R.refh_pml.argtypes = [C.c_int, C.c_int, C.c_float, C.c_float, C.c_float, C.c_int,
                               C.c_float, C.c_float, _fp, _fp]
        R.refh_pml.restype = C.c_int
        R.refh_coeffs.argtypes = [C.c_int, C.c_int, _fp, _fp, _fp, _fp, _fp]
        R.refh_coeffs.restype = None
        R.refh_run.argtypes = [C.c_int, C.c_int, C.c_float, C.c_float, C.c_int, C.c_int, C.c_float,
                               _fp, _fp, _fp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _fp, _fp]
        R.refh_run.restype = C.c_int
        _ref = R
    return _ref


# --------------------------------------------------------------------------- set-up
def pml_profiles(NX, NZ, dx, dz, dt, npoints, cp_max, f0=None, rcoef=1e-3, npower=2.0,
                 k_max=1.0, alpha_max=None, alpha_top_extra=0.10):
    """C-PML profiles (cu:985-1159); alpha_max defaults to 2*PI*(f0/2) (cu:845)."""
    if alpha_max is None:
        alpha_max = float(np.float32(2.0 * float(np.float32(3.1415926535897932)) * (float(np.float32(f0)) / 2.0)))
    px = np.zeros((6, NX + 1), np.float32)
    pz = np.zeros((6, NZ + 1), np.float32)
    lib().orc_pml_profiles(NX, NZ, dx, dz, dt, npoints, rcoef, npower, k_max, alpha_max,
                           alpha_top_extra, cp_max, _f(px), _f(pz))
    return px, pz


def coeffs_from_medium(medium, cp, cs, rho_sat, table):
    n = medium.size
    coef = np.zeros((8,) + medium.shape, np.float32)
    t = np.ascontiguousarray(table, np.float32)
    bad = lib().orc_coeffs_from_medium(n, _f(np.ascontiguousarray(medium, np.float32)),
                                       _f(np.ascontiguousarray(cp, np.float32)),
                                       _f(np.ascontiguousarray(cs, np.float32)),
                                       _f(np.ascontiguousarray(rho_sat, np.float32)),
                                       _f(t), t.shape[0], _f(coef))
    return coef, bad


def coeffs_biot(materials, ids):
    """The 8 coefficient planes from direct Biot parameters, one material per
    id, and the largest fast-P velocity of the high-frequency Biot dispersion
    relation.  This parameterisation has no reference counterpart (the
    reference derives its coefficients from cp, cs and rho, cu:682-713, with
    K_s = K_b / (1 - phi)); it restates cu:697-708 with K_b = K_frame and K_s
    given, in float64 from the float32 parameters, each plane rounded to
    float32 once.  materials: dicts with rho_s phi k_s k_frame mu_frame rho_f
    k_f eta kappa tortuosity."""
    f32 = np.float32
    tab = np.zeros((len(materials), 8), np.float32)
    vmax = 0.0
    for i, q in enumerate(materials):
        q = {k: float(f32(v)) for k, v in q.items()}
        phi, ks, kb, mu, kf, rf = q["phi"], q["k_s"], q["k_frame"], q["mu_frame"], q["k_f"], q["rho_f"]
        rho = (1.0 - phi) * q["rho_s"] + phi * rf
        m = q["tortuosity"] * rf / phi
        eok = 0.0 if (q["eta"] == 0.0 or q["kappa"] == 0.0) else q["eta"] / q["kappa"]
        alpha = 1.0 - kb / ks
        M = 1.0 / (phi / kf + (alpha - phi) / ks)
        lc = kb - 2.0 / 3.0 * mu + alpha * alpha * M
        tab[i] = [rho, rf, m, eok, lc, mu, alpha, M]
        H, Cc = lc + 2.0 * mu, alpha * M
        A2, B2, C2 = rho * m - rf * rf, H * m + rho * M - 2.0 * Cc * rf, H * M - Cc * Cc
        v2 = (B2 + np.sqrt(max(B2 * B2 - 4.0 * A2 * C2, 0.0))) / (2.0 * A2)
        if v2 > 0.0:
            vmax = max(vmax, float(np.sqrt(v2)))
    ids = np.asarray(ids, np.uint8)
    return np.ascontiguousarray(np.moveaxis(tab[ids], -1, 0)), float(f32(vmax))


def source_table(kind, f0, dt, nsteps, amplitude=1.0, t_cut=0.4, dx=1.0, dz=1.0):
    tab = np.zeros(max(nsteps, 1), np.float32)
    n = lib().orc_source_table(kind, f0, amplitude, t_cut, dt, dx, dz, nsteps, _f(tab))
    return tab[:n].copy()


# --------------------------------------------------------------------------- loop
class Oracle:
    """One shot of the reference time loop on the CPU."""

    def __init__(self, mode, NX, NZ, dx, dz, dt, coef, prof_x, prof_z, threads=None):
        self.NX, self.NZ = NX, NZ
        self._coef = np.ascontiguousarray(coef, np.float32)
        self._px = np.ascontiguousarray(prof_x, np.float32)
        self._pz = np.ascontiguousarray(prof_z, np.float32)
        self.h = lib().orc_new(mode, NX, NZ, dx, dz, dt, _f(self._coef), _f(self._px), _f(self._pz))
        self.nrec = 0
        lib().orc_set_threads(self.h, threads or (os.cpu_count() or 1))

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_free(self.h)
            self.h = None

    def set_source(self, ix, iz, where, table):
        t = np.ascontiguousarray(table, np.float32)
        lib().orc_set_source(self.h, ix, iz, where, _f(t), t.size)

    def set_receivers(self, rec):
        r = np.ascontiguousarray(rec, np.int32).reshape(-1, 3)
        self.nrec = r.shape[0]
        lib().orc_set_receivers(self.h, self.nrec, r.ctypes.data_as(_ip))

    def set_threads(self, n):
        lib().orc_set_threads(self.h, n)

    def run(self, nsteps):
        tr = np.zeros((nsteps, max(self.nrec, 1)), np.float32)
        lib().orc_run(self.h, nsteps, _f(tr))
        return tr[:, :self.nrec]

    def field(self, name):
        out = np.empty((self.NZ + 1, self.NX + 1), np.float32)
        lib().orc_get_field(self.h, FIELD_ID.get(name, name), _f(out))
        return out

    def field64(self, name):
        out = np.empty((self.NZ + 1, self.NX + 1), np.float64)
        lib().orc_get_field64(self.h, FIELD_ID.get(name, name), out.ctypes.data_as(_dp))
        return out

    def set_field(self, name, arr):
        a = np.ascontiguousarray(arr, np.float32)
        lib().orc_set_field(self.h, FIELD_ID.get(name, name), _f(a))

    @property
    def steps(self):
        return lib().orc_steps_done(self.h)


# --------------------------------------------------------------------------- reference harness
def ref_pml(NX, NZ, dx, dz, dt, npoints, f0, cp_max):
    px = np.zeros((6, NX + 1), np.float32)
    pz = np.zeros((6, NZ + 1), np.float32)
    rc = ref().refh_pml(NX, NZ, dx, dz, dt, npoints, f0, cp_max, _f(px), _f(pz))
    return px, pz, rc


def ref_coeffs(medium, cp, cs, rho_sat):
    NZ1, NX1 = medium.shape
    coef = np.zeros((8, NZ1, NX1), np.float32)
    ref().refh_coeffs(NX1 - 1, NZ1 - 1, _f(np.ascontiguousarray(medium, np.float32)),
                      _f(np.ascontiguousarray(cp, np.float32)), _f(np.ascontiguousarray(cs, np.float32)),
                      _f(np.ascontiguousarray(rho_sat, np.float32)), _f(coef))
    return coef


def ref_run(NX, NZ, dx, dt, isrc, jsrc, f0, coef, prof_x, prof_z, nsteps, panj, panj2, a0, a1):
    """Run the reference kernels in the reference's launch order for nsteps."""
    n = (NX + 1) * (NZ + 1)
    fields = np.zeros((24, NZ + 1, NX + 1), np.float32)
    seis = np.zeros(2 * panj * nsteps + 2 * panj2 * nsteps + 4 * nsteps, np.float32)
    ig = ref().refh_run(NX, NZ, dx, dt, isrc, jsrc, f0,
                        _f(np.ascontiguousarray(coef, np.float32)),
                        _f(np.ascontiguousarray(prof_x, np.float32)),
                        _f(np.ascontiguousarray(prof_z, np.float32)),
                        nsteps, panj, panj2, a0, a1, _f(fields), _f(seis))
    o = 0
    out = {}
    for name, cnt in (("seismo", panj), ("deismo", panj), ("seismo1", panj2), ("deismo1", panj2),
                      ("seismo0", 1), ("seismo2", 1), ("seismo3", 1), ("seismo4", 1)):
        out[name] = seis[o:o + cnt * nsteps].reshape(nsteps, cnt)
        o += cnt * nsteps
    del n
    return {FIELDS[k]: fields[k] for k in range(24)}, out, ig
