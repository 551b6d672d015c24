"""Python face of the solver: set-up helpers and a context class over the C ABI.

The reference (thejatmik/poe2d) has no library interface; its operator is
``main()`` of seismic_CPML_2D_poroelastic_withCUDA.cu (cited cu:).  This
module exposes that program's stages under their own names so a caller can
drive them one by one: medium -> coefficients (cu:646-713), PML profiles
(cu:985-1159), Courant check (cu:1197-1212), the time loop (cu:1596-1736)
and its recordings (cu:114-201).  Every call goes through libpoe2d.so; the
GPU work is done by the sm_103a kernels and there is no CPU path.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L
from ._lib import BiotMaterial, Grid, PmlParams, PoeError, Receiver, Source, check

# The reference's fluid table, one row per medium ID 0..3:
# (K_f, eta, kappa, phi, tortuosity, rho_f)   (cu:565-568 and cu:574-575)
REFERENCE_FLUID_TABLE = np.array([
    [2.4e09, 0.003, 1.5e-17, 1.e-6, 2.0, 10.0],
    [2.4e09, 0.003, 500.0e-15, 1.e-6, 2.0, 10.0],
    [0.7e09, 0.03, 500.0e-15, 1.e-6, 2.0, 10.0],
    [0.02e09, 1.0e-5, 500.0e-15, 1.e-6, 2.0, 10.0],
], dtype=np.float32)

_fp = C.POINTER(C.c_float)


def _f(a):
    return a.ctypes.data_as(_fp)


def grid(NX, NZ, dx, dt, dz=None):
    """Grid of (NX+1) x (NZ+1) cells (cu:486-504); dz defaults to dx as in cu:495."""
    return Grid(int(NX), int(NZ), float(dx), float(dx if dz is None else dz), float(dt))


def pml_defaults(npoints, f0, cp_max):
    p = PmlParams()
    L.lib().poe_pml_defaults(C.byref(p), int(npoints), float(f0), float(cp_max))
    return p


def pml_profiles(g, npoints=None, f0=None, cp_max=None, params=None):
    """C-PML profiles (a, b, K at integer and half nodes), shapes (6, NX+1), (6, NZ+1)."""
    p = params if params is not None else pml_defaults(npoints, f0, cp_max)
    px = np.zeros((6, g.NX + 1), np.float32)
    pz = np.zeros((6, g.NZ + 1), np.float32)
    check(L.lib().poe_pml_build(C.byref(g), C.byref(p), _f(px), _f(pz)))
    return px, pz


def coeffs_from_medium(g, medium, cp, cs, rho_sat, table=REFERENCE_FLUID_TABLE):
    """8 coefficient planes from a medium-ID grid plus cp, cs, saturated density."""
    shape = (g.NZ + 1, g.NX + 1)
    arrs = [np.ascontiguousarray(np.asarray(a, np.float32).reshape(shape)) for a in (medium, cp, cs, rho_sat)]
    t = np.ascontiguousarray(table, np.float32)
    coef = np.zeros((8,) + shape, np.float32)
    check(L.lib().poe_coeffs_from_medium(C.byref(g), *[_f(a) for a in arrs], _f(t), t.shape[0], _f(coef)))
    return coef


def biot_material(rho_s, phi, k_s, k_frame, mu_frame, rho_f, k_f, eta, kappa, tortuosity):
    return BiotMaterial(rho_s, phi, k_s, k_frame, mu_frame, rho_f, k_f, eta, kappa, tortuosity)


def coeffs_biot(materials, ids):
    """8 coefficient planes from direct Biot materials indexed by ids; returns (coef, vp_fast_max)."""
    ids = np.ascontiguousarray(ids, np.uint8)
    mats = (BiotMaterial * len(materials))(*materials)
    coef = np.zeros((8,) + ids.shape, np.float32)
    vmax = C.c_float(0.0)
    check(L.lib().poe_coeffs_biot(ids.size, mats, len(materials), ids.ctypes.data_as(C.POINTER(C.c_uint8)),
                                  _f(coef), C.byref(vmax)))
    return coef, float(vmax.value)


def material_palette(coef, dt):
    """The palette a Solver builds for coef (8 planes) and time step dt:
    (ids of the cells' shape, rows of 14 floats per material: the 8
    coefficients, co, c1, c2, rho_f eta/kappa, 1/co, 1/c1), or None when the
    model runs on its 8 coefficient planes instead."""
    coef = np.ascontiguousarray(coef, np.float32)
    ncell = coef[0].size
    ids = np.zeros(coef.shape[1:], np.uint8)
    rows = np.zeros((L.MAX_MATERIALS, L.MROW), np.float32)
    n = C.c_int32(0)
    check(L.lib().poe_material_palette(_f(coef), ncell, float(dt), ids.ctypes.data_as(C.POINTER(C.c_uint8)),
                                       _f(rows), C.byref(n)))
    return (ids, rows[:n.value].copy()) if n.value else None


def check_courant(g, cp_max):
    """Raises PoeError(POE_ECFL) if the reference's Courant tests fail (cu:1197-1212)."""
    check(L.lib().poe_check_courant(C.byref(g), float(cp_max)))


def source(ix, iz, kind=L.SRC_REF_DGAUSS_P, f0=200.0, amplitude=1.0, t_cut=0.4):
    return Source(int(ix), int(iz), int(kind), float(f0), float(amplitude), float(t_cut))


def source_table(g, src, nsteps):
    tab = np.zeros(max(int(nsteps), 1), np.float32)
    n = C.c_int64(0)
    check(L.lib().poe_source_table(C.byref(g), C.byref(src), int(nsteps), _f(tab), C.byref(n)))
    return tab[:n.value].copy()


def receivers(rec):
    """(n, 3) array-like of (ix, iz, comp) -> ctypes array."""
    r = np.asarray(rec, np.int32).reshape(-1, 3)
    arr = (Receiver * max(len(r), 1))()
    for i, (ix, iz, c) in enumerate(r):
        arr[i] = Receiver(int(ix), int(iz), int(c))
    return arr, len(r)


def ref_receivers(g, isource, jsource, panj, panj2, a0_pos, a1_pos):
    """The save1_kernel geometry (cu:114-201) as an (n, 3) array of (ix, iz, comp)."""
    cap = 2 * panj + 2 * panj2 + 4
    arr = (Receiver * cap)()
    n = L.lib().poe_ref_receivers(C.byref(g), isource, jsource, panj, panj2, a0_pos, a1_pos, arr, cap)
    if n < 0:
        raise PoeError(L.POE_EINVAL, "ref_receivers")
    return np.array([(arr[i].ix, arr[i].iz, arr[i].comp) for i in range(n)], np.int32)


def checkpoint_info(image):
    """Header of a checkpoint image as a dict, checked on the host (no GPU):
    PoeError(EINVAL) for a buffer that is not a version-2 image or is shorter
    than its payload, PoeError(EIO) for a payload checksum mismatch."""
    buf = np.frombuffer(image, np.uint8)
    h = L.CheckpointHeader()
    check(L.lib().poe_checkpoint_info(buf.ctypes.data_as(C.c_void_p), buf.size, C.byref(h)))
    out = {name: getattr(h, name) for name, _ in L.CheckpointHeader._fields_ if not name.startswith("reserved")}
    out["magic"] = bytes(h.magic)
    return out


def wait_limit_check(polls=1000, device=0):
    """Run the step kernel's bounded waits against a barrier nothing arrives at
    and a tile flag nothing sets, and the flag wait against set flags
    (poe_wait_limit_check): True when the first two gave up at their limit and
    the third passed."""
    out = C.c_int32(0)
    check(L.lib().poe_wait_limit_check(int(device), int(polls), C.byref(out)))
    return out.value == 1


class Solver:
    """One model on the current CUDA device, with any number of shots.

    coef: (8, NZ+1, NX+1) float32; prof_x / prof_z from pml_profiles().
    stream: an integer cudaStream_t handle (e.g. torch.cuda.current_stream().cuda_stream)
    or None for a private stream.  fast=True selects plain FP32 stencils;
    palette=False keeps the 8 coefficient planes even for few-material models.
    """

    def __init__(self, g, coef, prof_x, prof_z, stream=None, fast=False, palette=True):
        self.g = g
        self.shape = (g.NZ + 1, g.NX + 1)
        coef = np.ascontiguousarray(coef, np.float32)
        px = np.ascontiguousarray(prof_x, np.float32)
        pz = np.ascontiguousarray(prof_z, np.float32)
        if coef.size != 8 * self.shape[0] * self.shape[1] or px.size != 6 * (g.NX + 1) or pz.size != 6 * (g.NZ + 1):
            raise PoeError(L.POE_EINVAL, "array sizes do not match the grid")
        h = C.c_void_p()
        check(L.lib().poe_create(C.byref(g), _f(coef), _f(px), _f(pz), C.c_void_p(stream or 0),
                                 (L.CTX_FAST_STENCIL if fast else 0) | (0 if palette else L.CTX_NO_PALETTE),
                                 C.byref(h)))
        self.h = h
        self.nrec = []

    def close(self):
        if getattr(self, "h", None):
            L.lib().poe_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, st):
        check(st, self.h)

    def add_shot(self, src=None, rec=()):
        arr, n = receivers(rec) if len(rec) else (None, 0)
        sid = C.c_int32(-1)
        self._check(L.lib().poe_add_shot(self.h, C.byref(src) if src is not None else None, arr, n, C.byref(sid)))
        self.nrec.append(n)
        return sid.value

    def run(self, nsteps):
        self._check(L.lib().poe_run(self.h, int(nsteps)))

    def sync(self):
        self._check(L.lib().poe_sync(self.h))

    def steps(self, shot=0):
        s = C.c_int64(0)
        self._check(L.lib().poe_steps_done(self.h, shot, C.byref(s)))
        return s.value

    def traces(self, shot=0):
        n = self.steps(shot)
        out = np.zeros((n, self.nrec[shot]), np.float32)
        if out.size:
            self._check(L.lib().poe_get_traces(self.h, shot, _f(out), out.size))
        return out

    def field(self, name, shot=0):
        fid = L.FIELDS.index(name) if isinstance(name, str) else int(name)
        out = np.empty(self.shape, np.float32)
        self._check(L.lib().poe_get_field(self.h, shot, fid, _f(out)))
        return out

    def derived_noalloc(self, name, shot=0):
        """sigma_xx, sigma_zz or p without any device allocation (static scratch plane)."""
        fid = L.FIELDS.index(name) if isinstance(name, str) else int(name)
        out = np.empty(self.shape, np.float32)
        self._check(L.lib().poe_get_derived_noalloc(self.h, shot, fid, _f(out)))
        return out

    def set_field(self, name, values, shot=0):
        fid = L.FIELDS.index(name) if isinstance(name, str) else int(name)
        a = np.ascontiguousarray(np.asarray(values, np.float32).reshape(self.shape))
        self._check(L.lib().poe_set_field(self.h, shot, fid, _f(a)))

    def tune(self, order=3, graph_steps=64):
        """Work-list order (0 rows, 1 columns, 2 tile-major across shots, 3 rows
        dealt for an even share of edge tiles per CTA) and graph length."""
        self._check(L.lib().poe_tune(self.h, int(order), int(graph_steps)))

    def tune_span(self, span=L.SPAN_AUTO):
        """1 (SPAN_ALWAYS): one step-spanning launch per captured graph (tiles of a
        step start as soon as their neighbourhood finished the previous one); 0
        (SPAN_NEVER): a launch per step; 2 (SPAN_AUTO, the default): spanning when
        a step holds at most 96 tiles per SM."""
        self._check(L.lib().poe_tune_span(self.h, int(span)))

    def tune_tile(self, tile_z):
        """The step kernel's tile height: 32 (default) or 16 (FAST stencils, outside a batch)."""
        self._check(L.lib().poe_tune_tile(self.h, int(tile_z)))

    def tuning(self):
        """The current tuning: dict(order, graph_steps, span, tile_z)."""
        v = [C.c_int32(0) for _ in range(4)]
        self._check(L.lib().poe_tuning(self.h, *[C.byref(x) for x in v]))
        return dict(zip(("order", "graph_steps", "span", "tile_z"), (x.value for x in v)))

    def autotune(self, trial_steps=128):
        """Time the 32 (tile height, order, graph_steps, span) candidates, keep the fastest;
        shots must be at step 0 and are reset after.  Returns (order, graph_steps, ms per
        candidate), candidate c = tile height (32, 16)[c // 16], order (c // 4) % 4,
        graph_steps (16, 64)[(c // 2) % 2], span c % 2 (ms -1: not a candidate for this
        context); tuning() reports the winner's tile height."""
        o, g = C.c_int32(0), C.c_int32(0)
        ms = np.zeros(L.AUTOTUNE_CANDIDATES, np.float32)
        self._check(L.lib().poe_autotune(self.h, int(trial_steps), C.byref(o), C.byref(g), _f(ms)))
        return o.value, g.value, ms

    def checkpoint(self, shot=0):
        """Full state of a shot as bytes (fields, C-PML memory, traces, clock)."""
        n = C.c_int64(0)
        self._check(L.lib().poe_checkpoint_size(self.h, shot, C.byref(n)))
        buf = np.empty(n.value, np.uint8)
        self._check(L.lib().poe_checkpoint_save(self.h, shot, buf.ctypes.data_as(C.c_void_p), n.value))
        return buf.tobytes()

    def restore(self, image, shot=0):
        """Load a checkpoint() image into a shot with the same definition."""
        buf = np.frombuffer(image, np.uint8)
        self._check(L.lib().poe_checkpoint_load(self.h, shot, buf.ctypes.data_as(C.c_void_p), buf.size))

    def reset_shot(self, shot=0):
        self._check(L.lib().poe_reset_shot(self.h, shot))

    def check_finite(self, shot=0, threshold=1e25):
        v = C.c_float(0.0)
        st = L.lib().poe_check_finite(self.h, shot, float(threshold), C.byref(v))
        return st, float(v.value)

    @property
    def launches(self):
        n = C.c_int64(0)
        self._check(L.lib().poe_kernel_launches(self.h, C.byref(n)))
        return n.value


class Batch:
    """Several Solvers advanced together, one persistent launch per time step.

    Every solver must use the same stencil mode, and either all use the
    material palette (the default for patchy models) or none does.
    run(steps) takes one step count per solver (or one for all); each
    solver's shots end exactly as after solver.run(steps[i]).  The solvers
    must stay open while the batch is used: run() and sync() refuse a batch
    one of whose solvers has been closed.
    """

    def __init__(self, solvers, stream=None):
        self.solvers = list(solvers)
        arr = (C.c_void_p * len(self.solvers))(*[s.h.value for s in self.solvers])
        h = C.c_void_p()
        st = L.lib().poe_batch_create(arr, len(self.solvers), C.c_void_p(stream or 0), C.byref(h))
        if st != L.POE_OK:
            msg = ""
            for s in self.solvers:
                m = L.lib().poe_last_error(s.h)
                if m:
                    msg = m.decode()
            raise PoeError(st, msg)
        self.h = h

    def _check(self, st):
        if st != L.POE_OK:
            m = L.lib().poe_batch_last_error(self.h)
            raise PoeError(st, m.decode() if m else "")

    def _live(self):
        if not getattr(self, "h", None):
            raise PoeError(L.POE_ESTATE, "batch is closed")
        if any(not s.h for s in self.solvers):
            raise PoeError(L.POE_ESTATE, "a solver of this batch has been closed")

    def run(self, steps):
        self._live()
        if np.isscalar(steps):
            steps = [int(steps)] * len(self.solvers)
        if len(steps) != len(self.solvers):
            raise PoeError(L.POE_EINVAL, "one step count per solver")
        arr = (C.c_int64 * len(steps))(*[int(v) for v in steps])
        self._check(L.lib().poe_batch_run(self.h, arr))

    def sync(self):
        self._live()
        self._check(L.lib().poe_batch_sync(self.h))

    def tune_span(self, span=L.SPAN_AUTO):
        """Step-spanning launches for the batch (see Solver.tune_span; AUTO decides
        per run segment, by the tiles of the models still stepping)."""
        self._live()
        self._check(L.lib().poe_batch_tune_span(self.h, int(span)))

    @property
    def launches(self):
        n = C.c_int64(0)
        self._check(L.lib().poe_batch_launches(self.h, C.byref(n)))
        return n.value

    def close(self):
        if getattr(self, "h", None):
            L.lib().poe_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()
