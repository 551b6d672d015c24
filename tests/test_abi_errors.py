"""C ABI error behaviour that needs no GPU: every entry point answers a null
handle or an invalid argument with a status code (POE_EINVAL, or POE_ESTATE
where the call is out of order), never with a crash or an exit, and the
error-text calls accept null handles.  The reference exits through
HANDLE_ERROR instead (cu:1203, 1212)."""
import ctypes as C

import numpy as np
import pytest

EINVAL = 1


@pytest.fixture(scope="module")
def L(poe):
    return poe.lib()


def _fp(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def test_context_calls_reject_null_handles(L, poe):
    buf = np.zeros(16, np.float32)
    i32, i64, f32 = C.c_int32(0), C.c_int64(0), C.c_float(0)
    calls = [
        lambda: L.poe_add_shot(None, None, None, 0, C.byref(i32)),
        lambda: L.poe_run(None, 10),
        lambda: L.poe_sync(None),
        lambda: L.poe_get_traces(None, 0, _fp(buf), buf.size),
        lambda: L.poe_get_field(None, 0, 0, _fp(buf)),
        lambda: L.poe_set_field(None, 0, 0, _fp(buf)),
        lambda: L.poe_get_derived_noalloc(None, 0, 4, _fp(buf)),
        lambda: L.poe_checkpoint_size(None, 0, C.byref(i64)),
        lambda: L.poe_checkpoint_save(None, 0, buf.ctypes.data_as(C.c_void_p), buf.nbytes),
        lambda: L.poe_checkpoint_load(None, 0, buf.ctypes.data_as(C.c_void_p), buf.nbytes),
        lambda: L.poe_tune(None, 0, 64),
        lambda: L.poe_autotune(None, 32, None, None, None),
        lambda: L.poe_steps_done(None, 0, C.byref(i64)),
        lambda: L.poe_reset_shot(None, 0),
        lambda: L.poe_check_finite(None, 0, 1e25, C.byref(f32)),
        lambda: L.poe_kernel_launches(None, C.byref(i64)),
        lambda: L.poe_batch_run(None, (C.c_int64 * 1)(5)),
        lambda: L.poe_batch_sync(None),
        lambda: L.poe_batch_launches(None, C.byref(i64)),
        lambda: L.poe_sg_param_count(None, C.byref(i64)),
        lambda: L.poe_sg_get_params(None, _fp(buf), buf.size),
        lambda: L.poe_sg_set_params(None, _fp(buf), buf.size),
        lambda: L.poe_sg_get_grads(None, _fp(buf), buf.size),
        lambda: L.poe_sg_forward(None, None, None, 1, None),
        lambda: L.poe_sg_loss_grad(None, None, None, None, 8, None),
        lambda: L.poe_sg_adam(None, 1e-3),
        lambda: L.poe_sg_train_step(None, None, None, None, 8, 1e-3, None),
        lambda: L.poe_sg_launches(None, C.byref(i64)),
        lambda: L.poe_sg_gemm(None, 0, None, 0, 1, 1, 1, 1.0, None, 0, None, None, 0, 0, None, 0, None, None),
    ]
    for k, call in enumerate(calls):
        assert call() == EINVAL, k
    # error text and destruction accept null handles
    assert L.poe_last_error(None) == b"null context"
    assert L.poe_batch_last_error(None) == b"null batch"
    assert L.poe_sg_last_error(None) == b"null network"
    L.poe_destroy(None)
    L.poe_batch_destroy(None)
    L.poe_sg_destroy(None)


def test_create_rejects_bad_grids_before_touching_a_device(L, poe):
    n = 9
    coef = np.zeros((8, n, n), np.float32)
    px = np.zeros((6, n), np.float32)
    out = C.c_void_p(1234)
    good = dict(NX=n - 1, NZ=n - 1, dx=0.5, dz=0.5, dt=5e-5)
    for bad in (dict(NX=3), dict(NZ=2), dict(dx=0.0), dict(dz=-1.0), dict(dt=float("nan")), dict(dt=0.0)):
        g = poe.solver.Grid(**{**good, **bad})
        assert L.poe_create(C.byref(g), _fp(coef), _fp(px), _fp(px), None, 0, C.byref(out)) == EINVAL, bad
        assert out.value is None                  # *out is cleared on failure
        out = C.c_void_p(1234)
    g = poe.solver.Grid(**good)
    assert L.poe_create(C.byref(g), None, _fp(px), _fp(px), None, 0, C.byref(out)) == EINVAL
    assert L.poe_create(C.byref(g), _fp(coef), _fp(px), _fp(px), None, 0, None) == EINVAL


def test_batch_and_device_checks_reject_bad_arguments(L):
    out = C.c_void_p(0)
    ctxs = (C.c_void_p * 2)(None, None)
    assert L.poe_batch_create(None, 1, None, C.byref(out)) == EINVAL
    assert L.poe_batch_create(ctxs, 0, None, C.byref(out)) == EINVAL
    assert L.poe_batch_create(ctxs, 2, None, C.byref(out)) == EINVAL      # null contexts
    assert L.poe_batch_create(ctxs, 2, None, None) == EINVAL
    gave = C.c_int32(0)
    assert L.poe_wait_limit_check(0, 0, C.byref(gave)) == EINVAL         # polls < 1
    assert L.poe_wait_limit_check(0, 1 << 25, C.byref(gave)) == EINVAL   # above the limit
    assert L.poe_wait_limit_check(0, 100, None) == EINVAL
    assert L.poe_sg_create(0, 1, None, C.byref(out)) == EINVAL           # max_batch < 1


def test_setup_calls_reject_bad_arguments(L, poe):
    g = poe.grid(40, 30, 0.5, 5e-5)
    px = np.zeros((6, 41), np.float32)
    pz = np.zeros((6, 31), np.float32)
    par = poe.pml_defaults(10, 200.0, 3000.0)
    assert L.poe_pml_build(None, C.byref(par), _fp(px), _fp(pz)) == EINVAL
    assert L.poe_pml_build(C.byref(g), None, _fp(px), _fp(pz)) == EINVAL
    tab = np.zeros(16, np.float32)
    nact = C.c_int64(0)
    src = poe.source(5, 5)
    assert L.poe_source_table(None, C.byref(src), 16, _fp(tab), C.byref(nact)) == EINVAL
    assert L.poe_source_table(C.byref(g), None, 16, _fp(tab), C.byref(nact)) == EINVAL
    ids = np.zeros(4, np.uint8)
    nm = C.c_int32(0)
    assert L.poe_material_palette(None, 4, 5e-5, ids.ctypes.data_as(C.POINTER(C.c_uint8)), _fp(tab),
                                  C.byref(nm)) == EINVAL
    for code in range(9):
        assert L.poe_status_string(code)
