"""Host-side behaviour of the Python binding that needs no GPU."""
import ctypes as C

import pytest


def test_batch_refuses_closed_solvers_and_closed_batches(poe):
    """A batch keeps raw context pointers: once one of its solvers is closed
    (its context destroyed), run() and sync() must raise instead of handing
    the library a freed context."""
    from poe2d_gb300.solver import Batch

    class Closed:
        h = None

    b = Batch.__new__(Batch)          # the state Batch.__init__ leaves, without a device
    b.solvers = [Closed()]
    b.h = C.c_void_p(1)               # never passed to the library: the guard raises first
    try:
        for call in (lambda: b.run(5), b.sync):
            with pytest.raises(poe.PoeError) as e:
                call()
            assert e.value.status == 8 and "solver" in str(e.value)
    finally:
        b.h = None                    # Batch.__del__ must not destroy the fake handle
    for call in (lambda: b.run(5), b.sync):
        with pytest.raises(poe.PoeError) as e:
            call()
        assert "batch is closed" in str(e.value)
