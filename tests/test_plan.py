"""The work-list planner of the persistent step kernel (poe2d_plan.h), built
for the host: the balanced order is a permutation of the tiles, keeps edge
and interior tiles each in their order, and gives the busiest CTA no more
work than the water-filling optimum (tile 1, edge tile 2), never more than
rows order does.  The CTA of position p is p mod slots, as in the kernel."""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def plan(tmp_path_factory):
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("no g++")
    out = str(tmp_path_factory.mktemp("plan") / "libplan.so")
    subprocess.run([cxx, "-O2", "-std=c++17", "-fPIC", "-shared", "-I", os.path.join(ROOT, "poe2d_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "plan_harness.cpp"), "-o", out], check=True)
    lib = C.CDLL(out)
    lib.balanced_order_c.argtypes = [C.POINTER(C.c_uint8), C.c_int, C.c_int, C.POINTER(C.c_int)]

    def run(edge, slots):
        e = np.ascontiguousarray(edge, np.uint8)
        o = np.zeros(max(e.size, 1), np.int32)
        n = lib.balanced_order_c(e.ctypes.data_as(C.POINTER(C.c_uint8)), e.size, slots,
                                 o.ctypes.data_as(C.POINTER(C.c_int)))
        return o[:n]
    return run


def busiest(edge, order, slots):
    s = max(1, min(slots, len(edge)))
    w = 1 + np.asarray(edge, np.int64)[order]
    return int(np.bincount(np.arange(len(order)) % s, weights=w, minlength=s).max()) if len(order) else 0


def optimum(edge, slots):
    """Smallest busiest-CTA work any assignment of these counts allows."""
    n, E = len(edge), int(np.sum(edge))
    if n == 0:
        return 0
    s = max(1, min(slots, n))
    npos = np.array([n // s + (1 if b < n % s else 0) for b in range(s)])
    L = n // s
    while np.minimum(npos, np.maximum(L - npos, 0)).sum() < E:
        L += 1
    return max(L, int(npos.max()))           # a CTA with one position more works at least that


def tiles(n, npml, shots=1):
    """Edge flags of the 60 x 32 tiles of an n x n grid with an npml C-PML
    (strip reach approximated by npml + 4 cells), rows order."""
    ntx, ntz = -(-n // 60), -(-n // 32)
    lo, hi = npml + 4, n - npml - 4
    e = np.zeros((ntz, ntx), np.uint8)
    for j in range(ntz):
        for i in range(ntx):
            e[j, i] = (i * 60 - 2 < lo) or (i * 60 + 61 > hi) or (j * 32 - 2 < lo) or (j * 32 + 33 > hi)
    return np.tile(e.ravel(), shots)


def check(plan, edge, slots):
    edge = np.asarray(edge, np.uint8)
    o = plan(edge, slots)
    assert sorted(o.tolist()) == list(range(len(edge)))
    for cls in (0, 1):                       # each class keeps its order
        seq = [i for i in o.tolist() if edge[i] == cls]
        assert seq == sorted(seq)
    b = busiest(edge, o, slots)
    assert b == optimum(edge, slots), (b, optimum(edge, slots))
    assert b <= busiest(edge, np.arange(len(edge)), slots)
    return b


def test_benchmark_grids(plan):
    # one 2001^2 shot, 40-cell C-PML, 152 SMs: rows order leaves the busiest CTA 19 units
    e = tiles(2001, 40)
    assert busiest(e, np.arange(len(e)), 152) == 19
    assert check(plan, e, 152) == 17
    # one 1001^2 shot, 30-cell C-PML: 544 tiles on 152 CTAs, 7 units in rows order
    e = tiles(1001, 30)
    assert busiest(e, np.arange(len(e)), 152) == 7
    assert check(plan, e, 152) == 5
    check(plan, tiles(1001, 30, 16), 152)
    check(plan, tiles(1001, 30, 64), 152)


@pytest.mark.parametrize("seed", range(12))
def test_random_lists(plan, seed):
    rng = np.random.default_rng(seed)
    n = int(rng.integers(1, 3000))
    edge = (rng.random(n) < rng.random()).astype(np.uint8)
    check(plan, edge, int(rng.integers(1, 300)))


def test_degenerate_lists(plan):
    assert plan(np.zeros(0, np.uint8), 152).size == 0
    for n in (1, 5, 151, 152, 153):
        for frac in (0.0, 1.0):
            check(plan, np.full(n, frac, np.uint8), 152)
    check(plan, np.array([1, 0, 1, 1, 0], np.uint8), 1)
