"""The EXACT stencil arithmetic against the FP64 expressions it reproduces.

The reference evaluates its stencils (cu:64-65, 76-77, 220-221, 297-299,
342-344), the sigma_xz update (cu:226) and sigma_xx / sigma_zz (cu:241-242) in
FP64 because of its double literals, and rounds once to float.  The step
kernel rebuilds those results from FP32 error-free transformations
(poe2d_math.cuh).  Here the same helpers, compiled for the host, meet numpy's
float64 evaluation of the reference's expressions in the reference's order,
bit for bit, on millions of operand tuples: smooth neighbouring values with
heavy cancellation, independent values over many binades, exact ties, zeros
and tiny values down into the subnormal range.  Spacings whose 24 h is a
float of few bits (0.5, 1, 1.25, ...: ties are common) take the kernels'
float tie resolution; all others (0.1, 0.3, ...) a float quotient that is
kept only where its rounding is certain, the reference's own FP64 line
elsewhere.
"""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
_fp = C.POINTER(C.c_float)


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("no g++")
    out = str(tmp_path_factory.mktemp("exact") / "libexact.so")
    subprocess.run([cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", "-I",
                    os.path.join(ROOT, "poe2d_gb300", "csrc"), os.path.join(ROOT, "tests", "exact_math_harness.cpp"),
                    "-o", out], check=True)
    lib = C.CDLL(out)
    lib.d4_many.argtypes = [_fp, _fp, _fp, _fp, C.c_long, C.c_float, _fp, _fp]
    lib.sxz_many.argtypes = [_fp, _fp, _fp, C.c_long, C.c_float, _fp]
    lib.div24_info.argtypes = [C.c_float, _fp, _fp, C.POINTER(C.c_int)]
    lib.div_by_many.argtypes = [_fp, _fp, C.c_long, _fp]
    lib.sxx_szz_many.argtypes = [_fp] * 6 + [C.c_long, _fp, _fp]
    return lib


def _p(a):
    return a.ctypes.data_as(_fp)


def _f32(a):
    return np.ascontiguousarray(a, np.float32)


def _operands(rng, n):
    """a, b, c, d as a stencil sees them, in several regimes."""
    k = n // 5
    # smooth field: four neighbours of one smooth signal, any scale
    base = rng.standard_normal(k) * 10.0 ** rng.uniform(-30, 10, k)
    slope = base * 10.0 ** rng.uniform(-8, -1, k) * rng.choice([-1, 1], k)
    curv = slope * 10.0 ** rng.uniform(-6, 0, k)
    smooth = [base + slope * t + curv * t * t for t in (0.5, -0.5, 1.5, -1.5)]
    # independent values over many binades
    ind = [rng.standard_normal(k) * 10.0 ** rng.uniform(-20, 20, k) for _ in range(4)]
    # small integers and half-integers: exact sums, frequent exact ties in /12
    ints = [rng.integers(-4096, 4097, k) * 0.5 for _ in range(4)]
    # zeros mixed in
    zer = [np.where(rng.random(k) < 0.3, 0.0, rng.standard_normal(k)) for _ in range(4)]
    # tiny values, down into the float subnormal range
    tiny = [rng.standard_normal(k) * 10.0 ** rng.uniform(-44, -28, k) for _ in range(4)]
    cols = [np.concatenate([g[i] for g in (smooth, ind, ints, zer, tiny)]) for i in range(4)]
    return [_f32(c) for c in cols]


@pytest.mark.parametrize("h", [0.5, 1.0, 0.25, 2.0, 1.25, 0.3, 0.1, 0.2, 0.7])
def test_d4_exact_matches_fp64_expression(harness, h):
    rng = np.random.default_rng(int(h * 1000))
    a, b, c, d = _operands(rng, 2_000_000)
    n = a.size
    ex, fa = np.empty(n, np.float32), np.empty(n, np.float32)
    harness.d4_many(_p(a), _p(b), _p(c), _p(d), n, h, _p(ex), _p(fa))
    A, B, Cc, D = (x.astype(np.float64) for x in (a, b, c, d))
    with np.errstate(all="ignore"):
        ref = ((((27.0 * A - 27.0 * B) - Cc) + D) / np.float64(np.float32(h)) / 24.0).astype(np.float32)
    ok = np.isfinite(ref)
    # operands whose magnitudes span more than 2^40: the reference's FP64
    # sums drop the smallest term, which can flip a float tie; the four
    # neighbouring cells of a field never differ that much (zeros are exact)
    with np.errstate(all="ignore"):
        mags = np.abs(np.stack([27.0 * A, 27.0 * B, Cc, D]))
        wide = mags.max(0) > 2.0 ** 40 * np.where(mags > 0, mags, np.inf).min(0)
    bad = np.flatnonzero(ok & ~wide & (ex.view(np.uint32) != ref.view(np.uint32)))
    assert bad.size == 0, (bad.size, a[bad[:3]], b[bad[:3]], c[bad[:3]], d[bad[:3]], ex[bad[:3]], ref[bad[:3]])
    D64 = 24.0 * np.float64(np.float32(h))
    few_bits = np.float64(np.float32(D64)) == D64 and (np.float32(D64).view(np.uint32) & 0xFFFF) == 0
    if not few_bits:
        # the other spacings decide every doubtful rounding by the
        # reference's own FP64 line: no exception at all
        assert np.array_equal(ex[ok].view(np.uint32), ref[ok].view(np.uint32))
    # the FAST stencil stays within a few ulps where nothing cancels badly
    scale = np.maximum(np.abs(27.0 * A) + np.abs(27.0 * B) + np.abs(Cc) + np.abs(D), 1e-300) / (24.0 * h)
    rel = np.abs(fa.astype(np.float64) - ref.astype(np.float64)) / scale
    assert np.nanmax(rel[ok & (scale < 1e30) & (scale > 1e-30)]) < 1e-6


def test_sxz_exact_matches_fp64_expression(harness):
    rng = np.random.default_rng(3)
    n = 2_000_000
    s = _f32(rng.standard_normal(n) * 10.0 ** rng.uniform(-10, 8, n))
    c33 = _f32(rng.uniform(1e8, 3e10, n))
    S = _f32(rng.standard_normal(n) * 10.0 ** rng.uniform(-12, 2, n))
    for dt in (5e-5, 4e-5, 1e-4):
        out = np.empty(n, np.float32)
        harness.sxz_many(_p(s), _p(c33), _p(S), n, dt, _p(out))
        ref = (s.astype(np.float64) + c33.astype(np.float64) / 1.0 * S.astype(np.float64)
               * np.float64(np.float32(dt))).astype(np.float32)
        bad = np.flatnonzero(out.view(np.uint32) != ref.view(np.uint32))
        assert bad.size == 0, (dt, bad.size, s[bad[:3]], c33[bad[:3]], S[bad[:3]])


def test_sxx_szz_exact_match_fp64_expressions(harness):
    rng = np.random.default_rng(4)
    n = 2_000_000
    lam = _f32(rng.uniform(1e8, 3e10, n))
    mu = _f32(rng.uniform(0.0, 1.5e10, n))
    g1 = _f32(rng.standard_normal(n) * 10.0 ** rng.uniform(-14, -2, n))
    g2 = _f32(np.where(rng.random(n) < 0.5, -g1 * rng.uniform(0.5, 1.5, n), rng.standard_normal(n) * 1e-6))
    al = _f32(rng.uniform(0.0, 1.0, n))
    p = _f32(rng.standard_normal(n) * 10.0 ** rng.uniform(-4, 6, n))
    sxx, szz = np.empty(n, np.float32), np.empty(n, np.float32)
    harness.sxx_szz_many(_p(lam), _p(mu), _p(g1), _p(g2), _p(al), _p(p), n, _p(sxx), _p(szz))
    L, M, G1, G2 = (x.astype(np.float64) for x in (lam, mu, g1, g2))
    lg1 = (lam * g1).astype(np.float64)          # float products, as the reference rounds them
    lg2 = (lam * g2).astype(np.float64)
    ap = (al * p).astype(np.float64)
    ref_xx = ((L + 2.0 * M) * G1 + lg2 - ap).astype(np.float32)
    ref_zz = (lg1 + (L + 2.0 * M) * G2 - ap).astype(np.float32)
    assert np.array_equal(sxx.view(np.uint32), ref_xx.view(np.uint32))
    assert np.array_equal(szz.view(np.uint32), ref_zz.view(np.uint32))


@pytest.mark.parametrize("h, few", [(0.5, 1), (1.0, 1), (1.25, 1), (2.5, 1), (5.0, 1), (10.0, 1), (0.25, 1),
                                    (0.1, 0), (0.3, 0), (0.7, 0), (0.2, 0), (3.3, 0)])
def test_divisor_split_and_kind(harness, h, few):
    """24 h = D + Dl exactly (D its float rounding, Dl the rest), and the
    few-bit tie resolution only for a float D of at most 8 significant bits."""
    D, Dl, fb = C.c_float(), C.c_float(), C.c_int()
    harness.div24_info(h, C.byref(D), C.byref(Dl), C.byref(fb))
    exact = 24.0 * float(np.float32(h))
    assert float(D.value) + float(Dl.value) == exact
    assert np.float32(D.value) == np.float32(exact)
    assert fb.value == few


def test_markstein_division_is_correctly_rounded(harness):
    """The palette kernel divides by c1 and co with q0 = a y, r = fma(-b, q0, a),
    q = fma(r, y, q0) and y = RN(1/b) from the material table: IEEE-rounded
    quotients for operands away from overflow and underflow, as the
    reference's own float divisions (cu:307-311)."""
    rng = np.random.default_rng(5)
    n = 4_000_000
    a = _f32(rng.standard_normal(n) * 10.0 ** rng.uniform(-20, 20, n))
    b = _f32(rng.uniform(1.0, 2.0, n) * 10.0 ** rng.uniform(-12, 12, n) * rng.choice([-1, 1], n))
    out = np.empty(n, np.float32)
    harness.div_by_many(_p(a), _p(b), n, _p(out))
    ref = a / b                                          # numpy float32 division: IEEE round to nearest
    assert np.array_equal(out.view(np.uint32), ref.view(np.uint32))
