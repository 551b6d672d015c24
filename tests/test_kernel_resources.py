"""Register and local-memory use of every kernel, from ptxas's own report
(``-Xptxas -v``, kept by the build in ``poe2d_gb300/_build/*.ptxas.txt``).

The step kernel runs 608 threads per CTA on 60 x 32 tiles (18 compute warps
+ 1 producer; 640 with the step-spanning variants' publisher warp) at one CTA
per SM, so ptxas caps it at 96 registers; what does not fit goes to local
memory.  The 60 x 16 variants (FAST, single model) run 10 compute warps and
may take 128.  The single-model variants and the batch variants the batched
benchmarks run (palette models with K = 1, FAST or few-bit EXACT stencils)
must not spill.  The remaining batch variants (K != 1, per-cell
coefficients, or EXACT at a spacing whose 24 h needs more than 8 bits) spill
a few dozen bytes per thread to L1-resident local memory; the bound below
keeps that from growing unnoticed.  The surrogate kernels must not spill
either.
"""
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

# the step kernel's stencil modes, in template order
MODES = {0: "FAST", 1: "EXACT_FEW", 2: "EXACT_ANY"}


def _parse(text):
    """{mangled name: (registers, stack bytes, spill store bytes, spill load bytes)}"""
    out, cur, frame = {}, None, (0, 0, 0)
    for ln in text.splitlines():
        m = re.search(r"Function properties for (\S+)", ln)
        if m:
            cur, frame = m.group(1), (0, 0, 0)
            continue
        m = re.search(r"(\d+) bytes stack frame, (\d+) bytes spill stores, (\d+) bytes spill loads", ln)
        if m and cur:
            frame = tuple(int(v) for v in m.groups())
            continue
        m = re.search(r"Used (\d+) registers", ln)
        if m and cur:
            out[cur] = (int(m.group(1)),) + frame
            cur = None
    return out


@pytest.fixture(scope="module")
def reports():
    from poe2d_gb300 import build as B
    B.build()
    got = {}
    for src in B.SOURCES:
        if src.endswith(".cu"):
            with open(B.resource_report(src)) as f:
                got[src] = _parse(f.read())
    return got


TILE_UNITS = ("poe2d_tile_fast.cu", "poe2d_tile_exact.cu", "poe2d_tile_exact_any.cu", "poe2d_tile_fast16.cu")


def _step_variants(reports):
    out = {}
    for unit in TILE_UNITS:
        for name, res in reports[unit].items():
            m = re.search(r"k_tile_palILi(\d)ELb(\d)ELb(\d)ELb(\d)ELb(\d)ELi(\d+)E", name)
            if m:
                sm, kone, multi, coef, span, tz = (int(v) for v in m.groups())
                out[(MODES[sm], bool(kone), bool(multi), bool(coef), bool(span), tz)] = res
    return out


def test_every_step_kernel_variant_is_built(reports):
    v = _step_variants(reports)
    assert len([k for k in v if k[5] == 32]) == 3 * 2 * 2 * 2 * 2, sorted(v)
    small = sorted(k for k in v if k[5] == 16)
    assert len(small) == 2 * 2 * 2 and all(k[0] == "FAST" and not k[2] for k in small), small
    for key, (regs, _, _, _) in v.items():
        assert regs <= (96 if key[5] == 32 else 128), (key, regs)   # threads at one CTA per SM


def test_single_model_and_benchmarked_batch_variants_do_not_spill(reports):
    v = _step_variants(reports)
    for key, (regs, stack, st, ld) in v.items():
        mode, kone, multi, coef, span, tz = key
        benchmarked_batch = multi and kone and not coef and mode in ("FAST", "EXACT_FEW")
        if not multi or benchmarked_batch:
            assert st == 0 and ld == 0, (key, st, ld)
        else:
            assert st <= 128 and ld <= 256, (key, st, ld)


def test_surrogate_kernels_do_not_spill(reports):
    for src in ("sg_gemm.cu", "sg_ops.cu"):
        assert reports[src], src
        for name, (regs, stack, st, ld) in reports[src].items():
            assert st == 0 and ld == 0, (name, st, ld)
