"""The surrogate's tensor-core GEMM (tcgen05, TMA, TMEM) against an FP32
matmul of the same bf16 operands.

C = alpha * A . B^T (+ bias) (ReLU) (+= C) with A: M x K, B: N x K (bf16,
K contiguous).  FP32 accumulation in a different order than torch's, so the
bar is a relative tolerance of 1e-4 of the result's scale.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _gemm(lib, A, B, alpha=1.0, bias=None, relu=False, out32=None, out16=None, accumulate=False, ws=None):
    M, K = A.shape
    N = B.shape[0]
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    ldc = (out32 if out32 is not None else out16).shape[1]
    st = lib.poe_sg_gemm(A.data_ptr(), A.stride(0), B.data_ptr(), B.stride(0), M, N, K, alpha,
                         bias.data_ptr() if bias is not None else None, int(relu),
                         out32.data_ptr() if out32 is not None else None,
                         out16.data_ptr() if out16 is not None else None, ldc, int(accumulate),
                         ws.data_ptr() if ws is not None else None, ws.numel() if ws is not None else 0,
                         err.data_ptr(), torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert st == 0
    assert int(err.item()) == 0
    return out32 if out32 is not None else out16


@pytest.mark.parametrize("M,N,K,bias,relu", [
    (128, 128, 64, False, False),
    (300, 200, 520, True, True),      # tails in every dimension
    (64, 384, 192, True, False),      # fewer rows than one tile
    (1024, 256, 1152, True, True),
    (64, 2048, 256, True, True),
    (65536 // 8, 64, 576, True, True),
])
def test_gemm_matches_fp32(poe, M, N, K, bias, relu):
    lib = poe.lib()
    g = torch.Generator(device="cuda").manual_seed(M + N + K)
    A = torch.randn(M, K, device="cuda", generator=g).to(torch.bfloat16)
    B = torch.randn(N, K, device="cuda", generator=g).to(torch.bfloat16)
    b = torch.randn(N, device="cuda", generator=g) if bias else None
    out = torch.full((M, N), 7.0, device="cuda")
    _gemm(lib, A, B, 0.5, b, relu, out32=out)
    ref = 0.5 * (A.float() @ B.float().T)
    if bias:
        ref = ref + b
    if relu:
        ref = torch.relu(ref)
    scale = float(ref.abs().max())
    assert float((out - ref).abs().max()) <= 1e-4 * scale


def test_gemm_split_k_accumulate_and_bf16_out(poe):
    lib = poe.lib()
    g = torch.Generator(device="cuda").manual_seed(5)
    M, N, K = 384, 192, 65536
    A = torch.randn(M, K, device="cuda", generator=g).to(torch.bfloat16)
    B = torch.randn(N, K, device="cuda", generator=g).to(torch.bfloat16)
    ws = torch.empty(16 * M * N, device="cuda")
    base = torch.randn(M, N, device="cuda", generator=g)
    out = base.clone()
    _gemm(lib, A, B, 1.0 / K, out32=out, accumulate=True, ws=ws)
    ref = base + (A.float() @ B.float().T) / K
    assert float((out - ref).abs().max()) <= 1e-4 * float(ref.abs().max())
    # the same product twice gives the same bits (fixed split order)
    out2 = base.clone()
    _gemm(lib, A, B, 1.0 / K, out32=out2, accumulate=True, ws=ws)
    assert torch.equal(out, out2)
    o16 = torch.zeros(M, N, dtype=torch.bfloat16, device="cuda")
    _gemm(lib, A[:, :512], B[:, :512], 1.0, out16=o16)
    ref16 = (A[:, :512].float() @ B[:, :512].float().T)
    assert float((o16.float() - ref16).abs().max()) <= 1e-2 * float(ref16.abs().max())


def test_gemm_rejects_bad_pitch(poe):
    lib = poe.lib()
    A = torch.zeros(64, 70, dtype=torch.bfloat16, device="cuda")      # pitch 70: not a multiple of 8
    B = torch.zeros(64, 72, dtype=torch.bfloat16, device="cuda")
    out = torch.zeros(64, 64, device="cuda")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    st = lib.poe_sg_gemm(A.data_ptr(), 70, B.data_ptr(), 72, 64, 64, 64, 1.0, None, 0, out.data_ptr(), None, 64, 0,
                         None, 0, err.data_ptr(), None)
    assert st == 1


@pytest.mark.parametrize("f32,M,N,ldc", [
    (True, 300, 200, 208),     # TMA-store epilogue, a padded pitch: columns N.. ldc stay untouched
    (True, 300, 200, 202),     # pitch not a multiple of 16 bytes: per-thread stores
    (False, 300, 200, 200),    # bf16 through TMA stores, tails in both dimensions
    (False, 1000, 48, 56),     # bf16, a 64-wide tile, padded pitch
    (False, 300, 200, 204),    # bf16 pitch not a multiple of 16 bytes
])
def test_gemm_output_paths_and_pitches(poe, f32, M, N, ldc):
    """Both epilogues (TMA stores of the staged tile, per-thread stores) write
    exactly the M x N result and nothing past it in the row pitch."""
    lib = poe.lib()
    g = torch.Generator(device="cuda").manual_seed(M * 7 + N + ldc)
    K = 192
    A = torch.randn(M, K, device="cuda", generator=g).to(torch.bfloat16)
    B = torch.randn(N, K, device="cuda", generator=g).to(torch.bfloat16)
    b = torch.randn(N, device="cuda", generator=g)
    if f32:
        buf = torch.full((M, ldc), 7.0, device="cuda")
        _gemm(lib, A, B, 1.0, b, True, out32=buf)
        got = buf[:, :N]
        assert bool((buf[:, N:] == 7.0).all())
    else:
        buf = torch.full((M, ldc), 7.0, device="cuda").to(torch.bfloat16)
        _gemm(lib, A, B, 1.0, b, True, out16=buf)
        got = buf[:, :N].float()
        assert bool((buf[:, N:].float() == 7.0).all())
    ref = torch.relu(A.float() @ B.float().T + b)
    tol = 1e-4 if f32 else 1e-2
    assert float((got - ref).abs().max()) <= tol * float(ref.abs().max())
