"""Python face of the learned surrogate (include/poe2d_surrogate.h).

``Surrogate`` wraps one network: parameters, inference, training steps.  The
tensors it takes are torch CUDA tensors (device memory and streams come from
torch; every kernel is the library's own).  ``Ensemble`` holds four members
trained from different seeds; where their predictions disagree by more than a
threshold the caller falls back to the solver.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L
from ._lib import PoeError

MAP, MAP_CH, SCALARS, SAMPLES, CHANNELS = 64, 2, 3, 1024, 384

# (GEMM rows per sample, reduction length, output channels) of every layer
_LAYER_GEMMS = [(32 * 32, 18, 64), (16 * 16, 576, 128), (8 * 8, 1152, 128), (4 * 4, 1152, 256),
                (1, 4099, 256), (1, 256, 2048), (32, 384, 128), (64, 384, 128), (128, 384, 128),
                (256, 384, 64), (512, 192, 64), (1024, 192, 64), (1024, 192, 384)]


def gather_rows(t, idx, stream=None):
    """t[idx] for a contiguous CUDA tensor t and an int64 CUDA index vector,
    by the library's row-gather kernel (poe_sg_gather_rows) on `stream`
    (default: torch's current stream)."""
    import torch
    assert t.is_cuda and t.is_contiguous() and idx.dtype == torch.int64 and idx.is_cuda
    out = torch.empty((idx.numel(),) + tuple(t.shape[1:]), dtype=t.dtype, device=t.device)
    row = t[0].numel() * t.element_size() if t.shape[0] else 0
    st = stream if stream is not None else torch.cuda.current_stream().cuda_stream
    rc = L.lib().poe_sg_gather_rows(C.c_void_p(t.data_ptr()), row, C.c_void_p(idx.data_ptr()), idx.numel(),
                                    C.c_void_p(out.data_ptr()), C.c_void_p(st))
    if rc != L.POE_OK:
        raise PoeError(rc, "poe_sg_gather_rows")
    return out


def forward_flops_per_sample():
    """Multiply-add FLOPs (2 per MAC) of one gather's forward pass."""
    return sum(2 * m * k * n for m, k, n in _LAYER_GEMMS)


class Surrogate:
    def __init__(self, max_batch=256, seed=0, stream=None):
        h = C.c_void_p()
        st = L.lib().poe_sg_create(int(max_batch), int(seed), C.c_void_p(stream or 0), C.byref(h))
        if st != L.POE_OK:
            raise PoeError(st, "poe_sg_create")
        self.h = h
        self.max_batch = max_batch
        n = C.c_int64(0)
        L.lib().poe_sg_param_count(self.h, C.byref(n))
        self.nparam = n.value

    def _check(self, st):
        if st != L.POE_OK:
            m = L.lib().poe_sg_last_error(self.h)
            raise PoeError(st, m.decode() if m else "")

    def close(self):
        if getattr(self, "h", None):
            L.lib().poe_sg_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def params(self):
        out = np.empty(self.nparam, np.float32)
        self._check(L.lib().poe_sg_get_params(self.h, out.ctypes.data_as(L._fp), self.nparam))
        return out

    def set_params(self, p):
        p = np.ascontiguousarray(p, np.float32)
        self._check(L.lib().poe_sg_set_params(self.h, p.ctypes.data_as(L._fp), p.size))

    def grads(self):
        out = np.empty(self.nparam, np.float32)
        self._check(L.lib().poe_sg_get_grads(self.h, out.ctypes.data_as(L._fp), self.nparam))
        return out

    def forward(self, maps, scalars, out=None):
        """maps: bf16 [B, 64, 64, 2], scalars: f32 [B, 3] (CUDA) -> f32 [B, 1024, 384]."""
        import torch
        B = maps.shape[0]
        if out is None:
            out = torch.empty((B, SAMPLES, CHANNELS), dtype=torch.float32, device=maps.device)
        self._check(L.lib().poe_sg_forward(self.h, maps.data_ptr(), scalars.data_ptr(), B, out.data_ptr()))
        return out

    def loss_grad(self, maps, scalars, targets):
        loss = C.c_float(0.0)
        self._check(L.lib().poe_sg_loss_grad(self.h, maps.data_ptr(), scalars.data_ptr(), targets.data_ptr(),
                                             maps.shape[0], C.byref(loss)))
        return loss.value

    def state(self):
        """Adam state: (m, v, bf16 weight copy as FP32, steps taken), compact layout."""
        m, v, w16 = (np.empty(self.nparam, np.float32) for _ in range(3))
        t = C.c_int32(0)
        self._check(L.lib().poe_sg_get_state(self.h, m.ctypes.data_as(L._fp), v.ctypes.data_as(L._fp),
                                             w16.ctypes.data_as(L._fp), self.nparam, C.byref(t)))
        return m, v, w16, t.value

    def adam(self, lr):
        self._check(L.lib().poe_sg_adam(self.h, float(lr)))

    def train_step(self, maps, scalars, targets, lr):
        loss = C.c_float(0.0)
        self._check(L.lib().poe_sg_train_step(self.h, maps.data_ptr(), scalars.data_ptr(), targets.data_ptr(),
                                              maps.shape[0], float(lr), C.byref(loss)))
        return loss.value

    @property
    def launches(self):
        n = C.c_int64(0)
        self._check(L.lib().poe_sg_launches(self.h, C.byref(n)))
        return n.value


def _bench(argv=None):
    """python -m poe2d_gb300.surrogate [--batch 256] [--members 4] [--reps 5]:
    inference throughput of an ensemble (weights do not change the work)."""
    import argparse
    import json

    import torch
    ap = argparse.ArgumentParser()
    ap.add_argument("--batch", type=int, default=256)
    ap.add_argument("--members", type=int, default=4)
    ap.add_argument("--reps", type=int, default=5)
    a = ap.parse_args(argv)
    st = torch.cuda.Stream()
    torch.cuda.set_stream(st)
    nets = [Surrogate(max_batch=a.batch, seed=k, stream=st.cuda_stream) for k in range(a.members)]
    g = torch.Generator().manual_seed(0)
    maps = torch.rand((a.batch, MAP, MAP, MAP_CH), generator=g).to(torch.bfloat16).cuda()
    sc = torch.rand((a.batch, SCALARS), generator=g).cuda()
    out = torch.empty((a.members, a.batch, SAMPLES, CHANNELS), device="cuda")

    def run():
        for k, net in enumerate(nets):
            net.forward(maps, sc, out=out[k])
    run()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    for _ in range(a.reps):
        run()
    e1.record(st)
    torch.cuda.synchronize()
    t = e0.elapsed_time(e1) * 1e-3 / a.reps
    print(json.dumps({"gathers_per_s": a.batch / t, "members": a.members, "batch": a.batch,
                      "tensor_tflops": forward_flops_per_sample() * a.batch * a.members / t / 1e12}))
    for net in nets:
        net.close()


if __name__ == "__main__":
    _bench()
