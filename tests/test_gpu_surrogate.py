"""The surrogate network on the tensor cores against its CPU reference
(oracle/surrogate_ref.py, bf16 rounding emulated at the same points): the
forward pass, the loss and every parameter gradient; plus determinism and a
training run that must fit a fixed batch."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _batch(B, seed):
    g = torch.Generator().manual_seed(seed)
    maps = torch.rand((B, 64, 64, 2), generator=g)
    sc = torch.rand((B, 3), generator=g)
    tgt = 0.05 * torch.randn((B, 1024, 384), generator=g)
    return maps, sc, tgt


def _dev(maps, sc, tgt):
    return (maps.to(torch.bfloat16).cuda(), sc.float().cuda(), tgt.to(torch.bfloat16).cuda())


def _rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def test_forward_loss_and_gradients_match_reference(poe):
    from oracle import surrogate_ref as R
    from poe2d_gb300.surrogate import Surrogate
    net = Surrogate(max_batch=16, seed=3)
    assert net.nparam == R.param_count()
    p = net.params()
    maps, sc, tgt = _batch(8, 1)
    dm, ds, dt = _dev(maps, sc, tgt)
    out = net.forward(dm, ds).cpu().numpy()
    mq = dm.float().cpu().numpy()
    tq = dt.float().cpu().numpy()
    ref = R.forward(p, mq, sc.numpy())
    assert _rel(out, ref) <= 1e-2
    loss = net.loss_grad(dm, ds, dt)
    g = net.grads()
    rloss, rg = R.loss_and_grads(p, mq, sc.numpy(), tq)
    assert abs(loss - rloss) <= 1e-3 * rloss
    q = 0
    for i, (kind, ci, co, *_) in enumerate(R.LAYERS):
        n = co * R._k(kind, ci) + co
        a, b = g[q:q + n], rg[q:q + n]
        cos = float(np.dot(a, b) / (np.linalg.norm(a) * np.linalg.norm(b) + 1e-300))
        assert _rel(a, b) <= 5e-2 and cos >= 0.998, (i, _rel(a, b), cos)
        q += n
    # deterministic: the same batch gives the same gradient bits
    net.loss_grad(dm, ds, dt)
    assert np.array_equal(net.grads().view(np.uint32), g.view(np.uint32))
    net.close()


def test_params_roundtrip_and_training_fits_a_batch(poe):
    from poe2d_gb300.surrogate import Surrogate
    net = Surrogate(max_batch=16, seed=5)
    p = net.params()
    net.set_params(p * 0.5)
    assert np.array_equal(net.params(), (p * 0.5).astype(np.float32))
    net.set_params(p)
    maps, sc, _ = _batch(16, 2)
    # targets the network can represent: another network's output
    teacher = Surrogate(max_batch=16, seed=9)
    dm, ds = maps.to(torch.bfloat16).cuda(), sc.float().cuda()
    tgt = teacher.forward(dm, ds).to(torch.bfloat16)
    l0 = net.loss_grad(dm, ds, tgt)
    for _ in range(60):
        loss = net.train_step(dm, ds, tgt, 1e-3)
    assert loss < 0.2 * l0, (l0, loss)
    assert net.launches > 0
    net.close()
    teacher.close()


def test_adam_steps_match_numpy_adam(poe):
    """Three poe_sg_adam steps on gradients of three batches against numpy's
    Adam (oracle/surrogate_ref.py: bias-corrected moments, float64), each step
    from the GPU's own state before it.  The moments m and v agree within
    1e-6 of the magnitudes they are summed from, and the FP32 weights within
    1e-6 of |w| + |w_new| of numpy's update from the GPU's new moments (the
    kernel folds the bias corrections into its step size and epsilon; its
    FP32 rounding is far below those bounds, also where a sum cancels).  The
    bf16 weight copy equals the FP32 weights rounded to nearest-even bit for
    bit, and the step counter counts."""
    from oracle import surrogate_ref as R
    from poe2d_gb300.surrogate import Surrogate
    net = Surrogate(max_batch=8, seed=11)
    w = net.params().astype(np.float64)
    m = np.zeros_like(w)
    v = np.zeros_like(w)
    lr = 1e-3
    b1, one_b1 = float(R.ADAM_B1), float(np.float32(1) - R.ADAM_B1)
    for t in (1, 2, 3):
        maps, sc, tgt = _batch(8, 20 + t)
        dm, ds, dt = _dev(maps, sc, tgt)
        net.loss_grad(dm, ds, dt)
        g = net.grads().astype(np.float64)
        assert np.count_nonzero(g) > 0.25 * g.size        # ReLU zeroes some units' gradients
        net.adam(lr)
        _, m1, v1 = R.adam_step(w, g, m, v, t, lr)
        gm, gv, w16, steps = net.state()
        gw = net.params().astype(np.float64)
        assert steps == t
        # the weights: numpy's update from the moments the GPU holds now
        c1, c2 = 1.0 - b1 ** t, 1.0 - float(R.ADAM_B2) ** t
        w1 = w - lr * (gm / c1) / (np.sqrt(gv / c2) + R.ADAM_EPS)
        bounds = (("m", gm, m1, b1 * np.abs(m) + one_b1 * np.abs(g)), ("v", gv, v1, np.abs(v1)),
                  ("w", gw, w1, np.abs(w) + np.abs(w1)))
        for name, a, b, mag in bounds:
            err = np.abs(np.asarray(a, np.float64) - b)
            assert np.all(err <= 1e-6 * mag + 1e-37), (t, name, float((err / (mag + 1e-37)).max()))
        assert np.array_equal(w16.view(np.uint32), R.bf16_bits(gw.astype(np.float32))), t
        w, m, v = gw, gm.astype(np.float64), gv.astype(np.float64)
    net.close()


def test_forward_of_an_item_does_not_depend_on_its_batch(poe):
    """Each gather depends on its own map only: the time convolutions read
    whole items (several per 128-row tile at the short early lengths, with the
    rows past an item's end as zeros), so a model's output is the same bits in
    a batch of 1, 3 or 8."""
    from poe2d_gb300.surrogate import Surrogate
    net = Surrogate(max_batch=8, seed=5)
    maps, sc, tgt = _batch(8, 2)
    dm, ds, _ = _dev(maps, sc, tgt)
    full = net.forward(dm, ds).cpu().numpy()
    for n, first in ((1, 0), (3, 2), (1, 7)):
        part = net.forward(dm[first:first + n].contiguous(), ds[first:first + n].contiguous()).cpu().numpy()
        assert np.array_equal(part.view(np.uint32), full[first:first + n].view(np.uint32)), (n, first)
    net.close()


@pytest.mark.parametrize("shape,dtype", [((40, 64, 64, 2), torch.bfloat16), ((40, 3), torch.float32),
                                         ((40, 1024, 384), torch.bfloat16), ((5, 7), torch.int32)])
def test_gather_rows_equals_indexing(poe, shape, dtype):
    """The training batch gather (16-byte vectors, or 4-byte words for rows
    such as the 3 scalars) returns t[idx] bit for bit, repeats included."""
    from poe2d_gb300.surrogate import gather_rows
    g = torch.Generator().manual_seed(len(shape) * 31 + shape[0])
    t = (torch.randn(shape, generator=g) * 100).to(dtype).cuda()
    idx = torch.randint(0, shape[0], (17,), generator=g).cuda()
    got = gather_rows(t, idx)
    torch.cuda.synchronize()
    assert got.shape == (17,) + shape[1:] and torch.equal(got, t[idx])


def test_forward_rejects_an_unaligned_output(poe):
    """The output layer writes `out` with TMA stores: a pointer off a 16-byte
    boundary is refused with POE_EINVAL, nothing is launched."""
    from poe2d_gb300 import _lib as L
    from poe2d_gb300.surrogate import Surrogate
    net = Surrogate(max_batch=8, seed=1)
    maps, sc, tgt = _batch(2, 3)
    dm, ds, _ = _dev(maps, sc, tgt)
    buf = torch.empty(2 * 1024 * 384 + 4, dtype=torch.float32, device="cuda")
    rc = L.lib().poe_sg_forward(net.h, dm.data_ptr(), ds.data_ptr(), 2, buf.data_ptr() + 4)
    assert rc == L.POE_EINVAL
    net.forward(dm, ds, out=buf[4:].view(2, 1024, 384))      # 16 bytes in: accepted
    net.close()
