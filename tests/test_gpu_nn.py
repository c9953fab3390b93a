"""Learned warm start kernels (include/glgpu_nn.h) against the NumPy reference
(oracle/nn_np.py) on bfloat16-rounded operands, and the autograd wrappers end
to end.  Tolerances: outputs are rounded to bfloat16 (8 significant bits), the
float32 accumulations differ only in order, so 2e-2 of the output's max."""
import numpy as np
import pytest

from oracle import nn_np as R

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _bf(a):
    return torch.from_numpy(R.bf16_round(a)).to("cuda", torch.bfloat16)


def _np(t):
    return t.detach().float().cpu().numpy().astype(np.float64)


def _close(x, ref, tol=2e-2):
    scale = max(np.abs(ref).max(), 1e-30)
    err = np.abs(x - ref).max() / scale
    assert err < tol, err


@pytest.mark.parametrize("relu", [0, 1])
@pytest.mark.parametrize("shape", [(2, 10, 12, 16, 8, 24), (1, 9, 7, 8, 0, 8), (3, 16, 16, 32, 32, 64)])
def test_conv3x3_forward_and_gradients(relu, shape):
    from svirl_gb300 import learned as L
    n, h, w, c1, c2, cout = shape
    rng = np.random.default_rng(1)
    x1 = R.bf16_round(rng.standard_normal((n, h, w, c1)).astype(np.float32))
    x2 = R.bf16_round(rng.standard_normal((n, h, w, c2)).astype(np.float32)) if c2 else None
    W = (rng.standard_normal((cout, 3, 3, c1 + c2)) * 0.2).astype(np.float32)
    b = (rng.standard_normal(cout) * 0.1).astype(np.float32)
    Wr = R.bf16_round(W)
    xc = x1 if x2 is None else np.concatenate([x1, x2], axis=3)
    y_ref = R.conv3x3(xc, Wr, b, relu)

    tx1 = _bf(x1).requires_grad_()
    tx2 = _bf(x2).requires_grad_() if c2 else None
    tW = torch.from_numpy(W).cuda().requires_grad_()
    tb = torch.from_numpy(b).cuda().requires_grad_()
    y = L.Conv3x3.apply(tx1, tx2, tW, tb, relu)
    _close(_np(y), y_ref)

    dy = R.bf16_round(rng.standard_normal(y.shape).astype(np.float32))
    y_used = _np(y)  # the ReLU derivative is taken from the stored (bf16) output
    dx_ref, dw_ref, db_ref = R.conv3x3_bwd(xc, Wr, y_used, dy, relu)
    grads = torch.autograd.grad(y, [tx1, tW, tb] + ([tx2] if c2 else []), grad_outputs=_bf(dy))
    dx = _np(grads[0]) if not c2 else np.concatenate([_np(grads[0]), _np(grads[3])], axis=3)
    _close(dx, dx_ref)
    _close(_np(grads[1]), dw_ref, 5e-3)
    _close(_np(grads[2]), db_ref, 5e-3)


def test_pool_up_add():
    from svirl_gb300 import learned as L
    rng = np.random.default_rng(2)
    x = R.bf16_round(rng.standard_normal((2, 8, 6, 16)).astype(np.float32))
    tx = _bf(x).requires_grad_()
    y = L.Pool2.apply(tx)
    _close(_np(y), R.pool2(x), 1e-2)
    dy = R.bf16_round(rng.standard_normal(y.shape).astype(np.float32))
    (dx,) = torch.autograd.grad(y, tx, grad_outputs=_bf(dy))
    _close(_np(dx), R.up2(dy) * 0.25, 1e-2)
    u = L.Up2.apply(tx)
    _close(_np(u), R.up2(x), 1e-6)
    du = R.bf16_round(rng.standard_normal(u.shape).astype(np.float32))
    (dxu,) = torch.autograd.grad(u, tx, grad_outputs=_bf(du))
    _close(_np(dxu), R.pool2(du) * 4.0, 1e-2)
    lib = L._lib_nn()
    a, b2 = _bf(x), _bf(x * 0.5)
    out = torch.empty_like(a)
    assert lib.glnn_add(L._ptr(a), L._ptr(b2), L._ptr(out), a.numel(), L._stream()) == 0
    _close(_np(out), 1.5 * x, 1e-2)


def test_mse_and_adam():
    from svirl_gb300 import learned as L
    rng = np.random.default_rng(3)
    pred = R.bf16_round(rng.standard_normal((2, 4, 4, 8)).astype(np.float32))
    tgt = rng.standard_normal((2, 4, 4, 4)).astype(np.float32)
    cw = np.array([1.0, 2.0, 0.5, 3.0], dtype=np.float32)
    tp = _bf(pred).requires_grad_()
    loss = L.WeightedMSE.apply(tp, torch.from_numpy(tgt).cuda(), torch.from_numpy(cw).cuda())
    e = pred[..., :4].astype(np.float64) - tgt
    npix = 2 * 4 * 4
    ref = float((cw * e * e).sum() / npix)
    assert abs(float(loss.detach()) - ref) < 1e-5 * abs(ref)
    (g,) = torch.autograd.grad(loss, tp)
    gref = np.zeros_like(pred, dtype=np.float64)
    gref[..., :4] = 2 * cw * e / npix
    _close(_np(g), gref, 1e-2)

    w = rng.standard_normal(1000).astype(np.float32)
    gr = rng.standard_normal(1000).astype(np.float32)
    m = np.zeros(1000, np.float32)
    v = np.zeros(1000, np.float32)
    tw, tg, tm, tv = (torch.from_numpy(a.copy()).cuda() for a in (w, gr, m, v))
    wr, mr, vr = w.astype(np.float64), m.astype(np.float64), v.astype(np.float64)
    for step in (1, 2, 3):
        L.adam_step([tw], [tg], [tm], [tv], step, lr=1e-2, weight_decay=1e-3)
        wr, mr, vr = R.adam(wr, gr.astype(np.float64), mr, vr, 1e-2, 0.9, 0.999, 1e-8, 1e-3, step)
    assert np.abs(tw.cpu().numpy() - wr).max() < 1e-5


def test_network_overfits_one_batch():
    """The wrappers, kernels and optimiser train: the loss on a fixed batch falls."""
    from svirl_gb300 import learned as L
    net = L.WarmStartNet(seed=0, levels=(8, 16, 16, 16))
    rng = np.random.default_rng(4)
    x = _bf(rng.standard_normal((4, 16, 16, 8)).astype(np.float32))
    yy = np.stack(np.meshgrid(np.linspace(-1, 1, 16), np.linspace(-1, 1, 16)), -1)
    y = np.concatenate([yy, yy ** 2], -1)[None].repeat(4, 0).astype(np.float32)
    ty = torch.from_numpy(y).cuda()
    cw = torch.ones(4, device="cuda")
    first = float(net.train_step(x, ty, cw, lr=3e-3))
    for _ in range(150):
        last = float(net.train_step(x, ty, cw, lr=3e-3))
    assert last < 0.1 * first, (first, last)
    assert 1.0e6 < L.WarmStartNet(seed=0).n_params() < 1.5e6


@pytest.mark.parametrize("shape", [(2, 32, 24, 64, 64, 128), (1, 8, 8, 256, 0, 72), (1, 7, 9, 16, 0, 136)])
@pytest.mark.parametrize("relu", [0, 1])
def test_conv3x3_tcgen05_larger_tiles(relu, shape):
    """The tcgen05 forward and data-gradient kernels on shapes with several K
    chunks and N tiles, and a channel count that is not a multiple of the tile;
    no bounded wait may run out."""
    from svirl_gb300 import learned as L
    n, h, w, c1, c2, cout = shape
    rng = np.random.default_rng(5)
    x1 = R.bf16_round(rng.standard_normal((n, h, w, c1)).astype(np.float32))
    x2 = R.bf16_round(rng.standard_normal((n, h, w, c2)).astype(np.float32)) if c2 else None
    W = (rng.standard_normal((cout, 3, 3, c1 + c2)) * 0.1).astype(np.float32)
    b = (rng.standard_normal(cout) * 0.1).astype(np.float32)
    xc = x1 if x2 is None else np.concatenate([x1, x2], axis=3)
    y_ref = R.conv3x3(xc, R.bf16_round(W), b, relu)
    tx1 = _bf(x1).requires_grad_()
    tx2 = _bf(x2).requires_grad_() if c2 else None
    tW = torch.from_numpy(W).cuda().requires_grad_()
    tb = torch.from_numpy(b).cuda().requires_grad_()
    y = L.Conv3x3.apply(tx1, tx2, tW, tb, relu)
    _close(_np(y), y_ref)
    dy = R.bf16_round(rng.standard_normal(y.shape).astype(np.float32))
    dx_ref, _, _ = R.conv3x3_bwd(xc, R.bf16_round(W), _np(y), dy, relu)
    grads = torch.autograd.grad(y, [tx1] + ([tx2] if c2 else []), grad_outputs=_bf(dy))
    dx = _np(grads[0]) if not c2 else np.concatenate([_np(grads[0]), _np(grads[1])], axis=3)
    _close(dx, dx_ref)
    L.check_kernel_errors()
