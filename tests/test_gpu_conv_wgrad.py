"""The backward pass of the 3x3 convolution with TMA operands.  Weight gradient on
tcgen05 (M = two taps x 64 input channels, N = 64 output channels, K = pixels; both
operands MN-major boxes loaded by TMA, split-K partial sums reduced in a fixed
order) against the NumPy reference (oracle/nn_np.py) on bfloat16-rounded operands
(5e-3 of the gradient's max, as the other weight-gradient tests) and against the
mma.sync kernel on the same inputs (1e-4 of max: the same bf16 products, summed in
FP32 in another order).  Data gradient from the TMA kernel (dy masked once by
glnn_relu_mask, shifted boxes of dy, Wt as a 3-D tensor) against the reference
(2e-2 of max: bf16 outputs) and against the thread-gather kernel (bitwise: the same
products in the same order).  Shapes: pixel chunks that are runs of one row
(w = 64, 128) or groups of rows (w = 16, 32), channel concatenation, several
channel tiles, a pixel count that gives a single split.  No bounded wait may run
out."""
import numpy as np
import pytest

from oracle import nn_np as R

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _grads(L, x1, x2, W, b, dy, relu, mode):
    lib = L._lib_nn()
    lib.glnn_set_conv_tma(mode)
    try:
        tx1 = torch.from_numpy(x1).to("cuda", torch.bfloat16).requires_grad_()
        tx2 = torch.from_numpy(x2).to("cuda", torch.bfloat16).requires_grad_() if x2 is not None else None
        tW = torch.from_numpy(W).cuda().requires_grad_()
        tb = torch.from_numpy(b).cuda().requires_grad_()
        y = L.Conv3x3.apply(tx1, tx2, tW, tb, relu)
        ins = [tW, tb, tx1] + ([tx2] if tx2 is not None else [])
        g = torch.autograd.grad(y, ins, grad_outputs=torch.from_numpy(dy).to("cuda", torch.bfloat16))
        torch.cuda.synchronize()
        f = lambda t: t.detach().float().cpu().numpy().astype(np.float64)
        dx = f(g[2]) if tx2 is None else np.concatenate([f(g[2]), f(g[3])], axis=3)
        return f(y), f(g[0]), f(g[1]), dx
    finally:
        lib.glnn_set_conv_tma(2)


@pytest.mark.parametrize("shape", [(2, 16, 16, 64, 0, 64), (1, 32, 128, 64, 64, 128), (1, 8, 64, 128, 0, 64),
                                   (4, 8, 32, 64, 64, 64), (1, 2, 32, 64, 0, 64), (8, 64, 64, 64, 0, 64),
                                   (1, 8, 64, 64, 0, 192)])
@pytest.mark.parametrize("relu", [0, 1])
def test_tcgen05_weight_gradient(shape, relu):
    from svirl_gb300 import learned as L
    n, h, w, c1, c2, cout = shape
    rng = np.random.default_rng(17)
    x1 = R.bf16_round(rng.standard_normal((n, h, w, c1)).astype(np.float32))
    x2 = R.bf16_round(rng.standard_normal((n, h, w, c2)).astype(np.float32)) if c2 else None
    W = (rng.standard_normal((cout, 3, 3, c1 + c2)) * 0.1).astype(np.float32)
    b = (rng.standard_normal(cout) * 0.1).astype(np.float32)
    dy = R.bf16_round(rng.standard_normal((n, h, w, cout)).astype(np.float32))
    xc = x1 if x2 is None else np.concatenate([x1, x2], axis=3)
    y_t, gw_t, gb_t, dx_t = _grads(L, x1, x2, W, b, dy, relu, 2)
    L.check_kernel_errors()
    y_1, gw_1, gb_1, dx_1 = _grads(L, x1, x2, W, b, dy, relu, 1)
    L.check_kernel_errors()
    y_m, gw_m, gb_m, dx_m = _grads(L, x1, x2, W, b, dy, relu, 0)
    # one tile per CTA and persistent: the same values
    assert np.array_equal(y_t, y_1) and np.array_equal(dx_t, dx_1) and np.array_equal(gw_t, gw_1)
    dx_ref, dw_ref, db_ref = R.conv3x3_bwd(xc, R.bf16_round(W), y_t, dy, relu)
    e_dx = np.abs(dx_t - dx_ref).max() / np.abs(dx_ref).max()
    print("shape %s relu %d: TMA dx vs reference %.2e, vs gather max |diff| %.2e"
          % (shape, relu, e_dx, np.abs(dx_t - dx_m).max()))
    assert e_dx < 2e-2 and np.array_equal(dx_t, dx_m)
    scale = np.abs(dw_ref).max()
    e_ref = np.abs(gw_t - dw_ref).max() / scale
    e_mma = np.abs(gw_t - gw_m).max() / scale
    print("shape %s relu %d: tcgen05 dW vs reference %.2e, vs mma %.2e" % (shape, relu, e_ref, e_mma))
    assert e_ref < 5e-3 and e_mma < 1e-4
    assert np.abs(gb_t - db_ref).max() / np.abs(db_ref).max() < 5e-3
