"""The TMA-fed forward convolution (operands loaded with cp.async.bulk.tensor from
4-D / 2-D tensor maps, mbarrier pipeline, tcgen05 MMAs), one output tile per CTA
(mode 1) and persistent (mode 2: CTAs loop over tiles, two TMEM accumulators),
against the NumPy reference (oracle/nn_np.py) on bfloat16-rounded operands, at the
tolerance of the other convolution tests (2e-2 of the output's max: bfloat16
outputs), and against the thread-gather kernel on the same inputs (bitwise: the
same products accumulated in the same order); on the shapes the TMA path takes:
whole-row tiles (w = 128, 256), groups of rows (w = 16, 32), channel concatenation,
several output tiles; mode 2 keeps the weights resident in shared memory for up to
two 64-channel input chunks and streams them for more (the last shape).  No
bounded wait may run out."""
import numpy as np
import pytest

from oracle import nn_np as R

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _fwd(L, x1, x2, W, b, relu, mode):
    import ctypes as C
    lib = L._lib_nn()
    lib.glnn_set_conv_tma(mode)
    try:
        tx1 = torch.from_numpy(x1).to("cuda", torch.bfloat16)
        tx2 = torch.from_numpy(x2).to("cuda", torch.bfloat16) if x2 is not None else None
        tW = torch.from_numpy(W).cuda()
        tb = torch.from_numpy(b).cuda()
        y = L.Conv3x3.apply(tx1, tx2, tW, tb, relu)
        torch.cuda.synchronize()
        return y.float().cpu().numpy().astype(np.float64)
    finally:
        lib.glnn_set_conv_tma(2)
        del C


@pytest.mark.parametrize("shape", [(2, 16, 16, 64, 0, 64), (1, 32, 128, 64, 64, 128), (1, 8, 256, 128, 0, 64),
                                   (4, 8, 32, 64, 64, 64), (1, 8, 128, 128, 64, 64)])
@pytest.mark.parametrize("relu", [0, 1])
@pytest.mark.parametrize("mode", [1, 2])
def test_tma_forward_matches_reference_and_gather(shape, relu, mode):
    from svirl_gb300 import learned as L
    n, h, w, c1, c2, cout = shape
    rng = np.random.default_rng(11)
    x1 = R.bf16_round(rng.standard_normal((n, h, w, c1)).astype(np.float32))
    x2 = R.bf16_round(rng.standard_normal((n, h, w, c2)).astype(np.float32)) if c2 else None
    W = (rng.standard_normal((cout, 3, 3, c1 + c2)) * 0.1).astype(np.float32)
    b = (rng.standard_normal(cout) * 0.1).astype(np.float32)
    xc = x1 if x2 is None else np.concatenate([x1, x2], axis=3)
    y_ref = R.conv3x3(xc, R.bf16_round(W), b, relu)
    y_tma = _fwd(L, x1, x2, W, b, relu, mode)
    L.check_kernel_errors()
    y_gat = _fwd(L, x1, x2, W, b, relu, 0)
    scale = np.abs(y_ref).max()
    e_ref = np.abs(y_tma - y_ref).max() / scale
    e_gat = np.abs(y_tma - y_gat).max() / scale
    print("shape %s relu %d mode %d: TMA vs reference %.2e, vs gather %.2e" % (shape, relu, mode, e_ref, e_gat))
    assert e_ref < 2e-2 and np.array_equal(y_tma, y_gat)
