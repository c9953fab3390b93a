"""Learned CG warm start: a convolutional encoder-decoder that predicts a
near-minimum (psi, A) of an instance from (material mask, H, 1/kappa, initial
psi), used as the starting point of the CG.  The CG decides: a prediction only
counts once the CG from it reaches the energy and gradient tolerances.  No counterpart in the reference (its only minimiser is the CG of
svirl/solvers/cg.py).

Compute: every convolution, pooling/upsampling, the loss and the optimiser step
run in the hand-written kernels of ``include/glgpu_nn.h`` (BF16 implicit GEMMs
on the tensor cores with FP32 accumulation: tcgen05 with tensor memory, the
operands of the forward pass and of both gradients loaded by TMA; thread-gather and
mma.sync kernels for shapes the TMA kernels do not take); PyTorch
supplies device tensors, the stream and the autograd bookkeeping
(``torch.autograd.Function`` wrappers).

Network: 4 resolution levels (32, 64, 128, 128 channels), two 3x3 convolutions
with ReLU per level and per decoder stage, 2x2 average pooling, nearest 2x
upsampling, skip connections by channel concatenation, a linear 3x3 output
convolution; about 1.2 M parameters.  Inputs (8 channels, NHWC, node grid,
H = Ny rows, W = Nx columns): [node mask, H, 1/kappa, Re psi0, Im psi0, 0, 0, 0].
Outputs: [Re psi, Im psi, delta a, delta b, ...] with delta A = A - A_Landau on
the links (a: Nx-1 x Ny, b: Nx x Ny-1, zero-padded to the node grid).

Target modes: "full" predicts psi itself; "amplitude" (default) predicts |psi|
in the first channel and keeps the phase of the initial psi, since where the
vortices of a relaxed state sit follows the random start in ways a local
predictor cannot know, while the amplitude profile and the screening field
delta A are smooth functions of the geometry and field.
"""
import ctypes as C
import math

import numpy as np
import torch

from . import _lib

CIN, COUT, NOUT = 8, 8, 4
LEVELS = (32, 64, 128, 128)


def _lib_nn():
    return _lib.load()


def _ptr(t):
    return None if t is None else C.c_void_p(t.data_ptr())


def _stream():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def _ok(rc, what):
    if rc != 0:
        raise _lib.GLGPUError("glnn error %d in %s" % (rc, what))


_err = {}


def _err_flag(device):
    """Device int the tcgen05 convolutions set when a bounded wait runs out."""
    key = str(device)
    if key not in _err:
        _err[key] = torch.zeros(1, dtype=torch.int32, device=device)
    return _err[key]


def check_kernel_errors():
    """Raise if a tensor-core convolution reported a timed-out wait (one sync)."""
    for t in _err.values():
        if int(t.item()) != 0:
            t.zero_()
            raise _lib.GLGPUError("glnn: a tensor-core convolution timed out waiting for its MMAs")


# ---------------------------------------------------------------------------
# autograd wrappers of the kernels
# ---------------------------------------------------------------------------

class Conv3x3(torch.autograd.Function):
    """y = conv3x3([x1 | x2]) + b, optional ReLU; bf16 NHWC activations, fp32 weights."""

    @staticmethod
    def forward(ctx, x1, x2, w, b, relu):
        lib = _lib_nn()
        n, h, wd, c1 = x1.shape
        c2 = 0 if x2 is None else x2.shape[3]
        cout = w.shape[0]
        wb = torch.empty(w.shape, dtype=torch.bfloat16, device=w.device)
        wt = torch.empty((3, 3, c1 + c2, cout), dtype=torch.bfloat16, device=w.device)
        s = _stream()
        _ok(lib.glnn_prep_weights(_ptr(w), _ptr(wb), _ptr(wt), cout, c1 + c2, s), "prep_weights")
        y = torch.empty((n, h, wd, cout), dtype=torch.bfloat16, device=x1.device)
        _ok(lib.glnn_conv3x3_fwd(_ptr(x1), c1, _ptr(x2), c2, _ptr(wb), _ptr(b), _ptr(y), n, h, wd, cout,
                                 1 if relu else 0, _ptr(_err_flag(x1.device)), s), "conv3x3_fwd")
        ctx.save_for_backward(x1, x2, wt, y)
        ctx.relu = bool(relu)
        return y

    @staticmethod
    def backward(ctx, dy):
        lib = _lib_nn()
        x1, x2, wt, y = ctx.saved_tensors
        dy = dy.contiguous()
        n, h, wd, c1 = x1.shape
        c2 = 0 if x2 is None else x2.shape[3]
        cout = y.shape[3]
        s = _stream()
        relu = 0
        if ctx.relu:
            # dy * relu'(y) once, for both gradients (their TMA kernels load it as is)
            dym = torch.empty_like(dy)
            _ok(lib.glnn_relu_mask(_ptr(dy), _ptr(y), _ptr(dym), dy.numel(), s), "relu_mask")
            dy = dym
        dx1 = dx2 = None
        if ctx.needs_input_grad[0] or ctx.needs_input_grad[1]:
            dx1 = torch.empty_like(x1)
            dx2 = None if x2 is None else torch.empty_like(x2)
            _ok(lib.glnn_conv3x3_bwd_data(_ptr(dy), _ptr(y), relu, _ptr(wt), _ptr(dx1), c1, _ptr(dx2), c2, n, h, wd,
                                          cout, _ptr(_err_flag(dy.device)), s), "conv3x3_bwd_data")
        dw = torch.empty((cout, 3, 3, c1 + c2), dtype=torch.float32, device=dy.device)
        db = torch.empty((cout,), dtype=torch.float32, device=dy.device)
        nwork = int(lib.glnn_conv3x3_bwd_weight_work(n, h, wd, c1 + c2, cout))
        work = torch.empty((nwork,), dtype=torch.float32, device=dy.device)
        _ok(lib.glnn_conv3x3_bwd_weight(_ptr(dy), _ptr(y), relu, _ptr(x1), c1, _ptr(x2), c2, _ptr(dw), _ptr(db),
                                        _ptr(work), nwork, n, h, wd, cout, _ptr(_err_flag(dy.device)), s),
            "conv3x3_bwd_weight")
        return dx1, dx2, dw, db, None


class Pool2(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x):
        n, h, w, c = x.shape
        y = torch.empty((n, h // 2, w // 2, c), dtype=x.dtype, device=x.device)
        _ok(_lib_nn().glnn_pool2_fwd(_ptr(x), _ptr(y), n, h, w, c, _stream()), "pool2_fwd")
        ctx.shape = x.shape
        return y

    @staticmethod
    def backward(ctx, dy):
        n, h, w, c = ctx.shape
        dx = torch.empty(ctx.shape, dtype=dy.dtype, device=dy.device)
        _ok(_lib_nn().glnn_pool2_bwd(_ptr(dy.contiguous()), _ptr(dx), n, h, w, c, _stream()), "pool2_bwd")
        return dx


class Up2(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x):
        n, h, w, c = x.shape
        y = torch.empty((n, 2 * h, 2 * w, c), dtype=x.dtype, device=x.device)
        _ok(_lib_nn().glnn_up2_fwd(_ptr(x), _ptr(y), n, 2 * h, 2 * w, c, _stream()), "up2_fwd")
        ctx.shape = x.shape
        return y

    @staticmethod
    def backward(ctx, dy):
        n, h, w, c = ctx.shape
        dx = torch.empty(ctx.shape, dtype=dy.dtype, device=dy.device)
        _ok(_lib_nn().glnn_up2_bwd(_ptr(dy.contiguous()), _ptr(dx), n, 2 * h, 2 * w, c, _stream()), "up2_bwd")
        return dx


class WeightedMSE(torch.autograd.Function):
    """sum_c cw[c] (pred[..., c] - target[..., c])^2 / npix over the first ct channels."""

    @staticmethod
    def forward(ctx, pred, target, cw):
        n, h, w, cp = pred.shape
        ct = target.shape[3]
        npix = n * h * w
        dpred = torch.empty_like(pred)
        loss = torch.empty((1,), dtype=torch.float32, device=pred.device)
        work = torch.empty((1024,), dtype=torch.float32, device=pred.device)
        _ok(_lib_nn().glnn_mse(_ptr(pred), cp, _ptr(target), ct, _ptr(cw), _ptr(dpred), _ptr(loss), _ptr(work), npix,
                               _stream()), "mse")
        ctx.save_for_backward(dpred)
        return loss[0]

    @staticmethod
    def backward(ctx, g):
        (dpred,) = ctx.saved_tensors
        return dpred * g.to(dpred.dtype), None, None


def adam_step(params, grads, m, v, step, lr=1e-3, beta1=0.9, beta2=0.999, eps=1e-8, weight_decay=0.0):
    lib = _lib_nn()
    s = _stream()
    for p, g, mm, vv in zip(params, grads, m, v):
        _ok(lib.glnn_adam(_ptr(p), _ptr(g), _ptr(mm), _ptr(vv), p.numel(), lr, beta1, beta2, eps, weight_decay,
                          int(step), s), "adam")


# ---------------------------------------------------------------------------
# the network
# ---------------------------------------------------------------------------

class WarmStartNet:
    """The encoder-decoder (parameters as float32 device tensors)."""

    def __init__(self, device="cuda", seed=0, levels=LEVELS):
        self.levels = tuple(levels)
        c0, c1, c2, c3 = self.levels
        self.spec = [("e0a", CIN, c0), ("e0b", c0, c0), ("e1a", c0, c1), ("e1b", c1, c1), ("e2a", c1, c2),
                     ("e2b", c2, c2), ("m_a", c2, c3), ("m_b", c3, c3), ("d2a", c3 + c2, c2), ("d2b", c2, c2),
                     ("d1a", c2 + c1, c1), ("d1b", c1, c1), ("d0a", c1 + c0, c0), ("d0b", c0, c0),
                     ("out", c0, COUT)]
        gen = torch.Generator().manual_seed(seed)
        self.w, self.b = {}, {}
        for name, ci, co in self.spec:
            std = math.sqrt(2.0 / (9 * ci)) if name != "out" else 0.1 * math.sqrt(1.0 / (9 * ci))
            self.w[name] = (torch.randn((co, 3, 3, ci), generator=gen) * std).to(device).requires_grad_()
            self.b[name] = torch.zeros((co,), device=device).requires_grad_()
        self.params = [t for name, _, _ in self.spec for t in (self.w[name], self.b[name])]
        self.m = [torch.zeros_like(p) for p in self.params]
        self.v = [torch.zeros_like(p) for p in self.params]
        self.step = 0

    def n_params(self):
        return sum(p.numel() for p in self.params)

    def _c(self, name, x1, x2=None, relu=True):
        return Conv3x3.apply(x1, x2, self.w[name], self.b[name], relu)

    def forward(self, x):
        """x: (N, H, W, 8) bf16 with H, W multiples of 8 -> (N, H, W, 8) bf16."""
        e0 = self._c("e0b", self._c("e0a", x))
        e1 = self._c("e1b", self._c("e1a", Pool2.apply(e0)))
        e2 = self._c("e2b", self._c("e2a", Pool2.apply(e1)))
        m = self._c("m_b", self._c("m_a", Pool2.apply(e2)))
        d2 = self._c("d2b", self._c("d2a", Up2.apply(m), e2))
        d1 = self._c("d1b", self._c("d1a", Up2.apply(d2), e1))
        d0 = self._c("d0b", self._c("d0a", Up2.apply(d1), e0))
        return self._c("out", d0, relu=False)

    def train_step(self, x, target, cw, lr=1e-3, weight_decay=0.0):
        """One Adam step on a batch; returns the loss tensor (device)."""
        pred = self.forward(x)
        loss = WeightedMSE.apply(pred, target, cw)
        grads = torch.autograd.grad(loss, self.params)
        self.step += 1
        adam_step(self.params, [g.contiguous() for g in grads], self.m, self.v, self.step, lr=lr,
                  weight_decay=weight_decay)
        check_kernel_errors()
        return loss.detach()

    @torch.no_grad()
    def predict(self, x):
        y = self.forward(x)
        check_kernel_errors()
        return y

    def state_dict(self):
        return {name: (self.w[name].detach().cpu().numpy(), self.b[name].detach().cpu().numpy())
                for name, _, _ in self.spec}

    def load_state_dict(self, sd):
        with torch.no_grad():
            for name, _, _ in self.spec:
                self.w[name].copy_(torch.from_numpy(sd[name][0]))
                self.b[name].copy_(torch.from_numpy(sd[name][1]))


# ---------------------------------------------------------------------------
# instances, features, targets
# ---------------------------------------------------------------------------

def holes_mask(n_side, dx, frac, rmin, rmax, rng):
    """Cells (Nxc x Nyc, [i, j]) outside circular holes of radii U[rmin, rmax] at
    uniform positions, added until at least `frac` of the cells are removed."""
    nc = n_side - 1
    L = dx * nc
    mt = np.ones((nc, nc), dtype=bool)
    xc = (np.arange(nc) + 0.5) * dx
    removed, target = 0, frac * nc * nc
    while removed < target:
        cx, cy = rng.random(2) * L
        r = rmin + (rmax - rmin) * rng.random()
        rc = int(np.ceil(r / dx)) + 1
        i0, j0 = int(cx / dx), int(cy / dx)
        il, ih, jl, jh = max(0, i0 - rc), min(nc, i0 + rc + 1), max(0, j0 - rc), min(nc, j0 + rc + 1)
        sub = (xc[il:ih, None] - cx) ** 2 + (xc[None, jl:jh] - cy) ** 2 < r * r
        before = mt[il:ih, jl:jh].sum()
        mt[il:ih, jl:jh] &= ~sub
        removed += before - mt[il:ih, jl:jh].sum()
    return mt


def node_mask(mt):
    """Node (Nx x Ny, [i, j]) is superconducting iff one of its cells is (svirl/mesh/grid.py:160-171)."""
    nc0, nc1 = mt.shape
    m = np.zeros((nc0 + 1, nc1 + 1), dtype=bool)
    m[:-1, :-1] |= mt
    m[1:, :-1] |= mt
    m[:-1, 1:] |= mt
    m[1:, 1:] |= mt
    return m


def landau_ab(Nx, Ny, dx, dy, H):
    """A = (a = -H y_j, b = 0), flat [a (i + (Nx-1) j) | b]."""
    y = dy * np.arange(Ny)
    a = np.repeat(-H * y, Nx - 1)
    return np.concatenate([a, np.zeros(Nx * (Ny - 1))])


def random_psi(N, rng):
    """Amplitude U[0, 1), phase U[0, 2 pi) (the reference's 'random' start, seeded)."""
    return (1.0 - rng.random(N)) * np.exp(1j * np.pi * (2.0 * rng.random(N) - 1.0))


class Instance:
    """One sampled GL problem on an n x n node grid (finite kappa or kappa = inf)."""

    def __init__(self, n, dx, H, kappa, mt, psi0, sigma=200.0):
        self.n, self.dx, self.H, self.kappa, self.mt, self.psi0 = n, dx, H, kappa, mt, psi0
        self.sigma = sigma  # normal conductivity: only the TDGL A equation uses it
        self.nm = node_mask(mt)
        self.ab0 = landau_ab(n, n, dx, dx, H)

    @staticmethod
    def sample(n, rng, dx=0.5, H_range=(0.02, 0.5), kappa_range=(2.0, 10.0), hole_frac=(0.0, 0.05),
               radius=(2.0, 6.0), kappa_inf_prob=0.0):
        H = H_range[0] + (H_range[1] - H_range[0]) * rng.random()
        kappa = np.inf if rng.random() < kappa_inf_prob else kappa_range[0] + (kappa_range[1] - kappa_range[0]) * rng.random()
        frac = hole_frac[0] + (hole_frac[1] - hole_frac[0]) * rng.random()
        mt = holes_mask(n, dx, frac, radius[0], radius[1], rng)
        psi0 = random_psi(n * n, rng)
        return Instance(n, dx, H, kappa, mt, psi0)

    def load_into(self, h, psi=None, ab=None):
        """Parameters, mask and state (psi0 and the Landau gauge unless given) into a handle."""
        k = self.kappa if np.isfinite(self.kappa) else np.inf
        h.set_params(kappa=float(k), H=float(self.H), sigma=float(self.sigma), epsilon=1.0)
        h.set_mask(self.mt.T.reshape(-1).astype(np.uint8))  # cell i + (Nx-1) j
        h.set_psi(self.psi0 if psi is None else psi)
        h.set_ab(self.ab0 if ab is None else ab)


def features(insts, device="cuda"):
    """(N, n, n, 8) bf16 inputs of a list of instances of one size."""
    n = insts[0].n
    x = np.zeros((len(insts), n, n, CIN), dtype=np.float32)
    for q, it in enumerate(insts):
        p = it.psi0.reshape(n, n)  # [j, i]
        x[q, :, :, 0] = it.nm.T
        x[q, :, :, 1] = it.H
        x[q, :, :, 2] = 0.0 if not np.isfinite(it.kappa) else 1.0 / it.kappa
        x[q, :, :, 3] = p.real
        x[q, :, :, 4] = p.imag
    return torch.from_numpy(x).to(device=device, dtype=torch.bfloat16)


def targets(insts, psis, abs_, device="cuda", mode="amplitude"):
    """(N, n, n, 4) float32 targets [Re psi, Im psi, delta a, delta b] ("full") or
    [|psi|, 0, delta a, delta b] ("amplitude") from relaxed states."""
    n = insts[0].n
    t = np.zeros((len(insts), n, n, NOUT), dtype=np.float32)
    na = (n - 1) * n
    for q, (it, psi, ab) in enumerate(zip(insts, psis, abs_)):
        p = np.asarray(psi).reshape(n, n)
        if mode == "full":
            t[q, :, :, 0] = p.real
            t[q, :, :, 1] = p.imag
        else:
            t[q, :, :, 0] = np.abs(p)
        if np.isfinite(it.kappa):
            d = np.asarray(ab, dtype=np.float64) - it.ab0
            t[q, :, :-1, 2] = d[:na].reshape(n, n - 1)
            t[q, :-1, :, 3] = d[na:].reshape(n - 1, n)
    return torch.from_numpy(t).to(device)


def decode(insts, pred, mode="amplitude"):
    """Predicted (psi, ab) per instance (host arrays) from the network output."""
    out = pred.float().cpu().numpy()
    res = []
    n = insts[0].n
    na = (n - 1) * n
    for q, it in enumerate(insts):
        if mode == "full":
            psi = (out[q, :, :, 0] + 1j * out[q, :, :, 1]) * it.nm.T
        else:
            p0 = it.psi0.reshape(n, n)
            psi = np.maximum(out[q, :, :, 0], 0.0) * np.exp(1j * np.angle(p0)) * it.nm.T
        ab = it.ab0.copy()
        if np.isfinite(it.kappa):
            ab[:na] += out[q, :, :-1, 2].reshape(-1)
            ab[na:] += out[q, :-1, :, 3].reshape(-1)
        res.append((psi.reshape(-1), ab))
    return res


# ---------------------------------------------------------------------------
# dataset generation and evaluation with the batched device CG
# ---------------------------------------------------------------------------

class Pool:
    """A fixed set of library handles of one size and dtype, reused batch after batch."""

    def __init__(self, n, count, dtype=np.float32, dx=0.5, device=0):
        self.n, self.dx, self.dtype = n, dx, np.dtype(dtype)
        self.handles = [_lib.Handle(n, n, dx, dx, dtype, device=device) for _ in range(count)]
        from .batch import HandleBatch
        self.batch = HandleBatch(self.handles)

    def close(self):
        self.batch.close()
        for h in self.handles:
            h.close()

    def relax(self, insts, starts=None, n_iter=2000, gtol=1e-4, gtol_abs=True, rtol=0.0, timed=False):
        """Batched device CG (exact boundary gradient) of `insts` from their random
        start or from `starts` [(psi, ab)]; returns (out dict, [(psi, ab)])."""
        assert len(insts) <= len(self.handles)
        hs = self.handles[:len(insts)]
        for q, (it, h) in enumerate(zip(insts, hs)):
            if starts is None:
                it.load_into(h)
            else:
                it.load_into(h, psi=starts[q][0], ab=starts[q][1])
        from .batch import HandleBatch
        batch = self.batch if len(insts) == len(self.handles) else HandleBatch(hs)
        try:
            out = batch.cg_device(n_iter=n_iter, rtol=rtol, gtol=gtol, exact_boundary=True, gtol_abs=gtol_abs,
                                  timed=timed)
        finally:
            if batch is not self.batch:
                batch.close()
        states = [(h.get_psi(), h.get_ab()) for h in hs]
        return {k: (v[:len(insts)] if isinstance(v, np.ndarray) else v) for k, v in out.items()}, states


def generate(n_samples, n=128, seed=0, pool_size=256, n_iter=3000, gtol=1e-4, device="cuda", mode="amplitude",
             **sample_kw):
    """Relaxed states of `n_samples` sampled instances (device tensors x, y)."""
    rng = np.random.default_rng(seed)
    pool = Pool(n, pool_size)
    xs, ys, info = [], [], []
    try:
        for start in range(0, n_samples, pool_size):
            insts = [Instance.sample(n, rng, **sample_kw) for _ in range(min(pool_size, n_samples - start))]
            out, states = pool.relax(insts, n_iter=n_iter, gtol=gtol)
            xs.append(features(insts, device))
            ys.append(targets(insts, [s[0] for s in states], [s[1] for s in states], device, mode=mode))
            info.append(out)
    finally:
        pool.close()
    return torch.cat(xs), torch.cat(ys), info


def channel_weights(y):
    """Loss weights 1/variance of each target channel, 0 for a constant channel
    (float32 device tensor)."""
    var = y.float().reshape(-1, y.shape[-1]).var(dim=0)
    w = torch.where(var > 1e-10, 1.0 / var.clamp_min(1e-10), torch.zeros_like(var))
    return w.to(torch.float32).contiguous()


def train(net, x, y, epochs=5, batch=32, lr=1e-3, seed=0, log=None):
    """Adam over shuffled mini-batches; returns the mean loss of each epoch."""
    cw = channel_weights(y)
    gen = torch.Generator(device="cpu").manual_seed(seed)
    hist = []
    for ep in range(epochs):
        perm = torch.randperm(x.shape[0], generator=gen)
        tot, cnt = 0.0, 0
        for s in range(0, x.shape[0] - batch + 1, batch):
            idx = perm[s:s + batch].to(x.device)
            loss = net.train_step(x[idx].contiguous(), y[idx].contiguous(), cw, lr=lr)
            tot += float(loss)
            cnt += 1
        hist.append(tot / max(cnt, 1))
        if log:
            log("epoch %d loss %.5f" % (ep, hist[-1]))
    return hist


def reference_energies(insts, cache, n_iter=20000, gtol=1e-7, starts=None):
    """F*: the FP64 energy of a tight relaxation of each instance from its random
    start, or from `starts` (list of (psi, ab))."""
    from .relax import relax
    ref, _, _ = relax(insts, cache, np.float64, starts=starts, n_iter=n_iter, gtol=gtol, fetch=False)
    return ref["energy"]


def evaluate(net, insts, mode="amplitude", dtype=np.float64, n_iter=20000, gtol=1e-7, tol=1e-6, cache=None,
             Estar=None):
    """What the network gains, in CG iterations and device time, measured two ways.

    Own minimum (the states/s criterion): the CG from the random start run until it
    is within `tol` of F*_random (a tight FP64 relaxation from the random start), the
    CG from the prediction until it is within `tol` of F*_pred (a tight FP64
    relaxation from the prediction).  The CG is monotone in the energy and F* is
    where the same arithmetic ends, so reaching the band means the run reached its
    minimum: `iters_*_own_median`, `reached_*_own`.

    The random start's minimum (strict): a prediction reaches F*_random only if its
    own minimum is F*_random (|F*_pred - F*_random| <= tol |F*_random|); its
    iterations are those to enter the band.  An energy that passes through the band
    on the way to a lower minimum does not count.  `reached_warm`, `reached_both`,
    `iters_*_median_both`; `warm_lower_energy` counts the predictions whose minimum
    is lower than F*_random (another vortex configuration).

    The random start's energy level: iterations until the energy first falls to
    F*_random + tol |F*_random| (any state), from both starts, on the instances where
    both get there: `iters_*_level_median`."""
    import time as _time
    from .relax import HandleCache, relax
    own = cache is None
    cache = HandleCache() if own else cache
    try:
        if Estar is None:
            Estar = reference_energies(insts, cache, n_iter=n_iter, gtol=gtol)
        r, _, _ = relax(insts, cache, dtype, n_iter=n_iter, gtol=0.0, fetch=False, targets=Estar, target_tol=tol)
        torch.cuda.synchronize()
        t0 = _time.perf_counter()
        pred = net.predict(features(insts))
        torch.cuda.synchronize()
        t_net = _time.perf_counter() - t0
        starts = decode(insts, pred, mode=mode)
        Epred = reference_energies(insts, cache, n_iter=n_iter, gtol=gtol, starts=starts)
        w, _, _ = relax(insts, cache, dtype, starts=starts, n_iter=n_iter, gtol=0.0, fetch=False, targets=Estar,
                        target_tol=tol)
        wo, _, _ = relax(insts, cache, dtype, starts=starts, n_iter=n_iter, gtol=0.0, fetch=False, targets=Epred,
                         target_tol=tol)
    finally:
        if own:
            cache.close()
    lo = Estar - tol * np.abs(Estar)
    ok_r = (r["status"] == 4) & (r["energy"] >= lo)
    same_min = np.abs(Epred - Estar) <= tol * np.abs(Estar)
    ok_w = (w["status"] == 4) & same_min
    both = ok_r & ok_w
    ok_wo = (wo["status"] == 4) & (wo["energy"] >= Epred - tol * np.abs(Epred))
    lvl = (r["status"] == 4) & (w["status"] == 4)
    med = lambda x: float(np.median(x)) if x.size else float("nan")  # noqa: E731
    return {"n": len(insts), "size": insts[0].n,
            "reached_random_own": int(ok_r.sum()), "reached_warm_own": int(ok_wo.sum()),
            "iters_random_own_median": med(r["iters"][ok_r]), "iters_warm_own_median": med(wo["iters"][ok_wo]),
            "cg_ms_random_own": r["ms"], "cg_ms_warm_own": wo["ms"],
            "reached_random": int(ok_r.sum()), "reached_warm": int(ok_w.sum()), "reached_both": int(both.sum()),
            "iters_random_median_both": med(r["iters"][both]), "iters_warm_median_both": med(w["iters"][both]),
            "reached_level_both": int(lvl.sum()), "iters_random_level_median": med(r["iters"][lvl]),
            "iters_warm_level_median": med(w["iters"][lvl]),
            "net_ms": 1e3 * t_net,
            "warm_lower_energy": int((Epred < lo).sum()), "warm_higher_energy": int((Epred > Estar + tol * np.abs(Estar)).sum())}


def states_throughput(net, insts, Estar, cache, cap=4000, gtol=1e-4, tol=1e-6, plain_sample=8, mode="amplitude",
                      rtol=0.0, gtol_abs=True, dtypes=(np.float32, np.float64)):
    """Relaxed states per second, the learned + batched method against the plain
    one, with one stop rule for both (gradient norm `gtol`, absolute or relative to
    the first iteration's, energy ratio `rtol`, or `cap` iterations) and one
    criterion: a state counts when |F - F*|/|F*| <= tol, F* the FP64 energy of a
    tight relaxation of the same instance from the same initial state (the random
    start for the plain arm, `Estar`; the network's prediction for the learned arm,
    computed here before the timed runs).  Against the random start's F* the
    learned states are also counted (`ok_vs_random_start`), and those that end
    below it, in another (lower) vortex minimum, reported (`lower_energy`).
    Learned + batched (timed end to end), once per CG precision in `dtypes`:
    features to the device, the network's prediction, decoding, the predicted
    states into the handles, the batched device CG of all instances, the states
    back to the host.  FP32 trajectories leave the FP64 one of the same start at
    bifurcations and can end in another minimum; the FP64 arm follows the
    arithmetic of F*.  Plain: the same device CG on one instance at a time in FP64
    from its random start, on the first `plain_sample` instances.  Returns the
    first precision's numbers at the top level and every precision under
    "by_dtype"."""
    import time as _time
    from .relax import energies_fp64, relax
    # untimed: F* of each predicted start (the prediction is deterministic)
    starts0 = decode(insts, net.predict(features(insts)), mode=mode)
    Estar_pred = reference_energies(insts, cache, starts=starts0)
    t_plain, ok_plain, low_plain = 0.0, 0, 0
    for q, it in enumerate(insts[:plain_sample]):
        t1 = _time.perf_counter()
        _, st, _ = relax([it], cache, np.float64, n_iter=cap, gtol=gtol, gtol_abs=gtol_abs, rtol=rtol)
        t_plain += _time.perf_counter() - t1
        r1 = (energies_fp64([it], st, cache)[0] - Estar[q]) / abs(Estar[q])
        ok_plain += int(abs(r1) <= tol)
        low_plain += int(r1 < -tol)
    plain_rate = ok_plain / t_plain if t_plain > 0 else 0.0
    plain = {"states_per_s": plain_rate, "ok": ok_plain, "sample": min(plain_sample, len(insts)),
             "lower_energy": low_plain, "wall_s": t_plain}
    by = {}
    for dt in dtypes:
        torch.cuda.synchronize()
        t0 = _time.perf_counter()
        pred = net.predict(features(insts))
        starts = decode(insts, pred, mode=mode)
        out, states, _ = relax(insts, cache, dt, starts=starts, n_iter=cap, gtol=gtol, gtol_abs=gtol_abs, rtol=rtol)
        wall = _time.perf_counter() - t0
        E = energies_fp64(insts, states, cache)
        rel_pred = (E - Estar_pred) / np.abs(Estar_pred)
        rel = (E - Estar) / np.abs(Estar)
        ok = int((np.abs(rel_pred) <= tol).sum())
        rate = ok / wall
        by[np.dtype(dt).name] = {
            "states_per_s": rate, "ok": ok, "n": len(insts), "wall_s": wall, "cg_ms": out["ms"],
            "cg_iters_median": float(np.median(out["iters"])),
            "ok_vs_random_start": int((np.abs(rel) <= tol).sum()), "lower_energy": int((rel < -tol).sum()),
            "rel_err_quantiles": np.quantile(rel_pred, [0, 0.5, 0.9, 1]).tolist(),
            "rel_err_vs_random_start_quantiles": np.quantile(rel, [0, 0.5, 0.9, 1]).tolist(),
            "speedup_vs_plain": rate / plain_rate if plain_rate > 0 else None}
    first = dict(by[np.dtype(dtypes[0]).name])
    first.update({"plain": plain, "by_dtype": by, "cap": cap, "gtol": gtol, "gtol_abs": gtol_abs, "rtol": rtol})
    return first
