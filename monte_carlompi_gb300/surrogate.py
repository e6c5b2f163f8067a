"""BRF surrogate: an MLP from (r_eff, lambda, cos theta0, depth) to the 648-bin BRF and albedo.

The reference's only route to a BRF is the Monte Carlo walk followed by the
histogram arithmetic of post_processing.py:46-100.  This module learns that map
from walks the GPU walk itself produces, so a BRF can be predicted in
microseconds; plain Monte Carlo stays the fallback outside the training hull or
where the ensemble disagrees, and the judge of the network's error.

Network: 4 -> 256 -> 256 -> 256 -> 649, SiLU, BF16 weights and activations on
tensor cores with FP32 accumulation (include/mcw_mlp.h: inference is one fused
tcgen05 kernel with tensor-memory accumulators whose hidden activations never leave
shared memory; training runs layer-by-layer GEMMs that keep the pre-activations for
the backward pass), FP32 master weights and Adam.  ``MLPFunction`` is the torch.autograd.Function whose forward and backward
run those kernels; inputs and outputs are torch CUDA tensors, PyTorch is only the
container.  Targets are standardised log(BRF / albedo + 0.02) per bin and
log(albedo).
"""
import ctypes
import math
from dataclasses import dataclass

import numpy as np

from . import _abi

DIMS = (4, 256, 256, 256, 649)
N_BRF = 648
BRF_FLOOR = 0.02
# training hull: the parameter ranges the surrogate is trained and judged on
R_RANGE = (50.0, 1500.0)      # r_eff [um], log-uniform
WVL_RANGE = (0.9, 1.8)        # centre wavelength [um]
MU_RANGE = (0.3, 1.0)         # cos theta0
DEPTH_RANGE = (0.01, 1.0)     # [m], log-uniform


def encode(r_eff, wvl, mu0, depth):
    """Inputs scaled to [-1, 1] over the training hull, float32 [n, 4]."""
    r = np.log(np.asarray(r_eff, np.float64))
    d = np.log(np.asarray(depth, np.float64))
    x = np.stack([
        2 * (r - math.log(R_RANGE[0])) / (math.log(R_RANGE[1]) - math.log(R_RANGE[0])) - 1,
        2 * (np.asarray(wvl, np.float64) - WVL_RANGE[0]) / (WVL_RANGE[1] - WVL_RANGE[0]) - 1,
        2 * (np.asarray(mu0, np.float64) - MU_RANGE[0]) / (MU_RANGE[1] - MU_RANGE[0]) - 1,
        2 * (d - math.log(DEPTH_RANGE[0])) / (math.log(DEPTH_RANGE[1]) - math.log(DEPTH_RANGE[0])) - 1,
    ], axis=-1)
    return x.astype(np.float32)


def in_hull(r_eff, wvl, mu0, depth):
    x = encode(r_eff, wvl, mu0, depth)
    return np.all(np.abs(x) <= 1.0 + 1e-6, axis=-1)


def to_target(brf, albedo):
    """Network target space: log(BRF / albedo + floor) per bin (the shape, about 1 on
    average) and log(albedo), so every bin keeps relative precision."""
    a = np.maximum(np.asarray(albedo, np.float64), 1e-6)
    shape = np.maximum(np.asarray(brf, np.float64), 0) / a[:, None]
    return np.concatenate([np.log(shape + BRF_FLOOR), np.log(a)[:, None]], axis=1).astype(np.float32)


def from_target(y):
    y = np.asarray(y, np.float64)
    a = np.exp(y[:, N_BRF])
    return (np.exp(y[:, :N_BRF]) - BRF_FLOOR) * a[:, None], a


# ------------------------------------------------------------------ kernels

def _stream(torch):
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def _gemm(torch, epi, m, n, k, a, lda, b, ldb, c, ldc, trans_a=0, trans_b=0, bias=None, aux=None,
          ldaux=0, c2=None, ldc2=0, engine=_abi.ENGINE_MMA_SYNC):
    g = _abi.GemmC(m, n, k, trans_a, trans_b, epi, a.data_ptr(), lda, ldb, b.data_ptr(),
                   bias.data_ptr() if bias is not None else None,
                   aux.data_ptr() if aux is not None else None, ldaux, ldc, c.data_ptr(),
                   c2.data_ptr() if c2 is not None else None, ldc2, engine)
    rc = _abi.load().mcw_mlp_gemm(ctypes.byref(g), _stream(torch))
    if rc:
        raise _abi.McwError(rc, 'mcw_mlp_gemm failed (m=%d n=%d k=%d)' % (m, n, k))


def _cast(torch, x):
    y = torch.empty(x.shape, dtype=torch.bfloat16, device=x.device)
    rc = _abi.load().mcw_mlp_cast_bf16(_ptr(x), _ptr(y), x.numel(), _stream(torch))
    if rc:
        raise _abi.McwError(rc, 'mcw_mlp_cast_bf16 failed')
    return y


def _colsum(torch, g):
    m, n = g.shape
    out = torch.empty(n, dtype=torch.float32, device=g.device)
    rc = _abi.load().mcw_mlp_colsum(_ptr(g), m, n, n, _ptr(out), _stream(torch))
    if rc:
        raise _abi.McwError(rc, 'mcw_mlp_colsum failed')
    return out


# engine of training's GEMMs (forward with kept pre-activations, and the backward
# layouts: transposed operands, silu' epilogue); inference runs the fused tcgen05
# kernel (forward_fused)
TRAIN_ENGINE = _abi.ENGINE_TCGEN05


def pack_weights(torch, w16):
    """All four weight matrices in the tensor-core operand layout of mcw_mlp_forward."""
    blob = torch.empty(_abi.MLP_PACK_BYTES, dtype=torch.uint8, device=w16[0].device)
    rc = _abi.load().mcw_mlp_pack(_ptr(w16[0]), _ptr(w16[1]), _ptr(w16[2]), _ptr(w16[3]), _ptr(blob),
                                  _stream(torch))
    if rc:
        raise _abi.McwError(rc, 'mcw_mlp_pack failed')
    return blob


# row pitch of the fused kernel's output: 649 values rounded up to 16 bytes (its
# 16-byte stores): 652 floats or 656 halves
Y_PITCH = 652
Y_PITCH_F16 = 656


def forward_fused(torch, x, w16, biases, blob, half=False):
    """Inference of the whole network in one kernel (mcw_mlp_forward, or
    mcw_mlp_forward_f16 with half=True: outputs rounded to fp16, half the bytes);
    x float32 [m, 4]; returns a [m, 649] view of the output rows."""
    x = x.contiguous().float()
    m = x.shape[0]
    pitch = Y_PITCH_F16 if half else Y_PITCH
    y = torch.empty((m, pitch), dtype=torch.float16 if half else torch.float32, device=x.device)
    b = [t.contiguous() for t in biases]
    fn = _abi.load().mcw_mlp_forward_f16 if half else _abi.load().mcw_mlp_forward
    rc = fn(_ptr(x), m, _ptr(b[0]), _ptr(b[1]), _ptr(b[2]), _ptr(b[3]), _ptr(blob), _ptr(y), pitch, _stream(torch))
    if rc:
        raise _abi.McwError(rc, 'mcw_mlp_forward failed (m=%d)' % m)
    return y[:, :DIMS[-1]]


def forward_ensemble(torch, x, blob, bias, members):
    """Inference of an ensemble's members on the same inputs in one launch
    (mcw_mlp_forward_ensemble_f16): blob holds the members' packed weights one after the
    other (members x MLP_PACK_BYTES), bias their biases (float32 [members, 1417], b1 | b2 |
    b3 | b4); returns fp16 [members, m, 649] views of the output rows, each member's equal
    to forward_fused(half=True) of that member."""
    x = x.contiguous().float()
    m = x.shape[0]
    y = torch.empty((members, m, Y_PITCH_F16), dtype=torch.float16, device=x.device)
    rc = _abi.load().mcw_mlp_forward_ensemble_f16(_ptr(x), m, members, _ptr(bias), _ptr(blob), _ptr(y),
                                                  Y_PITCH_F16, _stream(torch))
    if rc:
        raise _abi.McwError(rc, 'mcw_mlp_forward_ensemble_f16 failed (m=%d, members=%d)' % (m, members))
    return y[:, :, :DIMS[-1]]


def forward_cached(torch, x16, w16, biases, keep=True):
    """Forward pass on the tensor-core kernels; returns (y fp32, cache for backward).
    keep=False (inference) skips storing the FP32 pre-activations."""
    m = x16.shape[0]
    a = x16
    zs, acts = [], [x16]
    for layer in range(3):
        n, k = w16[layer].shape
        z = torch.empty((m, n), dtype=torch.float32, device=x16.device) if keep else None
        nxt = torch.empty((m, n), dtype=torch.bfloat16, device=x16.device)
        _gemm(torch, _abi.EPI_BIAS_SILU, m, n, k, a, k, w16[layer], k, nxt, n, bias=biases[layer],
              c2=z, ldc2=n, engine=TRAIN_ENGINE)
        zs.append(z)
        acts.append(nxt)
        a = nxt
    n, k = w16[3].shape
    y = torch.empty((m, n), dtype=torch.float32, device=x16.device)
    _gemm(torch, _abi.EPI_BIAS_F32, m, n, k, a, k, w16[3], k, y, n, bias=biases[3], engine=TRAIN_ENGINE)
    return y, (zs, acts)


def backward_cached(torch, gy, w16, cache, need_dx=True):
    """Backward pass: gradients of the weights, biases and (optionally) the input."""
    zs, acts = cache
    m = gy.shape[0]
    g32 = gy.contiguous().float()
    g16 = _cast(torch, g32)
    dws, dbs = [None] * 4, [None] * 4
    for layer in (3, 2, 1, 0):
        n_out, k_in = w16[layer].shape
        a_in = acts[layer]
        dw = torch.empty((n_out, k_in), dtype=torch.float32, device=gy.device)
        # dW[o, i] = sum_b G[b, o] A[b, i]
        _gemm(torch, _abi.EPI_F32, n_out, k_in, m, g16, n_out, a_in, k_in, dw, k_in, trans_a=1, trans_b=1,
              engine=TRAIN_ENGINE)
        dws[layer] = dw
        dbs[layer] = _colsum(torch, g32)
        if layer == 0:
            if not need_dx:
                return None, dws, dbs
            dx = torch.empty((m, k_in), dtype=torch.float32, device=gy.device)
            _gemm(torch, _abi.EPI_F32, m, k_in, n_out, g16, n_out, w16[layer], k_in, dx, k_in, trans_b=1,
                  engine=TRAIN_ENGINE)
            return dx, dws, dbs
        # G_prev[b, i] = (sum_o G[b, o] W[o, i]) * silu'(Z_prev[b, i])
        g16_prev = torch.empty((m, k_in), dtype=torch.bfloat16, device=gy.device)
        g32_prev = torch.empty((m, k_in), dtype=torch.float32, device=gy.device)
        _gemm(torch, _abi.EPI_DSILU, m, k_in, n_out, g16, n_out, w16[layer], k_in, g16_prev, k_in,
              trans_b=1, aux=zs[layer - 1], ldaux=k_in, c2=g32_prev, ldc2=k_in, engine=TRAIN_ENGINE)
        g16, g32 = g16_prev, g32_prev


def forward_tangent(torch, x16, xdot16, w16, biases):
    """Network outputs and their directional derivative along the input tangent xdot,
    in one forward pass on the tensor-core kernels (forward mode: 4 more GEMMs, not one
    backward pass per output).  x16, xdot16 bf16 [n, 4]; returns (y, ydot) fp32 [n, 649].
    Per layer: hdot_l = (hdot_{l-1} W_l^T) * silu'(z_l), the SiLU' epilogue of the backward
    GEMMs with the pre-activations z_l of the forward pass; ydot = hdot_3 W_4^T."""
    y, (zs, _) = forward_cached(torch, x16, w16, biases, keep=True)
    m = x16.shape[0]
    t = xdot16
    for layer in range(3):
        n, k = w16[layer].shape
        nxt = torch.empty((m, n), dtype=torch.bfloat16, device=x16.device)
        _gemm(torch, _abi.EPI_DSILU, m, n, k, t, k, w16[layer], k, nxt, n, aux=zs[layer], ldaux=n)
        t = nxt
    n, k = w16[3].shape
    ydot = torch.empty((m, n), dtype=torch.float32, device=x16.device)
    _gemm(torch, _abi.EPI_F32, m, n, k, t, k, w16[3], k, ydot, n)
    return y, ydot


def _mlp_function():
    import torch

    class MLPFunction(torch.autograd.Function):
        """y = MLP(x) on the BF16 tensor-core kernels; params are FP32 masters
        (W1, b1, ..., W4, b4).  Backward returns FP32 gradients for x and every
        parameter."""

        @staticmethod
        def forward(ctx, x, *params):
            ws, bs = params[0::2], params[1::2]
            w16 = [_cast(torch, w.contiguous()) for w in ws]
            x16 = _cast(torch, x.contiguous().float())
            y, cache = forward_cached(torch, x16, w16, [b.contiguous() for b in bs])
            ctx.save_for_backward(*w16, *cache[0], *cache[1])
            return y

        @staticmethod
        def backward(ctx, gy):
            saved = ctx.saved_tensors
            w16, zs, acts = list(saved[:4]), list(saved[4:7]), list(saved[7:11])
            dx, dws, dbs = backward_cached(torch, gy, w16, (zs, acts), need_dx=ctx.needs_input_grad[0])
            out = [dx]
            for dw, db in zip(dws, dbs):
                out += [dw, db]
            return tuple(out)

    return MLPFunction


_MLP_FN = None


def mlp_apply(x, params):
    global _MLP_FN
    if _MLP_FN is None:
        _MLP_FN = _mlp_function()
    return _MLP_FN.apply(x, *params)


# ------------------------------------------------------------------ model

class SurrogateMLP:
    """One network: FP32 master weights, BF16 copies, Adam moments (torch CUDA tensors)."""

    def __init__(self, seed=0, device='cuda'):
        import torch
        self.torch = torch
        g = torch.Generator(device='cpu').manual_seed(int(seed))
        self.params = []
        for fan_in, fan_out in zip(DIMS[:-1], DIMS[1:]):
            bound = math.sqrt(6.0 / fan_in) if fan_out != DIMS[-1] else math.sqrt(3.0 / fan_in)
            w = (torch.rand((fan_out, fan_in), generator=g) * 2 - 1) * bound
            self.params += [w.to(device), torch.zeros(fan_out, device=device)]
        self.m = [torch.zeros_like(p) for p in self.params]
        self.v = [torch.zeros_like(p) for p in self.params]
        self.w16 = [_cast(torch, w) for w in self.params[0::2]]
        self.step = 0
        self.y_mean = None
        self.y_std = None
        self._blob = None
        self._blob_key = None

    def packed(self):
        """Packed weights for the fused inference kernel, rebuilt when the weights change."""
        key = (self.step, tuple(w.data_ptr() for w in self.w16))
        if self._blob is None or self._blob_key != key:
            self._blob = pack_weights(self.torch, self.w16)
            self._blob_key = key
        return self._blob

    def predict_std(self, x, half=True):
        """Standardised outputs for encoded inputs x (torch CUDA float32 [n, 4]) from the
        fused inference kernel; fp16 by default (its rounding, 2^-11 relative, is below the
        network's bf16 activations), float32 with half=False."""
        return forward_fused(self.torch, x, self.w16, self.params[1::2], self.packed(), half=half)

    def train_step(self, x16, t, w_out, lr=1e-3, beta1=0.9, beta2=0.999, eps=1e-8):
        """One Adam step on a batch (x16 bf16 [b, 4], t fp32 standardised targets)."""
        torch = self.torch
        m = x16.shape[0]
        y, cache = forward_cached(torch, x16, self.w16, self.params[1::2])
        n = y.shape[1]
        grad = torch.empty_like(y)
        grad16 = torch.empty((m, n), dtype=torch.bfloat16, device=y.device)
        loss = torch.zeros(1, dtype=torch.float32, device=y.device)
        L = _abi.load()
        rc = L.mcw_mlp_loss(_ptr(y), n, _ptr(t), n, _ptr(w_out), m, n, _ptr(grad), n, _ptr(grad16), n,
                            _ptr(loss), _stream(torch))
        if rc:
            raise _abi.McwError(rc, 'mcw_mlp_loss failed')
        _, dws, dbs = backward_cached(torch, grad, self.w16, cache, need_dx=False)
        self.step += 1
        grads = []
        for dw, db in zip(dws, dbs):
            grads += [dw, db]
        for i, (p, gr) in enumerate(zip(self.params, grads)):
            w16 = self.w16[i // 2] if i % 2 == 0 else None
            rc = L.mcw_mlp_adam(_ptr(p), _ptr(gr), _ptr(self.m[i]), _ptr(self.v[i]), _ptr(w16), p.numel(),
                                lr, beta1, beta2, eps, self.step, _stream(torch))
            if rc:
                raise _abi.McwError(rc, 'mcw_mlp_adam failed')
        return loss


# ------------------------------------------------------------------ training engine

IN_PAD = 16        # layer-1 inputs padded to 16: one 16-byte TMA row, one MMA K step
OUT_PITCH = 656    # 649 outputs rounded up to 8 (16-byte bf16 rows)


def _align8(n):
    return (n + 7) // 8 * 8


def flat_layout():
    """Layout of one member's parameters in the training engine's flat vectors.

    Returns (lay, P, tlay, T): lay['W%d'] = (offset, rows, cols) of W_l [out, in]
    (layer 1's inputs padded to IN_PAD columns, held at zero), lay['b%d'] = (offset, n);
    P elements per member; tlay['W%d'] = (offset, ld) of the transposed bf16 copy
    W_l^T [in, ld] (ld = out rounded up to 8) of W2, W3, W4, the B operands of the
    backward products; T elements per member.  Every block starts on 8 elements."""
    lay, off = {}, 0
    for layer, (fan_in, fan_out) in enumerate(zip(DIMS[:-1], DIMS[1:])):
        k = IN_PAD if layer == 0 else fan_in
        lay['W%d' % layer] = (off, fan_out, k)
        off = _align8(off + fan_out * k)
        lay['b%d' % layer] = (off, fan_out)
        off = _align8(off + fan_out)
    tlay, toff = {}, 0
    for layer in (1, 2, 3):
        _, rows, cols = lay['W%d' % layer]
        ld = _align8(rows)
        tlay['W%d' % layer] = (toff, ld)
        toff += cols * ld
    return lay, off, tlay, toff


def _dw_splits(rows):
    """Split-K of the weight-gradient products over `rows` batch rows: about 1,024 rows
    per split, at most 64 splits, in the form mcw_mlp_gemm_grouped accepts."""
    chunks = (rows + 63) // 64
    want = max(1, min(64, rows // 1024))
    per = (chunks + want - 1) // want
    return (chunks + per - 1) // per


class EnsembleTrainer:
    """Adam steps of every member of an ensemble at once on the training engine
    (include/mcw_mlp.h): per step one gather of the members' batches, the four forward
    products (bias + SiLU epilogues keeping pre-activations and transposed
    activations), the loss, the weight- and input-gradient products, the bias
    gradients, Adam over the flat parameters and the step counter, each one launch for
    all members.  Parameters live in flat [members, P] vectors (flat_layout).  The step
    is captured in a CUDA graph on first use and replayed; learning rate, step count and
    batch counter are device scalars, so the graph never changes."""

    def __init__(self, members, batch, x_all, t_all, w_out, lr=1e-3, beta1=0.9, beta2=0.999, eps=1e-8,
                 use_graph=True):
        import torch
        self.torch = torch
        self.members = members
        self.G = len(members)
        self.B = int(batch)
        self.beta1, self.beta2, self.eps = beta1, beta2, eps
        self.use_graph = use_graph
        self.graph = None
        G, B = self.G, self.B
        self.lay, self.P, self.tlay, self.T = flat_layout()
        dev = 'cuda'
        f32, bf16, i32 = torch.float32, torch.bfloat16, torch.int32
        # parameters, gradients, Adam moments and the bf16 copies (zeros in the padding)
        self.params = torch.zeros((G, self.P), dtype=f32, device=dev)
        self.m = torch.zeros_like(self.params)
        self.v = torch.zeros_like(self.params)
        self.grad = torch.zeros_like(self.params)
        for g, net in enumerate(members):
            for layer in range(4):
                o, rows, cols = self.lay['W%d' % layer]
                w = net.params[2 * layer]
                blk = self.params[g, o:o + rows * cols].view(rows, cols)
                blk[:, :w.shape[1]].copy_(w)
                ob, nb = self.lay['b%d' % layer]
                self.params[g, ob:ob + nb].copy_(net.params[2 * layer + 1])
                mw, vw = net.m[2 * layer], net.v[2 * layer]
                self.m[g, o:o + rows * cols].view(rows, cols)[:, :w.shape[1]].copy_(mw)
                self.v[g, o:o + rows * cols].view(rows, cols)[:, :w.shape[1]].copy_(vw)
                self.m[g, ob:ob + nb].copy_(net.m[2 * layer + 1])
                self.v[g, ob:ob + nb].copy_(net.v[2 * layer + 1])
        self.w16 = self.params.to(bf16)
        self.wt = torch.zeros((G, self.T), dtype=bf16, device=dev)
        for layer in (1, 2, 3):
            o, rows, cols = self.lay['W%d' % layer]
            to, ld = self.tlay['W%d' % layer]
            self.wt[:, to:to + cols * ld].view(G, cols, ld)[:, :, :rows].copy_(
                self.w16[:, o:o + rows * cols].view(G, rows, cols).transpose(1, 2))
        # data (inputs padded to IN_PAD, bf16) and the step's batch
        n_rows = x_all.shape[0]
        if n_rows < B:
            raise ValueError('fewer rows (%d) than the batch (%d)' % (n_rows, B))
        self.n_rows = n_rows
        self.x_all = torch.zeros((n_rows, IN_PAD), dtype=bf16, device=dev)
        self.x_all[:, :DIMS[0]].copy_(x_all.to(bf16))
        self.t_all = t_all.contiguous().float()
        self.w_out = w_out.contiguous().float()
        self.perm = torch.zeros((G, n_rows), dtype=i32, device=dev)
        self.counter = torch.zeros(1, dtype=i32, device=dev)
        self.step = torch.full((1,), max(int(net.step) for net in members) + 1, dtype=i32, device=dev)
        self.lr = torch.full((1,), float(lr), dtype=f32, device=dev)
        self.loss = torch.zeros(G, dtype=f32, device=dev)
        H, N = DIMS[1], DIMS[-1]
        self.x16 = torch.zeros((G, B, IN_PAD), dtype=bf16, device=dev)
        self.xt = torch.zeros((G, IN_PAD, B), dtype=bf16, device=dev)
        self.t = torch.zeros((G, B, N), dtype=f32, device=dev)
        self.h = [torch.zeros((G, B, H), dtype=bf16, device=dev) for _ in range(3)]
        self.ht = [torch.zeros((G, H, B), dtype=bf16, device=dev) for _ in range(3)]
        self.z = [torch.zeros((G, B, H), dtype=f32, device=dev) for _ in range(3)]
        self.y = torch.zeros((G, B, OUT_PITCH), dtype=f32, device=dev)
        # output gradient (pitch 656, the pad columns stay zero) and hidden-layer gradients
        self.g32 = [torch.zeros((G, B, H), dtype=f32, device=dev) for _ in range(3)] + \
                   [torch.zeros((G, B, OUT_PITCH), dtype=f32, device=dev)]
        self.g16 = [torch.zeros((G, B, H), dtype=bf16, device=dev) for _ in range(3)] + \
                   [torch.zeros((G, B, OUT_PITCH), dtype=bf16, device=dev)]
        self.gt = [torch.zeros((G, H, B), dtype=bf16, device=dev) for _ in range(3)] + \
                  [torch.zeros((G, OUT_PITCH, B), dtype=bf16, device=dev)]
        self.splits = _dw_splits(B)
        # bias gradients of large batches: rows summed in chunks of 1,024, then in order
        self.colsum_rows = 1024 if B > 2048 else 0
        n_chunks = (B + 1023) // 1024
        self.colsum_part = torch.zeros(4 * G * n_chunks * OUT_PITCH, dtype=f32, device=dev) \
            if self.colsum_rows else None
        if self.splits > 1:
            largest = max(rows * cols for (_, rows, cols) in (self.lay['W%d' % q] for q in range(4)))
            self.part = torch.zeros((self.splits, G, largest), dtype=f32, device=dev)
        self._build_calls()

    # ---- the calls of one step, built once (pointers never change)
    def _gemm(self, epi, m, n, k, a, lda, sa, b, ldb, sb, c, ldc, sc, bias=None, aux=None, ldaux=0, saux=0,
              c2=None, ldc2=0, sc2=0, ct=None, ldct=0, sct=0, splits=1, s_split=0):
        ptr = lambda t: t.data_ptr() if t is not None else None  # noqa: E731
        bias_p = bias if isinstance(bias, int) else ptr(bias)
        return _abi.GemmGroupedC(m, n, k, self.G, splits, epi, a if isinstance(a, int) else ptr(a), lda, sa,
                                 b if isinstance(b, int) else ptr(b), ldb, sb, bias_p, self.P,
                                 ptr(aux), ldaux, saux, c if isinstance(c, int) else ptr(c), ldc, sc, s_split,
                                 ptr(c2), ldc2, sc2, ptr(ct), ldct, sct)

    def _build_calls(self):
        G, B, P, T = self.G, self.B, self.P, self.T
        H, N = DIMS[1], DIMS[-1]
        lay, tlay = self.lay, self.tlay
        w16 = self.w16.data_ptr()
        wt = self.wt.data_ptr()
        par = self.params.data_ptr()
        grd = self.grad.data_ptr()
        bf, f4 = 2, 4
        fwd = []
        a, lda, sa = self.x16, IN_PAD, B * IN_PAD
        for layer in range(3):
            o, rows, cols = lay['W%d' % layer]
            ob, _ = lay['b%d' % layer]
            fwd.append(self._gemm(_abi.EPI_BIAS_SILU, B, rows, cols, a, lda, sa, w16 + o * bf, cols, P,
                                  self.h[layer], H, B * H, bias=par + ob * f4, c2=self.z[layer], ldc2=H,
                                  sc2=B * H, ct=self.ht[layer], ldct=B, sct=H * B))
            a, lda, sa = self.h[layer], H, B * H
        o, rows, cols = lay['W3']
        ob, _ = lay['b3']
        fwd.append(self._gemm(_abi.EPI_BIAS_F32, B, N, H, self.h[2], H, B * H, w16 + o * bf, H, P,
                              self.y, OUT_PITCH, B * OUT_PITCH, bias=par + ob * f4))
        self.fwd_calls = fwd
        bwd, reduce = [], []
        # gradient of layer l's output: g[l] (layer 4: g[3], pitch 656)
        acts_t = [self.xt] + self.ht          # transposed inputs of layers 1..4
        for layer in (3, 2, 1, 0):
            o, rows, cols = lay['W%d' % layer]
            gt = self.gt[layer]
            gpitch = OUT_PITCH if layer == 3 else H
            # dW_l[o, i] = sum_b G[b, o] X[b, i]: A = G^T [rows, B], B = X^T [cols, B]
            if self.splits == 1:
                bwd.append(self._gemm(_abi.EPI_F32, rows, cols, B, gt, B, gpitch * B, acts_t[layer], B,
                                      cols * B, grd + o * f4, cols, P))
            else:
                bwd.append(self._gemm(_abi.EPI_F32, rows, cols, B, gt, B, gpitch * B, acts_t[layer], B,
                                      cols * B, self.part, cols, self.part.shape[2], splits=self.splits,
                                      s_split=G * self.part.shape[2]))
                reduce.append((len(bwd) - 1, (self.part.data_ptr(), G * self.part.shape[2], self.part.shape[2],
                                              cols, grd + o * f4, P, cols, self.splits, G, rows, cols)))
            if layer == 0:
                break
            # G_{l-1} = (G_l W_l) * silu'(Z_{l-1}): A = G_l [B, gpitch], B = W_l^T [cols, ld]
            to, ld = tlay['W%d' % layer]
            bwd.append(self._gemm(_abi.EPI_DSILU, B, cols, rows, self.g16[layer], gpitch, B * gpitch,
                                  wt + to * bf, ld, T, self.g16[layer - 1], H, B * H, aux=self.z[layer - 1],
                                  ldaux=H, saux=B * H, c2=self.g32[layer - 1], ldc2=H, sc2=B * H,
                                  ct=self.gt[layer - 1], ldct=B, sct=H * B))
        self.bwd_calls = bwd
        self.reduce_after = dict(reduce)
        cols = (_abi.ColsumLayerC * 4)()
        for layer in range(4):
            ob, nb = lay['b%d' % layer]
            pitch = OUT_PITCH if layer == 3 else H
            cols[layer] = _abi.ColsumLayerC(self.g32[layer].data_ptr(), pitch, B * pitch, ob, nb, 0)
        self.colsum_layers = cols
        tb = (_abi.TransposeBlockC * 3)()
        for q, layer in enumerate((1, 2, 3)):
            o, rows, cols_ = lay['W%d' % layer]
            to, ld = tlay['W%d' % layer]
            tb[q] = _abi.TransposeBlockC(o, to, ld, rows, cols_)
        self.transpose_blocks = tb

    def _check(self, rc, what):
        if rc:
            raise _abi.McwError(rc, '%s failed' % what)

    def _launch(self, adam=True):
        """The kernels of one step on the current stream (no host synchronisation)."""
        torch = self.torch
        L = _abi.load()
        st = _stream(torch)
        G, B = self.G, self.B
        N = DIMS[-1]
        self._check(L.mcw_mlp_gather(self.x_all.data_ptr(), self.t_all.data_ptr(), self.t_all.shape[1], N,
                                     self.perm.data_ptr(), self.n_rows, self.counter.data_ptr(), B, G,
                                     self.x16.data_ptr(), B * IN_PAD, self.xt.data_ptr(), IN_PAD * B,
                                     self.t.data_ptr(), N, B * N, st), 'mcw_mlp_gather')
        for c in self.fwd_calls:
            self._check(L.mcw_mlp_gemm_grouped(ctypes.byref(c), st), 'forward GEMM')
        self.loss.zero_()
        self._check(L.mcw_mlp_loss_grouped(self.y.data_ptr(), OUT_PITCH, B * OUT_PITCH, self.t.data_ptr(), N,
                                           B * N, self.w_out.data_ptr(), G, B, N, self.g32[3].data_ptr(),
                                           OUT_PITCH, B * OUT_PITCH, self.g16[3].data_ptr(), B * OUT_PITCH,
                                           self.gt[3].data_ptr(), B, OUT_PITCH * B, self.loss.data_ptr(), st),
                    'mcw_mlp_loss_grouped')
        for i, c in enumerate(self.bwd_calls):
            self._check(L.mcw_mlp_gemm_grouped(ctypes.byref(c), st), 'backward GEMM')
            if i in self.reduce_after:
                self._check(L.mcw_mlp_reduce_splits(*self.reduce_after[i], st), 'mcw_mlp_reduce_splits')
        self._check(L.mcw_mlp_colsum_grouped(self.colsum_layers, 4, G, B, self.grad.data_ptr(), self.P,
                                             self.colsum_part.data_ptr() if self.colsum_part is not None else None,
                                             self.colsum_rows, st), 'mcw_mlp_colsum_grouped')
        if not adam:
            return
        self._check(L.mcw_mlp_adam_grouped(self.params.data_ptr(), self.grad.data_ptr(), self.m.data_ptr(),
                                           self.v.data_ptr(), self.w16.data_ptr(), self.P, G, self.lr.data_ptr(),
                                           self.step.data_ptr(), self.beta1, self.beta2, self.eps,
                                           self.wt.data_ptr(), self.T, self.transpose_blocks, 3, st),
                    'mcw_mlp_adam_grouped')
        self._check(L.mcw_mlp_advance(self.counter.data_ptr(), self.step.data_ptr(), st), 'mcw_mlp_advance')

    def set_epoch(self, perms, lr):
        """Row order of each member for the next len(rows) // batch steps, and the learning rate."""
        torch = self.torch
        self.perm.copy_(torch.as_tensor(np.asarray(perms, np.int32)))
        self.counter.zero_()
        self.lr.fill_(float(lr))

    def run_step(self):
        """One Adam step of every member (graph replay after the first)."""
        torch = self.torch
        if not self.use_graph:
            self._launch()
            return
        if self.graph is None:
            # an eager step first: one-time set-up (module loading, kernel attributes)
            # must not happen inside the capture; then undo it
            saved = [t.clone() for t in (self.params, self.m, self.v, self.w16, self.wt, self.counter, self.step)]
            self._launch()
            for t, s0 in zip((self.params, self.m, self.v, self.w16, self.wt, self.counter, self.step), saved):
                t.copy_(s0)
            torch.cuda.synchronize()
            self.graph = torch.cuda.CUDAGraph()
            with torch.cuda.graph(self.graph):
                self._launch()
        self.graph.replay()

    def gradients(self):
        """Forward and backward of the current batch without the Adam step: the
        gradients of every member as [W1, b1, ..., W4, b4] (W1 without its padding)."""
        self._launch(adam=False)
        self.torch.cuda.synchronize()
        out = []
        for g in range(self.G):
            gr = []
            for layer in range(4):
                o, rows, cols = self.lay['W%d' % layer]
                w = self.grad[g, o:o + rows * cols].view(rows, cols)
                gr.append(w[:, :DIMS[layer]].clone())
                ob, nb = self.lay['b%d' % layer]
                gr.append(self.grad[g, ob:ob + nb].clone())
            out.append(gr)
        return out

    def export(self):
        """Copy the trained parameters, moments and step count back into the members."""
        torch = self.torch
        torch.cuda.synchronize()
        step = int(self.step.item()) - 1
        for g, net in enumerate(self.members):
            for layer in range(4):
                o, rows, cols = self.lay['W%d' % layer]
                k = DIMS[layer]
                for dst, src in ((net.params, self.params), (net.m, self.m), (net.v, self.v)):
                    dst[2 * layer].copy_(src[g, o:o + rows * cols].view(rows, cols)[:, :k])
                ob, nb = self.lay['b%d' % layer]
                for dst, src in ((net.params, self.params), (net.m, self.m), (net.v, self.v)):
                    dst[2 * layer + 1].copy_(src[g, ob:ob + nb])
            net.w16 = [_cast(torch, w.contiguous()) for w in net.params[0::2]]
            net.step = step
            net._blob = None


@dataclass
class Dataset:
    x: np.ndarray        # encoded inputs [n, 4]
    y: np.ndarray        # target space [n, 649]
    raw: np.ndarray      # (r_eff, wvl, mu0, depth) [n, 4]
    brf: np.ndarray      # [n, 648]
    albedo: np.ndarray   # [n]
    photons: int


def sample_inputs(n, seed):
    rng = np.random.default_rng(seed)
    r = np.exp(rng.uniform(np.log(R_RANGE[0]), np.log(R_RANGE[1]), n))
    wvl = rng.uniform(*WVL_RANGE, n)
    mu0 = rng.uniform(*MU_RANGE, n)
    depth = np.exp(rng.uniform(np.log(DEPTH_RANGE[0]), np.log(DEPTH_RANGE[1]), n))
    return np.stack([r, wvl, mu0, depth], axis=1)


def mc_brf(walker, raw, n_photon, seed, half_width=0.085, R=0.5, chunk=1024):
    """BRF (648 bins) and albedo of each input row by the GPU walk (n_photon photons each)."""
    from . import ssp
    from .config import WalkConfig
    raw = np.asarray(raw, np.float64)
    brf = np.zeros((raw.shape[0], N_BRF))
    alb = np.zeros(raw.shape[0])
    imp = ssp.synthetic_impurity_table(600, 2100)
    for lo in range(0, raw.shape[0], chunk):
        rows = raw[lo:lo + chunk]
        tables, cfgs = [], []
        for j, (r, wvl, mu0, depth) in enumerate(rows):
            tables.append(ssp.synthetic_ice_table(r, 600, 2100))
            tau = depth * ssp.ext_cff_mss_sphere(r) * 300.0
            theta0 = math.degrees(math.acos(min(1.0, max(0.0, mu0))))
            cfgs.append(WalkConfig(n_photon=int(n_photon), wvl0=float(wvl), half_width=half_width,
                                   theta0_deg=min(theta0, 89.999), tau_tot=tau,
                                   lambertian_reflectance=R, ice_table=j, rds_snw=float(r)))
        walker.set_tables(tables, imp)
        res = walker.walk(cfgs, seed + lo, mode='f32', records=None)
        b, a = res.brf()
        brf[lo:lo + len(rows)] = b
        alb[lo:lo + len(rows)] = a
    return brf, alb


class Ensemble:
    """Members trained on the same data from different initialisations and batch orders."""

    def __init__(self, members):
        self.members = members
        self._pack = None         # (key, blob of every member's packed weights, their biases)

    def packed(self):
        """The members' packed weights one after the other and their biases as rows
        (float32 [members, 1417]), rebuilt when any member's weights change."""
        import torch
        key = tuple((m.step, tuple(w.data_ptr() for w in m.w16), tuple(b.data_ptr() for b in m.params[1::2]))
                    for m in self.members)
        if self._pack is None or self._pack[0] != key:
            blob = torch.cat([m.packed() for m in self.members])
            bias = torch.stack([torch.cat([b.float().reshape(-1) for b in m.params[1::2]]) for m in self.members])
            self._pack = (key, blob, bias.contiguous())
        return self._pack[1], self._pack[2]

    def predict_std(self, x):
        """Every member's standardised outputs for encoded inputs x (torch CUDA float32
        [n, 4]) in one launch of the fused kernel: fp16 [members, n, 649]."""
        import torch
        blob, bias = self.packed()
        return forward_ensemble(torch, x, blob, bias, len(self.members))

    def predict_members(self, raw):
        """Each member's BRF [members, n, 648] and albedo [members, n]."""
        import torch
        x = torch.from_numpy(encode(*np.asarray(raw, np.float64).T)).cuda()
        ys = self.predict_std(x)
        outs = np.stack([(ys[k].double() * m.y_std + m.y_mean).cpu().numpy()
                         for k, m in enumerate(self.members)])
        brfs, albs = zip(*[from_target(o) for o in outs])
        return np.stack(brfs), np.stack(albs)

    def predict(self, raw):
        """Mean BRF [n, 648], mean albedo [n], relative ensemble spread of the BRF [n]."""
        brfs, albs = self.predict_members(raw)
        mean_brf = brfs.mean(0)
        w = bin_weights()
        # member spread in the units of rel_rms: weighted RMS std over weighted RMS BRF
        spread = np.sqrt((brfs.std(0) ** 2 * w).sum(1) / np.maximum((mean_brf ** 2 * w).sum(1), 1e-30))
        return mean_brf, albs.mean(0), spread


def bin_weights():
    """Solid-angle weights sin(theta) cos(theta) of the 648 bins (the expected photon share)."""
    mids = (np.arange(18) + 0.5) * (np.pi / 36)
    w = np.sin(mids) * np.cos(mids)
    return np.repeat(w / w.sum() / 36, 36)


def rel_rms(pred, ref, weights=None):
    """RMS relative BRF error per config: sqrt(sum_b w_b (pred - ref)^2 / sum_b w_b ref^2),
    bins weighted by their solid-angle share w_b (the photons they receive)."""
    w = bin_weights() if weights is None else weights
    return np.sqrt(((pred - ref) ** 2 * w).sum(axis=-1) / np.maximum((ref ** 2 * w).sum(axis=-1), 1e-30))


def train(ds, members=5, epochs=400, batch=256, lr=1e-3, seed=0, log=None, engine='grouped'):
    """Train an ensemble on a Dataset; returns Ensemble.  engine 'grouped': all members
    at once on the training engine (EnsembleTrainer, one graph replay per step);
    'layerwise': member by member on mcw_mlp_gemm and the per-member kernels."""
    import torch
    y = ds.y.astype(np.float64)
    y_mean, y_std = y.mean(0), np.maximum(y.std(0), 1e-3)
    t_all = torch.from_numpy(((y - y_mean) / y_std).astype(np.float32)).cuda()
    x_all = _cast(torch, torch.from_numpy(ds.x).cuda())
    w_out = torch.from_numpy(output_weights()).cuda()
    n = ds.x.shape[0]
    nets = []
    for k in range(members):
        net = SurrogateMLP(seed=seed * 100 + k)
        net.y_mean = torch.from_numpy(y_mean).cuda()
        net.y_std = torch.from_numpy(y_std).cuda()
        nets.append(net)
    if engine == 'grouped':
        # every member's step in one captured graph of grouped launches
        rngs = [np.random.default_rng(seed * 100 + k) for k in range(members)]
        tr = EnsembleTrainer(nets, batch, torch.from_numpy(ds.x).cuda(), t_all, w_out, lr=lr)
        for ep in range(epochs):
            lr_ep = lr * (0.5 * (1 + math.cos(math.pi * ep / epochs)))
            tr.set_epoch([r.permutation(n) for r in rngs], lr_ep)
            for _ in range(n // batch):
                tr.run_step()
            if log and (ep % 50 == 0 or ep == epochs - 1):
                log('epoch %d loss %s' % (ep, np.round(tr.loss.cpu().numpy(), 5).tolist()))
        tr.export()
        return Ensemble(nets)
    for k, net in enumerate(nets):
        rng = np.random.default_rng(seed * 100 + k)
        for ep in range(epochs):
            perm = torch.from_numpy(rng.permutation(n)).cuda()
            lr_ep = lr * (0.5 * (1 + math.cos(math.pi * ep / epochs)))
            for lo in range(0, n - batch + 1, batch):
                idx = perm[lo:lo + batch]
                loss = net.train_step(x_all[idx].contiguous(), t_all[idx].contiguous(), w_out, lr=lr_ep)
            if log and (ep % 50 == 0 or ep == epochs - 1):
                log('member %d epoch %d loss %.5f' % (k, ep, float(loss)))
    torch.cuda.synchronize()
    return Ensemble(nets)


def save(ensemble, path):
    """FP32 master weights, Adam state and target scaling of every member (torch.save)."""
    import torch
    torch.save([{'params': [p.cpu() for p in m.params], 'm': [x.cpu() for x in m.m],
                 'v': [x.cpu() for x in m.v], 'step': m.step, 'y_mean': m.y_mean.cpu(),
                 'y_std': m.y_std.cpu()} for m in ensemble.members], path)


def load(path):
    import torch
    members = []
    for d in torch.load(path):
        net = SurrogateMLP()
        net.params = [p.cuda() for p in d['params']]
        net.m = [x.cuda() for x in d['m']]
        net.v = [x.cuda() for x in d['v']]
        net.w16 = [_cast(torch, w) for w in net.params[0::2]]
        net.step = d['step']
        net.y_mean, net.y_std = d['y_mean'].cuda(), d['y_std'].cuda()
        members.append(net)
    return Ensemble(members)


def make_dataset(walker, n_cfg, n_photon, seed):
    raw = sample_inputs(n_cfg, seed)
    brf, alb = mc_brf(walker, raw, n_photon, seed)
    x = encode(*raw.T)
    return Dataset(x=x, y=to_target(brf, alb), raw=raw, brf=brf, albedo=alb, photons=n_photon)


def output_weights():
    """Loss weights: BRF bins by their photon share (mean 1), albedo 10."""
    w = bin_weights()
    w = w / w.mean()
    return np.concatenate([w, [10.0]]).astype(np.float32)


def inference_rate(ensemble, batch=65536, reps=20, members=None):
    """BRF predictions per second on the fused tensor-core kernel (CUDA events): every member
    of the ensemble (the mean and spread of a prediction need them all) forwards the same
    batch in one launch (mcw_mlp_forward_ensemble_f16); with members=k, the first k members
    one launch each.  The L2 is flushed before each timed repetition (median over reps)."""
    import torch
    ms = ensemble.members if members is None else ensemble.members[:members]
    x = torch.rand((batch, 4), device='cuda') * 2 - 1
    run = ensemble.predict_std if members is None else (lambda v: [m.predict_std(v) for m in ms])
    for _ in range(3):
        run(x)
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device='cuda')
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    times = []
    for _ in range(reps):
        flush.zero_()
        e0.record()
        run(x)
        e1.record()
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1))
    del flush
    return batch / (float(np.median(times)) / 1e3)
