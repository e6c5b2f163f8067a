"""The surrogate's training engine on the GPU (include/mcw_mlp.h, EnsembleTrainer):
the grouped TMA-fed tcgen05 GEMM against float64 on the same bf16 operands (every
epilogue, groups, split-K, transposed copies), one ensemble step's gradients against
float64 CPU autograd of each member, the grouped Adam against its formula, the
captured step against the same step run eagerly, and training that converges."""
import ctypes
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip('torch')

from monte_carlompi_gb300 import _abi, surrogate  # noqa: E402
from tests.helpers import reference_mlp  # noqa: E402


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _status_clear():
    flags = ctypes.c_uint32(0)
    assert _abi.load().mcw_mlp_status(1, ctypes.byref(flags)) == 0


def _status_ok():
    flags = ctypes.c_uint32(0)
    assert _abi.load().mcw_mlp_status(0, ctypes.byref(flags)) == 0
    assert flags.value == 0, flags.value


def _grouped(epi, m, n, k, a, b, c, groups=1, splits=1, bias=None, aux=None, c2=None, ct=None, s_split=0):
    """a [G, m, lda], b [G, n, ldb] bf16; c [G, m, ldc] (split partials: [S, G, m, ldc])."""
    lda, ldb = a.shape[-1], b.shape[-1]
    ldc = c.shape[-1]
    p = _abi.GemmGroupedC(m, n, k, groups, splits, epi, a.data_ptr(), lda, a.shape[-2] * lda,
                          b.data_ptr(), ldb, b.shape[-2] * ldb,
                          bias.data_ptr() if bias is not None else None, bias.shape[-1] if bias is not None else 0,
                          aux.data_ptr() if aux is not None else None, aux.shape[-1] if aux is not None else 0,
                          aux.shape[-2] * aux.shape[-1] if aux is not None else 0,
                          c.data_ptr(), ldc, c.shape[-2] * ldc, s_split,
                          c2.data_ptr() if c2 is not None else None, c2.shape[-1] if c2 is not None else 0,
                          c2.shape[-2] * c2.shape[-1] if c2 is not None else 0,
                          ct.data_ptr() if ct is not None else None, ct.shape[-1] if ct is not None else 0,
                          ct.shape[-2] * ct.shape[-1] if ct is not None else 0)
    return _abi.load().mcw_mlp_gemm_grouped(ctypes.byref(p), _stream())


@pytest.mark.parametrize('m,n,k,groups', [(128, 128, 64, 1), (300, 200, 256, 3), (256, 649, 256, 5),
                                          (1000, 256, 16, 2), (77, 40, 1000, 2), (649, 256, 4096, 1)])
def test_grouped_gemm_matches_float64(m, n, k, groups):
    g = torch.Generator().manual_seed(m + n + k + groups)
    ka = (k + 7) // 8 * 8
    a = torch.zeros(groups, m, ka)
    b = torch.zeros(groups, n, ka)
    a[:, :, :k] = torch.randn(groups, m, k, generator=g)
    b[:, :, :k] = torch.randn(groups, n, k, generator=g) * 0.1
    a16, b16 = a.to(torch.bfloat16).cuda(), b.to(torch.bfloat16).cuda()
    c = torch.full((groups, m, n), 7.0, device='cuda')
    _status_clear()
    assert _grouped(_abi.EPI_F32, m, n, k, a16, b16, c, groups=groups) == 0
    torch.cuda.synchronize()
    _status_ok()
    ref = a16.cpu().double()[:, :, :k] @ b16.cpu().double()[:, :, :k].transpose(1, 2)
    err = (c.cpu().double() - ref).abs().max().item()
    assert err <= 1e-4 * max(1.0, ref.abs().max().item()) + 1e-5 * math.sqrt(k), err


def test_grouped_gemm_split_k_partials_add_up():
    """K = 4,096 cut into 4 ranges: the partial products add up to the whole product."""
    groups, m, n, k, splits = 2, 300, 256, 4096, 4
    g = torch.Generator().manual_seed(3)
    a16 = torch.randn(groups, m, k, generator=g).to(torch.bfloat16).cuda()
    b16 = (torch.randn(groups, n, k, generator=g) * 0.1).to(torch.bfloat16).cuda()
    part = torch.zeros(splits, groups, m, n, device='cuda')
    assert _grouped(_abi.EPI_F32, m, n, k, a16, b16, part, groups=groups, splits=splits,
                    s_split=groups * m * n) == 0
    out = torch.zeros(groups, m, n, device='cuda')
    rc = _abi.load().mcw_mlp_reduce_splits(part.data_ptr(), groups * m * n, m * n, n, out.data_ptr(), m * n, n,
                                           splits, groups, m, n, _stream())
    assert rc == 0
    torch.cuda.synchronize()
    ref = a16.cpu().double() @ b16.cpu().double().transpose(1, 2)
    assert (out.cpu().double() - ref).abs().max().item() < 1e-4 * ref.abs().max().item()
    # a split count the K range cannot be cut into (64 chunks: 9 splits of 8 chunks are 8) is refused
    assert _grouped(_abi.EPI_F32, m, n, k, a16, b16, part, groups=groups, splits=9, s_split=groups * m * n) == -1


def test_grouped_gemm_epilogues_and_transposed_copies():
    groups, m, n, k = 3, 200, 256, 256
    g = torch.Generator().manual_seed(9)
    a16 = torch.randn(groups, m, k, generator=g).to(torch.bfloat16).cuda()
    w16 = (torch.randn(groups, n, k, generator=g) * 0.1).to(torch.bfloat16).cuda()
    bias = torch.randn(groups, n, generator=g).cuda()
    act = torch.zeros(groups, m, n, dtype=torch.bfloat16, device='cuda')
    z = torch.zeros(groups, m, n, device='cuda')
    act_t = torch.zeros(groups, n, m, dtype=torch.bfloat16, device='cuda')
    assert _grouped(_abi.EPI_BIAS_SILU, m, n, k, a16, w16, act, groups=groups, bias=bias, c2=z, ct=act_t) == 0
    torch.cuda.synchronize()
    zr = a16.cpu().double() @ w16.cpu().double().transpose(1, 2) + bias.cpu().double()[:, None, :]
    assert (z.cpu().double() - zr).abs().max().item() < 1e-4 * zr.abs().max().item()
    sr = zr * torch.sigmoid(zr)
    assert (act.cpu().double() - sr).abs().max().item() <= 0.01 * sr.abs().max().item()
    assert torch.equal(act_t.cpu(), act.cpu().transpose(1, 2))
    # SiLU' product with its copies
    gout = torch.zeros(groups, m, n, dtype=torch.bfloat16, device='cuda')
    g32 = torch.zeros(groups, m, n, device='cuda')
    gt = torch.zeros(groups, n, m, dtype=torch.bfloat16, device='cuda')
    assert _grouped(_abi.EPI_DSILU, m, n, k, a16, w16, gout, groups=groups, aux=z, c2=g32, ct=gt) == 0
    torch.cuda.synchronize()
    s = torch.sigmoid(z.cpu().double())
    gr = (a16.cpu().double() @ w16.cpu().double().transpose(1, 2)) * s * (1 + z.cpu().double() * (1 - s))
    assert (g32.cpu().double() - gr).abs().max().item() < 1e-3 * gr.abs().max().item()
    assert torch.equal(gt.cpu(), gout.cpu().transpose(1, 2))
    assert torch.equal(gout.cpu(), g32.cpu().to(torch.bfloat16))


def test_grouped_gemm_refuses_operands_tma_cannot_copy():
    a16 = torch.zeros(1, 64, 20, dtype=torch.bfloat16, device='cuda')      # rows of 40 bytes
    b16 = torch.zeros(1, 64, 24, dtype=torch.bfloat16, device='cuda')
    c = torch.zeros(1, 64, 64, device='cuda')
    assert _grouped(_abi.EPI_F32, 64, 64, 20, a16, b16, c) == -1
    flat = torch.zeros(64 * 24 + 4, dtype=torch.bfloat16, device='cuda')
    off = flat[4:].view(1, 64, 24)                                          # 8-byte aligned base
    assert _grouped(_abi.EPI_F32, 64, 64, 24, off, b16, c) == -1


def _members(n, seed):
    nets = [surrogate.SurrogateMLP(seed=seed + k) for k in range(n)]
    g = torch.Generator().manual_seed(seed)
    for net in nets:                                    # non-zero biases
        for i in range(1, 8, 2):
            net.params[i].copy_((torch.randn(net.params[i].shape, generator=g) * 0.3).cuda())
        net.w16 = [surrogate._cast(torch, w) for w in net.params[0::2]]
    return nets


def _data(n_rows, seed):
    g = torch.Generator().manual_seed(seed)
    x = torch.rand(n_rows, 4, generator=g) * 2 - 1
    t = torch.randn(n_rows, 649, generator=g)
    w = torch.from_numpy(surrogate.output_weights())
    return x, t, w


@pytest.mark.parametrize('batch,n_rows', [(256, 1024), (4096, 4096)])
def test_ensemble_gradients_match_cpu_autograd(batch, n_rows):
    """Forward, loss and backward of three members on their own batches (one launch per
    product for all members; at 4,096 rows the weight gradients are split-K) against
    float64 CPU autograd of each member (same bf16 roundings of weights, inputs and
    activations)."""
    nets = _members(3, 50)
    x, t, w = _data(n_rows, 4)
    tr = surrogate.EnsembleTrainer(nets, batch, x.cuda(), t.cuda(), w.cuda(), use_graph=False)
    rng = np.random.default_rng(1)
    perms = [rng.permutation(n_rows) for _ in nets]
    tr.set_epoch(perms, 1e-3)
    _status_clear()
    grads = tr.gradients()
    _status_ok()
    for k, net in enumerate(nets):
        idx = torch.from_numpy(perms[k][:batch])
        params = [p.detach().cpu().double().requires_grad_(True) for p in net.params]
        xb = x[idx].double()
        y = reference_mlp(xb, params)
        d = y - t[idx].double()
        loss = (w.double() * d * d).sum() / (batch * 649)
        loss.backward()
        assert abs(float(tr.loss[k]) - loss.item()) < 1e-3 * loss.item()
        for got, ref in zip(grads[k], params):
            got = got.cpu().double().flatten()
            ref = ref.grad.flatten()
            rel = (got - ref).norm() / ref.norm()
            cos = torch.dot(got, ref) / (got.norm() * ref.norm())
            assert rel < 3e-2 and cos > 0.999, (k, rel.item(), cos.item())


def test_ensemble_adam_matches_formula_and_graph_matches_eager():
    """Three captured steps equal three eager steps bit for bit; one step's update equals
    Adam's formula on the gradients the engine computed."""
    x, t, w = _data(1024, 6)
    rng = np.random.default_rng(2)
    perms = [rng.permutation(1024) for _ in range(2)]
    a = surrogate.EnsembleTrainer(_members(2, 70), 256, x.cuda(), t.cuda(), w.cuda(), use_graph=True)
    b = surrogate.EnsembleTrainer(_members(2, 70), 256, x.cuda(), t.cuda(), w.cuda(), use_graph=False)
    for tr in (a, b):
        tr.set_epoch(perms, 2e-3)
        for _ in range(3):
            tr.run_step()
    torch.cuda.synchronize()
    assert torch.equal(a.params, b.params) and torch.equal(a.m, b.m) and torch.equal(a.v, b.v)
    assert torch.equal(a.w16, b.w16) and torch.equal(a.wt, b.wt)
    assert int(a.step.item()) == 4 and int(a.counter.item()) == 3
    # one more step on b, checked against the formula
    w0, m0, v0 = b.params.clone(), b.m.clone(), b.v.clone()
    grads = b.gradients()            # the gradients of the next batch (counter 3)
    flat = b.grad.clone()
    b.run_step()
    torch.cuda.synchronize()
    lr, b1, b2, eps, step = 2e-3, 0.9, 0.999, 1e-8, 4
    m1 = b1 * m0 + (1 - b1) * flat
    v1 = b2 * v0 + (1 - b2) * flat * flat
    w1 = w0 - lr * (m1 / (1 - b1 ** step)) / (torch.sqrt(v1 / (1 - b2 ** step)) + eps)
    assert torch.allclose(b.params, w1, atol=1e-6, rtol=1e-5)
    assert torch.equal(b.w16, b.params.to(torch.bfloat16))
    o, rows, cols = b.lay['W3']
    to, ld = b.tlay['W3']
    wt = b.wt[:, to:to + cols * ld].view(2, cols, ld)
    assert torch.equal(wt[:, :, :rows], b.w16[:, o:o + rows * cols].view(2, rows, cols).transpose(1, 2))
    assert (wt[:, :, rows:] == 0).all()
    assert len(grads) == 2 and grads[0][6].shape == (649, 256)


def test_ensemble_training_fits_a_smooth_map():
    """Two members trained together on a smooth 4 -> 649 map: each member's loss falls a
    hundredfold, and the exported networks predict through the fused inference kernel."""
    rng = np.random.default_rng(0)
    n = 2048
    x = rng.uniform(-1, 1, (n, 4)).astype(np.float32)
    basis = rng.standard_normal((4, 649)) * 0.7
    y = np.tanh(x @ basis) + 0.3 * np.sin(2 * x[:, :1])
    y = ((y - y.mean(0)) / y.std(0)).astype(np.float32)
    nets = [surrogate.SurrogateMLP(seed=1 + k) for k in range(2)]
    tr = surrogate.EnsembleTrainer(nets, 256, torch.from_numpy(x).cuda(), torch.from_numpy(y).cuda(),
                                   torch.ones(649, device='cuda'), lr=2e-3)
    first = None
    for ep in range(120):
        tr.set_epoch([rng.permutation(n) for _ in nets], 2e-3)
        for _ in range(n // 256):
            tr.run_step()
        if first is None:
            torch.cuda.synchronize()
            first = tr.loss.cpu().numpy().copy()
    last = tr.loss.cpu().numpy()
    assert np.all(last < first / 100), (first, last)
    tr.export()
    xt = torch.from_numpy(x[:512]).cuda()
    for net in nets:
        pred = net.predict_std(xt, half=False)
        err = ((pred - torch.from_numpy(y[:512]).cuda()) ** 2).mean().item()
        assert err < 0.05, err
