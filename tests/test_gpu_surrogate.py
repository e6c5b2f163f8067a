"""Surrogate network kernels (GPU): BF16 tensor-core GEMMs with FP32 accumulation
against a float64 reference of the same bf16 operands, the autograd Function's
gradients against CPU float64 autograd, Adam against its formula, and training."""
import ctypes
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip('torch')

from monte_carlompi_gb300 import _abi, surrogate  # noqa: E402


def _bf16(t):
    return t.to(torch.bfloat16)


ENGINES = [_abi.ENGINE_MMA_SYNC, _abi.ENGINE_TCGEN05]


@pytest.mark.parametrize('engine', ENGINES)
@pytest.mark.parametrize('trans_a,trans_b', [(0, 0), (0, 1), (1, 0), (1, 1)])
@pytest.mark.parametrize('m,n,k', [(100, 70, 37), (256, 649, 256), (64, 64, 4), (1, 5, 300), (300, 130, 200)])
def test_gemm_layouts_match_float64(trans_a, trans_b, m, n, k, engine):
    g = torch.Generator().manual_seed(m * 7 + n * 3 + k)
    a = torch.randn((k, m) if trans_a else (m, k), generator=g)
    b = torch.randn((k, n) if trans_b else (n, k), generator=g)
    a16, b16 = _bf16(a).cuda(), _bf16(b).cuda()
    c = torch.empty((m, n), dtype=torch.float32, device='cuda')
    surrogate._gemm(torch, _abi.EPI_F32, m, n, k, a16, a16.shape[1], b16, b16.shape[1], c, n,
                    trans_a=trans_a, trans_b=trans_b, engine=engine)
    A = a16.cpu().double()
    B = b16.cpu().double()
    ref = (A.T if trans_a else A) @ (B if trans_b else B.T)
    err = (c.cpu().double() - ref).abs().max().item()
    assert err <= 1e-4 * max(1.0, ref.abs().max().item()) + 1e-5 * math.sqrt(k), err


@pytest.mark.parametrize('engine', ENGINES)
def test_gemm_epilogues(engine):
    g = torch.Generator().manual_seed(5)
    m, n, k = 96, 200, 64
    a16 = _bf16(torch.randn(m, k, generator=g)).cuda()
    w16 = _bf16(torch.randn(n, k, generator=g) * 0.2).cuda()
    bias = torch.randn(n, generator=g).cuda()
    z = torch.empty((m, n), device='cuda')
    act = torch.empty((m, n), dtype=torch.bfloat16, device='cuda')
    surrogate._gemm(torch, _abi.EPI_BIAS_SILU, m, n, k, a16, k, w16, k, act, n, bias=bias, c2=z, ldc2=n,
                    engine=engine)
    zr = a16.cpu().double() @ w16.cpu().double().T + bias.cpu().double()
    assert (z.cpu().double() - zr).abs().max().item() < 1e-4
    ar = zr * torch.sigmoid(zr)
    assert (act.cpu().double() - ar).abs().max().item() <= 0.01 * ar.abs().max().item()
    # silu' epilogue on the same product
    gout16 = torch.empty((m, n), dtype=torch.bfloat16, device='cuda')
    gout32 = torch.empty((m, n), device='cuda')
    surrogate._gemm(torch, _abi.EPI_DSILU, m, n, k, a16, k, w16, k, gout16, n, aux=z, ldaux=n,
                    c2=gout32, ldc2=n, engine=engine)
    s = torch.sigmoid(z.cpu().double())
    ds = s * (1 + z.cpu().double() * (1 - s))
    gr = (a16.cpu().double() @ w16.cpu().double().T) * ds
    assert (gout32.cpu().double() - gr).abs().max().item() < 1e-3 * gr.abs().max().item()


def _st(v):
    """bf16 rounding in the forward pass, identity in the backward pass (as the kernels do)."""
    return v + (v.to(torch.bfloat16).double() - v).detach()


def _reference_mlp(x, params):
    """float64 CPU network with the kernels' bf16 roundings of weights, input and activations."""
    h = _st(x)
    ws, bs = params[0::2], params[1::2]
    for layer in range(4):
        z = h @ _st(ws[layer]).T + bs[layer]
        h = _st(z * torch.sigmoid(z)) if layer < 3 else z
    return h


def test_autograd_function_gradients_match_cpu():
    net = surrogate.SurrogateMLP(seed=3)
    g = torch.Generator().manual_seed(11)
    x = (torch.rand(64, 4, generator=g) * 2 - 1)
    params = [p.detach().clone().requires_grad_(True) for p in net.params]
    xg = x.cuda().requires_grad_(True)
    y = surrogate.mlp_apply(xg, params)
    gy = torch.randn(y.shape, generator=g)
    y.backward(gy.cuda())
    cparams = [p.detach().cpu().double().requires_grad_(True) for p in net.params]
    xc = x.double().requires_grad_(True)
    yc = _reference_mlp(xc, cparams)
    assert (y.detach().cpu().double() - yc.detach()).abs().max().item() < 2e-2 * yc.abs().max().item()
    yc.backward(gy.double())
    pairs = [(xg.grad, xc.grad)] + [(p.grad, c.grad) for p, c in zip(params, cparams)]
    for got, ref in pairs:
        got = got.detach().cpu().double().flatten()
        ref = ref.detach().flatten()
        rel = (got - ref).norm() / ref.norm()
        cos = torch.dot(got, ref) / (got.norm() * ref.norm())
        assert rel < 3e-2 and cos > 0.999, (rel.item(), cos.item())


def test_adam_kernel_matches_formula():
    n = 1000
    g = torch.Generator().manual_seed(2)
    w = torch.randn(n, generator=g)
    gr = torch.randn(n, generator=g)
    m = torch.randn(n, generator=g) * 0.1
    v = torch.rand(n, generator=g) * 0.1
    wd, gd, md, vd = w.cuda(), gr.cuda(), m.cuda(), v.cuda()
    w16 = torch.empty(n, dtype=torch.bfloat16, device='cuda')
    step, lr, b1, b2, eps = 7, 1e-3, 0.9, 0.999, 1e-8
    rc = _abi.load().mcw_mlp_adam(wd.data_ptr(), gd.data_ptr(), md.data_ptr(), vd.data_ptr(),
                                  w16.data_ptr(), n, lr, b1, b2, eps, step,
                                  ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == 0
    m2 = b1 * m + (1 - b1) * gr
    v2 = b2 * v + (1 - b2) * gr * gr
    w2 = w - lr * (m2 / (1 - b1 ** step)) / (torch.sqrt(v2 / (1 - b2 ** step)) + eps)
    assert torch.allclose(wd.cpu(), w2, atol=1e-6)
    assert torch.allclose(md.cpu(), m2, atol=1e-7) and torch.allclose(vd.cpu(), v2, atol=1e-7)
    assert torch.equal(w16.cpu(), w2.to(torch.bfloat16))


def test_training_fits_a_smooth_map():
    """Train one network on a smooth 4 -> 649 map; the loss must fall a hundredfold."""
    rng = np.random.default_rng(0)
    n = 2048
    x = rng.uniform(-1, 1, (n, 4)).astype(np.float32)
    basis = rng.standard_normal((4, 649)) * 0.7
    y = np.tanh(x @ basis) + 0.3 * np.sin(2 * x[:, :1])
    y = ((y - y.mean(0)) / y.std(0)).astype(np.float32)
    net = surrogate.SurrogateMLP(seed=1)
    x16 = surrogate._cast(torch, torch.from_numpy(x).cuda())
    t = torch.from_numpy(y).cuda()
    w = torch.ones(649, device='cuda')
    first = None
    for ep in range(120):
        perm = torch.from_numpy(rng.permutation(n)).cuda()
        for lo in range(0, n, 256):
            idx = perm[lo:lo + 256]
            loss = float(net.train_step(x16[idx].contiguous(), t[idx].contiguous(), w, lr=2e-3))
            first = loss if first is None else first
    assert loss < first / 100, (first, loss)


@pytest.mark.parametrize('m,n,k,epi', [(128, 128, 64, 0), (300, 200, 256, 1), (1000, 649, 256, 1),
                                       (257, 256, 256, 2), (64, 16, 16, 0), (130, 256, 4, 2)])
def test_tcgen05_gemm_matches_float64(m, n, k, epi):
    """The tcgen05 (tensor memory) forward GEMM against float64 on the same bf16 operands."""
    g = torch.Generator().manual_seed(m + n + k)
    a16 = _bf16(torch.randn(m, k, generator=g)).cuda()
    w16 = _bf16(torch.randn(n, k, generator=g) * 0.1).cuda()
    bias = torch.randn(n, generator=g).cuda()
    ref = a16.cpu().double() @ w16.cpu().double().T
    flags = ctypes.c_uint32(0)
    lib = _abi.load()
    assert lib.mcw_mlp_status(1, ctypes.byref(flags)) == 0
    if epi == _abi.EPI_BIAS_SILU:
        act = torch.empty((m, n), dtype=torch.bfloat16, device='cuda')
        z = torch.empty((m, n), device='cuda')
        surrogate._gemm(torch, epi, m, n, k, a16, k, w16, k, act, n, bias=bias, c2=z, ldc2=n,
                        engine=_abi.ENGINE_TCGEN05)
        torch.cuda.synchronize()
        zr = ref + bias.cpu().double()
        assert (z.cpu().double() - zr).abs().max().item() < 1e-4 * max(1.0, zr.abs().max().item())
        sr = zr * torch.sigmoid(zr)
        assert (act.cpu().double() - sr).abs().max().item() <= 0.01 * max(1.0, sr.abs().max().item())
    else:
        c = torch.empty((m, n), device='cuda')
        surrogate._gemm(torch, epi, m, n, k, a16, k, w16, k, c, n, bias=bias if epi else None,
                        engine=_abi.ENGINE_TCGEN05)
        torch.cuda.synchronize()
        r = ref + (bias.cpu().double() if epi else 0)
        assert (c.cpu().double() - r).abs().max().item() < 1e-4 * max(1.0, r.abs().max().item())
    assert lib.mcw_mlp_status(0, ctypes.byref(flags)) == 0 and flags.value == 0


def _random_net(seed):
    net = surrogate.SurrogateMLP(seed=seed)
    g = torch.Generator().manual_seed(seed + 1)
    for i in range(1, 8, 2):                       # non-zero biases
        net.params[i].copy_((torch.randn(net.params[i].shape, generator=g) * 0.3).cuda())
    return net


@pytest.mark.parametrize('m', [1, 127, 128, 129, 1000, 4097, 65536 + 77])
def test_fused_forward_matches_layerwise_and_float64(m):
    """mcw_mlp_forward (one tcgen05 kernel, activations in shared memory) against float64
    with the same bf16 roundings, and against the layer-by-layer GEMM forward."""
    net = _random_net(40 + m)
    g = torch.Generator().manual_seed(m)
    x = (torch.rand(m, 4, generator=g) * 2 - 1).cuda()
    flags = ctypes.c_uint32(0)
    lib = _abi.load()
    assert lib.mcw_mlp_status(1, ctypes.byref(flags)) == 0
    y = net.predict_std(x, half=False)
    y16 = net.predict_std(x).float()
    y_layer, _ = surrogate.forward_cached(torch, surrogate._cast(torch, x), net.w16, net.params[1::2], keep=False)
    torch.cuda.synchronize()
    assert lib.mcw_mlp_status(0, ctypes.byref(flags)) == 0 and flags.value == 0
    # fp16 output: y rounded to 11 significant bits
    assert (y16 - y).abs().max().item() <= 2.0 ** -10 * y.abs().max().item()
    ref = _reference_mlp(x.cpu().double(), [p.cpu().double() for p in net.params])
    scale = ref.abs().max().item()
    assert y.shape == (m, 649) and torch.isfinite(y).all()
    assert (y.cpu().double() - ref).abs().max().item() < 2e-2 * scale
    assert (y - y_layer).abs().max().item() < 5e-3 * scale


@pytest.mark.parametrize('m', [1000, 1001, 4096])
def test_ensemble_forward_equals_member_forwards(m):
    """One launch over three members (mcw_mlp_forward_ensemble_f16) gives each member the
    bits of its own forward (mcw_mlp_forward_f16), at a row count that is a multiple of the
    128-row tile, one that is not, and one that is not a multiple of the 8-row output box;
    the padding columns and rows of the next member are not written."""
    nets = [_random_net(30 + k) for k in range(3)]
    ens = surrogate.Ensemble(nets)
    x = (torch.rand(m, 4, generator=torch.Generator().manual_seed(5)) * 2 - 1).cuda()
    blob, bias = ens.packed()
    y = torch.full((3, m, surrogate.Y_PITCH_F16), 3.0, dtype=torch.float16, device='cuda')
    rc = _abi.load().mcw_mlp_forward_ensemble_f16(surrogate._ptr(x), m, 3, surrogate._ptr(bias),
                                                  surrogate._ptr(blob), surrogate._ptr(y), surrogate.Y_PITCH_F16,
                                                  surrogate._stream(torch))
    assert rc == 0
    for k, net in enumerate(nets):
        ref = net.predict_std(x)
        torch.cuda.synchronize()
        assert torch.equal(y[k, :, :649], ref), k
    assert (y[:, :, 649:] == 3.0).all()
    assert torch.equal(ens.predict_std(x), y[:, :, :649])
    assert _abi.load().mcw_mlp_forward_ensemble_f16(surrogate._ptr(x), m, 0, surrogate._ptr(bias),
                                                    surrogate._ptr(blob), surrogate._ptr(y), surrogate.Y_PITCH_F16,
                                                    surrogate._stream(torch)) == -1


def test_fused_forward_leading_dimension_and_repack():
    """Rows land at stride ldy without touching the padding columns or the rows past m;
    after an Adam step the packed weights are rebuilt so inference follows the new weights."""
    net = _random_net(7)
    m, ldy = 300, 700
    x = (torch.rand(m, 4, generator=torch.Generator().manual_seed(2)) * 2 - 1).cuda()
    full = torch.full((m + 40, ldy), 12345.0, device='cuda')
    out = full[:m]
    b = [t.contiguous() for t in net.params[1::2]]
    rc = _abi.load().mcw_mlp_forward(surrogate._ptr(x), m, surrogate._ptr(b[0]), surrogate._ptr(b[1]),
                                     surrogate._ptr(b[2]), surrogate._ptr(b[3]), surrogate._ptr(net.packed()),
                                     surrogate._ptr(out), ldy, surrogate._stream(torch))
    assert rc == 0
    y = net.predict_std(x, half=False)
    torch.cuda.synchronize()
    assert torch.equal(out[:, :649], y)
    assert (out[:, 649:] == 12345.0).all()
    assert (full[m:] == 12345.0).all()
    bad = _abi.load().mcw_mlp_forward(surrogate._ptr(x), m, surrogate._ptr(b[0]), surrogate._ptr(b[1]),
                                      surrogate._ptr(b[2]), surrogate._ptr(b[3]), surrogate._ptr(net.packed()),
                                      surrogate._ptr(out), 600, surrogate._stream(torch))
    assert bad == -1
    bad = _abi.load().mcw_mlp_forward(surrogate._ptr(x), m, surrogate._ptr(b[0]), surrogate._ptr(b[1]),
                                      surrogate._ptr(b[2]), surrogate._ptr(b[3]), surrogate._ptr(net.packed()),
                                      surrogate._ptr(out), 650, surrogate._stream(torch))
    assert bad == -1                               # row pitch not a multiple of 16 bytes
    # fp16 rows at pitch 664: padding and rows past m untouched; odd pitches refused
    full16 = torch.full((m + 40, 664), 7.0, dtype=torch.float16, device='cuda')
    rc = _abi.load().mcw_mlp_forward_f16(surrogate._ptr(x), m, surrogate._ptr(b[0]), surrogate._ptr(b[1]),
                                         surrogate._ptr(b[2]), surrogate._ptr(b[3]), surrogate._ptr(net.packed()),
                                         surrogate._ptr(full16), 664, surrogate._stream(torch))
    assert rc == 0
    torch.cuda.synchronize()
    assert torch.equal(full16[:m, :649], net.predict_std(x))
    assert (full16[:m, 649:] == 7.0).all() and (full16[m:] == 7.0).all()
    assert _abi.load().mcw_mlp_forward_f16(surrogate._ptr(x), m, surrogate._ptr(b[0]), surrogate._ptr(b[1]),
                                           surrogate._ptr(b[2]), surrogate._ptr(b[3]), surrogate._ptr(net.packed()),
                                           surrogate._ptr(full16), 660, surrogate._stream(torch)) == -1
    before = net.predict_std(x).clone()
    t = torch.randn(64, 649, device='cuda')
    w_out = torch.from_numpy(surrogate.output_weights()).cuda()
    net.train_step(surrogate._cast(torch, x[:64].contiguous()), t, w_out, lr=1e-2)
    after = net.predict_std(x)
    y_layer, _ = surrogate.forward_cached(torch, surrogate._cast(torch, x), net.w16, net.params[1::2], keep=False)
    torch.cuda.synchronize()
    assert not torch.equal(before, after)
    assert (after - y_layer).abs().max().item() < 5e-3 * y_layer.abs().max().item()


def test_forward_tangent_matches_cpu_jvp():
    """surrogate.forward_tangent (forward mode on the kernels: SiLU' epilogue GEMMs) against
    float64 CPU forward-mode autograd of the same bf16-rounded network."""
    net = _random_net(21)
    g = torch.Generator().manual_seed(5)
    x = torch.rand(300, 4, generator=g) * 2 - 1
    xdot = torch.zeros_like(x)
    xdot[:, 0] = 0.57
    y, ydot = surrogate.forward_tangent(torch, surrogate._cast(torch, x.cuda()), surrogate._cast(torch, xdot.cuda()),
                                        net.w16, net.params[1::2])
    params = [p.detach().cpu().double() for p in net.params]
    _, ref = torch.autograd.functional.jvp(lambda v: _reference_mlp(v, params), x.double(), xdot.double())
    ydot = ydot.cpu().double()
    rel = (ydot - ref).norm(dim=1) / ref.norm(dim=1)
    assert torch.isfinite(ydot).all()
    assert rel.median().item() < 0.02 and rel.max().item() < 0.08, (rel.median().item(), rel.max().item())
