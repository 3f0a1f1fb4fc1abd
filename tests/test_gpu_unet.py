"""The learned warm start: tensor-core convolutions against a float64 CPU
oracle (torch CPU conv3d / autograd on the same BF16-rounded inputs), and the
V-cycle gain of the trained network over the solver without it."""
import numpy as np
import pytest

import saras_gb300 as S
from saras_gb300 import _abi as F
from tests import _cases as C

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

SHAPES = [(16, 16), (16, 32), (32, 64), (64, 32), (48, 16), (96, 32), (32, 96)]
DIMS = (5, 9, 131)      # 5895 voxels: tiles straddle rows and the domain edge


def inputs(cin, cout, seed):
    rng = np.random.default_rng(seed)
    D, H, W = DIMS
    x = rng.standard_normal((D, H, W, cin)).astype(np.float32)
    dy = rng.standard_normal((D, H, W, cout)).astype(np.float32)
    w = (rng.standard_normal((cout, 27, cin)) / np.sqrt(27 * cin)).astype(np.float32)
    b = rng.standard_normal(cout).astype(np.float32)
    xb, dyb = S.to_bf16_bits(x), S.to_bf16_bits(dy)
    wb = S.from_bf16_bits(S.to_bf16_bits(w))          # the kernel consumes BF16 weights
    return xb, dyb, w, wb, b


def torch_ref(x, w, cin, cout):
    D, H, W = DIMS
    xt = torch.tensor(x.reshape(D, H, W, cin), dtype=torch.float64).permute(3, 0, 1, 2)[None]
    wt = torch.tensor(w.reshape(cout, 3, 3, 3, cin), dtype=torch.float64).permute(0, 4, 1, 2, 3)
    return xt, wt


def bf16_close(a, ref, rel=1.5e-2):
    scale = np.max(np.abs(ref)) + 1e-30
    err = np.max(np.abs(a - ref)) / scale
    assert err < rel, err


@pytest.mark.parametrize("cin,cout", SHAPES)
def test_conv_forward(cin, cout):
    xb, _, w, wb, b = inputs(cin, cout, 1)
    out = S.conv3d_check(0, xb, None, w, b, 1, DIMS, cin, cout)
    xt, wt = torch_ref(S.from_bf16_bits(xb), wb, cin, cout)
    ref = torch.relu(torch.nn.functional.conv3d(xt, wt, torch.tensor(b, dtype=torch.float64), padding=1))
    ref = ref[0].permute(1, 2, 3, 0).reshape(-1).numpy()
    bf16_close(out, ref)


@pytest.mark.parametrize("cin,cout", SHAPES)
def test_conv_input_gradient(cin, cout):
    xb, dyb, w, wb, b = inputs(cin, cout, 2)
    out = S.conv3d_check(1, None, dyb, w, None, 0, DIMS, cin, cout)
    D, H, W = DIMS
    xt, wt = torch_ref(S.from_bf16_bits(xb), wb, cin, cout)
    xt.requires_grad_(True)
    y = torch.nn.functional.conv3d(xt, wt, padding=1)
    g = torch.tensor(S.from_bf16_bits(dyb).reshape(D, H, W, cout), dtype=torch.float64).permute(3, 0, 1, 2)[None]
    (y * g).sum().backward()
    ref = xt.grad[0].permute(1, 2, 3, 0).reshape(-1).numpy()
    bf16_close(out, ref)


@pytest.mark.parametrize("cin,cout", [(16, 16), (32, 64), (96, 32)])
def test_conv_weight_gradient(cin, cout):
    xb, dyb, w, wb, b = inputs(cin, cout, 3)
    out = S.conv3d_check(2, xb, dyb, w, None, 0, DIMS, cin, cout)
    D, H, W = DIMS
    xt, wt = torch_ref(S.from_bf16_bits(xb), wb, cin, cout)
    wt.requires_grad_(True)
    bt = torch.zeros(cout, dtype=torch.float64, requires_grad=True)
    y = torch.nn.functional.conv3d(xt, wt, bt, padding=1)
    g = torch.tensor(S.from_bf16_bits(dyb).reshape(D, H, W, cout), dtype=torch.float64).permute(3, 0, 1, 2)[None]
    (y * g).sum().backward()
    dw_ref = wt.grad.permute(0, 2, 3, 4, 1).reshape(-1).numpy()
    np.testing.assert_allclose(out[:27 * cin * cout], dw_ref, rtol=1e-4, atol=1e-3 * np.max(np.abs(dw_ref)))
    np.testing.assert_allclose(out[27 * cin * cout:], bt.grad.numpy(), rtol=1e-4, atol=1e-3 * np.max(np.abs(bt.grad.numpy())))


def _tgv_solver(guess):
    p = C.tgv(ind=6, depth=4, dt=5e-4)
    p.mgMode = F.MG_MIXED
    p.mgTarget = 1e-8
    p.mgMaxCycles = 100
    p.jacobiWeight = 6.0 / 7.0
    p.fastKernels = 1
    p.guessMode = F.GUESS_PREVIOUS
    g = S.Solver(p)
    C.initialise(g, p, "tgv")
    return g


def test_learned_guess_reduces_vcycles():
    """Four identical runs; after a warm-up that collects pairs, the trained
    network is used by the per-solve selector (learned), in every solve
    (network alone), and compared with plain extrapolation and with the
    previous pressure (the method without any history).  What is asserted is
    what holds: the network's guess starts closer than the previous pressure
    and needs fewer V-cycles than it; the selector is never worse than
    extrapolation by more than half a cycle a solve.  The network is not
    asserted to beat extrapolation: on this flow its guess leaves about the
    residual extrapolation leaves (both printed)."""
    names = ("learned", "network", "extrap", "prev")
    runs = {name: _tgv_solver(F.GUESS_PREVIOUS) for name in names}
    runs["learned"].unet_collect()
    runs["network"].unet_collect()
    for _ in range(12):
        for g in runs.values():
            s, st = g.time_advance()
            assert s == 0
    for k in ("learned", "network"):
        loss = runs[k].unet_train(150, 2e-3)
        assert np.isfinite(loss)
    runs["learned"].set_guess_mode(F.GUESS_LEARNED)
    runs["network"].set_guess_mode(F.GUESS_NETWORK)
    runs["extrap"].set_guess_mode(F.GUESS_EXTRAPOLATE)
    cycles = {k: [] for k in runs}
    start = {k: [] for k in runs}
    sources = {k: [] for k in runs}
    for _ in range(8):
        for k, g in runs.items():
            s, st = g.time_advance()
            assert s == 0 and st.fine_residual <= 1e-8
            cycles[k].append(st.vcycles)
            start[k].append(st.guess_residual)
            sources[k].append(st.guess_source)
    mean = {k: float(np.mean(v)) for k, v in cycles.items()}
    med = {k: float(np.median(v)) for k, v in start.items()}
    print("V-cycles per step:", mean, "median start residual / max|b|:", med, "sources:", sources)
    # the network-only run used the network once its histories were complete
    assert sources["network"][-4:] == [F.GUESS_LEARNED] * 4, sources["network"]
    assert med["network"] < med["prev"]
    assert mean["network"] < mean["prev"]
    assert mean["learned"] <= mean["extrap"] + 0.5
    # all runs solve to the same residual target: the fields agree
    for k in ("learned", "network", "extrap"):
        for f in (F.FIELD_VX, F.FIELD_P):
            assert C.rel_err(runs[k].get(f), runs["prev"].get(f)) < 1e-7, (k, f)


# layer table of the U-Net (unet.cu): input channels (main, skip), output channels, level, ReLU
UNET_LAYERS = [(16, 0, 16, 0, True), (16, 0, 16, 0, True), (16, 0, 32, 1, True), (32, 0, 32, 1, True),
               (32, 0, 64, 2, True), (64, 0, 64, 2, True), (64, 32, 32, 1, True), (32, 0, 32, 1, True),
               (32, 16, 16, 0, True), (16, 0, 16, 0, True), (16, 0, 16, 0, False)]


def _torch_unet(params, x0):
    """The U-Net in torch float64: 3x3x3 convolutions with zero padding,
    full-weighting restriction (stride-2 [1/4 1/2 1/4]^3), trilinear vertex
    prolongation, skip connections by concatenation; weights BF16-rounded as
    the tensor cores use them."""
    F_ = torch.nn.functional
    ws, off = [], 0
    for c0, c1, co, lvl, relu in UNET_LAYERS:
        cin = c0 + c1
        w = params[off:off + 27 * cin * co]
        off += 27 * cin * co
        b = params[off:off + co]
        off += co
        wb = S.from_bf16_bits(S.to_bf16_bits(w))
        wt = torch.tensor(wb.reshape(co, 3, 3, 3, cin), dtype=torch.float64).permute(0, 4, 1, 2, 3).contiguous()
        ws.append((wt.requires_grad_(True), torch.tensor(b, dtype=torch.float64, requires_grad=True), relu))

    def conv(q, x):
        w, b, relu = ws[q]
        y = F_.conv3d(x, w, b, padding=1)
        return torch.relu(y) if relu else y

    def down(x):
        C = x.shape[1]
        k1 = torch.tensor([0.25, 0.5, 0.25], dtype=torch.float64)
        k = (k1[:, None, None] * k1[None, :, None] * k1[None, None, :]).expand(C, 1, 3, 3, 3)
        return F_.conv3d(x, k, stride=2, padding=1, groups=C)

    def up(x, shape):
        out = 0
        idx = []
        for n_f, n_c in zip(shape, x.shape[2:]):
            f = torch.arange(n_f)
            i0 = f // 2
            i1 = torch.clamp(i0 + (f % 2), max=n_c - 1)
            idx.append((i0, i1))
        for a in idx[0]:
            for b in idx[1]:
                for c in idx[2]:
                    out = out + x[:, :, a][:, :, :, b][:, :, :, :, c]
        return 0.125 * out

    a0 = conv(0, x0)
    e1 = conv(1, a0)
    p1 = down(e1)
    e2 = conv(3, conv(2, p1))
    p2 = down(e2)
    e3 = conv(5, conv(4, p2))
    u2 = up(e3, e2.shape[2:])
    f2 = conv(7, conv(6, torch.cat([u2, e2], 1)))
    u1 = up(f2, e1.shape[2:])
    f1 = conv(9, conv(8, torch.cat([u1, e1], 1)))
    y = conv(10, f1)
    return y[0, 0], ws


def test_unet_backward_matches_torch_autograd():
    """The whole U-Net -- convolutions (tcgen05 forward and input gradient),
    restriction and prolongation, skip connections, ReLU masks, the loss and the
    weight gradients -- against torch float64 autograd of the same network on
    the same BF16-rounded input and weights: output, loss and every layer's
    weight and bias gradient agree to the accuracy of BF16 activations (output
    and loss to 5e-2, each layer's gradient to a relative L2 error of 1e-1 --
    a wrong mask, skip path or transfer gives errors of order 1)."""
    g = _tgv_solver(F.GUESS_PREVIOUS)
    nparam, dims = g.unet_shape()
    rng = np.random.default_rng(5)
    params = np.empty(nparam, dtype=np.float32)
    off = 0
    for c0, c1, co, lvl, relu in UNET_LAYERS:
        cin = c0 + c1
        params[off:off + 27 * cin * co] = rng.uniform(-1, 1, 27 * cin * co) * np.sqrt(6.0 / (27 * cin))
        off += 27 * cin * co
        params[off:off + co] = rng.uniform(-0.1, 0.1, co)
        off += co
    assert off == nparam
    feat = rng.standard_normal(dims + (3,)).astype(np.float32)
    target = rng.standard_normal(dims).astype(np.float32)
    d, loss, grad = g.unet_grad_check(feat, target, params)
    x0 = np.zeros((1, 16) + dims)
    x0[0, :3] = np.moveaxis(S.from_bf16_bits(S.to_bf16_bits(feat)), -1, 0)
    y, ws = _torch_unet(params, torch.tensor(x0, dtype=torch.float64))
    tt = torch.tensor(target, dtype=torch.float64)
    L = 0.5 * torch.mean((y - tt) ** 2)
    L.backward()
    yn = y.detach().numpy()
    assert np.max(np.abs(d - yn)) <= 5e-2 * np.max(np.abs(yn)), np.max(np.abs(d - yn)) / np.max(np.abs(yn))
    assert abs(loss - L.item()) <= 5e-2 * L.item(), (loss, L.item())
    off = 0
    for q, (c0, c1, co, lvl, relu) in enumerate(UNET_LAYERS):
        cin = c0 + c1
        gw = grad[off:off + 27 * cin * co]
        off += 27 * cin * co
        gb = grad[off:off + co]
        off += co
        rw = ws[q][0].grad.permute(0, 2, 3, 4, 1).reshape(-1).numpy()
        rb = ws[q][1].grad.numpy()
        ew = np.linalg.norm(gw - rw) / max(np.linalg.norm(rw), 1e-30)
        eb = np.linalg.norm(gb - rb) / max(np.linalg.norm(rb), 1e-30)
        print("layer %d: relative gradient error W %.3e b %.3e" % (q, ew, eb))
        assert ew < 1e-1 and eb < 1e-1, (q, ew, eb)
