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
    """Three identical runs; after a warm-up that collects pairs, one continues
    with the trained network, one with plain extrapolation, one with the
    previous pressure (the method without the network)."""
    runs = {name: _tgv_solver(F.GUESS_PREVIOUS) for name in ("net", "extrap", "prev")}
    runs["net"].unet_collect()
    for _ in range(12):
        for g in runs.values():
            s, st = g.time_advance()
            assert s == 0
    loss = runs["net"].unet_train(150, 2e-3)
    assert np.isfinite(loss)
    runs["net"].set_guess_mode(F.GUESS_LEARNED)
    runs["extrap"].set_guess_mode(F.GUESS_EXTRAPOLATE)
    cycles = {k: [] for k in runs}
    sources = []
    for _ in range(6):
        for k, g in runs.items():
            s, st = g.time_advance()
            assert s == 0 and st.fine_residual <= 1e-8
            cycles[k].append(st.vcycles)
            if k == "net":
                sources.append(st.guess_source)
    mean = {k: float(np.mean(v)) for k, v in cycles.items()}
    print("V-cycles per step:", mean, "guess sources:", sources, "loss:", loss)
    assert mean["net"] <= mean["prev"]
    # all three runs solve to the same residual target: the fields agree
    for f in (F.FIELD_VX, F.FIELD_P):
        assert C.rel_err(runs["net"].get(f), runs["prev"].get(f)) < 1e-7
