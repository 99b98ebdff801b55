"""Tensor-core convolution kernels of the openness surrogate against PyTorch
float32 references on the same BF16-rounded operands, and a short training
run of the surrogate on exact-kernel labels."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def S():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from fujishadergpu_gb300.surrogate import openness_cnn
    return openness_cnn


def _bf(t):
    return t.to(torch.bfloat16).to(torch.float32)


def _ref_conv(x, w, b, dil, cin, flip=False):
    """x [B][H][W][C>=cin], w [9][cin][32] -> [B][H][W][32] (float32 conv of the given values)."""
    xt = x[..., :cin].permute(0, 3, 1, 2)
    wt = w.reshape(3, 3, cin, 32).permute(3, 2, 0, 1)  # [co][ci][ky][kx]
    if flip:
        wt = torch.flip(wt, dims=(2, 3))
    y = torch.nn.functional.conv2d(xt, wt, bias=b, padding=dil, dilation=dil)
    return y.permute(0, 2, 3, 1)


@pytest.mark.parametrize("cin,dil", [(32, 1), (32, 5), (3, 2)])
def test_conv_forward_matches_float32_reference(S, cin, dil):
    g = torch.Generator(device="cpu").manual_seed(cin * 10 + dil)
    cpad = 16 if cin <= 16 else 32
    x = torch.zeros(2, 40, 48, cpad)
    x[..., :cin] = torch.randn(2, 40, 48, cin, generator=g)
    x = x.cuda()
    w = (torch.randn(9, cin, 32, generator=g) * 0.2).cuda()
    b = torch.randn(32, generator=g).cuda()
    res = torch.randn(2, 40, 48, 32, generator=g).cuda()
    y = S._conv(x, S._pack(w, cin), cpad, dil, bias=b, relu=True, res=res)
    ref = torch.relu(_ref_conv(_bf(x), _bf(w), b, dil, cin)) + res
    assert torch.allclose(y, ref, rtol=1e-4, atol=1e-4), float((y - ref).abs().max())


def test_conv_data_and_weight_gradients_match_autograd(S):
    g = torch.Generator(device="cpu").manual_seed(7)
    x = torch.randn(1, 32, 64, 32, generator=g).cuda()
    w = (torch.randn(9, 32, 32, generator=g) * 0.2).cuda()
    gz = torch.randn(1, 32, 64, 32, generator=g).cuda()
    dil = 3
    # data gradient: the flipped conv with the transposed table
    gx = S._conv(gz, S._pack(w, 32, transpose=True), 32, dil, flip=True)
    xr = _bf(x).requires_grad_()
    out = _ref_conv(xr, _bf(w), None, dil, 32)
    out.backward(_bf(gz))
    assert torch.allclose(gx, xr.grad, rtol=1e-4, atol=1e-3), float((gx - xr.grad).abs().max())
    # weight gradient
    import ctypes as C
    from fujishadergpu_gb300 import _native as N
    dw = torch.zeros_like(w)
    N.check(N.lib().fsg_conv3x3_wgrad(C.c_void_p(x.data_ptr()), 32, 32, 1, 32, 64, dil, C.c_void_p(gz.data_ptr()),
                                      C.c_void_p(dw.data_ptr()), S._stream()))
    wr = _bf(w).requires_grad_()
    out = _ref_conv(_bf(x), wr, None, dil, 32)
    out.backward(_bf(gz))
    assert torch.allclose(dw, wr.grad, rtol=1e-3, atol=1e-2), float((dw - wr.grad).abs().max())


def test_head_forward_and_backward(S):
    Conv, Head = S._fns()
    h = torch.randn(2, 8, 16, 32, device="cuda").requires_grad_()
    w = torch.randn(32, device="cuda").requires_grad_()
    b = torch.tensor([0.3], device="cuda").requires_grad_()
    out = Head.apply(h, w, b)
    ref = (h * w).sum(-1) + b
    assert torch.allclose(out, ref, rtol=1e-5, atol=1e-5)
    go = torch.randn_like(out)
    gh, gw, gb = torch.autograd.grad(out, (h, w, b), go)
    rh, rw, rb = torch.autograd.grad(ref, (h, w, b), go)
    assert torch.allclose(gh, rh, rtol=1e-5, atol=1e-5)
    assert torch.allclose(gw, rw, rtol=1e-4, atol=1e-3)
    assert torch.allclose(gb, rb, rtol=1e-4, atol=1e-4)


def test_short_training_run_reduces_the_error(S):
    """Labels from the exact kernel (R = 32 here); the loss falls well below its start."""
    torch.manual_seed(0)
    wins = S.training_windows(4, 256, seed=11, pixel_size=5.0, max_distance=32)
    model = S.OpennessSurrogate(seed=1)
    assert 60_000 < model.n_params() < 110_000
    hist = S.train(model, wins, steps=150, batch=2, lr=2e-3, margin=32)
    assert np.mean(hist[-10:]) < 0.5 * np.mean(hist[:5]), (hist[:5], hist[-10:])
