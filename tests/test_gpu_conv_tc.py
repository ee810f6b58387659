"""The tensor-core (tcgen05) 3x3 convolutions of libmantiis_cnn.so against the
CUDA-core ones and the FP64 oracle: forward (with bias and ReLU) and the data
gradient, on shapes that cover partial pixel tiles, channel counts that are not
multiples of the 16-channel chunk and more than one chunk, and one output channel
tile of up to 256."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SHAPES = [(2, 2, 32, 64, 64), (1, 32, 64, 40, 48), (2, 64, 3, 32, 32), (1, 256, 256, 16, 24), (1, 17, 40, 9, 13)]


def bf16_round(w):
    u = np.asarray(w, np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) >> 16
    return u.astype(np.uint16)


def conv_ref(x, w, b, transpose=False):
    """FP64 3x3 convolution, zero padding (w: [cout][cin][3][3] in FP64)."""
    n, cin, h, wd = x.shape
    if transpose:
        w = np.flip(w.transpose(1, 0, 2, 3), axis=(2, 3))
    cout = w.shape[0]
    xp = np.zeros((n, cin, h + 2, wd + 2))
    xp[:, :, 1:-1, 1:-1] = x
    y = np.zeros((n, cout, h, wd))
    for ky in range(3):
        for kx in range(3):
            y += np.einsum("oc,nchw->nohw", w[:, :, ky, kx], xp[:, :, ky:ky + h, kx:kx + wd])
    if b is not None:
        y += b[None, :, None, None]
    return y


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("transpose", [False, True])
def test_tensor_core_conv_matches(shape, transpose):
    import torch

    from mantiis_gb300 import surrogate as S

    n, cin, cout, h, wd = shape
    rng = np.random.default_rng(cin * 1000 + cout)
    w32 = (rng.standard_normal((cout, cin, 3, 3)) / np.sqrt(9 * cin)).astype(np.float32)
    w16 = bf16_round(w32)
    wq = (w16.astype(np.uint32) << 16).view(np.float32).astype(np.float64)
    b = rng.standard_normal(cout).astype(np.float32)
    c_in, c_out = (cout, cin) if transpose else (cin, cout)
    x = rng.standard_normal((n, c_in, h, wd)).astype(np.float32)
    X = torch.tensor(x, device="cuda")
    W = torch.tensor(w16.view(np.int16).reshape(-1), device="cuda")
    B = torch.tensor(b, device="cuda")
    Y_tc = torch.zeros((n, c_out, h, wd), device="cuda")
    Y_cc = torch.zeros((n, c_out, h, wd), device="cuda")
    L = S.cnn_lib()
    st = S._stream()
    if transpose:
        assert L.cnn_conv3x3_backward_data_tc(S._ptr(X), S._ptr(W), S._ptr(Y_tc), n, cin, cout, h, wd, st) == 0
        assert L.cnn_conv3x3_backward_data(S._ptr(X), S._ptr(W), S._ptr(Y_cc), n, cin, cout, h, wd, st) == 0
        ref = conv_ref(x.astype(np.float64), wq, None, transpose=True)
    else:
        assert L.cnn_conv3x3_forward_tc(S._ptr(X), S._ptr(W), S._ptr(B), S._ptr(Y_tc), n, cin, cout, h, wd, 0, st) == 0
        assert L.cnn_conv3x3_forward(S._ptr(X), S._ptr(W), S._ptr(B), S._ptr(Y_cc), n, cin, cout, h, wd, 0, st) == 0
        ref = conv_ref(x.astype(np.float64), wq, b.astype(np.float64))
    torch.cuda.synchronize()
    assert L.cnn_tc_error() == 0
    y_tc, y_cc = Y_tc.cpu().numpy(), Y_cc.cpu().numpy()
    scale = np.abs(ref).max()
    e_tc = np.abs(y_tc - ref).max() / scale
    e_cc = np.abs(y_cc - ref).max() / scale
    from test_gpu_transport import record

    record(f"conv_tc_{'bw' if transpose else 'fw'}_{cin}_{cout}_{h}x{wd}", tc=e_tc, cuda_core=e_cc)
    # measured on a GB300: 2.1e-6 .. 5.2e-6 (the CUDA-core kernels 1.3e-7 .. 1.8e-6)
    assert e_tc < 5e-5, (e_tc, e_cc)


def wgrad_ref(x, dy):
    """FP64 weight and bias gradients of a 3x3 convolution (x: input, dy: output gradient)."""
    n, cin, h, wd = x.shape
    xp = np.zeros((n, cin, h + 2, wd + 2))
    xp[:, :, 1:-1, 1:-1] = x
    dw = np.zeros((dy.shape[1], cin, 3, 3))
    for ky in range(3):
        for kx in range(3):
            dw[:, :, ky, kx] = np.einsum("nohw,nchw->oc", dy, xp[:, :, ky:ky + h, kx:kx + wd])
    return dw, dy.sum(axis=(0, 2, 3))


@pytest.mark.parametrize("shape", SHAPES)
def test_tensor_core_weight_gradient_matches(shape):
    import torch

    from mantiis_gb300 import surrogate as S

    n, cin, cout, h, wd = shape
    rng = np.random.default_rng(cin * 7 + cout)
    x = rng.standard_normal((n, cin, h, wd)).astype(np.float32)
    dy = rng.standard_normal((n, cout, h, wd)).astype(np.float32)
    X, DY = torch.tensor(x, device="cuda"), torch.tensor(dy, device="cuda")
    L = S.cnn_lib()
    st = S._stream()
    out = {}
    for name, fn in (("tc", L.cnn_conv3x3_backward_weight_tc), ("cc", L.cnn_conv3x3_backward_weight)):
        dw = torch.zeros(cout * cin * 9, device="cuda")
        db = torch.zeros(cout, device="cuda")
        assert fn(S._ptr(X), S._ptr(DY), S._ptr(dw), S._ptr(db), n, cin, cout, h, wd, st) == 0
        torch.cuda.synchronize()
        out[name] = (dw.cpu().numpy().reshape(cout, cin, 3, 3), db.cpu().numpy())
    assert L.cnn_tc_error() == 0
    ref_w, ref_b = wgrad_ref(x.astype(np.float64), dy.astype(np.float64))
    e = {k: np.abs(v[0] - ref_w).max() / np.abs(ref_w).max() for k, v in out.items()}
    e_b = np.abs(out["tc"][1] - ref_b).max() / np.abs(ref_b).max()
    from test_gpu_transport import record

    record(f"conv_tc_wgrad_{cin}_{cout}_{h}x{wd}", tc=e["tc"], cuda_core=e["cc"], bias=e_b)
    assert e["tc"] < 5e-5 and e_b < 1e-5, (e, e_b)
