"""The surrogate oracle against first principles (CPU): the tap convention of its
3x3 dilated convolution against a direct loop, its AdamW against the update
formula written out, its input packing against the definition, and the C-ABI
structures of include/fds_surrogate.h."""
import ctypes as C

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from oracle import surrogate_oracle as so  # noqa: E402
from pyfds_gb300 import _capi  # noqa: E402


def test_conv_tap_convention_matches_direct_loop():
    rng = np.random.default_rng(0)
    B, H, W, cin, cout, d = 1, 7, 9, 3, 2, 2
    x = rng.standard_normal((B, H, W, cin))
    w = rng.standard_normal((9, cout, cin))
    b = rng.standard_normal(cout)
    y = so.conv3x3(torch.tensor(x), torch.tensor(w), torch.tensor(b), d).numpy()
    ref = np.zeros((B, H, W, cout))
    for yy in range(H):
        for xx in range(W):
            acc = b.copy()
            for dy in range(3):
                for dx in range(3):
                    sy, sx = yy + (dy - 1) * d, xx + (dx - 1) * d
                    if 0 <= sy < H and 0 <= sx < W:
                        acc += w[3 * dy + dx] @ x[0, sy, sx]
            ref[0, yy, xx] = acc
    assert np.allclose(y, ref, rtol=1e-12, atol=1e-12)


def test_adamw_formula():
    rng = np.random.default_rng(1)
    w = rng.standard_normal((9, 2, 3)).astype(np.float32)
    b = rng.standard_normal(2).astype(np.float32)
    gw = rng.standard_normal(w.shape).astype(np.float32)
    gb = rng.standard_normal(b.shape).astype(np.float32)
    lr, b1, b2, eps, wd = 1e-2, 0.9, 0.999, 1e-8, 0.01
    rw, rb = so.adamw_step(w, b, gw, gb, lr=lr, step=2)
    x = np.concatenate([w.ravel(), b]).astype(np.float64)
    g = np.concatenate([gw.ravel(), gb]).astype(np.float64)
    m = v = 0.0
    for t in (1, 2):
        x = x * (1 - lr * wd)
        m = b1 * m + (1 - b1) * g
        v = b2 * v + (1 - b2) * g * g
        x = x - lr / (1 - b1 ** t) * m / (np.sqrt(v) / np.sqrt(1 - b2 ** t) + eps)
    assert np.allclose(np.concatenate([rw.ravel(), rb]), x, rtol=1e-5, atol=1e-6)


def test_pack_inputs_definition():
    rng = np.random.default_rng(2)
    st = rng.standard_normal((3, 4, 5)) * np.array([1.0, 1e-6, 2e-6])[:, None, None]
    media = rng.standard_normal((2, 4, 5))
    x, s, sc = so.pack_inputs(st, media, 0.25, 1.5e6)
    e = st[0] ** 2 + (1.5e6 * st[1]) ** 2 + (1.5e6 * st[2]) ** 2
    assert np.isclose(sc, np.sqrt(e.mean()))
    assert np.allclose(x[..., 3], 1.5e6 * st[1] / sc)
    assert np.allclose(x[..., 5], 0.25) and np.all(x[..., 6:] == 0)
    assert np.allclose(s[..., :3], x[..., 2:5]) and np.all(s[..., 3] == 0)


def test_surrogate_struct_layouts():
    assert C.sizeof(_capi.FdsConvArgs) == 8 * 4 + 9 * 8
    assert C.sizeof(_capi.FdsWgradArgs) == 6 * 4 + 3 * 8 + 2 * 4 + 8
    assert C.sizeof(_capi.FdsAdamArgs) == 4 * 4 + 6 * 4 + 8 * 8
    assert C.sizeof(_capi.FdsSurrData) == 6 * 4 + 10 * 8


def test_float32_twin_matches_the_oracle_network():
    """The float32 twin of the precision study (pyfds_gb300.surrogate_twin) computes
    the oracle's network (tap convention, dilations, GELU, residuals) on the same
    initial weights, within float32 rounding."""
    import torch
    from pyfds_gb300 import surrogate as S
    from pyfds_gb300 import surrogate_twin as T
    tw = T.TwinNet(seed=3, device="cpu")
    ws = S.initial_weights(S.DEFAULT_LAYERS, 3)
    # larger biases and output weights than the initial ones exercise every term
    rng = np.random.default_rng(5)
    ws = [(w * (20.0 if k == len(ws) - 1 else 1.0), rng.standard_normal(b.shape) * 0.1)
          for k, (w, b) in enumerate(ws)]
    with torch.no_grad():
        for conv, (w, b) in zip(tw.convs, ws):
            cout, cin = w.shape[1], w.shape[2]
            conv.weight.copy_(torch.tensor(np.asarray(w, dtype=np.float32).reshape(
                3, 3, cout, cin).transpose(2, 3, 0, 1).copy()))
            conv.bias.copy_(torch.tensor(np.asarray(b, dtype=np.float32)))
    x = rng.standard_normal((2, 24, 20, 16))
    params = [(torch.tensor(np.asarray(w, dtype=np.float32).astype(np.float64)),
               torch.tensor(np.asarray(b, dtype=np.float32).astype(np.float64)))
              for w, b in ws]
    y_o, _ = so.forward(torch.tensor(x), params, S.DEFAULT_LAYERS, bf16=False)
    with torch.no_grad():
        y_t = tw.forward(torch.tensor(x, dtype=torch.float32).permute(0, 3, 1, 2))
    y_t = y_t.permute(0, 2, 3, 1).double().numpy()
    err = np.linalg.norm(y_t - y_o.numpy()) / np.linalg.norm(y_o.numpy())
    assert err < 1e-5, err
