"""CPU oracle of the surrogate network (test infrastructure, never the product).

float64 autograd in PyTorch on the CPU, on the same weights and inputs as the GPU
kernels of pyfds_gb300.surrogate. It restates, layer by layer, what
libfdsgpu.so's fds_conv3x3 / fds_conv3x3_wgrad / fds_adamw / fds_surr_* compute:

* conv3x3: zero-padded 3x3 cross-correlation with dilation d (padding d); weight
  layout [tap = 3 dy + dx][cout][cin], tap (dy, dx) reading pixel
  (y + (dy - 1) d, x + (dx - 1) d);
* GELU in tanh form, 0.5 v (1 + tanh(sqrt(2/pi) (v + 0.044715 v^3)));
* layer kinds: "first" h = gelu(z), "res" h = h_prev + gelu(z), "out" y = z;
* loss: mean over count x H x W x 3 of (s + y[..., :3] - t)^2;
* AdamW: torch.optim.AdamW semantics (decoupled decay, bias-corrected moments).

``bf16=True`` rounds every stored activation (z, h, the input x) to bfloat16 in the
forward pass, as the GPU stores them, with straight-through gradients.

The reference (emtpb/pyfds) has no learned component; this oracle pins the
surrogate kernels to their mathematical definition, not to a reference output.
"""
import numpy as np
import torch
import torch.nn.functional as F


def _round_bf16(t):
    return t + (t.to(torch.bfloat16).to(t.dtype) - t).detach()


def gelu(v):
    return F.gelu(v, approximate="tanh")


def conv3x3(x, w, b, dil):
    """x [B][H][W][cin] float64, w [9][cout][cin], b [cout] or None -> [B][H][W][cout]."""
    cout, cin = w.shape[1], w.shape[2]
    wt = w.reshape(3, 3, cout, cin).permute(2, 3, 0, 1)
    y = F.conv2d(x.permute(0, 3, 1, 2), wt, bias=b, padding=dil, dilation=dil)
    return y.permute(0, 2, 3, 1)


def forward(x, params, layers, bf16=True):
    """Returns (y, activations dict). params: [(w, b)] float64 tensors."""
    h = _round_bf16(x) if bf16 else x
    zs, hs = [], []
    for (w, b), (cin, cout, dil, kind) in zip(params, layers):
        z = conv3x3(h, w, b, dil)
        if kind == "out":
            return z, {"z": zs, "h": hs}
        a = gelu(z)
        hn = h + a if kind == "res" else a
        if bf16:
            z_s = _round_bf16(z)
            hn = _round_bf16(hn)
        else:
            z_s = z
        zs.append(z_s)
        hs.append(hn)
        h = hn
    raise ValueError("layers must end with an 'out' layer")


def loss(y, s, t):
    e = s[..., :3] + y[..., :3] - t[..., :3]
    return (e * e).mean()


def gradients(x, s, t, weights, layers, bf16=True):
    """Loss and [(dw [9][cout][cin], db [cout])] float64 numpy arrays for float32
    master weights ``weights`` (the GPU packs them to bf16: the oracle does too)."""
    params = []
    for w, b in weights:
        wt = torch.tensor(np.asarray(w, dtype=np.float32)).to(torch.bfloat16).to(torch.float64)
        params.append((wt.requires_grad_(True),
                       torch.tensor(np.asarray(b, dtype=np.float64)).requires_grad_(True)))
    xt = torch.as_tensor(np.asarray(x, dtype=np.float64))
    y, _ = forward(xt, params, layers, bf16)
    L = loss(y, torch.as_tensor(np.asarray(s, dtype=np.float64)),
             torch.as_tensor(np.asarray(t, dtype=np.float64)))
    L.backward()
    return float(L.detach()), [(w.grad.numpy(), b.grad.numpy()) for w, b in params]


def adamw_step(w, b, gw, gb, lr, step, m=None, v=None, beta1=0.9, beta2=0.999, eps=1e-8,
               weight_decay=0.01):
    """One torch.optim.AdamW step in float32 on (w, b) with gradients (gw, gb)."""
    pw = torch.nn.Parameter(torch.tensor(np.asarray(w, dtype=np.float32)))
    pb = torch.nn.Parameter(torch.tensor(np.asarray(b, dtype=np.float32)))
    opt = torch.optim.AdamW([pw, pb], lr=lr, betas=(beta1, beta2), eps=eps,
                            weight_decay=weight_decay)
    for _ in range(step):
        pw.grad = torch.tensor(np.asarray(gw, dtype=np.float32))
        pb.grad = torch.tensor(np.asarray(gb, dtype=np.float32))
        opt.step()
    return pw.detach().numpy(), pb.detach().numpy()


def pack_inputs(state, media, freq, zref):
    """Network input and normalised state of one sample, as fds_surr_pack builds
    them: state [3][H][W] (p, vx, vy), media [2][H][W] -> x [H][W][16] float64,
    s [H][W][4], scale."""
    p, vx, vy = (np.asarray(c, dtype=np.float64) for c in state)
    z = float(zref)
    scale = np.sqrt(np.mean(p * p + (z * vx) ** 2 + (z * vy) ** 2))
    inv = 1.0 / scale if scale > 0 else 0.0
    H, W = p.shape
    x = np.zeros((H, W, 16))
    x[..., 0] = media[0]
    x[..., 1] = media[1]
    x[..., 2] = p * inv
    x[..., 3] = z * vx * inv
    x[..., 4] = z * vy * inv
    x[..., 5] = freq
    s = np.zeros((H, W, 4))
    s[..., :3] = x[..., 2:5]
    return x, s, scale
