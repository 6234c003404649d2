"""Float32 twin of the learned surrogate, for the precision study only.

The same network as ``pyfds_gb300.surrogate`` (layers, seeded initial weights, input
normalisation, global residual, pressure forced to 0 on the edges), the same
training pairs, batches, loss and AdamW/cosine schedule, evaluated in float32 with
PyTorch's own convolutions (cuDNN, TF32 off). It is not on any product path and
shares no code with the tcgen05 kernels: ``bench.py --study surrogate-precision``
trains it beside them to separate what the kernels' bf16 storage costs from what
the network's capacity and training objective allow, and to try objectives that
the kernels do not implement (a loss over several chained jumps).

Relative L2 error of a jump, as the rollout's check measures it (fds_surr_compare):
over p, Z vx, Z vy of the whole grid, || pred - ref || / || ref ||.
"""
import math
import time

import numpy as np

from .surrogate import DEFAULT_LAYERS, initial_weights


def _torch():
    import torch
    return torch


class TwinNet:
    """The surrogate network in float32 (PyTorch modules, NCHW)."""

    def __init__(self, layers=DEFAULT_LAYERS, seed=0, device="cuda"):
        torch = _torch()
        nn = torch.nn
        self.layers = [tuple(l) for l in layers]
        self.convs = nn.ModuleList()
        for (cin, cout, dil, _), (w, b) in zip(self.layers, initial_weights(self.layers, seed)):
            c = nn.Conv2d(cin, cout, 3, padding=dil, dilation=dil)
            with torch.no_grad():
                wt = np.asarray(w, dtype=np.float32).reshape(3, 3, cout, cin).transpose(2, 3, 0, 1)
                c.weight.copy_(torch.from_numpy(np.ascontiguousarray(wt)))
                c.bias.copy_(torch.from_numpy(np.asarray(b, dtype=np.float32)))
            self.convs.append(c)
        self.convs.to(device)

    def parameters(self):
        return self.convs.parameters()

    def forward(self, x):
        """x [B][16][H][W] -> y [B][16][H][W] (channels 0..2: change of the state)."""
        F = _torch().nn.functional
        h = x
        for conv, (_, _, _, kind) in zip(self.convs, self.layers):
            z = conv(h)
            if kind == "out":
                return z
            a = F.gelu(z, approximate="tanh")
            h = h + a if kind == "res" else a
        raise ValueError("layers must end with an 'out' layer")


def _normalise(st, z):
    """State [B][3][H][W] (p, vx, vy) -> energy-normalised (p, Z vx, Z vy) / scale
    and the scale (root mean square over the grid, per sample)."""
    torch = _torch()
    e = torch.stack([st[:, 0], st[:, 1] * z, st[:, 2] * z], dim=1)
    scale = torch.sqrt((e * e).sum(dim=1).mean(dim=(1, 2)))
    inv = torch.where(scale > 0, 1.0 / scale, torch.zeros_like(scale))
    return e * inv[:, None, None, None], scale


def _inputs(s, media, freq):
    torch = _torch()
    B, _, H, W = s.shape
    x = torch.zeros((B, 16, H, W), dtype=s.dtype, device=s.device)
    x[:, 0:2] = media
    x[:, 2:5] = s
    x[:, 5] = freq[:, None, None]
    return x


def _edge_mask(H, W, device):
    torch = _torch()
    m = torch.ones((1, 3, H, W), device=device)
    m[:, 0, 0, :] = 0
    m[:, 0, -1, :] = 0
    m[:, 0, :, 0] = 0
    m[:, 0, :, -1] = 0
    return m


def chain(net, data, inst, snap, jumps, mask):
    """Differentiable rollout of ``jumps`` network jumps from snapshot ``snap`` of the
    instances ``inst``; returns the list of (prediction, target) pairs, each in the
    normalised units of the jump's own input (as the next jump re-normalises)."""
    torch = _torch()
    z = data.zref[inst][:, None, None]
    media = data.media[inst]
    freq = data.freq[inst]
    s, scale = _normalise(data.state[inst, snap], z)
    out = []
    for j in range(jumps):
        y = net.forward(_inputs(s, media, freq))
        pred = (s + y[:, :3]) * mask
        # the target in this jump's units: the solver's state over this input's scale
        t_raw = torch.stack([data.state[inst, snap + j + 1][:, 0],
                             data.state[inst, snap + j + 1][:, 1] * z,
                             data.state[inst, snap + j + 1][:, 2] * z], dim=1)
        inv = torch.where(scale > 0, 1.0 / scale, torch.zeros_like(scale))
        out.append((pred, t_raw * inv[:, None, None, None]))
        if j + 1 < jumps:
            # the next jump starts from the prediction, re-normalised
            e = pred * scale[:, None, None, None]
            scale = torch.sqrt((e * e).sum(dim=1).mean(dim=(1, 2)))
            inv = torch.where(scale > 0, 1.0 / scale, torch.zeros_like(scale))
            s = e * inv[:, None, None, None]
    return out


def train(net, data, epochs=20, batch=32, lr=1e-3, seed=0, unroll=1, max_steps=None):
    """AdamW (weight decay 0.01, cosine schedule from ``lr`` to 0) on the pairs of
    ``data`` in the batches and order ``surrogate.train`` uses; with ``unroll`` > 1
    the loss sums the squared error of ``unroll`` chained jumps (samples whose chain
    would run past the last snapshot are dropped). Returns (losses, wall seconds)."""
    torch = _torch()
    torch.backends.cudnn.allow_tf32 = False
    torch.backends.cuda.matmul.allow_tf32 = False
    torch.backends.cudnn.benchmark = True
    pairs = data.pairs()
    if unroll > 1:
        pairs = pairs[pairs[:, 1] + unroll < data.nsnap]
    iters = len(pairs) // batch
    total = epochs * iters if max_steps is None else min(max_steps, epochs * iters)
    rng = np.random.default_rng(seed)
    order = np.concatenate([pairs[rng.permutation(len(pairs))][:iters * batch]
                            for _ in range(epochs)])[:total * batch]
    dev = data.state.device
    inst_all = torch.tensor(order[:, 0].copy(), dtype=torch.long, device=dev)
    snap_all = torch.tensor(order[:, 1].copy(), dtype=torch.long, device=dev)
    opt = torch.optim.AdamW(net.parameters(), lr=lr, betas=(0.9, 0.999), eps=1e-8,
                            weight_decay=0.01)
    mask = _edge_mask(data.n, data.n, dev)
    ones = torch.ones_like(mask)
    losses = []
    sync = torch.cuda.synchronize if dev.type == "cuda" else (lambda: None)
    sync()
    t0 = time.perf_counter()
    for it in range(total):
        sl = slice(it * batch, (it + 1) * batch)
        # the kernels' loss does not mask the edges; neither does the one-jump twin
        outs = chain(net, data, inst_all[sl], snap_all[sl], unroll, mask if unroll > 1 else ones)
        loss = sum(((p - t) ** 2).mean() for p, t in outs) / len(outs)
        for g in opt.param_groups:
            g["lr"] = 0.5 * lr * (1.0 + math.cos(math.pi * it / total))
        opt.zero_grad(set_to_none=True)
        loss.backward()
        opt.step()
        if it % max(1, iters) == 0 or it == total - 1:
            losses.append((it, float(loss.detach())))
    sync()
    return losses, time.perf_counter() - t0


def evaluate(net, data, jumps):
    """Relative L2 error of each instance after 1 .. ``jumps`` chained network jumps
    from snapshot 0, against the solver's snapshots: array [instances][jumps]."""
    torch = _torch()
    mask = _edge_mask(data.n, data.n, data.state.device)
    errs = []
    with torch.no_grad():
        for i0 in range(0, data.count, 16):
            inst = torch.arange(i0, min(i0 + 16, data.count), device=data.state.device)
            snap = torch.zeros_like(inst)
            outs = chain(net, data, inst, snap, jumps, mask)
            e = [torch.linalg.vector_norm((p - t).flatten(1), dim=1)
                 / torch.linalg.vector_norm(t.flatten(1), dim=1) for p, t in outs]
            errs.append(torch.stack(e, dim=1).cpu().numpy())
    return np.concatenate(errs, axis=0)
