"""Learned surrogate for batched Acoustic2D parameter sweeps.

A residual CNN of 3x3 convolutions maps the state of a 2-D staggered acoustic field
(p, vx, vy on an n x n grid, plus the medium and the source frequency) to the
state ``JUMP`` = 64 time steps later. Around it the finite-difference engine does
three jobs:

* it generates the training data: the batched solver (``batch.BatchRunner``, the
  engine behind ``Acoustic2D.sim_step``, pyfds/acoustics.py:111-128) advances many
  layered media and snapshots of (t, t + 64) are copied on the device;
* it checks the network during a rollout: every ``check_every`` jumps the FP64
  solver advances the same state by 64 steps and the jump's relative L2 error is
  measured against it;
* it takes over: an instance whose check exceeds the tolerance continues with the
  solver alone.

Every network operation runs in libfdsgpu.so (include/fds_surrogate.h): the
convolutions, their data and weight gradients on the tensor cores (tcgen05, BF16
operands, FP32 accumulation), the fused AdamW step, and the packing of states.
PyTorch only owns the device memory. There is no CPU path: the library must be
built and a GPU present. Activations are bf16 in the channel-group blocked layout
[batch][channels/8][height][width][8] of include/fds_surrogate.h.

Network (``DEFAULT_LAYERS``): 8 convolution layers, 48 channels, GELU (tanh form),
residual connections on layers 1..6, dilations 1, 2, 4, 8, 8, 4, 2, 1 so that the
receptive field (30 cells) covers the distance a wave travels in 64 steps at CFL
0.4 (25.6 cells). Input channels: local Courant number c dt/dx, rho / mean(rho),
p / s, Z vx / s, Z vy / s, normalised source frequency (s = the state's energy norm
per sample, Z = mean(rho c)), padded to 16. Output: the change of the three
normalised state channels over the jump (global residual); the pressure on the
outermost cells is set to 0, the solver's boundary condition.
"""
import ctypes as C
import math
import time

import numpy as np

from . import _capi, workloads
from ._engine import require_cuda
from .batch import BatchRunner, simulate_batch

JUMP = 64
IN_CH = 16
OUT_CH = 16
T_SRC = 704  # steps of solver-only source phase before snapshots / jumps

# (cin, cout, dilation, kind); kind: "first" gelu, "res" gelu + residual, "out" linear
DEFAULT_LAYERS = ((16, 48, 1, "first"), (48, 48, 2, "res"), (48, 48, 4, "res"),
                  (48, 48, 8, "res"), (48, 48, 8, "res"), (48, 48, 4, "res"),
                  (48, 48, 2, "res"), (48, 16, 1, "out"))


def initial_weights(layers, seed):
    """Seeded initial weights [(w [9][cout][cin], b [cout]), ...]: He-scaled normal
    draws, shrunk on the residual (0.2) and output (0.05) layers, zero biases."""
    rng = np.random.default_rng(seed)
    ws = []
    for cin, cout, dil, kind in layers:
        std = math.sqrt(2.0 / (9 * cin)) * {"first": 1.0, "res": 0.2, "out": 0.05}[kind]
        ws.append((rng.standard_normal((9, cout, cin)) * std, np.zeros(cout)))
    return ws


def _ptr(t):
    return C.c_void_p(t.data_ptr()) if t is not None else None


def _stream(torch):
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


class ConvNet:
    """The surrogate network: float32 master weights and AdamW moments on the
    device, bf16 packed operands for the tensor-core convolutions, activation
    buffers per input shape."""

    def __init__(self, layers=DEFAULT_LAYERS, seed=0):
        torch = require_cuda()
        self.torch = torch
        self.lib = _capi.load()
        self.dev = torch.device("cuda", torch.cuda.current_device())
        self.layers = [tuple(l) for l in layers]
        kinds = [l[3] for l in self.layers]
        if kinds[0] != "first" or kinds[-1] != "out" or any(k != "res" for k in kinds[1:-1]):
            raise ValueError("layers must be first, res..., out")
        if self.layers[0][0] != IN_CH or self.layers[-1][1] != OUT_CH:
            raise ValueError("the first layer takes %d channels, the last gives %d"
                             % (IN_CH, OUT_CH))
        self.params = [None] * len(self.layers)
        self.set_weights(initial_weights(self.layers, seed))
        self.status = torch.zeros(1, dtype=torch.int32, device=self.dev)
        self.step_count = 0
        self.grid = int(self.lib.fds_conv_wgrad_max_grid())
        self._bufs = {}

    # ------------------------------------------------------------------ weights
    def set_weights(self, ws):
        """Load float32 master weights [(w [9][cout][cin], b [cout]), ...] and reset
        the optimiser moments."""
        torch = self.torch
        for i, ((cin, cout, _, _), (w, b)) in enumerate(zip(self.layers, ws)):
            w = np.asarray(w, dtype=np.float32)
            if w.shape != (9, cout, cin):
                raise ValueError("layer %d weight shape %s, expected %s"
                                 % (i, w.shape, (9, cout, cin)))
            n = 9 * cout * cin + cout
            L = {"w": torch.tensor(w, device=self.dev).contiguous(),
                 "b": torch.tensor(np.asarray(b, dtype=np.float32), device=self.dev),
                 "m": torch.zeros(n, dtype=torch.float32, device=self.dev),
                 "v": torch.zeros(n, dtype=torch.float32, device=self.dev),
                 "wfwd": torch.empty(9 * cin * cout, dtype=torch.bfloat16, device=self.dev),
                 "wbwd": torch.empty(9 * cin * cout, dtype=torch.bfloat16, device=self.dev),
                 "partial": None}
            _capi.check(self.lib.fds_conv_pack(cin, cout, _ptr(L["w"]), _ptr(L["wfwd"]),
                                               _ptr(L["wbwd"]), _stream(torch)))
            self.params[i] = L
        self.step_count = 0

    def get_weights(self):
        return [(L["w"].cpu().numpy().copy(), L["b"].cpu().numpy().copy()) for L in self.params]

    # ------------------------------------------------------------------ buffers
    def buffers(self, batch, height, width, train):
        key = (batch, height, width, train)
        if key in self._bufs:
            return self._bufs[key]
        torch, dev = self.torch, self.dev
        bf, f32 = torch.bfloat16, torch.float32
        hw = (batch, height, width)
        nl = len(self.layers)
        c = lambda l: self.layers[l][1]
        cmax = max(max(l[0], l[1]) for l in self.layers)

        def act(ch, dtype=bf, zero=False):  # [batch][ch/8][height][width][8]
            f = torch.zeros if zero else torch.empty
            return f((batch, ch // 8, height, width, 8), dtype=dtype, device=dev)

        b = {"x": act(IN_CH, zero=True),
             "s": torch.zeros(hw + (4,), dtype=f32, device=dev),
             "t": torch.zeros(hw + (4,), dtype=f32, device=dev) if train else None,
             "scale": torch.zeros(batch, dtype=f32, device=dev),
             "y": act(OUT_CH, f32, zero=True)}
        if train:
            b["z"] = [act(c(l)) for l in range(nl - 1)]
            b["h"] = [act(c(l)) for l in range(nl - 1)]
            b["dy"] = act(OUT_CH)
            b["dz"] = [act(cmax) for _ in range(2)]
            b["dh"] = [act(cmax) for _ in range(2)]
            nparts = self.lib.fds_surr_loss_parts(batch, height, width)
            b["loss_parts"] = torch.zeros(nparts, dtype=f32, device=dev)
        else:
            b["h"] = [act(cmax) for _ in range(2)]
        self._bufs[key] = b
        return b

    def _conv(self, shape, l, mode, x, weight, out_z=None, out_h=None, out_f32=None,
              resid=None, zin=None, bias=None, cin=None, cout=None):
        a = _capi.FdsConvArgs()
        a.batch, a.height, a.width = shape
        a.cin = cin or self.layers[l][0]
        a.cout = cout or self.layers[l][1]
        a.dilation = self.layers[l][2]
        a.mode = mode
        a.x, a.weight, a.bias = _ptr(x), _ptr(weight), _ptr(bias)
        a.resid, a.zin = _ptr(resid), _ptr(zin)
        a.out_z, a.out_h, a.out_f32 = _ptr(out_z), _ptr(out_h), _ptr(out_f32)
        a.status = _ptr(self.status)
        _capi.check(self.lib.fds_conv3x3(C.byref(a), _stream(self.torch)))

    # ------------------------------------------------------------------ passes
    def forward(self, b, shape, train):
        """x -> y for the batch buffers ``b`` (``train`` keeps z and h for backward)."""
        h = b["x"]
        for l, (cin, cout, dil, kind) in enumerate(self.layers):
            L = self.params[l]
            if kind == "out":
                self._conv(shape, l, _capi.CONV_FWD_LINEAR, h, L["wfwd"], out_f32=b["y"],
                           bias=L["b"])
            else:
                out = b["h"][l] if train else b["h"][l % 2]
                self._conv(shape, l, _capi.CONV_FWD_GELU, h, L["wfwd"],
                           out_z=b["z"][l] if train else None, out_h=out,
                           resid=h if kind == "res" else None, bias=L["b"])
                h = out
        return b["y"]

    def _wgrad(self, shape, l, x, dz):
        L = self.params[l]
        cin, cout, dil, _ = self.layers[l]
        if L["partial"] is None:
            L["partial"] = self.torch.empty((self.grid, 9 * cout * cin + cout),
                                            dtype=self.torch.float32, device=self.dev)
        a = _capi.FdsWgradArgs()
        a.batch, a.height, a.width = shape
        a.cin, a.cout, a.dilation = cin, cout, dil
        a.x, a.dz, a.partial = _ptr(x), _ptr(dz), _ptr(L["partial"])
        a.grid = self.grid
        a.status = _ptr(self.status)
        _capi.check(self.lib.fds_conv3x3_wgrad(C.byref(a), _stream(self.torch)))

    def backward(self, b, shape):
        """Gradient partial sums of every layer from dy = dL/dy in ``b["dy"]``."""
        nl = len(self.layers)
        last = nl - 1
        self._wgrad(shape, last, b["h"][last - 1], b["dy"])
        cin, cout, _, _ = self.layers[last]
        cur = 0
        self._conv(shape, last, _capi.CONV_BWD_DATA, b["dy"], self.params[last]["wbwd"],
                   out_z=b["dz"][cur], out_h=b["dh"][cur], zin=b["z"][last - 1],
                   cin=cout, cout=cin)
        for l in range(last - 1, 0, -1):
            self._wgrad(shape, l, b["h"][l - 1], b["dz"][cur])
            cin, cout, _, _ = self.layers[l]
            prev_res = self.layers[l - 1][3] == "res"
            self._conv(shape, l, _capi.CONV_BWD_DATA, b["dz"][cur], self.params[l]["wbwd"],
                       out_z=b["dz"][1 - cur], out_h=b["dh"][1 - cur] if prev_res else None,
                       resid=b["dh"][cur], zin=b["z"][l - 1], cin=cout, cout=cin)
            cur = 1 - cur
        self._wgrad(shape, 0, b["x"], b["dz"][cur])

    def _adam(self, l, lr, grad_out=None, weight_decay=0.01):
        L = self.params[l]
        cin, cout, _, _ = self.layers[l]
        a = _capi.FdsAdamArgs()
        a.cin, a.cout, a.nparts = cin, cout, self.grid
        a.step = max(self.step_count, 1)
        a.lr, a.beta1, a.beta2, a.eps, a.weight_decay = lr, 0.9, 0.999, 1e-8, weight_decay
        a.grad_scale = 1.0
        a.partial = _ptr(L["partial"])
        a.weight, a.bias, a.m, a.v = _ptr(L["w"]), _ptr(L["b"]), _ptr(L["m"]), _ptr(L["v"])
        a.wfwd, a.wbwd = _ptr(L["wfwd"]), _ptr(L["wbwd"])
        a.grad_out = _ptr(grad_out)
        _capi.check(self.lib.fds_adamw(C.byref(a), _stream(self.torch)))

    def step(self, lr, weight_decay=0.01):
        """One AdamW step on every layer with the gradients of the last backward."""
        self.step_count += 1
        for l in range(len(self.layers)):
            self._adam(l, lr, weight_decay=weight_decay)

    def gradients(self):
        """The reduced gradients of the last backward: [(dw [9][cout][cin], db), ...]."""
        out = []
        for l, (cin, cout, _, _) in enumerate(self.layers):
            g = self.torch.empty(9 * cout * cin + cout, dtype=self.torch.float32, device=self.dev)
            self._adam(l, 0.0, grad_out=g)
            g = g.cpu().numpy()
            out.append((g[:9 * cout * cin].reshape(9, cout, cin), g[9 * cout * cin:]))
        return out

    def check_status(self):
        st = int(self.status.item())
        if st:
            self.status.zero_()
            raise _capi.FdsError(_capi.FDS_E_TIMEOUT,
                                 "a surrogate kernel reported status 0x%x" % st)


class SurrogateData:
    """Device-resident snapshots of many instances: state [inst][snap][3][n][n],
    media [inst][2][n][n], per-instance frequency and impedance scale."""

    def __init__(self, state, media, freq, zref):
        self.state, self.media, self.freq, self.zref = state, media, freq, zref
        self.count, self.nsnap = int(state.shape[0]), int(state.shape[1])
        self.n = int(state.shape[-1])

    def pairs(self):
        """Every (instance, snapshot) whose successor exists."""
        i, s = np.meshgrid(np.arange(self.count), np.arange(self.nsnap - 1), indexing="ij")
        return np.stack([i.reshape(-1), s.reshape(-1)], axis=1).astype(np.int32)


def media_tensors(specs, torch, dev):
    """Network medium channels for a list of surrogate_media specs."""
    n = specs[0]["nx"]
    media = np.empty((len(specs), 2, n, n), dtype=np.float32)
    freq = np.empty(len(specs), dtype=np.float32)
    zref = np.empty(len(specs), dtype=np.float32)
    for i, sp in enumerate(specs):
        c, rho = sp["c_map"], sp["rho_map"]
        media[i, 0] = c * sp["dt"] / sp["dx"]
        media[i, 1] = rho / rho.mean()
        freq[i] = (sp["frequency"] - 2.75e6) / 2.25e6
        zref[i] = float(np.mean(rho * c))
    return (torch.tensor(media, device=dev), torch.tensor(freq, device=dev),
            torch.tensor(zref, device=dev))


def _fd_runner(fields, warmup=True):
    """A captured 64-step batched solver run over ``fields`` (their state is restored
    after the warm-up launch that precedes the capture)."""
    r = BatchRunner(fields, JUMP)
    if warmup:
        saved = []
        for f in fields:
            eng = f._engine()
            saved.append([eng.buffers[nm][0].clone() for nm in f._stag_components])
        r.capture()
        for f, sv in zip(fields, saved):
            eng = f._engine()
            for nm, t in zip(f._stag_components, sv):
                eng.buffers[nm][0].copy_(t)
    else:
        r.capture(warmup=False)
    return r


def generate_data(count, nsnap, seed, n=256, jump=JUMP):
    """Snapshots from the batched FP64 solver: ``count`` media (surrogate_media),
    ``T_SRC`` solver steps through the source pulse, then ``nsnap`` snapshots
    ``jump`` steps apart (64, the network's jump; state copied on the device,
    float32)."""
    torch = require_cuda()
    dev = torch.device("cuda", torch.cuda.current_device())
    specs = workloads.surrogate_media(count, seed, n=n, nt=T_SRC + nsnap * jump + jump)
    fields = [workloads.build_field(s) for s in specs]
    simulate_batch(fields, T_SRC)
    state = torch.empty((count, nsnap, 3, n, n), dtype=torch.float32, device=dev)

    def snap(k):
        for i, f in enumerate(fields):
            eng = f._engine()
            for c, nm in enumerate(f._stag_components):
                state[i, k, c].copy_(eng.buffers[nm][0].view(n, n))

    snap(0)
    r = BatchRunner(fields, jump)
    r.capture()  # the warm-up launch is the first jump
    for k in range(1, nsnap):
        if k > 1:
            r.replay()
        snap(k)
    torch.cuda.synchronize()
    media, freq, zref = media_tensors(specs, torch, dev)
    del fields, r
    return SurrogateData(state, media, freq, zref)


def _surr_data(torch, data_state, media, freq, zref, nsnap, inst, snap, b, n, f64,
               target=True):
    d = _capi.FdsSurrData()
    d.count = int(inst.shape[0])
    d.height = d.width = n
    d.state_f64 = 1 if f64 else 0
    d.nsnap = nsnap
    d.edge_zero_p = 1
    d.inst, d.snap, d.state = _ptr(inst), _ptr(snap), _ptr(data_state)
    d.media, d.freq, d.zref = _ptr(media), _ptr(freq), _ptr(zref)
    d.scale, d.x, d.s = _ptr(b["scale"]), _ptr(b["x"]), _ptr(b["s"])
    d.t = _ptr(b["t"]) if target else None
    return d


def train(net, data, epochs=20, batch=32, lr=1e-3, seed=0, log_every=0, max_steps=None):
    """AdamW (weight decay 0.01) with a cosine learning-rate schedule from ``lr`` to
    0 over all steps, on every (t, t + 64) pair of ``data``, reshuffled each epoch.
    Returns the per-step mean squared error (normalised units) at the logged steps
    and the wall time of the loop."""
    torch = net.torch
    lib = net.lib
    pairs = data.pairs()
    iters = len(pairs) // batch
    total = epochs * iters if max_steps is None else min(max_steps, epochs * iters)
    rng = np.random.default_rng(seed)
    order = np.concatenate([pairs[rng.permutation(len(pairs))][:iters * batch]
                            for _ in range(epochs)])[:total * batch]
    inst_all = torch.tensor(order[:, 0].copy(), dtype=torch.int32, device=net.dev)
    snap_all = torch.tensor(order[:, 1].copy(), dtype=torch.int32, device=net.dev)
    n = data.n
    shape = (batch, n, n)
    b = net.buffers(batch, n, n, train=True)
    losses = []
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for it in range(total):
        sl = slice(it * batch, (it + 1) * batch)
        d = _surr_data(torch, data.state, data.media, data.freq, data.zref, data.nsnap,
                       inst_all[sl], snap_all[sl], b, n, f64=False)
        _capi.check(lib.fds_surr_pack(C.byref(d), _stream(torch)))
        net.forward(b, shape, train=True)
        _capi.check(lib.fds_surr_loss(C.byref(d), _ptr(b["y"]), _ptr(b["dy"]),
                                      _ptr(b["loss_parts"]), _stream(torch)))
        net.backward(b, shape)
        lr_t = 0.5 * lr * (1.0 + math.cos(math.pi * it / total))
        net.step(lr_t)
        if log_every and (it % log_every == 0 or it == total - 1):
            mse = float(b["loss_parts"].sum().item()) / (3.0 * batch * n * n)
            losses.append((it, mse))
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    net.check_status()
    return losses, wall


def jump(net, state, media, freq, zref, inst, chunk=64):
    """One surrogate jump, in place, of the instances ``inst`` (int32 device tensor)
    of a float64 state [inst][3][n][n]."""
    torch = net.torch
    n = int(state.shape[-1])
    for c0 in range(0, int(inst.shape[0]), chunk):
        ii = inst[c0:c0 + chunk]
        cnt = int(ii.shape[0])
        b = net.buffers(cnt, n, n, train=False)
        zeros = _zeros_i32(torch, cnt, net.dev)
        d = _surr_data(torch, state, media, freq, zref, 1, ii, zeros, b, n, f64=True,
                       target=False)
        _capi.check(net.lib.fds_surr_pack(C.byref(d), _stream(torch)))
        net.forward(b, (cnt, n, n), train=False)
        _capi.check(net.lib.fds_surr_unpack(C.byref(d), _ptr(b["y"]), _stream(torch)))


_ZEROS = {}


def _zeros_i32(torch, n, dev):
    """A cached device vector of n int32 zeros (the snapshot index of every sample)."""
    key = (str(dev), n)
    if key not in _ZEROS:
        _ZEROS[key] = torch.zeros(n, dtype=torch.int32, device=dev)
    return _ZEROS[key]


def rel_l2(net, a, b, zref, inst):
    """Per-instance relative L2 error of state a against b (energy-weighted)."""
    torch = net.torch
    n = int(a.shape[-1])
    out = torch.empty(2 * int(inst.shape[0]), dtype=torch.float64, device=net.dev)
    _capi.check(net.lib.fds_surr_compare(int(inst.shape[0]), n, n, _ptr(inst), _ptr(a), _ptr(b),
                                         _ptr(zref), _ptr(out), _stream(torch)))
    o = out.cpu().numpy().reshape(-1, 2)
    return np.sqrt(o[:, 0] / np.maximum(o[:, 1], 1e-300))


def evaluate_jumps(net, data, jumps, chunk=64):
    """Relative L2 error (rel_l2) of each instance of ``data`` after 1 .. ``jumps``
    chained network jumps from its snapshot 0, against the solver's snapshots:
    array [instances][jumps]."""
    torch = net.torch
    S = data.state[:, 0].to(torch.float64).contiguous()
    inst = torch.arange(data.count, dtype=torch.int32, device=net.dev)
    errs = []
    for j in range(jumps):
        jump(net, S, data.media, data.freq, data.zref, inst, chunk)
        ref = data.state[:, j + 1].to(torch.float64).contiguous()
        errs.append(rel_l2(net, S, ref, data.zref, inst))
    net.check_status()
    return np.stack(errs, axis=1)


def _alias_state(fields, n, torch, dev):
    """Batched float64 state [inst][3][n][n] that the fields' engines step in place
    (every runner must be built after this call: runners hold buffer addresses)."""
    S = torch.empty((len(fields), 3, n, n), dtype=torch.float64, device=dev)
    for i, f in enumerate(fields):
        if not f.matrices_assembled:
            f.assemble_matrices()
        eng = f._engine()
        eng._upload_coefs(torch, dev)
        eng._sync_state_to_device(torch, dev)
        for c, nm in enumerate(f._stag_components):
            S[i, c].copy_(eng.buffers[nm][0].view(n, n))
            eng.buffers[nm][0] = S[i, c].view(-1)
    return S


def _rollout_setup(fields, n, torch, dev):
    """Aliased state, a captured source-phase run (steps 0 .. T_SRC-1) and a captured
    64-step run for the source-free windows (planned at step T_SRC, where the
    source signal is zero, and replayed for every later window)."""
    S = _alias_state(fields, n, torch, dev)
    init = S.clone()
    r_src = BatchRunner(fields, T_SRC)
    r_src.capture()
    # every later runner (this one, and the fallback runners of a rollout) is
    # planned at step T_SRC, where the source signal is zero: the fields stay there
    for f in fields:
        f.step = T_SRC
    r = _fd_runner(fields)
    S.copy_(init)
    return S, r_src, r


def fd_rollout(specs, total_steps):
    """The plain FP64 batched solver over ``total_steps``: returns the final
    float64 state [inst][3][n][n] and the device time of the stepping (s)."""
    torch = require_cuda()
    dev = torch.device("cuda", torch.cuda.current_device())
    n = specs[0]["nx"]
    fields = [workloads.build_field(s) for s in specs]
    S, r_src, r = _rollout_setup(fields, n, torch, dev)
    njumps = (total_steps - T_SRC) // JUMP
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    r_src.replay()
    for _ in range(njumps):
        r.replay()
    e1.record()
    torch.cuda.synchronize()
    return S.clone(), e0.elapsed_time(e1) / 1e3


def surrogate_rollout(net, specs, total_steps, check_every=8, tol=0.01, chunk=64):
    """Rollout with the network and FD check windows.

    The solver runs the source phase (``T_SRC`` steps); then jumps of 64 steps.
    Jump j with j % check_every == 0 is a check: the network's jump and 64 solver
    steps start from the same state; instances whose relative L2 error exceeds
    ``tol`` continue with the solver alone; every instance keeps the solver's
    result of that window. Other jumps are network jumps for the instances still
    on the network and solver windows for the others.
    Returns (final state, device seconds, report dict)."""
    torch = require_cuda()
    dev = torch.device("cuda", torch.cuda.current_device())
    n = specs[0]["nx"]
    N = len(specs)
    fields = [workloads.build_field(s) for s in specs]
    media, freq, zref = media_tensors(specs, torch, dev)
    S, r_src, r_all = _rollout_setup(fields, n, torch, dev)
    Snn = torch.empty_like(S)
    njumps = (total_steps - T_SRC) // JUMP
    active = np.ones(N, dtype=bool)
    r_fb = None
    checks = []
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    r_src.replay()
    nn_jumps = fd_windows = 0
    for j in range(njumps):
        if j % check_every == 0:
            act = torch.tensor(np.nonzero(active)[0].astype(np.int32), device=dev)
            if act.numel():
                Snn.copy_(S)
                jump(net, Snn, media, freq, zref, act, chunk)
                nn_jumps += int(act.numel())
            r_all.replay()
            fd_windows += N
            if act.numel():
                err = rel_l2(net, Snn, S, zref, act)
                ids = np.nonzero(active)[0]
                checks.append((j, float(np.median(err)), float(err.max()),
                               int((err > tol).sum())))
                failed = ids[err > tol]
                if failed.size:
                    active[failed] = False
                    fb = [fields[i] for i in np.nonzero(~active)[0]]
                    r_fb = _fd_runner(fb, warmup=False)
        else:
            if active.any():
                act = torch.tensor(np.nonzero(active)[0].astype(np.int32), device=dev)
                jump(net, S, media, freq, zref, act, chunk)
                nn_jumps += int(act.numel())
            if (~active).any():
                r_fb.replay()
                fd_windows += int((~active).sum())
    e1.record()
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    net.check_status()
    report = {"checks": checks, "fallback_instances": int((~active).sum()),
              "network_jumps": nn_jumps, "solver_windows": fd_windows,
              "wall_s": wall}
    return S.clone(), e0.elapsed_time(e1) / 1e3, report
