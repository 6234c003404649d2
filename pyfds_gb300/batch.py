"""Batched time stepping: many independent 2-D fields advanced together.

``simulate_batch(fields, n)`` is equivalent to ``f.simulate(n)`` for every field
(pyfds/fields.py:67-95 once per field), but each time step is ONE kernel launch
covering every tile of every field (``fds_stag_batch_run``). The fields may differ
in grid size, media, boundaries and outputs; they must share the class, the
precision and the tile shape, be lossless 2-D fields (no absorption, not
``exact``) and stand at the same step.

``BatchRunner`` splits the call into an upload phase (descriptors, tables) and a
launch-only phase, so the launch sequence of a run can be captured once in a CUDA
graph and replayed (parameter sweeps that reset and rerun the same set of fields).
"""
import ctypes as C


from . import _capi
from ._engine import HostUpload, require_cuda


class BatchRunner:
    """Device-side plan of one batched run of ``num_steps`` steps."""

    def __init__(self, fields, num_steps, tile=None, stages=None):
        """``tile`` / ``stages`` override the fields' own (None: keep them; a field
        stage of 0 lets the engine choose, two steps per tile where the tile has a
        two-step kernel)."""
        if not fields:
            raise ValueError("empty batch")
        self.torch = require_cuda()
        self.fields = list(fields)
        self.num_steps = int(num_steps)
        f0 = self.fields[0]
        for f in self.fields:
            if type(f) is not type(f0) or f.precision != f0.precision:
                raise ValueError("batched fields must share class and precision")
            if f.step != f0.step:
                raise ValueError("batched fields must stand at the same step")
            if tile is not None:
                f.tile = tuple(tile)
            if stages is not None:
                f.stages = int(stages)
            if not f.matrices_assembled:
                f.assemble_matrices()
        self.step0 = int(f0.step)
        # every instance's coefficients, state and tables in one host-to-device copy;
        # tables are reused while an instance's boundaries and outputs are unchanged
        dev = self.torch.device("cuda", self.torch.cuda.current_device())
        up = HostUpload(self.torch, dev)
        self.plans = [f._engine().prepare(self.step0, self.num_steps, cache_tables=True,
                                          batched=True, up=up)
                      for f in self.fields]
        up.flush()
        n = len(self.fields)
        self.probs = (_capi.FdsStagProblem * n)(*[p["prob"] for p in self.plans])
        self.tables = (_capi.FdsStagTables * n)(*[p["tstruct"] for p in self.plans])
        self.states = (_capi.FdsStagState * n)()
        self.total_tiles = sum(p["geo"].ntiles for p in self.plans)
        lib = _capi.load()
        nbytes = lib.fds_stag_batch_workspace_bytes(n, self.total_tiles)
        self.workspace = self.torch.empty(nbytes, dtype=self.torch.uint8, device=dev)
        self._fill_states()
        self._call(_capi.BATCH_UPLOAD)
        self.graph = None

    # ------------------------------------------------------------------ helpers
    def _fill_states(self):
        for i, f in enumerate(self.fields):
            eng = f._engine()
            for k, name in enumerate(f._stag_components):
                cur, nxt = eng.buffers[name]
                self.states[i].cur[k] = cur.data_ptr()
                self.states[i].nxt[k] = nxt.data_ptr()

    def _call(self, mode):
        lib = _capi.load()
        store_flux = 1 if self.fields[0]._stag_family == _capi.FAMILY_ACOUSTIC else 0
        stream = self.torch.cuda.current_stream().cuda_stream
        code = lib.fds_stag_batch_run(self.probs, self.states, self.tables, len(self.fields),
                                      C.c_void_p(self.workspace.data_ptr()),
                                      self.workspace.numel(), self.step0, self.num_steps,
                                      store_flux, mode, C.c_void_p(stream))
        _capi.check(code)

    # ------------------------------------------------------------------ phases
    def launch(self):
        """Enqueue the steps (kernels only) on the current stream."""
        self._fill_states()
        self._call(_capi.BATCH_LAUNCH)

    def steps_per_launch(self):
        """2 when the batch runs two steps per tile (stages 3), else 1."""
        return 2 if int(self.probs[0].stages) == 3 else 1

    def launches(self):
        """Kernel launches of one run (launch_count)."""
        return launch_count(self.num_steps, self.steps_per_launch())

    def capture(self, warmup=True):
        """Capture ``launch`` in a CUDA graph (an even number of kernel launches keeps
        the ping-pong buffers of every replay in the same place: an even step count,
        or any count of two or more with two steps per tile). The warm-up launch
        before the capture (kernel attributes, caches) advances the fields;
        ``warmup=False`` skips it, for a process that has already launched this
        kernel variant."""
        if self.launches() % 2:
            raise ValueError("graph replays need an even number of launches (%d steps, %d "
                             "launches)" % (self.num_steps, self.launches()))
        torch = self.torch
        if warmup:
            self.launch()
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self._call(_capi.BATCH_LAUNCH)
        self.graph = g
        return g

    def replay(self):
        self.graph.replay()

    def finish(self):
        """Record outputs into ``Output.signals`` and advance every field's step; then
        report the fields whose potential came out non-finite. The status words and
        outputs of all instances come to the host in one copy each."""
        torch = self.torch
        engs = [f._engine() for f in self.fields]
        status = torch.cat([e.status for e in engs]).cpu().numpy()
        outs = [o for p in self.plans for o in p["outs"] if o is not None]
        flat = torch.cat([o.reshape(-1) for o in outs]).cpu().numpy() if outs else None
        pos = 0
        diverged = []
        for f, eng, plan, st in zip(self.fields, engs, self.plans, status):
            host_outs = []
            for o in plan["outs"]:
                if o is None:
                    host_outs.append(None)
                else:
                    host_outs.append(flat[pos:pos + o.numel()].reshape(tuple(o.shape)))
                    pos += o.numel()
            for name in f._stag_components:
                getattr(f, name)._where = "device"
            eng._last = plan
            if eng.finish(plan, status=st, host_outs=host_outs):
                diverged.append(f)
            f.step += self.num_steps
        for f in diverged:
            f._engine().report_nonfinite(f.step)


def launch_count(num_steps, steps_per_launch):
    """Kernel launches fds_stag_batch_run issues for a run: one per step, or with two
    steps per tile n2 launches of two steps, then n1 of one, with n2 + n1 even
    whenever there are two steps or more."""
    n = int(num_steps)
    if steps_per_launch == 1:
        return n
    n2, n1 = n // 2, n % 2
    if (n2 + n1) % 2 and n2 > 0:
        n2, n1 = n2 - 1, n1 + 2
    return n2 + n1


def simulate_batch(fields, num_steps=None, tile=None, stages=None):
    """Advance every field by ``num_steps`` (default: the first field's
    ``t.samples``) with one launch per step for the whole batch."""
    if not num_steps:
        num_steps = fields[0].t.samples
    r = BatchRunner(fields, num_steps, tile=tile, stages=stages)
    r.launch()
    # the launch swapped the state pointers in `states`; mirror it in the engines
    for i, f in enumerate(r.fields):
        eng = f._engine()
        for k, name in enumerate(f._stag_components):
            bufs = eng.buffers[name]
            if r.states[i].cur[k] != bufs[0].data_ptr():
                bufs.reverse()
    r.finish()
    return r
