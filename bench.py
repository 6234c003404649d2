"""Benchmark of the pyfds GB300 time-stepping path.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload acoustic2d|acoustic1d|axi|thermal|batched|flow|nonlinear1d]
                    [--precision f64|f32|f32_t64|dw]

One benchmark step is one full ``simulate()`` of the workload (default: the
2048 x 2048 water/steel Acoustic2D field, 4000 time steps, float64). Prints one
JSON line with Gcell-updates/s: ``value`` with the state resident in HBM (CUDA
events on the launching stream), ``e2e`` through the public API with host
buffers (host-to-device inputs and device-to-host outputs inside the timed
region), the roofline of the step kernel against the measured HBM peak, the CPU
baseline (the oracle restatement of the reference's scipy step, one replica per
host core, on a bounded sample) and the SM clocks sampled while timing.

``--impl reference`` times that CPU restatement alone (the reference itself is
pure Python/scipy and is not shipped): every step is a bounded sample of the same
workload on all host cores. Under torchrun only rank 0 runs it.
"""
import argparse
import json
import os
import re
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    # name: (workload builder, kwargs, bytes per cell-update at f64 / f32 / f32_t64;
    # double words (dw) move the float64 bytes)
    "acoustic2d": ("acoustic2d_steel_block", {}, {"f64": 64, "f32": 32, "dw": 64}),
    "acoustic1d": ("acoustic1d_water", {}, {"f64": 48, "f32": 24, "dw": 48}),
    "axi": ("axi_disc_source", {}, {"f64": 64, "f32": 32, "dw": 64}),
    "thermal": ("thermal2d_two_materials", {"nt": 2000}, {"f64": 32, "f32": 16, "f32_t64": 24, "dw": 32}),
    "batched": ("layered_media_batch", {}, {"f64": 64, "f32": 32, "dw": 64}),
    # the moving-medium shift adds 6 x 8 B per cell every `period` (10) steps
    "flow": ("acoustic_flow_block", {}, {"f64": 64, "f32": 32, "dw": 64}),
    # p, v, rho read + written, 4 coefficient arrays (the whole field stays in L1/L2)
    "nonlinear1d": ("ideal_gas_column", {}, {"f64": 80}),
}
# CPU sample per process and step of the reference arm (time steps), per workload
CPU_SAMPLE_STEPS = {"acoustic2d": 20, "acoustic1d": 2000, "axi": 8, "thermal": 10,
                    "batched": 60, "flow": 20, "nonlinear1d": 400}
L2_BYTES = 129 * 2 ** 20


def _l2_label(nbytes, what):
    """How the timed steps stand to the L2 cache: inputs larger than L2 stream from
    HBM on every step; a set that fits stays resident (no flush between steps)."""
    mb, l2 = nbytes / 2 ** 20, L2_BYTES / 2 ** 20
    if nbytes > L2_BYTES:
        return "inputs larger than L2 (%s %.0f MB > %.0f MB)" % (what, mb, l2)
    return "fits in L2 (%s %.2f MB <= %.0f MB; resident between steps, no flush)" % (what, mb, l2)


def _workload_label(wname, count=None, nt=None):
    """The workload string of a line's config, the same for both arms. For the
    layered-media batch `count` and `nt` default to its builder's defaults."""
    builder, kwargs, _ = WORKLOADS[wname]
    if wname != "batched":
        return "%s: %s" % (wname, builder)
    if count is None or nt is None:
        import inspect
        from pyfds_gb300 import workloads
        params = inspect.signature(getattr(workloads, builder)).parameters
        defaults = {k: v.default for k, v in params.items()}
        defaults.update(kwargs)
        count = defaults["count"] if count is None else count
        nt = defaults["nt"] if nt is None else nt
    return ("batched: %d layered-media Acoustic2D instances, n in [128, 1024] log-uniform, "
            "%d steps each" % (count, nt))


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def _init_replicas(backend="nccl"):
    """Join the process group of a multi-replica run (WORLD_SIZE > 1): one
    independent replica per rank, no data-path collective. Returns (ws, rank, local)."""
    ws, rank, local = _dist()
    if ws > 1:
        import torch
        import torch.distributed as dist
        if backend == "nccl":
            torch.cuda.set_device(local)
            dist.init_process_group("nccl", device_id=torch.device("cuda", local))
        else:
            dist.init_process_group(backend)
    return ws, rank, local


def _max_over_ranks(ms, device="cuda"):
    """The slowest replica's time: the job's time for weak-scaled replicas."""
    ws, _, _ = _dist()
    if ws == 1:
        return ms
    import torch
    import torch.distributed as dist
    t = torch.tensor([ms], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def _max_sm_mhz():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as fh:
            return float(json.load(fh).get("sm_max_mhz", 2070.0))
    return 2070.0


def _peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def _traffic_from_profiles(key, what="traffic_bytes_per_launch"):
    """A per-launch figure of the step kernel (DRAM bytes, or DFMA instructions with
    ``what="dfma_per_launch"``) from the committed ncu summaries."""
    pdir = os.path.join(ROOT, "profiles")
    if not os.path.isdir(pdir):
        return None
    pat = re.compile(r"%s\[%s\]\s*[:=]\s*([0-9.eE+]+)" % (re.escape(what), re.escape(key)))
    for name in sorted(os.listdir(pdir)):
        if not name.endswith((".md", ".txt")):
            continue
        with open(os.path.join(pdir, name)) as fh:
            m = pat.search(fh.read())
        if m:
            return float(m.group(1))
    return None


class ClockSampler:
    """nvidia-smi clock/throttle samples while the timed region runs."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.QUERY,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.out = ""
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                self.out, _ = self.proc.communicate()

    def summary(self):
        rows = [r.split(",") for r in (self.out or "").strip().splitlines() if r.count(",") >= 8]
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        sm = [float(r[1]) for r in rows if r[1].strip().replace(".", "").isdigit()]
        smax = [float(r[2]) for r in rows if r[2].strip().replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4)
                          if r[5 + k].strip().lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None, "reasons": reasons,
                "samples": len(rows)}


def cpu_sample(wname, steps_per_proc, procs, repeats=1, warmup=0):
    """Oracle replicas on `procs` host processes; returns (Gcell/s per repeat, cells)."""
    import multiprocessing as mp
    from oracle import bench_worker
    builder, kwargs, _ = WORKLOADS[wname]
    ctx = mp.get_context("spawn")
    if wname == "batched":
        # one batch instance per process, run concurrently
        with ctx.Pool(procs) as pool:
            vals = []
            tasks = [(builder, kwargs, k, steps_per_proc) for k in range(procs)]
            pool.map(bench_worker.run_batch_instance,
                     [(builder, kwargs, k, 1) for k in range(procs)], chunksize=1)
            for r in range(warmup + repeats):
                res = pool.map(bench_worker.run_batch_instance, tasks, chunksize=1)
                if r >= warmup:
                    vals.append(sum(c * steps_per_proc for c, _ in res) / max(t for _, t in res)
                                / 1e9)
            return vals, sum(c for c, _ in res)
    with ctx.Pool(procs, initializer=bench_worker.setup, initargs=(builder, kwargs)) as pool:
        cells = pool.apply(bench_worker.cells)
        pool.map(bench_worker.run, [1] * procs)  # touch every replica once
        vals = []
        for r in range(warmup + repeats):
            t0 = time.perf_counter()
            pool.map(bench_worker.run, [steps_per_proc] * procs, chunksize=1)
            dt = time.perf_counter() - t0
            if r >= warmup:
                vals.append(procs * cells * steps_per_proc / dt / 1e9)
    return vals, cells


def run_reference(args):
    ws, rank, _ = _dist()
    if rank != 0:
        return 0
    procs = os.cpu_count() or 1
    steps = CPU_SAMPLE_STEPS[args.workload]
    vals, cells = cpu_sample(args.workload, steps, procs, repeats=args.steps, warmup=args.warmup)
    v = statistics.median(vals)
    line = {"impl": "reference", "metric": "Gcell-updates/s", "value": v, "unit": "Gcell/s",
            "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": procs * cells * steps / (v * 1e9) * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded workload generator)",
            "config": {"workload": _workload_label(args.workload), "cells": cells,
                       "precision": "f64",
                       "parallelism": "replicas" if ws > 1 else "single GPU"},
            "cpu_baseline": {"value": v, "unit": "Gcell/s", "cores": procs, "kind": "port",
                             "sample": "%d time steps of the full-size workload per process, "
                                       "%d processes (one replica each), numpy oracle"
                                       % (steps, procs)},
            "e2e": {"value": v, "unit": "Gcell/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def run_batched(args):
    """The layered-media batch: one launch per step for all instances, the whole
    run replayed from a CUDA graph; e2e through simulate_batch with host buffers."""
    import torch
    ws, rank, local = _init_replicas()
    from pyfds_gb300 import workloads
    from pyfds_gb300.batch import BatchRunner, simulate_batch
    builder, kwargs, balg = WORKLOADS["batched"]
    kwargs = dict(kwargs)
    if args.time_steps:
        kwargs["nt"] = args.time_steps
    if args.batch:
        kwargs["count"] = args.batch
    specs = getattr(workloads, builder)(**kwargs)
    nt = int(specs[0]["steps"])
    fields = [workloads.build_field(sp, precision=args.precision) for sp in specs]
    cells = sum(f.num_points for f in fields)
    # 8-byte values stage 64 x 12 tiles four CTAs per SM (batched, two steps per tile:
    # float64 57.4 against 54.9 Gcell/s at 64 x 16)
    tile = tuple(int(v) for v in args.tile.split("x")) if args.tile else \
        ((64, 12) if args.precision in ("dw", "f64") else (64, 16))
    stages = args.stages or None  # None: the engine's choice (two steps per tile)
    if args.autotune:
        from pyfds_gb300.autotune import autotune_batch
        tile, stages = autotune_batch(fields, steps=20)
    runner = BatchRunner(fields, nt, tile=tile, stages=stages)
    stages = int(runner.probs[0].stages)
    runner.capture()

    def reset():
        for f in fields:
            for bufs in f._engine().buffers.values():
                for t in bufs:
                    t.zero_()

    def barrier():
        if ws > 1:
            import torch.distributed as dist
            dist.barrier()
        torch.cuda.synchronize()

    for _ in range(args.warmup):
        reset()
        runner.replay()
    barrier()
    stream = torch.cuda.current_stream()
    total_ms = 0.0
    with ClockSampler(torch.cuda.current_device()) as clk:
        for _ in range(args.steps):
            reset()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            runner.replay()
            e1.record(stream)
            e1.synchronize()
            total_ms += e0.elapsed_time(e1)
    barrier()
    ms = _max_over_ranks(total_ms / args.steps)
    value = ws * cells * nt / (ms * 1e-3) / 1e9
    spl = runner.steps_per_launch()
    step_ms = ms / nt
    launch_ms = step_ms * spl
    # e2e: the public API with host state and host outputs, every step
    e2e_steps = 0 if args.no_e2e else 1
    h2d = d2h = 0
    e2e_value = None
    if e2e_steps:
        # host inputs made once (as a caller's arrays), handed in again every call
        inputs = [{name: np.zeros(f.num_points) for name in f._stag_components} for f in fields]
        for rep in range(2):  # the first call warms the allocator and pinned staging
            barrier()
            t0 = time.perf_counter()
            for f, init in zip(fields, inputs):
                for name in f._stag_components:
                    getattr(f, name).values = init[name]
                f._coef_version += 1
                f.step = 0
                for o in f.pressure.outputs:
                    o.signals = []
            r = simulate_batch(fields, nt, tile=tile, stages=stages)
            finals = [f.pressure.values for f in fields]
            barrier()
            e2e_s = time.perf_counter() - t0
        e2e_value = ws * cells * nt / e2e_s / 1e9
        esz = 8 if args.precision in ("f64", "dw") else 4
        h2d = sum(f.num_points * esz * 5 for f in fields) + sum(
            int(p["tabs"]["blob"].numel()) for p in r.plans) + int(r.workspace.numel())
        d2h = sum(sum(o.numel() * 8 for o in p["outs"] if o is not None) for p in r.plans) + \
            sum(a.size * esz for a in finals)
    if rank != 0:
        return 0
    peak, peak_kind = _peaks()
    bpc = balg.get(args.precision)
    achieved = cells * bpc / (step_ms * 1e-3) / 1e9 if bpc else None
    line = {"metric": "Gcell-updates/s", "value": value, "unit": "Gcell/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": {"dw": "f32x2 (double-word)"}.get(args.precision, args.precision),
            "data": "synthetic (seeded layered media, no dataset)",
            "config": {"workload": _workload_label("batched", len(fields), nt),
                       "cells": cells, "time_steps_per_step": nt, "precision": args.precision,
                       "tile": "%dx%d" % tuple(tile), "stages": stages,
                       "launch": "one kernel per time step for all instances, whole run "
                                 "replayed from one CUDA graph",
                       "l2": _l2_label(cells * 6 * (8 if args.precision in ("f64", "dw")
                                                    else 4), "state"),
                       "parallelism": "replicas" if ws > 1 else "single GPU"},
            "e2e": {"value": e2e_value, "unit": "Gcell/s", "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h)},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak if achieved else None,
                         "traffic": _traffic_from_profiles(
                             "batched_%s%s" % (args.precision, "_tb2" if spl == 2 else "")),
                         "peak_kind": peak_kind, "kernel": "stag_batch_kernel",
                         "bytes_per_cell": bpc, "launch_ms": launch_ms, "steps_per_launch": spl,
                         **({"limit": "the field stays on chip (no DRAM traffic per step): "
                                      "the step is bound by the dependent FP64 chain, 4 DFMA "
                                      "per step at 64 cycles each on GB300"}
                            if resident_1d else {})},
            "clocks": clk.summary(),
            # per replay: the prologue, then one launch per step (per two with stages 3)
            "gpu_launches": int(args.steps * (runner.launches() + 1))}
    if ws == 1 and not args.no_cpu_baseline:
        procs = os.cpu_count() or 1
        steps = CPU_SAMPLE_STEPS["batched"]
        vals, _ = cpu_sample("batched", steps, procs, repeats=1)
        one, _ = cpu_sample("batched", steps, 1, repeats=1)
        line["cpu_baseline"] = {"value": vals[0], "unit": "Gcell/s", "cores": procs,
                                "kind": "port",
                                "sample": "%d time steps of one batch instance per process, "
                                          "%d processes (the first %d instances), numpy oracle"
                                          % (steps, procs, procs),
                                "one_process": {"value": one[0], "unit": "Gcell/s", "cores": 1,
                                                "sample": "%d time steps of instance 0 in one "
                                                          "process" % steps}}
    print(json.dumps(line), flush=True)
    return 0


def _batched_leg(precision, replays=2):
    """The layered-media batch (256 instances x 2000 steps, the batched workload) for
    the default line: device value of a graph replay (mean of ``replays``, inputs
    larger than L2), end to end through simulate_batch with host state and outputs
    (after one warm call), and the recorded outputs of the last replay."""
    import torch
    from pyfds_gb300 import workloads
    from pyfds_gb300.batch import BatchRunner, simulate_batch
    specs = workloads.layered_media_batch()
    nt = int(specs[0]["steps"])
    fields = [workloads.build_field(sp, precision=precision) for sp in specs]
    cells = sum(f.num_points for f in fields)
    tile = (64, 12) if precision in ("dw", "f64") else (64, 16)
    runner = BatchRunner(fields, nt, tile=tile)
    runner.capture()

    def reset():
        for f in fields:
            for bufs in f._engine().buffers.values():
                for t in bufs:
                    t.zero_()

    stream = torch.cuda.current_stream()
    total = 0.0
    for _ in range(replays):
        reset()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        runner.replay()
        e1.record(stream)
        e1.synchronize()
        total += e0.elapsed_time(e1)
    outs = [p["outs"][0].cpu().numpy().T.copy() for p in runner.plans]  # [points, steps]
    status = int(sum(int(f._engine().status.item()) for f in fields))
    ms = total / replays
    e2e_s = None
    # host inputs made once (as a caller's arrays), handed in again every call
    inputs = [{name: np.zeros(f.num_points) for name in f._stag_components} for f in fields]
    for rep in range(2):
        for f, init in zip(fields, inputs):
            for name in f._stag_components:
                getattr(f, name).values = init[name]
            f._coef_version += 1
            f.step = 0
            for o in f.pressure.outputs:
                o.signals = []
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        simulate_batch(fields, nt, tile=tile)
        _ = [f.pressure.values for f in fields]
        torch.cuda.synchronize()
        e2e_s = time.perf_counter() - t0
    del runner, fields
    torch.cuda.empty_cache()
    return {"value": cells * nt / (ms * 1e-3) / 1e9, "e2e": cells * nt / e2e_s / 1e9,
            "ms_per_run": ms, "e2e_s_per_run": e2e_s, "tile": "%dx%d" % tile,
            "kernel_status": status}, outs


def _batched_legs():
    """Pattern 2 on the default line: the batch in float64 and float32 (one launch per
    two steps for all 256 instances, replayed from a CUDA graph), with the float32
    outputs' error against float64 per instance."""
    specs_note = "256 layered media (sides 128..1024), 2000 steps, 16 outputs each"
    r64, o64 = _batched_leg("f64")
    r32, o32 = _batched_leg("f32")
    errs = [_errors(a, b) for a, b in zip(o32, o64)]
    return {"workload": specs_note, "f64": r64, "f32": r32,
            "speedup_f32_over_f64": r32["value"] / r64["value"],
            "speedup_f32_over_f64_e2e": r32["e2e"] / r64["e2e"],
            "f32_rel_l2_max": float(max(e["rel_l2_max"] for e in errs)),
            "f32_rel_l2_median": float(np.median([e["rel_l2_median"] for e in errs])),
            "f32_unreached_outputs": int(sum(e["unreached_outputs"] for e in errs)),
            "l2": "inputs larger than L2 (about 3 GB of float64 state and coefficients)"}


def _precision_legs(time_steps=0):
    """Pattern 1 on the default line: the axisymmetric disc (1024 x 4096, 6000 steps)
    and the thermal aluminium/polymer plate (4096^2, 50 000 steps, or ``time_steps``)
    in float32 against float64 on the same box, per recorded output (relative L2 of
    the outputs the wave or heat has reached; the others by their largest
    magnitude), with the speedup of one simulate call's device time."""
    from pyfds_gb300 import workloads
    out = {}
    for key, spec, comp, offset in (
            ("axi", workloads.axi_disc_source(), "pressure", 0.0),
            ("thermal", workloads.thermal2d_two_materials(), "temperature", 293.15)):
        nt = time_steps or spec["steps"]
        ref, t64, n = _timed_simulate(spec, "f64", nt, comp)
        sig, t32, _ = _timed_simulate(spec, "f32", nt, comp)
        e = _errors(sig, ref, offset=offset)
        e.pop("per_output")
        out[key] = dict({"workload": "%s %dx%d, %d steps%s"
                                     % (spec["kind"], spec["nx"], spec["ny"], nt,
                                        " (error of the rise above 293.15 K)" if offset else ""),
                         "f64_gcells": n * nt / t64 / 1e6, "f32_gcells": n * nt / t32 / 1e6,
                         "speedup_f32_over_f64": t64 / t32}, **e)
    return out


def _flow_due_steps(field, nt):
    """Steps of a moving-medium run on which some row shifts (a shift launch and the
    next step's pressure bounds follow the step kernel); the others step at rest."""
    per = np.unique(np.asarray(field.flow_t_deltas, dtype=np.int64))
    steps = np.arange(nt, dtype=np.int64)
    due = np.zeros(nt, dtype=bool)
    for f in per:
        due |= (steps == steps) if f == 0 else (steps % f == 0)
    return int(due.sum())


def _timed_simulate(spec, precision, nsteps, comp, tile=None):
    """Run a workload on the GPU; returns ([points, steps] outputs, ms on the device)."""
    import torch
    from pyfds_gb300 import workloads
    f = workloads.build_field(spec, precision=precision, tile=tile)
    f.assemble_matrices()
    eng = f._engine()
    plan = eng.prepare(0, nsteps)
    torch.cuda.synchronize()
    s = torch.cuda.current_stream()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(s)
    eng.launch(plan)
    e1.record(s)
    torch.cuda.synchronize()
    eng.finish(plan)
    sig = np.array(getattr(f, comp).outputs[0].signals, dtype=np.float64)
    return sig, e0.elapsed_time(e1), f.num_points


def _errors(sig, ref, offset=0.0, floor=1e-6):
    """Per-output relative L2 errors of sig against ref (of sig - offset if given).

    Outputs whose reference norm is below ``floor`` times the largest one have not
    been reached by the signal (float64 keeps values of 1e-300 there that float32
    flushes to zero); they are counted separately with their largest magnitudes."""
    a_all = np.asarray(sig, dtype=np.float64) - offset
    b_all = np.asarray(ref, dtype=np.float64) - offset
    norms = np.linalg.norm(b_all, axis=1)
    scale = norms.max() if norms.size else 0.0
    errs, unreached = [], []
    for a, b, nb in zip(a_all, b_all, norms):
        if nb > floor * scale and nb > 0:
            errs.append(float(np.linalg.norm(a - b) / nb))
        else:
            unreached.append(max(float(np.abs(a).max()), float(np.abs(b).max())))
    e = np.array(errs) if errs else np.zeros(1)
    return {"rel_l2_max": float(e.max()), "rel_l2_median": float(np.median(e)),
            "outputs": len(errs), "per_output": [round(x, 9) for x in errs],
            "unreached_outputs": len(unreached),
            "unreached_max_abs": max(unreached) if unreached else 0.0}


def run_study(args):
    """Precision study: float32 paths against the float64 GPU path (itself pinned to
    the reference), per recorded output, with the speedup."""
    import torch
    from pyfds_gb300 import workloads
    out = []
    if args.study in ("precision", "axi"):
        spec = workloads.axi_disc_source()
        nt = spec["steps"]
        ref, t64, n = _timed_simulate(spec, "f64", nt, "pressure")
        s32, t32, _ = _timed_simulate(spec, "f32", nt, "pressure")
        line = {"study": "Acoustic3DAxi 1024x4096 water, disc source, %d steps: f32 vs f64" % nt,
                "f64_gcells": n * nt / t64 / 1e6, "f32_gcells": n * nt / t32 / 1e6,
                "speedup_f32_over_f64": t64 / t32}
        line.update(_errors(s32, ref))
        out.append(line)
    if args.study in ("precision", "thermal"):
        spec = workloads.thermal2d_two_materials()
        nt = args.time_steps or spec["steps"]
        ref, t64, n = _timed_simulate(spec, "f64", nt, "temperature")
        for prec in ("f32_t64", "f32"):
            sig, tp, _ = _timed_simulate(spec, prec, nt, "temperature")
            line = {"study": "Thermal2D 4096^2 aluminium/polymer, %d steps: %s vs f64 "
                             "(error of the temperature rise above 293.15 K)" % (nt, prec),
                    "f64_gcells": n * nt / t64 / 1e6, "gcells": n * nt / tp / 1e6,
                    "speedup_over_f64": t64 / tp}
            line.update(_errors(sig, ref, offset=293.15))
            out.append(line)
    if args.study in ("precision", "batched"):
        from pyfds_gb300.batch import simulate_batch
        specs = workloads.layered_media_batch()
        nt = specs[0]["steps"]
        res = {}
        for prec in ("f64", "f32"):
            fields = [workloads.build_field(sp, precision=prec) for sp in specs]
            torch.cuda.synchronize()
            import time as _t
            t0 = _t.perf_counter()
            simulate_batch(fields, nt, tile=(32, 32))
            torch.cuda.synchronize()
            res[prec] = (_t.perf_counter() - t0,
                         [np.array(f.pressure.outputs[0].signals) for f in fields])
        cells = sum(workloads.build_field(sp).num_points for sp in specs[:0]) or \
            sum(sp["nx"] * sp["ny"] for sp in specs)
        errs = [_errors(a, b)["rel_l2_max"] for a, b in zip(res["f32"][1], res["f64"][1])]
        unreached = sum(_errors(a, b)["unreached_outputs"]
                        for a, b in zip(res["f32"][1], res["f64"][1]))
        line = {"study": "batched layered media, %d instances x %d steps: f32 vs f64 "
                         "(end-to-end simulate_batch)" % (len(specs), nt),
                "f64_gcells_e2e": cells * nt / res["f64"][0] / 1e9,
                "f32_gcells_e2e": cells * nt / res["f32"][0] / 1e9,
                "speedup_f32_over_f64_e2e": res["f64"][0] / res["f32"][0],
                "rel_l2_max_over_instances": float(np.max(errs)),
                "rel_l2_median_over_instances": float(np.median(errs)),
                "unreached_outputs": int(unreached)}
        out.append(line)
    for line in out:
        print(json.dumps(line), flush=True)
    return 0


def _bf16_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as fh:
            d = json.load(fh)
        return float(d["bf16_tflops"]), float(d["bf16_tflops_sustained"]), "measured"
    return 1900.0, 1700.0, "fallback"


def run_surrogate(args):
    """Learned surrogate: snapshots from the batched FP64 solver, training on the
    GPU with the tensor-core kernels, then a rollout with FD check windows against
    the plain FP64 batched solver on unseen media."""
    import torch
    from pyfds_gb300 import surrogate as S
    from pyfds_gb300 import workloads
    torch.cuda.init()
    n = 256
    t0 = time.perf_counter()
    data = S.generate_data(args.surr_instances, args.surr_snaps, seed=11, n=n)
    t_data = time.perf_counter() - t0
    pairs = len(data.pairs())
    net = S.ConvNet(seed=0)
    # kernel throughput: one forward and one training iteration on a batch of 32
    B = args.surr_batch
    b = net.buffers(B, n, n, train=True)
    shape = (B, n, n)
    flops_fwd = sum(2 * 9 * cin * cout for cin, cout, _, _ in net.layers) * B * n * n
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    for _ in range(3):
        net.forward(b, shape, train=True)
    torch.cuda.synchronize()
    ev[0].record()
    for _ in range(10):
        net.forward(b, shape, train=True)
    ev[1].record()
    torch.cuda.synchronize()
    t_fwd = ev[0].elapsed_time(ev[1]) / 10 / 1e3
    inf = net.buffers(B, n, n, train=False)
    inf["x"].copy_(b["x"])
    ev[2].record()
    for _ in range(10):
        net.forward(inf, shape, train=False)
    ev[3].record()
    torch.cuda.synchronize()
    t_inf = ev[2].elapsed_time(ev[3]) / 10 / 1e3
    b["dy"].zero_()
    ev[0].record()
    for _ in range(5):
        net.backward(b, shape)
    ev[1].record()
    torch.cuda.synchronize()
    t_bwd = ev[0].elapsed_time(ev[1]) / 5 / 1e3
    net = S.ConvNet(seed=0)
    if args.surr_load:
        w = np.load(args.surr_load)
        net.set_weights([(w["w%d" % l], w["b%d" % l]) for l in range(len(net.layers))])
        losses, t_train = [], 0.0
    else:
        losses, t_train = S.train(net, data, epochs=args.surr_epochs, batch=B, lr=1e-3, seed=0,
                                  log_every=max(1, pairs // B))
        if args.surr_save:
            np.savez(args.surr_save, **{("%s%d" % (k, l)): a
                                        for l, wb in enumerate(net.get_weights())
                                        for k, a in zip(("w", "b"), wb)})
    steps = len(losses) and losses[-1][0] + 1
    del data
    torch.cuda.empty_cache()
    specs = workloads.surrogate_media(args.surr_eval, seed=99, n=n, nt=args.surr_steps)
    s_fd, t_fd, = S.fd_rollout(specs, args.surr_steps)
    torch.cuda.empty_cache()
    zref = S.media_tensors(specs, torch, torch.device("cuda", 0))[2]
    idx = torch.arange(len(specs), dtype=torch.int32, device="cuda")
    rollouts = {}
    for tol in (0.01, float("inf")):
        s_nn, t_nn, rep = S.surrogate_rollout(net, specs, args.surr_steps, check_every=8,
                                              tol=tol)
        err = S.rel_l2(net, s_nn, s_fd, zref, idx)
        rollouts[tol] = (t_nn, rep, err)
        del s_nn
        torch.cuda.empty_cache()
    t_nn, rep, err = rollouts[0.01]
    t_acc, rep_acc, err_acc = rollouts[float("inf")]
    peak, peak_s, how = _bf16_peak()
    iters = steps
    train_flops = 3 * flops_fwd * iters
    line = {"study": "learned surrogate: 8-layer dilated residual CNN, 48 ch, bf16 tcgen05 "
                     "kernels; %d pairs at %dx%d, K=64; eval %d unseen media x %d steps"
                     % (pairs, n, n, len(specs), args.surr_steps),
            "data_generation_s": t_data, "pairs": pairs,
            "forward_ms_batch%d" % B: t_fwd * 1e3,
            "forward_tflops": flops_fwd / t_fwd / 1e12,
            "inference_tflops": flops_fwd / t_inf / 1e12,
            "backward_ms_batch%d" % B: t_bwd * 1e3,
            "backward_tflops": 2 * flops_fwd / t_bwd / 1e12,
            "peak_bf16_tflops": peak, "peak_note": how + " (burst, cuBLAS)",
            "train_steps": iters, "train_s": t_train,
            "train_tflops": train_flops / t_train / 1e12 if t_train else None,
            "loss_first": losses[0][1] if losses else None,
            "loss_last": losses[-1][1] if losses else None,
            "loss_per_epoch": [l for _, l in losses],
            "fd_rollout_s": t_fd, "surrogate_rollout_s": t_nn,
            "speedup_vs_fd64": t_fd / t_nn,
            "final_rel_l2_median": float(np.median(err)), "final_rel_l2_max": float(np.max(err)),
            "final_rel_l2_p90": float(np.percentile(err, 90)),
            "fallback_instances": rep["fallback_instances"],
            "network_jumps": rep["network_jumps"], "solver_windows": rep["solver_windows"],
            "checks": rep["checks"],
            "accept_all": {"note": "the same rollout with every check accepted (no fallback)",
                           "surrogate_rollout_s": t_acc, "speedup_vs_fd64": t_fd / t_acc,
                           "final_rel_l2_median": float(np.median(err_acc)),
                           "final_rel_l2_p90": float(np.percentile(err_acc, 90)),
                           "final_rel_l2_max": float(np.max(err_acc)),
                           "checks": rep_acc["checks"]}}
    print(json.dumps(line), flush=True)
    return 0


def run_surrogate_precision(args):
    """What limits the surrogate's jump error: the tcgen05 kernels (bf16 storage of
    activations and operands) against a float32 twin of the same network trained on
    the same pairs in the same order with the same schedule (PyTorch convolutions,
    TF32 off), and the twin trained on a loss over two chained jumps. Errors are the
    rollout check's relative L2 on unseen media after 1 .. 8 chained jumps from the
    first source-free snapshot; "no network" keeps the state unchanged."""
    import torch
    from pyfds_gb300 import surrogate as S
    from pyfds_gb300 import surrogate_twin as T
    torch.cuda.init()
    n = 256
    jump = args.surr_jump
    data = S.generate_data(args.surr_instances, args.surr_snaps, seed=11, n=n, jump=jump)
    ev = S.generate_data(args.surr_eval_media, 9, seed=99, n=n, jump=jump)
    jumps = 8

    def summary(err):
        return {"median_per_jump": [float(np.median(err[:, j])) for j in range(err.shape[1])],
                "p90_first_jump": float(np.percentile(err[:, 0], 90)),
                "max_first_jump": float(np.max(err[:, 0])),
                "within_1pct_first_jump": int((err[:, 0] <= 0.01).sum())}

    with torch.no_grad():
        s0, _ = T._normalise(ev.state[:, 0], ev.zref[:, None, None])
        ident = []
        for k in range(1, jumps + 1):
            tk, _ = T._normalise(ev.state[:, k], ev.zref[:, None, None])
            ident.append((torch.linalg.vector_norm((s0 - tk).flatten(1), dim=1)
                           / torch.linalg.vector_norm(tk.flatten(1), dim=1)).cpu().numpy())
        ident = np.stack(ident, axis=1)
    line = {"study": "surrogate precision: bf16 tcgen05 kernels vs a float32 twin; %d pairs "
                     "at %dx%d, K=%d; eval %d unseen media, chained jumps"
                     % (len(data.pairs()), n, n, jump, ev.count),
            "epochs": args.surr_epochs, "batch": args.surr_batch, "jump": jump,
            "no_network": summary(ident)}
    variants = [v for v in args.surr_variants.split(",") if v]
    for v in variants:
        torch.cuda.empty_cache()
        if v == "bf16":
            net = S.ConvNet(seed=0)
            losses, wall = S.train(net, data, epochs=args.surr_epochs, batch=args.surr_batch,
                                   lr=1e-3, seed=0, log_every=max(1, len(data.pairs())
                                                                  // args.surr_batch))
            err = S.evaluate_jumps(net, ev, jumps)
            del net
        else:
            unroll = 2 if v == "fp32x2" else 1
            tw = T.TwinNet(seed=0)
            losses, wall = T.train(tw, data, epochs=args.surr_epochs, batch=args.surr_batch,
                                   lr=1e-3, seed=0, unroll=unroll)
            err = T.evaluate(tw, ev, jumps)
            del tw
        line[v] = dict(summary(err), train_s=wall, loss_last=losses[-1][1] if losses else None,
                       loss_per_epoch=[l for _, l in losses])
    print(json.dumps(line), flush=True)
    return 0


def run_coupling_study(args):
    """ThermoAcoustic1D (1000 cells, coupling every 3 steps, accumulated): the
    one-call library stepping against the reference's loop (fields stepped one by
    one, coupling on the host copies), same field, same steps."""
    import torch
    import pyfds_gb300
    from oracle import scenarios
    from pyfds_gb300 import workloads
    out = {"study": "ThermoAcoustic1D 1000 cells, stepping 3 (accumulated), 500 steps"}
    for native in (True, False):
        spec = scenarios.coupled_scenario(5, "thermoacoustic3", nx=1000, steps=2000)
        obj = scenarios.build_coupled(pyfds_gb300, spec, workloads.build_field)
        if not native:
            obj._native_path = lambda: False
        obj.simulate(10)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        obj.simulate(500)
        torch.cuda.synchronize()
        us = (time.perf_counter() - t0) / 500 * 1e6
        out["native_us_per_step" if native else "step_by_step_us_per_step"] = us
    out["speedup"] = out["step_by_step_us_per_step"] / out["native_us_per_step"]
    print(json.dumps(out), flush=True)
    return 0


def run_surrogate_iter(args):
    """A few surrogate training iterations (batch 32 at 256^2, a 32-pair solver
    dataset) after 3 warm-up iterations: the small case the kernel profiles use."""
    import torch
    from pyfds_gb300 import surrogate as S
    torch.cuda.init()
    data = S.generate_data(args.surr_batch, 2, seed=3, n=256)
    net = S.ConvNet(seed=0)
    S.train(net, data, epochs=args.warmup, batch=args.surr_batch, lr=1e-3, seed=0)
    _, wall = S.train(net, data, epochs=args.steps, batch=args.surr_batch, lr=1e-3, seed=1)
    print(json.dumps({"study": "surrogate training iterations", "batch": args.surr_batch,
                      "iterations": args.steps, "ms_per_iteration": wall / args.steps * 1e3}))
    return 0


# workloads whose float64 line also times the double-word step (same field, same box)
DW_WORKLOADS = ("acoustic2d", "acoustic1d", "axi", "thermal")


def _reset_state(field, eng, spec, dev):
    """Zero the device state of a field and load the workload's initial values."""
    import torch
    from pyfds_gb300._engine import split_dw
    for name in field._stag_components:
        for t in eng.buffers[name]:
            t.zero_()
        if name in (spec.get("init") or {}):
            v = np.asarray(spec["init"][name], dtype=np.float64).reshape(-1)
            if field.precision == "dw":
                v = split_dw(v)
            eng.buffers[name][0].copy_(torch.as_tensor(v, device=dev,
                                                       dtype=eng.buffers[name][0].dtype))


def _double_word_leg(args, spec, nt, ref_outs, barrier, bytes_per_cell):
    """The same workload in double-word precision: throughput (same timing as the
    float64 line), its step kernel's launch time and HBM fraction, and the error of
    its outputs against the float64 outputs of this run (relative L2 per output the
    wave reached, i.e. norm >= 1e-6 of the largest; the others by absolute error
    relative to the largest output's norm)."""
    import torch
    from pyfds_gb300 import workloads
    f = workloads.build_field(spec, precision="dw")
    f.assemble_matrices()
    eng = f._engine()
    dev = torch.device("cuda", torch.cuda.current_device())
    plan = eng.prepare(0, nt)
    for _ in range(args.warmup):
        _reset_state(f, eng, spec, dev)
        eng.launch(plan)
    barrier()
    stream = torch.cuda.current_stream()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    ev[0].record(stream)
    for _ in range(args.steps):
        _reset_state(f, eng, spec, dev)
        eng.launch(plan)
    ev[1].record(stream)
    barrier()
    ms = ev[0].elapsed_time(ev[1]) / args.steps
    _reset_state(f, eng, spec, dev)
    ev[2].record(stream)
    eng.launch(plan)
    ev[3].record(stream)
    torch.cuda.synchronize()
    step_kernel_ms = ev[2].elapsed_time(ev[3]) / nt  # per time step
    spl = {3: 2, 4: nt}.get(eng.stages(), 1)  # steps per launch
    # the kernels' status word (a bounded wait that gave up leaves a tile's outputs
    # unwritten): checked here because launch() alone does not
    status = int(eng.status.item())
    rows = [r for o in plan["outs"] if o is not None for r in o.cpu().numpy().T]
    refs = [r for o in ref_outs if o is not None for r in o.T]
    top = max((float(np.linalg.norm(r)) for r in refs), default=0.0)
    worst, unreached, worst_abs = 0.0, 0, 0.0
    nonfinite = sum(int(not np.all(np.isfinite(a))) for a in rows)
    for a, b in zip(rows, refs):
        nb = float(np.linalg.norm(b))
        if nb >= 1e-6 * top and nb > 0:
            worst = max(worst, float(np.linalg.norm(a - b)) / nb)
        else:
            unreached += 1
            worst_abs = max(worst_abs, float(np.linalg.norm(a - b)) / top if top else 0.0)
    if nonfinite:  # never report a NaN comparison as agreement
        worst = worst_abs = None
    cells = f.num_points
    peak, _ = _peaks()
    achieved = cells * bytes_per_cell / (step_kernel_ms * 1e-3) / 1e9 if bytes_per_cell else None
    geo = eng._geometry()
    return {"value": cells * nt / (ms * 1e-3) / 1e9, "unit": "Gcell/s", "ms_per_step": ms,
            "dtype": "f32x2 (double-word)", "tile": "%dx%d" % (geo.tx, geo.ty),
            "launch_ms": step_kernel_ms * spl, "steps_per_launch": spl, "achieved_gbs": achieved,
            "hbm_frac": achieved / peak if achieved and peak else None,
            "max_rel_l2_vs_f64": worst, "unreached_outputs": unreached,
            "unreached_max_abs_vs_largest": worst_abs, "nonfinite_outputs": nonfinite,
            "kernel_status": status}


def run_ours(args):
    import torch
    ws, rank, local = _init_replicas()
    dev = torch.device("cuda", torch.cuda.current_device())
    from pyfds_gb300 import workloads
    builder, kwargs, balg = WORKLOADS[args.workload]
    kwargs = dict(kwargs)
    if args.time_steps:
        kwargs["nt"] = args.time_steps
    spec = getattr(workloads, builder)(**kwargs)
    nt = int(spec["steps"])
    tile = tuple(int(v) for v in args.tile.split("x")) if args.tile else None
    field = workloads.build_field(spec, precision=args.precision, tile=tile)
    field.stages = args.stages
    field.assemble_matrices()
    eng = field._engine()
    cells = field.num_points

    def barrier():
        if ws > 1:
            import torch.distributed as dist
            dist.barrier()
        torch.cuda.synchronize()

    def zero_state():
        _reset_state(field, eng, spec, dev)

    plan = eng.prepare(0, nt)
    for _ in range(args.warmup):
        zero_state()
        eng.launch(plan)
    barrier()
    stream = torch.cuda.current_stream()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    with ClockSampler(dev.index) as clk:
        ev0.record(stream)
        for _ in range(args.steps):
            zero_state()
            eng.launch(plan)
        ev1.record(stream)
        barrier()
    ms = _max_over_ranks(ev0.elapsed_time(ev1) / args.steps, device=dev)
    value = ws * cells * nt / (ms * 1e-3) / 1e9
    # step kernel alone: average launch over a timed run without the state reset
    ev2 = torch.cuda.Event(enable_timing=True)
    ev3 = torch.cuda.Event(enable_timing=True)
    zero_state()
    ev2.record(stream)
    eng.launch(plan)
    ev3.record(stream)
    torch.cuda.synchronize()
    # time per step of the step kernel (two steps per launch with stages 3)
    step_kernel_ms = ev2.elapsed_time(ev3) / nt
    kernel_status = int(eng.status.item()) if eng.status is not None else 0
    if kernel_status:
        raise RuntimeError("a kernel reported status 0x%x during the timed runs" % kernel_status)
    st_used = eng.stages()
    from pyfds_gb300 import _capi as _c
    # a 1-D field of at most 8192 cells runs every step of a call in one launch: from
    # 256 cells on the warps of a thread-block cluster (up to 4096 cells, else on
    # shared-memory windows of a cluster), below that in one CTA
    resident_1d = (args.workload != "nonlinear1d" and cells <= 8192 and st_used in (0, 4)
                   and not field._stag_flags() & _c.FLAG_HAS_V)
    kernel_1d = ("stag_1d_warp_kernel (every step of the call on the warps of one "
                 "thread-block cluster, a cell per lane)" if 256 <= cells <= 4096 else
                 "stag_1d_cluster_kernel (every step of the call on one thread-block "
                 "cluster)" if cells > 4096 else
                 "stag_1d_resident_kernel (every step of the call in one CTA)")
    # steps per launch: two with two steps per tile, every step of the call for the
    # wavefront kernel (stages 4, one launch per simulate call), else one
    spl = 2 if st_used == 3 else (nt if st_used == 4 or resident_1d else 1)
    launch_ms = step_kernel_ms * spl
    ref_outs = [o.cpu().numpy() if o is not None else None for o in plan["outs"]]
    dword = None
    if args.precision == "f64" and not args.no_dw and args.workload in DW_WORKLOADS:
        dword = _double_word_leg(args, spec, nt, ref_outs, barrier, balg.get("dw"))
    # ---------------- e2e through the public API with host buffers
    e2e_steps = 0 if args.no_e2e else max(1, args.steps)
    host_init = {name: np.zeros(cells) for name in field._stag_components}
    for name, v in (spec.get("init") or {}).items():
        host_init[name] = np.array(v, dtype=np.float64)
    for o in (field.pressure.outputs if hasattr(field, "pressure") else []):
        o.signals = []
    h2d = d2h = 0

    def e2e_call():
        for name in field._stag_components:
            getattr(field, name).values = host_init[name]  # (the setter keeps a reference)
        field._coef_version += 1  # coefficients count as this step's inputs
        field.step = 0
        field.simulate(nt)
        pot = getattr(field, field._stag_components[0])
        out = pot.values  # device -> host read of the final potential
        for o in pot.outputs:
            o.signals = []
        return out

    if e2e_steps:
        e2e_call()  # untimed: the first call compiles the tables and warms the allocators
    barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        result = e2e_call()
    barrier()
    e2e_s = (time.perf_counter() - t0) / max(e2e_steps, 1)
    if not e2e_steps:
        result = np.zeros(0)
    last = eng._last
    tab_bytes = int(last["tabs"]["blob"].numel())
    coef_bytes = sum(t.numel() * t.element_size() for t in eng.coef_tensors.values())
    state_bytes = sum(eng.buffers[n][0].numel() * eng.buffers[n][0].element_size()
                      for n in field._stag_components)
    out_bytes = sum(o.numel() * 8 for o in last["outs"] if o is not None)
    h2d = state_bytes + coef_bytes + tab_bytes
    # the final potential comes back as float64 for double words (joined on the device)
    d2h = out_bytes + result.size * (8 if args.precision == "dw" else
                                     eng.buffers[field._stag_components[0]][0].element_size())
    e2e_value = ws * cells * nt / e2e_s / 1e9 if e2e_steps else None
    if rank != 0:
        return 0
    peak, peak_kind = _peaks()
    bpc = balg.get(args.precision)
    # algorithmic bytes per cell update (one read and one write of the state, one read
    # of the coefficients per step) over the time per step; with two steps per launch
    # the kernel moves about half of that from DRAM (see "traffic", per launch)
    achieved = cells * bpc / (step_kernel_ms * 1e-3) / 1e9 if bpc else None
    pkey = "%s_%s%s" % (args.workload, args.precision,
                        {3: "_tb2", 4: "_wave"}.get(st_used, ""))
    traffic = _traffic_from_profiles(pkey)
    if st_used == 4:
        # the capture covers a shorter call: its DRAM bytes per step, scaled to this
        # launch's steps (the traffic grows with the steps a launch runs)
        per_step = _traffic_from_profiles(pkey, "traffic_bytes_per_step")
        traffic = per_step * nt if per_step else None
    line = {"metric": "Gcell-updates/s", "value": value, "unit": "Gcell/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": {"f64": "f64", "f32": "f32", "f32_t64": "f32+f64",
                      "dw": "f32x2 (double-word)"}[args.precision],
            "data": "synthetic (seeded workload generator, no dataset)",
            "config": {"workload": _workload_label(args.workload), "nx": field._nx,
                       "ny": field._ny, "cells": cells, "time_steps_per_step": nt,
                       "precision": args.precision, "tile": "%dx%d" % (eng._geometry().tx, eng._geometry().ty),
                       "stages": eng.stages(),
                       "l2": _l2_label(state_bytes * 2 + coef_bytes, "working set"),
                       "parallelism": "replicas" if ws > 1 else "single GPU"},
            "e2e": {"value": e2e_value, "unit": "Gcell/s", "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h)},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak if achieved else None,
                         "traffic": traffic, "peak_kind": peak_kind,
                         "kernel": {"flow": "stag_step_kernel per step; flow_shift_kernel and "
                                            "the next step's prologue on steps where a "
                                            "row shifts",
                                    "nonlinear1d": "nl1d_kernel (every step in one launch; the "
                                                   "field stays in L1/L2)"}.get(
                                        args.workload,
                                        kernel_1d if resident_1d else
                                        {3: "stag_tb2_kernel", 4: "stag_wave_kernel (every "
                                         "step of the call in one launch)"}.get(
                                            st_used, "stag_step_kernel")),
                         "bytes_per_cell": bpc, "launch_ms": launch_ms, "steps_per_launch": spl,
                         **({"limit": "the field stays on chip (no DRAM traffic per step): "
                                      "the step is bound by the dependent FP64 chain, 4 DFMA "
                                      "per step at 64 cycles each on GB300"}
                            if resident_1d else {})},
            "clocks": clk.summary(),
            # per simulate(): a prologue, then per step (per two steps with stages 3)
            # the step kernel (and, for a moving medium, the row shift and the next
            # step's pressure bounds)
            "gpu_launches": int(args.steps * (nt + 1 + 2 * _flow_due_steps(field, nt)
                                              if args.workload == "flow" else
                                              1 if args.workload == "nonlinear1d" else
                                              2 if st_used == 4 or resident_1d else
                                              (nt + spl - 1) // spl + 1))}
    if dword is not None:
        line["double_word"] = dword
    if (args.workload == "acoustic2d" and args.precision == "f64" and not args.no_studies
            and not args.time_steps and rank == 0):
        line["precision"] = _precision_legs()
        line["batched"] = _batched_legs()
    # DFMA per time step (the same count for one and for every step per launch)
    dfma = _traffic_from_profiles("%s_%s" % (args.workload, args.precision), "dfma_per_launch")
    if dfma and launch_ms and spl != 2:
        dfma *= spl
        # the FP64 pipe bounds the float64 step: its roofline beside the HBM one. Peak =
        # 2 DFMA per clock per SM (ncu's peak_sustained of the DFMA counter) x SMs x the
        # maximum SM clock
        sms = torch.cuda.get_device_properties(dev).multi_processor_count
        peak_g = 2.0 * sms * _max_sm_mhz() * 1e6 / 1e9
        got_g = dfma / (launch_ms * 1e-3) / 1e9
        line["fp64_pipe"] = {"dfma_per_launch": dfma, "achieved_gdfma_s": got_g,
                             "peak_gdfma_s": peak_g, "frac": got_g / peak_g,
                             "peak_kind": "2 per clock per SM x %d SMs x %.0f MHz"
                                          % (sms, _max_sm_mhz())}
    if args.time_steps:
        line["config"]["note"] = "time axis shortened for profiling; not a benchmark value"
    if ws == 1 and not args.no_cpu_baseline:
        procs = os.cpu_count() or 1
        steps = CPU_SAMPLE_STEPS[args.workload]
        vals, _ = cpu_sample(args.workload, steps, procs, repeats=1)
        one, _ = cpu_sample(args.workload, steps, 1, repeats=1)
        line["cpu_baseline"] = {"value": vals[0], "unit": "Gcell/s", "cores": procs,
                                "kind": "port",
                                "sample": "%d time steps of the full-size workload per process, "
                                          "%d processes (one replica each), numpy oracle"
                                          % (steps, procs),
                                # the oracle is single-threaded: the same sample in one process
                                "one_process": {"value": one[0], "unit": "Gcell/s", "cores": 1,
                                                "sample": "%d time steps of the full-size "
                                                          "workload in one process" % steps}}
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="acoustic2d")
    ap.add_argument("--precision", choices=["f64", "f32", "f32_t64", "dw"], default="f64")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end leg (profiling)")
    ap.add_argument("--no-studies", action="store_true",
                    help="default line: skip its precision and batched objects")
    ap.add_argument("--no-dw", action="store_true",
                    help="float64 lines: skip the double-word leg (the same workload in "
                         "precision='dw')")
    ap.add_argument("--tile", default="", help="tile shape XxY for lossless 2-D fields")
    ap.add_argument("--stages", type=int, default=0, choices=[0, 1, 2, 3, 4],
                    help="staging buffers per CTA (0: automatic)")
    ap.add_argument("--batch", type=int, default=0, help="instances of the batched workload")
    ap.add_argument("--autotune", action="store_true", help="autotune the batched tile shape")
    ap.add_argument("--study", default="",
                    choices=["", "precision", "axi", "thermal", "batched", "surrogate",
                             "surrogate-iter", "surrogate-precision", "coupling"],
                    help="print the precision study (float32 paths against float64) or the "
                         "learned-surrogate study instead")
    ap.add_argument("--surr-instances", type=int, default=625,
                    help="surrogate study: media simulated for the training set")
    ap.add_argument("--surr-snaps", type=int, default=33,
                    help="surrogate study: snapshots per medium (pairs = snaps - 1)")
    ap.add_argument("--surr-epochs", type=int, default=20)
    ap.add_argument("--surr-batch", type=int, default=32)
    ap.add_argument("--surr-eval", type=int, default=512, help="unseen media of the rollout")
    ap.add_argument("--surr-steps", type=int, default=4096, help="time steps of the rollout")
    ap.add_argument("--surr-save", default="", help="save the trained weights (.npz)")
    ap.add_argument("--surr-jump", type=int, default=64,
                    help="surrogate-precision study: time steps per jump")
    ap.add_argument("--surr-eval-media", type=int, default=64,
                    help="surrogate-precision study: unseen media evaluated")
    ap.add_argument("--surr-variants", default="bf16,fp32,fp32x2",
                    help="surrogate-precision study: bf16 (the kernels), fp32 (twin), "
                         "fp32x2 (twin, loss over two chained jumps)")
    ap.add_argument("--surr-load", default="", help="load trained weights instead of training")
    ap.add_argument("--time-steps", type=int, default=0,
                    help="override the workload's time steps per benchmark step (profiling)")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.study == "surrogate":
        return run_surrogate(args)
    if args.study == "surrogate-precision":
        return run_surrogate_precision(args)
    if args.study == "surrogate-iter":
        return run_surrogate_iter(args)
    if args.study == "coupling":
        return run_coupling_study(args)
    if args.study:
        return run_study(args)
    if args.workload == "batched":
        return run_batched(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
