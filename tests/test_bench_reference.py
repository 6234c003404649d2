"""The reference arm of bench.py (`--impl reference`: the CPU implementation of the
stepping timed on the host cores): under torchrun only rank 0 measures and prints;
its one JSON line carries the bench contract's keys. The CPU sample is replaced by
a stub here, so no oracle work runs."""
import argparse
import json
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import bench  # noqa: E402


def _args(workload="acoustic2d", steps=3, warmup=1):
    return argparse.Namespace(workload=workload, steps=steps, warmup=warmup)


def test_other_ranks_exit_without_work(monkeypatch, capsys):
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("LOCAL_RANK", "1")
    called = []
    monkeypatch.setattr(bench, "cpu_sample", lambda *a, **k: called.append(a))
    assert bench.run_reference(_args()) == 0
    assert called == [] and capsys.readouterr().out == ""


def test_rank0_line(monkeypatch, capsys):
    monkeypatch.setenv("WORLD_SIZE", "1")
    monkeypatch.setenv("RANK", "0")
    seen = {}

    def fake(wname, steps, procs, repeats=1, warmup=0):
        seen.update(wname=wname, steps=steps, procs=procs, repeats=repeats, warmup=warmup)
        return [1.0, 3.0, 2.0], 4096

    monkeypatch.setattr(bench, "cpu_sample", fake)
    assert bench.run_reference(_args(steps=3, warmup=1)) == 0
    lines = [l for l in capsys.readouterr().out.splitlines() if l.strip()]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert seen == {"wname": "acoustic2d", "steps": bench.CPU_SAMPLE_STEPS["acoustic2d"],
                    "procs": os.cpu_count() or 1, "repeats": 3, "warmup": 1}
    assert d["impl"] == "reference"
    assert d["metric"] == "Gcell-updates/s" and d["unit"] == "Gcell/s"
    assert d["value"] == 2.0 and d["higher_is_better"] is True
    assert d["steps"] == 3 and d["warmup"] == 1 and d["n_gpus"] == 1
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["kind"] in ("port", "reference")
    assert cb["cores"] == (os.cpu_count() or 1) and cb["sample"]
    assert d["e2e"] == {"value": 2.0, "unit": "Gcell/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}
    # the GPU arm's config names the workload the same way
    assert d["config"]["workload"] == bench._workload_label("acoustic2d") == \
        "acoustic2d: acoustic2d_steel_block"
    assert d["config"]["precision"] == "f64"


def test_every_workload_has_a_cpu_sample():
    assert set(bench.CPU_SAMPLE_STEPS) >= set(bench.WORKLOADS) | {"batched"}


def test_batched_label_follows_the_builder_defaults():
    from pyfds_gb300 import workloads
    specs = workloads.layered_media_batch(count=3, nt=5)
    assert len(specs) == 3
    assert bench._workload_label("batched") == bench._workload_label("batched", 256, 2000)
    assert "3 layered-media" in bench._workload_label("batched", 3, 5)
