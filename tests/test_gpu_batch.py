"""Batched stepping (one launch per step for many fields) against the single-field
path and the oracle, CUDA-graph replay, the persistent two-stage variant and the
autotuner."""
import numpy as np
import pytest

from oracle import fds_oracle as O
from oracle import scenarios as S
from helpers import build_field, field_results, max_rel_l2_signals, rel_l2
from pyfds_gb300 import workloads

pytestmark = pytest.mark.gpu

TOL = 1e-12


def specs(kind="Acoustic2D", seed=0):
    sizes = [(204, 77), (203, 64), (64, 256), (37, 19), (130, 130), (256, 32)]
    return [S.random_scenario(seed + k, kind, nx, ny, steps=14, mu=False)
            for k, (nx, ny) in enumerate(sizes)]


@pytest.mark.parametrize("kind", ["Acoustic2D", "Thermal2D", "Acoustic3DAxi"])
@pytest.mark.parametrize("stages", [1, 2])
def test_batch_matches_single_and_oracle(gpu, kind, stages):
    from pyfds_gb300.batch import simulate_batch
    sp = specs(kind, seed=40)
    batch = [build_field(s, tile=(64, 16)) for s in sp]
    simulate_batch(batch, 14, stages=stages)
    for s, fb in zip(sp, batch):
        single = build_field(s, tile=(64, 16))
        single.stages = 1
        single.simulate(14)
        a_st, a_sg = field_results(fb)
        b_st, b_sg = field_results(single)
        for c in a_st:
            assert np.array_equal(a_st[c], b_st[c]), c
            for x, y in zip(a_sg[c], b_sg[c]):
                assert np.array_equal(x, y)
        st_o, sg_o = O.simulate(s, 14)
        assert max_rel_l2_signals(a_sg, sg_o) <= TOL
        for c in st_o:
            assert rel_l2(a_st[c], st_o[c]) <= TOL, c
        assert fb.step == 14


def test_batch_float32_error(gpu):
    from pyfds_gb300.batch import simulate_batch
    sp = specs(seed=60)
    batch = [build_field(s, precision="f32") for s in sp]
    simulate_batch(batch, 14)
    for s, f in zip(sp, batch):
        st_o, sg_o = O.simulate(s, 14)
        st, sg = field_results(f)
        assert max_rel_l2_signals(sg, sg_o) <= 1e-4


def test_batch_graph_replay(gpu):
    import torch
    from pyfds_gb300.batch import BatchRunner, simulate_batch
    sp = specs(seed=80)
    ref = [build_field(s) for s in sp]
    simulate_batch(ref, 14)
    fields = [build_field(s) for s in sp]
    r = BatchRunner(fields, 14)
    init = [{n: b[0].clone() for n, b in f._engine().buffers.items()} for f in fields]
    r.capture()  # runs once (warm-up) and captures
    for _ in range(2):  # every replay restarts from the captured initial state
        for f, snap in zip(fields, init):
            for n, t in snap.items():
                f._engine().buffers[n][0].copy_(t)
        r.replay()
    torch.cuda.synchronize()
    r.finish()
    for fr, fg in zip(ref, fields):
        a, _ = field_results(fr)
        b, _ = field_results(fg)
        for c in a:
            assert np.array_equal(a[c], b[c]), c


def test_autotune_restores_state(gpu, tmp_path, monkeypatch):
    from pyfds_gb300.autotune import autotune_batch
    from pyfds_gb300.batch import simulate_batch
    monkeypatch.setenv("PYFDS_GB300_AUTOTUNE", str(tmp_path / "tune.json"))
    sp = specs(seed=90)
    fields = [build_field(s) for s in sp]
    tile, stages = autotune_batch(fields, steps=4)
    assert (tmp_path / "tune.json").exists()
    simulate_batch(fields, 14)
    for s, f in zip(sp, fields):
        st_o, sg_o = O.simulate(s, 14)
        st, sg = field_results(f)
        assert max_rel_l2_signals(sg, sg_o) <= TOL


def test_layered_batch_workload_runs(gpu):
    from pyfds_gb300.batch import simulate_batch
    sp = workloads.layered_media_batch(count=8, nt=40, n_max=300)
    fields = [workloads.build_field(s) for s in sp]
    simulate_batch(fields, 40)
    for s, f in zip(sp[:3], fields[:3]):
        st_o, sg_o = O.simulate(s, 40)
        st, sg = field_results(f)
        assert max_rel_l2_signals(sg, sg_o) <= TOL
