"""Two steps per tile (stages=3, the temporally blocked kernel) against the one-step
kernel with the same tile: the same arithmetic per cell in the same order, so every
state value and output must be identical bit for bit, for float64, float32 and
double words, acoustic and thermal, odd and even step counts (an odd call ends
with a one-step launch of the two-step kernel), TMA and cp.async staging. The
one-step kernel is pinned to the reference by the other parity tests."""
import numpy as np
import pytest

from oracle import scenarios as S
from helpers import build_field, field_results
from pyfds_gb300 import workloads

pytestmark = pytest.mark.gpu

TB2_TILES = [(64, 16), (64, 12), (64, 8), (32, 32)]


def run(spec, precision, tile, stages, steps):
    f = build_field(spec, precision=precision, tile=tile)
    f.stages = stages
    f.simulate(steps)
    return field_results(f)


def assert_same(a, b):
    sa, ga = a
    sb, gb = b
    for c in sa:
        assert np.array_equal(sa[c], sb[c]), c
        for x, y in zip(ga[c], gb[c]):
            assert np.array_equal(x, y), c


@pytest.mark.parametrize("precision", ["f64", "f32", "dw"])
@pytest.mark.parametrize("kind", ["Acoustic2D", "Thermal2D", "Acoustic3DAxi"])
@pytest.mark.parametrize("tile", TB2_TILES)
@pytest.mark.parametrize("nx,ny,steps", [(203, 77, 15), (204, 77, 16), (37, 19, 7), (5, 40, 6)])
def test_two_step_equals_one_step(gpu, precision, kind, tile, nx, ny, steps):
    spec = S.random_scenario(31, kind, nx, ny, steps=steps, mu=False)
    assert_same(run(spec, precision, tile, 3, steps), run(spec, precision, tile, 1, steps))


def test_two_step_full_size_double_words(gpu):
    """The 2048^2 water/steel field (L2 prefetch active), 40 steps, double words."""
    spec = workloads.acoustic2d_steel_block(nt=40)
    assert_same(run(spec, "dw", (64, 12), 3, 40), run(spec, "dw", (64, 12), 1, 40))


@pytest.mark.parametrize("precision,size", [("dw", 2048), ("f32", 2048), ("dw", 300)])
def test_two_step_is_deterministic(gpu, precision, size):
    """The same two-step run twice gives the same bits (no dependence on what the
    shared memory held before, no race between the two steps of a tile)."""
    spec = workloads.acoustic2d_steel_block(n=size, nt=60, n_probes=16)
    tile = (64, 12) if precision == "dw" else (64, 16)
    a = run(spec, precision, tile, 3, 60)
    b = run(spec, precision, tile, 3, 60)
    assert_same(a, b)
    for sig in a[1].values():
        for s in sig:
            assert np.all(np.isfinite(s))


def test_two_step_segmented_calls(gpu):
    """simulate(5) + simulate(6) with two steps per tile == simulate(11) one step per
    tile (host edits between calls are picked up)."""
    spec = S.random_scenario(33, "Acoustic2D", 130, 70, steps=11, mu=False)
    a = build_field(spec, precision="f64", tile=(64, 16))
    a.stages = 3
    a.simulate(5)
    a.simulate(6)
    b = build_field(spec, precision="f64", tile=(64, 16))
    b.stages = 1
    b.simulate(11)
    assert_same(field_results(a), field_results(b))


def test_two_step_rejects_what_it_does_not_cover(gpu):
    """Exact mode has no two-step kernel: the call fails loudly (no silent switch)."""
    from pyfds_gb300 import _capi
    spec = S.random_scenario(34, "Acoustic2D", 70, 30, steps=4, mu=False)
    f = build_field(spec, tile=(64, 16), exact=True)
    f.stages = 3
    with pytest.raises(_capi.FdsError):
        f.simulate(4)


@pytest.mark.parametrize("precision", ["f64", "f32", "dw"])
@pytest.mark.parametrize("kind", ["Acoustic2D", "Thermal2D"])
def test_batched_two_step_equals_single_one_step(gpu, precision, kind):
    """Six fields of uneven size batched with two steps per tile (odd step count):
    each equals its single-field one-step run bit for bit."""
    from pyfds_gb300.batch import simulate_batch
    sizes = [(204, 77), (203, 64), (64, 256), (37, 19), (130, 130), (256, 32)]
    specs = [S.random_scenario(90 + k, kind, nx, ny, steps=13, mu=False)
             for k, (nx, ny) in enumerate(sizes)]
    batch = [build_field(s, precision=precision) for s in specs]
    simulate_batch(batch, 13, tile=(64, 16), stages=3)
    for s, fb in zip(specs, batch):
        assert_same(field_results(fb), run(s, precision, (64, 16), 1, 13))


def test_batched_two_step_graph_replay(gpu):
    """A captured two-step batch (8 steps = 4 launches) replays to the state of the
    same launches issued directly."""
    import torch
    from pyfds_gb300.batch import BatchRunner
    specs = [S.random_scenario(95 + k, "Acoustic2D", 96, 40 + 8 * k, steps=8, mu=False)
             for k in range(3)]
    a = [build_field(s, precision="f32") for s in specs]
    b = [build_field(s, precision="f32") for s in specs]
    ra = BatchRunner(a, 8, tile=(64, 16), stages=3)
    assert ra.steps_per_launch() == 2
    ra.capture()
    ra.replay()
    rb = BatchRunner(b, 8, tile=(64, 16), stages=3)
    rb.launch()
    rb.launch()
    torch.cuda.synchronize()
    for fa, fb in zip(a, b):
        for name in fa._stag_components:
            assert torch.equal(fa._engine().buffers[name][0], fb._engine().buffers[name][0]), name
    # any step count of two or more captures: 6 steps run as 2 + 2 + 1 + 1
    r6 = BatchRunner(b, 6, tile=(64, 16), stages=3)
    assert r6.launches() == 4
    with pytest.raises(ValueError):
        BatchRunner(b, 1, tile=(64, 16), stages=3).capture()  # one launch
