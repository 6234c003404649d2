"""Every step of a call in one persistent launch (stages=4, the wavefront kernel)
against one launch per step (stages=1) with the same tile: each tile runs the same
compute_tile arithmetic, so every state value and output must be identical bit for
bit, for float64, float32 and double words, acoustic and thermal fields, odd and
even step counts, grids whose rows the TMA path cannot stage (which fall back to one
launch per step), segmented calls and the full 2048^2 workload. The one-step kernel
is pinned to the reference by the other parity tests; the full-size wavefront run is
also held to the reference fixture of the 2048^2 workload."""
import numpy as np
import pytest

from oracle import scenarios as S
from helpers import build_field, field_results
from pyfds_gb300 import workloads

pytestmark = pytest.mark.gpu


def run(spec, precision, stages, steps, chunks=None, tile=None):
    kw = {"precision": precision}
    if tile is not None:
        kw["tile"] = tile
    f = build_field(spec, **kw)
    f.stages = stages
    for n in (chunks or [steps]):
        f.simulate(n)
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
@pytest.mark.parametrize("nx,ny,steps", [(204, 77, 15), (256, 96, 24), (64, 48, 7),
                                         (200, 3, 5), (97, 41, 9)])
def test_wavefront_equals_one_launch_per_step(gpu, precision, kind, nx, ny, steps):
    spec = S.random_scenario(41, kind, nx, ny, steps=steps, mu=False)
    assert_same(run(spec, precision, 4, steps), run(spec, precision, 1, steps))


@pytest.mark.parametrize("precision", ["f64", "dw"])
def test_wavefront_segmented_calls(gpu, precision):
    """Three calls of 5, 1 and 12 steps (outputs appended, the first step's bounds
    from the prologue of each call) equal one call of 18 steps per launch."""
    spec = S.random_scenario(43, "Acoustic2D", 256, 80, steps=18, mu=False)
    assert_same(run(spec, precision, 4, 18, chunks=[5, 1, 12]), run(spec, precision, 1, 18))


def test_wavefront_tile_menu_shape(gpu):
    """A tile of the menu without a wavefront instantiation runs one launch per step."""
    spec = S.random_scenario(44, "Acoustic2D", 256, 64, steps=6, mu=False)
    assert_same(run(spec, "f64", 4, 6, tile=(32, 32)), run(spec, "f64", 1, 6, tile=(32, 32)))


def test_wavefront_full_size_float64(gpu):
    """The 2048^2 water/steel field for 200 steps: every one of the 4096 tiles per
    step waits on its neighbouring rows through the queue; same bits as one launch
    per step."""
    spec = workloads.acoustic2d_steel_block(nt=200)
    assert_same(run(spec, "f64", 4, 200), run(spec, "f64", 1, 200))


def test_wavefront_full_run_vs_reference(gpu):
    """The full 2048^2 workload (4000 steps, 64 outputs) through the wavefront kernel
    against the unmodified reference's outputs: the 1e-12 bar of the float64 path."""
    from golden_inputs import apply_inputs
    from test_gpu_parity import TOL, check_signals, check_state, golden
    from oracle import fds_oracle as O
    g = golden("acoustic2d_steel_2048.npz")
    spec = apply_inputs(workloads.acoustic2d_steel_block(), g)
    f = build_field(spec)
    f.stages = 4
    f.simulate(spec["steps"])
    st, sig = field_results(f)
    assert check_signals(sig, g, "", ["pressure"], exact=False) <= TOL
    check_state(st, g, "", O.components_of("Acoustic2D"), exact=False, tol=1e-11)
