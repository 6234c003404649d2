"""1-D fields in one launch against one launch per step (stages=1): a field of 256 to
8192 cells on a cluster of up to 16 CTAs (stag_1d_warp_kernel, or the shared-memory
window kernel stag_1d_cluster_kernel), a smaller one on one CTA
(stag_1d_resident_kernel). The per-cell arithmetic is the same, so every state value
and output must be identical bit for bit, for float64 (default and exact), float32,
double words and float32 with a float64 temperature, acoustic fields with and without
absorption and thermal fields, with every boundary and output mode of the random
scenarios, odd and even step counts, segmented calls, sizes up to the limit and one
cell past it (which steps one launch per step). The per-step path is pinned to the
reference by the other parity tests; the 1-D water workload is also held to its
reference fixture here."""
import numpy as np
import pytest

from oracle import scenarios as S
from helpers import build_field, field_results
from pyfds_gb300 import workloads

pytestmark = pytest.mark.gpu


def run(spec, stages, steps, chunks=None, **kw):
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


@pytest.mark.parametrize("kind,kw", [
    ("Acoustic1D", {}), ("Acoustic1D", {"exact": True}), ("Acoustic1D", {"precision": "f32"}),
    ("Acoustic1D", {"precision": "dw"}), ("Thermal1D", {}), ("Thermal1D", {"exact": True}),
    ("Thermal1D", {"precision": "f32"}), ("Thermal1D", {"precision": "f32_t64"}),
    ("Thermal1D", {"precision": "dw"})])
@pytest.mark.parametrize("nx,steps,mu", [(5, 13, True), (64, 30, False), (255, 40, True),
                                         (1000, 57, True), (3001, 24, True), (4096, 9, False),
                                         (8192, 35, True)])
def test_one_launch_equals_one_launch_per_step(gpu, kind, kw, nx, steps, mu):
    spec = S.random_scenario(61 + nx % 7, kind, nx, None, steps=steps, mu=mu)
    assert_same(run(spec, 0, steps, **kw), run(spec, 1, steps, **kw))


def test_segmented_calls_and_past_the_limit(gpu):
    spec = S.random_scenario(62, "Acoustic1D", 777, None, steps=20, mu=True)
    assert_same(run(spec, 0, 20, chunks=[7, 1, 12]), run(spec, 1, 20))
    # 8193 cells: more than a cluster's slots, stepped one launch per step
    spec = S.random_scenario(63, "Acoustic1D", 8193, None, steps=6, mu=False)
    assert_same(run(spec, 0, 6), run(spec, 1, 6))


def test_water_workload_vs_reference_in_one_launch(gpu):
    """The 1-D water workload (1000 cells, 2000 steps) in one launch, exact mode,
    against the unmodified reference's trajectory: bit for bit."""
    from golden_inputs import apply_inputs
    from test_gpu_parity import check_signals, check_state, golden
    from oracle import fds_oracle as O
    g = golden("acoustic1d_water.npz")
    spec = apply_inputs(workloads.acoustic1d_water(), g)
    f = build_field(spec, exact=True)
    f.simulate(spec["steps"])
    st, sig = field_results(f)
    check_signals(sig, g, "", ["pressure"], exact=True)
    check_state(st, g, "", O.components_of("Acoustic1D"), exact=True)


@pytest.mark.parametrize("kernel,ctas,block", [
    ("warp", "16", "1"), ("warp", "16", "3"), ("warp", "8", "9"), ("warp", "16", "0"),
    ("window", "16", "3"), ("window", "8", "40"), ("window", "16", "0")])
@pytest.mark.parametrize("kind,kw", [
    ("Acoustic1D", {}), ("Acoustic1D", {"exact": True}), ("Acoustic1D", {"precision": "dw"}),
    ("Acoustic1D", {"precision": "f32"}), ("Thermal1D", {}), ("Thermal1D", {"precision": "f32_t64"})])
@pytest.mark.parametrize("nx,steps,mu", [(300, 101, True), (1000, 140, True), (2049, 77, False)])
def test_cluster_exchange_blocks(gpu, monkeypatch, kernel, ctas, block, kind, kw, nx, steps,
                                 mu):
    """Fields on a cluster exchange their window edges once per block of K steps
    (FDS_CLUSTER_BLOCK_STEPS sets K, capped by the window; 0: the default), on warps
    with one cell per lane (stag_1d_warp_kernel, K up to 9) or on shared-memory windows
    (FDS_1D_KERNEL=window), on clusters of up to 16 or 8 CTAs (FDS_CLUSTER_CTAS), over
    calls of several blocks and a last partial one, with absorption (the flux reads
    both neighbours' old fluxes) and without; every value as one launch per step."""
    monkeypatch.setenv("FDS_1D_KERNEL", kernel)
    monkeypatch.setenv("FDS_CLUSTER_CTAS", ctas)
    monkeypatch.setenv("FDS_CLUSTER_BLOCK_STEPS", block)
    spec = S.random_scenario(64 + nx % 5, kind, nx, None, steps=steps, mu=mu)
    assert_same(run(spec, 0, steps, **kw), run(spec, 1, steps, **kw))
