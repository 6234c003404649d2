"""GPU parity of the fused time step against the reference.

Bar (float64 drop-in): every recorded output, and the final state, within a
relative L2 error of 1e-12 of the reference (TOL below); with ``exact=True`` the
GPU reproduces the reference bit for bit (np.array_equal). Fixtures come from the
unmodified reference (tests/golden/make_golden.py); sizes the reference cannot
finish here are checked against the oracle or through size-independent
properties.
"""
import json
import os

import numpy as np
import pytest

from oracle import fds_oracle as O
from oracle import scenarios as S
from golden_inputs import apply_inputs
from helpers import build_field, field_results, max_rel_l2_signals, rel_l2
from pyfds_gb300 import workloads

pytestmark = pytest.mark.gpu

TOL = 1e-12  # relative L2 per recorded output, float64
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def golden(name):
    path = os.path.join(GOLDEN, name)
    if not os.path.exists(path):
        pytest.skip("fixture %s not generated" % name)
    return np.load(path)


def check_state(st, g, prefix, comps, exact, tol=TOL):
    for c in comps:
        key = prefix + c + "/state"
        if key in g.files:
            if exact:
                assert np.array_equal(st[c], g[key]), c
            else:
                assert rel_l2(st[c], g[key]) <= tol, (c, rel_l2(st[c], g[key]))
        else:
            # only the norm and sum were stored; reductions are summed in a
            # platform-dependent order, so even exact mode compares them to ~ulps
            nrm = g[prefix + c + "/state_norm"]
            got = np.array([np.linalg.norm(st[c]), np.sum(st[c])])
            assert abs(got[0] - nrm[0]) <= max(tol, 1e-14) * max(abs(nrm[0]), 1e-300), c


def check_signals(sig, g, prefix, comps, exact, tol=TOL):
    worst = 0.0
    for c in comps:
        for j, s in enumerate(sig[c]):
            ref = g[prefix + c + "/sig%d" % j]
            assert s.shape == ref.shape, (c, j, s.shape, ref.shape)
            if exact:
                assert np.array_equal(s, ref), (c, j, np.max(np.abs(s - ref)))
            for k in range(ref.shape[0]):
                e = rel_l2(s[k], ref[k])
                worst = max(worst, e)
                assert e <= tol, (c, j, k, e)
    return worst


@pytest.mark.parametrize("exact", [True, False])
def test_random_scenarios_vs_reference(gpu, exact):
    g = golden("random_scenarios.npz")
    cases = json.loads(str(g["cases"]))
    for case in cases:
        spec = S.random_scenario(case["seed"], case["kind"], case["nx"], case["ny"],
                                 steps=case["steps"], mu=case["mu"])
        prefix = "s%d/" % case["seed"]
        apply_inputs(spec, g, prefix)
        f = build_field(spec, exact=exact)
        f.simulate(spec["steps"])
        st, sig = field_results(f)
        comps = O.components_of(case["kind"])
        check_state(st, g, prefix, comps, exact)
        check_signals(sig, g, prefix, comps, exact)


@pytest.mark.parametrize("exact", [True, False])
def test_acoustic1d_water_vs_reference(gpu, exact):
    g = golden("acoustic1d_water.npz")
    spec = apply_inputs(workloads.acoustic1d_water(), g)
    f = build_field(spec, exact=exact)
    f.simulate()
    assert f.step == 2000
    st, sig = field_results(f)
    check_state(st, g, "", ["pressure", "velocity"], exact)
    check_signals(sig, g, "", ["pressure"], exact)


@pytest.mark.parametrize("exact", [True, False])
def test_axi_small_vs_reference(gpu, exact):
    g = golden("axi_disc_256x1024.npz")
    spec = apply_inputs(workloads.axi_disc_source(256, 1024, 500, disc=50, probe_every=32), g)
    f = build_field(spec, exact=exact)
    f.simulate(spec["steps"])
    st, sig = field_results(f)
    check_signals(sig, g, "", ["pressure"], exact)
    check_state(st, g, "", O.components_of("Acoustic3DAxi"), exact)


@pytest.mark.parametrize("exact", [True, False])
def test_thermal2d_small_vs_reference(gpu, exact):
    g = golden("thermal2d_512.npz")
    spec = apply_inputs(workloads.thermal2d_two_materials(512, 500, 64), g)
    f = build_field(spec, exact=exact)
    f.simulate(spec["steps"])
    st, sig = field_results(f)
    check_signals(sig, g, "", ["temperature"], exact)
    check_state(st, g, "", ["temperature"], exact)


def test_acoustic2d_steel_2048_full_vs_reference(gpu):
    """The 2048^2 water/steel workload, all 4000 steps, 64 outputs."""
    g = golden("acoustic2d_steel_2048.npz")
    spec = apply_inputs(workloads.acoustic2d_steel_block(), g)
    f = build_field(spec)
    f.simulate(spec["steps"])
    st, sig = field_results(f)
    worst = check_signals(sig, g, "", ["pressure"], exact=False)
    assert worst <= TOL
    check_state(st, g, "", O.components_of("Acoustic2D"), exact=False, tol=1e-11)


@pytest.mark.parametrize("name,builder,comps", [
    ("axi_disc_full_prefix.npz", workloads.axi_disc_source, ["pressure"]),
    ("thermal2d_4096_prefix.npz", workloads.thermal2d_two_materials, ["temperature"]),
])
def test_full_size_prefix_vs_reference(gpu, name, builder, comps):
    g = golden(name)
    spec = apply_inputs(builder(), g)
    f = build_field(spec)
    f.simulate(100)
    st, sig = field_results(f)
    check_signals(sig, g, "", comps, exact=False)


@pytest.mark.parametrize("name,builder,comps,stages", [
    ("axi_disc_full_1000.npz", workloads.axi_disc_source, ["pressure"], 0),
    ("axi_disc_full_1000.npz", workloads.axi_disc_source, ["pressure"], 1),
    ("thermal2d_4096_1000.npz", workloads.thermal2d_two_materials, ["temperature"], 0),
])
def test_full_size_1000_steps_vs_reference(gpu, name, builder, comps, stages):
    """The full-size axisymmetric (1024 x 4096, 64 outputs) and thermal (4096^2, 64
    outputs) workloads for their first 1000 steps against the unmodified reference
    (pyfds/acoustics.py:205-225, pyfds/thermal.py:92-107), every output at the 1e-12
    bar: the automatic path (the wavefront run for the axisymmetric field) and one
    launch per step."""
    g = golden(name)
    spec = apply_inputs(builder(), g)
    f = build_field(spec)
    f.stages = stages
    f.simulate(1000)
    st, sig = field_results(f)
    assert check_signals(sig, g, "", comps, exact=False) <= TOL


def test_sim_step_loop_equals_simulate(gpu):
    spec = S.random_scenario(7, "Acoustic2D", 70, 40, steps=12)
    a = build_field(spec)
    a.simulate(12)
    b = build_field(spec)
    for _ in range(12):
        b.sim_step()
        b.step += 1
    sa, ga = field_results(a)
    sb, gb = field_results(b)
    for c in sa:
        assert np.array_equal(sa[c], sb[c])
        for x, y in zip(ga[c], gb[c]):
            assert np.array_equal(x, y)


def test_segmented_simulate_and_host_edits(gpu):
    """simulate(5); edit values on the host; simulate(7) == the oracle doing the same."""
    spec = S.random_scenario(8, "Thermal2D", 67, 35, steps=12)
    f = build_field(spec, exact=True)
    f.simulate(5)
    t = f.temperature.values
    t[100:110] += 3.0  # in-place edit of the returned array
    f.heat_flux_x.values = np.zeros(f.num_points)  # overwritten by the next step anyway
    f.simulate(7)
    st_g, sig_g = field_results(f)

    ops_state, sig1 = O.simulate(spec, 5)
    ops_state["temperature"][100:110] += 3.0
    st_o, sig2 = O.simulate(spec, 7, state=ops_state, step0=5)
    assert np.array_equal(st_g["temperature"], st_o["temperature"])
    for c in sig_g:
        for k, s in enumerate(sig_g[c]):
            assert np.array_equal(s, np.concatenate([sig1[c][k], sig2[c][k]], axis=1))


def test_reset_keeps_outputs(gpu):
    spec = workloads.acoustic1d_water(nt=300)
    f = build_field(spec)
    f.simulate(100)
    first = np.array(f.pressure.outputs[0].signals[0])
    f.reset()
    assert f.step == 0 and not np.any(f.pressure.values)
    f.simulate(100)
    sig = np.array(f.pressure.outputs[0].signals[0])
    assert sig.shape == (200,)
    assert np.array_equal(sig[:100], first) and np.array_equal(sig[100:], first)


def test_short_signal_raises_before_launch(gpu):
    spec = workloads.acoustic1d_water(nt=50)
    f = build_field(spec)
    f.simulate(20)
    before = f.pressure.values.copy()
    with pytest.raises(IndexError):
        f.simulate(40)  # the source signal has 50 samples, steps 20..59 are needed
    assert f.step == 20
    assert np.array_equal(f.pressure.values, before)


def test_overridden_sim_step_is_called_per_step(gpu):
    calls = []

    class Probe(type(build_field(workloads.acoustic1d_water(nt=10)))):
        def sim_step(self):
            calls.append(self.step)
            super().sim_step()

    spec = workloads.acoustic1d_water(nt=10)
    f = build_field(spec)
    f.__class__ = Probe
    f.simulate(10)
    assert calls == list(range(10))
    ref = build_field(spec)
    ref.simulate(10)
    assert np.array_equal(f.pressure.values, ref.pressure.values)


@pytest.mark.parametrize("precision,tol", [("f32", 2e-3)])
def test_float32_acoustic_error_vs_float64(gpu, precision, tol):
    g = golden("acoustic1d_water.npz")
    spec = apply_inputs(workloads.acoustic1d_water(), g)
    f = build_field(spec, precision=precision)
    f.simulate()
    e = rel_l2(f.pressure.outputs[0].signals[0], g["pressure/sig0"][0])
    assert e <= tol, e


@pytest.mark.parametrize("precision,tol", [("f32_t64", 1e-4), ("f32", 1e-3)])
def test_thermal_reduced_precision_error(gpu, precision, tol):
    """Float32 thermal paths against the reference: relative L2 of the temperature
    rise above 293.15 K per output (outputs the heat has reached)."""
    g = golden("thermal2d_512.npz")
    spec = apply_inputs(workloads.thermal2d_two_materials(512, 500, 64), g)
    f = build_field(spec, precision=precision)
    f.simulate(spec["steps"])
    sig = np.array(f.temperature.outputs[0].signals) - 293.15
    ref = g["temperature/sig0"] - 293.15
    scale = np.linalg.norm(ref, axis=1).max()
    worst = 0.0
    for a, b in zip(sig, ref):
        nb = np.linalg.norm(b)
        if nb > 1e-6 * scale:
            worst = max(worst, np.linalg.norm(a - b) / nb)
    assert worst <= tol, worst


MENU = [((64, 16), 1), ((32, 32), 1), ((128, 8), 1), ((64, 32), 1), ((128, 16), 1),
        ((64, 12), 1), ((64, 8), 1),
        ((64, 16), 2), ((32, 32), 2), ((128, 8), 2), ((64, 32), 2), ((128, 16), 2),
        ((64, 12), 2), ((64, 8), 2),
        ((62, 16), 1), ((62, 8), 1), ((62, 32), 1), ((30, 16), 1), ((30, 32), 1)]


@pytest.mark.parametrize("nx", [203, 204])  # 204: rows are 16-byte multiples -> TMA staging
@pytest.mark.parametrize("tile,stages", MENU)
@pytest.mark.parametrize("kind", ["Acoustic2D", "Thermal2D"])
@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_tile_menu_parity(gpu, tile, kind, stages, precision, nx):
    """Every tile shape of the autotuner's menu against the oracle (grids that are not
    multiples of the tile, so partial tiles and row-end wraps cross tile seams)."""
    from pyfds_gb300 import _capi
    assert tile in _capi.tile_menu()
    spec = S.random_scenario(21, kind, nx, 77, steps=15, mu=False)
    st_o, sg_o = O.simulate(spec, spec["steps"])
    from pyfds_gb300 import _capi as capi
    f = build_field(spec, tile=tile, precision=precision)
    f.stages = stages
    try:
        f.simulate(spec["steps"])
    except capi.FdsError as e:
        if e.code == capi.FDS_E_SIZE:
            pytest.skip("does not fit in shared memory: %s" % e)
        raise
    st, sig = field_results(f)
    tol = TOL if precision == "f64" else 1e-5
    assert max_rel_l2_signals(sig, sg_o) <= tol
    for c in st_o:
        assert rel_l2(st[c], st_o[c]) <= tol, c


def _flow_cases():
    g = golden("acoustic_flow.npz")
    return json.loads(str(g["cases"])), g


@pytest.mark.parametrize("exact", [True, False])
def test_acoustic_flow_vs_reference(gpu, exact):
    """AcousticFlow2D: moving-medium row shifts between steps, on the device."""
    import warnings
    cases, g = _flow_cases()
    for case in cases:
        with warnings.catch_warnings():
            warnings.simplefilter("ignore")
            spec = S.flow_scenario(case["seed"], case["nx"], case["ny"], steps=case["steps"],
                                   flow=case["flow"], mu=case["mu"])
            prefix = "f%d/" % case["seed"]
            apply_inputs(spec, g, prefix)
            f = build_field(spec, exact=exact)
        f.simulate(spec["steps"])
        st, sig = field_results(f)
        comps = O.components_of("AcousticFlow2D")
        check_state(st, g, prefix, comps, exact)
        check_signals(sig, g, prefix, comps, exact)


def test_acoustic_flow_sim_step_and_apply_flow(gpu):
    """sim_step loop == simulate; apply_flow alone == the oracle's shift."""
    import warnings
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        spec = S.flow_scenario(41, 130, 20, steps=10, flow="rows")
        a = build_field(spec)
        b = build_field(spec)
    a.simulate(10)
    for _ in range(10):
        b.sim_step()
        b.step += 1
    sa, ga = field_results(a)
    sb, gb = field_results(b)
    for c in sa:
        assert np.array_equal(sa[c], sb[c])
        for x, y in zip(ga[c], gb[c]):
            assert np.array_equal(x, y)
    # the shift alone, at a step where some rows are due
    st = {c: np.array(getattr(a, c).values) for c in O.components_of("AcousticFlow2D")}
    a.step = 12
    a.apply_flow()
    O.apply_flow(st, O.flow_periods(spec), 12, spec["nx"])
    for c in st:
        assert np.array_equal(np.array(getattr(a, c).values), st[c]), c


def test_acoustic_flow_large_grid_vs_oracle(gpu):
    """A 1000 x 300 flow field (rows of several shift chunks): the state against the
    oracle bit for bit (the probe signals of flow fields are compared with the
    reference's in test_acoustic_flow_vs_reference)."""
    import warnings
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        spec = S.flow_scenario(43, 1000, 300, steps=8, flow="rows", mu=False)
        f = build_field(spec, exact=True)
    f.simulate(8)
    st, _ = field_results(f)
    ref_st, _ = O.simulate(spec, 8)
    for c in st:
        assert np.array_equal(st[c], ref_st[c]), c


@pytest.mark.parametrize("exact", [True, False])
def test_nonlinear_1d_vs_reference(gpu, exact):
    """IdealGas1D / Acoustic2ndOrder1D in one launch per simulate() call. Exact mode
    is bit-identical except where the ideal-gas state equation calls pow (device and
    host libm may differ in the last bit): there the 1e-12 bar applies."""
    g = golden("nonlinear_1d.npz")
    for case in json.loads(str(g["cases"])):
        spec = S.nonlinear_scenario(case["seed"], case["kind"], case["nx"], steps=case["steps"],
                                    convective=case["convective"], nl_state=case["nl_state"],
                                    mu=case["mu"])
        prefix = "n%d/" % case["seed"]
        apply_inputs(spec, g, prefix)
        f = build_field(spec, exact=exact)
        f.simulate(spec["steps"])
        assert f.step == spec["steps"]
        st, sig = field_results(f)
        comps = O.components_of(case["kind"])
        bitwise = exact and not (case["kind"] == "IdealGas1D" and case["nl_state"])
        check_state(st, g, prefix, comps, bitwise)
        check_signals(sig, g, prefix, comps, bitwise)


def test_nonlinear_1d_additive_velocity_bound_at_tile_seams(gpu):
    """Additive velocity sources on cells where 64-cell tiles meet: the tile left of a
    seam also holds the cell (as its halo), and each source must still be added once
    per step (bit for bit the oracle in exact mode)."""
    spec = S.nonlinear_scenario(5, "Acoustic2ndOrder1D", 300, steps=40)
    t = np.arange(spec["nt"]) * spec["dt"]
    spec["bounds"]["velocity"].append({"indices": [64, 128, 129],
                                       "value": 1e-9 * np.sin(2e5 * t), "additive": True})
    st_o, sg_o = O.simulate(spec, spec["steps"])
    f = build_field(spec, exact=True)
    f.simulate(spec["steps"])
    st, sig = field_results(f)
    for c in st_o:
        assert np.array_equal(st[c], st_o[c]), c
        for x, y in zip(sig[c], sg_o[c]):
            assert np.array_equal(x, y), c


def test_nonlinear_1d_sim_step_loop_equals_simulate(gpu):
    spec = S.nonlinear_scenario(77, "Acoustic2ndOrder1D", 300, steps=25)
    a = build_field(spec)
    a.simulate(25)
    b = build_field(spec)
    for _ in range(25):
        b.sim_step()
        b.step += 1
    sa, ga = field_results(a)
    sb, gb = field_results(b)
    for c in sa:
        assert np.array_equal(sa[c], sb[c])
        for x, y in zip(ga[c], gb[c]):
            assert np.array_equal(x, y)


@pytest.mark.parametrize("exact", [True, False])
def test_coupled_fields_vs_reference(gpu, exact):
    """ThermoAcoustic1D and SynchronizedFields: every field steps on the GPU, the
    interactions run on the host copies. Exact mode is bit-identical except where a
    transfer function calls np.exp on the host (its last bit may differ between the
    machine that made the fixture and this one): there the 1e-12 bar applies."""
    import pyfds_gb300
    from coupled_helpers import compare, coupled_spec, kind_of
    from oracle import scenarios as S2
    g = golden("coupling.npz")
    for case in json.loads(str(g["cases"])):
        spec, prefix = coupled_spec(case, g)
        obj = S2.build_coupled(pyfds_gb300, spec, build_field, exact=exact)
        obj.simulate(spec["steps"])
        bitwise = exact and case["variant"] != "sync_exp"

        def check(a, b, where):
            if bitwise:
                assert np.array_equal(a, b), (case, where, np.max(np.abs(a - b)))
            else:
                assert rel_l2(a, b) <= TOL, (case, where, rel_l2(a, b))
        compare(S2.coupled_results(obj, kind_of), g, prefix, check)


@pytest.mark.parametrize("variant,nx,block", [("thermoacoustic", 45, "0"),
                                              ("thermoacoustic3", 45, "0"),
                                              ("thermoacoustic", 1000, "1"),
                                              ("thermoacoustic3", 1000, "3"),
                                              ("thermoacoustic3", 777, "8"),
                                              ("thermoacoustic3", 2100, "0")])
def test_thermoacoustic_native_equals_step_by_step(gpu, variant, nx, block, monkeypatch):
    """ThermoAcoustic1D's one-call stepping (fds_thermoacoustic_run) against the
    reference's loop (fields stepped one by one, coupling applied on the host), both
    exact; simulate is split into two chunks so that an accumulated transfer crosses
    a call boundary. One-call stepping runs every step of a call in one launch on the
    warps of a cluster, exchanging window edges every K steps (FDS_CLUSTER_BLOCK_STEPS;
    0: the default): the 45-cell cases on 3 CTAs of one warp, the 777- and 1000-cell
    cases on 8 warps per CTA; 2100 cells exceed a cluster's warps and step with one
    launch per field and step plus a loss kernel."""
    import pyfds_gb300
    from coupled_helpers import kind_of
    from oracle import scenarios as S2
    monkeypatch.setenv("FDS_CLUSTER_BLOCK_STEPS", block)
    spec = S2.coupled_scenario(77, variant, nx=nx, steps=27)
    a = S2.build_coupled(pyfds_gb300, spec, build_field, exact=True)
    assert a._native_path()
    a.simulate(7)
    a.simulate(20)
    b = S2.build_coupled(pyfds_gb300, spec, build_field, exact=True)
    monkeypatch.setattr(type(b), "_native_path", lambda self: False)
    b.simulate(7)
    b.simulate(20)
    assert a.step == b.step == 27
    for (sa, ga), (sb, gb) in zip(S2.coupled_results(a, kind_of), S2.coupled_results(b, kind_of)):
        for c in sa:
            assert np.array_equal(sa[c], sb[c]), c
            for x, y in zip(ga[c], gb[c]):
                assert np.array_equal(x, y), c


@pytest.mark.parametrize("kind,nx,ny", [("Acoustic2D", 1, 1), ("Acoustic2D", 1, 7),
                                        ("Acoustic2D", 7, 1), ("Acoustic2D", 2, 2),
                                        ("Thermal2D", 1, 5), ("Acoustic1D", 1, None),
                                        ("Thermal1D", 3, None)])
def test_degenerate_grids_vs_oracle(gpu, kind, nx, ny):
    """Grids of one row, one column, one cell: exact mode against the oracle."""
    spec = S.random_scenario(900 + nx * 10 + (ny or 0), kind, nx, ny, steps=9)
    f = build_field(spec, exact=True)
    f.simulate(spec["steps"])
    st, sig = field_results(f)
    ref_st, ref_sig = O.simulate(spec, spec["steps"])
    for c in st:
        assert np.array_equal(st[c], ref_st[c]), c
        for x, y in zip(sig[c], ref_sig[c]):
            assert np.array_equal(x, y), c


def test_largest_grid_scales_exactly(gpu):
    """8192^2 cells (the largest grid in the tests; 4.3 GB of state and coefficients):
    exact-mode time stepping is linear in the state and the sources, and scaling both
    by 2 is exact in IEEE arithmetic, so every value and output must double bit for
    bit."""
    n, steps = 8192, 6
    spec = workloads.acoustic2d_steel_block(n=n, nt=steps, n_probes=16)
    rng = np.random.default_rng(5)
    p0 = rng.standard_normal(n * n) * 1e-3
    results = []
    for k in (1.0, 2.0):
        sp = dict(spec)
        sp["init"] = {"pressure": k * p0}
        sp["bounds"] = {"pressure": [dict(b, value=k * np.asarray(b["value"]))
                                     for b in spec["bounds"]["pressure"]]}
        f = build_field(sp, exact=True)
        f.simulate(steps)
        results.append(field_results(f))
        del f
    (s1, g1), (s2, g2) = results
    for c in s1:
        assert np.array_equal(2.0 * s1[c], s2[c]), c
        assert np.count_nonzero(s1[c]) > 0
        for x, y in zip(g1[c], g2[c]):
            assert np.array_equal(2.0 * x, y), c
