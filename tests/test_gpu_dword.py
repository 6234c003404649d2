"""GPU parity of the double-word precision (precision="dw") against the reference.

A double word is a float32 pair hi + lo with a 48-bit significand (unit roundoff
2^-48 ~ 3.6e-15) computed with compensated float32 arithmetic, so the mode is
held to the float64 drop-in's bar: every recorded output and the final state
within a relative L2 error of 1e-12 of the unmodified reference (the fixtures of
tests/golden/make_golden.py), including the full 2048^2 x 4000-step water/steel
run. Grids the fixtures do not hold are checked against the oracle.

One difference from float64 is stated in the check: the float32 exponent range.
Ahead of a wavefront the reference carries precursor values down to 1e-300 that
double words flush to zero below ~1e-38, so outputs the wave has not reached
(reference norm below 1e-6 of the run's largest output) are held to an absolute
bar instead, 1e-12 of the largest output's norm.
"""
import json
import warnings

import numpy as np
import pytest

from oracle import fds_oracle as O
from oracle import scenarios as S
from golden_inputs import apply_inputs
from helpers import build_field, field_results, rel_l2
from pyfds_gb300 import workloads
from test_gpu_parity import MENU, TOL, check_state, golden

pytestmark = pytest.mark.gpu

FLOOR = 1e-6  # outputs below FLOOR x the largest output norm: not reached


def check_rows(rows, refs, tol=TOL, floor=FLOOR):
    """Relative L2 per reached output row, absolute (x the largest norm) for the
    others; returns (worst relative error, number of unreached rows)."""
    top = max((float(np.linalg.norm(r)) for r in refs), default=0.0)
    worst, unreached = 0.0, 0
    for a, b in zip(rows, refs):
        nb = float(np.linalg.norm(b))
        if nb >= floor * top and nb > 0:
            e = rel_l2(a, b)
            worst = max(worst, e)
            assert e <= tol, e
        else:
            unreached += 1
            assert float(np.linalg.norm(a - b)) <= tol * top
    return worst, unreached


# double words have unit roundoff 2^-48 against float64's 2^-53 (x 32); a
# compensated step rounds its low word up to three times where a float64 FMA rounds
# once, and the ratio of two rounding errors spreads: x 8 on top (the largest ratio
# measured on these scenarios' outputs is 154)
DW_FACTOR = 256


def check_rows_scaled(rows, rows64, refs, groups):
    """check_rows, with each reached row held to 1e-12 or DW_FACTOR x the float64
    step's largest error on the rows of its output (``groups``: an output id per
    row; the rows of one output sample the same quantity, so they share its
    conditioning, while a single row's float64 error can be small by chance)."""
    top = max((float(np.linalg.norm(r)) for r in refs), default=0.0)
    scale = {}
    for a64, b, gid in zip(rows64, refs, groups):
        if float(np.linalg.norm(b)) >= FLOOR * top and np.linalg.norm(b) > 0:
            scale[gid] = max(scale.get(gid, 0.0), rel_l2(a64, b))
    for a, b, gid in zip(rows, refs, groups):
        nb = float(np.linalg.norm(b))
        if nb >= FLOOR * top and nb > 0:
            assert rel_l2(a, b) <= max(TOL, DW_FACTOR * scale[gid]), gid
        else:
            assert float(np.linalg.norm(a - b)) <= TOL * top


def check_signals(sig, g, prefix, comps, exact=False, tol=TOL):
    rows, refs = [], []
    for c in comps:
        for j, s in enumerate(sig[c]):
            ref = g[prefix + c + "/sig%d" % j]
            assert s.shape == ref.shape, (c, j, s.shape, ref.shape)
            rows += list(s)
            refs += list(ref)
    return check_rows(rows, refs, tol)[0]


def test_random_scenarios_vs_reference(gpu):
    """Every field family (1-D, 2-D, axisymmetric; acoustic with and without
    absorption; thermal) on ragged grids. Each output and state is held to 1e-12 or,
    where the float64 step's own error on it exceeds 1e-12 / DW_FACTOR, to DW_FACTOR
    x that error: such outputs amplify rounding (these thermal scenarios put 0 K
    Dirichlet cells next to 300 K ones, and the heat flux is a difference of the
    two), and the amplification costs double words the bits they lack."""
    g = golden("random_scenarios.npz")
    cases = json.loads(str(g["cases"]))
    for case in cases:
        spec = S.random_scenario(case["seed"], case["kind"], case["nx"], case["ny"],
                                 steps=case["steps"], mu=case["mu"])
        prefix = "s%d/" % case["seed"]
        apply_inputs(spec, g, prefix)
        res = {}
        for prec in ("f64", "dw"):
            f = build_field(spec, precision=prec)
            f.simulate(spec["steps"])
            res[prec] = field_results(f)
        comps = O.components_of(case["kind"])
        rows, rows64, refs, groups = [], [], [], []
        for c in comps:
            key = prefix + c + "/state"
            if key in g.files:
                e64 = rel_l2(res["f64"][0][c], g[key])
                assert rel_l2(res["dw"][0][c], g[key]) <= max(TOL, DW_FACTOR * e64), c
            for j, sd in enumerate(res["dw"][1][c]):
                rows += list(sd)
                rows64 += list(res["f64"][1][c][j])
                refs += list(g[prefix + c + "/sig%d" % j])
                groups += [(c, j)] * len(sd)
        check_rows_scaled(rows, rows64, refs, groups)


def test_acoustic1d_water_vs_reference(gpu):
    g = golden("acoustic1d_water.npz")
    spec = apply_inputs(workloads.acoustic1d_water(), g)
    f = build_field(spec, precision="dw")
    f.simulate()
    st, sig = field_results(f)
    check_state(st, g, "", ["pressure", "velocity"], False)
    check_signals(sig, g, "", ["pressure"], False)


def test_axi_small_vs_reference(gpu):
    g = golden("axi_disc_256x1024.npz")
    spec = apply_inputs(workloads.axi_disc_source(256, 1024, 500, disc=50, probe_every=32), g)
    f = build_field(spec, precision="dw")
    f.simulate(spec["steps"])
    st, sig = field_results(f)
    check_signals(sig, g, "", ["pressure"], False)
    check_state(st, g, "", O.components_of("Acoustic3DAxi"), False)


def test_thermal2d_small_vs_reference(gpu):
    g = golden("thermal2d_512.npz")
    spec = apply_inputs(workloads.thermal2d_two_materials(512, 500, 64), g)
    f = build_field(spec, precision="dw")
    f.simulate(spec["steps"])
    st, sig = field_results(f)
    check_signals(sig, g, "", ["temperature"], False)
    check_state(st, g, "", ["temperature"], False)


def test_thermal2d_with_potential_offset(gpu):
    """A temperature offset near the field's temperatures: the 48 bits then resolve
    the deviation, and the result stays within the bar."""
    g = golden("thermal2d_512.npz")
    spec = apply_inputs(workloads.thermal2d_two_materials(512, 500, 64), g)
    f = build_field(spec, precision="dw")
    f.potential_offset = float(np.mean(f.temperature.values))
    f.simulate(spec["steps"])
    assert f._engine().offset == f.potential_offset != 0.0
    st, sig = field_results(f)
    check_signals(sig, g, "", ["temperature"], False)
    check_state(st, g, "", ["temperature"], False)


def test_acoustic2d_steel_2048_full_vs_reference(gpu):
    """The 2048^2 water/steel workload, all 4000 steps, 64 outputs: the same bar
    as the float64 step (outputs 1e-12; final state 1e-11, as for float64, whose
    velocity fields hold regions the wave has barely reached)."""
    g = golden("acoustic2d_steel_2048.npz")
    spec = apply_inputs(workloads.acoustic2d_steel_block(), g)
    f = build_field(spec, precision="dw")
    f.simulate(spec["steps"])
    st, sig = field_results(f)
    worst = check_signals(sig, g, "", ["pressure"], exact=False)
    assert worst <= TOL
    check_state(st, g, "", O.components_of("Acoustic2D"), exact=False, tol=1e-11)


def test_acoustic_flow_vs_reference(gpu):
    """Moving medium: the row shifts move double words as 8-byte units."""
    g = golden("acoustic_flow.npz")
    for case in json.loads(str(g["cases"])):
        with warnings.catch_warnings():
            warnings.simplefilter("ignore")
            spec = S.flow_scenario(case["seed"], case["nx"], case["ny"], steps=case["steps"],
                                   flow=case["flow"], mu=case["mu"])
            prefix = "f%d/" % case["seed"]
            apply_inputs(spec, g, prefix)
            f = build_field(spec, precision="dw")
        f.simulate(spec["steps"])
        st, sig = field_results(f)
        comps = O.components_of("AcousticFlow2D")
        check_state(st, g, prefix, comps, False)
        check_signals(sig, g, prefix, comps, False)


@pytest.mark.parametrize("kind,nx,ny", [("Acoustic2D", 1, 1), ("Acoustic2D", 1, 7),
                                        ("Acoustic2D", 7, 1), ("Thermal2D", 1, 5),
                                        ("Acoustic1D", 1, None), ("Thermal1D", 3, None)])
def test_degenerate_grids_vs_oracle(gpu, kind, nx, ny):
    spec = S.random_scenario(900 + nx * 10 + (ny or 0), kind, nx, ny, steps=9)
    f = build_field(spec, precision="dw")
    f.simulate(spec["steps"])
    st, sig = field_results(f)
    ref_st, ref_sig = O.simulate(spec, spec["steps"])
    rows, refs = [], []
    for c in st:
        assert rel_l2(st[c], ref_st[c]) <= TOL, c
        for x, y in zip(sig[c], ref_sig[c]):
            rows += list(x)
            refs += list(y)
    check_rows(rows, refs)


@pytest.mark.parametrize("nx", [203, 204])  # 204: rows are 16-byte multiples -> TMA staging
# shared-memory tiles have power-of-two widths; register-marching ones 32k - 2
@pytest.mark.parametrize("tile,stages", [m for m in MENU if (m[0][0] & (m[0][0] - 1)) == 0])
@pytest.mark.parametrize("kind", ["Acoustic2D", "Thermal2D"])
def test_tile_menu_parity(gpu, tile, kind, stages, nx):
    """The tile menu's shared-memory variants (the register-marching ones are
    float64 / float32 only) against the oracle."""
    from pyfds_gb300 import _capi
    spec = S.random_scenario(21, kind, nx, 77, steps=15, mu=False)
    st_o, sg_o = O.simulate(spec, spec["steps"])
    f = build_field(spec, tile=tile, precision="dw")
    f.stages = stages
    try:
        f.simulate(spec["steps"])
    except _capi.FdsError as e:
        if e.code == _capi.FDS_E_SIZE:
            pytest.skip("does not fit in shared memory: %s" % e)
        raise
    st, sig = field_results(f)
    rows, refs = [], []
    for c in st_o:
        assert rel_l2(st[c], st_o[c]) <= TOL, c
        for x, y in zip(sig[c], sg_o[c]):
            rows += list(x)
            refs += list(y)
    check_rows(rows, refs)


def test_sim_step_loop_equals_simulate(gpu):
    spec = S.random_scenario(7, "Acoustic2D", 70, 40, steps=12)
    a = build_field(spec, precision="dw")
    a.simulate(12)
    b = build_field(spec, precision="dw")
    for _ in range(12):
        b.sim_step()
        b.step += 1
    sa, ga = field_results(a)
    sb, gb = field_results(b)
    for c in sa:
        assert np.array_equal(sa[c], sb[c])
        for x, y in zip(ga[c], gb[c]):
            assert np.array_equal(x, y)


def test_values_round_trip(gpu):
    """Host values go up as (hi, lo) pairs and come back as hi + lo: 48 bits of
    every value survive (relative error <= 2^-48)."""
    spec = S.random_scenario(11, "Acoustic2D", 33, 17, steps=3)
    f = build_field(spec, precision="dw")
    f.assemble_matrices()
    x = np.random.default_rng(3).standard_normal(f.num_points) * 1e4
    f.pressure.values = x.copy()
    eng = f._engine()
    eng.prepare(0, 0)
    assert tuple(eng.buffers["pressure"][0].shape) == (f.num_points, 2)
    y = eng.download("pressure")
    assert np.all(np.abs(y - x) <= 2.0 ** -48 * np.abs(x))
    d = eng.device_values("pressure").cpu().numpy()
    assert np.array_equal(d, y)


def test_batch_matches_single_and_oracle(gpu):
    """Batched double words (one launch per step for six fields of uneven size) are
    the single-field double-word result bit for bit, and within the bar of the
    oracle (scaled by the float64 step's own error, as for the random scenarios)."""
    from pyfds_gb300.batch import simulate_batch
    sizes = [(204, 77), (203, 64), (64, 256), (37, 19), (130, 130), (256, 32)]
    for kind in ("Acoustic2D", "Thermal2D"):
        sp = [S.random_scenario(70 + k, kind, nx, ny, steps=14, mu=False)
              for k, (nx, ny) in enumerate(sizes)]
        batch = [build_field(s, precision="dw") for s in sp]
        simulate_batch(batch, 14)
        for s, fb in zip(sp, batch):
            single = build_field(s, precision="dw")
            single.simulate(14)
            f64 = build_field(s)
            f64.simulate(14)
            a_st, a_sg = field_results(fb)
            b_st, b_sg = field_results(single)
            c_st, c_sg = field_results(f64)
            st_o, sg_o = O.simulate(s, 14)
            rows, rows64, refs, groups = [], [], [], []
            for c in a_st:
                assert np.array_equal(a_st[c], b_st[c]), c
                e64 = rel_l2(c_st[c], st_o[c])
                assert rel_l2(a_st[c], st_o[c]) <= max(TOL, DW_FACTOR * e64), c
                for j, (x, y, x64, z) in enumerate(zip(a_sg[c], b_sg[c], c_sg[c], sg_o[c])):
                    assert np.array_equal(x, y)
                    rows += list(x)
                    rows64 += list(x64)
                    refs += list(z)
                    groups += [(c, j)] * len(x)
            check_rows_scaled(rows, rows64, refs, groups)


def test_batch_graph_replay(gpu):
    """A captured double-word batch (warm-up launch, then one replay) ends in the
    same state as two direct launches."""
    import torch
    from pyfds_gb300.batch import BatchRunner
    sp = [S.random_scenario(80 + k, "Acoustic2D", 96, 40 + 8 * k, steps=8, mu=False)
          for k in range(3)]
    a = [build_field(s, precision="dw") for s in sp]
    b = [build_field(s, precision="dw") for s in sp]
    ra = BatchRunner(a, 8)
    ra.capture()
    ra.replay()
    rb = BatchRunner(b, 8)
    rb.launch()
    rb.launch()
    torch.cuda.synchronize()
    for fa, fb in zip(a, b):
        for name in fa._stag_components:
            assert torch.equal(fa._engine().buffers[name][0], fb._engine().buffers[name][0]), name


def test_device_split_and_join_match_the_host(gpu):
    """fds_dw_split / fds_dw_join produce the bits of split_dw / join_dw."""
    import torch
    from pyfds_gb300._engine import device_join_dw, join_dw, split_dw, upload_dw
    rng = np.random.default_rng(12)
    x = np.concatenate([rng.standard_normal(100001) * 10.0 ** rng.integers(-30, 30, 100001),
                        [0.0, -0.0, 1.0, 3e38, -1e-40]])
    dev = torch.device("cuda", 0)
    pairs = upload_dw(torch, dev, x)
    assert np.array_equal(pairs.cpu().numpy().view(np.uint32), split_dw(x).view(np.uint32))
    back = device_join_dw(torch, pairs).cpu().numpy()
    assert np.array_equal(back.view(np.uint64), join_dw(split_dw(x)).view(np.uint64))
