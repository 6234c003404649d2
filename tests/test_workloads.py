"""The seeded synthetic workloads have the shapes, materials, regions, sources, probes
and time steps of the configurations the benchmarks are quoted on: Acoustic1D water
(1000 cells), Acoustic2D water with a steel block (2048^2), 256 layered-media
instances, Acoustic3DAxi disc source (1024 x 4096), Thermal2D aluminium/polymer
(4096^2) and the surrogate's 256^2 layered media. Sizes are checked at full scale where
building the spec is cheap; the oracle runs only the 1-D case. No GPU."""
import numpy as np
import pytest

from oracle import fds_oracle as O
from pyfds_gb300 import workloads as W


def _pulse(t, f, t0, sigma):
    return np.sin(2 * np.pi * f * t) * np.exp(-(t - t0) ** 2 / (2 * sigma ** 2))


def test_acoustic1d_water():
    for additive in (True, False):
        s = W.acoustic1d_water(additive=additive)
        assert (s["kind"], s["nx"], s["nt"]) == ("Acoustic1D", 1000, 2000)
        assert s["dx"] == 1e-4 and np.isclose(s["dt"], 0.5e-4 / 1500)
        assert s["materials"] == [(None, W.WATER)] and W.WATER["sound_velocity"] == 1500
        b = s["bounds"]["pressure"]
        assert [list(x["indices"]) for x in b] == [[0], [999], [100]]
        assert [x["additive"] for x in b] == [False, False, additive]
        assert b[0]["value"] == 0 and b[1]["value"] == 0
        t = np.arange(2000) * s["dt"]
        assert np.allclose(b[2]["value"], _pulse(t, 1e6, 2e-6, 0.5e-6), rtol=0, atol=1e-15)
        assert s["outputs"] == {"pressure": [[800]]}


def test_acoustic1d_water_probe_peak():
    """The additive case's probe peaks at |p| = 0.807 (a stated property of this
    configuration)."""
    s = W.acoustic1d_water()
    _, sig = O.simulate(s, s["steps"])
    assert round(float(np.abs(np.asarray(sig["pressure"][0])).max()), 3) == 0.807


def test_acoustic2d_steel_block():
    n = 2048
    s = W.acoustic2d_steel_block()
    assert (s["kind"], s["nx"], s["ny"], s["nt"]) == ("Acoustic2D", n, n, 4000)
    assert s["dx"] == s["dy"] == 5e-5
    assert np.isclose(s["dt"], 0.5 * 5e-5 / (5900 * np.sqrt(2)))
    (main, m0), (steel, m1) = s["materials"]
    assert main is None and m0 == W.WATER and m1 == W.STEEL
    assert (W.STEEL["sound_velocity"], W.STEEL["density"]) == (5900, 7850)
    # [800:1200, 1000:1600], x first (x outer, y inner)
    want = [x + y * n for x in range(800, 1200) for y in range(1000, 1600)]
    assert list(steel) == want
    edges, line = s["bounds"]["pressure"]
    cells = set(range(n)) | {(n - 1) * n + x for x in range(n)} | \
        {y * n for y in range(n)} | {y * n + n - 1 for y in range(n)}
    assert set(np.asarray(edges["indices"]).tolist()) == cells and len(edges["indices"]) == len(cells)
    assert edges["value"] == 0 and not edges["additive"]
    assert list(line["indices"]) == [200 * n + x for x in range(512, 1537)]
    assert line["additive"] and len(line["indices"]) == 1025
    t = np.arange(4000) * s["dt"]
    assert np.allclose(line["value"], _pulse(t, 1e6, 2e-6, 0.5e-6), rtol=0, atol=1e-15)
    probes = s["outputs"]["pressure"][0]
    assert len(probes) == 64 and len(set(probes)) == 64
    xs, ys = np.asarray(probes) % n, np.asarray(probes) // n
    assert xs.min() >= 1 and xs.max() <= n - 2 and ys.min() >= 1 and ys.max() <= n - 2
    assert probes == W.acoustic2d_steel_block()["outputs"]["pressure"][0]  # seeded


def test_layered_media_batch():
    specs = W.layered_media_batch()
    assert len(specs) == 256
    sides = np.array([s["nx"] for s in specs])
    assert all(s["nx"] == s["ny"] for s in specs)
    assert sides.min() >= 128 and sides.max() <= 1024
    # log-uniform sides: E[n^2] = (1024^2 - 128^2) / (2 ln 8), about 2.48e5
    assert 1.8e5 < np.mean(sides.astype(float) ** 2) < 3.2e5
    for s in specs[:32]:
        n = s["nx"]
        assert s["kind"] == "Acoustic2D" and s["nt"] == 2000
        mats = s["materials"]
        assert 3 <= len(mats) <= 8
        cs = [m["sound_velocity"] for _, m in mats]
        rhos = [m["density"] for _, m in mats]
        assert min(cs) >= 1000 and max(cs) <= 3000 and min(rhos) >= 800 and max(rhos) <= 2000
        assert np.isclose(s["dt"], 0.4 * s["dx"] / max(cs))          # Courant 0.4
        f = 1 / (20 * s["dx"]) * min(cs)                             # dx = c_min / (20 f)
        assert 0.5e6 <= f <= 5e6
        # the layers partition the rows: every cell of a later layer lies in its rows
        for idx, _ in mats[1:]:
            rows = np.unique(np.asarray(idx) // n)
            assert np.array_equal(rows, np.arange(rows[0], rows[-1] + 1))
            assert len(idx) == n * len(rows)
        bounds = s["bounds"]["pressure"]
        assert any(not b["additive"] and b["value"] == 0 for b in bounds)
        src = [b for b in bounds if b["additive"]]
        assert len(src) == 1 and len(src[0]["indices"]) == 1
        assert len(s["outputs"]["pressure"][0]) == 16


def test_axi_disc_source():
    s = W.axi_disc_source()
    assert (s["kind"], s["nx"], s["ny"], s["nt"]) == ("Acoustic3DAxi", 1024, 4096, 6000)
    assert s["dx"] == s["dy"] == 5e-5
    assert np.isclose(s["dt"], 0.5 * 5e-5 / (1500 * np.sqrt(2)))
    (src,) = s["bounds"]["pressure"]
    assert list(src["indices"]) == list(range(200)) and src["additive"]
    t = np.arange(6000) * s["dt"]
    assert np.allclose(src["value"], _pulse(t, 2e6, 1e-6, 0.25e-6), rtol=0, atol=1e-15)
    assert s["outputs"]["pressure"][0] == [y * 1024 for y in range(0, 4096, 64)]


def test_thermal2d_two_materials():
    n = 4096
    s = W.thermal2d_two_materials()
    assert (s["kind"], s["nx"], s["ny"], s["nt"]) == ("Thermal2D", n, n, 50000)
    assert s["dx"] == s["dy"] == 1e-4
    (_, alu), (poly, pm) = s["materials"]
    assert (alu["heat_capacity"], alu["density"], alu["thermal_conductivity_x"]) == (897, 2700, 237)
    assert (pm["heat_capacity"], pm["density"], pm["thermal_conductivity_x"]) == (1470, 1190, 0.19)
    alpha = 237 / (2700 * 897)
    assert np.isclose(s["dt"], 0.2 * 1e-8 / (4 * alpha)) and abs(s["dt"] - 5.1e-6) < 0.05e-6
    # the polymer lies above one interface row per column, around the middle
    poly = np.asarray(poly)
    x, y = poly % n, poly // n
    first = np.full(n, n)
    np.minimum.at(first, x, y)
    assert np.all(first > n * 0.3) and np.all(first < n * 0.7)
    assert len(poly) == np.sum(n - first)                    # every cell above it
    assert np.all(s["init"]["temperature"] == 293.15)
    (b,) = s["bounds"]["temperature"]
    assert list(b["indices"]) == [y * n for y in range(n)] and b["value"] == 373.15
    assert not b["additive"]
    probes = s["outputs"]["temperature"][0]
    assert len(probes) == 64


@pytest.mark.parametrize("builder", ["acoustic2d_steel_block", "layered_media_batch",
                                     "thermal2d_two_materials"])
def test_seeded_builders_are_deterministic(builder):
    a, b = getattr(W, builder)(), getattr(W, builder)()
    if isinstance(a, list):
        a, b = a[:4], b[:4]
    else:
        a, b = [a], [b]
    for x, y in zip(a, b):
        assert x["outputs"] == y["outputs"]
        for (ia, _), (ib, _) in zip(x["materials"], y["materials"]):
            assert (ia is None and ib is None) or np.array_equal(ia, ib)


def test_surrogate_media():
    """Surrogate training / evaluation media: the layered kind at a fixed 256^2 grid,
    the source cut to zero from step 704, per-cell c and rho maps consistent with the
    material regions (the oracle's material vector)."""
    specs = W.surrogate_media(12, seed=5)
    assert len(specs) == 12
    for s in specs:
        n = s["nx"]
        assert (n, s["ny"], s["nt"], s["t_src"]) == (256, 256, 4096, 704)
        cs = [m["sound_velocity"] for _, m in s["materials"]]
        assert 3 <= len(cs) <= 8 and np.isclose(s["dt"], 0.4 * s["dx"] / max(cs))
        assert np.isclose(s["dx"], min(cs) / (20 * s["frequency"]))
        assert 0.5e6 <= s["frequency"] <= 5e6
        src = [b for b in s["bounds"]["pressure"] if b["additive"]][0]["value"]
        assert np.all(src[704:] == 0) and np.any(src[:704] != 0)
        c = O.material_vector(n * n, s["materials"], "sound_velocity")
        rho = O.material_vector(n * n, s["materials"], "density")
        assert np.array_equal(s["c_map"].reshape(-1), c)
        assert np.array_equal(s["rho_map"].reshape(-1), rho)
    assert W.surrogate_media(3, seed=5)[0]["frequency"] == specs[0]["frequency"]
