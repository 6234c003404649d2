"""The batch autotuner's host side: every candidate is a tile shape the library builds
(two-step candidates are exactly the two-step tiles), its cache file round-trips and
a corrupt one is ignored, and the size key separates field class, precision, batch
size and instance size. No GPU (the timing trials themselves are GPU tests)."""
import json

import pytest

from oracle import scenarios as S
from pyfds_gb300 import _build, _capi, autotune, workloads


@pytest.fixture(scope="module")
def menu():
    _build.build()
    return _capi.tile_menu()


def test_candidates_are_built_shapes(menu):
    assert len(set(autotune.CANDIDATES)) == len(autotune.CANDIDATES)
    for tile, stages in autotune.CANDIDATES:
        assert tuple(tile) in menu, tile
        assert stages in (1, 2, 3)
    two_step = {tuple(t) for t, s in autotune.CANDIDATES if s == 3}
    assert two_step == set(_capi.TWO_STEP_TILES)


def test_cache_round_trip_and_corrupt_file(tmp_path, monkeypatch):
    path = tmp_path / "sub" / "tune.json"
    monkeypatch.setenv("PYFDS_GB300_AUTOTUNE", str(path))
    assert autotune.cache_path() == str(path)
    assert autotune._load() == {}                      # no file yet
    entry = {"Acoustic2D/f64/n2/mean2^8": {"tile": [64, 16], "stages": 3, "ms": 1.0}}
    autotune._save(entry)                              # creates the directory
    assert json.loads(path.read_text()) == entry
    assert autotune._load() == entry
    path.write_text("{not json")
    assert autotune._load() == {}


def _fields(count, n, precision="f64"):
    return [workloads.build_field(S.random_scenario(k, "Acoustic2D", n, n, steps=2, mu=False),
                                  precision=precision) for k in range(count)]


def test_size_key_separates_classes():
    base = autotune.size_key(_fields(4, 16))
    assert base == "Acoustic2D/f64/n2/mean2^8"
    assert autotune.size_key(_fields(4, 16, precision="f32")) != base
    assert autotune.size_key(_fields(8, 16)) != base
    assert autotune.size_key(_fields(4, 64)) != base
    # the same class for a batch of the same kind and size
    assert autotune.size_key(_fields(4, 16)) == base
