"""pyfds_gb300 exposes the reference's public Python interface: every module, every
name of each module's ``__all__`` at the package top level (the reference's
``__init__`` star-imports them), every class and function the module defines, the
public members of each class body, and constructor / function parameters that
accept the reference's calls (the same positional parameters in the same order,
the same defaults; extra parameters only after them). The interface is read from
tests/golden/api_surface.json (written by tests/golden/make_api_surface.py from the
reference); no GPU and no reference tree are needed."""
import importlib
import inspect
import json
import os

import pytest

import pyfds_gb300

HERE = os.path.dirname(os.path.abspath(__file__))
with open(os.path.join(HERE, "golden", "api_surface.json")) as f:
    SURFACE = json.load(f)["modules"]

# modules of the reference outside the time-stepping path, with the reason
OUT_OF_SCOPE = {
    "electrostatics": "Electrostatic1D/2D: a static Poisson solve through a sparse inverse, "
                      "not time stepping",
}
IN_SCOPE = sorted(m for m in SURFACE if m not in OUT_OF_SCOPE)

ITEMS = [(m, name) for m in IN_SCOPE for name in sorted(SURFACE[m]["names"])]


def _ours(module, name):
    mod = importlib.import_module("pyfds_gb300." + module)
    return getattr(mod, name, None)


@pytest.mark.parametrize("module", IN_SCOPE)
def test_module_and_exports(module):
    importlib.import_module("pyfds_gb300." + module)
    missing = [n for n in SURFACE[module]["all"] if not hasattr(pyfds_gb300, n)]
    assert not missing, missing


def _accepts(ref_params, ours):
    """Whether a callable with signature `ours` accepts every call the reference's
    parameter list allows."""
    if ref_params is None:
        return True
    kinds = {k for _, k, _ in ref_params}
    ref_names = [n for n, k, _ in ref_params if k == "POSITIONAL_OR_KEYWORD"]
    if ref_names and ref_names[0] == "self":
        ref_names = ref_names[1:]
    if not ref_names and kinds <= {"VAR_POSITIONAL", "VAR_KEYWORD", "POSITIONAL_OR_KEYWORD"}:
        # (self, *args, **kwargs): the reference forwards everything to a base class
        return True
    params = list(inspect.signature(ours).parameters.values())
    has_var_kw = any(p.kind == p.VAR_KEYWORD for p in params)
    has_var_pos = any(p.kind == p.VAR_POSITIONAL for p in params)
    pos = [p.name for p in params if p.kind == p.POSITIONAL_OR_KEYWORD]
    if pos and pos[0] == "self":
        pos = pos[1:]
    if pos[:len(ref_names)] != ref_names:
        return False
    names = {p.name: p for p in params}
    for n, k, default in ref_params:
        if k == "KEYWORD_ONLY" and n not in names and not has_var_kw:
            return False
        # a parameter the reference lets callers omit has the same default here
        if default is not None and n in names and repr(names[n].default) != default:
            return False
        if k == "VAR_POSITIONAL" and not has_var_pos:
            return False
        if k == "VAR_KEYWORD" and not has_var_kw:
            return False
    return True


@pytest.mark.parametrize("module,name", ITEMS)
def test_name(module, name):
    spec = SURFACE[module]["names"][name]
    ours = _ours(module, name)
    assert ours is not None, "pyfds_gb300.%s.%s is missing" % (module, name)
    if spec["kind"] == "class":
        assert inspect.isclass(ours)
        missing = [m for m in spec["members"] if not hasattr(ours, m)]
        assert not missing, missing
        assert _accepts(spec["params"], ours.__init__), (spec["params"],
                                                         str(inspect.signature(ours.__init__)))
    else:
        assert callable(ours)
        assert _accepts(spec["params"], ours), (spec["params"], str(inspect.signature(ours)))


def test_fixture_covers_the_reference_modules():
    assert set(SURFACE) == set(IN_SCOPE) | set(OUT_OF_SCOPE)
    assert sum(len(SURFACE[m]["names"]) for m in IN_SCOPE) >= 30


def test_output_blocks_become_lists():
    """Samples recorded by GPU calls (Output._record) read as the reference's lists:
    new lists when first read, lists that exist (and references to them) grow in
    place, a reset drops what was not read."""
    import numpy as np
    from pyfds_gb300 import regions
    o = regions.Output(regions.Region([1, 2], "out"))
    o._record(np.array([[1.0, 2.0], [3.0, 4.0]]))
    o._record(np.array([[5.0], [6.0]]))
    assert o.signals == [[1.0, 2.0, 5.0], [3.0, 4.0, 6.0]]
    held = o.signals[0]
    o._record(np.array([[7.0], [8.0]]))
    assert held == [1.0, 2.0, 5.0, 7.0]
    assert o.signals[1] == [3.0, 4.0, 6.0, 8.0]
    o.signals = []
    o._record(np.array([[9.0], [10.0]]))
    o.signals = []
    assert o.signals == []
