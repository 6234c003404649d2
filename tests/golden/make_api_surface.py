"""Record the reference package's public Python interface as tests/golden/api_surface.json.

Run here, where the reference source tree is available (it is read, never modified):

    python tests/golden/make_api_surface.py [/path/to/reference]

For every module of the reference package the fixture lists its ``__all__`` and,
for each class or function the module defines (public names only), the parameters
of the constructor or function (name, kind, repr of the default) and, for classes,
the public members the class body defines. Only names and default values are
recorded, no code. ``tests/test_api_surface.py`` checks pyfds_gb300 against it without
the reference.
"""
import importlib
import inspect
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
MODULES = ("acoustic_flow", "acoustics", "coupled_fields", "coupling", "electrostatics",
           "fields", "gfx", "nonlinear_acoustics", "regions", "thermal")


def _params(fn):
    try:
        sig = inspect.signature(fn)
    except (TypeError, ValueError):
        return None
    return [[p.name, p.kind.name, None if p.default is p.empty else repr(p.default)]
            for p in sig.parameters.values()]


def surface(pkg_name="pyfds"):
    out = {}
    for m in MODULES:
        mod = importlib.import_module(pkg_name + "." + m)
        names = {}
        for name, obj in sorted(vars(mod).items()):
            if name.startswith("_") or getattr(obj, "__module__", None) != mod.__name__:
                continue
            if inspect.isclass(obj):
                members = sorted(k for k in vars(obj) if not k.startswith("_"))
                names[name] = {"kind": "class", "params": _params(obj.__init__),
                               "members": members}
            elif inspect.isfunction(obj):
                names[name] = {"kind": "function", "params": _params(obj)}
        out[m] = {"all": sorted(getattr(mod, "__all__", [])), "names": names}
    return out


def main():
    sys.path.insert(0, ROOT)
    from oracle.ref_loader import DEFAULT_REFERENCE_ROOT, load_reference
    root = sys.argv[1] if len(sys.argv) > 1 else DEFAULT_REFERENCE_ROOT
    load_reference(root)
    data = {"package": "pyfds", "modules": surface()}
    path = os.path.join(HERE, "api_surface.json")
    with open(path, "w") as f:
        json.dump(data, f, indent=1, sort_keys=True, ensure_ascii=False)
        f.write("\n")
    print("wrote", path)


if __name__ == "__main__":
    main()
