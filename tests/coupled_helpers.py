"""Shared by the coupled-field tests: fixture inputs and results per field."""

from golden_inputs import apply_inputs
from oracle import scenarios as S


def coupled_spec(case, g):
    spec = S.coupled_scenario(case["seed"], case["variant"], case["nx"], case["steps"])
    prefix = "c%d/" % case["seed"]
    if spec["kind"] == "ThermoAcoustic1D":
        apply_inputs(spec, g, prefix)
    else:
        for k, f in enumerate(spec["fields"]):
            apply_inputs(f, g, prefix + "f%d/" % k)
    return spec, prefix


def compare(results, g, prefix, check):
    for k, (st, sig) in enumerate(results):
        for c in st:
            check(st[c], g[prefix + "f%d/%s/state" % (k, c)], (k, c))
            for j, x in enumerate(sig[c]):
                check(x, g[prefix + "f%d/%s/sig%d" % (k, c, j)], (k, c, j))


def kind_of(field):
    return type(field).__name__
