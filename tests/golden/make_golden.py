"""Generate the golden fixtures in this directory from the unmodified reference.

Run where the reference source tree is available (PYFDS_REFERENCE_ROOT, or a
``reference`` directory beside the repository checkout)::

    python tests/golden/make_golden.py [--skip-large]

The reference is imported with two harness shims (see oracle/ref_loader.py); its
source is not modified. Fixtures:

- operators.npz: dense DIA operators of small fields of every kind (random
  materials, absorption on, anisotropic conductivity), as the reference assembles
  them. Thermal2D/Thermal3DAxi operators have no known-answer test upstream.
- random_scenarios.npz: final states and every recorded output of seeded random
  scenarios (oracle/scenarios.py) covering all boundary/output modes.
- acoustic1d_water.npz: the 1-D water workload (1000 cells, 2000 steps), full.
- acoustic2d_steel_2048.npz: the 2048^2 water/steel workload, 4000 steps, its 64
  outputs (about 15 minutes of reference CPU time; --skip-large skips it).
- axi_disc_256x1024.npz, thermal2d_512.npz: reduced axisymmetric / thermal
  workloads (500 steps), outputs and final-state norms.
- axi_disc_full_prefix.npz, thermal2d_4096_prefix.npz: the full-size axisymmetric
  and thermal workloads for their first 100 steps (--skip-large skips them).
- axi_disc_full_1000.npz, thermal2d_4096_1000.npz: the same full-size workloads for
  their first 1000 steps, every output (about 12 and 7 minutes of reference CPU
  time; --skip-large skips them).
- acoustic_flow.npz: AcousticFlow2D (moving medium) scenarios, oracle/scenarios.py
  ``flow_scenario``: per-row and scalar flows, periods 1..9, negative and zero flows.
- coupling.npz: coupled fields (ThermoAcoustic1D with stepping 1 and 3,
  SynchronizedFields with boundary and material couplings), oracle/scenarios.py
  ``coupled_scenario``; inputs stored per field.
- nonlinear_1d.npz: IdealGas1D (convective or not, nonlinear or linear state
  equation) and Acoustic2ndOrder1D scenarios, oracle/scenarios.py
  ``nonlinear_scenario``.
"""
import argparse
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import ref_build, scenarios  # noqa: E402
from oracle.fds_oracle import components_of  # noqa: E402
from pyfds_gb300 import workloads  # noqa: E402
sys.path.insert(0, os.path.dirname(HERE))
from golden_digest import spec_digest  # noqa: E402
from golden_inputs import pack_inputs  # noqa: E402

RANDOM_CASES = []
for _seed in range(36):
    _kind = scenarios.ALL_KINDS[_seed % 6]
    if _kind.endswith("1D"):
        _nx, _ny = [5, 17, 33, 9, 64, 3][(_seed // 6) % 6], None
    else:
        _nx, _ny = [5, 7, 3, 11, 2, 9][_seed % 6], [4, 6, 9, 3, 5, 8][(_seed // 6) % 6]
    RANDOM_CASES.append({"seed": _seed, "kind": _kind, "nx": _nx, "ny": _ny, "steps": 30,
                         "mu": _seed % 3 != 0})


FLOW_CASES = [{"seed": 200 + k, "nx": nx, "ny": ny, "steps": 45, "flow": fl, "mu": mu}
              for k, (nx, ny, fl, mu) in enumerate([(9, 7, "rows", True), (16, 5, "rows", False),
                                                    (7, 11, "scalar", True), (33, 4, "rows", True),
                                                    (5, 9, "scalar", False), (12, 12, "rows", False),
                                                    (64, 3, "rows", True)])]


NL_CASES = [{"seed": 400 + k, "kind": kind, "nx": nx, "steps": 120, "convective": conv,
             "nl_state": nls, "mu": mu}
            for k, (kind, nx, conv, nls, mu) in enumerate([
                ("IdealGas1D", 40, True, True, True), ("IdealGas1D", 97, False, True, True),
                ("IdealGas1D", 64, True, False, False), ("IdealGas1D", 1500, True, True, True),
                ("Acoustic2ndOrder1D", 50, True, True, True),
                ("Acoustic2ndOrder1D", 1200, True, True, False)])]


def run_and_pack(spec, prefix, out, keep_state=True, steps=None, materials=False):
    pack_inputs(spec, out, prefix, materials=materials)
    state, sig = ref_build.run_reference(spec, steps or spec["steps"])
    for c in components_of(spec["kind"]):
        if keep_state:
            out[prefix + c + "/state"] = state[c]
        out[prefix + c + "/state_norm"] = np.array([np.linalg.norm(state[c]),
                                                    np.sum(state[c])])
        for j, s in enumerate(sig[c]):
            out[prefix + c + "/sig%d" % j] = s


def make_operators():
    pyfds = __import__("oracle.ref_loader", fromlist=["x"]).load_reference()
    out = {}
    rng = np.random.default_rng(11)
    for kind, names in (
            ("Acoustic1D", ["a_p_v", "a_v_p", "a_v_v"]),
            ("Acoustic2D", ["a_p_vx", "a_p_vy", "a_vx_p", "a_vy_p", "a_vx_vx"]),
            ("Acoustic3DAxi", ["a_p_vx", "a_p_vy", "a_vx_p", "a_vy_p", "a_vx_vx"]),
            ("Thermal1D", ["a_t_q", "a_q_t"]),
            ("Thermal2D", ["a_t_qx", "a_t_qy", "a_qx_t", "a_qy_t"]),
            ("Thermal3DAxi", ["a_t_qx", "a_t_qy", "a_qx_t", "a_qy_t"])):
        nx, ny = (7, None) if kind.endswith("1D") else (4, 3)
        spec = scenarios.random_scenario(int(rng.integers(1 << 30)), kind, nx, ny, steps=1,
                                         mu=True)
        fld = ref_build.build_reference_field(spec)
        fld.assemble_matrices()
        out[kind + "/spec_digest"] = np.array(spec_digest(spec))
        out[kind + "/seed_spec"] = np.array(json.dumps({"nx": nx, "ny": ny}))
        for nm in names:
            out[kind + "/" + nm] = getattr(fld, nm).toarray()
        # keep the spec's materials so the test can rebuild the same field
        out[kind + "/materials"] = np.array(json.dumps(
            [(None if i is None else list(map(int, i)), p) for i, p in spec["materials"]]))
        out[kind + "/grid"] = np.array([spec["nx"], spec.get("ny", 1), spec["dx"],
                                        spec.get("dy", spec["dx"]), spec["dt"]])
    np.savez_compressed(os.path.join(HERE, "operators.npz"), **out)


def make_random():
    out = {}
    for case in RANDOM_CASES:
        spec = scenarios.random_scenario(case["seed"], case["kind"], case["nx"], case["ny"],
                                         steps=case["steps"], mu=case["mu"])
        prefix = "s%d/" % case["seed"]
        out[prefix + "digest"] = np.array(spec_digest(spec))
        run_and_pack(spec, prefix, out, materials=True)
    out["cases"] = np.array(json.dumps(RANDOM_CASES))
    np.savez_compressed(os.path.join(HERE, "random_scenarios.npz"), **out)


def make_flow():
    import warnings
    out = {}
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")  # the reference warns about high flow velocities
        for case in FLOW_CASES:
            spec = scenarios.flow_scenario(case["seed"], case["nx"], case["ny"],
                                           steps=case["steps"], flow=case["flow"], mu=case["mu"])
            prefix = "f%d/" % case["seed"]
            out[prefix + "digest"] = np.array(spec_digest(spec))
            run_and_pack(spec, prefix, out, materials=True)
    out["cases"] = np.array(json.dumps(FLOW_CASES))
    np.savez_compressed(os.path.join(HERE, "acoustic_flow.npz"), **out)


def make_nonlinear():
    out = {}
    for case in NL_CASES:
        spec = scenarios.nonlinear_scenario(case["seed"], case["kind"], case["nx"],
                                            steps=case["steps"], convective=case["convective"],
                                            nl_state=case["nl_state"], mu=case["mu"])
        prefix = "n%d/" % case["seed"]
        out[prefix + "digest"] = np.array(spec_digest(spec))
        run_and_pack(spec, prefix, out, materials=True)
    out["cases"] = np.array(json.dumps(NL_CASES))
    np.savez_compressed(os.path.join(HERE, "nonlinear_1d.npz"), **out)


CPL_CASES = [{"seed": 500 + k, "variant": v, "nx": nx, "steps": 60}
             for k, (v, nx) in enumerate([("thermoacoustic", 30), ("thermoacoustic3", 41),
                                          ("sync", 30), ("sync_exp", 25)])]


def make_coupling():
    from oracle.ref_loader import load_reference
    ref = load_reference()
    import pyfds.regions
    ref.regions = pyfds.regions
    out = {}
    for case in CPL_CASES:
        spec = scenarios.coupled_scenario(case["seed"], case["variant"], case["nx"],
                                          case["steps"])
        prefix = "c%d/" % case["seed"]
        out[prefix + "digest"] = np.array(spec_digest(spec))
        if spec["kind"] == "ThermoAcoustic1D":
            pack_inputs(spec, out, prefix)
        else:
            for k, f in enumerate(spec["fields"]):
                pack_inputs(f, out, prefix + "f%d/" % k)
        obj = scenarios.build_coupled(ref, spec, ref_build.build_reference_field)
        obj.simulate(spec["steps"])
        for k, (st, sig) in enumerate(scenarios.coupled_results(obj, lambda f: type(f).__name__)):
            for c in st:
                out[prefix + "f%d/%s/state" % (k, c)] = st[c]
                for j, x in enumerate(sig[c]):
                    out[prefix + "f%d/%s/sig%d" % (k, c, j)] = x
    out["cases"] = np.array(json.dumps(CPL_CASES))
    np.savez_compressed(os.path.join(HERE, "coupling.npz"), **out)


def make_workload(name, spec, keep_state, steps=None):
    t0 = time.time()
    out = {"digest": np.array(spec_digest(spec))}
    run_and_pack(spec, "", out, keep_state=keep_state, steps=steps)
    np.savez_compressed(os.path.join(HERE, name), **out)
    print("%s: %.1f s" % (name, time.time() - t0), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--skip-large", action="store_true")
    ap.add_argument("--only", default=None)
    a = ap.parse_args()
    jobs = {
        "operators": make_operators,
        "random": make_random,
        "flow": make_flow,
        "nonlinear": make_nonlinear,
        "coupling": make_coupling,
        "acoustic1d": lambda: make_workload("acoustic1d_water.npz",
                                            workloads.acoustic1d_water(), True),
        "axi_small": lambda: make_workload(
            "axi_disc_256x1024.npz", workloads.axi_disc_source(256, 1024, 500, disc=50,
                                                               probe_every=32), False),
        "thermal_small": lambda: make_workload(
            "thermal2d_512.npz", workloads.thermal2d_two_materials(512, 500, 64), False),
    }
    large = {
        "axi_prefix": lambda: make_workload("axi_disc_full_prefix.npz",
                                            workloads.axi_disc_source(), False, steps=100),
        "thermal_prefix": lambda: make_workload(
            "thermal2d_4096_prefix.npz", workloads.thermal2d_two_materials(), False, steps=100),
        "axi_1000": lambda: make_workload("axi_disc_full_1000.npz",
                                          workloads.axi_disc_source(), False, steps=1000),
        "thermal_1000": lambda: make_workload(
            "thermal2d_4096_1000.npz", workloads.thermal2d_two_materials(), False, steps=1000),
        "acoustic2d": lambda: make_workload("acoustic2d_steel_2048.npz",
                                            workloads.acoustic2d_steel_block(), False),
    }
    if not a.skip_large:
        jobs.update(large)
    for name, fn in jobs.items():
        if a.only and name not in a.only.split(","):
            continue
        t0 = time.time()
        fn()
        print("done", name, "%.1f s" % (time.time() - t0), flush=True)


if __name__ == "__main__":
    main()
