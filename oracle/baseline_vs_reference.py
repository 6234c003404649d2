"""Time one step of the unmodified reference against the CPU-baseline worker, one
process each, on the same workload (validation of the CPU baseline; run where the
reference source tree is available):

    python oracle/baseline_vs_reference.py [workload builder] [steps]

The reference is imported from its source tree through ``oracle/ref_loader.py``;
the worker is ``oracle/bench_worker.py`` (scipy DIA products from the oracle's
diagonals, in-place updates). Prints seconds per step and Gcell/s for both.
"""
import os
import sys
import time

os.environ.setdefault("OMP_NUM_THREADS", "1")
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def main():
    from oracle import bench_worker, ref_build
    from oracle.ref_loader import load_reference
    from pyfds_gb300 import workloads
    builder = sys.argv[1] if len(sys.argv) > 1 else "acoustic2d_steel_block"
    steps = int(sys.argv[2]) if len(sys.argv) > 2 else 10
    load_reference()
    fld = ref_build.build_reference_field(getattr(workloads, builder)())
    fld.simulate(1)
    t0 = time.perf_counter()
    fld.simulate(steps)
    t_ref = (time.perf_counter() - t0) / steps
    bench_worker.setup(builder, {})
    bench_worker.run(1)
    t_w = bench_worker.run(steps) / steps
    cells = bench_worker.cells()
    print("%s, %d steps, one process each: reference %.3f s/step (%.4f Gcell/s), "
          "worker %.3f s/step (%.4f Gcell/s)"
          % (builder, steps, t_ref, cells / t_ref / 1e9, t_w, cells / t_w / 1e9))


if __name__ == "__main__":
    main()
