"""Anchor the CPU port's solver speed to the reference's own.

Runs the reference harness (oracle/_ref/ref_harness, built by `make -C oracle
ref`) on a cfg0-size square with inclusions, which times the reference's
ConjugateGradient::solve as Assembly::cgsolve drives it, then times the port's
restatement of the same solver (oracle_cg_amie) and its relative-residual PCG
on the matrix the harness exported, with the same OpenMP thread count.

Needs the reference tree (development container only):

    OMP_NUM_THREADS=8 python oracle/anchor_reference.py
"""
import os
import subprocess
import sys
import tempfile
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "tests", "golden"))

import numpy as np  # noqa: E402

import oracle as O  # noqa: E402
from make_golden import read_records  # noqa: E402


def main() -> int:
    harness = os.path.join(HERE, "_ref", "ref_harness")
    if not os.path.exists(harness):
        print("build the harness first: make -C oracle ref", file=sys.stderr)
        return 2
    out = os.path.join(tempfile.gettempdir(), "anchor_reference.bin")
    r = subprocess.run([harness, "incl", out, "sampling=64", "ninc=300", "seed=2024", "order=1", "size=0.04"],
                       capture_output=True, text=True, errors="replace")
    if r.returncode != 0:
        print(r.stderr[-2000:], file=sys.stderr)
        return r.returncode
    d = read_records(out)
    rs, ci, arr, b = d["row_size"], d["column_index"], d["array"], d["rhs"]
    n = len(b)
    ref_it, ref_s = int(d["cg_iterations"][0]), float(d["time_cg_s"][0])
    t0 = time.perf_counter()
    x, it, _ = O.cg_amie(2, rs, ci, arr, b, eps=float(d["epsilon"][0]), nssor=int(d["nssor"][0]))
    t1 = time.perf_counter()
    err = np.abs(x - d["u"]).max() / np.abs(d["u"]).max()
    print(f"threads {O.threads()}, n {n}, blocks {len(ci)}")
    print(f"reference ConjugateGradient::solve: {ref_it} iterations {ref_s:.3f} s {n * ref_it / ref_s:.3e} DOF-it/s")
    print(f"port, same algorithm:              {it} iterations {t1 - t0:.3f} s {n * it / (t1 - t0):.3e} DOF-it/s "
          f"(solution difference {err:.1e})")
    t0 = time.perf_counter()
    _, it2, _, _ = O.pcg(2, rs, ci, arr, b, rtol=1e-10)
    t1 = time.perf_counter()
    print(f"port PCG to 1e-10:                 {it2} iterations {t1 - t0:.3f} s {n * it2 / (t1 - t0):.3e} DOF-it/s")
    os.remove(out)
    return 0


if __name__ == "__main__":
    sys.exit(main())
