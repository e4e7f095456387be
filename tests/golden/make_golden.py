"""Generate the golden fixtures of this directory from the AMIE reference itself.

Runs ``oracle/_ref/ref_harness`` (built by ``make -C oracle ref`` from the
reference sources) on a handful of small problems and stores every array it
exports as a compressed ``.npz`` next to this script.  The fixtures pin the
CPU oracle (``oracle/amie_oracle.cpp``) and the GPU path to the reference's
own element matrices, sparsity pattern, Dirichlet elimination and CG solution.

This script needs the reference tree and runs in the development container
only; the committed ``.npz`` files are what the tests read.

    python tests/golden/make_golden.py [--only NAME]
"""
from __future__ import annotations

import argparse
import os
import re
import struct
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
HARNESS = os.path.join(REPO, "oracle", "_ref", "ref_harness")

# name -> (harness case, key=value arguments)
CASES = {
    # config-0 style: 2D plane stress P1, matrix 30 GPa + 60 GPa inclusions
    "incl_p1": ("incl", ["sampling=12", "ninc=30", "seed=7", "order=1"]),
    # same microstructure family on quadratic (P2) triangles
    "incl_p2": ("incl", ["sampling=8", "ninc=20", "seed=11", "order=2", "E=25e9"]),
    # straight Heaviside-enriched crack of length 0.3*width, P1 and P2
    "crack_p1": ("crack", ["sampling=16", "order=1", "E=25e9"]),
    "crack_p2": ("crack", ["sampling=10", "order=2", "E=25e9"]),
    # known-answer test of examples/test/test_stiffness.ini: 10 mm plate, 1 MPa imposed
    # stress on TOP (force multipliers), E = 10 GPa -> strain_yy = 1e-4 everywhere
    "plate": ("plate", ["size=0.01", "E=10e9", "nu=0.2", "sampling=4"]),
    # known-answer test of examples/test/test_stiffness_with_imposed_deformation.ini: the
    # same plate, free on rollers, imposed strain 1e-3 (induced force multipliers)
    # -> strain_yy = 1e-3, real stress 0
    "imposed": ("imposed", ["size=0.01", "E=10e9", "nu=0.2", "sampling=4", "imposed=1e-3"]),
    # incl_p1 with an inclined roller on RIGHT (SET_PROPORTIONAL_DISPLACEMENT_XI_ETA,
    # u_x = 0.5 u_y: Assembly::setPointProportional multipliers)
    "prop_p1": ("incl", ["sampling=12", "ninc=30", "seed=7", "order=1", "prop=0.5"]),
    # config-2 style: voxel file -> 6 linear tets per voxel, 16 lognormal phases,
    # uniaxial imposed strain 1e-4
    "voxel_t4": ("voxel", ["n=6", "nphase=16", "seed=5", "strain=1e-4"]),
    # config-3 style: 80 x 20 mm notched beam in three-point bending, P1,
    # StiffnessAndFracture + NonLocalMazars (eps0 1e-4, Gf 100 N/m, radius 2 mm)
    # + FiberBasedIsotropicLinearDamage; six load steps up to 40 um deflection
    "damage_p1": ("damage", ["sampling=16", "steps=6", "deflection=4e-5"]),
}

_TYPES = {"d": np.float64, "i": np.int32, "u": np.uint32, "q": np.int64, "b": np.int8}


def read_records(path: str) -> dict:
    out = {}
    with open(path, "rb") as f:
        data = f.read()
    pos = 0
    while pos < len(data):
        (n,) = struct.unpack_from("<I", data, pos)
        pos += 4
        name = data[pos:pos + n].decode()
        pos += n
        t = chr(data[pos])
        pos += 1
        (count,) = struct.unpack_from("<Q", data, pos)
        pos += 8
        dt = np.dtype(_TYPES[t])
        out[name] = np.frombuffer(data, dtype=dt, count=count, offset=pos).copy()
        pos += count * dt.itemsize
    return out


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--only", default=None)
    args = ap.parse_args()
    if not os.path.exists(HARNESS):
        print("build the harness first: make -C oracle ref", file=sys.stderr)
        return 2
    for name, (case, kv) in CASES.items():
        if args.only and name != args.only:
            continue
        tmp = os.path.join("/tmp", f"golden_{name}.bin")
        env = dict(os.environ, OMP_NUM_THREADS="1")
        r = subprocess.run([HARNESS, case, tmp] + kv, capture_output=True, text=True, env=env,
                           errors="replace")
        if r.returncode != 0:
            print(r.stderr[-2000:], file=sys.stderr)
            return r.returncode
        rec = read_records(tmp)
        if case == "damage":
            # passes of FeatureTree::stepInternal per load step, as the reference prints them
            # ("<passes>/<maxit>." before the step line of the harness)
            log = r.stderr.replace("\r", "\n")
            rec["sub_iterations"] = np.array([int(p) for p, _ in re.findall(r"(\d+)/\d+\.harness damage: step (\d+)", log)],
                                             np.int32)
        rec["harness_case"] = np.array(case)
        rec["harness_args"] = np.array(" ".join(kv))
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **rec)
        line = [l for l in r.stderr.replace("\r", "\n").splitlines() if "harness" in l]
        print(name, line[-1] if line else "")
        os.remove(tmp)
    return 0


if __name__ == "__main__":
    sys.exit(main())
