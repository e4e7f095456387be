"""The C++ mirror of AMIE's Assembly (xfem-amie_gb300/host/gpu_assembly.*),
compiled against the C-ABI and driven element by element like FeatureTree
drives the reference: pattern bit-exact, matrix and rhs to 1e-12, and with
ConjugateGradient semantics the reference's iteration count (+-3) and
displacements to 1e-9."""
import os
import subprocess

import numpy as np
import pytest

from conftest import REPO, load_golden

import amie_mesh

pytestmark = pytest.mark.gpu


def _write_case(d, path):
    os.makedirs(path, exist_ok=True)
    dim = int(d["dim"][0])
    keep = d["bc_types"] != amie_mesh.LM_PROPORTIONAL
    pids, poffs, pptr, pdofs, pcoefs = amie_mesh.golden_proportional(d)
    assert (np.diff(pptr) == 1).all()
    arrays = {"kind": d["elem_kind"].astype(np.uint8), "dof_ptr": d["elem_dof_ptr"].astype(np.uint32),
              "dof_ids": d["elem_dof_ids"].astype(np.uint32), "gp_ptr": d["gp_ptr"].astype(np.uint32),
              "gp": d["gp"], "jinv": d["jinv"], "cmat": d["cmat"], "bc_ids": d["bc_ids"][keep].astype(np.uint32),
              "bc_vals": d["bc_values"][keep],
              "meta": np.array([dim, d["ndofmax"][0], d["epsilon"][0], d["nssor"][0]], np.float64)}
    if len(pids):
        arrays.update(prop_ids=pids, prop_dofs=pdofs, prop_offsets=poffs, prop_coefs=pcoefs)
    for k, v in arrays.items():
        np.ascontiguousarray(v).tofile(os.path.join(path, k + ".bin"))


@pytest.mark.parametrize("name", ["incl_p1", "voxel_t4", "prop_p1"])
def test_cpp_assembly_matches_reference(tmp_path, name):
    import build as gpu_build
    exe = gpu_build.build_cpp_test()
    d = load_golden(name)
    if "elem_moved" in d and d["elem_moved"].any():
        pytest.skip("case has moved elements")
    case = str(tmp_path / name)
    _write_case(d, case)
    r = subprocess.run([exe, case, "2"], capture_output=True, text=True, timeout=300,
                       env=dict(os.environ, LD_LIBRARY_PATH=os.path.join(REPO, "xfem-amie_gb300")))
    assert r.returncode == 0, r.stderr
    u = np.fromfile(os.path.join(case, "u.bin"))
    rs = np.fromfile(os.path.join(case, "row_size.bin"), np.uint32)
    ci = np.fromfile(os.path.join(case, "column_index.bin"), np.uint32)
    arr = np.fromfile(os.path.join(case, "array.bin"))
    rhs = np.fromfile(os.path.join(case, "rhs.bin"))
    assert np.array_equal(rs, d["row_size"]) and np.array_equal(ci, d["column_index"])
    assert np.abs(arr - d["array"]).max() <= 1e-12 * np.abs(d["array"]).max()
    assert np.abs(rhs - d["rhs"]).max() <= 1e-12 * np.abs(d["rhs"]).max()
    # prop_p1: the reference's displacements after its post-solve substitution of
    # the proportional DOFs (Assembly::cgsolve, solvers/assembly.cpp:1881-1892)
    ref = d["u_post"] if "u_post" in d else d["u"]
    tol = {"voxel_t4": 1e-6, "prop_p1": 1e-8}.get(name, 1e-9)
    assert np.abs(u - ref).max() <= tol * np.abs(ref).max()
