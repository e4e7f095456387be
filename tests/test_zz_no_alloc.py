"""amie_pcg_solve_noalloc: the Jacobi-PCG entry point that allocates no device memory.

Some callers cannot allocate device memory when they solve: a code path that
runs while a CUDA graph is captured in a mode that forbids cudaMalloc, an
application that gave all device memory to its own pool allocator at start-up,
or a real-time loop that cannot absorb the device-wide synchronisation an
allocation may trigger.  They keep the matrix, right-hand side and solution in
their own device buffers (allocated here with torch, standing in for the
caller's pool) and the library works in a fixed static device array.

The test calls the entry point through the C-ABI twice in a row on the same
system and compares each answer with the existing entry point (amie_solve,
FP64 PCG, same relative-residual target) to the 1e-9 relative tolerance the
other FP64 solve tests use; it also checks the size limit is reported.  This
file is collected last so a failure here comes after every other test ran.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import load_golden

import amie_mesh as am

pytestmark = pytest.mark.gpu


def _bsr_from_golden(d):
    s = int(d["stride"][0])
    cl = s + s % 2
    rs = d["row_size"].astype(np.int64)
    row_ptr = np.concatenate([[0], np.cumsum(rs)]).astype(np.uint32)
    nnzb = len(d["column_index"])
    blocks = d["array"].reshape(nnzb, s, cl)[:, :, :s]      # [block][column][row] (AMIE layout)
    val = np.ascontiguousarray(blocks.transpose(0, 2, 1)).reshape(-1)   # row-major s x s
    return s, len(rs), row_ptr, d["column_index"].astype(np.uint32), val, d["rhs"].astype(np.float64)


def _noalloc(lib, s, n_rows, dev, use_x0=0):
    import amie_gpu
    st = amie_gpu.SolveStats()
    ptr = lambda t: C.c_void_p(t.data_ptr())   # noqa: E731
    rc = lib.amie_pcg_solve_noalloc(C.c_int32(s), C.c_uint32(n_rows), ptr(dev["row_ptr"]), ptr(dev["col"]),
                                    ptr(dev["val"]), ptr(dev["b"]), ptr(dev["x"]), C.c_double(1e-10),
                                    C.c_int64(0), C.c_int32(use_x0), None, C.byref(st))
    return rc, st


@pytest.mark.parametrize("name", ["incl_p1", "voxel_t4"])
def test_noalloc_matches_existing_solver_twice(gpu_ctx, name):
    torch = pytest.importorskip("torch")
    import amie_gpu
    lib = amie_gpu.lib()
    d = load_golden(name)
    s, n_rows, row_ptr, col, val, b = _bsr_from_golden(d)

    # the existing entry point on the same system
    m = am.from_golden(d, "tabulated")
    topo = amie_gpu.Topology(gpu_ctx, m)
    topo.assemble()
    topo.apply_dirichlet(*am.golden_bcs(d))
    x_ref, st_ref = topo.solve(amie_gpu.SOLVER_PCG_FP64, rtol=1e-10)
    topo.close()
    assert st_ref["relres"] <= 1e-10

    dev = {
        "row_ptr": torch.from_numpy(row_ptr.view(np.int32)).cuda(),
        "col": torch.from_numpy(col.view(np.int32)).cuda(),
        "val": torch.from_numpy(val).cuda(),
        "b": torch.from_numpy(b).cuda(),
        "x": torch.full((n_rows * s,), 7.0, dtype=torch.float64, device="cuda"),   # overwritten (use_x0 = 0)
    }
    torch.cuda.synchronize()
    for call in range(2):
        rc, st = _noalloc(lib, s, n_rows, dev)
        torch.cuda.synchronize()
        assert rc == amie_gpu.AMIE_OK, (call, rc, lib.amie_last_error())
        assert st.relres <= 1e-10 and st.iterations > 0
        x = dev["x"].cpu().numpy()
        assert np.abs(x - x_ref).max() <= 1e-9 * np.abs(x_ref).max(), call
        dev["x"].fill_(-3.0)


def test_noalloc_rejects_oversized_systems():
    torch = pytest.importorskip("torch")
    import amie_gpu
    lib = amie_gpu.lib()
    dummy = torch.zeros(8, dtype=torch.float64, device="cuda")
    p = C.c_void_p(dummy.data_ptr())
    st = amie_gpu.SolveStats()
    rc = lib.amie_pcg_solve_noalloc(C.c_int32(2), C.c_uint32(200000), p, p, p, p, p, C.c_double(1e-10),
                                    C.c_int64(0), C.c_int32(0), None, C.byref(st))
    assert rc == amie_gpu.AMIE_BAD_INPUT
    assert b"262144" in lib.amie_last_error()
