"""amie_pcg_solve_noalloc: the Jacobi-PCG entry point that allocates no device memory.

Some callers cannot allocate device memory when they solve: an application
that gave all device memory to its own pool allocator at start-up, or a
real-time loop that cannot absorb the device-wide synchronisation an
allocation may trigger.  They keep the matrix, right-hand side and solution in
their own device buffers (allocated here with torch, standing in for the
caller's pool) and the library works in a fixed static device array.

The test calls the entry point through the C-ABI twice in a row on the same
system and compares each answer with the existing entry point (amie_solve,
FP64 PCG, same relative-residual target) to the 1e-9 relative tolerance the
other FP64 solve tests use; it also checks the size limit is reported, and
the remaining branches: a warm start, a zero right-hand side, a side stream,
an iteration cap, and rows whose columns are not sorted.  This
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


def _noalloc(lib, s, n_rows, dev, use_x0=0, maxit=0, stream=None, b=None):
    import amie_gpu
    st = amie_gpu.SolveStats()
    ptr = lambda t: C.c_void_p(t.data_ptr())   # noqa: E731
    sp = C.c_void_p(stream.cuda_stream) if stream is not None else None
    rc = lib.amie_pcg_solve_noalloc(C.c_int32(s), C.c_uint32(n_rows), ptr(dev["row_ptr"]), ptr(dev["col"]),
                                    ptr(dev["val"]), ptr(dev["b"] if b is None else b), ptr(dev["x"]),
                                    C.c_double(1e-10), C.c_int64(maxit), C.c_int32(use_x0), sp, C.byref(st))
    return rc, st


def _system(gpu_ctx, name):
    """The golden system on the device (caller-owned buffers) and the existing entry point's solution."""
    torch = pytest.importorskip("torch")
    import amie_gpu
    d = load_golden(name)
    s, n_rows, row_ptr, col, val, b = _bsr_from_golden(d)
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
        "x": torch.zeros(n_rows * s, dtype=torch.float64, device="cuda"),
    }
    torch.cuda.synchronize()
    return s, n_rows, (row_ptr, col, val, b), dev, x_ref, st_ref


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


def test_noalloc_branches(gpu_ctx):
    """Warm start, zero right-hand side, side stream and iteration cap, each checked against amie_solve."""
    torch = pytest.importorskip("torch")
    import amie_gpu
    lib = amie_gpu.lib()
    s, n_rows, _, dev, x_ref, st_ref = _system(gpu_ctx, "incl_p1")
    scale = np.abs(x_ref).max()

    # warm start from the answer plus a small perturbation: few iterations, same answer
    rng = np.random.default_rng(5)
    x0 = x_ref * (1.0 + 1e-6 * rng.standard_normal(len(x_ref)))
    dev["x"].copy_(torch.from_numpy(x0))
    rc, st = _noalloc(lib, s, n_rows, dev, use_x0=1)
    torch.cuda.synchronize()
    assert rc == amie_gpu.AMIE_OK, lib.amie_last_error()
    assert 0 < st.iterations < st_ref["iterations"], (st.iterations, st_ref["iterations"])
    assert np.abs(dev["x"].cpu().numpy() - x_ref).max() <= 1e-9 * scale

    # zero right-hand side: x = 0 whatever it held, relative residual 0, no iteration
    zero = torch.zeros_like(dev["b"])
    dev["x"].fill_(5.0)
    rc, st = _noalloc(lib, s, n_rows, dev, b=zero)
    torch.cuda.synchronize()
    assert rc == amie_gpu.AMIE_OK and st.relres == 0.0 and st.iterations == 0
    assert not dev["x"].any().item()

    # a side stream: the same answer, in the caller's stream order
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):
        dev["x"].fill_(-1.0)
        rc, st = _noalloc(lib, s, n_rows, dev, stream=side)
        x_side = dev["x"].clone()
    side.synchronize()
    assert rc == amie_gpu.AMIE_OK, lib.amie_last_error()
    assert np.abs(x_side.cpu().numpy() - x_ref).max() <= 1e-9 * scale

    # an iteration cap below what the solve needs
    rc, st = _noalloc(lib, s, n_rows, dev, maxit=20)
    torch.cuda.synchronize()
    assert rc == amie_gpu.AMIE_NOT_CONVERGED, rc
    assert 0 < st.iterations <= 20 and st.relres > 1e-10


def test_noalloc_unsorted_columns(gpu_ctx):
    """Rows whose blocks are stored in reverse column order give the same answer."""
    torch = pytest.importorskip("torch")
    import amie_gpu
    lib = amie_gpu.lib()
    s, n_rows, (row_ptr, col, val, b), dev, x_ref, _ = _system(gpu_ctx, "voxel_t4")
    rp = row_ptr.astype(np.int64)
    perm = np.concatenate([np.arange(rp[k + 1] - 1, rp[k] - 1, -1) for k in range(n_rows)])
    assert len(perm) == len(col) and np.array_equal(np.sort(perm), np.arange(len(col)))
    col_r = np.ascontiguousarray(col[perm])
    val_r = np.ascontiguousarray(val.reshape(-1, s * s)[perm]).reshape(-1)
    dev["col"] = torch.from_numpy(col_r.view(np.int32)).cuda()
    dev["val"] = torch.from_numpy(val_r).cuda()
    torch.cuda.synchronize()
    rc, st = _noalloc(lib, s, n_rows, dev)
    torch.cuda.synchronize()
    assert rc == amie_gpu.AMIE_OK, lib.amie_last_error()
    assert np.abs(dev["x"].cpu().numpy() - x_ref).max() <= 1e-9 * np.abs(x_ref).max()
