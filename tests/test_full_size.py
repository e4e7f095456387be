"""Parity at the benchmark sizes (cfg0 44 k, cfg1 1.2 M, cfg2 824 k DOF) against
the oracle on the same seeded workloads: the sparsity pattern bit for bit, the
assembled and eliminated matrix and right-hand side to 1e-12, both solvers'
true relative residual ||b - A x|| / ||b|| computed by the oracle's own SpMV on
the oracle's matrix, and the node displacements of both solvers at rtol 1e-10
against a 1e-13 FP64 solution: FP64 within 1e-9, mixed within 1e-8 (relative
to the largest node displacement).

The 1e-13 solution is the oracle's own Jacobi-PCG on cfg0 and cfg2.  On cfg1
(1.2 M DOF, ~15 k iterations) the CPU solve is too slow for a test, so it is
the GPU FP64 solve at 1e-13, whose true residual is re-computed by the oracle's
SpMV on the oracle's matrix."""
import os
import sys

import numpy as np
import pytest

import oracle as O

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-9     # plain FP64 path vs the 1e-13 solution
MIXED_TOL = 1e-8    # FP32 inner / FP64 refinement vs the 1e-13 solution


def rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


@pytest.mark.parametrize("cfg", ["cfg0", "cfg1", "cfg2"])
def test_full_size_parity(gpu_ctx, cfg):
    import amie_gpu
    import bench
    m, bcs, meta, name = bench.make_workload(cfg)
    ids, vals, kinds = bcs
    R = O.assemble(m, ids, vals, kinds)
    t = amie_gpu.Topology(gpu_ctx, m)
    try:
        rs, ci = t.pattern()
        assert np.array_equal(rs, R["row_size"]) and np.array_equal(ci, R["column_index"])
        t.assemble()
        t.apply_dirichlet(ids, vals, kinds)
        arr, rhs = t.matrix()
        assert rel(arr, R["array"]) <= 1e-12 and rel(rhs, R["rhs"]) <= 1e-12
        b = R["rhs"]
        nb = np.linalg.norm(b)

        def relres(x):
            return np.linalg.norm(b - O.spmv(m.stride, R["row_size"], R["column_index"], R["array"], x)) / nb

        s = slice(0, meta["n_nodes"] * m.stride)
        if cfg == "cfg1":
            x_tight, _ = t.solve(amie_gpu.SOLVER_PCG_FP64, rtol=1e-13)
        else:
            x_tight, _, _, rc = O.pcg(m.stride, R["row_size"], R["column_index"], R["array"], b, rtol=1e-13)
            assert rc == 0
        assert relres(x_tight) <= 2e-13
        for solver, tol in ((amie_gpu.SOLVER_PCG_FP64, FP64_TOL), (amie_gpu.SOLVER_PCG_MIXED, MIXED_TOL)):
            x, st = t.solve(solver, rtol=1e-10)
            assert relres(x) <= 1.05e-10, (solver, st)
            err = rel(x[s], x_tight[s])
            assert err <= tol, (solver, err, st)
    finally:
        t.close()
