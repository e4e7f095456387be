"""Parity at the benchmark sizes (cfg0 44 k, cfg1 1.2 M, cfg2 824 k DOF) against
the oracle on the same seeded workloads: the sparsity pattern bit for bit, the
assembled and eliminated matrix and right-hand side to 1e-12, and both
solvers' solutions through a size-independent property, the true relative
residual ||b - A x|| / ||b|| computed by the oracle's own SpMV on the oracle's
matrix; the mixed solution also against the FP64 one (node displacements)."""
import os
import sys

import numpy as np
import pytest

import oracle as O

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)

pytestmark = pytest.mark.gpu


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
        sols = {}
        for solver in (amie_gpu.SOLVER_PCG_FP64, amie_gpu.SOLVER_PCG_MIXED):
            x, st = t.solve(solver, rtol=1e-10)
            r = b - O.spmv(m.stride, R["row_size"], R["column_index"], R["array"], x)
            assert np.linalg.norm(r) / nb <= 1.05e-10, (solver, st)
            sols[solver] = x
        s = slice(0, meta["n_nodes"] * m.stride)
        assert rel(sols[amie_gpu.SOLVER_PCG_MIXED][s], sols[amie_gpu.SOLVER_PCG_FP64][s]) <= 1e-8
    finally:
        t.close()
