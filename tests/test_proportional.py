"""Proportional displacement multipliers (Assembly::setPointProportional,
solvers/assembly.cpp:1636-1760; SET_PROPORTIONAL_DISPLACEMENT), pinned to the
reference's prop_p1 fixture: the incl_p1 plate with an inclined roller on its
right face (SET_PROPORTIONAL_DISPLACEMENT_XI_ETA, u_x = 0.5 u_y,
features/boundarycondition.cpp:256-259), exported after make_final with the
multipliers' DOFs and coefficients and the displacements Assembly::cgsolve
reports (the constrained DOFs set from theirs after the solve).

CPU: the oracle's elimination of the displacement multipliers followed by the
restated substitution (oracle.proportional) gives the reference's matrix and
right-hand side, and its solve plus the post-solve step the reference's
displacements.  GPU: the same through amie_set_proportional.
"""
import numpy as np
import pytest

from conftest import load_golden

import amie_mesh as am
import oracle as O


def rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def test_oracle_proportional_matches_reference():
    d = load_golden("prop_p1")
    m = am.from_golden(d, "auto")
    props = am.golden_proportional(d)
    assert len(props[0]) == 26 and np.all(props[4] == 0.5)
    R = O.assemble(m, *am.golden_bcs(d))
    arr, rhs = R["array"].copy(), R["rhs"].copy()
    O.proportional(2, R["row_size"], R["column_index"], arr, rhs, *props)
    assert np.array_equal(R["column_index"], d["column_index"])
    assert rel(arr, d["array"]) <= 1e-15
    assert rel(rhs, d["rhs"]) <= 1e-15
    x, _, _, rc = O.pcg(2, R["row_size"], R["column_index"], arr, rhs, rtol=1e-13)
    assert rc == 0
    O.proportional_solution(x, *props)
    assert rel(x, d["u_post"]) <= 1e-8
    ids, _, ptr, pids, coefs = props
    assert np.abs(x[ids] - 0.5 * x[pids]).max() <= 1e-15 * np.abs(x).max()


@pytest.mark.gpu
@pytest.mark.parametrize("solver", ["fp64", "mixed"])
def test_device_proportional(gpu_ctx, solver):
    import amie_gpu as G
    d = load_golden("prop_p1")
    m = am.from_golden(d, "auto")
    props = am.golden_proportional(d)
    t = G.Topology(gpu_ctx, m)
    try:
        t.assemble()
        t.set_proportional(*props)   # before the elimination
        t.apply_dirichlet(*am.golden_bcs(d))
        arr, rhs = t.matrix()
        assert rel(arr, d["array"]) <= 1e-12
        assert rel(rhs, d["rhs"]) <= 1e-12
        sv = G.SOLVER_PCG_FP64 if solver == "fp64" else G.SOLVER_PCG_MIXED
        x, st = t.solve(sv, rtol=1e-12 if solver == "fp64" else 1e-10)
        assert rel(x, d["u_post"]) <= (1e-8 if solver == "fp64" else 1e-7)
        ids, _, _, pids, _ = props
        assert np.abs(x[ids] - 0.5 * x[pids]).max() <= 1e-15 * np.abs(x).max()
        # set after the elimination: eliminated again from the original matrix
        t2 = G.Topology(gpu_ctx, m)
        t2.assemble()
        t2.apply_dirichlet(*am.golden_bcs(d))
        t2.set_proportional(*props)
        arr2, rhs2 = t2.matrix()
        assert np.array_equal(arr2, arr) and np.array_equal(rhs2, rhs)
        # removed again: the plain Dirichlet elimination
        t2.set_proportional(np.zeros(0, np.uint32), np.zeros(0), np.zeros(1, np.uint32), np.zeros(0, np.uint32),
                            np.zeros(0))
        arr3, rhs3 = t2.matrix()
        t3 = G.Topology(gpu_ctx, m)
        t3.assemble()
        t3.apply_dirichlet(*am.golden_bcs(d))
        arr4, rhs4 = t3.matrix()
        assert np.array_equal(arr3, arr4) and np.array_equal(rhs3, rhs4)
        assert not np.array_equal(arr3, arr)
        t3.close()
        t2.close()
    finally:
        t.close()
