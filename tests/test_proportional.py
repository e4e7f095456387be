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


@pytest.mark.gpu
def test_device_proportional_conflicts(gpu_ctx):
    """One multiplier per DOF: a proportional id given twice, or also fixed by the
    Dirichlet list (in either order), is refused and leaves the topology as it was."""
    import amie_gpu as G
    d = load_golden("prop_p1")
    m = am.from_golden(d, "auto")
    ids, offs, ptr, pids, coefs = am.golden_proportional(d)
    bc_ids, bc_vals, bc_kinds = am.golden_bcs(d)
    t = G.Topology(gpu_ctx, m)
    try:
        t.assemble()
        t.set_proportional(ids, offs, ptr, pids, coefs)
        t.apply_dirichlet(bc_ids, bc_vals, bc_kinds)
        arr, rhs = t.matrix()
        dup = np.concatenate([ids, ids[:1]])
        with pytest.raises(G.AmieError, match="BAD_INPUT"):
            t.set_proportional(dup, np.concatenate([offs, offs[:1]]), np.concatenate([ptr, ptr[-1:] + 1]),
                               np.concatenate([pids, pids[:1]]), np.concatenate([coefs, coefs[:1]]))
        fixed = np.concatenate([bc_ids, ids[:1]])
        order = np.argsort(fixed, kind="stable")
        with pytest.raises(G.AmieError, match="BAD_INPUT"):
            t.apply_dirichlet(fixed[order], np.concatenate([bc_vals, [0.0]])[order],
                              np.concatenate([bc_kinds, [am.BC_DISPLACEMENT]]).astype(np.uint8)[order])
        arr2, rhs2 = t.matrix()
        assert np.array_equal(arr2, arr) and np.array_equal(rhs2, rhs)
        # the other order: the Dirichlet list first, then a proportional multiplier on a fixed DOF
        t2 = G.Topology(gpu_ctx, m)
        t2.assemble()
        t2.apply_dirichlet(bc_ids, bc_vals, bc_kinds)
        with pytest.raises(G.AmieError, match="BAD_INPUT"):
            t2.set_proportional(bc_ids[:1], np.zeros(1), np.array([0, 1], np.uint32),
                                np.array([bc_ids[0] ^ 1], np.uint32), np.ones(1))
        t2.close()
    finally:
        t.close()


@pytest.mark.gpu
def test_assembly_mirror_proportional(gpu_ctx):
    """The Python Assembly mirror: setPointProportional gives the reference's
    post-solve displacements; moving a DOF between the displacement and the
    proportional multipliers between two solves gives what a fresh Assembly
    with the final multipliers gives."""
    import amie_gpu as G
    d = load_golden("prop_p1")
    m = am.from_golden(d, "auto")
    ids, offs, ptr, pids, coefs = am.golden_proportional(d)
    bc_ids, bc_vals, _ = am.golden_bcs(d)

    def build():
        A = G.Assembly(gpu_ctx)
        A.add(m)
        for i, v in zip(bc_ids, bc_vals):
            A.setPointAlong(int(i) % 2, float(v), int(i) // 2)
        for k, i in enumerate(ids):
            assert ptr[k + 1] - ptr[k] == 1 and pids[ptr[k]] // 2 == i // 2
            A.setPointProportional(int(i) % 2, int(pids[ptr[k]]) % 2, float(coefs[ptr[k]]), float(offs[k]),
                                   int(i) // 2)
        A.setSolver(G.SOLVER_PCG_FP64, 1e-12)
        return A

    A = build()
    assert A.cgsolve()
    assert rel(A.getDisplacements(), d["u_post"]) <= 1e-8
    # the first proportional DOF becomes fixed, the first fixed DOF of another node proportional
    moved_fixed = int(ids[0])
    free = next(int(i) for i in bc_ids if i // 2 != moved_fixed // 2)
    for B in (A, None):
        B = B or build()
        B.setPointAlong(moved_fixed % 2, 0.0, moved_fixed // 2)
        B.setPointProportional(free % 2, [(1 - free % 2, 0.25)], None, 0.0, free // 2)
        assert B.cgsolve()
        if B is A:
            u_moved = A.getDisplacements().copy()
            arr_moved = A.getMatrix()[2].copy()
        else:
            assert np.array_equal(B.getMatrix()[2], arr_moved)
            assert rel(B.getDisplacements(), u_moved) <= 1e-10
    assert abs(u_moved[moved_fixed]) <= 1e-10 * np.abs(u_moved).max()
    assert abs(u_moved[free] - 0.25 * u_moved[free ^ 1]) <= 1e-15 * np.abs(u_moved).max()


@pytest.mark.gpu
def test_device_proportional_3d_several_dofs(gpu_ctx):
    """3x3 blocks (k_proportional<3>) and multipliers on two DOFs each (the
    second setPointProportional overload, solvers/assembly.cpp:1699-1761): the
    device substitution equals the oracle's restatement applied to the device's
    own Dirichlet-eliminated matrix, and the solution meets every constraint."""
    import amie_gpu as G
    d = load_golden("voxel_t4")
    m = am.from_golden(d, "auto")
    bc_ids, bc_vals, bc_kinds = am.golden_bcs(d)
    n = len(d["rhs"])
    fixed = set(int(i) for i in bc_ids)
    free_nodes = [k for k in range(n // 3) if all(3 * k + a not in fixed for a in range(3))]
    nodes = free_nodes[:: max(1, len(free_nodes) // 12)][:12]
    assert len(nodes) >= 6
    ids = np.array([3 * k for k in nodes], np.uint32)                          # u_x of the node
    pids = np.array([[3 * k + 1, 3 * k + 2] for k in nodes], np.uint32).ravel()   # on u_y and u_z
    ptr = np.arange(0, len(pids) + 1, 2, dtype=np.uint32)
    coefs = np.tile([0.5, -0.25], len(ids))
    offs = np.linspace(1e-7, 2e-7, len(ids))
    t = G.Topology(gpu_ctx, m)
    try:
        t.assemble()
        t.apply_dirichlet(bc_ids, bc_vals, bc_kinds)
        arr0, rhs0 = t.matrix()
        rs, ci = t.pattern()
        t.set_proportional(ids, offs, ptr, pids, coefs)
        arr1, rhs1 = t.matrix()
        arr_o, rhs_o = arr0.copy(), rhs0.copy()
        O.proportional(3, rs, ci, arr_o, rhs_o, ids, offs, ptr, pids, coefs)
        assert not np.array_equal(arr1, arr0)
        assert rel(arr1, arr_o) <= 1e-14 and rel(rhs1, rhs_o) <= 1e-14
        x, st = t.solve(G.SOLVER_PCG_FP64, rtol=1e-12)
        assert st["relres"] <= 1e-12
        want = offs + 0.5 * x[pids[0::2]] - 0.25 * x[pids[1::2]]
        assert np.abs(x[ids] - want).max() <= 1e-14 * np.abs(x).max()
    finally:
        t.close()
