"""Edge cases of the device path against the oracle and the reference fixtures.

* elements given without Gauss points use their kind's default rule: the
  unenriched elements of the crack fixtures (3- and 6-node triangles), and the
  4-node tetrahedra of the voxel fixture, reproduce the reference's K_e;
* a single element: pattern, matrix and right-hand side as the oracle's;
* a zero right-hand side: every solver returns x = 0 after no iteration;
* every DOF prescribed: every solver returns the prescribed values;
* the mixed solver at an iteration cap reports AMIE_NOT_CONVERGED;
* the extrapolated warm start (amie_extrapolate) follows the reference's
  displacement history.
"""
import numpy as np
import pytest

from conftest import load_golden

import amie_mesh as am
import oracle as O

pytestmark = pytest.mark.gpu

SOLVERS = ("SOLVER_PCG_FP64", "SOLVER_PCG_MIXED", "SOLVER_AMIE_CG")


def rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def sub_mesh(m, elems, keep_gp=True):
    """The elements `elems` of m (unenriched), with their Gauss points or none."""
    kind, dof_ptr, dof_ids, gp_ptr, gp, jinv, mat, scale = [], [0], [], [0], [], [], [], []
    dd = m.dim * m.dim
    for e in elems:
        kind.append(m.kind[e])
        dof_ids.extend(m.dof_ids[m.dof_ptr[e]:m.dof_ptr[e + 1]])
        dof_ptr.append(len(dof_ids))
        if keep_gp:
            gp.extend(m.gp[(m.dim + 1) * m.gp_ptr[e]:(m.dim + 1) * m.gp_ptr[e + 1]])
            gp_ptr.append(gp_ptr[-1] + int(m.gp_ptr[e + 1] - m.gp_ptr[e]))
        else:
            gp_ptr.append(0)
        jinv.extend(m.jinv[dd * e:dd * (e + 1)])
        mat.append(m.mat[e])
        scale.append(m.scale[e] if m.scale is not None else 1.0)
    sub = am.MeshData(dim=m.dim, stride=m.stride, kind=kind, dof_ptr=dof_ptr, dof_ids=dof_ids, gp_ptr=gp_ptr,
                      gp=np.array(gp, np.float64), jinv=jinv, mat=mat, cmat_table=m.cmat_table, ndofmax=m.ndofmax,
                      scale=np.array(scale))
    sub.validate()
    return sub


def plain_elements(m):
    """Unenriched elements whose Jacobian is constant (not moved)."""
    nen = np.diff(m.enr_ptr.astype(np.int64))
    moved = m.moved if m.moved is not None else np.zeros(m.n_elem, np.uint8)
    return np.nonzero((nen == 0) & (moved == 0))[0]


@pytest.mark.parametrize("name", ["crack_p1", "crack_p2", "voxel_t4"])
def test_default_gauss_rule(gpu_ctx, name):
    import amie_gpu
    d = load_golden(name)
    m = am.from_golden(d, "tabulated")
    elems = plain_elements(m)
    assert len(elems) > 100
    sub = sub_mesh(m, elems, keep_gp=False)
    t = amie_gpu.Topology(gpu_ctx, sub)
    try:
        t.assemble()
        off, ke = t.element_matrices()
    finally:
        t.close()
    _, ko = O.element_matrices(sub)
    kp = d["ke_ptr"]
    for i, e in enumerate(elems):
        a, b = int(off[i]), int(off[i + 1])
        assert rel(ke[a:b], ko[a:b]) <= 1e-13, e
        assert rel(ke[a:b], d["ke"][kp[e]:kp[e + 1]]) <= 1e-12, e


def test_single_element(gpu_ctx):
    import amie_gpu
    d = load_golden("incl_p2")
    m = am.from_golden(d, "tabulated")
    e = int(plain_elements(m)[0])
    sub = sub_mesh(m, [e])
    ids = np.unique(sub.dof_ids)
    remap = np.zeros(int(ids.max()) + 1, np.uint32)
    remap[ids] = np.arange(len(ids), dtype=np.uint32)
    sub.dof_ids = remap[sub.dof_ids]
    sub.ndofmax = len(ids)
    # fix node 0 along both axes, pull node 1 along x
    bc_ids = np.array([0, 1, 2], np.uint32)
    bc_vals = np.array([0.0, 0.0, 1e-6])
    kinds = np.zeros(3, np.uint8)
    R = O.assemble(sub, bc_ids, bc_vals, kinds)
    t = amie_gpu.Topology(gpu_ctx, sub)
    try:
        rs, ci = t.pattern()
        assert np.array_equal(rs, R["row_size"]) and np.array_equal(ci, R["column_index"])
        t.assemble()
        t.apply_dirichlet(bc_ids, bc_vals, kinds)
        arr, rhs = t.matrix()
        assert rel(arr, R["array"]) <= 1e-14 and rel(rhs, R["rhs"]) <= 1e-14
    finally:
        t.close()


@pytest.mark.parametrize("solver", SOLVERS)
def test_zero_rhs_gives_zero_solution(gpu_ctx, solver):
    import amie_gpu
    d = load_golden("incl_p1")
    m = am.from_golden(d, "tabulated")
    ids, _, kinds = am.golden_bcs(d)
    t = amie_gpu.Topology(gpu_ctx, m)
    try:
        t.assemble()
        t.apply_dirichlet(ids, np.zeros(len(ids)), kinds)
        x, st = t.solve(getattr(amie_gpu, solver), rtol=1e-10, x0=np.zeros(t.n))
    finally:
        t.close()
    assert np.all(x == 0.0)
    assert st["iterations"] == 0


@pytest.mark.parametrize("solver", SOLVERS)
def test_every_dof_prescribed(gpu_ctx, solver):
    import amie_gpu
    d = load_golden("incl_p1")
    m = am.from_golden(d, "tabulated")
    n = m.stride * (int(m.dof_ids.max()) + 1)
    rng = np.random.default_rng(3)
    vals = rng.uniform(-1e-5, 1e-5, n)
    ids = np.arange(n, dtype=np.uint32)
    t = amie_gpu.Topology(gpu_ctx, m)
    try:
        t.assemble()
        t.apply_dirichlet(ids, vals, np.zeros(n, np.uint8))
        x, st = t.solve(getattr(amie_gpu, solver), rtol=1e-10)
    finally:
        t.close()
    assert rel(x[:n], vals) <= 1e-12


def test_mixed_iteration_cap_reports_not_converged(gpu_ctx):
    import amie_gpu
    d = load_golden("incl_p2")
    m = am.from_golden(d, "tabulated")
    t = amie_gpu.Topology(gpu_ctx, m)
    try:
        t.assemble()
        t.apply_dirichlet(*am.golden_bcs(d))
        x, st = t.solve(amie_gpu.SOLVER_PCG_MIXED, rtol=1e-12, maxit=20, accept=(amie_gpu.AMIE_NOT_CONVERGED,))
    finally:
        t.close()
    assert st["status"] == amie_gpu.AMIE_NOT_CONVERGED
    assert 0 < st["iterations"] <= 20 + 16
    assert np.all(np.isfinite(x))


def test_extrapolated_warm_start(gpu_ctx):
    """amie_extrapolate follows Assembly::extrapolate: after the first solve the
    next start is 2 u1 (history [0, u1]), then 2 u2 - u1; on a linear problem
    loaded proportionally the extrapolated start is the solution, so the warm
    solve needs far fewer iterations than the first."""
    import amie_gpu
    d = load_golden("incl_p1")
    m = am.from_golden(d, "tabulated")
    ids, vals, kinds = am.golden_bcs(d)
    t = amie_gpu.Topology(gpu_ctx, m)
    try:
        t.assemble()
        t.apply_dirichlet(ids, vals, kinds)
        st1 = t.solve_resident(amie_gpu.SOLVER_PCG_FP64, rtol=1e-12)
        u1 = t.solution()
        t.apply_dirichlet(ids, 2 * vals, kinds)
        t.extrapolate()
        assert np.array_equal(t.solution(), u1 + u1)
        st2 = t.solve_resident(amie_gpu.SOLVER_PCG_FP64, rtol=1e-12, use_x0=True)
        u2 = t.solution()
        assert rel(u2, 2 * u1) <= 1e-10
        assert st2["iterations"] < st1["iterations"] // 4
        t.extrapolate()
        assert np.array_equal(t.solution(), u2 + (u2 - u1))
    finally:
        t.close()
