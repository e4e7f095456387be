"""Every loop variant of the SELL SpMV gives the same solves.

The variant is read from AMIE_SELL_VARIANT when a topology is built (a tuning
override; 0 is the default).  All variants visit the blocks of a row in the
block-CSR order with the same FMA sequence, so each must reproduce the FP64
and mixed solves of the oracle on 2x2 (triangles) and 3x3 (tetrahedra) blocks.
"""
import numpy as np
import pytest

from conftest import load_golden
from test_gpu_parity import node_dofs

import amie_mesh as am
import oracle as O

pytestmark = pytest.mark.gpu

CASES = ["incl_p1", "crack_p1", "voxel_t4"]


def relres(d, m, x):
    r = d["rhs"] - O.spmv(m.stride, d["row_size"], d["column_index"], d["array"], x)
    return float(np.linalg.norm(r) / np.linalg.norm(d["rhs"]))


@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("variant", range(8))
def test_sell_variant_solves(gpu_ctx, monkeypatch, name, variant):
    import amie_gpu
    monkeypatch.setenv("AMIE_SELL_VARIANT", str(variant))
    d = load_golden(name)
    m = am.from_golden(d, "tabulated")
    t = amie_gpu.Topology(gpu_ctx, m)
    try:
        t.assemble()
        t.apply_dirichlet(*am.golden_bcs(d))
        x64, st64 = t.solve(amie_gpu.SOLVER_PCG_FP64, rtol=1e-12)
        assert st64["relres"] <= 1e-12
        assert relres(d, m, x64) <= 2e-12
        x32, st32 = t.solve(amie_gpu.SOLVER_PCG_MIXED, rtol=1e-10)
        assert st32["relres"] <= 1e-10
        assert relres(d, m, x32) <= 2e-10
        xo, _, _, _ = O.pcg(m.stride, d["row_size"], d["column_index"], d["array"], d["rhs"], rtol=1e-13)
        s = node_dofs(m)
        scale = np.abs(xo[s]).max()
        assert np.abs(x64[s] - xo[s]).max() <= 1e-9 * scale
        assert np.abs(x32[s] - xo[s]).max() <= 1e-8 * scale
    finally:
        t.close()


@pytest.mark.parametrize("name", CASES)
def test_folded_direction_is_bitwise_identical(gpu_ctx, monkeypatch, name):
    """FP32 graphs form p = z + beta p inside the SpMV (default) or in a separate
    kernel (AMIE_FOLD_DIR=0, read when a topology's solver state is made); both
    compute fma(beta, p, z), so the mixed solves must agree bit for bit."""
    import amie_gpu
    d = load_golden(name)
    m = am.from_golden(d, "tabulated")
    out = []
    for fold in ("1", "0"):
        monkeypatch.setenv("AMIE_FOLD_DIR", fold)
        t = amie_gpu.Topology(gpu_ctx, m)
        try:
            t.assemble()
            t.apply_dirichlet(*am.golden_bcs(d))
            out.append(t.solve(amie_gpu.SOLVER_PCG_MIXED, rtol=1e-10))
        finally:
            t.close()
    (x1, s1), (x0, s0) = out
    assert s1["iterations"] == s0["iterations"]
    assert np.array_equal(x1, x0)


@pytest.mark.parametrize("name", CASES)
def test_single_reduction_pcg_solves(gpu_ctx, monkeypatch, name):
    """The opt-in single-reduction (Chronopoulos-Gear) FP32 runs of the mixed
    solver (AMIE_CGCG=1, one kernel per iteration, reliable updates with the
    direction kept) reach the oracle's solution, and repeat bit for bit."""
    import amie_gpu
    monkeypatch.setenv("AMIE_CGCG", "1")
    d = load_golden(name)
    m = am.from_golden(d, "tabulated")
    t = amie_gpu.Topology(gpu_ctx, m)
    try:
        t.assemble()
        t.apply_dirichlet(*am.golden_bcs(d))
        x1, st1 = t.solve(amie_gpu.SOLVER_PCG_MIXED, rtol=1e-10)
        x2, st2 = t.solve(amie_gpu.SOLVER_PCG_MIXED, rtol=1e-10)
        assert st1["relres"] <= 1e-10 and relres(d, m, x1) <= 2e-10
        assert st1["refinements"] >= 2   # at least one resumed run
        assert np.array_equal(x1, x2) and st1["iterations"] == st2["iterations"]
        xo, _, _, _ = O.pcg(m.stride, d["row_size"], d["column_index"], d["array"], d["rhs"], rtol=1e-13)
        s = node_dofs(m)
        assert np.abs(x1[s] - xo[s]).max() <= 1e-8 * np.abs(xo[s]).max()
    finally:
        t.close()


@pytest.mark.parametrize("name", CASES)
def test_one_kernel_pcg_solves(gpu_ctx, monkeypatch, name):
    """The opt-in one-kernel FP32 PCG (AMIE_FUSED=1, k_sell_fused: the previous
    iteration's update and the direction formed inside the SpMV, r.z of the
    next step from the expansion of r - alpha q) reaches the oracle's solution
    and repeats bit for bit."""
    import amie_gpu
    monkeypatch.setenv("AMIE_FUSED", "1")
    d = load_golden(name)
    m = am.from_golden(d, "tabulated")
    t = amie_gpu.Topology(gpu_ctx, m)
    try:
        t.assemble()
        t.apply_dirichlet(*am.golden_bcs(d))
        x1, st1 = t.solve(amie_gpu.SOLVER_PCG_MIXED, rtol=1e-10)
        x2, st2 = t.solve(amie_gpu.SOLVER_PCG_MIXED, rtol=1e-10)
        assert st1["relres"] <= 1e-10 and relres(d, m, x1) <= 2e-10
        assert np.array_equal(x1, x2) and st1["iterations"] == st2["iterations"]
        xo, _, _, _ = O.pcg(m.stride, d["row_size"], d["column_index"], d["array"], d["rhs"], rtol=1e-13)
        s = node_dofs(m)
        assert np.abs(x1[s] - xo[s]).max() <= 1e-8 * np.abs(xo[s]).max()
    finally:
        t.close()
