"""The SELL-32-sigma layout of the solver SpMV built on the device
(k_sell_perm, k_sell_slots, csrc/assemble.cu) against the host build
(AMIE_SELL_HOST=1): the same permutation and slices, so the FP32 and FP64
solves give the same bits."""
import numpy as np
import pytest

from conftest import load_golden

import amie_mesh as am

pytestmark = pytest.mark.gpu


def _solve(ctx, m, bcs, solver, monkeypatch, host):
    import amie_gpu as G
    monkeypatch.setenv("AMIE_SELL_HOST", "1" if host else "0")
    t = G.Topology(ctx, m)
    try:
        t.assemble()
        t.apply_dirichlet(*bcs)
        return t.solve(solver, rtol=1e-10)
    finally:
        t.close()


@pytest.mark.parametrize("case", ["incl_p2", "crack_p2", "voxel_t4", "cfg0"])
def test_device_sell_build_matches_host(gpu_ctx, monkeypatch, case):
    import amie_gpu as G
    if case == "cfg0":
        import workloads as W
        m, bcs, _ = W.inclusion_square(141, L=0.04, order=1, n_inclusions=300, seed=2024)
    else:
        d = load_golden(case)
        m, bcs = am.from_golden(d, "auto"), am.golden_bcs(d)
    for solver in (G.SOLVER_PCG_MIXED, G.SOLVER_PCG_FP64):
        xd, sd = _solve(gpu_ctx, m, bcs, solver, monkeypatch, host=False)
        xh, sh = _solve(gpu_ctx, m, bcs, solver, monkeypatch, host=True)
        assert sd["iterations"] == sh["iterations"], (case, solver, sd, sh)
        assert np.array_equal(xd.view(np.uint64), xh.view(np.uint64)), (case, solver)
