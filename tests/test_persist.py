"""PCG runs as one cooperative launch (k_pcg_persist, xfem-amie_gb300/csrc/persist.cuh)
against the graphs of kernels: the same solutions and about the same number of
iterations, in 2D and 3D (the FP32 runs of the mixed solver, whose graphs fold
the direction update; FP64 runs keep their graphs); and a grid barrier that
gives up ends the launch with AMIE_TIMEOUT, after which the context still
solves."""
import numpy as np
import pytest

from conftest import load_golden

import amie_mesh as am

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def _solve(ctx, d, solver, rtol, monkeypatch, persist, unreachable=False):
    import amie_gpu as G
    monkeypatch.setenv("AMIE_PERSIST", "1" if persist else "0")
    monkeypatch.setenv("AMIE_PERSIST_BARRIER_TEST", "1" if unreachable else "0")
    m = am.from_golden(d, "auto")
    t = G.Topology(ctx, m)
    try:
        t.assemble()
        t.apply_dirichlet(*am.golden_bcs(d))
        return t.solve(solver, rtol=rtol)
    finally:
        t.close()


@pytest.mark.parametrize("name", ["incl_p1", "incl_p2", "crack_p2", "voxel_t4"])
@pytest.mark.parametrize("solver", ["mixed"])
def test_persistent_matches_graph(gpu_ctx, monkeypatch, name, solver):
    import amie_gpu as G
    d = load_golden(name)
    sv = G.SOLVER_PCG_MIXED if solver == "mixed" else G.SOLVER_PCG_FP64
    rtol = 1e-10 if solver == "mixed" else 1e-12
    xg, sg = _solve(gpu_ctx, d, sv, rtol, monkeypatch, persist=False)
    xp, sp = _solve(gpu_ctx, d, sv, rtol, monkeypatch, persist=True)
    assert sg["status"] == G.AMIE_OK and sp["status"] == G.AMIE_OK, (sg, sp)
    assert sp["relres"] <= rtol and sg["relres"] <= rtol
    assert rel(xp, xg) <= (1e-8 if solver == "mixed" else 1e-10), (rel(xp, xg), sg, sp)
    assert abs(sp["iterations"] - sg["iterations"]) <= 0.1 * sg["iterations"] + 5, (sg, sp)


def test_persistent_barrier_gives_up(gpu_ctx, monkeypatch):
    """Barriers that wait for one arrival more than the grid has: every CTA
    gives up after its poll limit (4096 polls) or on seeing the error flag,
    the launch ends and the solve reports AMIE_TIMEOUT; a solve with normal
    barriers then succeeds on the same context."""
    import amie_gpu as G
    d = load_golden("incl_p1")
    with pytest.raises(G.AmieError) as ei:
        _solve(gpu_ctx, d, G.SOLVER_PCG_MIXED, 1e-10, monkeypatch, persist=True, unreachable=True)
    assert ei.value.status == G.AMIE_TIMEOUT
    assert "grid barrier" in str(ei.value)
    x, st = _solve(gpu_ctx, d, G.SOLVER_PCG_MIXED, 1e-10, monkeypatch, persist=True)
    assert st["status"] == G.AMIE_OK and st["relres"] <= 1e-10
