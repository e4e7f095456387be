"""Continuous-batching server: results are the same alone and in a mix (within
the solve tolerance), requests arriving while others run are admitted, and the
failure paths are reported as statuses (all faults made on the host: an
impossible memory budget, a NaN right-hand side, a cancelled request, a drain
timeout).

Tolerance: every result reaches relative residual 1e-10; a request's
displacements alone and in the mix agree to 1e-12 relative (the server gives a
slot a CTA count that depends on its own size only, so its arithmetic does not
depend on the other requests) and to 1e-8 against a FP64 PCG solve to 1e-12.
"""
import time

import numpy as np
import pytest

import amie_mesh as am

pytestmark = pytest.mark.gpu


def _requests():
    import workloads as W
    out = []
    for i, (dof, frac) in enumerate([(3000, 0.3), (12000, 0.45), (40000, 0.25), (6000, 0.55)]):
        out.append(W.homogenisation_request(dof, frac, seed=100 + i))
    return out


def rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def _wait(srv, tickets, timeout=120):
    t_end = time.time() + timeout
    res = {}
    while len(res) < len(tickets) and time.time() < t_end:
        for t in tickets:
            if t not in res:
                r = srv.poll(t)
                if r is not None:
                    res[t] = r
        time.sleep(0.002)
    return res


@pytest.mark.parametrize("solver", ["mixed", "fp64", "mixed-persistent"])
def test_alone_equals_mix(gpu_ctx, monkeypatch, solver):
    """Each result is the same alone and in a mix (bitwise for the node displacements'
    1e-12 check); "mixed-persistent" runs the batches as one cooperative launch
    (AMIE_SERVER_PERSISTENT=1, read when a server starts)."""
    import amie_gpu as G
    if solver == "mixed-persistent":
        monkeypatch.setenv("AMIE_SERVER_PERSISTENT", "1")
    sv = G.SOLVER_PCG_FP64 if solver == "fp64" else G.SOLVER_PCG_MIXED
    reqs = _requests()
    alone = []
    for m, bcs, _ in reqs:
        srv = G.Server(gpu_ctx, solver=sv, rtol=1e-10)
        t = srv.submit(m, *bcs)
        assert srv.drain(60.0) == G.AMIE_OK
        (res, x), = _wait(srv, [t]).values()
        assert res["status"] == G.AMIE_OK and res["relres"] <= 1e-10
        alone.append(x)
        srv.stop()
    srv = G.Server(gpu_ctx, solver=sv, rtol=1e-10)
    tickets = []
    for k in range(3):   # staggered arrivals: later requests join while earlier ones run
        for m, bcs, _ in reqs:
            tickets.append(srv.submit(m, *bcs))
        time.sleep(0.003)
    assert srv.drain(120.0) == G.AMIE_OK
    res = _wait(srv, tickets)
    for i, t in enumerate(tickets):
        r, x = res[t]
        assert r["status"] == G.AMIE_OK and r["relres"] <= 1e-10
        assert rel(x, alone[i % len(reqs)]) <= 1e-12
    srv.stop()
    # against a plain FP64 solve of the same system
    for (m, bcs, _), x in zip(reqs, alone):
        t = G.Topology(gpu_ctx, m)
        t.assemble()
        t.apply_dirichlet(*bcs)
        xr, st = t.solve(G.SOLVER_PCG_FP64, rtol=1e-12)
        assert rel(x, xr) <= 1e-8
        t.close()


@pytest.mark.parametrize("solver", ["mixed", "fp64"])
def test_3d_requests_in_a_2d_mix(gpu_ctx, solver):
    """Tetrahedral (3x3-block) requests batch with triangle requests: a batch with a
    3D slot runs the kernels that hold both strides' bodies; each result equals
    the same request served alone (1e-12) and a plain FP64 solve (1e-8)."""
    import amie_gpu as G
    import workloads as W
    sv = G.SOLVER_PCG_FP64 if solver == "fp64" else G.SOLVER_PCG_MIXED
    reqs = [W.voxel_cube(nv=6, seed=11)[:2], W.homogenisation_request(8000, 0.4, seed=7)[:2],
            W.voxel_cube(nv=9, seed=12)[:2]]
    alone = []
    for m, bcs in reqs:
        srv = G.Server(gpu_ctx, solver=sv, rtol=1e-10)
        t = srv.submit(m, *bcs)
        assert srv.drain(60.0) == G.AMIE_OK
        (res, x), = _wait(srv, [t]).values()
        assert res["status"] == G.AMIE_OK and res["relres"] <= 1e-10
        alone.append(x)
        srv.stop()
    srv = G.Server(gpu_ctx, solver=sv, rtol=1e-10)
    tickets = [srv.submit(m, *bcs) for _ in range(2) for m, bcs in reqs]
    assert srv.drain(120.0) == G.AMIE_OK
    res = _wait(srv, tickets)
    for i, t in enumerate(tickets):
        r, x = res[t]
        assert r["status"] == G.AMIE_OK and r["relres"] <= 1e-10
        assert rel(x, alone[i % len(reqs)]) <= 1e-12
    srv.stop()
    for (m, bcs), x in zip(reqs, alone):
        t = G.Topology(gpu_ctx, m)
        t.assemble()
        t.apply_dirichlet(*bcs)
        xr, st = t.solve(G.SOLVER_PCG_FP64, rtol=1e-12)
        assert rel(x, xr) <= 1e-8
        t.close()


def test_failure_statuses(gpu_ctx):
    import amie_gpu as G
    (m, bcs, _), (m2, bcs2, _) = _requests()[:2]
    # an impossible budget: the request can never be admitted -> OOM, nothing else blocks
    srv = G.Server(gpu_ctx, solver=G.SOLVER_PCG_MIXED, hbm_budget_bytes=1 << 20)
    t = srv.submit(m, *bcs)
    assert srv.drain(30.0) == G.AMIE_OK
    (r, _), = _wait(srv, [t]).values()
    assert r["status"] == G.AMIE_OOM
    srv.stop()
    # NaN in the imposed values -> NAN, other requests unaffected
    srv = G.Server(gpu_ctx, solver=G.SOLVER_PCG_MIXED)
    vals = bcs[1].copy()
    vals[np.argmax(vals)] = np.nan
    t_bad = srv.submit(m, bcs[0], vals, bcs[2])
    t_ok = srv.submit(m2, *bcs2)
    assert srv.drain(60.0) == G.AMIE_OK
    res = _wait(srv, [t_bad, t_ok])
    assert res[t_bad][0]["status"] == G.AMIE_NAN
    assert res[t_ok][0]["status"] == G.AMIE_OK
    srv.stop()
    # cancellation of a queued request and a drain deadline
    srv = G.Server(gpu_ctx, solver=G.SOLVER_PCG_FP64)
    big = [srv.submit(m2, *bcs2) for _ in range(4)]
    tc = srv.submit(m, *bcs)
    srv.cancel(tc)
    assert srv.drain(1e-6) in (G.AMIE_TIMEOUT, G.AMIE_OK)
    assert srv.drain(60.0) == G.AMIE_OK
    res = _wait(srv, big + [tc])
    assert res[tc][0]["status"] in (G.AMIE_CANCELLED, G.AMIE_OK)
    assert all(res[t][0]["status"] == G.AMIE_OK for t in big)
    srv.stop()


def test_persistent_barrier_gives_up_and_server_recovers(gpu_ctx, monkeypatch):
    """A persistent batch whose slot barrier cannot be reached ends by itself:
    the host claims one CTA more for the first request's slot than it launches
    (AMIE_SERVER_SHORT_SLOT=1, a host-side fault), the slot barrier gives up after
    barrier_polls polls (~1 ms here), that request ends with AMIE_TIMEOUT, and
    the next request on the same server solves to 1e-10 and matches a direct solve."""
    import amie_gpu as G
    monkeypatch.setenv("AMIE_SERVER_PERSISTENT", "1")
    monkeypatch.setenv("AMIE_SERVER_ROWS_PER_CTA", "64")   # several CTAs per slot, one of them left out
    monkeypatch.setenv("AMIE_SERVER_SHORT_SLOT", "1")
    m, bcs, _ = _requests()[0]
    srv = G.Server(gpu_ctx, solver=G.SOLVER_PCG_MIXED, rtol=1e-10, barrier_polls=1 << 14)
    try:
        t1 = srv.submit(m, *bcs)
        r1 = _wait(srv, [t1], timeout=60)
        assert t1 in r1 and r1[t1][0]["status"] == G.AMIE_TIMEOUT, r1
        t2 = srv.submit(m, *bcs)
        r2 = _wait(srv, [t2], timeout=60)
        assert t2 in r2
        res, x = r2[t2]
        assert res["status"] == G.AMIE_OK and res["relres"] <= 1e-10, res
    finally:
        srv.stop()
    topo = G.Topology(gpu_ctx, m)
    topo.assemble()
    topo.apply_dirichlet(*bcs)
    x_ref, _ = topo.solve(G.SOLVER_PCG_FP64, rtol=1e-12)
    topo.close()
    assert rel(x, x_ref) <= 1e-8
