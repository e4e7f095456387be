"""Synthetic workloads (no GPU): sizes of the benchmark configurations, element
data consistency, and a small instance of each solved by the CPU oracle."""
import numpy as np
import pytest

import amie_mesh as am
import oracle as O
import workloads as W


def test_config1_full_size_shape():
    m, bcs, meta = W.cracked_square(387, L=0.1, order=2, n_inclusions=4000, seed=2024)
    m.validate()
    assert 1.15e6 < meta["n_dof"] < 1.25e6
    assert meta["n_elem"] == 2 * 387 * 387
    assert meta["n_inclusions"] > 3500
    assert meta["n_cut"] > 100 and meta["tip_elem"] >= 0
    nf = m.nf()
    assert nf.max() >= 6 + 3 + 4 and nf.min() == 6          # variable DOF count per element
    assert np.diff(m.gp_ptr).max() == 512                    # Monte-Carlo tip element
    ids, vals, kinds = bcs
    assert np.all(np.diff(ids.astype(np.int64)) > 0)        # sorted, unique


@pytest.mark.parametrize("order", [1, 2])
def test_cracked_square_small_solves(order):
    m, bcs, meta = W.cracked_square(24, order=order, n_inclusions=40, seed=3)
    m.validate()
    R = O.assemble(m, *bcs)
    # enriched element matrices are symmetric positive semi-definite
    off, ke = R["off"], R["ke"]
    for e in np.nonzero(np.diff(m.enr_ptr))[0]:
        K = ke[int(off[e]):int(off[e + 1])]
        k = int(np.sqrt(len(K)))
        K = K.reshape(k, k)
        assert np.allclose(K, K.T, rtol=0, atol=1e-9 * np.abs(K).max())
        ev = np.linalg.eigvalsh(K)
        assert ev.min() >= -1e-9 * ev.max()
    x, it, rr, rc = O.pcg(2, R["row_size"], R["column_index"], R["array"], R["rhs"], rtol=1e-10)
    assert rc == 0 and rr <= 1e-10


def test_voxel_cube_matches_voxelfilter_counts():
    m, bcs, meta = W.voxel_cube(4, seed=1)
    m.validate()
    assert meta["n_elem"] == 6 * 4 ** 3 and meta["n_dof"] == 3 * 5 ** 3
    R = O.assemble(m, *bcs)
    x, it, rr, rc = O.pcg(3, R["row_size"], R["column_index"], R["array"], R["rhs"], rtol=1e-10)
    assert rc == 0
    # uniaxial strain 1e-4 on a 1e-4 m cube: right face displaced by 1e-8 m
    assert abs(x.max() - 1e-8) < 1e-12


def test_homogenisation_request_sizes():
    for dof in (2000, 20000, 200000):
        m, bcs, meta = W.homogenisation_request(dof, 0.4, seed=1)
        assert 0.8 * dof < meta["n_dof"] < 1.25 * dof
        assert 0.3 < meta["fraction"] < 0.5
    specs, arrivals = W.serving_mix(64, 200.0)
    assert len(specs) == 64 and len(arrivals) == 64
    assert len({sp[2] for sp in specs}) == 64   # every request its own microstructure
    assert all(2000 <= sp[0] <= 200000 and 0.2 <= sp[1] <= 0.6 for sp in specs)
    assert 0.15 < arrivals[-1] < 0.6      # 64 Poisson arrivals at 200/s
    m, (ids, vals, kinds) = W.serving_request(specs[0])
    m.validate()
    assert len(ids) == len(vals) == len(kinds)


def test_fast_inclusion_helpers_match_the_plain_ones():
    import numpy as np
    rng = np.random.default_rng(3)
    x, y, conn, vx, vy, M = W.structured_triangles(60, 0.04, 1, 0.15, rng)
    cx, cy, cr = W.place_inclusions(np.random.default_rng(5), np.random.default_rng(6).uniform(0.3e-3, 1.5e-3, 120),
                                    0.04)
    gx, gy = vx.mean(1), vy.mean(1)
    h = 0.04 / 60
    assert np.array_equal(W._in_inclusions(gx, gy, cx, cy, cr, h, 60), W._in_circles_structured(gx, gy, 60, h, cx, cy, cr))
    J1, _ = W._tri_jinv(vx, vy)
    assert np.abs(J1 - W._jinv_closed(vx, vy)).max() <= 1e-14 * np.abs(J1).max()
    cx2, cy2, cr2 = W._place_inclusions_batched(np.random.default_rng(9), np.full(150, 1e-3), 0.04)
    d2 = (cx2[:, None] - cx2[None]) ** 2 + (cy2[:, None] - cy2[None]) ** 2
    np.fill_diagonal(d2, np.inf)
    assert (d2 > (2e-3) ** 2).all()   # no overlaps
