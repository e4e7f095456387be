"""Tip branch functions of BranchedCrack::enrichTip (features/crack.cpp:898-960)
evaluated in closed form, pinned to the reference's crack_p2 fixture.

The fixture is the harness's straight crack from (-L/2 + 1e-4, y0) to
(-L/2 + 0.3 L, y0) (L = 0.04, y0 = 0.0013; tests/golden/make_golden.py and
oracle/ref_harness.cpp); its tip-enriched elements carry, per Gauss point, the
reference's function values (VirtualMachine::eval) and local gradients
(VirtualMachine::deval, 4th-order central differences).

CPU: every non-Heaviside enrichment function of the fixture is a tip branch
function of the head tip (angle pi) with the reference's values to 1e-12; the
closed-form gradients agree with the reference's numerical ones to 5e-9 of
their scale, and the oracle's element matrices built from them agree with the
reference's K_e to 1e-8.  GPU (`-m gpu`): the device's AMIE_ENR_TIP element
matrices equal the oracle's from the tabulated closed form to 1e-12, and a
solve with them matches the oracle's.
"""
import numpy as np
import pytest

from conftest import load_golden

import amie_mesh as am
import oracle as O

L, Y0 = 0.04, 0.0013
TIPS = (((-L / 2 + 1e-4, Y0), np.pi), ((-L / 2 + 0.3 * L, Y0), 0.0))


def tip_mesh():
    d = load_golden("crack_p2")
    return d, am.from_golden(d, "tip", tips=TIPS)


def test_tip_functions_match_reference_values_and_gradients():
    d, m = tip_mesh()
    tips = np.nonzero(m.enr_type == am.ENR_TIP)[0]
    assert len(tips) == 12   # three elements, four branch functions each
    heav = np.count_nonzero(m.enr_type == am.ENR_HEAVISIDE)
    assert heav + len(tips) == len(m.enr_type)   # nothing left tabulated
    egp = d["enr_gp_ptr"]
    gp = m.gp.reshape(-1, 3)
    for f in tips:
        e = int(np.searchsorted(m.enr_ptr, f, side="right") - 1)
        pts = gp[m.gp_ptr[e]:m.gp_ptr[e + 1], :2]
        rec = m.enr_tip[8 * m.enr_data[f]:8 * m.enr_data[f] + 8]
        vals = d["enr_val"][egp[f]:egp[f + 1]]
        assert np.abs(am.tip_values(rec, int(m.enr_vertex[f]), pts[:, 0], pts[:, 1]) - vals).max() \
            <= 1e-12 * np.abs(vals).max()
        ref = d["enr_grad"][2 * egp[f]:2 * egp[f + 1]].reshape(-1, 2)
        mine = O.tip_gradients(rec, int(m.enr_vertex[f]), pts[:, 0], pts[:, 1])
        assert np.abs(mine - ref).max() <= 5e-9 * np.abs(ref).max(), f


def test_tip_element_matrices_match_reference():
    d, m = tip_mesh()
    mt = O.with_tabulated_tips(m)
    off, ke = O.element_matrices(mt)
    kp = d["ke_ptr"]
    for e in np.nonzero(np.diff(m.enr_ptr.astype(np.int64)))[0]:
        if not (m.enr_type[m.enr_ptr[e]:m.enr_ptr[e + 1]] == am.ENR_TIP).any():
            continue
        mine = ke[int(off[e]):int(off[e + 1])]
        ref = d["ke"][kp[e]:kp[e + 1]]
        assert np.abs(mine - ref).max() <= 1e-8 * np.abs(ref).max(), e


@pytest.mark.gpu
def test_device_tip_element_matrices(gpu_ctx):
    import amie_gpu as G
    from test_gpu_parity import node_dofs
    d, m = tip_mesh()
    mt = O.with_tabulated_tips(m)
    off_o, ke_o = O.element_matrices(mt)
    t = G.Topology(gpu_ctx, m)
    try:
        t.assemble()
        off, ke = t.element_matrices()
        assert np.array_equal(off, off_o)
        for e in range(m.n_elem):
            a, b = int(off[e]), int(off[e + 1])
            assert np.abs(ke[a:b] - ke_o[a:b]).max() <= 1e-12 * np.abs(ke_o[a:b]).max(), e
        # the same system solved on the device and by the oracle; node displacements
        # only (the tip-enriched P2 crack does not determine its enrichment amplitudes)
        ids, vals, kinds = am.golden_bcs(d)
        t.apply_dirichlet(ids, vals, kinds)
        x, st = t.solve(G.SOLVER_PCG_FP64, rtol=1e-12)
        assert st["relres"] <= 1e-12
        R = O.assemble(mt, ids, vals, kinds)
        xo, _, _, rc = O.pcg(2, R["row_size"], R["column_index"], R["array"], R["rhs"], rtol=1e-13)
        s = node_dofs(m)
        assert np.abs(x[s] - xo[s]).max() <= 1e-7 * np.abs(xo[s]).max()
    finally:
        t.close()
