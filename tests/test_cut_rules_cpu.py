"""CPU checks of the crack-rule restatement (oracle/cut_rules.py) on seeded
random triangles crossed by a straight crack: every rule it produces --
the reference's sub-triangulation where that one applies, the conforming
replacement where the reference would use Monte-Carlo -- integrates the
Heaviside-enriched P1 element matrix exactly, i.e. equals an independent
exact rule (three conforming pieces, Dunavant degree 4) to round-off.
Only triangles inside the crack's strip are used (all corners project into
the segment), where the crack's Heaviside is the side of the line."""
import numpy as np

import amie_mesh as am
import cut_rules as CR
import oracle as O

C_PLANE = np.array([[1.0, 0.2, 0.0], [0.2, 1.0, 0.0], [0.0, 0.0, 0.4]]) * 3e10 / (1 - 0.04)


def one_element_mesh(corners, rule):
    """A P1 triangle (DOFs 0-2) with the Heaviside functions of its three
    corners (DOFs 3-5) integrated by `rule` = [(xi, eta, w, h)], h_vertex from
    the same crack."""
    X = corners.reshape(3, 2)
    J = np.array([[X[2, 0] - X[1, 0], X[0, 0] - X[1, 0]], [X[2, 1] - X[1, 1], X[0, 1] - X[1, 1]]])
    jinv = np.linalg.inv(J).T          # the layout of the reference fixtures
    return X, jinv, rule


def ke_of(corners, line, rule):
    X, jinv, rule = one_element_mesh(corners, rule)
    w = CR.witness(line)
    hv = [CR.heaviside(tuple(x), line, w) for x in X]
    n = len(rule)
    gp = np.array([(p[0], p[1], p[2]) for p in rule]).ravel()
    jump = []
    for k in range(3):
        jump += [p[3] - hv[k] for p in rule]
    m = am.MeshData(dim=2, stride=2, kind=[am.TRI3], dof_ptr=[0, 6], dof_ids=[0, 1, 2, 3, 4, 5], gp_ptr=[0, n],
                    gp=gp, jinv=jinv.ravel(), mat=[0], cmat_table=C_PLANE.ravel(), ndofmax=6,
                    scale=np.ones(1), enr_ptr=[0, 3], enr_type=np.full(3, am.ENR_HEAVISIDE, np.uint8),
                    enr_vertex=[0, 1, 2], enr_data=[0, n, 2 * n], enr_jump=np.array(jump, np.int8),
                    enr_grad=np.zeros(2 * 3 * n))
    m.validate()
    _, ke = O.element_matrices(m)
    return ke


def random_strip_triangles(n, seed):
    rng = np.random.default_rng(seed)
    out = []
    while len(out) < n:
        c = np.array([rng.uniform(0.25, 0.75), rng.normal(0.0, 0.02)])
        size = rng.uniform(0.02, 0.15)
        ang = rng.uniform(0, 2 * np.pi) + np.array([0.0, 2.1, 4.2]) + rng.normal(0, 0.3, 3)
        pts = c + size * np.stack([np.cos(ang), np.sin(ang)], -1)
        if np.all((pts[:, 0] > 0.05) & (pts[:, 0] < 0.95)):
            out.append(pts.ravel())
    return np.array(out)


def test_rules_integrate_heaviside_elements_exactly():
    line = np.array([[0.0, 0.0], [1.0, 0.0]])
    corners = random_strip_triangles(400, 11)
    seen = {CR.OK: 0, CR.REPLACED: 0}
    for c in corners:
        st, rule, _ = CR.element_rule(c, line, CR.REPLACE_MONTE_CARLO)
        split = CR.split_rule_degree4(c, line)
        if st not in seen or split is None:
            continue
        seen[st] += 1
        ka, kb = ke_of(c, line, rule), ke_of(c, line, split)
        assert np.abs(ka - kb).max() <= 1e-12 * np.abs(kb).max(), (st, c)
    assert seen[CR.OK] > 50 and seen[CR.REPLACED] > 10, seen
