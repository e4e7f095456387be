"""Helpers for the crack-rule tests: the crack of a fixture, its Heaviside-enriched
elements, and a mesh of those elements integrated with generated rules."""
import numpy as np

import amie_mesh as am


def harness_args(d):
    kv = {}
    for tok in str(d["harness_args"]).split():
        k, _, v = tok.partition("=")
        kv[k] = v
    return kv


def crack_line(d):
    """The crack of the reference harness's crack case: a horizontal segment
    from (-L/2 + 1e-4, y0) to (-L/2 + 0.3 L, y0) in the square of side L."""
    kv = harness_args(d)
    L = float(kv.get("size", 0.04))
    y0 = float(kv.get("crack_y", 0.0013))
    return np.array([[-L / 2 + 1e-4, y0], [-L / 2 + 0.3 * L, y0]])


def heaviside_elements(m):
    """Elements whose enrichment functions are all Heaviside (the crack's
    enrichSegmentedLine elements; tip-enriched elements are left out)."""
    out = []
    for e in range(m.n_elem):
        a, b = int(m.enr_ptr[e]), int(m.enr_ptr[e + 1])
        if b > a and np.all(m.enr_type[a:b] == am.ENR_HEAVISIDE):
            out.append(e)
    return np.array(out, np.int64)


def corners(d, m, elems):
    """Corner coordinates [n, 6] at reference (0,1), (0,0), (1,0): the first
    three nodes of a 3-node triangle, nodes 0, 2, 4 of a 6-node one."""
    xy = d["elem_xy"].reshape(m.n_elem, -1)
    out = np.zeros((len(elems), 6))
    for i, e in enumerate(elems):
        idx = (0, 1, 2) if m.kind[e] == am.TRI3 else (0, 2, 4)
        out[i] = np.concatenate([xy[e, 2 * k:2 * k + 2] for k in idx])
    return out


def submesh(m, elems, count, rule, h_point, h_vertex):
    """MeshData of `elems` integrated with the generated rules; the Heaviside
    function of corner k takes the jump h_point - h_vertex[k] at each point."""
    kind, dof_ptr, dof_ids, gp_ptr, gp, jinv, mat, scale = [], [0], [], [0], [], [], [], []
    enr_ptr, enr_vertex, enr_data, enr_jump = [0], [], [], []
    for i, e in enumerate(elems):
        n = int(count[i])
        kind.append(m.kind[e])
        dof_ids.extend(m.dof_ids[m.dof_ptr[e]:m.dof_ptr[e + 1]])
        dof_ptr.append(len(dof_ids))
        gp.extend(rule[i, :n].reshape(-1))
        gp_ptr.append(gp_ptr[-1] + n)
        jinv.extend(m.jinv[4 * e:4 * e + 4])
        mat.append(m.mat[e])
        scale.append(m.scale[e] if m.scale is not None else 1.0)
        for j in range(int(m.enr_ptr[e]), int(m.enr_ptr[e + 1])):
            k = int(m.enr_vertex[j])
            enr_vertex.append(k)
            enr_data.append(len(enr_jump))
            enr_jump.extend(int(h) - int(h_vertex[i, k]) for h in h_point[i, :n])
        enr_ptr.append(len(enr_vertex))
    sub = am.MeshData(dim=2, stride=2, kind=kind, dof_ptr=dof_ptr, dof_ids=dof_ids, gp_ptr=gp_ptr, gp=gp, jinv=jinv,
                      mat=mat, cmat_table=m.cmat_table, ndofmax=m.ndofmax, scale=np.array(scale),
                      enr_ptr=enr_ptr, enr_type=np.full(len(enr_vertex), am.ENR_HEAVISIDE, np.uint8),
                      enr_vertex=enr_vertex, enr_data=enr_data, enr_jump=np.array(enr_jump, np.int8),
                      enr_grad=np.zeros(2 * len(enr_jump)))
    sub.validate()
    return sub


def golden_ke(d, e):
    kp = d["ke_ptr"]
    return d["ke"][kp[e]:kp[e + 1]]
