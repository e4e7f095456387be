"""ctypes binding of the CPU oracle (amie_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke`` and
by the CPU-baseline leg of ``bench.py`` -- never by the GPU library.

Functions take a ``MeshData`` (xfem-amie_gb300/amie_mesh.py) and numpy arrays
and return numpy arrays.  Matrices use AMIE's padded column-major block layout
(``row_size``, ``column_index``, ``array``) exactly as the reference's
CoordinateIndexedSparseMatrix stores them.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_port", "liboracle.so")

_lib = None


class _OracleMesh(C.Structure):
    _fields_ = [
        ("dim", C.c_int32), ("stride", C.c_int32), ("n_elem", C.c_uint32), ("ndofmax", C.c_uint32),
        ("kind", C.c_void_p), ("dof_ptr", C.c_void_p), ("dof_ids", C.c_void_p), ("gp_ptr", C.c_void_p),
        ("gp", C.c_void_p), ("jinv", C.c_void_p), ("moved", C.c_void_p), ("jinv_gp", C.c_void_p), ("mat", C.c_void_p), ("cmat_table", C.c_void_p),
        ("cscale", C.c_void_p), ("scale", C.c_void_p), ("enr_ptr", C.c_void_p), ("enr_type", C.c_void_p),
        ("enr_vertex", C.c_void_p), ("enr_data", C.c_void_p), ("enr_jump", C.c_void_p), ("enr_grad", C.c_void_p),
    ]


def build() -> str:
    """Compile liboracle.so (make -C oracle port)."""
    subprocess.run(["make", "-s", "-C", HERE, "port"], check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        _lib = C.CDLL(LIB_PATH)
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _mesh_struct(m):
    # tip branch functions enter the C oracle tabulated (with_tabulated_tips); the
    # converted mesh is kept on the struct so that its arrays outlive the call
    if getattr(m, "enr_tip", None) is not None and len(m.enr_tip):
        m = with_tabulated_tips(m)
    s = _OracleMesh(m.dim, m.stride, m.n_elem, m.ndofmax)
    for name in ("kind", "dof_ptr", "dof_ids", "gp_ptr", "gp", "jinv", "moved", "jinv_gp", "mat", "cmat_table", "cscale", "scale",
                 "enr_ptr", "enr_type", "enr_vertex", "enr_data", "enr_jump", "enr_grad"):
        setattr(s, name, _p(getattr(m, name)))
    s._keep = m
    return s


def threads() -> int:
    return int(lib().oracle_threads())


def element_matrices(m):
    off = m.ke_offsets()
    ke = np.zeros(int(off[-1]), np.float64)
    st = _mesh_struct(m)
    rc = lib().oracle_element_matrices(C.byref(st), _p(off), _p(ke))
    if rc != 0:
        raise RuntimeError(f"oracle_element_matrices failed: {rc}")
    return off, ke


def pattern(m):
    st = _mesh_struct(m)
    nr = C.c_uint32()
    nnz = C.c_uint64()
    lib().oracle_pattern(C.byref(st), C.byref(nr), C.byref(nnz), None, None)
    rs = np.zeros(nr.value, np.uint32)
    ci = np.zeros(nnz.value, np.uint32)
    lib().oracle_pattern(C.byref(st), C.byref(nr), C.byref(nnz), _p(rs), _p(ci))
    return rs, ci


def block_size(stride: int) -> int:
    return stride * (stride + stride % 2)


def scatter(m, off, ke, rs, ci):
    arr = np.zeros(len(ci) * block_size(m.stride), np.float64)
    st = _mesh_struct(m)
    rc = lib().oracle_scatter(C.byref(st), _p(off), _p(ke), C.c_uint32(len(rs)), _p(rs), _p(ci), _p(arr))
    if rc != 0:
        raise RuntimeError(f"oracle_scatter failed: {rc}")
    return arr


def dirichlet(stride, rs, ci, arr, ids, values, kinds, rhs):
    rc = lib().oracle_dirichlet(C.c_int32(stride), C.c_uint32(len(rs)), _p(rs), _p(ci), _p(arr),
                                C.c_uint32(len(ids)), _p(ids), _p(values), _p(kinds), _p(rhs))
    if rc != 0:
        raise RuntimeError(f"oracle_dirichlet failed: {rc}")


def spmv(stride, rs, ci, arr, x, y0=None):
    y = np.zeros(len(rs) * stride, np.float64)
    lib().oracle_spmv(C.c_int32(stride), C.c_uint32(len(rs)), _p(rs), _p(ci), _p(arr), _p(x), _p(y0), _p(y))
    return y


def cg_amie(stride, rs, ci, arr, b, x0=None, eps=1e-10, nssor=32, maxit=-1):
    x = np.zeros(len(rs) * stride) if x0 is None else np.array(x0, np.float64, copy=True)
    it = C.c_int64()
    rc = lib().oracle_cg_amie(C.c_int32(stride), C.c_uint32(len(rs)), _p(rs), _p(ci), _p(arr), _p(b), _p(x),
                              C.c_double(eps), C.c_int32(nssor), C.c_int64(maxit), C.byref(it))
    return x, int(it.value), int(rc)


def pcg(stride, rs, ci, arr, b, x0=None, rtol=1e-10, maxit=100000):
    x = np.zeros(len(rs) * stride) if x0 is None else np.array(x0, np.float64, copy=True)
    it = C.c_int64()
    rr = C.c_double()
    rc = lib().oracle_pcg(C.c_int32(stride), C.c_uint32(len(rs)), _p(rs), _p(ci), _p(arr), _p(b), _p(x),
                          C.c_double(rtol), C.c_int64(maxit), C.byref(it), C.byref(rr))
    return x, int(it.value), float(rr.value), int(rc)


def induced_forces(m, imposed, n):
    """Global force vector [n] of an imposed strain [n_elem, nv] (element order accumulation)."""
    f = np.zeros(n, np.float64)
    st = _mesh_struct(m)
    imp = np.ascontiguousarray(imposed, np.float64)
    rc = lib().oracle_induced_forces(C.byref(st), _p(imp), _p(f))
    if rc != 0:
        raise RuntimeError(f"oracle_induced_forces failed: {rc}")
    return f


def element_fields(m, u):
    """(strain, stress) per element, Voigt, from displacements u."""
    nv = m.nv
    eps = np.zeros(m.n_elem * nv)
    sig = np.zeros(m.n_elem * nv)
    st = _mesh_struct(m)
    u = np.ascontiguousarray(u, np.float64)
    lib().oracle_element_fields(C.byref(st), _p(u), _p(eps), _p(sig))
    return eps.reshape(-1, nv), sig.reshape(-1, nv)


def assemble(m, bc_ids, bc_values, bc_kinds, rhs0=None):
    """Full host pipeline: K_e -> pattern -> Kahan scatter -> Dirichlet."""
    off, ke = element_matrices(m)
    rs, ci = pattern(m)
    arr = scatter(m, off, ke, rs, ci)
    rhs = np.zeros(len(rs) * m.stride) if rhs0 is None else np.array(rhs0, np.float64, copy=True)
    dirichlet(m.stride, rs, ci, arr, np.ascontiguousarray(bc_ids, np.uint32),
              np.ascontiguousarray(bc_values, np.float64), np.ascontiguousarray(bc_kinds, np.uint8), rhs)
    return dict(off=off, ke=ke, row_size=rs, column_index=ci, array=arr, rhs=rhs)


# ---------------------------------------------------------------- damage (damage_oracle.cpp)

class DamageLaw(C.Structure):
    """NonLocalMazars + FiberBasedIsotropicLinearDamage parameters (oracle_damage_law)."""
    _fields_ = [(k, C.c_double) for k in ("threshold", "young", "poisson", "fracture_energy", "radius",
                                           "score_tolerance", "fibre", "cutoff", "residual")]


def damage_geometry(xy):
    """(centre [n,2], circumradius [n], area [n]) of triangles with corners xy [n,6]."""
    xy = np.ascontiguousarray(xy, np.float64).reshape(-1, 6)
    n = len(xy)
    c, r, a = np.zeros(2 * n), np.zeros(n), np.zeros(n)
    lib().oracle_damage_geometry(C.c_uint32(n), _p(xy), _p(c), _p(r), _p(a))
    return c.reshape(n, 2), r, a


def damage_cache(R, xy, centre, radius, area):
    """Smoothing caches (ptr, idx, coef) of every element."""
    xy = np.ascontiguousarray(xy, np.float64).reshape(-1, 6)
    n = len(xy)
    centre = np.ascontiguousarray(centre, np.float64)
    radius = np.ascontiguousarray(radius, np.float64)
    area = np.ascontiguousarray(area, np.float64)
    ptr = np.zeros(n + 1, np.uint64)
    lib().oracle_damage_cache(C.c_uint32(n), C.c_double(R), _p(xy), _p(centre), _p(radius), _p(area), _p(ptr),
                              None, None)
    idx = np.zeros(int(ptr[-1]), np.uint32)
    coef = np.zeros(int(ptr[-1]), np.float64)
    lib().oracle_damage_cache(C.c_uint32(n), C.c_double(R), _p(xy), _p(centre), _p(radius), _p(area), _p(ptr),
                              _p(idx), _p(coef))
    return ptr, idx, coef


def damage_grade(law, strain, cmat, state, area, gpw, cache):
    """(score [n], smoothed principal stress and strain [n,4])."""
    n = len(state)
    ptr, idx, coef = cache
    score = np.zeros(n)
    sm = np.zeros(4 * n)
    lib().oracle_damage_grade(C.c_uint32(n), C.byref(law), _p(np.ascontiguousarray(strain, np.float64)),
                              _p(np.ascontiguousarray(cmat, np.float64)), _p(np.ascontiguousarray(state, np.float64)),
                              _p(np.ascontiguousarray(area, np.float64)), _p(np.ascontiguousarray(gpw, np.float64)),
                              _p(ptr), _p(idx), _p(coef), _p(score), _p(sm))
    return score, sm.reshape(n, 4)


def damage_update(law, centre, radius, score, state):
    """FiberBasedIsotropicLinearDamage::step of every element; returns (new state, changed mask)."""
    st = np.array(state, np.float64, copy=True)
    ch = np.zeros(len(st), np.uint8)
    lib().oracle_damage_update(C.c_uint32(len(st)), C.byref(law), _p(np.ascontiguousarray(centre, np.float64)),
                               _p(np.ascontiguousarray(radius, np.float64)),
                               _p(np.ascontiguousarray(score, np.float64)), _p(st), _p(ch))
    return st, ch.astype(bool)


def tip_gradients(rec, vertex, xi, eta):
    """Local gradients (d/dxi, d/deta) of a tip branch function N_v (F_j(x) - F_j(x_v))
    at local points (xi, eta), restated from BranchedCrack::enrichTip
    (features/crack.cpp:898-960): F_j = sqrt(r) g_j(t), t = -atan2 of the position
    relative to the tip in the frame of the crack angle (the sign the reference's
    atan2 token gives), grad F = g_j grad r / (2 sqrt r) + sqrt(r) g_j'(t) grad t.
    rec: the 8 doubles of amie_mesh.tip_record."""
    xi = np.asarray(xi, float)
    eta = np.asarray(eta, float)
    a, j = rec[6], int(rec[7])

    def F(s0, s1, grad):
        dx = rec[0] + s0 * rec[2] + s1 * rec[4]
        dy = rec[1] + s0 * rec[3] + s1 * rec[5]
        r2 = dx * dx + dy * dy
        r = np.sqrt(r2)
        t = -np.arctan2(-np.sin(a) * dx + np.cos(a) * dy, np.cos(a) * dx + np.sin(a) * dy)
        s2, c2, st, ct = np.sin(t / 2), np.cos(t / 2), np.sin(t), np.cos(t)
        g = [s2, c2, s2 * st, c2 * st][j]
        if not grad:
            return np.sqrt(r) * g
        gp = [c2 / 2, -s2 / 2, c2 / 2 * st + s2 * ct, -s2 / 2 * st + c2 * ct][j]
        Fx = g / (2 * np.sqrt(r)) * dx / r + np.sqrt(r) * gp * dy / r2
        Fy = g / (2 * np.sqrt(r)) * dy / r - np.sqrt(r) * gp * dx / r2
        return np.sqrt(r) * g, Fx, Fy

    vx, vy = [(0.0, 1.0), (0.0, 0.0), (1.0, 0.0)][vertex]
    N = [eta, 1 - xi - eta, xi][vertex]
    dN = [(0.0, 1.0), (-1.0, -1.0), (1.0, 0.0)][vertex]
    Fg, Fx, Fy = F(xi, eta, True)
    dF = Fg - F(vx, vy, False)
    gxi = dN[0] * dF + N * (rec[2] * Fx + rec[3] * Fy)
    geta = dN[1] * dF + N * (rec[4] * Fx + rec[5] * Fy)
    return np.stack([gxi, geta], 1)


def with_tabulated_tips(m):
    """A copy of MeshData m whose tip branch functions (AMIE_ENR_TIP) are tabulated
    with the gradients of tip_gradients at their element's Gauss points (the
    oracle's element routines read tabulated gradients only)."""
    import copy
    import amie_mesh as am
    out = copy.copy(m)
    if m.enr_tip is None or not len(m.enr_tip):
        return out
    dim = m.dim
    grad = [m.enr_grad.reshape(-1, dim)]
    n_gp = len(m.enr_grad) // dim
    enr_type = m.enr_type.copy()
    enr_data = m.enr_data.copy()
    gp = m.gp.reshape(-1, dim + 1)
    for e in np.nonzero(np.diff(m.enr_ptr.astype(np.int64)))[0]:
        pts = gp[m.gp_ptr[e]:m.gp_ptr[e + 1], :dim]
        for f in range(m.enr_ptr[e], m.enr_ptr[e + 1]):
            if enr_type[f] != am.ENR_TIP:
                continue
            rec = m.enr_tip[8 * int(m.enr_data[f]):8 * int(m.enr_data[f]) + 8]
            grad.append(tip_gradients(rec, int(m.enr_vertex[f]), pts[:, 0], pts[:, 1]))
            enr_type[f] = am.ENR_TABULATED
            enr_data[f] = n_gp
            n_gp += len(pts)
    out.enr_type = enr_type
    out.enr_data = enr_data
    out.enr_grad = np.ascontiguousarray(np.concatenate(grad).reshape(-1))
    if len(out.enr_jump) < n_gp:
        out.enr_jump = np.concatenate([out.enr_jump, np.zeros(n_gp - len(out.enr_jump), np.int8)])
    out.enr_tip = None
    return out


def proportional(stride, rs, ci, arr, rhs, ids, offsets, ptr, prop_ids, coefs):
    """The SET_PROPORTIONAL_DISPLACEMENT branch of Assembly::setBoundaryConditions
    (solvers/assembly.cpp:279-318), restated entry by entry on AMIE's padded
    column-major block layout, in place: for each multiplier u_id = offset +
    sum c_k u_pk, in order, every other row j moves A_j,id onto A_j,pk and offset
    A_j,id onto f_j, the rows p_k take c_k times row id (and f_id), row id becomes
    a unit row with f_id = 0.  A missing entry reads as 0 and a write to it is
    dropped (SparseVector::operator[], sparse/sparse_vector.cpp:38-48)."""
    s = int(stride)
    cl = s + s % 2
    starts = np.concatenate([[0], np.cumsum(rs.astype(np.int64))])
    n = len(rs) * s

    def pos(i, j):
        row, cb = i // s, j // s
        a, b = int(starts[row]), int(starts[row + 1])
        k = int(np.searchsorted(ci[a:b], cb))
        if k < b - a and ci[a + k] == cb:
            return (a + k) * s * cl + (j % s) * cl + (i % s)
        return -1

    def get(i, j):
        p = pos(i, j)
        return arr[p] if p >= 0 else 0.0

    def add(i, j, v):
        p = pos(i, j)
        if p >= 0:
            arr[p] += v

    def put(i, j, v):
        p = pos(i, j)
        if p >= 0:
            arr[p] = v

    for m in range(len(ids)):
        i0, off = int(ids[m]), float(offsets[m])
        P = [int(q) for q in prop_ids[ptr[m]:ptr[m + 1]]]
        Cf = [float(c) for c in coefs[ptr[m]:ptr[m + 1]]]
        for j in range(n):
            if j == i0 or j in P:
                continue
            a = get(j, i0)
            rhs[j] -= off * a
            for p, c in zip(P, Cf):
                add(j, p, c * a)
            put(j, i0, 0.0)
        for p, c in zip(P, Cf):
            for j in range(n):
                add(p, j, c * get(i0, j))
            rhs[p] += c * rhs[i0]
            for p2, c2 in zip(P, Cf):
                add(p, p2, c2 * get(p, i0))
            rhs[p] -= off * get(p, i0)
            put(p, i0, 0.0)
        for j in range(n):
            put(i0, j, 1.0 if j == i0 else 0.0)
        rhs[i0] = 0.0


def proportional_solution(x, ids, offsets, ptr, prop_ids, coefs):
    """The proportional DOFs of a solution, in multiplier order (Assembly::cgsolve,
    solvers/assembly.cpp:1881-1892); in place."""
    for m in range(len(ids)):
        v = float(offsets[m])
        for k in range(int(ptr[m]), int(ptr[m + 1])):
            v += coefs[k] * x[prop_ids[k]]
        x[ids[m]] = v
