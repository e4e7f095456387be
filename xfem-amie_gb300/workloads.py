"""Seeded synthetic workloads with the shapes, sizes and value distributions of
the benchmark configurations, in the element-data format of ``MeshData``.

The reference builds these problems with its Delaunay mesher and feature
tree; here a structured triangulation (or AMIE's own 6-tetrahedra voxel split)
stands in for the mesher, with every per-element quantity the hot path
consumes built the way the reference defines it:

* node ids in lattice order, DOF ids = node ids then enrichment ids
  (elements/elements.cpp:204, features/features.cpp:3275);
* local node order of TriElement LINEAR / QUADRATIC (elements/elements.cpp:976-1060):
  v0 at (0,1), v1 at (0,0), v2 at (1,0), mid-nodes between them;
* inverse Jacobian of the element (elements/integrable_entity.cpp:641-740);
* materials from seeded non-overlapping circular inclusions (random sequential
  addition, utilities/placement.cpp:87), C from Tensor::cauchyGreen plane
  stress (utilities/tensor.cpp:1845: C00 = E/(1-nu^2), C01 = nu C00, C22 = (1-nu) C00);
* a straight crack: Heaviside enrichment N_k^{P1} (H - H_k) on cut elements and
  their neighbours (features/crack.cpp:1215-1414) with sub-triangulated Gauss
  points (4 points per quadratic sub-triangle, mesher/delaunay.cpp:2909-2940),
  and tip branch functions sqrt(r){sin t/2, cos t/2, sin t/2 sin t, cos t/2 sin t}
  times N_k^{P1} (features/crack.cpp:919-960) on the tip element, integrated with
  512 seeded random points as the reference's Monte-Carlo fallback does
  (mesher/delaunay.cpp:2941-2949), passed as AMIE_ENR_TIP records (closed form
  on the device) or as tabulated gradients;
* Dirichlet multipliers of BoundingBoxDefinedBoundaryCondition on the box faces.
"""
from __future__ import annotations

import numpy as np

import amie_mesh as am

# P2 4-point rule of TriElement::genGaussPoints (elements/elements.cpp:684-689).
P2_PTS = np.array([[0.2, 0.2], [0.6, 0.2], [0.2, 0.6], [0.33333333333333, 0.33333333333333]])
P2_W = np.array([0.260416666666667, 0.260416666666667, 0.260416666666667, -0.28125])


def plane_stress(E: float, nu: float) -> np.ndarray:
    c = E / (1 - nu * nu)
    return np.array([[c, nu * c, 0], [nu * c, c, 0], [0, 0, (1 - nu) * c]], np.float64)


def isotropic_3d(E: float, nu: float) -> np.ndarray:
    lam = E * nu / ((1 + nu) * (1 - 2 * nu))
    mu = E / (2 * (1 + nu))
    C = np.zeros((6, 6))
    C[:3, :3] = lam
    C[[0, 1, 2], [0, 1, 2]] = lam + 2 * mu
    C[[3, 4, 5], [3, 4, 5]] = mu
    return C


def powerlaw_radii(rng, n, rmin, rmax, exponent):
    """Inverse-CDF samples of p(r) ~ r^exponent on [rmin, rmax]."""
    a = exponent + 1.0
    u = rng.random(n)
    return (rmin ** a + u * (rmax ** a - rmin ** a)) ** (1.0 / a)


def place_inclusions(rng, radii, L, min_dist=1e-5, tries=200):
    """Random sequential addition of non-overlapping circles in [0, L]^2, largest first."""
    radii = np.sort(radii)[::-1]
    cx = np.zeros(len(radii))
    cy = np.zeros(len(radii))
    cr = np.zeros(len(radii))
    k = 0
    for r in radii:
        for _ in range(tries):
            x, y = rng.uniform(r, L - r, 2)
            if k == 0 or np.all((cx[:k] - x) ** 2 + (cy[:k] - y) ** 2 > (cr[:k] + r + min_dist) ** 2):
                cx[k], cy[k], cr[k] = x, y, r
                k += 1
                break
    return cx[:k], cy[:k], cr[:k]


def _in_inclusions(px, py, cx, cy, cr, h, nx):
    """Mask of points inside any circle; points lie on a structured grid of pitch h."""
    inside = np.zeros(len(px), bool)
    # bucket points by grid cell for per-circle local tests
    ix = np.clip((px / h).astype(np.int64), 0, nx - 1)
    iy = np.clip((py / h).astype(np.int64), 0, nx - 1)
    order = np.lexsort((ix, iy))
    key = iy[order] * nx + ix[order]
    for x, y, r in zip(cx, cy, cr):
        i0, i1 = max(int((x - r) / h) - 1, 0), min(int((x + r) / h) + 1, nx - 1)
        j0, j1 = max(int((y - r) / h) - 1, 0), min(int((y + r) / h) + 1, nx - 1)
        for j in range(j0, j1 + 1):
            a = np.searchsorted(key, j * nx + i0)
            b = np.searchsorted(key, j * nx + i1, side="right")
            idx = order[a:b]
            inside[idx] |= (px[idx] - x) ** 2 + (py[idx] - y) ** 2 < r * r
    return inside


def _tri_jinv(X, Y):
    """Inverse Jacobians (n,2,2) of P1 triangles with vertex arrays (n,3): J rows d/dxi, d/deta."""
    J = np.empty((len(X), 2, 2))
    J[:, 0, 0] = X[:, 2] - X[:, 1]
    J[:, 0, 1] = Y[:, 2] - Y[:, 1]
    J[:, 1, 0] = X[:, 0] - X[:, 1]
    J[:, 1, 1] = Y[:, 0] - Y[:, 1]
    return np.linalg.inv(J), np.linalg.det(J)


def structured_triangles(N, L, order, jitter, rng):
    """Triangulated N x N square grid on [0, L]^2.

    Returns node coordinates (lattice order), element node ids in local order,
    vertex coordinates per element (n,3) and lattice size.
    """
    h = L / N
    M = N * order + 1                       # lattice points per side
    I, J = np.meshgrid(np.arange(M), np.arange(M), indexing="xy")
    x = (I * (h / order)).astype(np.float64).ravel()
    y = (J * (h / order)).astype(np.float64).ravel()
    lid = lambda i, j: j * M + i            # noqa: E731
    # jitter interior vertices (lattice points with both indices multiple of order)
    vi = (I % order == 0) & (J % order == 0) & (I > 0) & (J > 0) & (I < M - 1) & (J < M - 1)
    vi = vi.ravel()
    if jitter > 0:
        x[vi] += rng.uniform(-jitter, jitter, vi.sum()) * h
        y[vi] += rng.uniform(-jitter, jitter, vi.sum()) * h
    ci, cj = np.meshgrid(np.arange(N), np.arange(N), indexing="xy")
    ci, cj = ci.ravel(), cj.ravel()
    o = order
    a = lid(o * ci, o * cj)
    b = lid(o * ci + o, o * cj)
    c = lid(o * ci + o, o * cj + o)
    d = lid(o * ci, o * cj + o)
    # T1 = (v0=c, v1=a, v2=b), T2 = (v0=d, v1=a, v2=c): counter-clockwise v1 -> v2 -> v0
    v0 = np.concatenate([c, d])
    v1 = np.concatenate([a, a])
    v2 = np.concatenate([b, c])
    if order == 1:
        conn = np.stack([v0, v1, v2], 1)
    else:
        # mid-nodes: v0-v1, v1-v2, v2-v0 (lattice midpoints), straight edges
        def mid(p, q):
            return ((p % M + q % M) // 2) + ((p // M + q // M) // 2) * M
        conn = np.stack([v0, mid(v0, v1), v1, mid(v1, v2), v2, mid(v2, v0)], 1)
        mids = conn[:, [1, 3, 5]].ravel()
        ends = np.stack([conn[:, [0, 2, 4]], conn[:, [2, 4, 0]]], 0)
        ends = ends.transpose(1, 2, 0).reshape(-1, 2)
        x[mids] = 0.5 * (x[ends[:, 0]] + x[ends[:, 1]])
        y[mids] = 0.5 * (y[ends[:, 0]] + y[ends[:, 1]])
    vx = np.stack([x[v0], x[v1], x[v2]], 1)
    vy = np.stack([y[v0], y[v1], y[v2]], 1)
    return x, y, conn.astype(np.uint32), vx, vy, M


def _box_bcs(x, y, L, stride, disp, tol=1e-12):
    """FIX_ALONG_XI / FIX_ALONG_ETA on BOTTOM, SET_ALONG_ETA = disp on TOP."""
    bottom = np.nonzero(np.abs(y) < tol * max(L, 1))[0]
    top = np.nonzero(np.abs(y - L) < tol * max(L, 1))[0]
    ids = np.concatenate([bottom * stride, bottom * stride + 1, top * stride + 1]).astype(np.uint32)
    vals = np.concatenate([np.zeros(2 * len(bottom)), np.full(len(top), disp)])
    order = np.argsort(ids)
    return ids[order], vals[order], np.zeros(len(ids), np.uint8)


def _sub_tri_points(sub_local, n_ref=P2_PTS, w_ref=P2_W):
    """Gauss points of the 4-point rule on each local-coordinate sub-triangle (k,3,2)."""
    pts, wts = [], []
    for tri in sub_local:
        a, b, c = tri
        area2 = abs((b[0] - a[0]) * (c[1] - a[1]) - (c[0] - a[0]) * (b[1] - a[1]))
        p = a + np.outer(n_ref[:, 0], b - a) + np.outer(n_ref[:, 1], c - a)
        pts.append(p)
        wts.append(w_ref * area2)
    return np.concatenate(pts), np.concatenate(wts)


def _to_local(X, Y, Jinv, px, py):
    """Local (xi, eta) of physical points in a P1 triangle with vertex arrays X, Y (len 3)."""
    dx, dy = px - X[1], py - Y[1]
    # [xi, eta] = J^-T [dx, dy] with x = x1 + xi (x2-x1) + eta (x0-x1)
    xi = Jinv[0, 0] * dx + Jinv[1, 0] * dy
    eta = Jinv[0, 1] * dx + Jinv[1, 1] * dy
    return xi, eta


def _split_triangle_by_line(P, y0):
    """Sub-triangles of triangle P (3,2) cut by the horizontal line y = y0."""
    above = P[:, 1] > y0
    if above.all() or (~above).all():
        return [P]
    lone = np.nonzero(above)[0] if above.sum() == 1 else np.nonzero(~above)[0]
    k = int(lone[0])
    a, b, c = P[k], P[(k + 1) % 3], P[(k + 2) % 3]
    t1 = (y0 - a[1]) / (b[1] - a[1])
    t2 = (y0 - a[1]) / (c[1] - a[1])
    p1 = a + t1 * (b - a)
    p2 = a + t2 * (c - a)
    return [np.array([a, p1, p2]), np.array([p1, b, c]), np.array([p1, c, p2])]


def cracked_square(N, L=0.1, order=2, n_inclusions=4000, E_matrix=25e9, E_inc=60e9, nu=0.2, rmin=1e-4,
                   rmax=2e-3, exponent=-2.5, crack_frac=0.3, disp=1e-5, seed=1, jitter=0.15, tip=True,
                   n_mc=512, tip_closed_form=True):
    """Config-1 family: P2 (or P1) square with power-law inclusions and a straight crack.
    The tip element's branch functions are AMIE_ENR_TIP records (evaluated with
    their exact gradients on the device, angle 0 at the crack's end xb), or, with
    tip_closed_form=False, gradients tabulated per Gauss point."""
    rng = np.random.default_rng(seed)
    x, y, conn, vx, vy, M = structured_triangles(N, L, order, jitter, rng)
    E_count = len(conn)
    h = L / N
    cx = cy = cr = np.zeros(0)
    if n_inclusions:
        radii = powerlaw_radii(rng, n_inclusions, rmin, rmax, exponent)
        cx, cy, cr = place_inclusions(rng, radii, L)
    gx, gy = vx.mean(1), vy.mean(1)
    mat = _in_inclusions(gx, gy, cx, cy, cr, h, N).astype(np.uint32)
    cmat = np.stack([plane_stress(E_matrix, nu), plane_stress(E_inc, nu)]).reshape(-1)
    Jinv, detJ = _tri_jinv(vx, vy)
    nshape = 3 if order == 1 else 6
    kind = np.full(E_count, am.TRI3 if order == 1 else am.TRI6, np.uint8)

    # ---- crack: edge crack along y = y0 from x = 0 to xb (y0 seeded, off the lattice lines).
    # H is the ray-crossing parity of PositionOperation (polynomial/vm_token.cpp:258-275) seen
    # from far above: -1 in the shadow below the crack (y < y0, x <= xb), +1 elsewhere.
    y0 = L * (0.35 + 0.3 * rng.random())
    y0 = (np.floor(y0 / h) + 0.37) * h
    xb = crack_frac * L
    H = lambda xx, yy: np.where((yy < y0) & (xx <= xb), -1, 1)  # noqa: E731
    ymin, ymax = vy.min(1), vy.max(1)
    xmin, xmax = vx.min(1), vx.max(1)
    cut = np.nonzero((ymin < y0) & (ymax > y0) & (xmin < xb))[0]
    tip_elem = cut[np.argmin(np.abs(gx[cut] - xb) + (xmax[cut] < xb) * 1e9)] if tip and len(cut) else -1
    vert_ids = conn[:, [0, 2, 4]] if order == 2 else conn
    enriched_nodes = np.unique(vert_ids[cut].ravel())
    n_nodes = len(x)
    heav_id = {int(nid): n_nodes + i for i, nid in enumerate(enriched_nodes)}
    next_id = n_nodes + len(enriched_nodes)
    tip_ids = {}
    if tip_elem >= 0:
        for k in range(3):
            tip_ids[int(vert_ids[tip_elem, k])] = next_id
            next_id += 4
    # blending neighbours: elements sharing an enriched vertex but not cut
    has_enr = np.isin(vert_ids, enriched_nodes)
    blend = np.nonzero(has_enr.any(1))[0]
    enr_elems = np.union1d(cut, blend)

    dof_lists = [None] * E_count
    gp_lists = [None] * E_count
    enr_functions = {}   # e -> list of (type, vertex, jumps or grads)
    cut_set = set(cut.tolist())
    for e in enr_elems:
        e = int(e)
        P = np.stack([vx[e], vy[e]], 1)
        Ji = Jinv[e]
        if e == tip_elem:
            # Monte-Carlo fallback: n_mc uniform points, equal weights (mesher/delaunay.cpp:2941-2949)
            u = rng.random((n_mc, 2))
            flip = u.sum(1) > 1
            u[flip] = 1 - u[flip]
            pts = u
            wts = np.full(n_mc, 0.5 / n_mc) * detJ[e]
        elif e in cut_set:
            subs = _split_triangle_by_line(P, y0)
            loc = []
            for s in subs:
                xi, eta = _to_local(vx[e], vy[e], Ji, s[:, 0], s[:, 1])
                loc.append(np.stack([xi, eta], 1))
            pts, wts = _sub_tri_points(loc)
            wts = wts * detJ[e]
        else:
            pts, wts = None, None
        funcs = []
        if pts is not None:
            gpx = vx[e, 1] + pts[:, 0] * (vx[e, 2] - vx[e, 1]) + pts[:, 1] * (vx[e, 0] - vx[e, 1])
            gpy = vy[e, 1] + pts[:, 0] * (vy[e, 2] - vy[e, 1]) + pts[:, 1] * (vy[e, 0] - vy[e, 1])
            Hg = H(gpx, gpy)
        else:
            # an element the crack does not cut lies on one side of it: H is its centroid's
            # value at every Gauss point of the element's default rule
            n_rule = 4 if order == 2 else 1
            Hg = np.full(n_rule, int(H(np.array([gx[e]]), np.array([gy[e]]))[0]))
        ids = list(conn[e])
        for k in range(3):
            nid = int(vert_ids[e, k])
            if nid in heav_id:
                jumps = (Hg - H(x[nid], y[nid])).astype(np.int8)
                funcs.append((am.ENR_HEAVISIDE, k, jumps))
                ids.append(heav_id[nid])
        if e == tip_elem and tip_closed_form:
            corners = [(x[int(vert_ids[e, k])], y[int(vert_ids[e, k])]) for k in range(3)]
            for k in range(3):
                nid = int(vert_ids[e, k])
                for fi in range(4):
                    funcs.append((am.ENR_TIP, k, am.tip_record(corners[0], corners[1], corners[2], (xb, y0), 0.0, fi)))
                    ids.append(tip_ids[nid] + fi)
        elif e == tip_elem:
            Nk = [pts[:, 1], 1 - pts[:, 0] - pts[:, 1], pts[:, 0]]
            dN = [(0.0, 1.0), (-1.0, -1.0), (1.0, 0.0)]
            rx, ry = gpx - xb, gpy - y0
            r = np.sqrt(rx * rx + ry * ry)
            th = np.arctan2(ry, rx)
            sr = np.sqrt(r)
            # branch functions and their physical gradients
            s2, c2, s1, c1 = np.sin(th / 2), np.cos(th / 2), np.sin(th), np.cos(th)
            F = [sr * s2, sr * c2, sr * s2 * s1, sr * c2 * s1]
            dr = (rx / r, ry / r)
            dth = (-ry / (r * r), rx / (r * r))
            dsr = (0.5 / sr * dr[0], 0.5 / sr * dr[1])

            def grad(fi):
                g = []
                for c_ in range(2):
                    if fi == 0:
                        g.append(dsr[c_] * s2 + sr * 0.5 * c2 * dth[c_])
                    elif fi == 1:
                        g.append(dsr[c_] * c2 - sr * 0.5 * s2 * dth[c_])
                    elif fi == 2:
                        g.append(dsr[c_] * s2 * s1 + sr * (0.5 * c2 * s1 + s2 * c1) * dth[c_])
                    else:
                        g.append(dsr[c_] * c2 * s1 + sr * (-0.5 * s2 * s1 + c2 * c1) * dth[c_])
                return g
            J = np.linalg.inv(Ji)    # rows: d(x,y)/dxi, d(x,y)/deta
            for k in range(3):
                nid = int(vert_ids[e, k])
                xk, yk = x[nid] - xb, y[nid] - y0
                rk, tk = np.hypot(xk, yk), np.arctan2(yk, xk)
                Fk = [np.sqrt(rk) * np.sin(tk / 2), np.sqrt(rk) * np.cos(tk / 2),
                      np.sqrt(rk) * np.sin(tk / 2) * np.sin(tk), np.sqrt(rk) * np.cos(tk / 2) * np.sin(tk)]
                for fi in range(4):
                    gphys = grad(fi)
                    # local gradient: d/dxi = dx/dxi d/dx + dy/dxi d/dy
                    gxi = J[0, 0] * gphys[0] + J[0, 1] * gphys[1]
                    geta = J[1, 0] * gphys[0] + J[1, 1] * gphys[1]
                    f = F[fi] - Fk[fi]
                    dxi = dN[k][0] * f + Nk[k] * gxi
                    deta = dN[k][1] * f + Nk[k] * geta
                    funcs.append((am.ENR_TABULATED, k, np.stack([dxi, deta], 1).ravel()))
                    ids.append(tip_ids[nid] + fi)
        dof_lists[e] = ids
        gp_lists[e] = (pts, wts)
        enr_functions[e] = funcs

    # ---- flatten
    nf = np.full(E_count, nshape, np.int64)
    for e, funcs in enr_functions.items():
        nf[e] += len(funcs)
    dof_ptr = np.zeros(E_count + 1, np.uint32)
    np.cumsum(nf, out=dof_ptr[1:])
    dof_ids = np.empty(int(dof_ptr[-1]), np.uint32)
    base = conn.astype(np.uint32)
    simple = np.ones(E_count, bool)
    simple[list(enr_functions.keys())] = False
    # unenriched elements: contiguous copy
    starts = dof_ptr[:-1].astype(np.int64)
    idx = starts[simple][:, None] + np.arange(nshape)[None, :]
    dof_ids[idx.ravel()] = base[simple].ravel()
    ngp = np.zeros(E_count, np.int64)
    for e in enr_functions:
        dof_ids[dof_ptr[e]:dof_ptr[e + 1]] = dof_lists[e]
        if gp_lists[e][0] is not None:
            ngp[e] = len(gp_lists[e][1])
    gp_ptr = np.zeros(E_count + 1, np.uint32)
    np.cumsum(ngp, out=gp_ptr[1:])
    gp = np.zeros(int(gp_ptr[-1]) * 3)
    enr_ptr = np.zeros(E_count + 1, np.uint32)
    ne = np.zeros(E_count, np.int64)
    for e, funcs in enr_functions.items():
        ne[e] = len(funcs)
    np.cumsum(ne, out=enr_ptr[1:])
    n_enr = int(enr_ptr[-1])
    enr_type = np.zeros(n_enr, np.uint8)
    enr_vertex = np.zeros(n_enr, np.uint8)
    enr_data = np.zeros(n_enr, np.uint32)
    jumps_all, grads_all, tip_recs = [], [], []
    cursor = 0
    for e in sorted(enr_functions):
        pts, wts = gp_lists[e]
        if pts is not None:
            g0 = int(gp_ptr[e])
            blk = np.concatenate([pts, wts[:, None]], 1)
            gp[g0 * 3:(g0 + len(wts)) * 3] = blk.ravel()
            n_g = len(wts)
        else:
            n_g = 4 if order == 2 else 1
        for j, (typ, k, data) in enumerate(enr_functions[e]):
            fj = int(enr_ptr[e]) + j
            enr_type[fj] = typ
            enr_vertex[fj] = k
            if typ == am.ENR_TIP:   # a record, no per-point data
                enr_data[fj] = len(tip_recs)
                tip_recs.append(data)
                continue
            enr_data[fj] = cursor
            if typ == am.ENR_HEAVISIDE:
                jumps_all.append(data.astype(np.int8))
                grads_all.append(np.zeros(2 * n_g))
            else:
                jumps_all.append(np.zeros(n_g, np.int8))
                grads_all.append(data)
            cursor += n_g
    enr_jump = np.concatenate(jumps_all) if jumps_all else np.zeros(0, np.int8)
    enr_grad = np.concatenate(grads_all) if grads_all else np.zeros(0)
    m = am.MeshData(dim=2, stride=2, kind=kind, dof_ptr=dof_ptr, dof_ids=dof_ids, gp_ptr=gp_ptr, gp=gp,
                    jinv=Jinv.reshape(-1), mat=mat, cmat_table=cmat, ndofmax=next_id, enr_ptr=enr_ptr,
                    enr_type=enr_type, enr_vertex=enr_vertex, enr_data=enr_data, enr_jump=enr_jump,
                    enr_grad=enr_grad, enr_tip=np.concatenate(tip_recs) if tip_recs else None)
    bcs = _box_bcs(x, y, L, 2, disp)
    meta = dict(n_nodes=n_nodes, n_elem=E_count, n_inclusions=len(cr), n_cut=len(cut), n_enriched=len(enr_elems),
                tip_elem=int(tip_elem), crack_y=y0, n_dof=2 * next_id, order=order)
    return m, bcs, meta


def inclusion_square(N, L=0.04, order=1, n_inclusions=300, E_matrix=30e9, E_inc=60e9, nu=0.2, rmin=0.3e-3,
                     rmax=1.5e-3, disp=1e-5, seed=1, jitter=0.15, uniform=True, fraction=None):
    """Config-0 family: square with uniform-radius inclusions (or a target area fraction), no crack."""
    rng = np.random.default_rng(seed)
    x, y, conn, vx, vy, M = structured_triangles(N, L, order, jitter, rng)
    h = L / N
    if fraction is not None:
        # draw radii until the target area fraction is reached
        radii = []
        area = 0.0
        while area < fraction * L * L and len(radii) < 100000:
            r = rng.uniform(rmin, rmax)
            radii.append(r)
            area += np.pi * r * r
        radii = np.array(radii)
    else:
        radii = rng.uniform(rmin, rmax, n_inclusions)
    cx, cy, cr = place_inclusions(rng, radii, L)
    gx, gy = vx.mean(1), vy.mean(1)
    mat = _in_inclusions(gx, gy, cx, cy, cr, h, N).astype(np.uint32)
    cmat = np.stack([plane_stress(E_matrix, nu), plane_stress(E_inc, nu)]).reshape(-1)
    Jinv, _ = _tri_jinv(vx, vy)
    nshape = conn.shape[1]
    E_count = len(conn)
    kind = np.full(E_count, am.TRI3 if order == 1 else am.TRI6, np.uint8)
    dof_ptr = (np.arange(E_count + 1) * nshape).astype(np.uint32)
    m = am.MeshData(dim=2, stride=2, kind=kind, dof_ptr=dof_ptr, dof_ids=conn.ravel(),
                    gp_ptr=np.zeros(E_count + 1, np.uint32), gp=np.zeros(0), jinv=Jinv.reshape(-1), mat=mat,
                    cmat_table=cmat, ndofmax=len(x))
    bcs = _box_bcs(x, y, L, 2, disp)
    meta = dict(n_nodes=len(x), n_elem=E_count, n_inclusions=len(cr), n_dof=2 * len(x), order=order,
                fraction=float(np.pi * (cr ** 2).sum() / (L * L)))
    return m, bcs, meta


def _jinv_closed(X, Y):
    """Inverse Jacobians (n,2,2) of P1 triangles, as _tri_jinv, in closed form."""
    a = X[:, 2] - X[:, 1]
    b = Y[:, 2] - Y[:, 1]
    c = X[:, 0] - X[:, 1]
    d = Y[:, 0] - Y[:, 1]
    det = a * d - b * c
    inv = np.empty((len(X), 2, 2))
    inv[:, 0, 0] = d / det
    inv[:, 0, 1] = -b / det
    inv[:, 1, 0] = -c / det
    inv[:, 1, 1] = a / det
    return inv


def _place_inclusions_batched(rng, radii, L, min_dist=1e-5, tries=200):
    """Random sequential addition of non-overlapping circles in [0, L]^2, largest
    first, up to `tries` candidate positions each (as place_inclusions), the
    candidates drawn and tested in growing batches: the first candidate clear
    of every placed circle wins."""
    radii = np.sort(radii)[::-1]
    cx = np.zeros(len(radii))
    cy = np.zeros(len(radii))
    cr = np.zeros(len(radii))
    k = 0
    for r in radii:
        left = tries
        for batch in (4, 16, 64):
            nb = min(batch, left)
            left -= nb
            cand = rng.uniform(r, L - r, (nb, 2))
            if k == 0:
                j = 0
            else:
                dx = cand[:, :1] - cx[None, :k]
                dy = cand[:, 1:] - cy[None, :k]
                ok = np.flatnonzero(((dx * dx + dy * dy) > (cr[None, :k] + r + min_dist) ** 2).all(1))
                if ok.size == 0:
                    if left == 0:
                        break
                    continue
                j = ok[0]
            cx[k], cy[k], cr[k] = cand[j, 0], cand[j, 1], r
            k += 1
            break
    return cx[:k], cy[:k], cr[:k]


def _in_circles_structured(gx, gy, N, h, cx, cy, cr):
    """Inclusion mask of the 2 N^2 triangles of structured_triangles(N, order=1)
    from their centroids: each circle tests the triangles of the grid cells its
    bounding box (plus one cell) covers."""
    if len(cx) == 0:
        return np.zeros(len(gx), bool)
    i0 = np.clip(np.floor((cx - cr) / h).astype(np.int64) - 1, 0, N - 1)
    i1 = np.clip(np.floor((cx + cr) / h).astype(np.int64) + 1, 0, N - 1)
    j0 = np.clip(np.floor((cy - cr) / h).astype(np.int64) - 1, 0, N - 1)
    j1 = np.clip(np.floor((cy + cr) / h).astype(np.int64) + 1, 0, N - 1)
    ni = i1 - i0 + 1
    cnt = ni * (j1 - j0 + 1)
    circ = np.repeat(np.arange(len(cx)), cnt)
    off = np.arange(int(cnt.sum())) - np.repeat(np.cumsum(cnt) - cnt, cnt)
    cell = (j0[circ] + off // ni[circ]) * N + i0[circ] + off % ni[circ]
    inside = np.zeros(len(gx), bool)
    for half in (0, N * N):   # the two triangles of each cell
        e = cell + half
        hit = (gx[e] - cx[circ]) ** 2 + (gy[e] - cy[circ]) ** 2 < cr[circ] ** 2
        inside[e[hit]] = True
    return inside


def homogenisation_request(target_dof, fraction, seed, L=0.04, strain=1e-4, E_matrix=30e9, E_inc=60e9, nu=0.2,
                           rmin=0.3e-3, rmax=1.5e-3, jitter=0.15):
    """Config-4 request: a config-0 style microstructure (P1 triangles on a
    jittered N x N grid, non-overlapping inclusions with radii U[rmin, rmax]
    drawn until the area fraction is reached) of about `target_dof` DOF, with
    the macro strain eps_yy imposed on the whole boundary (u_x = 0,
    u_y = strain * y).  Generated in a few milliseconds (batched placement and
    inclusion test, closed-form Jacobians), so that every request of a stream
    can carry its own microstructure."""
    rng = np.random.default_rng(seed)
    N = max(4, int(round(np.sqrt(target_dof / 2.0))) - 1)
    x, y, conn, vx, vy, M = structured_triangles(N, L, 1, jitter, rng)
    h = L / N
    radii = []
    area = 0.0
    while area < fraction * L * L and len(radii) < 100000:
        r = rng.uniform(rmin, rmax)
        radii.append(r)
        area += np.pi * r * r
    cx, cy, cr = _place_inclusions_batched(rng, np.array(radii), L)
    mat = _in_circles_structured(vx.mean(1), vy.mean(1), N, h, cx, cy, cr).astype(np.uint32)
    E_count = len(conn)
    m = am.MeshData(dim=2, stride=2, kind=np.full(E_count, am.TRI3, np.uint8),
                    dof_ptr=(np.arange(E_count + 1) * 3).astype(np.uint32), dof_ids=conn.ravel(),
                    gp_ptr=np.zeros(E_count + 1, np.uint32), gp=np.zeros(0), jinv=_jinv_closed(vx, vy).reshape(-1),
                    mat=mat, cmat_table=np.stack([plane_stress(E_matrix, nu), plane_stress(E_inc, nu)]).reshape(-1),
                    ndofmax=len(x))
    I, J = np.meshgrid(np.arange(M), np.arange(M), indexing="xy")
    I, J = I.ravel(), J.ravel()
    bnd = np.nonzero((I == 0) | (J == 0) | (I == M - 1) | (J == M - 1))[0]
    ids = np.concatenate([bnd * 2, bnd * 2 + 1]).astype(np.uint32)
    vals = np.concatenate([np.zeros(len(bnd)), strain * J[bnd] * h])
    order = np.argsort(ids)
    meta = dict(n_nodes=len(x), n_elem=E_count, n_inclusions=len(cr), n_dof=2 * len(x),
                fraction=float(np.pi * (cr ** 2).sum() / (L * L)))
    return m, (ids[order], vals[order], np.zeros(len(ids), np.uint8)), meta


def serving_mix(n_requests, rate, dof_min=2000, dof_max=200000, seed=7):
    """Config-4 arrival stream: Poisson arrivals at `rate` req/s, each request
    its own microstructure with log-uniform size in [dof_min, dof_max] and
    inclusion fraction U[0.2, 0.6].  Returns (specs, arrivals): specs[k] =
    (target_dof, fraction, seed) for serving_request; the meshes are built
    on demand (all of them at once would take gigabytes)."""
    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(np.log(dof_min), np.log(dof_max), n_requests))
    fracs = rng.uniform(0.2, 0.6, n_requests)
    arrivals = np.cumsum(rng.exponential(1.0 / rate, n_requests))
    specs = [(int(sz), float(f), seed * 100000 + k) for k, (sz, f) in enumerate(zip(sizes, fracs))]
    return specs, arrivals


def serving_request(spec):
    """The request of a serving_mix spec: (mesh, (ids, values, kinds))."""
    m, bcs, _ = homogenisation_request(*spec)
    return m, bcs


def notched_beam(nx=706, ny=176, Lx=0.4, Ly=0.1, notch_w=0.02, notch_h=0.002, E=35e9, nu=0.2, seed=3,
                 jitter=0.1, patch=0.02, support=0.02):
    """Config-3 family: 400 x 100 mm beam, P1 triangles, a 20 x 2 mm notch at the
    bottom of midspan (elements inside removed, as a VoidForm feature leaves them
    without stiffness; orphan nodes renumbered away), three-point bending on
    plates: the bottom nodes within `support` of either end fixed in y, the
    bottom-left corner also in x, and the top nodes of a `patch`-wide loading
    plate at midspan displaced downwards (the load of each step is a multiplier
    value; BoundingBoxAndRestriction conditions in the reference).  Plates rather
    than single nodes keep the strain at the supports finite, so damage starts
    at the notch.  meta["corners"]: the vertices of every element (n_elem x 6)
    for the damage setup; meta["notch_tip"]: (x, y) of the notch's top edge at
    midspan."""
    rng = np.random.default_rng(seed)
    hx, hy = Lx / nx, Ly / ny
    M = nx + 1
    I, J = np.meshgrid(np.arange(nx + 1), np.arange(ny + 1), indexing="xy")
    x = (I * hx).astype(np.float64).ravel()
    y = (J * hy).astype(np.float64).ravel()
    inner = ((I > 0) & (J > 0) & (I < nx) & (J < ny)).ravel()
    x[inner] += rng.uniform(-jitter, jitter, inner.sum()) * hx
    y[inner] += rng.uniform(-jitter, jitter, inner.sum()) * hy
    ci, cj = np.meshgrid(np.arange(nx), np.arange(ny), indexing="xy")
    ci, cj = ci.ravel(), cj.ravel()
    a = cj * M + ci
    b = a + 1
    c = a + M + 1
    d = a + M
    conn = np.concatenate([np.stack([c, a, b], 1), np.stack([d, a, c], 1)])
    cx = x[conn].mean(1)
    cy = y[conn].mean(1)
    keep = ~((np.abs(cx - Lx / 2) < notch_w / 2) & (cy < notch_h))
    conn = conn[keep]
    used = np.unique(conn)
    remap = np.full(len(x), -1, np.int64)
    remap[used] = np.arange(len(used))
    conn = remap[conn].astype(np.uint32)
    x, y = x[used], y[used]
    vx, vy = x[conn], y[conn]
    Jinv, _ = _tri_jinv(vx, vy)
    E_count = len(conn)
    m = am.MeshData(dim=2, stride=2, kind=np.full(E_count, am.TRI3, np.uint8),
                    dof_ptr=(np.arange(E_count + 1) * 3).astype(np.uint32), dof_ids=conn.ravel(),
                    gp_ptr=np.zeros(E_count + 1, np.uint32), gp=np.zeros(0), jinv=Jinv.reshape(-1),
                    mat=np.zeros(E_count, np.uint32), cmat_table=plane_stress(E, nu).reshape(-1), ndofmax=len(x))
    tol = 1e-12
    left = int(np.nonzero((np.abs(x) < tol) & (np.abs(y) < tol))[0][0])
    bottom = np.abs(y) < tol
    supports = np.nonzero(bottom & ((x <= support + tol) | (x >= Lx - support - tol)))[0]
    plate = np.nonzero((np.abs(y - Ly) < tol) & (np.abs(x - Lx / 2) <= patch / 2 + tol))[0]
    corners = np.stack([vx, vy], 2).reshape(E_count, 6)   # (x0, y0, x1, y1, x2, y2) per element
    meta = dict(n_nodes=len(x), n_elem=E_count, n_dof=2 * len(x), load_nodes=len(plate),
                support_nodes=len(supports), corners=corners, notch_tip=(Lx / 2, notch_h))
    fixed = sorted([2 * left] + (2 * supports + 1).tolist())
    loaded = set((2 * plate + 1).tolist())

    def bcs(deflection):
        ids = np.array(sorted(fixed + sorted(loaded)), np.uint32)
        vals = np.array([-deflection if int(i) in loaded else 0.0 for i in ids])
        return ids, vals, np.zeros(len(ids), np.uint8)
    return m, bcs, meta


def voxel_cube(nv=64, E_median=30e9, sigma_log=0.4, nu=0.2, strain=1e-4, seed=1, size=1e-4):
    """Config-2 family: n^3 voxels, 6 linear tetrahedra per voxel with the corner
    choice of VoxelFilter::read (filters/voxelfilter.cpp:352-400), lognormal E per
    element (through the per-element factor on C), uniaxial imposed strain."""
    rng = np.random.default_rng(seed)
    n1 = nv + 1
    i, j, k = np.meshgrid(np.arange(nv), np.arange(nv), np.arange(nv), indexing="ij")
    i, j, k = i.ravel(), j.ravel(), k.ravel()
    pid = lambda a, b, c: a * n1 * n1 + b * n1 + c   # noqa: E731  (points indexed i, j, k as the filter does)
    corner = [pid(i, j + 1, k), pid(i + 1, j + 1, k), pid(i, j + 1, k + 1), pid(i + 1, j + 1, k + 1),
              pid(i, j, k), pid(i + 1, j, k), pid(i, j, k + 1), pid(i + 1, j, k + 1)]
    tets = [(0, 1, 2, 4), (3, 5, 7, 6), (2, 3, 4, 6), (1, 2, 3, 4), (1, 3, 4, 5), (3, 4, 6, 5)]
    conn = np.stack([np.stack([corner[a], corner[b], corner[c], corner[d]], 1) for a, b, c, d in tets], 1)
    conn = conn.reshape(-1, 4).astype(np.uint32)
    g = np.arange(n1) * (size / nv)
    P = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3)
    X = P[conn]                                   # (E,4,3)
    # TET4 local order N0 = zeta, N1 = 1-x-y-z, N2 = xi, N3 = eta:
    # J rows: d/dxi = X2 - X1, d/deta = X3 - X1, d/dzeta = X0 - X1
    J = np.stack([X[:, 2] - X[:, 1], X[:, 3] - X[:, 1], X[:, 0] - X[:, 1]], 1)
    det = np.linalg.det(J)
    flip = det < 0
    if flip.any():   # keep positive orientation: swap nodes 2 and 3
        conn[flip] = conn[flip][:, [0, 1, 3, 2]]
        X = P[conn]
        J = np.stack([X[:, 2] - X[:, 1], X[:, 3] - X[:, 1], X[:, 0] - X[:, 1]], 1)
    Jinv = np.linalg.inv(J)
    E_count = len(conn)
    Ee = np.exp(np.log(E_median) + sigma_log * rng.standard_normal(E_count))
    m = am.MeshData(dim=3, stride=3, kind=np.full(E_count, am.TET4, np.uint8),
                    dof_ptr=(np.arange(E_count + 1) * 4).astype(np.uint32), dof_ids=conn.ravel(),
                    gp_ptr=np.zeros(E_count + 1, np.uint32), gp=np.zeros(0), jinv=Jinv.reshape(-1),
                    mat=np.zeros(E_count, np.uint32), cmat_table=isotropic_3d(1.0, nu).reshape(-1),
                    cscale=Ee, ndofmax=len(P))
    tol = 1e-9 * size
    left = np.nonzero(P[:, 0] < tol)[0]
    right = np.nonzero(P[:, 0] > size - tol)[0]
    bottom = np.nonzero(P[:, 1] < tol)[0]
    back = np.nonzero(P[:, 2] < tol)[0]
    ids = np.concatenate([left * 3, bottom * 3 + 1, back * 3 + 2, right * 3]).astype(np.uint32)
    vals = np.concatenate([np.zeros(len(left) + len(bottom) + len(back)), np.full(len(right), strain * size)])
    # a node on LEFT and RIGHT cannot happen; later multipliers replace earlier ones for the same id
    uniq, last = np.unique(ids[::-1], return_index=True)
    vals = vals[::-1][last]
    meta = dict(n_nodes=len(P), n_elem=E_count, n_dof=3 * len(P))
    return m, (uniq.astype(np.uint32), vals, np.zeros(len(uniq), np.uint8)), meta
