"""CPU restatement of the integration rules of crack-crossed triangles.

TEST INFRASTRUCTURE ONLY: the parity tests compare the device rules
(``amie_cut_rules``) with this module and pin this module against the
reference's fixtures; the GPU library never imports it.  Plain Python loops,
meant for the few hundred elements the tests use.

What it restates (paths relative to the AMIE source tree):

* the hints of an element: the points where the crack polyline crosses the
  element's edges and the polyline points inside it, in reference coordinates
  (BranchedCrack::enrichSegmentedLine, features/crack.cpp:1088-1175), after the
  corners (0,1), (0,0), (1,0) (DelaunayTriangle::getIntegrationHints,
  mesher/delaunay.cpp:2708-2723);
* DelaunayTriangle::getSubTriangulatedGaussPoints (mesher/delaunay.cpp:2895-2960):
  incremental Delaunay triangulation of the hints from the corner triangle,
  a hint dropped when it lies within 0.05 of a vertex of a triangle it
  conflicts with (DelaunayTree::insert, mesher/delaunay.cpp:2157-2196); fewer
  than three sub-triangles or a parent area off 0.5 by more than 1e-6 means
  the reference's 512 random points instead;
* the 4-point rule of TriPoint::getGaussPoints (geometry/geometry_base.cpp:5221-5245)
  on every sub-triangle, weights scaled to the element's area;
* the crack's Heaviside function, PositionOperation (polynomial/vm_token.cpp:242-271)
  with the witness of Segment::normal(const Point &) (geometry/geometry_base.cpp:4010-4022).

With REPLACE_MONTE_CARLO, elements the reference would integrate by
Monte-Carlo (or insertion-order dependently) are triangulated with no insertion
tolerance instead (status REPLACED).  `split_rule_degree4` is an independent
exact rule for a straight crossing (three crack-conforming pieces, Dunavant's
6-point degree-4 rule), used by the tests to check that the replaced rules
integrate exactly.
"""
from __future__ import annotations

import math

import numpy as np

MAX_HINTS = 6
MAX_POINTS = 52
OK, NOT_CUT, MONTE_CARLO, ORDER_DEPENDENT, TOO_MANY_HINTS, REPLACED = 0, 1, 2, 3, 4, 5
REPLACE_MONTE_CARLO = 1
INSERT_TOL = 0.05
FLAT = 1e-12
W_EDGE, W_CENTRE = 0.260416666666667, -0.28125
REF = ((0.0, 1.0), (0.0, 0.0), (1.0, 0.0))


def _orient(a, b, c):
    return (b[0] - a[0]) * (c[1] - a[1]) - (b[1] - a[1]) * (c[0] - a[0])


def _incircle(a, b, c, d):
    """> 0 when d is inside the circumcircle of the counter-clockwise a, b, c."""
    adx, ady = a[0] - d[0], a[1] - d[1]
    bdx, bdy = b[0] - d[0], b[1] - d[1]
    cdx, cdy = c[0] - d[0], c[1] - d[1]
    return ((adx * adx + ady * ady) * (bdx * cdy - cdx * bdy) - (bdx * bdx + bdy * bdy) * (adx * cdy - cdx * ady)
            + (cdx * cdx + cdy * cdy) * (adx * bdy - bdx * ady))


def witness(line):
    """Far point of PositionOperation: midpoint of the first segment + 10 x its
    unit normal pointing away from (-1000, -1000)."""
    (ax, ay), (bx, by) = line[0], line[1]
    vx, vy = bx - ax, by - ay
    nv = math.hypot(vx, vy)
    nx, ny = -vy / nv, vx / nv
    mx, my = 0.5 * (ax + bx), 0.5 * (ay + by)
    if (mx + 1000.0) * nx + (my + 1000.0) * ny <= 0.0:
        nx, ny = -nx, -ny
    return (mx + 10.0 * nx, my + 10.0 * ny)


def heaviside(p, line, w):
    """+1 when [p, w] crosses the polyline an odd number of times, else -1."""
    k = 0
    for s in range(len(line) - 1):
        a, b = line[s], line[s + 1]
        if _orient(a, b, p) * _orient(a, b, w) < 0.0 and _orient(p, w, a) * _orient(p, w, b) < 0.0:
            k += 1
    return 1 if k & 1 else -1


def _hints(X, line):
    hints = []
    for s in range(len(line) - 1):
        a, b = line[s], line[s + 1]
        for i in range(3):
            j = (i + 1) % 3
            fa, fb = _orient(a, b, X[i]), _orient(a, b, X[j])
            if fa * fb < 0.0 and _orient(X[i], X[j], a) * _orient(X[i], X[j], b) < 0.0:
                t = fa / (fa - fb)
                hints.append((REF[i][0] + t * (REF[j][0] - REF[i][0]), REF[i][1] + t * (REF[j][1] - REF[i][1])))
    a2 = _orient(X[0], X[1], X[2])
    for p in line:
        l0, l2 = _orient(p, X[1], X[2]) / a2, _orient(X[0], X[1], p) / a2
        if l0 > 0.0 and l2 > 0.0 and l0 + l2 < 1.0:
            hints.append((l2, l0))
    return hints


def _delaunay(V, n_hints, tol=INSERT_TOL):
    """Sub-triangles (vertex index triples, counter-clockwise) of the corner
    triangle after inserting V[3:] in order; a hint within `tol` of a vertex of
    a triangle it conflicts with is dropped."""
    tris = [(1, 2, 0)]
    for h in range(3, 3 + n_hints):
        p = V[h]
        con = [_incircle(V[t[0]], V[t[1]], V[t[2]], p) > 0.0 for t in tris]
        if any(c and min(math.dist(V[v], p) for v in t) < tol for c, t in zip(con, tris)):
            continue
        edges = {}
        for c, t in zip(con, tris):
            if not c:
                continue
            for k in range(3):
                u, v = t[k], t[(k + 1) % 3]
                if (v, u) in edges:
                    del edges[(v, u)]
                else:
                    edges[(u, v)] = True
        tris = [t for c, t in zip(con, tris) if not c]
        tris += [(u, v, h) for (u, v) in edges if _orient(V[u], V[v], p) > FLAT]
    return tris


def element_rule(corners, line, flags=0):
    """(status, [(xi, eta, weight, h), ...], [h at the three corners]) of one element."""
    X = [(corners[0], corners[1]), (corners[2], corners[3]), (corners[4], corners[5])]
    line = [tuple(p) for p in line]
    w = witness(line)
    hv = [heaviside(x, line, w) for x in X]
    hints = _hints(X, line)
    if len(hints) > MAX_HINTS:
        return TOO_MANY_HINTS, [], hv
    if not hints:
        return NOT_CUT, [], hv
    close = any(math.dist(hints[i], hints[j]) < INSERT_TOL for i in range(len(hints)) for j in range(i))
    V = list(REF) + hints
    status = ORDER_DEPENDENT if close else OK
    tris = [] if close else _delaunay(V, len(hints))
    if not close and len(tris) < 3:
        status = MONTE_CARLO
    if status != OK and flags & REPLACE_MONTE_CARLO:
        tris = _delaunay(V, len(hints), 0.0)
        status = REPLACED if len(tris) >= 3 else MONTE_CARLO
    if status not in (OK, REPLACED):
        return status, [], hv
    pts = []
    for t in tris:
        A, B, Cc = (V[v] for v in t)
        ar = abs(_orient(A, B, Cc))
        for r in range(3):
            lam = [0.2, 0.2, 0.2]
            lam[r] = 0.6
            pts.append((lam[0] * A[0] + lam[1] * B[0] + lam[2] * Cc[0], lam[0] * A[1] + lam[1] * B[1] + lam[2] * Cc[1],
                        W_EDGE * ar))
        pts.append(((A[0] + B[0] + Cc[0]) / 3.0, (A[1] + B[1] + Cc[1]) / 3.0, W_CENTRE * ar))
    parent = sum(p[2] for p in pts)
    if abs(parent - 0.5) > 1e-6:
        return MONTE_CARLO, [], hv
    scale = 0.5 * abs(_orient(X[0], X[1], X[2])) / parent
    out = []
    for xi, eta, wq in pts:
        z = 1.0 - xi - eta
        p = (eta * X[0][0] + z * X[1][0] + xi * X[2][0], eta * X[0][1] + z * X[1][1] + xi * X[2][1])
        out.append((xi, eta, wq * scale, heaviside(p, line, w)))
    return status, out, hv


def cut_rules(corners, line, flags=0):
    """Same outputs as amie_cut_rules: count [n], status [n], rule [n, 52, 3],
    h_point [n, 52], h_vertex [n, 3]."""
    c = np.asarray(corners, np.float64).reshape(-1, 6)
    ln = np.asarray(line, np.float64).reshape(-1, 2)
    n = len(c)
    count = np.zeros(n, np.uint32)
    status = np.zeros(n, np.int8)
    rule = np.zeros((n, MAX_POINTS, 3))
    hp = np.zeros((n, MAX_POINTS), np.int8)
    hv = np.zeros((n, 3), np.int8)
    for e in range(n):
        st, pts, h = element_rule(c[e], ln, flags)
        status[e] = st
        hv[e] = h
        count[e] = len(pts)
        for g, (xi, eta, wq, s) in enumerate(pts):
            rule[e, g] = (xi, eta, wq)
            hp[e, g] = s
    return count, status, rule, hp, hv


# Dunavant (1985), degree 4, positive weights: barycentric (a, b, b) and permutations
_DUN = ((0.108103018168070, 0.445948490915965, 0.223381589678011),
        (0.816847572980459, 0.091576213509771, 0.109951743655322))


def split_rule_degree4(corners, line):
    """Independent exact rule of an element crossed once by a straight piece of
    the crack (two edge crossings, no polyline point inside): the corner alone
    on its side with the two crossings, and the remaining quadrilateral as two
    triangles, each with Dunavant's 6-point rule; Heaviside by the same ray
    parity.  Returns [(xi, eta, weight, h), ...] or None when the element is not
    crossed that way."""
    X = [(corners[0], corners[1]), (corners[2], corners[3]), (corners[4], corners[5])]
    line = [tuple(p) for p in line]
    w = witness(line)
    hits = {}
    for s_ in range(len(line) - 1):
        a, b = line[s_], line[s_ + 1]
        for i in range(3):
            j = (i + 1) % 3
            fa, fb = _orient(a, b, X[i]), _orient(a, b, X[j])
            if fa * fb < 0.0 and _orient(X[i], X[j], a) * _orient(X[i], X[j], b) < 0.0:
                t = fa / (fa - fb)
                hits[(i, j)] = (REF[i][0] + t * (REF[j][0] - REF[i][0]), REF[i][1] + t * (REF[j][1] - REF[i][1]))
    if len(hits) != 2:
        return None
    (e1, p1), (e2, p2) = hits.items()
    lone = (set(e1) & set(e2)).pop()
    j1 = (set(e1) - {lone}).pop()
    j2 = (set(e2) - {lone}).pop()
    R = REF
    pieces = [(R[lone], p1, p2), (p1, R[j1], R[j2]), (p1, R[j2], p2)]
    area = 0.5 * abs(_orient(X[0], X[1], X[2]))
    out = []
    for A, B, Cc in pieces:
        ar = 0.5 * abs(_orient(A, B, Cc)) * area / 0.5
        for a_, b_, wt in _DUN:
            for r in range(3):
                lam = [b_, b_, b_]
                lam[r] = a_
                xi = lam[0] * A[0] + lam[1] * B[0] + lam[2] * Cc[0]
                eta = lam[0] * A[1] + lam[1] * B[1] + lam[2] * Cc[1]
                z = 1.0 - xi - eta
                p = (eta * X[0][0] + z * X[1][0] + xi * X[2][0], eta * X[0][1] + z * X[1][1] + xi * X[2][1])
                out.append((xi, eta, wt * ar, heaviside(p, line, w)))
    return out
