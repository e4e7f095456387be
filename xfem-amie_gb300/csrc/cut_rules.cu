// cut_rules.cu -- integration rules and Heaviside values of triangles crossed
// by a crack polyline, generated on the device, one thread per element.
//
// Reference, in the order the steps follow it:
// * hints: BranchedCrack::enrichSegmentedLine (features/crack.cpp:1088-1175)
//   gives the element the points where the polyline crosses its boundary and
//   the polyline points inside it, in reference coordinates;
//   DelaunayTriangle::getIntegrationHints (mesher/delaunay.cpp:2708-2723) puts
//   the corners (0,1), (0,0), (1,0) first;
// * DelaunayTriangle::getSubTriangulatedGaussPoints (mesher/delaunay.cpp:2801-2985):
//   incremental Delaunay triangulation of the hints starting from the corner
//   triangle, a hint being dropped when it lies within 0.05 of a vertex of a
//   triangle it conflicts with (DelaunayTree::insert, mesher/delaunay.cpp:2157-2196);
//   fewer than three sub-triangles (or a parent area off by more than 1e-6)
//   sends the reference to 512 random points, which cannot be reproduced:
//   status AMIE_CUT_MONTE_CARLO here, and the caller keeps its own rule;
// * per sub-triangle the 4-point rule of TriPoint::getGaussPoints
//   (geometry/geometry_base.cpp:5221-5245): barycentric (0.6, 0.2, 0.2) x 3
//   with weight 0.260416666666667, the centroid with -0.28125, times twice the
//   sub-triangle's area; the weights then scaled to the element's area;
// * Heaviside: PositionOperation::eval (polynomial/vm_token.cpp:242-271):
//   +1 when the segment from the point to a witness point crosses the polyline
//   an odd number of times, -1 otherwise; the witness is the midpoint of the
//   first segment moved by 10 along its unit normal pointing away from
//   (-1000, -1000) (Segment::normal(const Point&), geometry/geometry_base.cpp:4010).
//
// The reference shuffles the hints before inserting them; the result does not
// depend on the order unless two hints lie within the insertion tolerance of
// each other, which is reported (AMIE_CUT_ORDER_DEPENDENT) instead of guessed.
//
// With AMIE_CUT_REPLACE_MONTE_CARLO the elements the reference would integrate
// by Monte-Carlo (or in an insertion-order dependent way) get a deterministic
// rule instead (status AMIE_CUT_REPLACED): the same triangulation with no
// insertion tolerance, so every hint is a vertex and the sub-triangles conform
// to the crack; the rule then integrates the piecewise-polynomial Heaviside
// integrand exactly, where the reference's 512 random points do not.
// Exact-arithmetic degeneracies (a corner on the polyline, a polyline point on
// an edge, four co-circular points) are resolved by the strict orientation and
// in-circle signs below, where the reference applies POINT_TOLERANCE.
#include "internal.h"

namespace amie {

namespace {

constexpr int kMaxHints = AMIE_CUT_MAX_HINTS;
constexpr int kMaxVerts = 3 + kMaxHints;
constexpr int kMaxTris = AMIE_CUT_MAX_POINTS / 4;
constexpr int kMaxEdges = 3 * kMaxTris;
constexpr double kInsertTol = 0.05;   // DelaunayTree::insert minDist
constexpr double kFlat = 1e-12;       // doubled reference area of a sliver on a hull edge
constexpr double kW6 = 0.260416666666667, kWc = -0.28125;

struct P2d {
    double x, y;
};

__device__ inline double orient(P2d a, P2d b, P2d c) { return (b.x - a.x) * (c.y - a.y) - (b.y - a.y) * (c.x - a.x); }

__device__ inline double dist(P2d a, P2d b) { return hypot(a.x - b.x, a.y - b.y); }

// > 0 when d lies inside the circumcircle of the counter-clockwise a, b, c
__device__ inline double incircle(P2d a, P2d b, P2d c, P2d d)
{
    const double adx = a.x - d.x, ady = a.y - d.y, bdx = b.x - d.x, bdy = b.y - d.y, cdx = c.x - d.x, cdy = c.y - d.y;
    return (adx * adx + ady * ady) * (bdx * cdy - cdx * bdy) - (bdx * bdx + bdy * bdy) * (adx * cdy - cdx * ady) +
           (cdx * cdx + cdy * cdy) * (adx * bdy - bdx * ady);
}

__device__ inline bool crosses(P2d p, P2d q, P2d a, P2d b)
{
    return orient(a, b, p) * orient(a, b, q) < 0.0 && orient(p, q, a) * orient(p, q, b) < 0.0;
}

__device__ inline P2d line_pt(const double *line, uint32_t i) { return {line[2 * i], line[2 * i + 1]}; }

__device__ int8_t heaviside(P2d p, P2d w, const double *line, uint32_t n_line)
{
    uint32_t k = 0;
    for (uint32_t s = 0; s + 1 < n_line; s++) k += crosses(p, w, line_pt(line, s), line_pt(line, s + 1)) ? 1u : 0u;
    return (k & 1u) ? int8_t(1) : int8_t(-1);
}

// Incremental Delaunay (Bowyer-Watson) of the corners and the nh hints V[3..]
// from the corner triangle, counter-clockwise in reference coordinates; a hint
// within `tol` of a vertex of a triangle it conflicts with is dropped (the
// reference's insertion tolerance; 0 keeps every hint that is not already a
// vertex).  False when the triangle table would overflow.
__device__ bool triangulate(const P2d (&V)[kMaxVerts], int nh, double tol, uint8_t (&T)[kMaxTris][3], int &nt)
{
    nt = 1;
    T[0][0] = 1, T[0][1] = 2, T[0][2] = 0;
    for (int h = 3; h < 3 + nh; h++) {
        const P2d p = V[h];
        bool con[kMaxTris];
        bool skip = false;
        for (int t = 0; t < nt; t++) {
            con[t] = incircle(V[T[t][0]], V[T[t][1]], V[T[t][2]], p) > 0.0;
            if (con[t])
                for (int k = 0; k < 3; k++) skip |= dist(V[T[t][k]], p) < tol;
        }
        if (skip) continue;
        // boundary of the cavity: edges of conflicting triangles not shared by two of them
        uint8_t E[kMaxEdges][2];
        int ne = 0;
        for (int t = 0; t < nt; t++) {
            if (!con[t]) continue;
            for (int k = 0; k < 3; k++) {
                const uint8_t u = T[t][k], v = T[t][(k + 1) % 3];
                int found = -1;
                for (int q = 0; q < ne; q++)
                    if (E[q][0] == v && E[q][1] == u) found = q;
                if (found >= 0) {
                    E[found][0] = E[ne - 1][0], E[found][1] = E[ne - 1][1];
                    ne--;
                } else if (ne < kMaxEdges) {
                    E[ne][0] = u, E[ne][1] = v;
                    ne++;
                } else {
                    return false;
                }
            }
        }
        int w = 0;
        for (int t = 0; t < nt; t++)
            if (!con[t]) T[w][0] = T[t][0], T[w][1] = T[t][1], T[w][2] = T[t][2], w++;
        nt = w;
        for (int q = 0; q < ne; q++)
            if (orient(V[E[q][0]], V[E[q][1]], p) > kFlat) {
                if (nt == kMaxTris) return false;
                T[nt][0] = E[q][0], T[nt][1] = E[q][1], T[nt][2] = (uint8_t)h;
                nt++;
            }
    }
    return true;
}

}  // namespace

// corners: (x, y) of the corners at reference (0,1), (0,0), (1,0); line: the
// polyline (n_line points).  Writes count (points of the rule, 0 unless the
// status is AMIE_CUT_OK or AMIE_CUT_REPLACED), status, rule (xi, eta, weight),
// h_point (Heaviside at each point) and h_vertex (Heaviside at the three
// corners, always).
__global__ void k_cut_rules(uint32_t n, const double *__restrict__ corners, uint32_t n_line,
                            const double *__restrict__ line, uint32_t flags, uint32_t *count, int8_t *status,
                            double *rule, int8_t *h_point, int8_t *h_vertex)
{
    const uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n) return;
    const bool replace = (flags & AMIE_CUT_REPLACE_MONTE_CARLO) != 0;
    const double *c = corners + (size_t)e * 6;
    const P2d X[3] = {{c[0], c[1]}, {c[2], c[3]}, {c[4], c[5]}};
    const P2d R[3] = {{0.0, 1.0}, {0.0, 0.0}, {1.0, 0.0}};

    // witness point of the first segment
    const P2d a0 = line_pt(line, 0), b0 = line_pt(line, 1);
    const double vx = b0.x - a0.x, vy = b0.y - a0.y, nv = hypot(vx, vy);
    double nx = -vy / nv, ny = vx / nv;
    const double mx = 0.5 * (a0.x + b0.x), my = 0.5 * (a0.y + b0.y);
    if ((mx + 1000.0) * nx + (my + 1000.0) * ny <= 0.0) nx = -nx, ny = -ny;
    const P2d W = {mx + 10.0 * nx, my + 10.0 * ny};
    for (int i = 0; i < 3; i++) h_vertex[(size_t)e * 3 + i] = heaviside(X[i], W, line, n_line);
    count[e] = 0;

    // hints: crossings of each segment with the three edges, then the
    // polyline points strictly inside (barycentric coordinates)
    P2d V[kMaxVerts] = {R[0], R[1], R[2]};
    int nh = 0;
    bool overflow = false;
    const double A2 = orient(X[0], X[1], X[2]);
    for (uint32_t s = 0; s + 1 < n_line; s++) {
        const P2d a = line_pt(line, s), b = line_pt(line, s + 1);
        for (int i = 0; i < 3; i++) {
            const int j = (i + 1) % 3;
            const double fa = orient(a, b, X[i]), fb = orient(a, b, X[j]);
            if (fa * fb < 0.0 && orient(X[i], X[j], a) * orient(X[i], X[j], b) < 0.0) {
                const double t = fa / (fa - fb);
                if (nh == kMaxHints) { overflow = true; continue; }
                V[3 + nh++] = {R[i].x + t * (R[j].x - R[i].x), R[i].y + t * (R[j].y - R[i].y)};
            }
        }
    }
    for (uint32_t s = 0; s < n_line; s++) {
        const P2d p = line_pt(line, s);
        const double l0 = orient(p, X[1], X[2]) / A2, l2 = orient(X[0], X[1], p) / A2;
        if (l0 > 0.0 && l2 > 0.0 && l0 + l2 < 1.0) {
            if (nh == kMaxHints) { overflow = true; continue; }
            V[3 + nh++] = {l2, l0};
        }
    }
    if (overflow) { status[e] = AMIE_CUT_TOO_MANY_HINTS; return; }
    if (nh == 0) { status[e] = AMIE_CUT_NOT_CUT; return; }
    bool close = false;   // two hints within the insertion tolerance
    for (int i = 1; i < nh; i++)
        for (int j = 0; j < i; j++) close |= dist(V[3 + i], V[3 + j]) < kInsertTol;
    uint8_t T[kMaxTris][3];
    int nt = 0;
    int8_t st = AMIE_CUT_OK;
    if (close) st = AMIE_CUT_ORDER_DEPENDENT;
    else if (!triangulate(V, nh, kInsertTol, T, nt)) st = AMIE_CUT_TOO_MANY_HINTS;
    else if (nt < 3) st = AMIE_CUT_MONTE_CARLO;
    if ((st == AMIE_CUT_ORDER_DEPENDENT || st == AMIE_CUT_MONTE_CARLO) && replace) {
        if (!triangulate(V, nh, 0.0, T, nt)) st = AMIE_CUT_TOO_MANY_HINTS;
        else if (nt < 3) st = AMIE_CUT_MONTE_CARLO;
        else st = AMIE_CUT_REPLACED;
    }
    if (st != AMIE_CUT_OK && st != AMIE_CUT_REPLACED) { status[e] = st; return; }

    // the 4-point rule on each sub-triangle, weights scaled to the element's area
    double *out = rule + (size_t)e * AMIE_CUT_MAX_POINTS * 3;
    int8_t *hp = h_point + (size_t)e * AMIE_CUT_MAX_POINTS;
    double parent = 0.0;
    int k = 0;
    for (int t = 0; t < nt; t++) {
        const P2d A = V[T[t][0]], B = V[T[t][1]], C = V[T[t][2]];
        const double ar = fabs(orient(A, B, C));   // twice the area
        for (int r = 0; r < 4; r++) {
            double l[3] = {0.2, 0.2, 0.2};
            if (r < 3) l[r] = 0.6;
            else l[0] = l[1] = l[2] = 1.0 / 3.0;
            const double wq = (r < 3 ? kW6 : kWc) * ar;
            out[k * 3 + 0] = l[0] * A.x + l[1] * B.x + l[2] * C.x;
            out[k * 3 + 1] = l[0] * A.y + l[1] * B.y + l[2] * C.y;
            out[k * 3 + 2] = wq;
            parent += wq;
            k++;
        }
    }
    if (fabs(parent - 0.5) > 1e-6) { status[e] = AMIE_CUT_MONTE_CARLO; return; }
    const double scale = 0.5 * fabs(A2) / parent;
    for (int q = 0; q < k; q++) {
        const double xi = out[q * 3 + 0], eta = out[q * 3 + 1];
        out[q * 3 + 2] *= scale;
        const double zeta = 1.0 - xi - eta;
        const P2d p = {eta * X[0].x + zeta * X[1].x + xi * X[2].x, eta * X[0].y + zeta * X[1].y + xi * X[2].y};
        hp[q] = heaviside(p, W, line, n_line);
    }
    count[e] = (uint32_t)k;
    status[e] = st;
}

}  // namespace amie

using namespace amie;

extern "C" amie_status amie_cut_rules(amie_ctx *ctx, uint32_t n, const double *corners, uint32_t n_line,
                                      const double *line, uint32_t flags, uint32_t *count, int8_t *status,
                                      double *rule, int8_t *h_point, int8_t *h_vertex)
{
    if (!ctx || n_line < 2 || !line || (n && (!corners || !count || !status || !rule || !h_point || !h_vertex)))
        return AMIE_BAD_INPUT;
    if (line[0] == line[2] && line[1] == line[3]) return AMIE_BAD_INPUT;   // the witness needs a first segment
    if (flags & ~(uint32_t)AMIE_CUT_REPLACE_MONTE_CARLO) return AMIE_BAD_INPUT;
    if (!n) return AMIE_OK;
    AMIE_CUDA(cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;
    const size_t np = (size_t)n * AMIE_CUT_MAX_POINTS;
    DevArray<double> dc, dl, dr;
    DevArray<uint32_t> dn;
    DevArray<int8_t> dst, dhp, dhv;
    AMIE_TRY(dc.alloc(ctx, (size_t)n * 6));
    AMIE_TRY(dl.alloc(ctx, (size_t)n_line * 2));
    AMIE_TRY(dr.alloc(ctx, np * 3));
    AMIE_TRY(dn.alloc(ctx, n));
    AMIE_TRY(dst.alloc(ctx, n));
    AMIE_TRY(dhp.alloc(ctx, np));
    AMIE_TRY(dhv.alloc(ctx, (size_t)n * 3));
    AMIE_CUDA(cudaMemcpyAsync(dc.p, corners, (size_t)n * 6 * 8, cudaMemcpyHostToDevice, st));
    AMIE_CUDA(cudaMemcpyAsync(dl.p, line, (size_t)n_line * 2 * 8, cudaMemcpyHostToDevice, st));
    k_cut_rules<<<(n + 127) / 128, 128, 0, st>>>(n, dc.p, n_line, dl.p, flags, dn.p, dst.p, dr.p, dhp.p, dhv.p);
    g_launches += 1;
    AMIE_CUDA(cudaGetLastError());
    AMIE_CUDA(cudaMemcpyAsync(count, dn.p, (size_t)n * 4, cudaMemcpyDeviceToHost, st));
    AMIE_CUDA(cudaMemcpyAsync(status, dst.p, n, cudaMemcpyDeviceToHost, st));
    AMIE_CUDA(cudaMemcpyAsync(rule, dr.p, np * 3 * 8, cudaMemcpyDeviceToHost, st));
    AMIE_CUDA(cudaMemcpyAsync(h_point, dhp.p, np, cudaMemcpyDeviceToHost, st));
    AMIE_CUDA(cudaMemcpyAsync(h_vertex, dhv.p, (size_t)n * 3, cudaMemcpyDeviceToHost, st));
    AMIE_CUDA(cudaStreamSynchronize(st));
    return AMIE_OK;
}
