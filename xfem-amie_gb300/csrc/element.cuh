// element.cuh -- element-level device helpers shared by the quadrature,
// field-recovery and damage kernels: shape-function gradients, default Gauss
// rules, inverse-Jacobian algebra and the B^T C B contribution.
#pragma once

#include "internal.h"

namespace amie {


__host__ __device__ inline int nshape_of(int kind) { return kind == AMIE_TRI3 ? 3 : kind == AMIE_TRI6 ? 6 : kind == AMIE_TET4 ? 4 : 0; }

// Local gradients of the shape functions of TriElement LINEAR / QUADRATIC
// (elements/elements.cpp:976-1060) and TetrahedralElement LINEAR
// (elements/elements.cpp:2496-2530); x = xi, y = eta.
__device__ inline void shape_grad(int kind, int f, double x, double y, double g[3])
{
    g[2] = 0.0;
    if (kind == AMIE_TRI3) {
        const double gx[3] = {0.0, -1.0, 1.0}, gy[3] = {1.0, -1.0, 0.0};
        g[0] = gx[f]; g[1] = gy[f];
    } else if (kind == AMIE_TRI6) {
        switch (f) {
        case 0: g[0] = 0.0; g[1] = 4.0 * y - 1.0; break;
        case 1: g[0] = -4.0 * y; g[1] = 4.0 - 4.0 * x - 8.0 * y; break;
        case 2: g[0] = 4.0 * y + 4.0 * x - 3.0; g[1] = 4.0 * x + 4.0 * y - 3.0; break;
        case 3: g[0] = 4.0 - 8.0 * x - 4.0 * y; g[1] = -4.0 * x; break;
        case 4: g[0] = 4.0 * x - 1.0; g[1] = 0.0; break;
        default: g[0] = 4.0 * y; g[1] = 4.0 * x; break;
        }
    } else {
        const double gx[4] = {0.0, -1.0, 1.0, 0.0}, gy[4] = {0.0, -1.0, 0.0, 1.0}, gz[4] = {1.0, -1.0, 0.0, 0.0};
        g[0] = gx[f]; g[1] = gy[f]; g[2] = gz[f];
    }
}

// Default Gauss rules (elements/elements.cpp:666-697, 2397-2400), with the
// reference's literal coordinates and weights.
__device__ inline int default_rule(int kind, int g, double p[3], double *w)
{
    p[2] = 0.0;
    if (kind == AMIE_TRI3) {
        p[0] = p[1] = 0.333333333333333; *w = 0.5;
        return 1;
    }
    if (kind == AMIE_TRI6) {
        const double px[4] = {0.2, 0.6, 0.2, 0.33333333333333}, py[4] = {0.2, 0.2, 0.6, 0.33333333333333};
        const double pw[4] = {0.260416666666667, 0.260416666666667, 0.260416666666667, -0.28125};
        p[0] = px[g]; p[1] = py[g]; *w = pw[g];
        return 4;
    }
    p[0] = p[1] = p[2] = 0.25; *w = 0.1666666666666667;
    return 1;
}

template <int DIM>
__device__ inline double det_small(const double *J)
{
    if (DIM == 2) return J[0] * J[3] - J[1] * J[2];
    return J[0] * (J[4] * J[8] - J[5] * J[7]) - J[1] * (J[3] * J[8] - J[5] * J[6]) + J[2] * (J[3] * J[7] - J[4] * J[6]);
}

// Physical gradient d_r = sum_c g_c Jinv[r][c] (polynomial/vm_base.cpp:2251-2252).
template <int DIM>
__device__ inline void phys_grad(const double *J, const double *g, double *d)
{
#pragma unroll
    for (int r = 0; r < DIM; r++) {
        double a = 0.0;
#pragma unroll
        for (int c = 0; c < DIM; c++) a += g[c] * J[r * DIM + c];
        d[r] = a;
    }
}

// Contribution w * B_i C B_j^T (s x s) for the Voigt B of geval
// (polynomial/vm_base.cpp:2244-2255 in 2D, 2278-2296 in 3D).
template <int DIM>
__device__ inline void bcb(const double *di, const double *dj, const double *C, double w, double *out)
{
    constexpr int NV = DIM == 2 ? 3 : 6;
    double Bi[DIM][NV], Bj[DIM][NV];
#pragma unroll
    for (int r = 0; r < DIM; r++)
#pragma unroll
        for (int k = 0; k < NV; k++) { Bi[r][k] = 0.0; Bj[r][k] = 0.0; }
    if (DIM == 2) {
        Bi[0][0] = di[0]; Bi[0][2] = di[1]; Bi[1][1] = di[1]; Bi[1][2] = di[0];
        Bj[0][0] = dj[0]; Bj[0][2] = dj[1]; Bj[1][1] = dj[1]; Bj[1][2] = dj[0];
    } else {
        Bi[0][0] = di[0]; Bi[0][4] = di[2]; Bi[0][5] = di[1];
        Bi[1][1] = di[1]; Bi[1][3] = di[2]; Bi[1][5] = di[0];
        Bi[2][2] = di[2]; Bi[2][3] = di[1]; Bi[2][4] = di[0];
        Bj[0][0] = dj[0]; Bj[0][4] = dj[2]; Bj[0][5] = dj[1];
        Bj[1][1] = dj[1]; Bj[1][3] = dj[2]; Bj[1][5] = dj[0];
        Bj[2][2] = dj[2]; Bj[2][3] = dj[1]; Bj[2][4] = dj[0];
    }
#pragma unroll
    for (int r = 0; r < DIM; r++) {
        double BiC[NV];
#pragma unroll
        for (int l = 0; l < NV; l++) {
            double a = 0.0;
#pragma unroll
            for (int k = 0; k < NV; k++) a += Bi[r][k] * C[k * NV + l];
            BiC[l] = a;
        }
#pragma unroll
        for (int c = 0; c < DIM; c++) {
            double a = 0.0;
#pragma unroll
            for (int l = 0; l < NV; l++) a += BiC[l] * Bj[c][l];
            out[r * DIM + c] += w * a;
        }
    }
}


// Local gradient of one tip branch function N_v^{P1} (F_j(x) - F_j(x_v)) at
// local coordinates (xi, eta) (BranchedCrack::enrichTip, features/crack.cpp:898-960).
// rec: x(0,0) - x_tip, dx/dxi, dx/deta, crack angle a, branch j.  With (u, w)
// the position relative to the tip in the frame rotated by a, the reference's
// atan2 token gives t = -atan2(w, u) (its values of the four functions match
// this to 1e-14); F_j = sqrt(r) g_j(t), grad F = g_j grad r / (2 sqrt r) +
// sqrt(r) g_j'(t) grad t with grad t = (dy, -dx) / r^2.
__device__ inline void tip_function_grad(const double *rec, int v, double xi, double eta, double lg[3])
{
    const double a = rec[6];
    const int j = (int)rec[7];
    const double ca = cos(a), sa = sin(a);
    double F[2], Fx = 0.0, Fy = 0.0;
    // k = 0: the Gauss point, k = 1: the vertex the function is attached to
    const double vxi[3] = {0.0, 0.0, 1.0}, veta[3] = {1.0, 0.0, 0.0};
    for (int k = 0; k < 2; k++) {
        const double s0 = k ? vxi[v] : xi, s1 = k ? veta[v] : eta;
        const double dx = rec[0] + s0 * rec[2] + s1 * rec[4];
        const double dy = rec[1] + s0 * rec[3] + s1 * rec[5];
        const double r2 = dx * dx + dy * dy, r = sqrt(r2), sr = sqrt(r);
        const double t = -atan2(-sa * dx + ca * dy, ca * dx + sa * dy);
        const double s2 = sin(0.5 * t), c2 = cos(0.5 * t), st = sin(t), ct = cos(t);
        double g, gp;
        if (j == 0) { g = s2; gp = 0.5 * c2; }
        else if (j == 1) { g = c2; gp = -0.5 * s2; }
        else if (j == 2) { g = s2 * st; gp = 0.5 * c2 * st + s2 * ct; }
        else { g = c2 * st; gp = -0.5 * s2 * st + c2 * ct; }
        F[k] = sr * g;
        if (k == 0) {
            const double gr = g / (2.0 * sr * r);   // g / (2 sqrt r) / r, times dx or dy
            Fx = gr * dx + sr * gp * (dy / r2);
            Fy = gr * dy - sr * gp * (dx / r2);
        }
    }
    // P1 hat function of vertex v: vertex 0 at (0, 1), 1 at (0, 0), 2 at (1, 0)
    const double N = v == 0 ? eta : (v == 1 ? 1.0 - xi - eta : xi);
    const double dNx[3] = {0.0, -1.0, 1.0}, dNy[3] = {1.0, -1.0, 0.0};
    const double dF = F[0] - F[1];
    lg[0] = dNx[v] * dF + N * (rec[2] * Fx + rec[3] * Fy);
    lg[1] = dNy[v] * dF + N * (rec[4] * Fx + rec[5] * Fy);
    lg[2] = 0.0;
}

// Local gradient of enrichment function fj at Gauss point g of its element
// (local coordinates p): Heaviside (closed form), tip branch (closed form) or
// tabulated.
template <int DIM>
__device__ inline void enr_local_grad(const MeshView &m, uint32_t fj, uint32_t g, const double *p, double lg[3])
{
    const uint8_t type = m.enr_type[fj];
    if (DIM == 2 && type == AMIE_ENR_HEAVISIDE) {
        // grad(N_k^{P1} (H - H_k)) = grad N_k^{P1} * jump away from the crack
        // (features/crack.cpp:1316,1332,1347)
        const int v = m.enr_vertex[fj];
        const double jump = (double)m.enr_jump[(uint64_t)m.enr_data[fj] + g];
        const double gx[3] = {0.0, -1.0, 1.0}, gy[3] = {1.0, -1.0, 0.0};
        lg[0] = gx[v] * jump;
        lg[1] = gy[v] * jump;
    } else if (DIM == 2 && type == AMIE_ENR_TIP) {
        tip_function_grad(m.enr_tip + (uint64_t)m.enr_data[fj] * 8, m.enr_vertex[fj], p[0], p[1], lg);
    } else {
        const uint64_t off = (uint64_t)m.enr_data[fj] + g;
#pragma unroll
        for (int c = 0; c < DIM; c++) lg[c] = m.enr_grad[off * DIM + c];
    }
}

}  // namespace amie
