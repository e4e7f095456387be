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

}  // namespace amie
