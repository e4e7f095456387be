// amie_oracle.cpp -- CPU restatement of AMIE's FE hot path (see amie_oracle.h).
//
// TEST INFRASTRUCTURE ONLY.  Used by tests/ as the checker, by the smoke check
// and by the benchmark's CPU-baseline leg.  The GPU library never links it.
//
// Each function restates the reference algorithm named in its comment; file
// paths are relative to the AMIE source tree.

#include "amie_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// ---------------------------------------------------------------- elements

int shape_count(int kind)
{
    switch (kind) {
    case ORACLE_TRI3: return 3;
    case ORACLE_TRI6: return 6;
    case ORACLE_TET4: return 4;
    default: return 0;
    }
}

// Default Gauss rules of TriElement::genGaussPoints (elements/elements.cpp:666-697)
// and TetrahedralElement::genGaussPoints (elements/elements.cpp:2397-2400).  The
// literals are the reference's own (0.333333333333333, 0.260416666666667 ...):
// P2 gradients are linear, so the Gauss point coordinates enter K_e.
struct Rule { int n; double p[4][3]; double w[4]; };

Rule default_rule(int kind)
{
    Rule r{};
    if (kind == ORACLE_TRI3) {
        r.n = 1;
        r.p[0][0] = 0.333333333333333; r.p[0][1] = 0.333333333333333; r.w[0] = 0.5;
    } else if (kind == ORACLE_TRI6) {
        r.n = 4;
        const double pts[4][2] = {{0.2, 0.2}, {0.6, 0.2}, {0.2, 0.6}, {0.33333333333333, 0.33333333333333}};
        for (int g = 0; g < 4; g++) { r.p[g][0] = pts[g][0]; r.p[g][1] = pts[g][1]; }
        r.w[0] = r.w[1] = r.w[2] = 0.260416666666667;
        r.w[3] = -0.28125;
    } else if (kind == ORACLE_TET4) {
        r.n = 1;
        r.p[0][0] = r.p[0][1] = r.p[0][2] = 0.25;
        r.w[0] = 0.1666666666666667;
    }
    return r;
}

// Local-coordinate gradients of the shape functions (elements/elements.cpp:976-1060
// for triangles, 2496-2530 for the linear tetrahedron).  x = xi, y = eta, z = zeta.
void shape_grad(int kind, const double *p, double g[][3])
{
    const double x = p[0], y = p[1];
    if (kind == ORACLE_TRI3) {
        g[0][0] = 0;  g[0][1] = 1;    // N0 = y
        g[1][0] = -1; g[1][1] = -1;   // N1 = 1 - x - y
        g[2][0] = 1;  g[2][1] = 0;    // N2 = x
    } else if (kind == ORACLE_TRI6) {
        g[0][0] = 0;                 g[0][1] = 4 * y - 1;            // 2y^2 - y
        g[1][0] = -4 * y;            g[1][1] = 4 - 4 * x - 8 * y;    // 4y - 4xy - 4y^2
        g[2][0] = 4 * y + 4 * x - 3; g[2][1] = 4 * x + 4 * y - 3;    // 1-3x-3y+4xy+2x^2+2y^2
        g[3][0] = 4 - 8 * x - 4 * y; g[3][1] = -4 * x;               // 4x - 4x^2 - 4xy
        g[4][0] = 4 * x - 1;         g[4][1] = 0;                    // 2x^2 - x
        g[5][0] = 4 * y;             g[5][1] = 4 * x;                // 4xy
    } else if (kind == ORACLE_TET4) {
        g[0][0] = 0;  g[0][1] = 0;  g[0][2] = 1;    // N0 = z
        g[1][0] = -1; g[1][1] = -1; g[1][2] = -1;   // N1 = 1 - x - y - z
        g[2][0] = 1;  g[2][1] = 0;  g[2][2] = 0;    // N2 = x
        g[3][0] = 0;  g[3][1] = 1;  g[3][2] = 0;    // N3 = y
    }
}

// P1 triangle gradients used by the Heaviside enrichment N_k^{P1} (H - H_k)
// (features/crack.cpp:1224,1316,1332,1347).
const double P1_GRAD[3][2] = {{0, 1}, {-1, -1}, {1, 0}};

double det(int dim, const double *J)
{
    if (dim == 2) return J[0] * J[3] - J[1] * J[2];
    return J[0] * (J[4] * J[8] - J[5] * J[7]) - J[1] * (J[3] * J[8] - J[5] * J[6]) +
           J[2] * (J[3] * J[7] - J[4] * J[6]);
}

// Voigt B row layout of geval (polynomial/vm_base.cpp:2244-2255 in 2D,
// 2278-2296 in 3D): B is s x nv, built from the physical gradient d.
void make_B(int dim, const double *d, double *B)
{
    if (dim == 2) {
        // [[a, 0, b], [0, b, a]]
        B[0] = d[0]; B[1] = 0;    B[2] = d[1];
        B[3] = 0;    B[4] = d[1]; B[5] = d[0];
    } else {
        // rows x,y,z ; columns xx yy zz yz xz xy
        for (int i = 0; i < 18; i++) B[i] = 0;
        B[0 * 6 + 0] = d[0]; B[0 * 6 + 4] = d[2]; B[0 * 6 + 5] = d[1];
        B[1 * 6 + 1] = d[1]; B[1 * 6 + 3] = d[2]; B[1 * 6 + 5] = d[0];
        B[2 * 6 + 2] = d[2]; B[2 * 6 + 3] = d[1]; B[2 * 6 + 4] = d[0];
    }
}

}  // namespace

extern "C" int oracle_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

extern "C" int oracle_element_matrices(const oracle_mesh *m, const uint64_t *ke_off, double *ke)
{
    const int dim = m->dim, s = m->stride;
    const int nv = dim == 2 ? 3 : 6;
    if (s != dim) return -1;
    int bad = 0;
#pragma omp parallel for schedule(dynamic, 64) reduction(| : bad)
    for (int64_t e = 0; e < (int64_t)m->n_elem; e++) {
        const int kind = m->kind[e];
        const int nshape = shape_count(kind);
        const uint32_t e0 = m->enr_ptr ? m->enr_ptr[e] : 0, e1 = m->enr_ptr ? m->enr_ptr[e + 1] : 0;
        const int nenr = (int)(e1 - e0);
        const int nf = nshape + nenr;
        if (nshape == 0 || (int)(m->dof_ptr[e + 1] - m->dof_ptr[e]) != nf) { bad = 1; continue; }
        const double *Je = m->jinv + (size_t)e * dim * dim;
        // Effective constitutive matrix: (damage or per-element modulus factor) * C
        // (physics/stiffness_and_fracture.cpp:75-79).
        double C[36];
        const double cs = m->cscale ? m->cscale[e] : 1.0;
        const double *Ct = m->cmat_table + (size_t)m->mat[e] * nv * nv;
        for (int i = 0; i < nv * nv; i++) C[i] = cs * Ct[i];

        // Gauss points: explicit (already weighted by det J), or the default rule
        // with weight / det(J^-1) (elements/elements.cpp:939-945).
        std::vector<double> pts, wts;
        const uint32_t g0 = m->gp_ptr[e], g1 = m->gp_ptr[e + 1];
        if (g1 > g0) {
            for (uint32_t g = g0; g < g1; g++) {
                for (int c = 0; c < dim; c++) pts.push_back(m->gp[(size_t)g * (dim + 1) + c]);
                wts.push_back(m->gp[(size_t)g * (dim + 1) + dim]);
            }
        } else {
            Rule r = default_rule(kind);
            const double dj = det(dim, Je);
            for (int g = 0; g < r.n; g++) {
                for (int c = 0; c < dim; c++) pts.push_back(r.p[g][c]);
                wts.push_back(r.w[g] / dj);
            }
        }
        const int ngp = (int)wts.size();
        const bool moved = m->moved && m->moved[e] && g1 > g0;
        const int msz = nf * s;
        double *K = ke + ke_off[e];
        for (int i = 0; i < msz * msz; i++) K[i] = 0.0;

        std::vector<double> grads((size_t)nf * 3);
        std::vector<double> Bs((size_t)nf * s * nv);
        for (int g = 0; g < ngp; g++) {
            const double *p = &pts[(size_t)g * dim];
            double sg[6][3];
            shape_grad(kind, p, sg);
            for (int f = 0; f < nshape; f++)
                for (int c = 0; c < dim; c++) grads[f * 3 + c] = sg[f][c];
            for (int j = 0; j < nenr; j++) {
                const uint32_t fj = e0 + j;
                const size_t off = (size_t)m->enr_data[fj] + g;
                double *gr = &grads[(nshape + j) * 3];
                if (m->enr_type[fj] == ORACLE_ENR_HEAVISIDE) {
                    const int v = m->enr_vertex[fj];
                    const double jump = (double)m->enr_jump[off];
                    gr[0] = P1_GRAD[v][0] * jump;
                    gr[1] = P1_GRAD[v][1] * jump;
                    gr[2] = 0;
                } else {
                    for (int c = 0; c < dim; c++) gr[c] = m->enr_grad[off * dim + c];
                }
            }
            // physical gradient a_r = sum_c dN/dxi_c * Jinv[r][c] (polynomial/vm_base.cpp:2251-2252);
            // moved elements use the inverse Jacobian of each Gauss point (mesher/delaunay.cpp:2441-2447)
            const double *J = moved ? m->jinv_gp + (size_t)(g0 + g) * dim * dim : Je;
            for (int f = 0; f < nf; f++) {
                double d[3] = {0, 0, 0};
                for (int r = 0; r < dim; r++)
                    for (int c = 0; c < dim; c++) d[r] += grads[f * 3 + c] * J[r * dim + c];
                make_B(dim, d, &Bs[(size_t)f * s * nv]);
            }
            const double w = wts[g];
            // K[i][j] += w * B_i C B_j^T for i >= j; upper blocks are transposes
            // (mesher/delaunay.cpp:2462-2467).
            for (int i = 0; i < nf; i++) {
                const double *Bi = &Bs[(size_t)i * s * nv];
                double BiC[3 * 6];
                for (int r = 0; r < s; r++)
                    for (int l = 0; l < nv; l++) {
                        double acc = 0;
                        for (int k = 0; k < nv; k++) acc += Bi[r * nv + k] * C[k * nv + l];
                        BiC[r * nv + l] = acc;
                    }
                for (int j = 0; j <= i; j++) {
                    const double *Bj = &Bs[(size_t)j * s * nv];
                    for (int r = 0; r < s; r++)
                        for (int c = 0; c < s; c++) {
                            double acc = 0;
                            for (int l = 0; l < nv; l++) acc += BiC[r * nv + l] * Bj[c * nv + l];
                            K[(size_t)(i * s + r) * msz + j * s + c] += w * acc;
                        }
                }
            }
        }
        for (int i = 0; i < nf; i++)
            for (int j = 0; j < i; j++)
                for (int r = 0; r < s; r++)
                    for (int c = 0; c < s; c++)
                        K[(size_t)(j * s + c) * msz + i * s + r] = K[(size_t)(i * s + r) * msz + j * s + c];
    }
    return bad ? -2 : 0;
}

extern "C" int oracle_element_fields(const oracle_mesh *m, const double *u, double *strain, double *stress)
{
    const int dim = m->dim;
    const int nv = dim == 2 ? 3 : 6;
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < (int64_t)m->n_elem; e++) {
        const int kind = m->kind[e];
        const int nshape = shape_count(kind);
        const uint32_t e0 = m->enr_ptr ? m->enr_ptr[e] : 0, e1 = m->enr_ptr ? m->enr_ptr[e + 1] : 0;
        const int nf = nshape + (int)(e1 - e0);
        const double *Je = m->jinv + (size_t)e * dim * dim;
        const uint32_t g0 = m->gp_ptr[e], g1 = m->gp_ptr[e + 1];
        std::vector<double> pts, wts;
        if (g1 > g0) {
            for (uint32_t g = g0; g < g1; g++) {
                for (int c = 0; c < dim; c++) pts.push_back(m->gp[(size_t)g * (dim + 1) + c]);
                wts.push_back(m->gp[(size_t)g * (dim + 1) + dim]);
            }
        } else {
            Rule r = default_rule(kind);
            for (int g = 0; g < r.n; g++) {
                for (int c = 0; c < dim; c++) pts.push_back(r.p[g][c]);
                wts.push_back(r.w[g] / det(dim, Je));
            }
        }
        const bool moved = m->moved && m->moved[e] && g1 > g0;
        double eps[6] = {0, 0, 0, 0, 0, 0}, wsum = 0;
        for (size_t g = 0; g < wts.size(); g++) {
            double sg[6][3];
            shape_grad(kind, &pts[g * dim], sg);
            const double *J = moved ? m->jinv_gp + (size_t)(g0 + g) * dim * dim : Je;
            double eg[6] = {0, 0, 0, 0, 0, 0};
            for (int f = 0; f < nf; f++) {
                double lg[3] = {0, 0, 0};
                if (f < nshape) {
                    for (int c = 0; c < dim; c++) lg[c] = sg[f][c];
                } else {
                    const uint32_t fj = e0 + (f - nshape);
                    const size_t off = (size_t)m->enr_data[fj] + g;
                    if (m->enr_type[fj] == ORACLE_ENR_HEAVISIDE) {
                        lg[0] = P1_GRAD[m->enr_vertex[fj]][0] * m->enr_jump[off];
                        lg[1] = P1_GRAD[m->enr_vertex[fj]][1] * m->enr_jump[off];
                    } else {
                        for (int c = 0; c < dim; c++) lg[c] = m->enr_grad[off * dim + c];
                    }
                }
                double d[3] = {0, 0, 0};
                for (int r = 0; r < dim; r++)
                    for (int c = 0; c < dim; c++) d[r] += lg[c] * J[r * dim + c];
                const double *x = u + (size_t)m->dof_ids[m->dof_ptr[e] + f] * dim;
                if (dim == 2) {
                    eg[0] += d[0] * x[0];
                    eg[1] += d[1] * x[1];
                    eg[2] += d[1] * x[0] + d[0] * x[1];
                } else {
                    eg[0] += d[0] * x[0];
                    eg[1] += d[1] * x[1];
                    eg[2] += d[2] * x[2];
                    eg[3] += d[2] * x[1] + d[1] * x[2];
                    eg[4] += d[2] * x[0] + d[0] * x[2];
                    eg[5] += d[1] * x[0] + d[0] * x[1];
                }
            }
            for (int k = 0; k < nv; k++) eps[k] += wts[g] * eg[k];
            wsum += wts[g];
        }
        const double cs = m->cscale ? m->cscale[e] : 1.0;
        const double *C = m->cmat_table + (size_t)m->mat[e] * nv * nv;
        for (int k = 0; k < nv; k++) eps[k] /= wsum;
        for (int k = 0; k < nv; k++) {
            double s = 0;
            for (int l = 0; l < nv; l++) s += C[k * nv + l] * eps[l];
            strain[(size_t)e * nv + k] = eps[k];
            stress[(size_t)e * nv + k] = cs * s;
        }
    }
    return 0;
}

// Induced forces of an imposed strain eps0 (per element, Voigt): for every
// function f of every element, f_f += sum_g w_g B_f(g)^T (C eps0), added into
// the global force vector in element order -- the SET_VOLUMIC_STRESS_* forces
// StiffnessWithImposedStrain::getBoundaryConditions
// (physics/stiffness_with_imposed_deformation.cpp:83-110) hands to
// DofDefinedBoundaryCondition (features/boundarycondition.cpp:542-617), which
// Assembly::addForceOn (solvers/assembly.cpp:1477-1530) accumulates per DOF.
// C is the element's undamaged material matrix, as in the reference.
extern "C" int oracle_induced_forces(const oracle_mesh *m, const double *imposed, double *force)
{
    const int dim = m->dim;
    const int nv = dim == 2 ? 3 : 6;
    for (int64_t e = 0; e < (int64_t)m->n_elem; e++) {
        const double *C = m->cmat_table + (size_t)m->mat[e] * nv * nv;
        double sig[6] = {0, 0, 0, 0, 0, 0};
        for (int r = 0; r < nv; r++)
            for (int c = 0; c < nv; c++) sig[r] += C[r * nv + c] * imposed[(size_t)e * nv + c];
        const int kind = m->kind[e];
        const int nshape = shape_count(kind);
        const uint32_t e0 = m->enr_ptr ? m->enr_ptr[e] : 0, e1 = m->enr_ptr ? m->enr_ptr[e + 1] : 0;
        const int nf = nshape + (int)(e1 - e0);
        const double *Je = m->jinv + (size_t)e * dim * dim;
        const uint32_t g0 = m->gp_ptr[e], g1 = m->gp_ptr[e + 1];
        std::vector<double> pts, wts;
        if (g1 > g0) {
            for (uint32_t g = g0; g < g1; g++) {
                for (int c = 0; c < dim; c++) pts.push_back(m->gp[(size_t)g * (dim + 1) + c]);
                wts.push_back(m->gp[(size_t)g * (dim + 1) + dim]);
            }
        } else {
            Rule r = default_rule(kind);
            for (int g = 0; g < r.n; g++) {
                for (int c = 0; c < dim; c++) pts.push_back(r.p[g][c]);
                wts.push_back(r.w[g] / det(dim, Je));
            }
        }
        const bool moved = m->moved && m->moved[e] && g1 > g0;
        for (int f = 0; f < nf; f++) {
            double acc[3] = {0, 0, 0};
            for (size_t g = 0; g < wts.size(); g++) {
                double sg[6][3];
                shape_grad(kind, &pts[g * dim], sg);
                const double *J = moved ? m->jinv_gp + (size_t)(g0 + g) * dim * dim : Je;
                double lg[3] = {0, 0, 0};
                if (f < nshape) {
                    for (int c = 0; c < dim; c++) lg[c] = sg[f][c];
                } else {
                    const uint32_t fj = e0 + (f - nshape);
                    const size_t off = (size_t)m->enr_data[fj] + g;
                    if (m->enr_type[fj] == ORACLE_ENR_HEAVISIDE) {
                        lg[0] = P1_GRAD[m->enr_vertex[fj]][0] * m->enr_jump[off];
                        lg[1] = P1_GRAD[m->enr_vertex[fj]][1] * m->enr_jump[off];
                    } else {
                        for (int c = 0; c < dim; c++) lg[c] = m->enr_grad[off * dim + c];
                    }
                }
                double d[3] = {0, 0, 0};
                for (int r = 0; r < dim; r++)
                    for (int c = 0; c < dim; c++) d[r] += lg[c] * J[r * dim + c];
                const double w = wts[g];
                if (dim == 2) {
                    acc[0] += w * (d[0] * sig[0] + d[1] * sig[2]);
                    acc[1] += w * (d[1] * sig[1] + d[0] * sig[2]);
                } else {
                    acc[0] += w * (d[0] * sig[0] + d[2] * sig[4] + d[1] * sig[5]);
                    acc[1] += w * (d[1] * sig[1] + d[2] * sig[3] + d[0] * sig[5]);
                    acc[2] += w * (d[2] * sig[2] + d[1] * sig[3] + d[0] * sig[4]);
                }
            }
            const size_t id = m->dof_ids[m->dof_ptr[e] + f];
            for (int c = 0; c < dim; c++) force[id * dim + c] += acc[c];
        }
    }
    return 0;
}

extern "C" int oracle_pattern(const oracle_mesh *m, uint32_t *n_rows, uint64_t *nnzb, uint32_t *row_size,
                              uint32_t *column_index)
{
    // std::set<pair<uint,uint>> of make_final, built as a sorted unique list of
    // (row << 32 | col): every (ids[j], ids[k]) pair of every element, the
    // diagonal gap fill (i, i) for i < max id + 1, and (ndofmax-1, ndofmax-1)
    // (solvers/assembly.cpp:458-507).
    std::vector<uint64_t> keys;
    uint64_t maxid = 0;
    for (uint32_t e = 0; e < m->n_elem; e++) {
        const uint32_t a = m->dof_ptr[e], b = m->dof_ptr[e + 1];
        for (uint32_t j = a; j < b; j++) {
            maxid = std::max<uint64_t>(maxid, m->dof_ids[j]);
            for (uint32_t k = a; k < b; k++)
                keys.push_back(((uint64_t)m->dof_ids[j] << 32) | m->dof_ids[k]);
        }
    }
    for (uint64_t i = 0; i <= maxid; i++) keys.push_back((i << 32) | i);
    if (m->ndofmax > 0) keys.push_back(((uint64_t)(m->ndofmax - 1) << 32) | (m->ndofmax - 1));
    std::sort(keys.begin(), keys.end());
    keys.erase(std::unique(keys.begin(), keys.end()), keys.end());
    const uint32_t rows = (uint32_t)((keys.back() >> 32) + 1);
    *n_rows = rows;
    *nnzb = keys.size();
    if (!row_size) return 0;
    std::memset(row_size, 0, sizeof(uint32_t) * rows);
    for (size_t i = 0; i < keys.size(); i++) {
        row_size[keys[i] >> 32]++;
        column_index[i] = (uint32_t)(keys[i] & 0xffffffffu);
    }
    return 0;
}

namespace {

std::vector<uint64_t> row_starts(uint32_t n_rows, const uint32_t *row_size)
{
    std::vector<uint64_t> acc(n_rows + 1, 0);
    for (uint32_t i = 0; i < n_rows; i++) acc[i + 1] = acc[i] + row_size[i];
    return acc;
}

int64_t find_block(const std::vector<uint64_t> &acc, const uint32_t *column_index, uint32_t row, uint32_t col)
{
    const uint32_t *b = column_index + acc[row], *e = column_index + acc[row + 1];
    const uint32_t *p = std::lower_bound(b, e, col);
    if (p == e || *p != col) return -1;
    return (int64_t)(p - column_index);
}

}  // namespace

extern "C" int oracle_scatter(const oracle_mesh *m, const uint64_t *ke_off, const double *ke, uint32_t n_rows,
                              const uint32_t *row_size, const uint32_t *column_index, double *array)
{
    const int s = m->stride;
    const int cl = s + s % 2;          // padded column length
    const int bs = s * cl;             // doubles per block
    std::vector<uint64_t> acc = row_starts(n_rows, row_size);
    const size_t total = acc[n_rows] * bs;
    std::memset(array, 0, sizeof(double) * total);
    std::vector<double> comp(total, 0.0);   // Kahan compensation (solvers/assembly.cpp:657)
    for (uint32_t e = 0; e < m->n_elem; e++) {
        const uint32_t a = m->dof_ptr[e];
        const int nf = (int)(m->dof_ptr[e + 1] - a);
        const int msz = nf * s;
        const double sc = m->scale ? m->scale[e] : 1.0;
        const double *K = ke + ke_off[e];
        for (int j = 0; j < nf; j++)
            for (int k = 0; k < nf; k++) {
                const int64_t blk = find_block(acc, column_index, m->dof_ids[a + j], m->dof_ids[a + k]);
                if (blk < 0) return -3;
                for (int c = 0; c < s; c++)
                    for (int r = 0; r < s; r++) {
                        const size_t pos = (size_t)blk * bs + c * cl + r;
                        const double y = sc * K[(size_t)(j * s + r) * msz + k * s + c] - comp[pos];
                        const double t = array[pos] + y;
                        comp[pos] = (t - array[pos]) - y;
                        array[pos] = t;
                    }
            }
    }
    return 0;
}

extern "C" int oracle_dirichlet(int32_t stride, uint32_t n_rows, const uint32_t *row_size,
                                const uint32_t *column_index, double *array, uint32_t n_bc, const uint32_t *ids,
                                const double *values, const uint8_t *kinds, double *rhs)
{
    const int s = stride, cl = s + s % 2, bs = s * cl;
    const uint64_t n = (uint64_t)n_rows * s;
    std::vector<uint64_t> acc = row_starts(n_rows, row_size);
    // Displacement multipliers, sorted by id (std::sort in make_final,
    // solvers/assembly.cpp:428; ids are unique, setPointAlong erases duplicates).
    std::vector<int8_t> fixed(n, 0);
    std::vector<double> val(n, 0.0);
    for (uint32_t i = 0; i < n_bc; i++) {
        if (ids[i] >= n) return -4;
        if (kinds && kinds[i] == 1) continue;
        fixed[ids[i]] = 1;
        val[ids[i]] = values[i];
    }
    // Row by row, blocks in column order, constrained columns in id order: the
    // accumulation order of solvers/assembly.cpp:137-249.  A free row subtracts
    // value * A[row][col] for each constrained column and the entry is zeroed; a
    // constrained row becomes the unit row and its rhs the imposed value.
    for (uint32_t k = 0; k < n_rows; k++) {
        for (uint64_t p = acc[k]; p < acc[k + 1]; p++) {
            const uint32_t cb = column_index[p];
            double *blk = array + p * bs;
            for (int r = 0; r < s; r++) {
                const uint64_t row = (uint64_t)k * s + r;
                if (fixed[row]) {
                    for (int c = 0; c < s; c++) blk[c * cl + r] = ((uint64_t)cb * s + c == row) ? 1.0 : 0.0;
                    continue;
                }
                for (int c = 0; c < s; c++) {
                    const uint64_t col = (uint64_t)cb * s + c;
                    if (!fixed[col]) continue;
                    rhs[row] -= val[col] * blk[c * cl + r];
                    blk[c * cl + r] = 0.0;
                }
            }
        }
    }
    for (uint64_t i = 0; i < n; i++)
        if (fixed[i]) rhs[i] = val[i];
    // SET_FORCE_* multipliers are added after elimination (solvers/assembly.cpp:277-283).
    for (uint32_t i = 0; i < n_bc; i++)
        if (kinds && kinds[i] == 1) rhs[ids[i]] += values[i];
    return 0;
}

namespace {

struct Csr {
    int s, cl, bs;
    uint32_t nb;
    std::vector<uint64_t> acc;
    const uint32_t *col;
    const double *a;
};

// CoordinateIndexedSparseMatrix::inner_product for one block row, Kahan per
// output component (sparse/sparse_matrix.h:235-333).  dest holds the initial
// value (0, or -b for assign(r, A*x - b), sparse/sparse_matrix.cpp:462-505).
inline void row_product(const Csr &A, uint32_t k, const double *x, double *dest)
{
    double comp[3] = {0, 0, 0};
    for (uint64_t p = A.acc[k]; p < A.acc[k + 1]; p++) {
        const double *blk = A.a + p * A.bs;
        const double *v = x + (uint64_t)A.col[p] * A.s;
        for (int c = 0; c < A.s; c++)
            for (int r = 0; r < A.s; r++) {
                const double toAdd = blk[c * A.cl + r] * v[c] - comp[r];
                const double tot = dest[r] + toAdd;
                comp[r] = (tot - dest[r]) - toAdd;
                dest[r] = tot;
            }
    }
}

void spmv(const Csr &A, const double *x, const double *y0, double *y, double sign_y0)
{
#pragma omp parallel for schedule(static)
    for (int64_t k = 0; k < (int64_t)A.nb; k++) {
        double *d = y + (uint64_t)k * A.s;
        for (int r = 0; r < A.s; r++) d[r] = y0 ? sign_y0 * y0[(uint64_t)k * A.s + r] : 0.0;
        row_product(A, (uint32_t)k, x, d);
    }
}

// Kahan dot product (utilities/matrixops.h:246-280), made deterministic: Kahan
// partials over fixed chunks, summed in chunk order.
double kdot(const double *u, const double *v, int64_t n)
{
    const int64_t chunk = 1 << 14;
    const int64_t nch = (n + chunk - 1) / chunk;
    std::vector<double> part(nch > 0 ? nch : 1, 0.0);
#pragma omp parallel for schedule(static)
    for (int64_t c = 0; c < nch; c++) {
        double res = 0, comp = 0;
        const int64_t e = std::min(n, (c + 1) * chunk);
        for (int64_t i = c * chunk; i < e; i++) {
            const double y = u[i] * v[i] - comp;
            const double t = res + y;
            comp = (t - res) - y;
            res = t;
        }
        part[c] = res;
    }
    double s = 0;
    for (int64_t c = 0; c < nch; c++) s += part[c];
    return s;
}

Csr make_csr(int32_t stride, uint32_t n_rows, const uint32_t *row_size, const uint32_t *column_index,
             const double *array)
{
    Csr A;
    A.s = stride;
    A.cl = stride + stride % 2;
    A.bs = A.s * A.cl;
    A.nb = n_rows;
    A.acc = row_starts(n_rows, row_size);
    A.col = column_index;
    A.a = array;
    return A;
}

// InverseDiagonal (solvers/inversediagonal.cpp:48-67, sparse/sparse_matrix.cpp:216-231).
std::vector<double> inverse_diagonal(const Csr &A)
{
    const uint64_t n = (uint64_t)A.nb * A.s;
    std::vector<double> d(n, 0.0);
    for (uint32_t k = 0; k < A.nb; k++) {
        const int64_t p = find_block(A.acc, A.col, k, k);
        for (int r = 0; r < A.s; r++) {
            const double v = p >= 0 ? A.a[(uint64_t)p * A.bs + r * A.cl + r] : 0.0;
            d[(uint64_t)k * A.s + r] = std::abs(v) > 1e-12 ? 1.0 / v : 0.0;
        }
    }
    return d;
}

}  // namespace

extern "C" int oracle_spmv(int32_t stride, uint32_t n_rows, const uint32_t *row_size, const uint32_t *column_index,
                           const double *array, const double *x, const double *y0, double *y)
{
    Csr A = make_csr(stride, n_rows, row_size, column_index, array);
    spmv(A, x, y0, y, 1.0);
    return 0;
}

extern "C" int oracle_cg_amie(int32_t stride, uint32_t n_rows, const uint32_t *row_size,
                              const uint32_t *column_index, const double *array, const double *b, double *x,
                              double eps, int32_t nssor, int64_t maxit, int64_t *iterations)
{
    Csr A = make_csr(stride, n_rows, row_size, column_index, array);
    const int64_t n = (int64_t)n_rows * stride;
    *iterations = 0;
    // Homogeneous problem (solvers/conjugategradient.cpp:74-78): x stays 0.
    double bmax = 0;
    for (int64_t i = 0; i < n; i++) bmax = std::max(bmax, std::abs(b[i]));
    if (bmax < eps * eps) {
        std::fill(x, x + n, 0.0);
        return 0;
    }
    const std::vector<double> Dinv = inverse_diagonal(A);
    const double realeps = std::max(1e-12, eps);
    const int64_t Maxit = maxit >= 0 ? maxit : n / 2;
    std::vector<double> r(n), z(n), p(n), q(n), xmin(x, x + n), rc(n), xc(n);
    int64_t nit = 0;
    double perr = 1, errmin = 0;
    auto precond = [&](const std::vector<double> &v, std::vector<double> &t) {
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < n; i++) t[i] = v[i] * Dinv[i];
    };
    auto jacobi_step = [&]() {  // x -= D^-1 (A x - b), Kahan (solvers/conjugategradient.cpp:139-148)
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < n; i++) {
            const double yx = -r[i] - xc[i];
            const double xt = x[i] + yx;
            xc[i] = (xt - x[i]) - yx;
            x[i] = xt;
        }
    };
    auto kahan_update = [&](double alpha) {  // solvers/conjugategradient.cpp:198-209
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < n; i++) {
            const double yr = -q[i] * alpha - rc[i];
            const double yx = p[i] * alpha - xc[i];
            const double rt = r[i] + yr;
            const double xt = x[i] + yx;
            rc[i] = (rt - r[i]) - yr;
            xc[i] = (xt - x[i]) - yx;
            r[i] = rt;
            x[i] = xt;
        }
    };
    while (nit < Maxit) {
        int64_t localnit = 0;
        std::fill(rc.begin(), rc.end(), 0.0);
        std::fill(xc.begin(), xc.end(), 0.0);
        if (nssor) {  // pre-smoothing (solvers/conjugategradient.cpp:124-151)
            double err = 2, perr_s = 0;
            int iter = 0;
            while (iter++ < nssor && err > realeps) {
                spmv(A, x, b, r.data(), -1.0);
                perr_s = err;
                err = std::sqrt(kdot(r.data(), r.data(), n));
                if (err > perr_s) break;
                precond(r, r);
                jacobi_step();
            }
            std::fill(xc.begin(), xc.end(), 0.0);
        }
        spmv(A, x, b, r.data(), -1.0);
        for (int64_t i = 0; i < n; i++) r[i] = -r[i];
        const double err0 = std::sqrt(kdot(r.data(), r.data(), n));
        if (std::isnan(err0)) { *iterations = nit; return 2; }
        if (nit == 0) errmin = err0;
        if (err0 < realeps) { *iterations = nit; return 0; }
        perr = err0;
        precond(r, z);
        p = z;
        spmv(A, p.data(), nullptr, q.data(), 0.0);
        double last_rho = kdot(r.data(), z.data(), n);
        double pq = kdot(q.data(), p.data(), n);
        if (std::abs(pq) < 1e-12 * last_rho) { *iterations = nit; return 0; }
        double alpha = last_rho / pq;
        kahan_update(alpha);
        double rho = 0, beta = 0;
        while (std::sqrt(std::abs(last_rho)) > realeps && localnit < n) {  // :218-257
            localnit++;
            precond(r, z);
            rho = kdot(r.data(), z.data(), n);
            beta = rho / last_rho;
#pragma omp parallel for schedule(static)
            for (int64_t i = 0; i < n; i++) p[i] = p[i] * beta + z[i];
            spmv(A, p.data(), nullptr, q.data(), 0.0);
            pq = kdot(q.data(), p.data(), n);
            if (std::abs(pq) < 1e-24 * rho) { last_rho = rho; break; }
            alpha = rho / pq;
            kahan_update(alpha);
            last_rho = rho;
            nit++;
        }
        spmv(A, x, b, r.data(), -1.0);
        double err = std::sqrt(kdot(r.data(), r.data(), n));
        if (err < errmin) { errmin = std::sqrt(std::abs(rho)); xmin.assign(x, x + n); }
        if (nssor) {  // post-smoothing (solvers/conjugategradient.cpp:274-302)
            int64_t iters = 0;
            while (err > realeps && iters++ < n) {
                spmv(A, x, b, r.data(), -1.0);
                precond(r, r);
                jacobi_step();
                const double perr_p = err;
                err = std::sqrt(kdot(r.data(), r.data(), n));
                if (err > perr_p) break;
                xmin.assign(x, x + n);
            }
            if (iters > 2) std::copy(xmin.begin(), xmin.end(), x);
        }
        if (std::min(err, std::sqrt(std::abs(last_rho))) < std::sqrt(realeps)) { *iterations = nit; return 0; }
    }
    (void)perr;
    *iterations = nit;
    return 1;
}

extern "C" int oracle_pcg(int32_t stride, uint32_t n_rows, const uint32_t *row_size, const uint32_t *column_index,
                          const double *array, const double *b, double *x, double rtol, int64_t maxit,
                          int64_t *iterations, double *relres)
{
    Csr A = make_csr(stride, n_rows, row_size, column_index, array);
    const int64_t n = (int64_t)n_rows * stride;
    const std::vector<double> Dinv = inverse_diagonal(A);
    std::vector<double> r(n), z(n), p(n), q(n);
    const double bnorm = std::sqrt(kdot(b, b, n));
    *iterations = 0;
    if (bnorm == 0) {
        std::fill(x, x + n, 0.0);
        *relres = 0;
        return 0;
    }
    int64_t it = 0;
    // Restart from the true residual when the recursive one has converged but
    // the true one has not (at most a few times).
    for (int restart = 0; restart < 8; restart++) {
        spmv(A, x, b, r.data(), -1.0);
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < n; i++) { r[i] = -r[i]; z[i] = r[i] * Dinv[i]; p[i] = z[i]; }
        double rz = kdot(r.data(), z.data(), n);
        double rr = kdot(r.data(), r.data(), n);
        if (std::sqrt(rr) <= rtol * bnorm) break;
        while (it < maxit) {
            spmv(A, p.data(), nullptr, q.data(), 0.0);
            const double pq = kdot(p.data(), q.data(), n);
            if (pq == 0) break;
            const double alpha = rz / pq;
#pragma omp parallel for schedule(static)
            for (int64_t i = 0; i < n; i++) {
                x[i] += alpha * p[i];
                r[i] -= alpha * q[i];
                z[i] = r[i] * Dinv[i];
            }
            it++;
            rr = kdot(r.data(), r.data(), n);
            const double rzn = kdot(r.data(), z.data(), n);
            if (std::isnan(rr)) { *iterations = it; *relres = NAN; return 2; }
            if (std::sqrt(rr) <= rtol * bnorm) break;
            const double beta = rzn / rz;
            rz = rzn;
#pragma omp parallel for schedule(static)
            for (int64_t i = 0; i < n; i++) p[i] = z[i] + beta * p[i];
        }
        if (it >= maxit) break;
    }
    spmv(A, x, b, r.data(), -1.0);
    *relres = std::sqrt(kdot(r.data(), r.data(), n)) / bnorm;
    *iterations = it;
    return *relres <= rtol ? 0 : 1;
}
