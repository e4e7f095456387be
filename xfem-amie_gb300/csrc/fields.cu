// fields.cu -- strain / stress recovery on the device from the device-resident
// solution.
//
// Reference (paths relative to the AMIE source tree):
//   strain   FeatureTree::strainFromDisplacements  features/features.cpp:4223
//   stress   FeatureTree::stressFromDisplacements  features/features.cpp:3424
#include "element.cuh"

#include <algorithm>
#include <vector>

namespace amie {

// Weighted average over the element's Gauss points of the strain
// sum_f B_f^T u_f (Voigt, engineering shear) and of the stress C_eff strain.
template <int DIM>
__global__ void k_element_fields(MeshView m, const double *x, double *strain, double *stress)
{
    constexpr int NV = DIM == 2 ? 3 : 6;
    const uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= m.n_elem) return;
    const int kind = m.kind[e];
    const int nshape = nshape_of(kind);
    const uint32_t f0 = m.enr_ptr ? m.enr_ptr[e] : 0, f1 = m.enr_ptr ? m.enr_ptr[e + 1] : 0;
    const int nf = nshape + (int)(f1 - f0);
    const uint32_t d0 = m.dof_ptr[e];
    double Je[DIM * DIM];
#pragma unroll
    for (int i = 0; i < DIM * DIM; i++) Je[i] = m.jinv[(size_t)e * DIM * DIM + i];
    const uint32_t g0 = m.gp_ptr[e], g1 = m.gp_ptr[e + 1];
    const bool explicit_gp = g1 > g0;
    const bool moved = explicit_gp && m.moved && m.moved[e];
    const int ngp = explicit_gp ? (int)(g1 - g0) : (kind == AMIE_TRI6 ? 4 : 1);
    const double inv_det = 1.0 / det_small<DIM>(Je);
    double eps[NV], wsum = 0.0;
#pragma unroll
    for (int k = 0; k < NV; k++) eps[k] = 0.0;
    for (int g = 0; g < ngp; g++) {
        double p[3], w;
        if (explicit_gp) {
            const double *gp = m.gp + (size_t)(g0 + g) * (DIM + 1);
            p[0] = gp[0]; p[1] = gp[1]; p[2] = DIM == 3 ? gp[2] : 0.0;
            w = gp[DIM];
        } else {
            default_rule(kind, g, p, &w);
            w *= inv_det;
        }
        const double *J = moved ? m.jinv_gp + (size_t)(g0 + g) * DIM * DIM : Je;
        double eg[NV];
#pragma unroll
        for (int k = 0; k < NV; k++) eg[k] = 0.0;
        for (int f = 0; f < nf; f++) {
            double lg[3] = {0.0, 0.0, 0.0};
            if (f < nshape) {
                shape_grad(kind, f, p[0], p[1], lg);
            } else {
                enr_local_grad<DIM>(m, f0 + (f - nshape), g, p, lg);
            }
            double d[3];
            phys_grad<DIM>(J, lg, d);
            const double *u = x + (uint64_t)m.dof_ids[d0 + f] * DIM;
            if (DIM == 2) {
                eg[0] += d[0] * u[0];
                eg[1] += d[1] * u[1];
                eg[2] += d[1] * u[0] + d[0] * u[1];
            } else {
                eg[0] += d[0] * u[0];
                eg[1] += d[1] * u[1];
                eg[2] += d[2] * u[2];
                eg[3] += d[2] * u[1] + d[1] * u[2];
                eg[4] += d[2] * u[0] + d[0] * u[2];
                eg[5] += d[1] * u[0] + d[0] * u[1];
            }
        }
#pragma unroll
        for (int k = 0; k < NV; k++) eps[k] += w * eg[k];
        wsum += w;
    }
    const double inv = wsum != 0.0 ? 1.0 / wsum : 0.0;
    const double cs = m.cscale ? m.cscale[e] : 1.0;
    const double *C = m.cmat_table + (size_t)m.mat[e] * NV * NV;
#pragma unroll
    for (int k = 0; k < NV; k++) eps[k] *= inv;
    // real stress C (eps - eps0) with an imposed strain (REAL_STRESS_FIELD)
    double el[NV];
#pragma unroll
    for (int k = 0; k < NV; k++) el[k] = m.imposed ? eps[k] - m.imposed[(size_t)e * NV + k] : eps[k];
#pragma unroll
    for (int k = 0; k < NV; k++) {
        double s = 0.0;
#pragma unroll
        for (int l = 0; l < NV; l++) s += C[k * NV + l] * el[l];
        if (strain) strain[(size_t)e * NV + k] = eps[k];
        if (stress) stress[(size_t)e * NV + k] = cs * s;
    }
}

// Per-CTA sums of v_e f_e (nv components) and v_e, v_e the element's area
// (2D: 0.5 / |det J^-1|, the triangle of its corners) or volume (3D:
// (1/6) / |det J^-1|), J^-1 at the centroid.  Each thread Kahan-sums its
// elements in index order; the CTA adds its threads in a fixed tree.
// parts: [gridDim.x][nv + 1].
template <int DIM>
__global__ void __launch_bounds__(256) k_average_parts(uint32_t n_elem, const double *jinv, const double *field,
                                                       double *parts)
{
    constexpr int NV = DIM == 2 ? 3 : 6;
    __shared__ double sh[256];
    double acc[NV + 1], comp[NV + 1];
#pragma unroll
    for (int k = 0; k <= NV; k++) acc[k] = comp[k] = 0.0;
    for (uint32_t e = blockIdx.x * 256 + threadIdx.x; e < n_elem; e += gridDim.x * 256) {
        double J[DIM * DIM];
#pragma unroll
        for (int i = 0; i < DIM * DIM; i++) J[i] = jinv[(size_t)e * DIM * DIM + i];
        const double v = (DIM == 2 ? 0.5 : 1.0 / 6.0) / fabs(det_small<DIM>(J));
#pragma unroll
        for (int k = 0; k <= NV; k++) {
            const double term = (k < NV ? v * field[(size_t)e * NV + k] : v) - comp[k];
            const double sum = acc[k] + term;
            comp[k] = (sum - acc[k]) - term;
            acc[k] = sum;
        }
    }
#pragma unroll
    for (int k = 0; k <= NV; k++) {
        sh[threadIdx.x] = acc[k];
        __syncthreads();
        for (int o = 128; o > 0; o >>= 1) {
            if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
            __syncthreads();
        }
        if (threadIdx.x == 0) parts[(size_t)blockIdx.x * (NV + 1) + k] = sh[0];
        __syncthreads();
    }
}

MeshView mesh_view(amie_topo *t);

// t->strain = the element strains of the device solution (launch only).
amie_status element_strain_async(amie_topo *t)
{
    if (!t->strain.p) AMIE_TRY(t->strain.alloc(t->ctx, (size_t)t->n_elem * t->nv));
    const MeshView m = mesh_view(t);
    const unsigned blocks = (t->n_elem + 127) / 128;
    if (t->dim == 2) k_element_fields<2><<<blocks, 128, 0, t->ctx->stream>>>(m, t->x.p, t->strain.p, nullptr);
    else k_element_fields<3><<<blocks, 128, 0, t->ctx->stream>>>(m, t->x.p, t->strain.p, nullptr);
    AMIE_LAUNCHED();
    AMIE_CUDA(cudaGetLastError());
    return AMIE_OK;
}

}  // namespace amie

using namespace amie;

extern "C" amie_status amie_element_fields(amie_topo *t, double *strain, double *stress)
{
    if (!t) return AMIE_BAD_INPUT;
    AMIE_CUDA(cudaSetDevice(t->ctx->device));
    cudaStream_t st = t->ctx->stream;
    const int nv = t->nv;
    if (!t->strain.p) AMIE_TRY(t->strain.alloc(t->ctx, (size_t)t->n_elem * nv));
    DevArray<double> dstress;
    if (stress) AMIE_TRY(dstress.alloc(t->ctx, (size_t)t->n_elem * nv));
    MeshView m = mesh_view(t);
    const unsigned blocks = (t->n_elem + 127) / 128;
    if (t->dim == 2) k_element_fields<2><<<blocks, 128, 0, st>>>(m, t->x.p, t->strain.p, dstress.p);
    else k_element_fields<3><<<blocks, 128, 0, st>>>(m, t->x.p, t->strain.p, dstress.p);
    AMIE_LAUNCHED();
    if (strain) AMIE_CUDA(cudaMemcpyAsync(strain, t->strain.p, (size_t)t->n_elem * nv * 8, cudaMemcpyDeviceToHost, st));
    if (stress) AMIE_CUDA(cudaMemcpyAsync(stress, dstress.p, (size_t)t->n_elem * nv * 8, cudaMemcpyDeviceToHost, st));
    AMIE_CUDA(cudaStreamSynchronize(st));
    return AMIE_OK;
}

extern "C" amie_status amie_average_field(amie_topo *t, int32_t field, double *avg, double *measure)
{
    if (!t || !avg || (field != AMIE_FIELD_STRAIN && field != AMIE_FIELD_STRESS)) return AMIE_BAD_INPUT;
    AMIE_CUDA(cudaSetDevice(t->ctx->device));
    cudaStream_t st = t->ctx->stream;
    const int nv = t->nv;
    const uint32_t E = t->n_elem;
    if (!t->strain.p) AMIE_TRY(t->strain.alloc(t->ctx, (size_t)E * nv));
    DevArray<double> dstress, parts;
    if (field == AMIE_FIELD_STRESS) AMIE_TRY(dstress.alloc(t->ctx, (size_t)E * nv));
    const int grid = std::max(1, std::min<int>(t->ctx->num_sms * 4, (int)((E + 255) / 256)));
    AMIE_TRY(parts.alloc(t->ctx, (size_t)grid * (nv + 1)));
    const MeshView m = mesh_view(t);
    const int blocks = (int)((E + 127) / 128);
    const double *f = field == AMIE_FIELD_STRESS ? dstress.p : t->strain.p;
    if (t->dim == 2) {
        k_element_fields<2><<<blocks, 128, 0, st>>>(m, t->x.p, t->strain.p, dstress.p);
        k_average_parts<2><<<grid, 256, 0, st>>>(E, t->jinv.p, f, parts.p);
    } else {
        k_element_fields<3><<<blocks, 128, 0, st>>>(m, t->x.p, t->strain.p, dstress.p);
        k_average_parts<3><<<grid, 256, 0, st>>>(E, t->jinv.p, f, parts.p);
    }
    g_launches += 2;
    std::vector<double> h((size_t)grid * (nv + 1));
    AMIE_CUDA(cudaMemcpyAsync(h.data(), parts.p, h.size() * 8, cudaMemcpyDeviceToHost, st));
    AMIE_CUDA(cudaStreamSynchronize(st));
    // the CTA partials in index order (Kahan), then the reference's division
    std::vector<double> acc(nv + 1, 0.0), comp(nv + 1, 0.0);
    for (int b = 0; b < grid; b++)
        for (int k = 0; k <= nv; k++) {
            const double term = h[(size_t)b * (nv + 1) + k] - comp[k];
            const double sum = acc[k] + term;
            comp[k] = (sum - acc[k]) - term;
            acc[k] = sum;
        }
    const double w = acc[nv];
    for (int k = 0; k < nv; k++) avg[k] = w > 1e-24 ? acc[k] / w : acc[k];
    if (measure) *measure = w;
    return AMIE_OK;
}
