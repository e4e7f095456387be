// fields.cu -- strain / stress recovery and the scalar damage update of a
// damage loop, on the device, from the device-resident solution.
//
// Reference (paths relative to the AMIE source tree):
//   strain   FeatureTree::strainFromDisplacements  features/features.cpp:4223
//   stress   FeatureTree::stressFromDisplacements  features/features.cpp:3424
//   damage   StiffnessAndFracture::step            physics/stiffness_and_fracture.cpp:81-90,
//            the (1-d) C of IsotropicLinearDamage::apply (physics/damagemodels/isotropiclineardamage.cpp:39-46),
//            a Mazars equivalent strain (physics/fracturecriteria/mazars.cpp:153) with
//            exponential softening d = 1 - (eps0/eq) exp(-B (eq - eps0)).
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
                const uint32_t fj = f0 + (f - nshape);
                const uint64_t off = (uint64_t)m.enr_data[fj] + g;
                if (m.enr_type[fj] == AMIE_ENR_HEAVISIDE) {
                    const int v = m.enr_vertex[fj];
                    const double jump = (double)m.enr_jump[off];
                    const double gx[3] = {0.0, -1.0, 1.0}, gy[3] = {1.0, -1.0, 0.0};
                    lg[0] = gx[v] * jump;
                    lg[1] = gy[v] * jump;
                } else {
#pragma unroll
                    for (int c = 0; c < DIM; c++) lg[c] = m.enr_grad[off * DIM + c];
                }
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

// Mazars equivalent strain from the positive principal strains (2D plane
// strain tensor [exx, exy/2; exy/2, eyy]), exponential softening, irreversible
// damage, C factor = base * (1 - d).
__global__ void k_damage(uint32_t n_elem, const double *strain, amie_damage_params prm, double *damage,
                         const double *cscale_base, double *cscale, uint32_t *n_changed)
{
    const uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n_elem) return;
    const double exx = strain[(size_t)e * 3], eyy = strain[(size_t)e * 3 + 1], gxy = strain[(size_t)e * 3 + 2];
    const double c = 0.5 * (exx + eyy);
    const double rad = sqrt(0.25 * (exx - eyy) * (exx - eyy) + 0.25 * gxy * gxy);
    const double e1 = fmax(c + rad, 0.0), e2 = fmax(c - rad, 0.0);
    const double eq = sqrt(e1 * e1 + e2 * e2);
    double dn = 0.0;
    if (eq > prm.eps0) dn = 1.0 - (prm.eps0 / eq) * exp(-prm.softening * (eq - prm.eps0));
    const double dold = damage[e];
    const double d = fmin(prm.d_max, fmax(dold, dn));
    damage[e] = d;
    cscale[e] = (cscale_base ? cscale_base[e] : 1.0) * (1.0 - d);
    if (d - dold > prm.change_tol) atomicAdd(n_changed, 1u);
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

extern "C" amie_status amie_damage_step(amie_topo *t, const amie_damage_params *prm, uint32_t *n_changed,
                                        double *damage_out)
{
    if (!t || !prm) return AMIE_BAD_INPUT;
    if (t->dim != 2) {
        set_error("the damage update is implemented for 2D meshes");
        return AMIE_BAD_INPUT;
    }
    AMIE_CUDA(cudaSetDevice(t->ctx->device));
    cudaStream_t st = t->ctx->stream;
    const uint32_t E = t->n_elem;
    if (!t->damage.p) {
        AMIE_TRY(t->damage.alloc(t->ctx, E));
        AMIE_CUDA(cudaMemsetAsync(t->damage.p, 0, (size_t)E * 8, st));
        if (t->has_cscale) {   // keep the caller's factor (per-element modulus) as the base
            AMIE_TRY(t->cscale_base.alloc(t->ctx, E));
            AMIE_CUDA(cudaMemcpyAsync(t->cscale_base.p, t->cscale.p, (size_t)E * 8, cudaMemcpyDeviceToDevice, st));
        }
        if (!t->cscale.p) AMIE_TRY(t->cscale.alloc(t->ctx, E));
        t->has_cscale = true;
    }
    if (!t->strain.p) AMIE_TRY(t->strain.alloc(t->ctx, (size_t)E * t->nv));
    DevArray<uint32_t> counter;
    AMIE_TRY(counter.alloc(t->ctx, 1));
    AMIE_CUDA(cudaMemsetAsync(counter.p, 0, 4, st));
    MeshView m = mesh_view(t);
    const unsigned blocks = (E + 127) / 128;
    k_element_fields<2><<<blocks, 128, 0, st>>>(m, t->x.p, t->strain.p, nullptr);
    k_damage<<<blocks, 128, 0, st>>>(E, t->strain.p, *prm, t->damage.p, t->cscale_base.p, t->cscale.p, counter.p);
    g_launches += 2;
    uint32_t changed = 0;
    AMIE_CUDA(cudaMemcpyAsync(&changed, counter.p, 4, cudaMemcpyDeviceToHost, st));
    if (damage_out) AMIE_CUDA(cudaMemcpyAsync(damage_out, t->damage.p, (size_t)E * 8, cudaMemcpyDeviceToHost, st));
    AMIE_CUDA(cudaStreamSynchronize(st));
    if (n_changed) *n_changed = changed;
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
