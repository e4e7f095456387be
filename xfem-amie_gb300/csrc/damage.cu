// damage.cu -- non-local Mazars damage of StiffnessAndFracture on the device,
// linear triangles in plane stress.
//
// Reference (paths relative to the AMIE source tree):
//   neighbourhoods  FractureCriterion::initialiseCache (physics/fracturecriteria/fracturecriterion.cpp:171-196)
//                   through Mesh::generateCache (mesher/mesh.h:546-664): the elements whose centre
//                   lies in the circle R_e 2.5 + 1.5 r_e (smoothing) or max(6 R_e, 4 r_e) 2.5 + r_e
//                   (neighbourhood maxima) around the element's centre, R_e = max(R, 1.1 r_e),
//                   r_e the circumradius; smoothing weight mean_v max(w(v) a, 0) of the
//                   QUARTIC_COMPACT kernel w (fracturecriterion.cpp:46-52) at the neighbour's
//                   vertices, normalised over the neighbourhood
//   grade           FractureCriterion::step (fracturecriterion.cpp:534-560) ->
//                   Mesh::getSmoothedFields (mesher/mesh.h:1384-1790), toPrincipal
//                   (elements/integrable_entity.cpp:475-590), NonLocalMazars::gradeAtTime
//                   (physics/fracturecriteria/mazars.cpp:73-147)
//   update          FiberBasedIsotropicLinearDamage::step (physics/damagemodels/fiberbasedisotropiclineardamage.cpp:59-98)
//                   with FractureCriterion::getMaxScoreInNeighbourhood (fracturecriterion.cpp:251-280),
//                   elements stepped in mesh order (features/features.cpp:5062-5088)
//   load step       FeatureTree::stepInternal's loop (features/features.cpp:6188-6248)
//
// This file is compiled without floating-point contraction so that the
// grading arithmetic is the reference's operation for operation; only exp and
// the summation order of the neighbourhoods (cell order here, Delaunay-tree
// order there) differ, at the level of the last bit.
#include "element.cuh"

#include <cub/cub.cuh>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <vector>

namespace amie {

amie_status element_strain_async(amie_topo *t);   // fields.cu: t->strain = element strain from t->x
MeshView mesh_view(amie_topo *t);

constexpr double kPointTolerance = 1e-12;   // POINT_TOLERANCE (geometry/geometry_base.h:292)
constexpr double kKernelSize = 2.5;         // getSmoothingKernelSize (fracturecriterion.cpp:29-31)
constexpr int kMaxNewlyFractured = 1024;    // commit kernel: newly fractured elements tracked in shared memory

struct DamageConst {
    double threshold, nu, B_t, B_c, A_c;                 // NonLocalMazars
    double radius, tol, fibre, cutoff, residual;         // criterion radius, scoreTolerance, damage model
};

// Uniform grid of the element centres (host-built counting sort).
struct Grid {
    double x0, y0, h;
    int nx, ny;
    const uint32_t *cell_start;   // [nx*ny + 1]
    const uint32_t *items;        // element indices, cell by cell, index order inside a cell
};

struct DamageState {
    amie_damage_law law{};
    DamageConst k{};
    uint32_t n_elem = 0;
    DevArray<double> xy, centre, radius, area, gpw;
    DevArray<uint64_t> nb_ptr;
    DevArray<uint32_t> nb_idx;
    DevArray<double> nb_coef;
    DevArray<double> state, score, smoothed, base;
    bool has_base = false;
    DevArray<uint8_t> met_flag, decision, cub_tmp;
    DevArray<uint32_t> iota, met, counters;   // counters: [0] met, [1] changed, [2] damaged, [3] fractured
    DevArray<double> nmax;
    size_t cub_bytes = 0;
    bool dirty = false;   // damage changed since the stiffness was last assembled
    // the centres' grid of the set-up, kept for the bounded grading: per cell the
    // largest equivalent strain of its unfractured elements (float bits, rounded up)
    Grid grid{};
    DevArray<uint32_t> cell_start, cell_items, cell_of, cell_max;
    DevArray<unsigned long long> n_smoothed;   // elements smoothed by the gradings since the last reset
};

namespace {

__device__ __forceinline__ bool in_circle(double cx, double cy, double r, double r2, double x, double y)
{
    // Circle::in (geometry/geometry_2D.cpp:1472-1484)
    if (x < cx - r * 1.01 || x > cx + r * 1.01 || y < cy - r * 1.01 || y > cy + r * 1.01) return false;
    const double dx = x - cx, dy = y - cy;
    return dx * dx + dy * dy < r2;
}

__host__ __device__ __forceinline__ double reff(double R, double r) { return R < r * 1.1 ? r * 1.1 : R; }
__host__ __device__ __forceinline__ double smoothing_radius(double Re, double r) { return Re * kKernelSize + r * 1.5; }
__host__ __device__ __forceinline__ double neighbourhood_radius(double Re, double r)
{
    return (Re * 6. < r * 4. ? r * 4. : Re * 6.) * kKernelSize + r;
}

// QUARTIC_COMPACT kernel centred on (cx, cy): rrn = |p - c|^2 / R^2 / 2, (rrn - 1)^2 where 1 - rrn >= 0.
__device__ __forceinline__ double quartic(double x, double y, double cx, double cy, double R)
{
    const double dx = x - cx, dy = y - cy;
    double rrn = (dx * dx + dy * dy) / (R * R);
    rrn = rrn / 2.;
    const double pos = (1. - rrn) >= 0 ? 1. : 0.;
    return (rrn - 1.) * (rrn - 1.) * pos;
}

// toPrincipal, 2D: SINGLE_OFF_DIAGONAL_VALUES (stress) or DOUBLE_OFF_DIAGONAL_VALUES (strain).
__device__ __forceinline__ void principal(const double *v, bool engineering, double *out)
{
    const double trace = v[0] + v[1];
    const double det = engineering ? v[0] * v[1] - 0.25 * v[2] * v[2] : v[0] * v[1] - v[2] * v[2];
    const double delta = sqrt(trace * trace - 4. * det);
    const double angle = 0.5 * atan2(engineering ? 0.5 * v[2] : v[2], v[0] - v[1]);
    if (cos(angle) < 0) {
        out[0] = (trace + delta) * .5;
        out[1] = (trace - delta) * .5;
    } else {
        out[0] = (trace - delta) * .5;
        out[1] = (trace + delta) * .5;
    }
}

// NonLocalMazars::gradeAtTime, 2D plane stress: the branch sets tensionOnly,
// so talpha = 1, calpha = 0.
// The tensile strain norm of gradeAtTime (mazars.cpp:100-112) from principal
// strains: sqrt(<e0>+^2 + <e1>+^2 + <ezz>+^2), ezz = -nu (e0 + e1) / (1 - nu).
// As a function of the strain tensor it is convex (a symmetric convex function
// of the eigenvalues, the positive parts of linear forms under a monotone norm),
// so on a weighted average of strains it is at most the largest value on the
// averaged strains.
__device__ __forceinline__ double mazars_norm(const DamageConst &k, const double *strain)
{
    const double strainzz = -k.nu * (strain[0] + strain[1]) / (1. - k.nu);
    const double p0 = 0.5 * (fabs(strain[0]) + strain[0]);
    const double p1 = 0.5 * (fabs(strain[1]) + strain[1]);
    const double pz = 0.5 * (fabs(strainzz) + strainzz);
    return sqrt(p0 * p0 + p1 * p1 + pz * pz);
}

__device__ __forceinline__ double mazars(const DamageConst &k, const double *stress, const double *strain,
                                         double dama_predict)
{
    double gamma = 1.0;
    const double Trtsig = 0.5 * (fabs(stress[0]) + stress[0]) + 0.5 * (fabs(stress[1]) + stress[1]);
    const double Trcsig = fmin(0.0, stress[0]) + fmin(0.0, stress[1]);
    if (Trcsig < -kPointTolerance && fabs(Trtsig / Trcsig) < 1e-8)
        gamma = sqrt(fmin(0.0, stress[0]) * fmin(0.0, stress[0]) + fmin(0.0, stress[1]) * fmin(0.0, stress[1])) /
                (-Trcsig);
    const double maxStrain = gamma * fmax(0.0, mazars_norm(k, strain));
    const double talpha = 1.0, calpha = 1.0 - talpha;
    const double tt = k.threshold < maxStrain ? maxStrain : k.threshold;
    const double t = talpha * (1. - (k.threshold / tt) * exp(-k.B_t * (tt - k.threshold))) +
                     calpha * (1. - (k.threshold * (1 - k.A_c) / tt) - k.A_c * exp(-k.B_c * (tt - k.threshold)));
    const double pseudo = 1.0 < t ? 1.0 : t;
    return pseudo - dama_predict;
}

// Centre (Triangle::computeCenter), circumradius, area (Triangle::area) and the
// one-point Gauss weight (weight times det J) of every element.
__global__ void k_dmg_geometry(MeshView m, const double *xy, double *centre, double *radius, double *area, double *gpw)
{
    const uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= m.n_elem) return;
    const double *p = xy + (size_t)e * 6;
    const double x0 = p[0], y0 = p[1], x1 = p[2], y1 = p[3], x2 = p[4], y2 = p[5];
    centre[2 * e] = ((0. + x0) + x1 + x2) / 3.;
    centre[2 * e + 1] = ((0. + y0) + y1 + y2) / 3.;
    const double d = 2. * (x0 * (y1 - y2) + x1 * (y2 - y0) + x2 * (y0 - y1));
    const double s0 = x0 * x0 + y0 * y0, s1 = x1 * x1 + y1 * y1, s2 = x2 * x2 + y2 * y2;
    const double ux = (s0 * (y1 - y2) + s1 * (y2 - y0) + s2 * (y0 - y1)) / d;
    const double uy = (s0 * (x2 - x1) + s1 * (x0 - x2) + s2 * (x1 - x0)) / d;
    radius[e] = (hypot(x1 - ux, y1 - uy) + hypot(x0 - ux, y0 - uy)) / 2.;
    area[e] = 0.5 * fabs((x0 - x1) * (y0 - y2) - (y0 - y1) * (x0 - x2));
    const uint32_t g0 = m.gp_ptr[e], g1 = m.gp_ptr[e + 1];
    if (g1 > g0) {
        gpw[e] = m.gp[(size_t)g0 * 3 + 2];
    } else {
        double Je[4];
        for (int i = 0; i < 4; i++) Je[i] = m.jinv[(size_t)e * 4 + i];
        gpw[e] = 0.5 * (1.0 / det_small<2>(Je));
    }
}

// Smoothing neighbourhoods: count pass (idx == nullptr) or fill pass.
__global__ void k_dmg_cache(Grid g, uint32_t E, double R, const double *xy, const double *centre,
                            const double *radius, const double *area, const uint64_t *ptr, uint64_t *count,
                            uint32_t *idx, double *raw)
{
    const uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= E) return;
    const double re = radius[e], Re = reff(R, re), rho = smoothing_radius(Re, re);
    const double cx = centre[2 * e], cy = centre[2 * e + 1], r2 = rho * rho;
    const int ix0 = max(0, (int)floor((cx - rho * 1.01 - g.x0) / g.h));
    const int ix1 = min(g.nx - 1, (int)floor((cx + rho * 1.01 - g.x0) / g.h));
    const int iy0 = max(0, (int)floor((cy - rho * 1.01 - g.y0) / g.h));
    const int iy1 = min(g.ny - 1, (int)floor((cy + rho * 1.01 - g.y0) / g.h));
    uint64_t n = 0;
    const uint64_t base = idx ? ptr[e] : 0;
    for (int iy = iy0; iy <= iy1; iy++)
        for (int ix = ix0; ix <= ix1; ix++) {
            const int c = iy * g.nx + ix;
            for (uint32_t q = g.cell_start[c]; q < g.cell_start[c + 1]; q++) {
                const uint32_t j = g.items[q];
                if (!in_circle(cx, cy, rho, r2, centre[2 * j], centre[2 * j + 1])) continue;
                double w = 0;
                for (int v = 0; v < 3; v++)
                    w += fmax(quartic(xy[(size_t)j * 6 + 2 * v], xy[(size_t)j * 6 + 2 * v + 1], cx, cy, Re) * area[j],
                              0.);
                w /= 3;
                if (w < kPointTolerance * kPointTolerance) continue;
                if (idx) {
                    idx[base + n] = j;
                    raw[base + n] = w;
                }
                n++;
            }
        }
    if (!idx) count[e] = n;
}

__global__ void k_dmg_cache_norm(uint32_t E, const uint64_t *ptr, double *coef)
{
    const uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= E) return;
    double tot = 0;
    for (uint64_t k = ptr[e]; k < ptr[e + 1]; k++) tot += coef[k];
    for (uint64_t k = ptr[e]; k < ptr[e + 1]; k++) coef[k] = coef[k] / tot;
}

// FractureCriterion::step of every element: smoothed strain (Kahan, fractured
// neighbours left out; a neighbour whose Gauss weight times cache weight is at
// most POINT_TOLERANCE contributes a zero strain but its weight,
// elements/integrable_entity.cpp:2112-2131), the element's own damaged stress
// from it, principal values, Mazars score (-1 for a fractured element).
//
// Bounded (cell_max != nullptr, smoothed fields not wanted): an element whose
// smoothing cells hold no unfractured element with an equivalent strain above
// the threshold (with a relative margin of 1e-6 for rounding) has a smoothed
// equivalent strain at or below the threshold (mazars_norm is convex and the
// smoothing a weighted average), so gradeAtTime's score is 0 - d whatever the
// smoothed strain: it is formed from zero strains, bit for bit the value of
// the full evaluation, and the smoothing is skipped.  A fractured element's
// score is -1 either way.  Its smoothed fields are then not written.
__global__ void __launch_bounds__(128) k_dmg_grade(uint32_t E, DamageConst k, const double *strain,
                                                   const uint32_t *mat, const double *cmat_table, const double *state,
                                                   const double *area, const double *gpw, const uint64_t *ptr,
                                                   const uint32_t *idx, const double *coef, double *score,
                                                   double *smoothed, Grid grid, const uint32_t *cell_max,
                                                   const double *centre, const double *radius,
                                                   unsigned long long *n_smoothed)
{
    const uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= E) return;
    if (cell_max) {
        const bool fre = state[e] >= k.cutoff;
        float m = 0.f;
        if (!fre) {   // the cells k_dmg_cache searched for this element's neighbours
            const double re = radius[e], Re = reff(k.radius, re), rho = smoothing_radius(Re, re);
            const double cx = centre[2 * e], cy = centre[2 * e + 1];
            const int ix0 = max(0, (int)floor((cx - rho * 1.01 - grid.x0) / grid.h));
            const int ix1 = min(grid.nx - 1, (int)floor((cx + rho * 1.01 - grid.x0) / grid.h));
            const int iy0 = max(0, (int)floor((cy - rho * 1.01 - grid.y0) / grid.h));
            const int iy1 = min(grid.ny - 1, (int)floor((cy + rho * 1.01 - grid.y0) / grid.h));
            for (int iy = iy0; iy <= iy1; iy++)
                for (int ix = ix0; ix <= ix1; ix++) m = fmaxf(m, __uint_as_float(cell_max[iy * grid.nx + ix]));
        }
        if (fre || (double)m * (1. + 1e-6) <= k.threshold) {
            const double zero[2] = {0., 0.};
            score[e] = fre ? -1. : mazars(k, zero, zero, state[e]);
            return;
        }
        const unsigned act = __activemask();
        if ((int)(threadIdx.x & 31) == __ffs(act) - 1) atomicAdd(n_smoothed, (unsigned long long)__popc(act));
    }
    double sc[3] = {0, 0, 0}, corr[3] = {0, 0, 0}, sum = 0;
    for (uint64_t q = ptr[e]; q < ptr[e + 1]; q++) {
        const uint32_t j = idx[q];
        if (state[j] >= k.cutoff) continue;
        const double c = coef[q];
        const double v = area[j] * c;
        const double g = gpw[j];
        const double tot = g * c;
        for (int i = 0; i < 3; i++) {
            const double avg = tot > kPointTolerance ? strain[(size_t)j * 3 + i] * g * c / tot : 0.;
            const double y = avg * v - corr[i];
            const double t = sc[i] + y;
            corr[i] = (t - sc[i]) - y;
            sc[i] = t;
        }
        sum += v;
    }
    for (int i = 0; i < 3; i++) sc[i] = sum > kPointTolerance ? sc[i] / sum : 0.;
    const bool fr = state[e] >= k.cutoff;
    const double f = fr ? k.residual : 1. - state[e];
    const double *C = cmat_table + (size_t)mat[e] * 9;
    const double g = gpw[e];
    double sig[3];
    for (int i = 0; i < 3; i++) {   // Vector * Matrix: column i of the damaged C against the strain
        double s = 0;
        for (int q = 0; q < 3; q++) s = s + (C[q * 3 + i] * f) * sc[q];
        sig[i] = g > kPointTolerance * kPointTolerance ? s * g / g : s * g;
    }
    double ps[2], pe[2];
    principal(sig, false, ps);
    principal(sc, true, pe);
    score[e] = fr ? -1. : mazars(k, ps, pe, state[e]);
    if (cell_max) return;
    smoothed[4 * (size_t)e] = ps[0];
    smoothed[4 * (size_t)e + 1] = ps[1];
    smoothed[4 * (size_t)e + 2] = pe[0];
    smoothed[4 * (size_t)e + 3] = pe[1];
}

// Per grid cell, the largest tensile strain norm of its unfractured elements'
// own strains (rounded up to float; non-negative floats order like their bits).
__global__ void k_dmg_cell_max(uint32_t E, DamageConst k, const double *strain, const double *state,
                               const uint32_t *cell_of, uint32_t *cell_max)
{
    const uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= E || state[e] >= k.cutoff) return;
    double pe[2];
    principal(strain + (size_t)e * 3, true, pe);
    const double f = mazars_norm(k, pe);
    if (f > 0.) atomicMax(cell_max + cell_of[e], __float_as_uint(__double2float_ru(f)));
}

__global__ void k_dmg_met(uint32_t E, const double *score, uint8_t *flag)
{
    const uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e < E) flag[e] = score[e] > 0;
}

__global__ void k_dmg_iota(uint32_t E, uint32_t *v)
{
    const uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e < E) v[e] = e;
}

// Largest score in each met element's neighbourhood with the fractured states
// of the last grade (elements that are not met have scores <= 0 and never
// raise a met element's maximum), and the step decision taken with it.
__global__ void __launch_bounds__(256) k_dmg_nmax(const uint32_t *n_met, const uint32_t *met, DamageConst k,
                                                  const double *centre, const double *radius, const double *score,
                                                  double *nmax, uint8_t *decision)
{
    __shared__ double sx[256], sy[256], ss[256];
    const uint32_t M = *n_met;
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    const bool active = t < M;
    uint32_t i = 0;
    double cx = 0, cy = 0, rho = 0, r2 = 0, nm = 0;
    if (active) {
        i = met[t];
        const double re = radius[i];
        rho = neighbourhood_radius(reff(k.radius, re), re);
        r2 = rho * rho;
        cx = centre[2 * i];
        cy = centre[2 * i + 1];
        nm = score[i];
    }
    for (uint32_t b = 0; b < M; b += 256) {
        __syncthreads();
        if (b + threadIdx.x < M) {
            const uint32_t j = met[b + threadIdx.x];
            sx[threadIdx.x] = centre[2 * j];
            sy[threadIdx.x] = centre[2 * j + 1];
            ss[threadIdx.x] = score[j];
        }
        __syncthreads();
        const uint32_t cnt = min(256u, M - b);
        if (active)
            for (uint32_t q = 0; q < cnt; q++)
                if (in_circle(cx, cy, rho, r2, sx[q], sy[q]) && nm < ss[q]) nm = ss[q];
    }
    if (active) {
        nmax[t] = nm;
        decision[t] = fabs(score[i] - nm) < k.tol;
    }
}

// The damage model's step of the met elements in mesh order, by one warp: an
// element that became fractured earlier in this pass is no longer a candidate
// of the neighbourhood maxima of the elements after it, so their decision is
// re-taken when one such element lies in their neighbourhood.  Increments the
// damage, sets the factor on C and counts the changes.
__global__ void __launch_bounds__(32) k_dmg_commit(const uint32_t *n_met, const uint32_t *met, DamageConst k,
                                                   const double *centre, const double *radius, const double *score,
                                                   const uint8_t *decision, double *state, const double *base,
                                                   double *cscale, uint32_t *n_changed)
{
    __shared__ uint32_t newly[kMaxNewlyFractured];
    const unsigned lane = threadIdx.x;
    const uint32_t M = *n_met;
    uint32_t changed = 0, nn = 0;
    bool overflow = false;
    for (uint32_t t = 0; t < M; t++) {
        const uint32_t i = met[t];
        bool dec = decision[t] != 0;
        if (nn > 0 || overflow) {
            const double re = radius[i];
            const double rho = neighbourhood_radius(reff(k.radius, re), re), r2 = rho * rho;
            const double cx = centre[2 * i], cy = centre[2 * i + 1];
            bool hit = overflow;
            for (uint32_t q = lane; q < nn && !hit; q += 32) {
                const uint32_t j = newly[q];
                hit = in_circle(cx, cy, rho, r2, centre[2 * j], centre[2 * j + 1]);
            }
            if (__any_sync(0xffffffffu, hit)) {
                double nm = score[i];
                for (uint32_t q = lane; q < M; q += 32) {
                    const uint32_t j = met[q];
                    if (state[j] < k.cutoff && in_circle(cx, cy, rho, r2, centre[2 * j], centre[2 * j + 1]) &&
                        nm < score[j])
                        nm = score[j];
                }
                for (int o = 16; o > 0; o >>= 1) {
                    const double other = __shfl_xor_sync(0xffffffffu, nm, o);
                    if (nm < other) nm = other;
                }
                dec = fabs(score[i] - nm) < k.tol;
            }
        }
        if (dec) {
            double s = state[i] + k.fibre;
            if (s > 1) s = 1;
            const bool fr = s >= k.cutoff;
            __syncwarp();
            if (lane == 0) {
                state[i] = s;
                const double f = fr ? k.residual : 1. - s;
                cscale[i] = base ? base[i] * f : f;
                if (fr && nn < kMaxNewlyFractured) newly[nn] = i;
            }
            changed++;
            if (fr) {
                if (nn < kMaxNewlyFractured) nn++;
                else overflow = true;
            }
            __syncwarp();
        }
    }
    if (lane == 0) *n_changed = changed;
}

__global__ void k_dmg_counts(uint32_t E, const double *state, double cutoff, uint32_t *counters)
{
    const uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
    const bool damaged = e < E && state[e] > 0, fractured = e < E && state[e] >= cutoff;
    const unsigned bd = __ballot_sync(0xffffffffu, damaged), bf = __ballot_sync(0xffffffffu, fractured);
    if ((threadIdx.x & 31) == 0) {
        if (bd) atomicAdd(counters + 2, (uint32_t)__popc(bd));
        if (bf) atomicAdd(counters + 3, (uint32_t)__popc(bf));
    }
}

__global__ void k_dmg_factors(uint32_t E, DamageConst k, const double *state, const double *base, double *cscale)
{
    const uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= E) return;
    const double f = state[e] >= k.cutoff ? k.residual : 1. - state[e];
    cscale[e] = base ? base[e] * f : f;
}

unsigned blocks(uint64_t n, unsigned b) { return (unsigned)((n + b - 1) / b); }

amie_status need_damage(amie_topo *t)
{
    if (!t || !t->dmg) {
        set_error("amie_damage_setup has not been called for this topology");
        return AMIE_BAD_INPUT;
    }
    return AMIE_OK;
}

}  // namespace
}  // namespace amie

using namespace amie;

void release_damage(amie_topo *t)
{
    delete t->dmg;
    t->dmg = nullptr;
}

extern "C" amie_status amie_damage_setup(amie_topo *t, const amie_damage_law *law, const double *corners)
{
    if (!t || !law || !corners) return AMIE_BAD_INPUT;
    if (law->model != AMIE_DAMAGE_FIBER_ISOTROPIC) {
        set_error("amie_damage_setup: unknown damage model %d", law->model);
        return AMIE_BAD_INPUT;
    }
    if (!(law->threshold > 0) || !(law->young > 0) || !(law->radius > 0) || !(law->poisson < 1)) {
        set_error("amie_damage_setup: threshold, young and radius must be positive, poisson below 1");
        return AMIE_BAD_INPUT;
    }
    if (t->dim != 2) {
        set_error("amie_damage_setup: the damage path serves 2D meshes (plane stress)");
        return AMIE_BAD_INPUT;
    }
    AMIE_CUDA(cudaSetDevice(t->ctx->device));
    cudaStream_t st = t->ctx->stream;
    const uint32_t E = t->n_elem;
    {   // every element a linear triangle with its one-point rule and no enrichment
        std::vector<uint8_t> kind(E);
        std::vector<uint32_t> gp_ptr(E + 1), enr_ptr;
        AMIE_CUDA(cudaMemcpyAsync(kind.data(), t->kind.p, E, cudaMemcpyDeviceToHost, st));
        AMIE_CUDA(cudaMemcpyAsync(gp_ptr.data(), t->gp_ptr.p, (E + 1) * 4, cudaMemcpyDeviceToHost, st));
        if (t->enr_ptr.p) {
            enr_ptr.resize(E + 1);
            AMIE_CUDA(cudaMemcpyAsync(enr_ptr.data(), t->enr_ptr.p, (E + 1) * 4, cudaMemcpyDeviceToHost, st));
        }
        AMIE_CUDA(cudaStreamSynchronize(st));
        for (uint32_t e = 0; e < E; e++)
            if (kind[e] != AMIE_TRI3 || gp_ptr[e + 1] - gp_ptr[e] > 1 || (!enr_ptr.empty() && enr_ptr[e + 1] != enr_ptr[e])) {
                set_error("amie_damage_setup: element %u is not a linear triangle with its one-point rule and no "
                          "enrichment", e);
                return AMIE_BAD_INPUT;
            }
    }
    release_damage(t);
    DamageState *d = new DamageState();
    t->dmg = d;
    d->law = *law;
    d->n_elem = E;
    DamageConst &k = d->k;
    {   // NonLocalMazars(thresh, E, nu, Gf, radius, PLANE_STRESS), mazars.cpp:27-35 (cstrain = cstress = -1)
        const double thresh = law->threshold, Ey = law->young, nu = law->poisson, cstrain = -1., cstress = -1.;
        k.threshold = std::abs(thresh);
        k.nu = nu;
        k.B_t = (0.1 * Ey * thresh) / (law->fracture_energy - Ey * 0.1 * thresh * thresh * 0.5);
        k.B_c = -1. / (std::sqrt(2.) * nu * cstrain);
        k.A_c = -(Ey * thresh + std::sqrt(2.) * cstress * nu) / ((Ey * std::exp(k.B_c * thresh - 1.) / k.B_c) - Ey * thresh);
    }
    k.radius = law->radius;
    k.tol = law->score_tolerance > 0 ? law->score_tolerance : 2e-3;
    k.fibre = law->fibre_fraction > 0 ? law->fibre_fraction : 0.1;
    k.cutoff = law->cutoff > 0 ? law->cutoff : 0.6;
    k.residual = law->residual > 0 ? law->residual : 1e-4;

    Ctx *c = t->ctx;
    AMIE_TRY(d->xy.alloc(c, (size_t)E * 6));
    AMIE_TRY(d->centre.alloc(c, (size_t)E * 2));
    AMIE_TRY(d->radius.alloc(c, E));
    AMIE_TRY(d->area.alloc(c, E));
    AMIE_TRY(d->gpw.alloc(c, E));
    AMIE_CUDA(cudaMemcpyAsync(d->xy.p, corners, (size_t)E * 48, cudaMemcpyHostToDevice, st));
    const MeshView m = mesh_view(t);
    k_dmg_geometry<<<blocks(E, 128), 128, 0, st>>>(m, d->xy.p, d->centre.p, d->radius.p, d->area.p, d->gpw.p);
    AMIE_LAUNCHED();

    // grid of the centres, cell size from the smoothing radii
    std::vector<double> cen((size_t)E * 2), rad(E);
    AMIE_CUDA(cudaMemcpyAsync(cen.data(), d->centre.p, (size_t)E * 16, cudaMemcpyDeviceToHost, st));
    AMIE_CUDA(cudaMemcpyAsync(rad.data(), d->radius.p, (size_t)E * 8, cudaMemcpyDeviceToHost, st));
    AMIE_CUDA(cudaStreamSynchronize(st));
    double xmin = cen[0], xmax = cen[0], ymin = cen[1], ymax = cen[1], rho_max = 0;
    for (uint32_t e = 0; e < E; e++) {
        xmin = std::min(xmin, cen[2 * e]);
        xmax = std::max(xmax, cen[2 * e]);
        ymin = std::min(ymin, cen[2 * e + 1]);
        ymax = std::max(ymax, cen[2 * e + 1]);
        rho_max = std::max(rho_max, smoothing_radius(reff(k.radius, rad[e]), rad[e]));
    }
    Grid g;
    g.h = std::max({rho_max, (xmax - xmin) / 2048.0, (ymax - ymin) / 2048.0, 1e-300});
    g.x0 = xmin;
    g.y0 = ymin;
    g.nx = (int)std::floor((xmax - xmin) / g.h) + 1;
    g.ny = (int)std::floor((ymax - ymin) / g.h) + 1;
    const size_t ncell = (size_t)g.nx * g.ny;
    std::vector<uint32_t> cell_start(ncell + 1, 0), items(E);
    std::vector<uint32_t> cell_of(E);
    for (uint32_t e = 0; e < E; e++) {
        const int ix = std::min(g.nx - 1, (int)std::floor((cen[2 * e] - g.x0) / g.h));
        const int iy = std::min(g.ny - 1, (int)std::floor((cen[2 * e + 1] - g.y0) / g.h));
        cell_of[e] = (uint32_t)(iy * g.nx + ix);
        cell_start[cell_of[e] + 1]++;
    }
    for (size_t q = 0; q < ncell; q++) cell_start[q + 1] += cell_start[q];
    {
        std::vector<uint32_t> fill(cell_start.begin(), cell_start.end() - 1);
        for (uint32_t e = 0; e < E; e++) items[fill[cell_of[e]]++] = e;
    }
    AMIE_TRY(d->cell_start.alloc(c, ncell + 1));
    AMIE_TRY(d->cell_items.alloc(c, E));
    AMIE_TRY(d->cell_of.alloc(c, E));
    AMIE_TRY(d->cell_max.alloc(c, ncell));
    AMIE_TRY(d->n_smoothed.alloc(c, 1));
    AMIE_CUDA(cudaMemsetAsync(d->n_smoothed.p, 0, 8, st));
    AMIE_CUDA(cudaMemcpyAsync(d->cell_start.p, cell_start.data(), (ncell + 1) * 4, cudaMemcpyHostToDevice, st));
    AMIE_CUDA(cudaMemcpyAsync(d->cell_items.p, items.data(), (size_t)E * 4, cudaMemcpyHostToDevice, st));
    AMIE_CUDA(cudaMemcpyAsync(d->cell_of.p, cell_of.data(), (size_t)E * 4, cudaMemcpyHostToDevice, st));
    g.cell_start = d->cell_start.p;
    g.items = d->cell_items.p;
    d->grid = g;

    // neighbourhoods: count, scan, fill, normalise
    DevArray<uint64_t> counts;
    AMIE_TRY(counts.alloc(c, (size_t)E + 1));
    AMIE_TRY(d->nb_ptr.alloc(c, (size_t)E + 1));
    AMIE_CUDA(cudaMemsetAsync(counts.p + E, 0, 8, st));
    k_dmg_cache<<<blocks(E, 128), 128, 0, st>>>(g, E, k.radius, d->xy.p, d->centre.p, d->radius.p, d->area.p, nullptr,
                                                 counts.p, nullptr, nullptr);
    AMIE_LAUNCHED();
    size_t scan_bytes = 0;
    AMIE_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, scan_bytes, counts.p, d->nb_ptr.p, (int)(E + 1), st));
    DevArray<uint8_t> scan_tmp;
    AMIE_TRY(scan_tmp.alloc(c, std::max<size_t>(scan_bytes, 16)));
    AMIE_CUDA(cub::DeviceScan::ExclusiveSum(scan_tmp.p, scan_bytes, counts.p, d->nb_ptr.p, (int)(E + 1), st));
    uint64_t total = 0;
    AMIE_CUDA(cudaMemcpyAsync(&total, d->nb_ptr.p + E, 8, cudaMemcpyDeviceToHost, st));
    AMIE_CUDA(cudaStreamSynchronize(st));
    AMIE_TRY(d->nb_idx.alloc(c, std::max<uint64_t>(total, 1)));
    AMIE_TRY(d->nb_coef.alloc(c, std::max<uint64_t>(total, 1)));
    k_dmg_cache<<<blocks(E, 128), 128, 0, st>>>(g, E, k.radius, d->xy.p, d->centre.p, d->radius.p, d->area.p,
                                                 d->nb_ptr.p, nullptr, d->nb_idx.p, d->nb_coef.p);
    k_dmg_cache_norm<<<blocks(E, 128), 128, 0, st>>>(E, d->nb_ptr.p, d->nb_coef.p);
    g_launches += 2;

    // damage state, scores, the factor on C (the caller's factor, if any, is the base)
    AMIE_TRY(d->state.alloc(c, E));
    AMIE_TRY(d->score.alloc(c, E));
    AMIE_TRY(d->smoothed.alloc(c, (size_t)E * 4));
    AMIE_TRY(d->met_flag.alloc(c, E));
    AMIE_TRY(d->decision.alloc(c, E));
    AMIE_TRY(d->met.alloc(c, E));
    AMIE_TRY(d->nmax.alloc(c, E));
    AMIE_TRY(d->counters.alloc(c, 4));
    AMIE_CUDA(cudaMemsetAsync(d->state.p, 0, (size_t)E * 8, st));
    AMIE_CUDA(cudaMemsetAsync(d->score.p, 0, (size_t)E * 8, st));
    if (t->has_cscale) {
        AMIE_TRY(d->base.alloc(c, E));
        AMIE_CUDA(cudaMemcpyAsync(d->base.p, t->cscale.p, (size_t)E * 8, cudaMemcpyDeviceToDevice, st));
        d->has_base = true;
    } else {
        AMIE_TRY(t->cscale.alloc(c, E));
    }
    k_dmg_factors<<<blocks(E, 256), 256, 0, st>>>(E, k, d->state.p, d->has_base ? d->base.p : nullptr, t->cscale.p);
    AMIE_LAUNCHED();
    t->has_cscale = true;
    size_t sel_bytes = 0;
    AMIE_TRY(d->iota.alloc(c, E));
    k_dmg_iota<<<blocks(E, 256), 256, 0, st>>>(E, d->iota.p);
    AMIE_LAUNCHED();
    AMIE_CUDA(cub::DeviceSelect::Flagged(nullptr, sel_bytes, d->iota.p, d->met_flag.p, d->met.p, d->counters.p,
                                         (int)E, st));
    d->cub_bytes = std::max<size_t>(sel_bytes, 16);
    AMIE_TRY(d->cub_tmp.alloc(c, d->cub_bytes));
    d->dirty = true;
    AMIE_CUDA(cudaStreamSynchronize(st));
    return AMIE_OK;
}

extern "C" amie_status amie_damage_set_state(amie_topo *t, const double *damage)
{
    AMIE_TRY(need_damage(t));
    AMIE_CUDA(cudaSetDevice(t->ctx->device));
    DamageState *d = t->dmg;
    cudaStream_t st = t->ctx->stream;
    const uint32_t E = d->n_elem;
    if (damage) AMIE_CUDA(cudaMemcpyAsync(d->state.p, damage, (size_t)E * 8, cudaMemcpyHostToDevice, st));
    else AMIE_CUDA(cudaMemsetAsync(d->state.p, 0, (size_t)E * 8, st));
    k_dmg_factors<<<blocks(E, 256), 256, 0, st>>>(E, d->k, d->state.p, d->has_base ? d->base.p : nullptr, t->cscale.p);
    AMIE_LAUNCHED();
    d->dirty = true;
    AMIE_CUDA(cudaStreamSynchronize(st));
    return AMIE_OK;
}

extern "C" amie_status amie_damage_get_state(amie_topo *t, double *damage)
{
    AMIE_TRY(need_damage(t));
    if (!damage) return AMIE_BAD_INPUT;
    AMIE_CUDA(cudaSetDevice(t->ctx->device));
    AMIE_CUDA(cudaMemcpyAsync(damage, t->dmg->state.p, (size_t)t->n_elem * 8, cudaMemcpyDeviceToHost, t->ctx->stream));
    AMIE_CUDA(cudaStreamSynchronize(t->ctx->stream));
    return AMIE_OK;
}

namespace amie {
namespace {

// Scores of every element from the current solution; with `bounded` the
// smoothing is skipped where the cell bound proves the score (k_dmg_grade) and
// the smoothed fields are not written.
amie_status grade_async(amie_topo *t, bool bounded)
{
    DamageState *d = t->dmg;
    cudaStream_t st = t->ctx->stream;
    AMIE_TRY(element_strain_async(t));
    if (bounded) {
        const Grid &g = d->grid;
        AMIE_CUDA(cudaMemsetAsync(d->cell_max.p, 0, (size_t)g.nx * g.ny * 4, st));
        k_dmg_cell_max<<<blocks(d->n_elem, 256), 256, 0, st>>>(d->n_elem, d->k, t->strain.p, d->state.p,
                                                               d->cell_of.p, d->cell_max.p);
        AMIE_LAUNCHED();
    }
    k_dmg_grade<<<blocks(d->n_elem, 128), 128, 0, st>>>(d->n_elem, d->k, t->strain.p, t->mat.p, t->cmat_table.p,
                                                        d->state.p, d->area.p, d->gpw.p, d->nb_ptr.p, d->nb_idx.p,
                                                        d->nb_coef.p, d->score.p, d->smoothed.p, d->grid,
                                                        bounded ? d->cell_max.p : nullptr, d->centre.p, d->radius.p,
                                                        d->n_smoothed.p);
    AMIE_LAUNCHED();
    AMIE_CUDA(cudaGetLastError());
    return AMIE_OK;
}

amie_status update(amie_topo *t, uint32_t *n_changed)
{
    DamageState *d = t->dmg;
    cudaStream_t st = t->ctx->stream;
    const uint32_t E = d->n_elem;
    k_dmg_met<<<blocks(E, 256), 256, 0, st>>>(E, d->score.p, d->met_flag.p);
    AMIE_LAUNCHED();
    size_t bytes = d->cub_bytes;
    AMIE_CUDA(cub::DeviceSelect::Flagged(d->cub_tmp.p, bytes, d->iota.p, d->met_flag.p, d->met.p, d->counters.p,
                                         (int)E, st));
    uint32_t M = 0;
    AMIE_CUDA(cudaMemcpyAsync(&M, d->counters.p, 4, cudaMemcpyDeviceToHost, st));
    AMIE_CUDA(cudaStreamSynchronize(st));
    *n_changed = 0;
    if (M == 0) return AMIE_OK;
    k_dmg_nmax<<<blocks(M, 256), 256, 0, st>>>(d->counters.p, d->met.p, d->k, d->centre.p, d->radius.p, d->score.p,
                                              d->nmax.p, d->decision.p);
    k_dmg_commit<<<1, 32, 0, st>>>(d->counters.p, d->met.p, d->k, d->centre.p, d->radius.p, d->score.p,
                                   d->decision.p, d->state.p, d->has_base ? d->base.p : nullptr, t->cscale.p,
                                   d->counters.p + 1);
    g_launches += 2;
    uint32_t changed = 0;
    AMIE_CUDA(cudaMemcpyAsync(&changed, d->counters.p + 1, 4, cudaMemcpyDeviceToHost, st));
    AMIE_CUDA(cudaStreamSynchronize(st));
    *n_changed = changed;
    if (changed) d->dirty = true;
    return AMIE_OK;
}

}  // namespace
}  // namespace amie

extern "C" amie_status amie_damage_grade(amie_topo *t, double *score, double *smoothed)
{
    AMIE_TRY(need_damage(t));
    AMIE_CUDA(cudaSetDevice(t->ctx->device));
    cudaStream_t st = t->ctx->stream;
    AMIE_TRY(grade_async(t, smoothed == nullptr));
    const uint32_t E = t->dmg->n_elem;
    if (score) AMIE_CUDA(cudaMemcpyAsync(score, t->dmg->score.p, (size_t)E * 8, cudaMemcpyDeviceToHost, st));
    if (smoothed) AMIE_CUDA(cudaMemcpyAsync(smoothed, t->dmg->smoothed.p, (size_t)E * 32, cudaMemcpyDeviceToHost, st));
    AMIE_CUDA(cudaStreamSynchronize(st));
    return AMIE_OK;
}

extern "C" amie_status amie_damage_update(amie_topo *t, uint32_t *n_changed)
{
    AMIE_TRY(need_damage(t));
    AMIE_CUDA(cudaSetDevice(t->ctx->device));
    uint32_t changed = 0;
    AMIE_TRY(update(t, &changed));
    if (n_changed) *n_changed = changed;
    return AMIE_OK;
}

extern "C" amie_status amie_damage_load_step(amie_topo *t, const amie_solve_opts *opts, int32_t max_sub_iterations,
                                             amie_damage_step_stats *stats)
{
    AMIE_TRY(need_damage(t));
    if (!t->bc_set) {
        set_error("amie_damage_load_step before amie_apply_dirichlet");
        return AMIE_BAD_INPUT;
    }
    AMIE_CUDA(cudaSetDevice(t->ctx->device));
    DamageState *d = t->dmg;
    cudaStream_t st = t->ctx->stream;
    amie_damage_step_stats s{};
    const auto t0 = std::chrono::steady_clock::now();
    amie_solve_opts o = opts ? *opts : amie_solve_opts{AMIE_SOLVER_PCG_FP64, 1e-10, 1e-10, 32, 0, 0.0, 0};
    const int32_t cap = max_sub_iterations > 0 ? max_sub_iterations : 10000;
    s.status = AMIE_NOT_CONVERGED;
    AMIE_CUDA(cudaMemsetAsync(d->n_smoothed.p, 0, 8, st));
    for (int32_t pass = 0; pass < cap; pass++) {
        if (d->dirty) {   // the damaged stiffness, eliminated with the stored multipliers
            AMIE_TRY(amie_assemble(t));
            d->dirty = false;
        }
        amie_solve_stats ss{};
        amie_status rc = amie_solve_resident(t, &o, &ss);
        if (rc != AMIE_OK) {
            set_error("amie_damage_load_step: solve of pass %d returned %d", pass + 1, (int)rc);
            return rc;
        }
        o.use_x0 = 1;   // the next passes start from this solution
        s.cg_iterations += ss.iterations;
        s.sub_iterations++;
        AMIE_TRY(grade_async(t, true));
        uint32_t changed = 0;
        AMIE_TRY(update(t, &changed));
        s.changes += changed;
        if (changed == 0) {
            s.status = AMIE_OK;
            break;
        }
    }
    AMIE_CUDA(cudaMemsetAsync(d->counters.p + 2, 0, 8, st));
    k_dmg_counts<<<blocks(d->n_elem, 256), 256, 0, st>>>(d->n_elem, d->state.p, d->k.cutoff, d->counters.p);
    AMIE_LAUNCHED();
    uint32_t h[2] = {0, 0};
    unsigned long long ns = 0;
    AMIE_CUDA(cudaMemcpyAsync(h, d->counters.p + 2, 8, cudaMemcpyDeviceToHost, st));
    AMIE_CUDA(cudaMemcpyAsync(&ns, d->n_smoothed.p, 8, cudaMemcpyDeviceToHost, st));
    AMIE_CUDA(cudaStreamSynchronize(st));
    s.damaged = h[0];
    s.fractured = h[1];
    s.smoothed = ns;
    s.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (stats) *stats = s;
    return (amie_status)s.status;
}
