// assemble.cu -- topology (pattern + scatter map), element stiffness
// quadrature, atomic-free gather assembly and Dirichlet elimination.
//
// Reference path (paths relative to the AMIE source tree):
//   pattern     Assembly::make_final            solvers/assembly.cpp:445-537
//   K_e         DelaunayTriangle::getElementaryMatrix  mesher/delaunay.cpp:2408-2535
//               Stiffness::apply                physics/stiffness.cpp:43-48
//               VirtualMachine::ieval / geval   polynomial/vm_base.cpp:2974-2989, 2156-2298
//   scatter     Assembly::make_final            solvers/assembly.cpp:657-803 (Kahan)
//   Dirichlet   Assembly::setBoundaryConditions solvers/assembly.cpp:125-283
#include "internal.h"

#include <cub/cub.cuh>

#include <algorithm>
#include <chrono>
#include <cstdlib>
#include <cstring>

#include "element.cuh"

namespace amie {

// ------------------------------------------------------------------ kernels

// Nonzeros of row r of the Voigt B of a function with physical gradient d
// (polynomial/vm_base.cpp:2244-2255, 2278-2296): B[r][col] = d[comp], in
// increasing column order.
template <int DIM>
struct BRow;
template <>
struct BRow<2> {
    static constexpr int N = 2;
    static __device__ constexpr int col(int r, int k) { return r == 0 ? (k == 0 ? 0 : 2) : (k == 0 ? 1 : 2); }
    static __device__ constexpr int comp(int r, int k) { return r == 0 ? (k == 0 ? 0 : 1) : (k == 0 ? 1 : 0); }
};
template <>
struct BRow<3> {
    static constexpr int N = 3;
    static __device__ constexpr int col(int r, int k) { return r == 0 ? (k == 0 ? 0 : k == 1 ? 4 : 5)
                                                        : r == 1 ? (k == 0 ? 1 : k == 1 ? 3 : 5)
                                                                 : (k == 0 ? 2 : k == 1 ? 3 : 4); }
    static __device__ constexpr int comp(int r, int k) { return r == 0 ? (k == 0 ? 0 : k == 1 ? 2 : 1)
                                                         : r == 1 ? (k == 0 ? 1 : k == 1 ? 2 : 0)
                                                                  : (k == 0 ? 2 : k == 1 ? 1 : 0); }
};

// Default-rule element (NG points of its kind, inverse Jacobian at the
// centroid): the physical gradient of every function at every point once, then
// per column function j the products w_g C B_j^T, then every block
// K_ij = sum_g B_i (w_g C B_j^T), i >= j, with the zero entries of B skipped.
template <int DIM, int NF, int NG>
__device__ __forceinline__ void quad_default(int kind, const double *C, const double *Je, double *K)
{
    constexpr int NV = DIM == 2 ? 3 : 6;
    using B = BRow<DIM>;
    const double inv_det = 1.0 / det_small<DIM>(Je);
    double d[NF][NG][DIM], w[NG];
#pragma unroll
    for (int g = 0; g < NG; g++) {
        double p[3];
        default_rule(kind, g, p, &w[g]);
        w[g] *= inv_det;   // weight / det(J^-1) (elements/elements.cpp:939-945)
#pragma unroll
        for (int f = 0; f < NF; f++) {
            double lg[3];
            shape_grad(kind, f, p[0], p[1], lg);
            phys_grad<DIM>(Je, lg, d[f][g]);
        }
    }
#pragma unroll
    for (int j = 0; j < NF; j++) {
        double cb[NG][NV][DIM];   // w_g C B_j^T
#pragma unroll
        for (int g = 0; g < NG; g++)
#pragma unroll
            for (int l = 0; l < NV; l++)
#pragma unroll
                for (int c = 0; c < DIM; c++) {
                    double a = 0.0;
#pragma unroll
                    for (int k = 0; k < B::N; k++) a += C[l * NV + B::col(c, k)] * d[j][g][B::comp(c, k)];
                    cb[g][l][c] = w[g] * a;
                }
#pragma unroll
        for (int i = j; i < NF; i++) {
            double acc[DIM * DIM];
#pragma unroll
            for (int q = 0; q < DIM * DIM; q++) acc[q] = 0.0;
#pragma unroll
            for (int g = 0; g < NG; g++)
#pragma unroll
                for (int r = 0; r < DIM; r++)
#pragma unroll
                    for (int c = 0; c < DIM; c++)
#pragma unroll
                        for (int k = 0; k < B::N; k++)
                            acc[r * DIM + c] = fma(d[i][g][B::comp(r, k)], cb[g][B::col(r, k)][c], acc[r * DIM + c]);
            double *Kij = K + (size_t)(i * NF + j) * DIM * DIM;
            double *Kji = K + (size_t)(j * NF + i) * DIM * DIM;
#pragma unroll
            for (int r = 0; r < DIM; r++)
#pragma unroll
                for (int c = 0; c < DIM; c++) {
                    Kij[r * DIM + c] = acc[r * DIM + c];
                    if (i != j) Kji[c * DIM + r] = acc[r * DIM + c];
                }
        }
    }
}

// Thread per unenriched element: loops over lower block pairs (i >= j), and
// for each pair over the Gauss points; writes block (i,j) and its transpose
// (j,i), as the reference does (mesher/delaunay.cpp:2462-2467).  Elements on
// their kind's default rule take the hoisted path above.
template <int DIM>
__global__ void __launch_bounds__(128) k_quad_simple(MeshView m, const uint32_t *list, uint32_t count)
{
    constexpr int NV = DIM == 2 ? 3 : 6;
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= count) return;
    const uint32_t e = list[t];
    const int kind = m.kind[e];
    const int nf = nshape_of(kind);
    double C[NV * NV];
    const double cs = m.cscale ? m.cscale[e] : 1.0;
    const double *Ct = m.cmat_table + (size_t)m.mat[e] * NV * NV;
#pragma unroll
    for (int i = 0; i < NV * NV; i++) C[i] = cs * Ct[i];
    double Je[DIM * DIM];
#pragma unroll
    for (int i = 0; i < DIM * DIM; i++) Je[i] = m.jinv[(size_t)e * DIM * DIM + i];
    const uint32_t g0 = m.gp_ptr[e], g1 = m.gp_ptr[e + 1];
    const bool explicit_gp = g1 > g0;
    double *K = m.ke + m.blk_off[e] * DIM * DIM;
    if (!explicit_gp) {
        if (DIM == 2 && kind == AMIE_TRI6) quad_default<DIM, 6, 4>(kind, C, Je, K);
        else if (DIM == 2) quad_default<DIM, 3, 1>(kind, C, Je, K);
        else quad_default<DIM, 4, 1>(kind, C, Je, K);
        return;
    }
    const bool moved = m.moved && m.moved[e];
    const int ngp = (int)(g1 - g0);
    for (int i = 0; i < nf; i++) {
        for (int j = 0; j <= i; j++) {
            double acc[DIM * DIM];
#pragma unroll
            for (int q = 0; q < DIM * DIM; q++) acc[q] = 0.0;
            for (int g = 0; g < ngp; g++) {
                double p[3];
                const double *gp = m.gp + (size_t)(g0 + g) * (DIM + 1);
                p[0] = gp[0]; p[1] = gp[1]; p[2] = DIM == 3 ? gp[2] : 0.0;
                const double w = gp[DIM];
                const double *J = moved ? m.jinv_gp + (size_t)(g0 + g) * DIM * DIM : Je;
                double gi[3], gj[3], di[3], dj[3];
                shape_grad(kind, i, p[0], p[1], gi);
                shape_grad(kind, j, p[0], p[1], gj);
                phys_grad<DIM>(J, gi, di);
                phys_grad<DIM>(J, gj, dj);
                bcb<DIM>(di, dj, C, w, acc);
            }
            double *Kij = K + (size_t)(i * nf + j) * DIM * DIM;
            double *Kji = K + (size_t)(j * nf + i) * DIM * DIM;
#pragma unroll
            for (int r = 0; r < DIM; r++)
#pragma unroll
                for (int c = 0; c < DIM; c++) {
                    Kij[r * DIM + c] = acc[r * DIM + c];
                    if (i != j) Kji[c * DIM + r] = acc[r * DIM + c];
                }
        }
    }
}

// Warp quadrature of enriched elements (any number of functions <=
// kMaxFunctions and any number of Gauss points).  Gauss points are processed in
// tiles: the lanes first stage the physical gradients of every function at the
// tile's points in shared memory, then each lane accumulates its own lower
// block pairs.
template <int DIM>
struct WarpQuadSmem {
    static constexpr int NV = DIM == 2 ? 3 : 6;
    static constexpr int NPAIR = kMaxFunctions * (kMaxFunctions + 1) / 2;
    double C[NV * NV];
    double grad[kMaxGpWarpTile][kMaxFunctions][DIM];
    double w[kMaxGpWarpTile];
    double acc[NPAIR * DIM * DIM];
};

__device__ __forceinline__ void pair_of(int pidx, int &i, int &j)
{
    // pair index -> (i, j), i >= j, row-major lower triangle
    i = (int)((sqrt(8.0 * pidx + 1.0) - 1.0) * 0.5);
    while ((i + 1) * (i + 2) / 2 <= pidx) i++;
    while (i * (i + 1) / 2 > pidx) i--;
    j = pidx - i * (i + 1) / 2;
}

// Stages C (times the element's factor) and zeroes the pair accumulators.
template <int DIM>
__device__ void warp_quad_begin(const MeshView &m, uint32_t e, int npair, WarpQuadSmem<DIM> &sm)
{
    constexpr int NV = WarpQuadSmem<DIM>::NV;
    const int lane = threadIdx.x & 31;
    const double cs = m.cscale ? m.cscale[e] : 1.0;
    for (int i = lane; i < NV * NV; i += 32) sm.C[i] = cs * m.cmat_table[(size_t)m.mat[e] * NV * NV + i];
    for (int i = lane; i < npair * DIM * DIM; i += 32) sm.acc[i] = 0.0;
    __syncwarp();
}

// Accumulates the Gauss points [gb, ge) of element e into sm.acc.
template <int DIM>
__device__ void warp_quad_range(const MeshView &m, uint32_t e, int gb, int ge, WarpQuadSmem<DIM> &sm)
{
    constexpr int T = kMaxGpWarpTile;
    const int lane = threadIdx.x & 31;
    const int kind = m.kind[e];
    const int nshape = nshape_of(kind);
    const uint32_t f0 = m.enr_ptr[e], f1 = m.enr_ptr[e + 1];
    const int nf = nshape + (int)(f1 - f0);
    const int npair = nf * (nf + 1) / 2;
    double Je[DIM * DIM];
#pragma unroll
    for (int i = 0; i < DIM * DIM; i++) Je[i] = m.jinv[(size_t)e * DIM * DIM + i];
    const uint32_t g0 = m.gp_ptr[e], g1 = m.gp_ptr[e + 1];
    const bool explicit_gp = g1 > g0;
    const bool moved = explicit_gp && m.moved && m.moved[e];
    const double inv_det = 1.0 / det_small<DIM>(Je);
    for (int t0 = gb; t0 < ge; t0 += T) {
        const int nt = min(T, ge - t0);
        for (int item = lane; item < nt * nf; item += 32) {
            const int tg = item / nf, f = item % nf, g = t0 + tg;
            double p[3], wt;
            if (explicit_gp) {
                const double *gp = m.gp + (size_t)(g0 + g) * (DIM + 1);
                p[0] = gp[0]; p[1] = gp[1]; p[2] = DIM == 3 ? gp[2] : 0.0;
                wt = gp[DIM];
            } else {
                default_rule(kind, g, p, &wt);
                wt *= inv_det;
            }
            double lg[3] = {0.0, 0.0, 0.0};
            if (f < nshape) {
                shape_grad(kind, f, p[0], p[1], lg);
            } else {
                enr_local_grad<DIM>(m, f0 + (f - nshape), g, p, lg);
            }
            const double *J = moved ? m.jinv_gp + (size_t)(g0 + g) * DIM * DIM : Je;
            double d[3];
            phys_grad<DIM>(J, lg, d);
#pragma unroll
            for (int c = 0; c < DIM; c++) sm.grad[tg][f][c] = d[c];
            if (f == 0) sm.w[tg] = wt;
        }
        __syncwarp();
        for (int pidx = lane; pidx < npair; pidx += 32) {
            int i, j;
            pair_of(pidx, i, j);
            double acc[DIM * DIM];
#pragma unroll
            for (int q = 0; q < DIM * DIM; q++) acc[q] = sm.acc[pidx * DIM * DIM + q];
            for (int tg = 0; tg < nt; tg++) bcb<DIM>(sm.grad[tg][i], sm.grad[tg][j], sm.C, sm.w[tg], acc);
#pragma unroll
            for (int q = 0; q < DIM * DIM; q++) sm.acc[pidx * DIM * DIM + q] = acc[q];
        }
        __syncwarp();
    }
}

// Writes the accumulated pairs as blocks (i,j) and (j,i) of the staged K_e.
template <int DIM>
__device__ void warp_quad_store(const MeshView &m, uint32_t e, int nf, const double *acc)
{
    const int lane = threadIdx.x & 31;
    const int npair = nf * (nf + 1) / 2;
    double *K = m.ke + m.blk_off[e] * DIM * DIM;
    for (int pidx = lane; pidx < npair; pidx += 32) {
        int i, j;
        pair_of(pidx, i, j);
        double *Kij = K + (size_t)(i * nf + j) * DIM * DIM;
        double *Kji = K + (size_t)(j * nf + i) * DIM * DIM;
#pragma unroll
        for (int r = 0; r < DIM; r++)
#pragma unroll
            for (int c = 0; c < DIM; c++) {
                const double v = acc[pidx * DIM * DIM + r * DIM + c];
                Kij[r * DIM + c] = v;
                if (i != j) Kji[c * DIM + r] = v;
            }
    }
}

__device__ __forceinline__ int nf_of(const MeshView &m, uint32_t e)
{
    return nshape_of(m.kind[e]) + (int)(m.enr_ptr[e + 1] - m.enr_ptr[e]);
}

__device__ __forceinline__ int ngp_of(const MeshView &m, uint32_t e)
{
    const uint32_t g0 = m.gp_ptr[e], g1 = m.gp_ptr[e + 1];
    return g1 > g0 ? (int)(g1 - g0) : (m.kind[e] == AMIE_TRI6 ? 4 : 1);
}

// Warp per enriched element with at most kLongGp Gauss points.
template <int DIM>
__global__ void __launch_bounds__(32) k_quad_warp(MeshView m, const uint32_t *list, uint32_t count)
{
    __shared__ WarpQuadSmem<DIM> sm;
    const uint32_t w = blockIdx.x;
    if (w >= count) return;
    const uint32_t e = list[w];
    const int nf = nf_of(m, e);
    warp_quad_begin<DIM>(m, e, nf * (nf + 1) / 2, sm);
    warp_quad_range<DIM>(m, e, 0, ngp_of(m, e), sm);
    warp_quad_store<DIM>(m, e, nf, sm.acc);
}

// Elements with many Gauss points (the 512-point Monte-Carlo rule of a tip
// element): one warp per chunk of kChunkGp points, each on its own SM, writes
// its partial pair sums; k_quad_chunk_sum then adds the chunks of each element
// in chunk order (a fixed order: the result does not depend on scheduling).
template <int DIM>
__global__ void __launch_bounds__(32) k_quad_chunk(MeshView m, const QuadChunk *chunks, uint32_t count,
                                                   double *partial)
{
    __shared__ WarpQuadSmem<DIM> sm;
    if (blockIdx.x >= count) return;
    const QuadChunk c = chunks[blockIdx.x];
    const int nf = nf_of(m, c.elem);
    const int npair = nf * (nf + 1) / 2;
    warp_quad_begin<DIM>(m, c.elem, npair, sm);
    warp_quad_range<DIM>(m, c.elem, (int)c.gp_begin, (int)c.gp_end, sm);
    for (int i = threadIdx.x; i < npair * DIM * DIM; i += 32) partial[c.out + i] = sm.acc[i];
}

constexpr int kChunkSumThreads = 256;
constexpr int kChunkSumSplit = 4;   // CTAs per long element, each on a quarter of its pair sums

// Sum of the chunk partials of each long element in chunk order, written as
// blocks (i,j) and (j,i) of its staged K_e: CTA (element, part) takes every
// kChunkSumSplit-th group of its pair sums.
template <int DIM>
__global__ void __launch_bounds__(kChunkSumThreads) k_quad_chunk_sum(MeshView m, const QuadLong *longs, uint32_t count,
                                                                     const QuadChunk *chunks, const double *partial)
{
    const uint32_t li = blockIdx.x / kChunkSumSplit, part = blockIdx.x % kChunkSumSplit;
    if (li >= count) return;
    const QuadLong L = longs[li];
    const int nf = nf_of(m, L.elem);
    const int npair = nf * (nf + 1) / 2;
    const int n = npair * DIM * DIM;
    double *K = m.ke + m.blk_off[L.elem] * DIM * DIM;
    // an element's chunks are consecutive, n partial sums apart
    const double *p0 = partial + chunks[L.chunk_first].out;
    for (int k = (int)part * kChunkSumThreads + threadIdx.x; k < n; k += kChunkSumSplit * kChunkSumThreads) {
        double a = 0.0;
#pragma unroll 8
        for (uint32_t c = 0; c < L.chunk_count; c++) a += p0[(uint64_t)c * n + k];
        const int pidx = k / (DIM * DIM), q = k % (DIM * DIM), r = q / DIM, cc = q % DIM;
        int i, j;
        pair_of(pidx, i, j);
        K[(size_t)(i * nf + j) * DIM * DIM + r * DIM + cc] = a;
        if (i != j) K[(size_t)(j * nf + i) * DIM * DIM + cc * DIM + r] = a;
    }
}

// Pattern keys: (row << 32 | col) for every (ids[j], ids[k]) of every element
// (value = staged block index, so a stable sort keeps each slot's contributions
// in element order) plus the diagonal gap fill and (ndofmax-1, ndofmax-1)
// (value = no contribution).
constexpr uint32_t kNoContribution = 0xffffffffu;

__global__ void k_pattern_keys(uint32_t n_elem, const uint32_t *dof_ptr, const uint32_t *dof_ids,
                               const uint64_t *blk_off, uint64_t *keys, uint32_t *vals)
{
    const uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n_elem) return;
    const uint32_t a = dof_ptr[e], nf = dof_ptr[e + 1] - a;
    const uint64_t base = blk_off[e];
    for (uint32_t j = 0; j < nf; j++) {
        const uint64_t rj = (uint64_t)dof_ids[a + j] << 32;
        for (uint32_t k = 0; k < nf; k++) {
            keys[base + j * nf + k] = rj | dof_ids[a + k];
            vals[base + j * nf + k] = (uint32_t)(base + j * nf + k);
        }
    }
}

__global__ void k_fill_keys(uint64_t offset, uint32_t n_diag, uint32_t last, uint64_t *keys, uint32_t *vals)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n_diag) {
        keys[offset + i] = ((uint64_t)i << 32) | i;
        vals[offset + i] = kNoContribution;
    } else if (i == n_diag) {
        keys[offset + i] = ((uint64_t)last << 32) | last;
        vals[offset + i] = kNoContribution;
    }
}

__global__ void k_unique_flags(uint64_t n, const uint64_t *keys, const uint32_t *vals, uint32_t *is_new,
                               uint32_t *is_contrib)
{
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    is_new[i] = (i == 0 || keys[i] != keys[i - 1]) ? 1u : 0u;
    is_contrib[i] = vals[i] != kNoContribution ? 1u : 0u;
}

__global__ void k_pattern_emit(uint64_t n, const uint64_t *keys, const uint32_t *vals, const uint32_t *is_new,
                               const uint32_t *slot_scan, const uint32_t *contrib_scan, uint32_t *col,
                               uint32_t *row_count, uint64_t *map_ptr, uint32_t *map)
{
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (is_new[i]) {
        const uint32_t slot = slot_scan[i];
        col[slot] = (uint32_t)(keys[i] & 0xffffffffu);
        atomicAdd(&row_count[keys[i] >> 32], 1u);
        map_ptr[slot] = contrib_scan[i];
    }
    if (vals[i] != kNoContribution) map[contrib_scan[i]] = vals[i];
}

__global__ void k_diag_pos(uint32_t n_rows, const uint32_t *row_ptr, const uint32_t *col, uint32_t *diag_pos)
{
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n_rows) return;
    uint32_t lo = row_ptr[k], hi = row_ptr[k + 1];
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (col[mid] < k) lo = mid + 1; else hi = mid;
    }
    diag_pos[k] = lo;   // the diagonal gap fill guarantees (k, k) exists
}

__global__ void k_block_elem(uint32_t n_elem, const uint64_t *blk_off, uint32_t *blk_elem)
{
    const uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n_elem) return;
    for (uint64_t b = blk_off[e]; b < blk_off[e + 1]; b++) blk_elem[b] = e;
}

// Gather assembly: one thread per stored block, summing its contributions in
// element order with the Kahan compensation of solvers/assembly.cpp:676-694:
//   y = scale*K - c; t = a + y; c = (t - a) - y; a = t.
template <int S>
__global__ void k_gather(uint64_t nnzb, const uint64_t *map_ptr, const uint32_t *map, const double *ke,
                         const uint32_t *blk_elem, const double *scale, double *val)
{
    const uint64_t b = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nnzb) return;
    double a[S * S], c[S * S];
    const uint64_t k0 = map_ptr[b], k1 = map_ptr[b + 1];
    // the first contribution enters as sc*K: from a = c = 0 the update gives
    // y = sc*K, t = y, c = (y - 0) - y = 0 exactly, so nothing else is computed
    // for it (most blocks have one or two contributions; FP64 issue bounds this kernel)
    if (k0 < k1) {
        const uint32_t blk = map[k0];
        const double sc = scale ? scale[blk_elem[blk]] : 1.0;
        const double *src = ke + (uint64_t)blk * S * S;
#pragma unroll
        for (int q = 0; q < S * S; q++) {
            a[q] = sc * src[q];
            c[q] = 0.0;
        }
    } else {
#pragma unroll
        for (int q = 0; q < S * S; q++) { a[q] = 0.0; c[q] = 0.0; }
    }
    // the middle contributions with the full update; the compensation of the last
    // one would never be used, so its update stops at a = t
    for (uint64_t k = k0 + 1; k + 1 < k1; k++) {
        const uint32_t blk = map[k];
        const double sc = scale ? scale[blk_elem[blk]] : 1.0;
        const double *src = ke + (uint64_t)blk * S * S;
#pragma unroll
        for (int q = 0; q < S * S; q++) {
            const double y = sc * src[q] - c[q];
            const double t = a[q] + y;
            c[q] = (t - a[q]) - y;
            a[q] = t;
        }
    }
    if (k1 > k0 + 1) {
        const uint32_t blk = map[k1 - 1];
        const double sc = scale ? scale[blk_elem[blk]] : 1.0;
        const double *src = ke + (uint64_t)blk * S * S;
#pragma unroll
        for (int q = 0; q < S * S; q++) a[q] = a[q] + (sc * src[q] - c[q]);
    }
#pragma unroll
    for (int q = 0; q < S * S; q++) val[b * S * S + q] = a[q];
}

// Dirichlet elimination, one thread per block row, blocks in column order and
// constrained columns in increasing id order: the accumulation order of
// solvers/assembly.cpp:137-249.  Free rows move value * A[row][col] of every
// constrained column to the right-hand side and zero the entry; constrained
// rows become unit rows.
template <int S>
__global__ void k_dirichlet(uint32_t n_rows, const uint32_t *row_ptr, const uint32_t *col, double *val,
                            const uint8_t *fixed, const double *fixval, double *rhs)
{
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n_rows) return;
    for (int r = 0; r < S; r++) {
        const uint64_t row = (uint64_t)k * S + r;
        if (fixed[row]) {
            for (uint32_t p = row_ptr[k]; p < row_ptr[k + 1]; p++)
                for (int c = 0; c < S; c++)
                    val[(uint64_t)p * S * S + r * S + c] = ((uint64_t)col[p] * S + c == row) ? 1.0 : 0.0;
            rhs[row] = fixval[row];
            continue;
        }
        double f = rhs[row];
        for (uint32_t p = row_ptr[k]; p < row_ptr[k + 1]; p++) {
            const uint64_t cb = (uint64_t)col[p] * S;
            for (int c = 0; c < S; c++) {
                if (!fixed[cb + c]) continue;
                double *a = &val[(uint64_t)p * S * S + r * S + c];
                f -= fixval[cb + c] * *a;
                *a = 0.0;
            }
        }
        rhs[row] = f;
    }
}

__global__ void k_mark_fixed(uint32_t n_bc, const uint32_t *ids, const double *vals, const uint8_t *kinds,
                             uint8_t *fixed, double *fixval)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_bc) return;
    if (kinds && kinds[i] == AMIE_BC_FORCE) return;
    fixed[ids[i]] = 1;
    fixval[ids[i]] = vals[i];
}

// SET_FORCE_* multipliers, added in multiplier order after elimination
// (solvers/assembly.cpp:277-283): the force multipliers only, one thread each
// when no DOF has two of them (no order to keep), else one thread in order.
__global__ void k_add_forces(uint32_t n_force, const uint32_t *ids, const double *vals, int unique, double *rhs)
{
    if (unique) {
        const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
        if (i < n_force) rhs[ids[i]] += vals[i];
        return;
    }
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    for (uint32_t i = 0; i < n_force; i++) rhs[ids[i]] += vals[i];
}

// InverseDiagonal: 1/A_ii if |A_ii| > 1e-12 else 0 (sparse/sparse_matrix.cpp:216-231),
// plus the FP32 copies used by the mixed-precision solver.
template <int S>
__global__ void k_invdiag(uint32_t n_rows, const uint32_t *diag_pos, const double *val, double *inv, float *inv32)
{
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (uint64_t)n_rows * S) return;
    const uint32_t k = (uint32_t)(i / S), r = (uint32_t)(i % S);
    const double v = val[(uint64_t)diag_pos[k] * S * S + r * S + r];
    const double d = fabs(v) > 1e-12 ? 1.0 / v : 0.0;
    inv[i] = d;
    if (inv32) inv32[i] = (float)d;
}

__global__ void k_to_f32(uint64_t n, const double *a, float *b)
{
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        b[i] = (float)a[i];
}

// Unpadded row-major blocks -> AMIE's column-major, even-padded blocks
// (sparse/sparse_vector.cpp:57: array[blk*s*cl + c*cl + r]).
template <int S>
__global__ void k_to_amie_layout(uint64_t nnzb, const double *val, double *out)
{
    constexpr int CL = S + S % 2;
    const uint64_t b = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nnzb) return;
#pragma unroll
    for (int c = 0; c < S; c++) {
#pragma unroll
        for (int r = 0; r < S; r++) out[b * S * CL + c * CL + r] = val[b * S * S + r * S + c];
        if (CL != S) out[b * S * CL + c * CL + S] = 0.0;
    }
}

inline unsigned blocks_for(uint64_t n, unsigned threads) { return (unsigned)((n + threads - 1) / threads); }

// SELL slots of one slice per warp: block index (kSellNone for padding) and column.
__global__ void k_sell_fill(uint32_t n_rows, uint32_t n_slices, const uint32_t *perm, const uint64_t *slice_ptr,
                            const uint32_t *row_ptr, const uint32_t *col, uint32_t *sell_blk, uint32_t *sell_col)
{
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t warp = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint64_t n_warps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    for (uint64_t sl = warp; sl < n_slices; sl += n_warps) {
        const uint32_t row = perm[sl * 32 + lane];
        const uint32_t b = row < n_rows ? row_ptr[row] : 0u, e = row < n_rows ? row_ptr[row + 1] : 0u;
        const uint64_t g0 = slice_ptr[sl];
        const uint32_t len = (uint32_t)((slice_ptr[sl + 1] - g0) >> 5);
        for (uint32_t j = 0; j < len; j++) {
            const uint64_t slot = g0 + (uint64_t)j * 32 + lane;
            const bool real = b + j < e;
            sell_blk[slot] = real ? b + j : kSellNone;
            sell_col[slot] = real ? col[b + j] : (row < n_rows ? row : 0u);
        }
    }
}

// SELL-32-sigma order on the device: one CTA per window of `sigma` rows (blockDim
// >= sigma) places every row of the window at its rank in a stable sort by
// descending length (rows with more blocks first, equal lengths in row order),
// the order std::stable_sort gives; perm entries past n_rows keep the padding
// value n_rows (set before).
__global__ void k_sell_perm(uint32_t n_rows, uint32_t sigma, const uint32_t *row_ptr, uint32_t *perm)
{
    extern __shared__ uint32_t win_len[];
    const uint32_t w0 = blockIdx.x * sigma;
    const uint32_t cnt = min(sigma, n_rows - w0);
    for (uint32_t i = threadIdx.x; i < cnt; i += blockDim.x) win_len[i] = row_ptr[w0 + i + 1] - row_ptr[w0 + i];
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < cnt; i += blockDim.x) {
        const uint32_t li = win_len[i];
        uint32_t rank = 0;
        for (uint32_t q = 0; q < cnt; q++) {
            const uint32_t lq = win_len[q];
            rank += (lq > li || (lq == li && q < i)) ? 1u : 0u;
        }
        perm[w0 + rank] = w0 + i;
    }
}

// Slots of every slice: 32 x the longest row among its lanes.
__global__ void k_sell_slots(uint32_t n_rows, uint32_t n_slices, const uint32_t *perm, const uint32_t *row_ptr,
                             uint64_t *slots)
{
    const uint64_t warp = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t lane = threadIdx.x & 31;
    if (warp >= n_slices) return;
    const uint32_t r = perm[warp * 32 + lane];
    uint32_t len = r < n_rows ? row_ptr[r + 1] - row_ptr[r] : 0u;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) len = max(len, __shfl_xor_sync(0xffffffffu, len, o));
    if (lane == 0) slots[warp] = 32ull * len;
}

__global__ void k_fill_u32(uint64_t n, uint32_t v, uint32_t *out)
{
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        out[i] = v;
}

// Copy of the BSR values (row-major s x s blocks) into the chunked SELL layout.
template <int S, typename T>
__global__ void k_to_sell(uint64_t n_slots, const uint32_t *sell_blk, const double *val, T *out)
{
    for (uint64_t slot = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; slot < n_slots;
         slot += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t blk = sell_blk[slot];
        T *group = out + (slot & ~uint64_t(31)) * (S * S);
        const uint32_t lane = (uint32_t)(slot & 31);
#pragma unroll
        for (int c = 0; c < S * S; c++) {
            const double v = blk != kSellNone ? val[(uint64_t)blk * (S * S) + c] : 0.0;
            group[sell_off<S, T>(c, (int)lane)] = (T)v;
        }
    }
}

// Induced forces of the imposed strain, one thread per element: for every
// function f, sum_g w_g B_f(g)^T (C eps0) into the staging slot of (element, f)
// (StiffnessWithImposedStrain::getBoundaryConditions,
// physics/stiffness_with_imposed_deformation.cpp:83-110, through the
// SET_VOLUMIC_STRESS_* conditions of features/boundarycondition.cpp:542-617;
// C undamaged, as there).
template <int DIM>
__global__ void k_elem_forces(MeshView m, double *fstage)
{
    constexpr int NV = DIM == 2 ? 3 : 6;
    const uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= m.n_elem) return;
    const double *C = m.cmat_table + (size_t)m.mat[e] * NV * NV;
    double sig[NV];
#pragma unroll
    for (int r = 0; r < NV; r++) {
        double a = 0.0;
#pragma unroll
        for (int c = 0; c < NV; c++) a += C[r * NV + c] * m.imposed[(size_t)e * NV + c];
        sig[r] = a;
    }
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
    for (int f = 0; f < nf; f++) {
        double acc[DIM];
#pragma unroll
        for (int c = 0; c < DIM; c++) acc[c] = 0.0;
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
            double lg[3] = {0.0, 0.0, 0.0};
            if (f < nshape) {
                shape_grad(kind, f, p[0], p[1], lg);
            } else {
                enr_local_grad<DIM>(m, f0 + (f - nshape), g, p, lg);
            }
            double d[3];
            phys_grad<DIM>(J, lg, d);
            if (DIM == 2) {
                acc[0] += w * (d[0] * sig[0] + d[1] * sig[2]);
                acc[1] += w * (d[1] * sig[1] + d[0] * sig[2]);
            } else {
                acc[0] += w * (d[0] * sig[0] + d[2] * sig[4] + d[1] * sig[5]);
                acc[1] += w * (d[1] * sig[1] + d[2] * sig[3] + d[0] * sig[5]);
                acc[2] += w * (d[2] * sig[2] + d[1] * sig[3] + d[0] * sig[4]);
            }
        }
#pragma unroll
        for (int c = 0; c < DIM; c++) fstage[(uint64_t)(d0 + f) * DIM + c] = acc[c];
    }
}

// rhs += the staged forces of each block row, summed in element order.
template <int S>
__global__ void k_force_gather(uint32_t n_rows, const uint32_t *fmap_ptr, const uint32_t *fmap, const double *fstage,
                               double *rhs)
{
    const uint32_t row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= n_rows) return;
    double acc[S];
#pragma unroll
    for (int c = 0; c < S; c++) acc[c] = 0.0;
    for (uint32_t k = fmap_ptr[row]; k < fmap_ptr[row + 1]; k++) {
        const uint64_t src = (uint64_t)fmap[k] * S;
#pragma unroll
        for (int c = 0; c < S; c++) acc[c] += fstage[src + c];
    }
#pragma unroll
    for (int c = 0; c < S; c++) rhs[(uint64_t)row * S + c] += acc[c];
}

template <typename T>
amie_status upload(amie_ctx *ctx, DevArray<T> &d, const T *h, size_t n)
{
    AMIE_TRY(d.alloc(ctx, n));
    if (n) AMIE_CUDA(cudaMemcpyAsync(d.p, h, n * sizeof(T), cudaMemcpyHostToDevice, ctx->stream));
    return AMIE_OK;
}

MeshView mesh_view(amie_topo *t)
{
    MeshView m;
    m.dim = t->dim; m.s = t->s; m.nv = t->nv; m.n_elem = t->n_elem;
    m.kind = t->kind.p; m.dof_ptr = t->dof_ptr.p; m.dof_ids = t->dof_ids.p;
    m.gp_ptr = t->gp_ptr.p; m.gp = t->gp.p; m.jinv = t->jinv.p;
    m.moved = t->has_moved ? t->moved.p : nullptr; m.jinv_gp = t->jinv_gp.p;
    m.mat = t->mat.p; m.cmat_table = t->cmat_table.p; m.cscale = t->has_cscale ? t->cscale.p : nullptr;
    m.enr_ptr = t->enr_ptr.p; m.enr_type = t->enr_type.p; m.enr_vertex = t->enr_vertex.p;
    m.enr_data = t->enr_data.p; m.enr_jump = t->enr_jump.p; m.enr_grad = t->enr_grad.p;
    m.enr_tip = t->enr_tip.p;
    m.blk_off = t->blk_off.p; m.ke = t->ke.p;
    m.imposed = t->has_imposed ? t->imposed.p : nullptr;
    return m;
}

amie_status validate_mesh(const amie_mesh *m, std::vector<uint32_t> &nf, uint64_t &n_gp, uint32_t &max_id)
{
    if (!m || (m->dim != 2 && m->dim != 3) || m->stride != m->dim) {
        set_error("dim must be 2 or 3 and stride == dim");
        return AMIE_BAD_INPUT;
    }
    if (!m->kind || !m->dof_ptr || !m->dof_ids || !m->gp_ptr || !m->jinv || !m->mat || !m->cmat_table ||
        m->n_mat == 0) {
        set_error("missing element arrays");
        return AMIE_BAD_INPUT;
    }
    if (m->n_elem == 0) {
        set_error("empty mesh");
        return AMIE_BAD_INPUT;
    }
    nf.resize(m->n_elem);
    max_id = 0;
    if (m->dof_ptr[0] != 0 || m->gp_ptr[0] != 0 || (m->enr_ptr && m->enr_ptr[0] != 0)) {
        set_error("offset arrays must start at 0");
        return AMIE_BAD_INPUT;
    }
    for (uint32_t e = 0; e < m->n_elem; e++) {
        const int ns = nshape_of(m->kind[e]);
        if (ns == 0 || (m->dim == 2) != (m->kind[e] != AMIE_TET4)) {
            set_error("element %u: kind %d does not match dim %d", e, m->kind[e], m->dim);
            return AMIE_BAD_INPUT;
        }
        if (m->dof_ptr[e + 1] < m->dof_ptr[e] || m->gp_ptr[e + 1] < m->gp_ptr[e]) {
            set_error("element %u: offsets decrease", e);
            return AMIE_BAD_INPUT;
        }
        const uint32_t ne = m->enr_ptr ? m->enr_ptr[e + 1] - m->enr_ptr[e] : 0;
        if (m->enr_ptr && m->enr_ptr[e + 1] < m->enr_ptr[e]) {
            set_error("element %u: enrichment offsets decrease", e);
            return AMIE_BAD_INPUT;
        }
        nf[e] = m->dof_ptr[e + 1] - m->dof_ptr[e];
        if (nf[e] != (uint32_t)ns + ne || nf[e] > (uint32_t)kMaxFunctions) {
            set_error("element %u: %u DOF ids for %d shape + %u enrichment functions (max %d)", e, nf[e], ns, ne,
                      kMaxFunctions);
            return AMIE_BAD_INPUT;
        }
        if (m->mat[e] >= m->n_mat) {
            set_error("element %u: material %u >= n_mat %u", e, m->mat[e], m->n_mat);
            return AMIE_BAD_INPUT;
        }
        if (ne) {
            const uint32_t ngp = m->gp_ptr[e + 1] - m->gp_ptr[e];
            const uint32_t ngp_eff = ngp ? ngp : (m->kind[e] == AMIE_TRI6 ? 4 : 1);
            for (uint32_t j = m->enr_ptr[e]; j < m->enr_ptr[e + 1]; j++) {
                if (m->enr_type[j] == AMIE_ENR_TIP) {
                    // a record of its own; the element's map is affine (straight sides)
                    if (!m->enr_tip || m->enr_data[j] >= m->n_enr_tip || m->enr_vertex[j] > 2 || m->dim != 2 ||
                        (m->moved && m->moved[e])) {
                        set_error("element %u: bad tip enrichment function %u", e, j);
                        return AMIE_BAD_INPUT;
                    }
                    const double br = m->enr_tip[(uint64_t)m->enr_data[j] * 8 + 7];
                    if (!(br == 0.0 || br == 1.0 || br == 2.0 || br == 3.0)) {
                        set_error("element %u: tip enrichment function %u: branch %g not in 0..3", e, j, br);
                        return AMIE_BAD_INPUT;
                    }
                    continue;
                }
                if ((uint64_t)m->enr_data[j] + ngp_eff > m->n_enr_gp) {
                    set_error("element %u: enrichment data of function %u out of range", e, j);
                    return AMIE_BAD_INPUT;
                }
                if (m->enr_type[j] == AMIE_ENR_HEAVISIDE ? (!m->enr_jump || m->enr_vertex[j] > 2 || m->dim != 2)
                                                         : (m->enr_type[j] != AMIE_ENR_TABULATED || !m->enr_grad)) {
                    set_error("element %u: bad enrichment function %u", e, j);
                    return AMIE_BAD_INPUT;
                }
            }
        }
        if (m->moved && m->moved[e] && (m->gp_ptr[e + 1] == m->gp_ptr[e] || !m->jinv_gp)) {
            set_error("element %u: moved elements need explicit Gauss points and jinv_gp", e);
            return AMIE_BAD_INPUT;
        }
        for (uint32_t k = m->dof_ptr[e]; k < m->dof_ptr[e + 1]; k++) max_id = std::max(max_id, m->dof_ids[k]);
    }
    if (max_id >= 0x7fffffffu || (m->ndofmax && m->ndofmax >= 0x7fffffffu)) {
        set_error("DOF ids too large");
        return AMIE_BAD_INPUT;
    }
    n_gp = m->gp_ptr[m->n_elem];
    return AMIE_OK;
}

}  // namespace amie

using namespace amie;

extern "C" amie_status amie_topology_build(amie_ctx *ctx, const amie_mesh *mesh, amie_topo **out)
{
    if (!ctx || !out) return AMIE_BAD_INPUT;
    *out = nullptr;
    std::vector<uint32_t> nf;
    uint64_t n_gp = 0;
    uint32_t max_id = 0;
    AMIE_TRY(validate_mesh(mesh, nf, n_gp, max_id));
    AMIE_CUDA(cudaSetDevice(ctx->device));
    amie_topo *t = new amie_topo();
    auto fail = [&](amie_status s) {
        delete t;
        return s;
    };
    t->ctx = ctx;
    t->dim = mesh->dim;
    t->s = mesh->stride;
    t->nv = mesh->dim == 2 ? 3 : 6;
    t->n_elem = mesh->n_elem;
    t->n_mat = mesh->n_mat;
    t->ndofmax = mesh->ndofmax;
    const uint32_t E = mesh->n_elem;
    const int s = t->s;
    cudaStream_t st = ctx->stream;

    // staged block offsets and kernel partition
    std::vector<uint64_t> blk_off(E + 1, 0);
    std::vector<uint32_t> simple, warp;
    std::vector<QuadChunk> chunks;
    std::vector<QuadLong> longs;
    uint64_t partial = 0;
    for (uint32_t e = 0; e < E; e++) {
        blk_off[e + 1] = blk_off[e] + (uint64_t)nf[e] * nf[e];
        const uint32_t ne = mesh->enr_ptr ? mesh->enr_ptr[e + 1] - mesh->enr_ptr[e] : 0;
        const uint32_t ngp = mesh->gp_ptr[e + 1] - mesh->gp_ptr[e];
        if (!ne) {
            simple.push_back(e);
        } else if (ngp <= (uint32_t)kLongGp) {
            warp.push_back(e);
        } else {   // many Gauss points: chunks on separate SMs, summed in chunk order
            QuadLong L{e, (uint32_t)chunks.size(), 0};
            const uint64_t n_acc = (uint64_t)nf[e] * (nf[e] + 1) / 2 * s * s;
            for (uint32_t g = 0; g < ngp; g += kChunkGp, L.chunk_count++) {
                chunks.push_back(QuadChunk{e, g, std::min<uint32_t>(ngp, g + kChunkGp), partial});
                partial += n_acc;
            }
            longs.push_back(L);
        }
    }
    t->n_blocks_staged = blk_off[E];
    if (t->n_blocks_staged >= 0xffffffffull) {
        delete t;
        set_error("too many element blocks (%llu)", (unsigned long long)blk_off[E]);
        return AMIE_BAD_INPUT;
    }
    t->h_dof_ptr.assign(mesh->dof_ptr, mesh->dof_ptr + E + 1);
    t->n_simple = (uint32_t)simple.size();
    t->n_warp = (uint32_t)warp.size();

    amie_status rc;
#define UP(dst, src, cnt)                                   \
    if ((rc = upload(ctx, dst, src, cnt)) != AMIE_OK) return fail(rc);
    UP(t->kind, mesh->kind, E);
    UP(t->dof_ptr, mesh->dof_ptr, E + 1);
    UP(t->dof_ids, mesh->dof_ids, mesh->dof_ptr[E]);
    UP(t->gp_ptr, mesh->gp_ptr, E + 1);
    UP(t->gp, mesh->gp, n_gp * (t->dim + 1));
    UP(t->jinv, mesh->jinv, (size_t)E * t->dim * t->dim);
    if (mesh->moved) {
        t->has_moved = true;
        UP(t->moved, mesh->moved, E);
        if (mesh->jinv_gp) UP(t->jinv_gp, mesh->jinv_gp, n_gp * t->dim * t->dim);
    }
    UP(t->mat, mesh->mat, E);
    UP(t->cmat_table, mesh->cmat_table, (size_t)mesh->n_mat * t->nv * t->nv);
    if (mesh->cscale) {
        t->has_cscale = true;
        UP(t->cscale, mesh->cscale, E);
    }
    if (mesh->enr_ptr) {
        const uint32_t n_enr = mesh->enr_ptr[E];
        UP(t->enr_ptr, mesh->enr_ptr, E + 1);
        UP(t->enr_type, mesh->enr_type, n_enr);
        UP(t->enr_vertex, mesh->enr_vertex, n_enr);
        UP(t->enr_data, mesh->enr_data, n_enr);
        if (mesh->enr_jump) UP(t->enr_jump, mesh->enr_jump, mesh->n_enr_gp);
        if (mesh->enr_grad) UP(t->enr_grad, mesh->enr_grad, mesh->n_enr_gp * t->dim);
        if (mesh->enr_tip && mesh->n_enr_tip) UP(t->enr_tip, mesh->enr_tip, (size_t)mesh->n_enr_tip * 8);
    }
    UP(t->blk_off, blk_off.data(), E + 1);
    UP(t->simple_list, simple.data(), simple.size());
    UP(t->warp_list, warp.data(), warp.size());
    t->n_chunks = (uint32_t)chunks.size();
    t->n_long = (uint32_t)longs.size();
    if (t->n_long) {
        UP(t->quad_chunks, chunks.data(), chunks.size());
        UP(t->quad_long, longs.data(), longs.size());
        if ((rc = t->quad_partial.alloc(ctx, partial)) != AMIE_OK) return fail(rc);
    }
    if (mesh->scale) {
        bool all_one = true;
        for (uint32_t e = 0; e < E; e++) all_one &= mesh->scale[e] == 1.0;
        if (!all_one) {
            t->has_scale = true;
            UP(t->scale, mesh->scale, E);
            if ((rc = t->blk_elem.alloc(ctx, t->n_blocks_staged)) != AMIE_OK) return fail(rc);
            k_block_elem<<<blocks_for(E, 256), 256, 0, st>>>(E, t->blk_off.p, t->blk_elem.p);
            AMIE_LAUNCHED();
        }
    }
#undef UP

    // ---- pattern: keys of all element pairs + fills, stable radix sort, unique
    const uint32_t n_diag = max_id + 1;
    const uint32_t last = mesh->ndofmax ? mesh->ndofmax - 1 : max_id;
    const uint64_t N = t->n_blocks_staged + n_diag + 1;
    DevArray<uint64_t> keys, keys2;
    DevArray<uint32_t> vals, vals2, is_new, is_contrib, slot_scan, contrib_scan, row_count;
    if ((rc = keys.alloc(ctx, N)) || (rc = keys2.alloc(ctx, N)) || (rc = vals.alloc(ctx, N)) ||
        (rc = vals2.alloc(ctx, N)))
        return fail(rc);
    k_pattern_keys<<<blocks_for(E, 128), 128, 0, st>>>(E, t->dof_ptr.p, t->dof_ids.p, t->blk_off.p, keys.p, vals.p);
    k_fill_keys<<<blocks_for(n_diag + 1, 256), 256, 0, st>>>(t->n_blocks_staged, n_diag, last, keys.p, vals.p);
    g_launches += 2;
    const uint32_t max_row = std::max(max_id, last);
    int end_bit = 32;
    while (end_bit < 64 && (max_row >> (end_bit - 32)) != 0) end_bit++;
    size_t temp_bytes = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, temp_bytes, keys.p, keys2.p, vals.p, vals2.p, (int64_t)N, 0, end_bit, st);
    DevArray<uint8_t> temp;
    size_t scan_bytes = 0;
    cub::DeviceScan::ExclusiveSum(nullptr, scan_bytes, (const uint32_t *)nullptr, (uint32_t *)nullptr, (int64_t)N, st);
    if ((rc = temp.alloc(ctx, std::max(temp_bytes, scan_bytes) + 256))) return fail(rc);
    size_t tb = temp.n;
    AMIE_CUDA(cub::DeviceRadixSort::SortPairs(temp.p, tb, keys.p, keys2.p, vals.p, vals2.p, (int64_t)N, 0, end_bit, st));
    keys.release();
    vals.release();
    if ((rc = is_new.alloc(ctx, N)) || (rc = is_contrib.alloc(ctx, N)) || (rc = slot_scan.alloc(ctx, N)) ||
        (rc = contrib_scan.alloc(ctx, N)))
        return fail(rc);
    k_unique_flags<<<blocks_for(N, 256), 256, 0, st>>>(N, keys2.p, vals2.p, is_new.p, is_contrib.p);
    g_launches += 1;
    tb = temp.n;
    AMIE_CUDA(cub::DeviceScan::ExclusiveSum(temp.p, tb, is_new.p, slot_scan.p, (int64_t)N, st));
    tb = temp.n;
    AMIE_CUDA(cub::DeviceScan::ExclusiveSum(temp.p, tb, is_contrib.p, contrib_scan.p, (int64_t)N, st));
    uint32_t tail[4];
    AMIE_CUDA(cudaMemcpyAsync(&tail[0], slot_scan.p + N - 1, 4, cudaMemcpyDeviceToHost, st));
    AMIE_CUDA(cudaMemcpyAsync(&tail[1], is_new.p + N - 1, 4, cudaMemcpyDeviceToHost, st));
    AMIE_CUDA(cudaMemcpyAsync(&tail[2], contrib_scan.p + N - 1, 4, cudaMemcpyDeviceToHost, st));
    AMIE_CUDA(cudaMemcpyAsync(&tail[3], is_contrib.p + N - 1, 4, cudaMemcpyDeviceToHost, st));
    AMIE_CUDA(cudaStreamSynchronize(st));
    t->nnzb = (uint64_t)tail[0] + tail[1];
    t->n_contrib = (uint64_t)tail[2] + tail[3];
    t->n_rows = max_row + 1;
    t->n = (uint64_t)t->n_rows * s;
    if ((rc = t->col.alloc(ctx, t->nnzb)) || (rc = t->map.alloc(ctx, t->n_contrib)) ||
        (rc = t->map_ptr.alloc(ctx, t->nnzb + 1)) || (rc = row_count.alloc(ctx, t->n_rows + 1)) ||
        (rc = t->row_ptr.alloc(ctx, t->n_rows + 1)))
        return fail(rc);
    AMIE_CUDA(cudaMemsetAsync(row_count.p, 0, (t->n_rows + 1) * 4, st));
    k_pattern_emit<<<blocks_for(N, 256), 256, 0, st>>>(N, keys2.p, vals2.p, is_new.p, slot_scan.p, contrib_scan.p,
                                                       t->col.p, row_count.p, t->map_ptr.p, t->map.p);
    g_launches += 1;
    const uint64_t nc = t->n_contrib;
    AMIE_CUDA(cudaMemcpyAsync(t->map_ptr.p + t->nnzb, &nc, 8, cudaMemcpyHostToDevice, st));
    tb = temp.n;
    AMIE_CUDA(cub::DeviceScan::ExclusiveSum(temp.p, tb, row_count.p, t->row_ptr.p, (int64_t)t->n_rows + 1, st));
    if ((rc = t->diag_pos.alloc(ctx, t->n_rows))) return fail(rc);
    k_diag_pos<<<blocks_for(t->n_rows, 256), 256, 0, st>>>(t->n_rows, t->row_ptr.p, t->col.p, t->diag_pos.p);
    g_launches += 1;
    AMIE_CUDA(cudaStreamSynchronize(st));   // nc lives on this stack frame
    if (t->nnzb >= 0xffffffffull) return fail(AMIE_BAD_INPUT);

    // rows ~ blocks per row -> lanes per block row in the SpMV
    const double avg = (double)t->nnzb / t->n_rows;
    t->spmv_group = avg <= 12 ? 1 : avg <= 24 ? 2 : 4;
    // tuning overrides for measurements: AMIE_SPMV_GROUP = 1, 2, 4, 8, 16 or 32 lanes per
    // block row (block-CSR kernel); AMIE_SELL_VARIANT = 0..7 (SELL kernel loop, see amie_topo)
    if (const char *g = std::getenv("AMIE_SPMV_GROUP")) {
        const int v = std::atoi(g);
        if (v == 1 || v == 2 || v == 4 || v == 8 || v == 16 || v == 32) t->spmv_group = v;
    }
    if (const char *g = std::getenv("AMIE_SELL_VARIANT")) {
        const int v = std::atoi(g);
        if (v >= 0 && v <= 7) t->sell_variant = v;
    }

    // SELL-32-sigma structure: rows sorted by length inside windows, slices of 32.
    // Built on the device (k_sell_perm, k_sell_slots, a scan); the host build below
    // is kept for windows wider than 1024 rows and for AMIE_SELL_HOST=1 (tests
    // compare the two)
    t->n_slices = (t->n_rows + 31) / 32;
    // window of the length sort; tuning override for measurements: AMIE_SELL_SIGMA
    // (a multiple of 32; 32 keeps every slice on 32 consecutive rows)
    uint32_t sigma = kSellSigma;
    if (const char *e = std::getenv("AMIE_SELL_SIGMA")) {
        const long v = std::atol(e);
        if (v >= 32 && v <= (1l << 24) && v % 32 == 0) sigma = (uint32_t)v;
    }
    bool sell_host = sigma > 1024;
    if (const char *e = std::getenv("AMIE_SELL_HOST")) sell_host = sell_host || std::atoi(e) != 0;
    if (!sell_host) {
        const uint64_t n_perm = (uint64_t)t->n_slices * 32;
        DevArray<uint64_t> slots;
        if ((rc = t->sell_perm.alloc(ctx, n_perm)) || (rc = t->sell_ptr.alloc(ctx, (size_t)t->n_slices + 1)) ||
            (rc = slots.alloc(ctx, (size_t)t->n_slices + 1)))
            return fail(rc);
        k_fill_u32<<<blocks_for(n_perm, 256), 256, 0, st>>>(n_perm, t->n_rows, t->sell_perm.p);
        const uint32_t n_win = (t->n_rows + sigma - 1) / sigma;
        k_sell_perm<<<n_win, std::min<uint32_t>(sigma, 1024), sigma * 4, st>>>(t->n_rows, sigma, t->row_ptr.p,
                                                                             t->sell_perm.p);
        k_sell_slots<<<blocks_for((uint64_t)t->n_slices * 32, 256), 256, 0, st>>>(t->n_rows, t->n_slices,
                                                                                 t->sell_perm.p, t->row_ptr.p,
                                                                                 slots.p);
        g_launches += 3;
        AMIE_CUDA(cudaMemsetAsync(slots.p + t->n_slices, 0, 8, st));
        size_t sb = 0;
        AMIE_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, sb, slots.p, t->sell_ptr.p, (int64_t)t->n_slices + 1, st));
        tb = temp.n;
        if (sb > tb) {
            temp.release();
            if ((rc = temp.alloc(ctx, sb))) return fail(rc);
            tb = temp.n;
        }
        AMIE_CUDA(cub::DeviceScan::ExclusiveSum(temp.p, tb, slots.p, t->sell_ptr.p, (int64_t)t->n_slices + 1, st));
        t->h_sell_ptr.resize((size_t)t->n_slices + 1);
        AMIE_CUDA(cudaMemcpyAsync(t->h_sell_ptr.data(), t->sell_ptr.p, ((size_t)t->n_slices + 1) * 8,
                                  cudaMemcpyDeviceToHost, st));
        AMIE_CUDA(cudaStreamSynchronize(st));   // slots and temp are released at the end of this scope
        t->n_slots = t->h_sell_ptr[t->n_slices];
        if ((rc = t->sell_blk.alloc(ctx, t->n_slots)) || (rc = t->sell_col.alloc(ctx, t->n_slots)) ||
            (rc = t->sell_dot.alloc(ctx, t->n_slices)))
            return fail(rc);
        k_sell_fill<<<t->ctx->num_sms * 8, 256, 0, st>>>(t->n_rows, t->n_slices, t->sell_perm.p, t->sell_ptr.p,
                                                         t->row_ptr.p, t->col.p, t->sell_blk.p, t->sell_col.p);
        g_launches += 1;
        AMIE_CUDA(cudaGetLastError());
    } else {
        std::vector<uint32_t> h_rp(t->n_rows + 1);
        AMIE_CUDA(cudaMemcpyAsync(h_rp.data(), t->row_ptr.p, h_rp.size() * 4, cudaMemcpyDeviceToHost, st));
        AMIE_CUDA(cudaStreamSynchronize(st));
        std::vector<uint32_t> perm((size_t)t->n_slices * 32, t->n_rows);
        std::vector<uint64_t> sptr(t->n_slices + 1, 0);
        for (uint32_t w0 = 0; w0 < t->n_rows; w0 += sigma) {
            const uint32_t w1 = std::min<uint32_t>(t->n_rows, w0 + sigma);
            for (uint32_t r = w0; r < w1; r++) perm[r] = r;
            std::stable_sort(perm.begin() + w0, perm.begin() + w1, [&](uint32_t a, uint32_t b) {
                return h_rp[a + 1] - h_rp[a] > h_rp[b + 1] - h_rp[b];
            });
        }
        for (uint32_t sl = 0; sl < t->n_slices; sl++) {
            uint32_t len = 0;
            for (uint32_t l = 0; l < 32; l++) {
                const uint32_t r = perm[(size_t)sl * 32 + l];
                if (r < t->n_rows) len = std::max(len, h_rp[r + 1] - h_rp[r]);
            }
            sptr[sl + 1] = sptr[sl] + 32ull * len;
        }
        t->n_slots = sptr[t->n_slices];
        t->h_sell_ptr = sptr;
        if ((rc = upload(ctx, t->sell_perm, perm.data(), perm.size())) ||
            (rc = upload(ctx, t->sell_ptr, sptr.data(), sptr.size())) ||
            (rc = t->sell_blk.alloc(ctx, t->n_slots)) || (rc = t->sell_col.alloc(ctx, t->n_slots)) ||
            (rc = t->sell_dot.alloc(ctx, t->n_slices)))
            return fail(rc);
        k_sell_fill<<<t->ctx->num_sms * 8, 256, 0, st>>>(t->n_rows, t->n_slices, t->sell_perm.p, t->sell_ptr.p,
                                                         t->row_ptr.p, t->col.p, t->sell_blk.p, t->sell_col.p);
        g_launches += 1;
        AMIE_CUDA(cudaGetLastError());
    }

    // matrix, vectors and staging
    const uint64_t n = t->n;
    if ((rc = t->ke.alloc(ctx, t->n_blocks_staged * s * s)) || (rc = t->val.alloc(ctx, t->nnzb * s * s)) ||
        (rc = t->invdiag.alloc(ctx, n)) || (rc = t->rhs.alloc(ctx, n)) || (rc = t->x.alloc(ctx, n)) ||
        (rc = t->fixed.alloc(ctx, n)) || (rc = t->fixval.alloc(ctx, n)))
        return fail(rc);
    AMIE_CUDA(cudaMemsetAsync(t->rhs.p, 0, n * 8, st));
    AMIE_CUDA(cudaMemsetAsync(t->x.p, 0, n * 8, st));
    AMIE_CUDA(cudaMemsetAsync(t->fixed.p, 0, n, st));
    AMIE_CUDA(cudaStreamSynchronize(st));
    *out = t;
    return AMIE_OK;
}

namespace amie {
void release_solver_state(const amie_topo *t);
}

void release_topology(amie_topo *t)
{
    release_solver_state(t);
    release_damage(t);
    delete t;
}

extern "C" amie_status amie_topology_destroy(amie_topo *t)
{
    if (!t) return AMIE_OK;
    cudaSetDevice(t->ctx->device);
    cudaStreamSynchronize(t->ctx->stream);
    release_topology(t);
    return AMIE_OK;
}

extern "C" amie_status amie_topology_sizes(const amie_topo *t, uint32_t *n_rows, uint64_t *nnzb, uint64_t *n)
{
    if (!t) return AMIE_BAD_INPUT;
    if (n_rows) *n_rows = t->n_rows;
    if (nnzb) *nnzb = t->nnzb;
    if (n) *n = t->n;
    return AMIE_OK;
}

extern "C" amie_status amie_topology_spmv_lanes(const amie_topo *t, int32_t *lanes)
{
    if (!t || !lanes) return AMIE_BAD_INPUT;
    *lanes = t->spmv_group;
    return AMIE_OK;
}

extern "C" amie_status amie_topology_pattern(const amie_topo *t, uint32_t *row_size, uint32_t *column_index)
{
    if (!t) return AMIE_BAD_INPUT;
    cudaSetDevice(t->ctx->device);
    cudaStream_t st = t->ctx->stream;
    if (row_size) {
        std::vector<uint32_t> rp(t->n_rows + 1);
        AMIE_CUDA(cudaMemcpyAsync(rp.data(), t->row_ptr.p, rp.size() * 4, cudaMemcpyDeviceToHost, st));
        AMIE_CUDA(cudaStreamSynchronize(st));
        for (uint32_t k = 0; k < t->n_rows; k++) row_size[k] = rp[k + 1] - rp[k];
    }
    if (column_index) {
        AMIE_CUDA(cudaMemcpyAsync(column_index, t->col.p, t->nnzb * 4, cudaMemcpyDeviceToHost, st));
        AMIE_CUDA(cudaStreamSynchronize(st));
    }
    return AMIE_OK;
}

namespace amie {

// Element matrices + gather on the topology's stream (no synchronisation).
amie_status assemble_async(amie_topo *t)
{
    cudaStream_t st = t->ctx->stream;
    MeshView m = mesh_view(t);
    if (t->n_simple) {
        if (t->dim == 2)
            k_quad_simple<2><<<blocks_for(t->n_simple, 128), 128, 0, st>>>(m, t->simple_list.p, t->n_simple);
        else
            k_quad_simple<3><<<blocks_for(t->n_simple, 128), 128, 0, st>>>(m, t->simple_list.p, t->n_simple);
        AMIE_LAUNCHED();
    }
    if (t->n_long) {
        if (t->dim == 2) {
            k_quad_chunk<2><<<t->n_chunks, 32, 0, st>>>(m, t->quad_chunks.p, t->n_chunks, t->quad_partial.p);
            k_quad_chunk_sum<2><<<t->n_long * kChunkSumSplit, kChunkSumThreads, 0, st>>>(m, t->quad_long.p, t->n_long, t->quad_chunks.p,
                                                           t->quad_partial.p);
        } else {
            k_quad_chunk<3><<<t->n_chunks, 32, 0, st>>>(m, t->quad_chunks.p, t->n_chunks, t->quad_partial.p);
            k_quad_chunk_sum<3><<<t->n_long * kChunkSumSplit, kChunkSumThreads, 0, st>>>(m, t->quad_long.p, t->n_long, t->quad_chunks.p,
                                                           t->quad_partial.p);
        }
        g_launches += 2;
    }
    if (t->n_warp) {
        if (t->dim == 2)
            k_quad_warp<2><<<t->n_warp, 32, 0, st>>>(m, t->warp_list.p, t->n_warp);
        else
            k_quad_warp<3><<<t->n_warp, 32, 0, st>>>(m, t->warp_list.p, t->n_warp);
        AMIE_LAUNCHED();
    }
    const double *sc = t->has_scale ? t->scale.p : nullptr;
    if (t->s == 2)
        k_gather<2><<<blocks_for(t->nnzb, 256), 256, 0, st>>>(t->nnzb, t->map_ptr.p, t->map.p, t->ke.p, t->blk_elem.p, sc,
                                                             t->val.p);
    else
        k_gather<3><<<blocks_for(t->nnzb, 256), 256, 0, st>>>(t->nnzb, t->map_ptr.p, t->map.p, t->ke.p, t->blk_elem.p, sc,
                                                             t->val.p);
    AMIE_LAUNCHED();
    AMIE_CUDA(cudaGetLastError());
    AMIE_CUDA(cudaMemsetAsync(t->rhs.p, 0, t->n * 8, st));
    t->assembled = true;
    t->eliminated = false;
    t->have32 = false;
    return AMIE_OK;
}

// Inverse diagonal (and FP32 copies) of the current matrix.
amie_status finalize_matrix_async(amie_topo *t, bool want32)
{
    cudaStream_t st = t->ctx->stream;
    const uint64_t n = t->n;
    t->sell64_ok = false;
    t->sell32_ok = false;
    float *inv32 = nullptr;
    if (want32) {
        if (!t->val32.p) AMIE_TRY(t->val32.alloc(t->ctx, t->nnzb * t->s * t->s));
        if (!t->invdiag32.p) AMIE_TRY(t->invdiag32.alloc(t->ctx, n));
        inv32 = t->invdiag32.p;
    }
    if (t->s == 2)
        k_invdiag<2><<<blocks_for(n, 256), 256, 0, st>>>(t->n_rows, t->diag_pos.p, t->val.p, t->invdiag.p, inv32);
    else
        k_invdiag<3><<<blocks_for(n, 256), 256, 0, st>>>(t->n_rows, t->diag_pos.p, t->val.p, t->invdiag.p, inv32);
    AMIE_LAUNCHED();
    if (want32) {
        k_to_f32<<<t->ctx->num_sms * 8, 256, 0, st>>>(t->nnzb * t->s * t->s, t->val.p, t->val32.p);
        AMIE_LAUNCHED();
        t->have32 = true;
    }
    AMIE_CUDA(cudaGetLastError());
    return AMIE_OK;
}

// SELL values of the current matrix in FP64 and/or FP32 (allocated on first use).
amie_status ensure_sell(amie_topo *t, bool want64, bool want32)
{
    cudaStream_t st = t->ctx->stream;
    const int g = t->ctx->num_sms * 8;
    if (want64 && !t->sell64_ok) {
        if (!t->sell_val.p) AMIE_TRY(t->sell_val.alloc(t->ctx, t->n_slots * t->s * t->s));
        if (t->s == 2) k_to_sell<2, double><<<g, 256, 0, st>>>(t->n_slots, t->sell_blk.p, t->val.p, t->sell_val.p);
        else k_to_sell<3, double><<<g, 256, 0, st>>>(t->n_slots, t->sell_blk.p, t->val.p, t->sell_val.p);
        AMIE_LAUNCHED();
        t->sell64_ok = true;
    }
    if (want32 && !t->sell32_ok) {
        if (!t->sell_val32.p) AMIE_TRY(t->sell_val32.alloc(t->ctx, t->n_slots * t->s * t->s));
        if (t->s == 2) k_to_sell<2, float><<<g, 256, 0, st>>>(t->n_slots, t->sell_blk.p, t->val.p, t->sell_val32.p);
        else k_to_sell<3, float><<<g, 256, 0, st>>>(t->n_slots, t->sell_blk.p, t->val.p, t->sell_val32.p);
        AMIE_LAUNCHED();
        t->sell32_ok = true;
    }
    AMIE_CUDA(cudaGetLastError());
    return AMIE_OK;
}

// Slice ranges of the CTAs of a SELL SpMV launch with `grid` CTAs: contiguous,
// with about the same number of slots each (built once per grid, synchronously,
// so before any graph capture that uses it).
amie_status ensure_sell_partition(amie_topo *t, int grid)
{
    if (t->sell_cta_first.count(grid)) return AMIE_OK;
    const std::vector<uint64_t> &sp = t->h_sell_ptr;
    std::vector<uint32_t> first(grid + 1);
    const uint64_t total = t->n_slots;
    uint32_t sl = 0;
    for (int b = 0; b <= grid; b++) {
        const uint64_t target = total * (uint64_t)b / (uint64_t)grid;
        while (sl < t->n_slices && sp[sl] < target) sl++;
        first[b] = b == grid ? t->n_slices : sl;
    }
    DevArray<uint32_t> &d = t->sell_cta_first[grid];
    AMIE_TRY(upload(t->ctx, d, first.data(), first.size()));
    AMIE_CUDA(cudaStreamSynchronize(t->ctx->stream));
    return AMIE_OK;
}

amie_status dirichlet_async(amie_topo *t, uint32_t n_bc, const uint32_t *ids_dev, const double *vals_dev,
                            const uint8_t *kinds_dev)
{
    cudaStream_t st = t->ctx->stream;
    AMIE_CUDA(cudaMemsetAsync(t->fixed.p, 0, t->n, st));
    if (n_bc) {
        k_mark_fixed<<<blocks_for(n_bc, 256), 256, 0, st>>>(n_bc, ids_dev, vals_dev, kinds_dev, t->fixed.p, t->fixval.p);
        AMIE_LAUNCHED();
    }
    if (t->s == 2)
        k_dirichlet<2><<<blocks_for(t->n_rows, 128), 128, 0, st>>>(t->n_rows, t->row_ptr.p, t->col.p, t->val.p,
                                                                 t->fixed.p, t->fixval.p, t->rhs.p);
    else
        k_dirichlet<3><<<blocks_for(t->n_rows, 128), 128, 0, st>>>(t->n_rows, t->row_ptr.p, t->col.p, t->val.p,
                                                                 t->fixed.p, t->fixval.p, t->rhs.p);
    AMIE_LAUNCHED();
    if (t->n_force) {
        const uint32_t nf = t->n_force;
        k_add_forces<<<t->force_unique ? blocks_for(nf, 256) : 1, t->force_unique ? 256 : 32, 0, st>>>(
            nf, t->force_ids.p, t->force_vals.p, t->force_unique ? 1 : 0, t->rhs.p);
        AMIE_LAUNCHED();
    }
    AMIE_CUDA(cudaGetLastError());
    t->eliminated = true;
    return AMIE_OK;
}

}  // namespace amie

namespace amie {

// Elimination with the stored multipliers (after a fresh gather).
// rhs += the forces induced by the imposed strain (before elimination: a
// constrained row's right-hand side is then replaced by its value, as the
// reference's force multipliers never reach a constrained DOF).
amie_status add_induced_forces_async(amie_topo *t)
{
    if (!t->has_imposed) return AMIE_OK;
    cudaStream_t st = t->ctx->stream;
    const MeshView m = mesh_view(t);
    if (t->dim == 2) k_elem_forces<2><<<blocks_for(t->n_elem, 128), 128, 0, st>>>(m, t->fstage.p);
    else k_elem_forces<3><<<blocks_for(t->n_elem, 128), 128, 0, st>>>(m, t->fstage.p);
    if (t->s == 2)
        k_force_gather<2><<<blocks_for(t->n_rows, 256), 256, 0, st>>>(t->n_rows, t->fmap_ptr.p, t->fmap.p, t->fstage.p,
                                                                      t->rhs.p);
    else
        k_force_gather<3><<<blocks_for(t->n_rows, 256), 256, 0, st>>>(t->n_rows, t->fmap_ptr.p, t->fmap.p, t->fstage.p,
                                                                      t->rhs.p);
    g_launches += 2;
    AMIE_CUDA(cudaGetLastError());
    return AMIE_OK;
}


// ------------------------------------------------------------------ proportional displacements
// Position of block (row, col) in the block-CSR pattern, or -1 (columns of a
// row are sorted).
__device__ __forceinline__ int64_t find_block(const uint32_t *row_ptr, const uint32_t *col, uint32_t row, uint32_t c)
{
    uint32_t lo = row_ptr[row], hi = row_ptr[row + 1];
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (col[mid] < c) lo = mid + 1;
        else hi = mid;
    }
    return (lo < row_ptr[row + 1] && col[lo] == c) ? (int64_t)lo : -1;
}

// The SET_PROPORTIONAL_DISPLACEMENT branch of Assembly::setBoundaryConditions
// (solvers/assembly.cpp:279-318) for every proportional multiplier in order, one
// CTA: u_id = offset + sum_k c_k u_(p_k) is substituted.  (1) every other row j
// of column id: f_j -= offset A_j,id, A_j,pk += c_k A_j,id, A_j,id = 0; (2) for
// each k in order: row p_k += c_k row id, f_pk += c_k f_id, A_pk,pj += c_j A_pk,id,
// f_pk -= offset A_pk,id, A_pk,id = 0; (3) row id = unit row, f_id = 0.  The
// rows holding column id are the columns of row id (symmetric pattern); an
// entry outside the pattern is dropped, as SparseVector::operator[] drops it
// (sparse/sparse_vector.cpp:38-48).  Every entry sees the reference's
// operations in the reference's order.
template <int S>
__global__ void __launch_bounds__(256) k_proportional(const uint32_t *row_ptr, const uint32_t *col, double *val,
                                                     double *rhs, uint32_t n_prop, const uint32_t *ids,
                                                     const double *offs, const uint32_t *ptr, const uint32_t *dofs,
                                                     const double *coefs)
{
    for (uint32_t m = 0; m < n_prop; m++) {
        const uint32_t id = ids[m], B = id / S, ci = id % S;
        const double off = offs[m];
        const uint32_t k0 = ptr[m], k1 = ptr[m + 1];
        const uint32_t b0 = row_ptr[B], b1 = row_ptr[B + 1];
        // (1) column id, rows other than id and its DOFs
        for (uint32_t t = b0 * S + threadIdx.x; t < b1 * S; t += blockDim.x) {
            const uint32_t J = col[t / S], r = t % S, j = J * S + r;
            bool skip = j == id;
            for (uint32_t k = k0; k < k1; k++) skip |= j == dofs[k];
            if (skip) continue;
            const int64_t q = find_block(row_ptr, col, J, B);
            if (q < 0) continue;
            double *aj = val + (uint64_t)q * S * S + r * S + ci;
            const double a = *aj;
            rhs[j] -= off * a;
            for (uint32_t k = k0; k < k1; k++) {
                const uint32_t p = dofs[k];
                const int64_t qp = find_block(row_ptr, col, J, p / S);
                if (qp >= 0) val[(uint64_t)qp * S * S + r * S + p % S] += coefs[k] * a;
            }
            *aj = 0.0;
        }
        __syncthreads();
        // (2) the rows of its DOFs, in order
        for (uint32_t k = k0; k < k1; k++) {
            const uint32_t p = dofs[k], P = p / S, pr = p % S;
            const double c = coefs[k];
            for (uint32_t t = b0 * S + threadIdx.x; t < b1 * S; t += blockDim.x) {
                const uint32_t C = col[t / S], cc = t % S;
                const int64_t qp = find_block(row_ptr, col, P, C);
                if (qp >= 0) val[(uint64_t)qp * S * S + pr * S + cc] += c * val[(uint64_t)(t / S) * S * S + ci * S + cc];
            }
            __syncthreads();
            if (threadIdx.x == 0) {
                rhs[p] += c * rhs[id];
                const int64_t qi = find_block(row_ptr, col, P, B);
                for (uint32_t k2 = k0; k2 < k1; k2++) {
                    const uint32_t p2 = dofs[k2];
                    const int64_t q2 = find_block(row_ptr, col, P, p2 / S);
                    const double api = qi >= 0 ? val[(uint64_t)qi * S * S + pr * S + ci] : 0.0;
                    if (q2 >= 0) val[(uint64_t)q2 * S * S + pr * S + p2 % S] += coefs[k2] * api;
                }
                const double api = qi >= 0 ? val[(uint64_t)qi * S * S + pr * S + ci] : 0.0;
                rhs[p] -= off * api;
                if (qi >= 0) val[(uint64_t)qi * S * S + pr * S + ci] = 0.0;
            }
            __syncthreads();
        }
        // (3) row id
        for (uint32_t t = b0 * S + threadIdx.x; t < b1 * S; t += blockDim.x) {
            const uint32_t C = col[t / S], cc = t % S;
            val[(uint64_t)(t / S) * S * S + ci * S + cc] = (C * S + cc == id) ? 1.0 : 0.0;
        }
        if (threadIdx.x == 0) rhs[id] = 0.0;
        __syncthreads();
    }
}

// The proportional DOFs of the solution, in multiplier order (Assembly::cgsolve,
// solvers/assembly.cpp:1881-1892): u_id = offset, then u_id += c_k u_(p_k).
__global__ void k_proportional_solution(uint32_t n_prop, const uint32_t *ids, const double *offs, const uint32_t *ptr,
                                        const uint32_t *dofs, const double *coefs, double *x)
{
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    for (uint32_t m = 0; m < n_prop; m++) {
        double v = offs[m];
        for (uint32_t k = ptr[m]; k < ptr[m + 1]; k++) v += coefs[k] * x[dofs[k]];
        x[ids[m]] = v;
    }
}

amie_status proportional_solution_async(amie_topo *t)
{
    if (!t->n_prop) return AMIE_OK;
    k_proportional_solution<<<1, 32, 0, t->ctx->stream>>>(t->n_prop, t->prop_ids.p, t->prop_off.p, t->prop_ptr.p,
                                                          t->prop_dofs.p, t->prop_coefs.p, t->x.p);
    AMIE_LAUNCHED();
    AMIE_CUDA(cudaGetLastError());
    return AMIE_OK;
}

amie_status reapply_dirichlet_async(amie_topo *t)
{
    cudaStream_t st = t->ctx->stream;
    if (t->has_rhs0) AMIE_CUDA(cudaMemcpyAsync(t->rhs.p, t->rhs0.p, t->n * 8, cudaMemcpyDeviceToDevice, st));
    AMIE_TRY(add_induced_forces_async(t));
    AMIE_TRY(dirichlet_async(t, t->n_bc, t->bc_ids.p, t->bc_vals.p, t->has_bc_kinds ? t->bc_kinds.p : nullptr));
    if (t->n_prop) {
        if (t->s == 2)
            k_proportional<2><<<1, 256, 0, st>>>(t->row_ptr.p, t->col.p, t->val.p, t->rhs.p, t->n_prop, t->prop_ids.p,
                                                t->prop_off.p, t->prop_ptr.p, t->prop_dofs.p, t->prop_coefs.p);
        else
            k_proportional<3><<<1, 256, 0, st>>>(t->row_ptr.p, t->col.p, t->val.p, t->rhs.p, t->n_prop, t->prop_ids.p,
                                                t->prop_off.p, t->prop_ptr.p, t->prop_dofs.p, t->prop_coefs.p);
        AMIE_LAUNCHED();
        AMIE_CUDA(cudaGetLastError());
    }
    return AMIE_OK;
}

}  // namespace amie

extern "C" amie_status amie_assemble(amie_topo *t)
{
    if (!t) return AMIE_BAD_INPUT;
    AMIE_CUDA(cudaSetDevice(t->ctx->device));
    AMIE_TRY(assemble_async(t));
    if (t->bc_set || t->n_prop) AMIE_TRY(reapply_dirichlet_async(t));
    else AMIE_TRY(add_induced_forces_async(t));
    AMIE_TRY(finalize_matrix_async(t, false));
    AMIE_CUDA(cudaStreamSynchronize(t->ctx->stream));
    return AMIE_OK;
}

extern "C" amie_status amie_set_imposed_strain(amie_topo *t, const double *eps0)
{
    if (!t) return AMIE_BAD_INPUT;
    AMIE_CUDA(cudaSetDevice(t->ctx->device));
    cudaStream_t st = t->ctx->stream;
    if (!eps0) {
        t->has_imposed = false;
    } else {
        if (!t->fmap_ptr.p) {
            // block row -> staging slots of its (element, function) pairs, in element order
            const uint32_t nfun = t->h_dof_ptr[t->n_elem];
            std::vector<uint32_t> ids(nfun);
            AMIE_CUDA(cudaMemcpyAsync(ids.data(), t->dof_ids.p, (size_t)nfun * 4, cudaMemcpyDeviceToHost, st));
            AMIE_CUDA(cudaStreamSynchronize(st));
            std::vector<uint32_t> ptr(t->n_rows + 1, 0), map(nfun);
            for (uint32_t c = 0; c < nfun; c++) {
                if (ids[c] >= t->n_rows) {
                    set_error("DOF id %u >= %u rows", ids[c], t->n_rows);
                    return AMIE_BAD_INPUT;
                }
                ptr[ids[c] + 1]++;
            }
            for (uint32_t r = 0; r < t->n_rows; r++) ptr[r + 1] += ptr[r];
            std::vector<uint32_t> fill(ptr.begin(), ptr.end() - 1);
            for (uint32_t c = 0; c < nfun; c++) map[fill[ids[c]]++] = c;
            AMIE_TRY(upload(t->ctx, t->fmap_ptr, ptr.data(), ptr.size()));
            AMIE_TRY(upload(t->ctx, t->fmap, map.data(), map.size()));
            AMIE_TRY(t->fstage.alloc(t->ctx, (size_t)nfun * t->s));
        }
        AMIE_TRY(upload(t->ctx, t->imposed, eps0, (size_t)t->n_elem * t->nv));
        t->has_imposed = true;
    }
    AMIE_CUDA(cudaStreamSynchronize(st));
    // an assembled topology gets its right-hand side rebuilt from the original matrix
    if (t->assembled) return amie_assemble(t);
    return AMIE_OK;
}

extern "C" amie_status amie_set_cscale(amie_topo *t, const double *cscale)
{
    if (!t || !cscale) return AMIE_BAD_INPUT;
    AMIE_CUDA(cudaSetDevice(t->ctx->device));
    if (!t->cscale.p) AMIE_TRY(t->cscale.alloc(t->ctx, t->n_elem));
    AMIE_CUDA(cudaMemcpyAsync(t->cscale.p, cscale, (size_t)t->n_elem * 8, cudaMemcpyHostToDevice, t->ctx->stream));
    t->has_cscale = true;
    AMIE_CUDA(cudaStreamSynchronize(t->ctx->stream));
    return AMIE_OK;
}

extern "C" amie_status amie_element_matrices(const amie_topo *t, double *ke, uint64_t capacity)
{
    if (!t || !ke) return AMIE_BAD_INPUT;
    AMIE_CUDA(cudaSetDevice(t->ctx->device));
    const int s = t->s;
    if (capacity < t->n_blocks_staged * s * s) {
        set_error("capacity %llu < %llu", (unsigned long long)capacity,
                  (unsigned long long)(t->n_blocks_staged * s * s));
        return AMIE_BAD_INPUT;
    }
    std::vector<double> blocks(t->n_blocks_staged * s * s);
    AMIE_CUDA(cudaMemcpyAsync(blocks.data(), t->ke.p, blocks.size() * 8, cudaMemcpyDeviceToHost, t->ctx->stream));
    AMIE_CUDA(cudaStreamSynchronize(t->ctx->stream));
    uint64_t off = 0, boff = 0;
    for (uint32_t e = 0; e < t->n_elem; e++) {
        const uint32_t nf = t->h_dof_ptr[e + 1] - t->h_dof_ptr[e];
        const uint32_t msz = nf * s;
        for (uint32_t i = 0; i < nf; i++)
            for (uint32_t j = 0; j < nf; j++)
                for (int r = 0; r < s; r++)
                    for (int c = 0; c < s; c++)
                        ke[off + (uint64_t)(i * s + r) * msz + j * s + c] = blocks[(boff + i * nf + j) * s * s + r * s + c];
        off += (uint64_t)msz * msz;
        boff += (uint64_t)nf * nf;
    }
    return AMIE_OK;
}

extern "C" amie_status amie_apply_dirichlet(amie_topo *t, uint32_t n_bc, const uint32_t *ids, const double *values,
                                            const uint8_t *kinds, const double *rhs0)
{
    if (!t || (n_bc && (!ids || !values))) return AMIE_BAD_INPUT;
    if (!t->assembled) {
        set_error("amie_apply_dirichlet before amie_assemble");
        return AMIE_BAD_INPUT;
    }
    for (uint32_t i = 0; i < n_bc; i++)
        if (ids[i] >= t->n) {
            set_error("multiplier %u: id %u >= n %llu", i, ids[i], (unsigned long long)t->n);
            return AMIE_BAD_INPUT;
        }
    std::vector<uint32_t> fixed;
    for (uint32_t i = 0; i < n_bc; i++)
        if (!kinds || kinds[i] != AMIE_BC_FORCE) fixed.push_back(ids[i]);
    std::sort(fixed.begin(), fixed.end());
    for (uint32_t id : fixed)
        if (std::binary_search(t->prop_sorted.begin(), t->prop_sorted.end(), id)) {
            set_error("DOF %u has a displacement and a proportional multiplier", id);
            return AMIE_BAD_INPUT;
        }
    AMIE_CUDA(cudaSetDevice(t->ctx->device));
    cudaStream_t st = t->ctx->stream;
    if (t->eliminated) {   // re-eliminating needs the original matrix
        AMIE_TRY(assemble_async(t));
    }
    AMIE_CUDA(cudaStreamSynchronize(st));   // the stored multipliers may be replaced below
    t->n_bc = n_bc;
    AMIE_TRY(upload(t->ctx, t->bc_ids, ids, n_bc));
    AMIE_TRY(upload(t->ctx, t->bc_vals, values, n_bc));
    t->has_bc_kinds = kinds != nullptr;
    if (kinds) AMIE_TRY(upload(t->ctx, t->bc_kinds, kinds, n_bc));
    {
        // the force multipliers in multiplier order, and whether a DOF has two
        std::vector<uint32_t> fid;
        std::vector<double> fval;
        for (uint32_t i = 0; kinds && i < n_bc; i++)
            if (kinds[i] == AMIE_BC_FORCE) {
                fid.push_back(ids[i]);
                fval.push_back(values[i]);
            }
        std::vector<uint32_t> sorted(fid);
        std::sort(sorted.begin(), sorted.end());
        t->force_unique = std::adjacent_find(sorted.begin(), sorted.end()) == sorted.end();
        t->n_force = (uint32_t)fid.size();
        if (t->n_force) {
            AMIE_TRY(upload(t->ctx, t->force_ids, fid.data(), fid.size()));
            AMIE_TRY(upload(t->ctx, t->force_vals, fval.data(), fval.size()));
        }
    }
    t->fixed_sorted = std::move(fixed);
    t->has_rhs0 = rhs0 != nullptr;
    if (rhs0) AMIE_TRY(upload(t->ctx, t->rhs0, rhs0, t->n));
    else AMIE_CUDA(cudaMemsetAsync(t->rhs.p, 0, t->n * 8, st));
    t->bc_set = true;
    AMIE_TRY(reapply_dirichlet_async(t));
    AMIE_TRY(finalize_matrix_async(t, false));
    AMIE_CUDA(cudaStreamSynchronize(st));
    return AMIE_OK;
}

extern "C" amie_status amie_set_proportional(amie_topo *t, uint32_t n, const uint32_t *ids, const double *offsets,
                                             const uint32_t *ptr, const uint32_t *prop_ids, const double *coefs)
{
    if (!t || (n && (!ids || !offsets || !ptr))) return AMIE_BAD_INPUT;
    if (n) {
        if (ptr[0] != 0 || (ptr[n] && (!prop_ids || !coefs))) {
            set_error("proportional multipliers: ptr must start at 0 and the DOF arrays be given");
            return AMIE_BAD_INPUT;
        }
        for (uint32_t i = 0; i < n; i++) {
            if (ids[i] >= t->n || ptr[i + 1] < ptr[i]) {
                set_error("proportional multiplier %u: id %u (n %llu) or ptr out of order", i, ids[i],
                          (unsigned long long)t->n);
                return AMIE_BAD_INPUT;
            }
            for (uint32_t k = ptr[i]; k < ptr[i + 1]; k++)
                if (prop_ids[k] >= t->n || prop_ids[k] == ids[i]) {
                    set_error("proportional multiplier %u: DOF %u out of range or the constrained DOF", i, prop_ids[k]);
                    return AMIE_BAD_INPUT;
                }
        }
    }
    std::vector<uint32_t> sorted(ids, ids + n);
    std::sort(sorted.begin(), sorted.end());
    for (uint32_t i = 0; i < n; i++) {
        if (i && sorted[i] == sorted[i - 1]) {
            set_error("proportional multipliers: DOF %u appears twice", sorted[i]);
            return AMIE_BAD_INPUT;
        }
        if (std::binary_search(t->fixed_sorted.begin(), t->fixed_sorted.end(), sorted[i])) {
            set_error("DOF %u has a displacement and a proportional multiplier", sorted[i]);
            return AMIE_BAD_INPUT;
        }
    }
    AMIE_CUDA(cudaSetDevice(t->ctx->device));
    cudaStream_t st = t->ctx->stream;
    AMIE_CUDA(cudaStreamSynchronize(st));   // the stored arrays are replaced below
    t->n_prop = n;
    t->prop_sorted = std::move(sorted);
    if (n) {
        AMIE_TRY(upload(t->ctx, t->prop_ids, ids, n));
        AMIE_TRY(upload(t->ctx, t->prop_off, offsets, n));
        AMIE_TRY(upload(t->ctx, t->prop_ptr, ptr, (size_t)n + 1));
        if (ptr[n]) {
            AMIE_TRY(upload(t->ctx, t->prop_dofs, prop_ids, ptr[n]));
            AMIE_TRY(upload(t->ctx, t->prop_coefs, coefs, ptr[n]));
        }
    }
    if (t->assembled) {   // the original matrix, eliminated again with every stored multiplier
        AMIE_TRY(assemble_async(t));
        if (t->bc_set || t->n_prop) AMIE_TRY(reapply_dirichlet_async(t));
        else AMIE_TRY(add_induced_forces_async(t));
        AMIE_TRY(finalize_matrix_async(t, false));
    }
    AMIE_CUDA(cudaStreamSynchronize(st));
    return AMIE_OK;
}

extern "C" amie_status amie_matrix_download(const amie_topo *t, double *array, double *rhs)
{
    if (!t) return AMIE_BAD_INPUT;
    AMIE_CUDA(cudaSetDevice(t->ctx->device));
    cudaStream_t st = t->ctx->stream;
    if (array) {
        const int s = t->s, cl = s + s % 2;
        DevArray<double> out;
        AMIE_TRY(out.alloc(t->ctx, t->nnzb * s * cl));
        if (s == 2) k_to_amie_layout<2><<<blocks_for(t->nnzb, 256), 256, 0, st>>>(t->nnzb, t->val.p, out.p);
        else k_to_amie_layout<3><<<blocks_for(t->nnzb, 256), 256, 0, st>>>(t->nnzb, t->val.p, out.p);
        AMIE_LAUNCHED();
        AMIE_CUDA(cudaMemcpyAsync(array, out.p, out.bytes(), cudaMemcpyDeviceToHost, st));
        AMIE_CUDA(cudaStreamSynchronize(st));
    }
    if (rhs) {
        AMIE_CUDA(cudaMemcpyAsync(rhs, t->rhs.p, t->n * 8, cudaMemcpyDeviceToHost, st));
        AMIE_CUDA(cudaStreamSynchronize(st));
    }
    return AMIE_OK;
}
