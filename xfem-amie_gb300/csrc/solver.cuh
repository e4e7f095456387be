// solver.cuh -- block-CSR SpMV and fused Jacobi-PCG kernels.
//
// Reference path (paths relative to the AMIE source tree):
//   SpMV       CoordinateIndexedSparseMatrix::inner_product / assign
//              sparse/sparse_matrix.h:203-678, sparse/sparse_matrix.cpp:462-547
//   Jacobi     InverseDiagonal::precondition  solvers/inversediagonal.cpp:62-67
//   dots       parallel_inner_product          utilities/matrixops.h:246-280
//   CG         ConjugateGradient::solve        solvers/conjugategradient.cpp:69-318
//
// One PCG iteration is three kernels:
//   A: q = A p, partial p.q;                         last CTA: pq, alpha = rz / pq
//   B: x += alpha p; r -= alpha q; z = D^-1 r, partial r.z, r.r;
//                                                    last CTA: rz, rr, stop test, beta
//   C: p = z + beta p
// Each reduction is finished once, by the last CTA of the kernel that produced
// the per-CTA partials (a ticket counter; the partials are summed in index
// order, so results are deterministic), and the next kernel reads scalars from
// the control block: no host round trip, no device-wide barrier, no waiting.
// Every kernel returns at once when `done` is set, so a CUDA graph of many
// iterations stops doing work as soon as the solve has converged.
#pragma once

#include "internal.h"

namespace amie {

constexpr int kVecThreads = 256;

// Solver control block in device memory.  `done` is the first member: the
// SpMV kernel's early exit also reads it from the AMIE_CG control block.
struct PcgCtl {
    int32_t done;          // 1 = converged or iteration cap reached
    uint32_t ticket;       // CTAs finished in the current kernel
    int64_t iterations;    // completed iterations of the current run
    int64_t maxit;         // iteration cap of the current run
    double tol2;           // stop when r.r <= tol2
    double alpha, beta, rz, rr, pq;
};

// Per-CTA partial sums.
struct PcgParts {
    double *pq;       // [grid]
    double *rz;       // [grid]
    double *rr;       // [grid]
    double *spare;    // [grid]
};

template <typename T>
struct PcgVecs {
    BsrView<T> A;
    const T *dinv;
    T *x, *r, *z, *p, *q;
};

__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Sum of one value per thread over the CTA (kVecThreads threads); result valid in thread 0.
__device__ __forceinline__ double block_sum(double v, double *sh)
{
    v = warp_sum(v);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) sh[w] = v;
    __syncthreads();
    double r = 0.0;
    if (w == 0) {
        r = l < (kVecThreads >> 5) ? sh[l] : 0.0;
        r = warp_sum(r);
    }
    __syncthreads();
    return r;
}

// Deterministic sum of `n` partials (index order per thread, then a fixed
// tree); read through L2 because other CTAs wrote them.  Valid in thread 0.
__device__ __forceinline__ double ordered_sum(const double *parts, int n, double *sh)
{
    double v = 0.0;
    for (int i = threadIdx.x; i < n; i += kVecThreads) v += __ldcg(parts + i);
    return block_sum(v, sh);
}

// Deterministic sum of `n` partials computed identically by every CTA that
// needs it; broadcast to all threads of the CTA.
__device__ __forceinline__ double sum_parts(const double *parts, int n, double *sh)
{
    double v = 0.0;
    for (int i = threadIdx.x; i < n; i += kVecThreads) v += parts[i];
    v = block_sum(v, sh);
    if (threadIdx.x == 0) sh[32] = v;
    __syncthreads();
    const double r = sh[32];
    __syncthreads();
    return r;
}

// Every CTA calls this after thread 0 stored the CTA's partials; returns true
// in the last CTA to finish (all partials of the kernel are then visible).
__device__ __forceinline__ bool last_cta(uint32_t *ticket, int *sh_flag)
{
    if (threadIdx.x == 0) {
        __threadfence();
        const uint32_t t = atomicAdd(ticket, 1u);
        *sh_flag = (t == gridDim.x - 1) ? 1 : 0;
    }
    __syncthreads();
    const bool last = *sh_flag != 0;
    if (last) __threadfence();
    return last;
}

template <typename T> struct Vec2;
template <> struct Vec2<double> { using type = double2; };
template <> struct Vec2<float> { using type = float2; };

// Load one s x s block (row-major).
template <int S, typename T>
__device__ __forceinline__ void load_block(const T *__restrict__ val, uint64_t p, T blk[S * S])
{
    if constexpr (S == 2 && sizeof(T) == 8) {
        const double2 *v = reinterpret_cast<const double2 *>(val + p * 4);
        const double2 a = __ldg(v), b = __ldg(v + 1);
        blk[0] = a.x; blk[1] = a.y; blk[2] = b.x; blk[3] = b.y;
    } else if constexpr (S == 2 && sizeof(T) == 4) {
        const float4 a = __ldg(reinterpret_cast<const float4 *>(val + p * 4));
        blk[0] = a.x; blk[1] = a.y; blk[2] = a.z; blk[3] = a.w;
    } else {
#pragma unroll
        for (int q = 0; q < S * S; q++) blk[q] = __ldg(val + p * S * S + q);
    }
}

template <int S, typename T>
__device__ __forceinline__ void load_x(const T *__restrict__ x, uint32_t c, T xv[S])
{
    if constexpr (S == 2) {
        using V = typename Vec2<T>::type;
        const V a = __ldg(reinterpret_cast<const V *>(x + (uint64_t)c * 2));
        xv[0] = a.x; xv[1] = a.y;
    } else {
#pragma unroll
        for (int q = 0; q < S; q++) xv[q] = __ldg(x + (uint64_t)c * S + q);
    }
}

constexpr int kSpmvUnroll = 4;

// y = A x over a group of G lanes per block row; acc in the precision of T.
// Blocks are fetched kSpmvUnroll at a time (columns and values first, then the
// x entries they select) so each lane keeps several independent loads in
// flight.  Returns, in lane 0 of each group, the row's S outputs.  Every lane
// of the warp must call this (the group reduction shuffles over the full
// warp); a lane whose row is past the end passes b == e and contributes zero.
template <int S, int G, typename T>
__device__ __forceinline__ void row_spmv(const BsrView<T> &A, const T *__restrict__ x, uint32_t b, uint32_t e, int lane,
                                         T acc[S])
{
#pragma unroll
    for (int r = 0; r < S; r++) acc[r] = T(0);
    for (uint32_t p0 = b + lane; p0 < e; p0 += kSpmvUnroll * G) {
        uint32_t c[kSpmvUnroll];
        T blk[kSpmvUnroll][S * S];
#pragma unroll
        for (int u = 0; u < kSpmvUnroll; u++) {
            const uint32_t p = p0 + u * G;
            if (p < e) {
                c[u] = __ldg(A.col + p);
                load_block<S, T>(A.val, p, blk[u]);
            }
        }
#pragma unroll
        for (int u = 0; u < kSpmvUnroll; u++) {
            if (p0 + u * G < e) {
                T xv[S];
                load_x<S, T>(x, c[u], xv);
#pragma unroll
                for (int r = 0; r < S; r++)
#pragma unroll
                    for (int cc = 0; cc < S; cc++) acc[r] = fma(blk[u][r * S + cc], xv[cc], acc[r]);
            }
        }
    }
    if constexpr (G > 1) {
#pragma unroll
        for (int o = G / 2; o > 0; o >>= 1)
#pragma unroll
            for (int r = 0; r < S; r++) acc[r] += __shfl_xor_sync(0xffffffffu, acc[r], o, G);
    }
}

// Kernel A: q = A p and per-CTA partial of p.q.  `done` (nullable) stops the
// kernel; `fin` (nullable) receives pq and alpha = rz / pq from the last CTA.
template <int S, int G, typename T>
__global__ void __launch_bounds__(kVecThreads) k_spmv_pq(PcgVecs<T> v, double *part_pq, const int32_t *done, PcgCtl *fin)
{
    __shared__ double sh[33];
    __shared__ int flag;
    if (done && *done) return;
    constexpr int RPB = kVecThreads / G;
    const int lane = threadIdx.x % G;
    const uint32_t n_rows = v.A.n_rows;
    double dot = 0.0;
    // the trip count depends on the CTA only, so every lane of a warp reaches the shuffles;
    // the next pass's row bounds are fetched while the current row is processed
    uint32_t row = blockIdx.x * RPB + threadIdx.x / G;
    uint32_t b = row < n_rows ? __ldg(v.A.row_ptr + row) : 0u, e = row < n_rows ? __ldg(v.A.row_ptr + row + 1) : 0u;
    for (uint32_t base = blockIdx.x * RPB; base < n_rows; base += gridDim.x * RPB) {
        const uint32_t nrow = row + gridDim.x * RPB;
        const uint32_t nb = nrow < n_rows ? __ldg(v.A.row_ptr + nrow) : 0u;
        const uint32_t ne = nrow < n_rows ? __ldg(v.A.row_ptr + nrow + 1) : 0u;
        T acc[S];
        row_spmv<S, G, T>(v.A, v.p, b, e, lane, acc);
        if (row < n_rows && lane == 0) {
#pragma unroll
            for (int r = 0; r < S; r++) {
                v.q[(uint64_t)row * S + r] = acc[r];
                dot += (double)acc[r] * (double)v.p[(uint64_t)row * S + r];
            }
        }
        row = nrow;
        b = nb;
        e = ne;
    }
    dot = block_sum(dot, sh);
    if (threadIdx.x == 0) part_pq[blockIdx.x] = dot;
    if (!fin) return;
    if (!last_cta(&fin->ticket, &flag)) return;
    const double pq = ordered_sum(part_pq, gridDim.x, sh);
    if (threadIdx.x == 0) {
        fin->pq = pq;
        fin->alpha = pq != 0.0 ? fin->rz / pq : 0.0;
        fin->ticket = 0;
    }
}

// Plain y = A x (+ optional y = b - A x with partial of y.y).
template <int S, int G, typename T>
__global__ void __launch_bounds__(kVecThreads) k_spmv(BsrView<T> A, const T *x, const T *bvec, T *y, double *part_yy)
{
    __shared__ double sh[33];
    constexpr int RPB = kVecThreads / G;
    const int lane = threadIdx.x % G;
    double dot = 0.0;
    for (uint32_t base = blockIdx.x * RPB; base < A.n_rows; base += gridDim.x * RPB) {
        const uint32_t row = base + threadIdx.x / G;
        const bool valid = row < A.n_rows;
        const uint32_t b = valid ? __ldg(A.row_ptr + row) : 0u, e = valid ? __ldg(A.row_ptr + row + 1) : 0u;
        T acc[S];
        row_spmv<S, G, T>(A, x, b, e, lane, acc);
        if (valid && lane == 0) {
#pragma unroll
            for (int r = 0; r < S; r++) {
                const T yv = bvec ? bvec[(uint64_t)row * S + r] - acc[r] : acc[r];
                y[(uint64_t)row * S + r] = yv;
                dot += (double)yv * (double)yv;
            }
        }
    }
    if (part_yy) {
        dot = block_sum(dot, sh);
        if (threadIdx.x == 0) part_yy[blockIdx.x] = dot;
    }
}

// Kernel B: x += alpha p; r -= alpha q; z = D^-1 r; partials r.z, r.r.
// Last CTA: totals, iteration count, stop test, beta = rz_new / rz.
template <typename T>
__global__ void __launch_bounds__(kVecThreads) k_update(PcgVecs<T> v, uint64_t n, PcgParts parts, PcgCtl *ctl)
{
    __shared__ double sh[33];
    __shared__ int flag;
    if (ctl->done) return;
    const T a = (T)ctl->alpha;
    double drz = 0.0, drr = 0.0;
    for (uint64_t i = (uint64_t)blockIdx.x * kVecThreads + threadIdx.x; i < n; i += (uint64_t)gridDim.x * kVecThreads) {
        const T ri = v.r[i] - a * v.q[i];
        v.x[i] += a * v.p[i];
        v.r[i] = ri;
        const T zi = ri * v.dinv[i];
        v.z[i] = zi;
        drz += (double)ri * (double)zi;
        drr += (double)ri * (double)ri;
    }
    drz = block_sum(drz, sh);
    drr = block_sum(drr, sh);
    if (threadIdx.x == 0) {
        parts.rz[blockIdx.x] = drz;
        parts.rr[blockIdx.x] = drr;
    }
    if (!last_cta(&ctl->ticket, &flag)) return;
    const double rz_new = ordered_sum(parts.rz, gridDim.x, sh);
    const double rr = ordered_sum(parts.rr, gridDim.x, sh);
    if (threadIdx.x == 0) {
        const int64_t it = ctl->iterations + 1;
        ctl->iterations = it;
        ctl->rr = rr;
        const bool stop = rr <= ctl->tol2 || it >= ctl->maxit || !(rr == rr);
        if (stop) {
            ctl->done = 1;
        } else {
            ctl->beta = ctl->rz != 0.0 ? rz_new / ctl->rz : 0.0;
        }
        ctl->rz = rz_new;
        ctl->ticket = 0;
    }
}

// Kernel C: p = z + beta p.
template <typename T>
__global__ void __launch_bounds__(kVecThreads) k_direction(PcgVecs<T> v, uint64_t n, const PcgCtl *ctl)
{
    if (ctl->done) return;
    const T bt = (T)ctl->beta;
    for (uint64_t i = (uint64_t)blockIdx.x * kVecThreads + threadIdx.x; i < n; i += (uint64_t)gridDim.x * kVecThreads)
        v.p[i] = v.z[i] + bt * v.p[i];
}

// Start of a PCG run from the residual r (already holding b - A x):
// z = D^-1 r, p = z; last CTA: rz and rr into the control block.
template <typename T>
__global__ void __launch_bounds__(kVecThreads) k_pcg_start(PcgVecs<T> v, uint64_t n, PcgParts parts, PcgCtl *ctl)
{
    __shared__ double sh[33];
    __shared__ int flag;
    double drz = 0.0, drr = 0.0;
    for (uint64_t i = (uint64_t)blockIdx.x * kVecThreads + threadIdx.x; i < n; i += (uint64_t)gridDim.x * kVecThreads) {
        const T ri = v.r[i];
        const T zi = ri * v.dinv[i];
        v.z[i] = zi;
        v.p[i] = zi;
        drz += (double)ri * (double)zi;
        drr += (double)ri * (double)ri;
    }
    drz = block_sum(drz, sh);
    drr = block_sum(drr, sh);
    if (threadIdx.x == 0) {
        parts.rz[blockIdx.x] = drz;
        parts.rr[blockIdx.x] = drr;
    }
    if (!last_cta(&ctl->ticket, &flag)) return;
    const double rz = ordered_sum(parts.rz, gridDim.x, sh);
    const double rr = ordered_sum(parts.rr, gridDim.x, sh);
    if (threadIdx.x == 0) {
        ctl->rz = rz;
        ctl->rr = rr;
        ctl->ticket = 0;
    }
}

}  // namespace amie
