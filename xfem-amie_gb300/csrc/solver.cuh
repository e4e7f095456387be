// solver.cuh -- block-CSR SpMV and fused Jacobi-PCG kernels.
//
// Reference path (paths relative to the AMIE source tree):
//   SpMV       CoordinateIndexedSparseMatrix::inner_product / assign
//              sparse/sparse_matrix.h:203-678, sparse/sparse_matrix.cpp:462-547
//   Jacobi     InverseDiagonal::precondition  solvers/inversediagonal.cpp:62-67
//   dots       parallel_inner_product          utilities/matrixops.h:246-280
//   CG         ConjugateGradient::solve        solvers/conjugategradient.cpp:69-318
//
// One PCG iteration is three kernels, each reading its scalars (alpha, beta,
// the convergence decision) by summing the per-CTA partials of the previous
// kernel itself -- no host round trip and no device-wide barrier:
//   A: q = A p, partial p.q
//   B: alpha = rz / sum(p.q); x += alpha p; r -= alpha q; z = D^-1 r; partial r.z, r.r
//   C: beta = rz_new / rz_old; p = z + beta p   (or set `done` and stop)
// Every kernel returns at once when `done` is set, so a CUDA graph of many
// iterations stops doing work as soon as the solve has converged.
#pragma once

#include "internal.h"

namespace amie {

constexpr int kVecThreads = 256;

// Solver control block in device memory.
struct PcgCtl {
    int32_t done;          // 1 = converged or iteration cap reached
    int32_t pad;
    int64_t iterations;    // completed iterations of the current run
    int64_t maxit;         // iteration cap of the current run
    double tol2;           // stop when r.r <= tol2
    double alpha, beta, rz, rr;   // last values (diagnostics)
};

// Per-CTA partial sums.  rz is double-buffered by iteration parity.
struct PcgParts {
    double *pq;       // [grid]
    double *rz[2];    // [grid] each
    double *rr;       // [grid]
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

// Deterministic sum of `n` partials, computed identically by every CTA that
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

template <typename T> struct Vec2;
template <> struct Vec2<double> { using type = double2; };
template <> struct Vec2<float> { using type = float2; };

// Load one s x s block (row-major) and the s entries of x it multiplies.
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

// y = A x over a group of G lanes per block row; acc in the precision of T.
// Returns, in lane 0 of each group, the row's S outputs.  Every lane of the
// warp must call this (the group reduction shuffles over the full warp); a
// lane whose row is past the end passes valid = false and contributes zero.
template <int S, int G, typename T>
__device__ __forceinline__ void row_spmv(const BsrView<T> &A, const T *__restrict__ x, uint32_t row, bool valid,
                                         int lane, T acc[S])
{
#pragma unroll
    for (int r = 0; r < S; r++) acc[r] = T(0);
    const uint32_t b = valid ? __ldg(A.row_ptr + row) : 0u, e = valid ? __ldg(A.row_ptr + row + 1) : 0u;
    for (uint32_t p = b + lane; p < e; p += G) {
        T blk[S * S], xv[S];
        load_block<S, T>(A.val, p, blk);
        load_x<S, T>(x, __ldg(A.col + p), xv);
#pragma unroll
        for (int r = 0; r < S; r++)
#pragma unroll
            for (int c = 0; c < S; c++) acc[r] = fma(blk[r * S + c], xv[c], acc[r]);
    }
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1)
#pragma unroll
        for (int r = 0; r < S; r++) acc[r] += __shfl_xor_sync(0xffffffffu, acc[r], o, G);
}

// Kernel A: q = A p and per-CTA partial of p.q.
template <int S, int G, typename T>
__global__ void __launch_bounds__(kVecThreads) k_spmv_pq(PcgVecs<T> v, double *part_pq, const PcgCtl *ctl)
{
    __shared__ double sh[33];
    if (ctl && ctl->done) return;
    constexpr int RPB = kVecThreads / G;
    const int lane = threadIdx.x % G;
    double dot = 0.0;
    // the trip count depends on the CTA only, so every lane of a warp reaches the shuffles
    for (uint32_t base = blockIdx.x * RPB; base < v.A.n_rows; base += gridDim.x * RPB) {
        const uint32_t row = base + threadIdx.x / G;
        const bool valid = row < v.A.n_rows;
        T acc[S];
        row_spmv<S, G, T>(v.A, v.p, row, valid, lane, acc);
        if (valid && lane == 0) {
#pragma unroll
            for (int r = 0; r < S; r++) {
                v.q[(uint64_t)row * S + r] = acc[r];
                dot += (double)acc[r] * (double)v.p[(uint64_t)row * S + r];
            }
        }
    }
    dot = block_sum(dot, sh);
    if (threadIdx.x == 0) part_pq[blockIdx.x] = dot;
}

// Plain y = A x (+ optional y = b - A x with partial of y.y).
template <int S, int G, typename T>
__global__ void __launch_bounds__(kVecThreads) k_spmv(BsrView<T> A, const T *x, const T *b, T *y, double *part_yy)
{
    __shared__ double sh[33];
    constexpr int RPB = kVecThreads / G;
    const int lane = threadIdx.x % G;
    double dot = 0.0;
    for (uint32_t base = blockIdx.x * RPB; base < A.n_rows; base += gridDim.x * RPB) {
        const uint32_t row = base + threadIdx.x / G;
        const bool valid = row < A.n_rows;
        T acc[S];
        row_spmv<S, G, T>(A, x, row, valid, lane, acc);
        if (valid && lane == 0) {
#pragma unroll
            for (int r = 0; r < S; r++) {
                const T yv = b ? b[(uint64_t)row * S + r] - acc[r] : acc[r];
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

// Kernel B: alpha = rz / pq; x += alpha p; r -= alpha q; z = D^-1 r; partials r.z, r.r.
template <typename T>
__global__ void __launch_bounds__(kVecThreads) k_update(PcgVecs<T> v, uint64_t n, PcgParts parts, int parity, PcgCtl *ctl)
{
    __shared__ double sh[33];
    if (ctl->done) return;
    const int nparts = gridDim.x;
    const double pq = sum_parts(parts.pq, nparts, sh);
    double *const rz_new_parts = parity ? parts.rz[1] : parts.rz[0];   // select, not a local-memory index
    const double rz = sum_parts(parity ? parts.rz[0] : parts.rz[1], nparts, sh);
    const double alpha = pq != 0.0 ? rz / pq : 0.0;
    const T a = (T)alpha;
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
        rz_new_parts[blockIdx.x] = drz;
        parts.rr[blockIdx.x] = drr;
        if (blockIdx.x == 0) {
            ctl->alpha = alpha;
            ctl->iterations += 1;
        }
    }
}

// Kernel C: convergence test, then beta and p = z + beta p.
template <typename T>
__global__ void __launch_bounds__(kVecThreads) k_direction(PcgVecs<T> v, uint64_t n, PcgParts parts, int parity, PcgCtl *ctl)
{
    __shared__ double sh[33];
    if (ctl->done) return;
    const int nparts = gridDim.x;
    const double rz_new = sum_parts(parity ? parts.rz[1] : parts.rz[0], nparts, sh);
    const double rz_old = sum_parts(parity ? parts.rz[0] : parts.rz[1], nparts, sh);
    const double rr = sum_parts(parts.rr, nparts, sh);
    const int64_t it = ctl->iterations;   // written by the previous kernel
    const bool stop = rr <= ctl->tol2 || it >= ctl->maxit || !(rr == rr);
    if (stop) {
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            ctl->done = 1;
            ctl->rr = rr;
            ctl->rz = rz_new;
        }
        return;
    }
    const double beta = rz_old != 0.0 ? rz_new / rz_old : 0.0;
    const T bt = (T)beta;
    for (uint64_t i = (uint64_t)blockIdx.x * kVecThreads + threadIdx.x; i < n; i += (uint64_t)gridDim.x * kVecThreads)
        v.p[i] = v.z[i] + bt * v.p[i];
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        ctl->beta = beta;
        ctl->rr = rr;
        ctl->rz = rz_new;
    }
}

// Start of a PCG run from the residual r (already holding b - A x):
// z = D^-1 r, p = z, partials r.z (into rz[1], read by iteration 0) and r.r.
template <typename T>
__global__ void __launch_bounds__(kVecThreads) k_pcg_start(PcgVecs<T> v, uint64_t n, PcgParts parts)
{
    __shared__ double sh[33];
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
        parts.rz[1][blockIdx.x] = drz;
        parts.rr[blockIdx.x] = drr;
    }
}

}  // namespace amie
