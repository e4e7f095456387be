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

#include <type_traits>

namespace amie {

constexpr int kVecThreads = 256;

// Stopping targets of the PCG drivers, as fractions of the requested relative
// residual rtol.  FP64: once the true residual meets rtol (first stage,
// recursive target 0.5 rtol) the recursion continues towards kFp64StopFraction
// rtol within a quarter more iterations; at rtol = 1e-10 this keeps node
// displacements within 1e-9 (relative to the largest) of a 1e-13 solve on the
// 1.2 M-DOF P2 workload (5.8e-10; 4.1e-9 when stopped at 0.5 rtol) for 3.5 %
// more iterations.  Mixed: the FP32 recursion is replaced by the true residual
// after every reduction by kMixedInner, the last FP32 segment aims at
// kMixedLastTarget rtol and the solve stops once the true residual is below
// rtol.  A run whose segments take more than kMixedLongSegment iterations
// drifts in FP32 and is ill-conditioned: it is replaced after every reduction
// by kMixedInnerLong and stops below kMixedStopLong rtol.  Measured (mixed,
// rtol 1e-10; iterations, node error vs a 1e-13 solve):
//   1.2 M-DOF P2   inner 0.1: 19,307, 4.3e-9; 0.3: 16,109, 1.0e-8 (over the
//                  1e-8 bound); 0.3 with the stop at 0.5 rtol: 16,702, 6.7e-9
//                  (620 instead of 720 ms)
//   40 k-DOF P1    inner 0.1: 1,585 in 18.4 ms; 0.3: 1,581 in 19.9 ms (nine
//                  more replacements, no fewer iterations)
//   824 k-DOF tets inner 0.1: 1,281 in 63.7 ms; 0.3: 1,281 in 65.5 ms
// Segments there: ~1,700, ~160 and ~130 iterations.  Switching to 0.5 with the
// stop at 0.2 rtol instead made the 1.2 M-DOF step 799 ms (21,415 iterations):
// segments that only halve the residual meet the restart rule of solve_pcg (a
// true residual that fell by less than half) and lose their directions; with
// that rule scaled to the segment's target (restart below a fall of 2x the
// target) it was 625 ms (16,683 iterations, stop at 0.3 rtol).  The serving
// path keeps its own constants.
constexpr double kFp64StopFraction = 0.1;
constexpr double kMixedLastTarget = 0.2;
constexpr double kMixedInner = 0.1;
constexpr int64_t kMixedLongSegment = 1000;
constexpr double kMixedInnerLong = 0.3;
constexpr double kMixedStopLong = 0.5;

// Programmatic dependent launch: a kernel launched with programmatic stream
// serialization may start while its predecessor finishes; pdl_wait() blocks
// (in hardware) until the predecessor grid has completed and its writes are
// visible, pdl_release() lets the successor grid be scheduled.  Both are
// no-ops for a kernel launched without the attribute.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_release() { asm volatile("griddepcontrol.launch_dependents;" :::); }

// Solver control block in device memory.  `done` is the first member: the
// SpMV kernel's early exit also reads it from the AMIE_CG control block.
struct PcgCtl {
    int32_t done;          // 1 = converged or iteration cap reached
    uint32_t ticket;       // CTAs finished in the current kernel
    int64_t iterations;    // completed iterations of the current run
    int64_t maxit;         // iteration cap of the current run
    double tol2;           // stop when r.r <= tol2
    double alpha, beta, rz, rr, pq;
    double rz_prev;        // r.z of the iteration before the last one (kept for a resumed run)
    int32_t pcur;          // with two direction buffers: the one holding the latest p (0 = p, 1 = p2)
    int32_t first;         // one-kernel PCG: the next kernel starts a run (alpha = 0, not an iteration)
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
    T *p2 = nullptr;   // second direction buffer: p = z + beta p is then formed inside k_sell_dir
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

// CTA sum of one value per thread given in the vector precision T: the warp
// levels add in T, the per-warp sums in FP64.  Result valid in thread 0.
template <typename T>
__device__ __forceinline__ double block_sum_v(T v, double *sh)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) sh[w] = (double)v;
    __syncthreads();
    double r = 0.0;
    if (w == 0) {
        r = l < (kVecThreads >> 5) ? sh[l] : 0.0;
#pragma unroll
        for (int o = (kVecThreads >> 6); o > 0; o >>= 1) r += __shfl_xor_sync(0xffffffffu, r, o);
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

// CTA sums of two values per thread (vector precision T, per-warp sums in
// FP64) with one pair of barriers.  Results valid in thread 0.
template <typename T>
__device__ __forceinline__ void block_sum2_v(T a, T b, double *sh, double &ra, double &rb)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_xor_sync(0xffffffffu, a, o);
        b += __shfl_xor_sync(0xffffffffu, b, o);
    }
    constexpr int NW = kVecThreads >> 5;
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) {
        sh[w] = (double)a;
        sh[NW + w] = (double)b;
    }
    __syncthreads();
    double x = 0.0, y = 0.0;
    if (w == 0) {
        x = l < NW ? sh[l] : 0.0;
        y = l < NW ? sh[NW + l] : 0.0;
#pragma unroll
        for (int o = NW >> 1; o > 0; o >>= 1) {
            x += __shfl_xor_sync(0xffffffffu, x, o);
            y += __shfl_xor_sync(0xffffffffu, y, o);
        }
    }
    __syncthreads();
    ra = x;
    rb = y;
}

// ordered_sum of two partial arrays in one pass.  Valid in thread 0.
__device__ __forceinline__ void ordered_sum2(const double *pa, const double *pb, int n, double *sh, double &ra,
                                             double &rb)
{
    double a = 0.0, b = 0.0;
    for (int i = threadIdx.x; i < n; i += kVecThreads) {
        a += __ldcg(pa + i);
        b += __ldcg(pb + i);
    }
    block_sum2_v<double>(a, b, sh, ra, rb);
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

// Position of a CTA in the group of CTAs that share one reduction and one
// control block: the whole grid for a single solve, one slot's CTA range in a
// batched launch (the kernel bodies below take it explicitly).
struct Cta {
    uint32_t id, n;
};
__device__ __forceinline__ Cta grid_cta() { return Cta{blockIdx.x, gridDim.x}; }

// Every CTA of a group of `n` calls this after thread 0 stored the CTA's
// partials; returns true in the last CTA to finish (all partials of the group
// are then visible).
__device__ __forceinline__ bool last_cta(uint32_t *ticket, int *sh_flag, uint32_t n)
{
    if (threadIdx.x == 0) {
        __threadfence();
        const uint32_t t = atomicAdd(ticket, 1u);
        *sh_flag = (t == n - 1) ? 1 : 0;
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

// load_x through L2 only (ld.global.cg): for vectors other CTAs of a running
// persistent kernel rewrite between its phases (an SM's L1 is not coherent
// with the others' stores).
template <int S, typename T>
__device__ __forceinline__ void load_x_cg(const T *x, uint32_t c, T xv[S])
{
    if constexpr (S == 2) {
        using V = typename Vec2<T>::type;
        const V a = __ldcg(reinterpret_cast<const V *>(x + (uint64_t)c * 2));
        xv[0] = a.x; xv[1] = a.y;
    } else {
#pragma unroll
        for (int q = 0; q < S; q++) xv[q] = __ldcg(x + (uint64_t)c * S + q);
    }
}

// A control-block field: inside a persistent kernel (CG) written by other CTAs
// during the launch, so read through L2; otherwise a plain load (the writer
// was an earlier kernel).
template <bool CG, typename F>
__device__ __forceinline__ F ctl_ld(const F *p)
{
    if constexpr (CG) return __ldcg(p);
    else return *p;
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

// Per-CTA partial of p.q; with `fin`, the last CTA stores pq and alpha = rz / pq.
template <typename T, bool CG = false>
__device__ __forceinline__ void finish_pq(T dot_t, double *part_pq, PcgCtl *fin, double *sh, int *flag, Cta c)
{
    // r.z was stored by the previous update: fetched now, it arrives during the reductions
    const double rz = (fin && threadIdx.x == 0) ? ctl_ld<CG>(&fin->rz) : 0.0;
    const double dot = block_sum_v<T>(dot_t, sh);
    if (threadIdx.x == 0) part_pq[c.id] = dot;
    if (!fin) return;
    if (!last_cta(&fin->ticket, flag, c.n)) return;
    const double pq = ordered_sum(part_pq, c.n, sh);
    if (threadIdx.x == 0) {
        fin->pq = pq;
        fin->alpha = pq != 0.0 ? rz / pq : 0.0;
        fin->ticket = 0;
    }
}

// Kernel A: q = A p and per-CTA partial of p.q.  `done` (nullable) stops the
// kernel; `fin` (nullable) receives pq and alpha = rz / pq from the last CTA.
template <int S, int G, typename T>
__global__ void __launch_bounds__(kVecThreads) k_spmv_pq(PcgVecs<T> v, double *part_pq, const int32_t *done, PcgCtl *fin)
{
    __shared__ double sh[33];
    __shared__ int flag;
    pdl_wait();
    pdl_release();
    if (done && *done) return;
    constexpr int RPB = kVecThreads / G;
    const int lane = threadIdx.x % G;
    const uint32_t n_rows = v.A.n_rows;
    T dot = T(0);
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
                dot = fma(acc[r], v.p[(uint64_t)row * S + r], dot);
            }
        }
        row = nrow;
        b = nb;
        e = ne;
    }
    finish_pq<T>(dot, part_pq, fin, sh, &flag, grid_cta());
}

// Matrix-stream loads with an L2 eviction hint.  HINT 0: plain read-only
// loads; 1: ld.global.cs (lines allocated evict-first in L1 and L2); 2: an L2
// evict-first access policy (createpolicy).  The matrix is read once per
// iteration and is larger than L2, so without a hint it pushes the iteration's
// vectors out of L2.  Measured on the 1.2 M-DOF P2 problem (FP32 matrix 150 MB,
// vectors 29 MB): the SpMV+direction kernel takes 32.1 us with 0, 26.7 us
// with 1 (the vector gathers and the next kernel's reads stay in L2) and
// 45 us with 2.  1 is the default of the single-solve kernels; the batched
// server passes 0, its small matrices being re-read from L2 every iteration.
constexpr int kMatrixHint = 1;
template <int HINT>
__device__ __forceinline__ uint64_t stream_policy()
{
    uint64_t pol = 0;
    if constexpr (HINT == 2) asm("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
    return pol;
}

template <int HINT, typename V>
__device__ __forceinline__ V ld_stream(const V *p, uint64_t pol)
{
    if constexpr (HINT == 1) {
        return __ldcs(p);
    } else if constexpr (HINT == 2) {
        V v;
        if constexpr (sizeof(V) == 16 && std::is_same_v<V, float4>)
            asm volatile("ld.global.nc.L2::cache_hint.v4.f32 {%0, %1, %2, %3}, [%4], %5;"
                         : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w) : "l"(p), "l"(pol));
        else if constexpr (std::is_same_v<V, double2>)
            asm volatile("ld.global.nc.L2::cache_hint.v2.f64 {%0, %1}, [%2], %3;"
                         : "=d"(v.x), "=d"(v.y) : "l"(p), "l"(pol));
        else if constexpr (std::is_same_v<V, float>)
            asm volatile("ld.global.nc.L2::cache_hint.f32 %0, [%1], %2;" : "=f"(v) : "l"(p), "l"(pol));
        else if constexpr (std::is_same_v<V, double>)
            asm volatile("ld.global.nc.L2::cache_hint.f64 %0, [%1], %2;" : "=d"(v) : "l"(p), "l"(pol));
        else
            asm volatile("ld.global.nc.L2::cache_hint.u32 %0, [%1], %2;" : "=r"(v) : "l"(p), "l"(pol));
        return v;
    } else {
        return __ldg(p);
    }
}

// One s x s block of the lane's row from a 32-slot SELL group (chunked layout).
template <int S, typename T, int HINT = kMatrixHint>
__device__ __forceinline__ void load_sell_block(const T *__restrict__ group, uint32_t lane, T blk[S * S],
                                                uint64_t pol = 0)
{
    constexpr int V = kSellVec<S, T>;
    if constexpr (S == 2 && V == 4) {
        const float4 a = ld_stream<HINT>(reinterpret_cast<const float4 *>(group) + lane, pol);
        blk[0] = a.x; blk[1] = a.y; blk[2] = a.z; blk[3] = a.w;
    } else if constexpr (S == 2 && V == 2) {
        const double2 a = ld_stream<HINT>(reinterpret_cast<const double2 *>(group) + lane, pol);
        const double2 b = ld_stream<HINT>(reinterpret_cast<const double2 *>(group + 64) + lane, pol);
        blk[0] = a.x; blk[1] = a.y; blk[2] = b.x; blk[3] = b.y;
    } else if constexpr (S == 3 && V == 4) {
        // components 0-3 and 4-7 as two 16-byte chunks, component 8 on its own
        const float4 a = ld_stream<HINT>(reinterpret_cast<const float4 *>(group) + lane, pol);
        const float4 b = ld_stream<HINT>(reinterpret_cast<const float4 *>(group + 128) + lane, pol);
        blk[0] = a.x; blk[1] = a.y; blk[2] = a.z; blk[3] = a.w;
        blk[4] = b.x; blk[5] = b.y; blk[6] = b.z; blk[7] = b.w;
        blk[8] = ld_stream<HINT>(group + 256 + lane, pol);
    } else {
#pragma unroll
        for (int c = 0; c < S * S; c++) blk[c] = ld_stream<HINT>(group + sell_off<S, T>(c, (int)lane), pol);
    }
}

// Columns and blocks of slots j0 .. j0+U-1 of the lane's row (those < len).
template <int S, int U, typename T, int HINT = kMatrixHint>
__device__ __forceinline__ void load_sell_group(const SellView<T> &A, uint64_t g0, uint32_t j0, uint32_t len,
                                                uint32_t lane, uint32_t (&c)[U], T (&blk)[U][S * S],
                                                uint64_t pol = 0)
{
#pragma unroll
    for (int u = 0; u < U; u++) {
        if (j0 + u < len) {   // uniform over the warp
            const uint64_t gs = g0 + (uint64_t)(j0 + u) * 32;
            c[u] = ld_stream<HINT>(A.col + gs + lane, pol);
            load_sell_block<S, T, HINT>(A.val + gs * (S * S), lane, blk[u], pol);
        }
    }
}

// Kernel A on the SELL copy: one warp per slice, one lane per block row; every
// load of blocks and columns is one contiguous run per warp.  Each CTA works on
// its own contiguous range of slices (A.cta_first, balanced by slots, so the x
// entries its warps gather are close together) and its warps take the range's
// slices one at a time from a shared counter (no warp idles while another still
// has several slices to go); the dot partial of each slice goes to its own slot
// and the CTA adds its slots in index order, so the result does not depend on
// which warp took which slice.  U slots are
// fetched per step; with PIPE the next step's columns and blocks are fetched
// before the current step's x entries are gathered, so the matrix stream is
// never idle while x is read.  Blocks of a row are visited in the order of the
// block-CSR row with the same FMA sequence as row_spmv with one lane per row,
// so q is bitwise that of k_spmv_pq<S,1,T>.
// MINB (2x2 FP32 blocks only) asks the compiler for MINB resident CTAs per SM.
template <int S, int U, bool PIPE, typename T, int HINT = kMatrixHint>
__device__ __forceinline__ void sell_pq_body(const SellView<T> &A, const T *__restrict__ x, T *__restrict__ y,
                                             double *part_pq, PcgCtl *fin, double *sh, int *flag, uint32_t *next_sl,
                                             Cta cta)
{
    constexpr uint32_t WPB = kVecThreads / 32;
    const uint32_t lane = threadIdx.x & 31;
    // the CTA's contiguous, slot-balanced range of slices; its warps take slices in turn
    const uint32_t s_beg = __ldg(A.cta_first + cta.id), s_end = __ldg(A.cta_first + cta.id + 1);
    if (threadIdx.x == 0) *next_sl = s_beg + WPB;
    __syncthreads();
    for (uint32_t sl = s_beg + (threadIdx.x >> 5); sl < s_end;) {
        const uint32_t row = __ldg(A.perm + (uint64_t)sl * 32 + lane);
        const uint64_t g0 = __ldg(A.slice_ptr + sl);
        const uint32_t len = (uint32_t)((__ldg(A.slice_ptr + sl + 1) - g0) >> 5);
        T acc[S];
#pragma unroll
        for (int r = 0; r < S; r++) acc[r] = T(0);
        uint32_t c[U];
        T blk[U][S * S];
        if constexpr (PIPE) load_sell_group<S, U, T, HINT>(A, g0, 0, len, lane, c, blk);
        for (uint32_t j0 = 0; j0 < len; j0 += U) {
            if constexpr (!PIPE) load_sell_group<S, U, T, HINT>(A, g0, j0, len, lane, c, blk);
            T xv[U][S];
#pragma unroll
            for (int u = 0; u < U; u++)
                if (j0 + u < len) load_x<S, T>(x, c[u], xv[u]);
            uint32_t cn[U];
            T bn[U][S * S];
            if constexpr (PIPE) load_sell_group<S, U, T, HINT>(A, g0, j0 + U, len, lane, cn, bn);
#pragma unroll
            for (int u = 0; u < U; u++) {
                if (j0 + u < len) {
#pragma unroll
                    for (int r = 0; r < S; r++)
#pragma unroll
                        for (int cc = 0; cc < S; cc++) acc[r] = fma(blk[u][r * S + cc], xv[u][cc], acc[r]);
                }
            }
            if constexpr (PIPE) {
#pragma unroll
                for (int u = 0; u < U; u++) {
                    c[u] = cn[u];
#pragma unroll
                    for (int q = 0; q < S * S; q++) blk[u][q] = bn[u][q];
                }
            }
        }
        // the slice's share of p.q, summed in a fixed order whichever warp took the
        // slice (in the vector precision: FP64 issue slots are scarce on this part)
        T dot = T(0);
        if (row < A.n_rows) {
#pragma unroll
            for (int r = 0; r < S; r++) {
                y[(uint64_t)row * S + r] = acc[r];
                dot = fma(acc[r], x[(uint64_t)row * S + r], dot);
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) dot += __shfl_xor_sync(0xffffffffu, dot, o);
        if (lane == 0) A.slice_dot[sl] = dot;
        uint32_t nx = 0;
        if (lane == 0) nx = atomicAdd(next_sl, 1u);
        sl = __shfl_sync(0xffffffffu, nx, 0);
    }
    __syncthreads();   // the CTA's slice partials are visible to all its threads
    T dot = T(0);
    for (uint32_t i = s_beg + threadIdx.x; i < s_end; i += kVecThreads) dot += A.slice_dot[i];
    finish_pq<T>(dot, part_pq, fin, sh, flag, cta);
}

template <int S, int U, bool PIPE, int MINB, typename T>
__global__ void __launch_bounds__(kVecThreads, (S == 2 && sizeof(T) == 4) ? MINB : 1)
    k_sell_pq(SellView<T> A, const T *__restrict__ x, T *__restrict__ y, double *part_pq, const int32_t *done,
              PcgCtl *fin)
{
    __shared__ double sh[33];
    __shared__ int flag;
    __shared__ uint32_t next_sl;
    pdl_wait();
    pdl_release();
    if (done && *done) return;
    sell_pq_body<S, U, PIPE, T>(A, x, y, part_pq, fin, sh, &flag, &next_sl, grid_cta());
}

// Kernel A with the direction update folded in (used with two direction
// buffers): p_new = z + beta p_old is formed for every x entry the SpMV gathers
// and stored for the warp's own rows, q = A p_new, partial p_new.q; last CTA:
// pq and alpha.  p_old / p_new are chosen by ctl->pcur (flipped by k_update),
// so a graph of iterations needs no copies.  Same scheduling, FMA order and
// fixed-order dot as k_sell_pq; p_new equals k_direction's fma(beta, p, z).
template <int S, typename T, int HINT = kMatrixHint>
__global__ void __launch_bounds__(kVecThreads) k_sell_dir(SellView<T> A, PcgVecs<T> v, double *part_pq, PcgCtl *ctl,
                                                          int fin)
{
    __shared__ double sh[33];
    __shared__ int flag;
    __shared__ uint32_t next_sl;
    if (A.prefetch_bytes && threadIdx.x == 0) {
        // the matrix does not change during a solve: start streaming the head of
        // this CTA's contiguous slot range into L2 while the predecessor finishes
        const uint32_t sb = __ldg(A.cta_first + blockIdx.x), se = __ldg(A.cta_first + blockIdx.x + 1);
        const uint64_t g0 = __ldg(A.slice_ptr + sb), g1 = __ldg(A.slice_ptr + se);
        // g0 is a multiple of 32 slots, so both starts are 128-byte aligned; sizes are whole 16-byte units
        const uint64_t vfull = (g1 - g0) * (S * S * sizeof(T)), cfull = (g1 - g0) * 4;
        const uint64_t vcap = A.prefetch_bytes, ccap = A.prefetch_bytes / (S * S);
        const uint64_t vb = (vfull < vcap ? vfull : vcap) & ~uint64_t(15);
        const uint64_t cbytes = (cfull < ccap ? cfull : ccap) & ~uint64_t(15);
        if (vb) asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(A.val + g0 * (S * S)), "r"((uint32_t)vb) : "memory");
        if (cbytes) asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(A.col + g0), "r"((uint32_t)cbytes) : "memory");
    }
    pdl_wait();
    pdl_release();
    if (ctl->done) return;
    constexpr int U = kSpmvUnroll;
    constexpr uint32_t WPB = kVecThreads / 32;
    const uint32_t lane = threadIdx.x & 31;
    const T bt = (T)ctl->beta;
    const bool second = ctl->pcur != 0;
    const T *__restrict__ pold = second ? v.p2 : v.p;
    T *__restrict__ pnew = second ? v.p : v.p2;
    const T *__restrict__ z = v.z;
    T *__restrict__ q = v.q;
    const uint32_t s_beg = __ldg(A.cta_first + blockIdx.x), s_end = __ldg(A.cta_first + blockIdx.x + 1);
    const uint64_t pol = stream_policy<HINT>();
    if (threadIdx.x == 0) next_sl = s_beg + WPB;
    __syncthreads();
    for (uint32_t sl = s_beg + (threadIdx.x >> 5); sl < s_end;) {
        const uint32_t row = __ldg(A.perm + (uint64_t)sl * 32 + lane);
        const uint64_t g0 = __ldg(A.slice_ptr + sl);
        const uint32_t len = (uint32_t)((__ldg(A.slice_ptr + sl + 1) - g0) >> 5);
        T acc[S];
#pragma unroll
        for (int r = 0; r < S; r++) acc[r] = T(0);
        uint32_t c[U];
        T blk[U][S * S];
        for (uint32_t j0 = 0; j0 < len; j0 += U) {
            load_sell_group<S, U, T, HINT>(A, g0, j0, len, lane, c, blk, pol);
            T zv[U][S], pv[U][S];
#pragma unroll
            for (int u = 0; u < U; u++) {
                if (j0 + u < len) {
                    load_x<S, T>(z, c[u], zv[u]);
                    load_x<S, T>(pold, c[u], pv[u]);
                }
            }
#pragma unroll
            for (int u = 0; u < U; u++) {
                if (j0 + u < len) {
#pragma unroll
                    for (int r = 0; r < S; r++)
#pragma unroll
                        for (int cc = 0; cc < S; cc++)
                            acc[r] = fma(blk[u][r * S + cc], fma(bt, pv[u][cc], zv[u][cc]), acc[r]);
                }
            }
        }
        T dot = T(0);
        if (row < A.n_rows) {
#pragma unroll
            for (int r = 0; r < S; r++) {
                const uint64_t i = (uint64_t)row * S + r;
                const T pn = fma(bt, pold[i], z[i]);
                pnew[i] = pn;
                q[i] = acc[r];
                dot = fma(acc[r], pn, dot);
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) dot += __shfl_xor_sync(0xffffffffu, dot, o);
        if (lane == 0) A.slice_dot[sl] = dot;
        uint32_t nx = 0;
        if (lane == 0) nx = atomicAdd(&next_sl, 1u);
        sl = __shfl_sync(0xffffffffu, nx, 0);
    }
    __syncthreads();
    T dot = T(0);
    for (uint32_t i = s_beg + threadIdx.x; i < s_end; i += kVecThreads) dot += A.slice_dot[i];
    finish_pq<T>(dot, part_pq, fin ? ctl : nullptr, sh, &flag, grid_cta());
}

// k_sell_dir for a group of CTAs given explicitly (one slot's CTAs in a batched
// launch; plain matrix loads: a batch's small matrices are re-read every
// iteration from L2, and evict-first lines there raised the serving p99 from
// 0.28 s to 0.45 s).  The single-solve kernel below is kept as its own copy: with the
// group position and the views held as values the compiler keeps fewer loads in
// flight at the kernel's 64-register budget (49 us instead of 33 us on the
// 1.2 M-DOF P2 problem).
template <int S, typename T, bool CG = false>
__device__ __forceinline__ void sell_dir_body(const SellView<T> &A, const PcgVecs<T> &v, double *part_pq, PcgCtl *ctl,
                                              bool fin, Cta cta)
{
    __shared__ double sh[33];
    __shared__ int flag;
    __shared__ uint32_t next_sl;
    constexpr int U = kSpmvUnroll;
    constexpr uint32_t WPB = kVecThreads / 32;
    const uint32_t lane = threadIdx.x & 31;
    const T bt = (T)ctl_ld<CG>(&ctl->beta);
    const bool second = ctl_ld<CG>(&ctl->pcur) != 0;
    const T *__restrict__ pold = second ? v.p2 : v.p;
    T *__restrict__ pnew = second ? v.p : v.p2;
    const T *__restrict__ z = v.z;
    T *__restrict__ q = v.q;
    const uint32_t s_beg = __ldg(A.cta_first + cta.id), s_end = __ldg(A.cta_first + cta.id + 1);
    if (threadIdx.x == 0) next_sl = s_beg + WPB;
    __syncthreads();
    for (uint32_t sl = s_beg + (threadIdx.x >> 5); sl < s_end;) {
        const uint32_t row = __ldg(A.perm + (uint64_t)sl * 32 + lane);
        const uint64_t g0 = __ldg(A.slice_ptr + sl);
        const uint32_t len = (uint32_t)((__ldg(A.slice_ptr + sl + 1) - g0) >> 5);
        T acc[S];
#pragma unroll
        for (int r = 0; r < S; r++) acc[r] = T(0);
        uint32_t c[U];
        T blk[U][S * S];
        for (uint32_t j0 = 0; j0 < len; j0 += U) {
            load_sell_group<S, U, T, 0>(A, g0, j0, len, lane, c, blk);
            T zv[U][S], pv[U][S];
#pragma unroll
            for (int u = 0; u < U; u++) {
                if (j0 + u < len) {
                    if constexpr (CG) {
                        load_x_cg<S, T>(z, c[u], zv[u]);
                        load_x_cg<S, T>(pold, c[u], pv[u]);
                    } else {
                        load_x<S, T>(z, c[u], zv[u]);
                        load_x<S, T>(pold, c[u], pv[u]);
                    }
                }
            }
#pragma unroll
            for (int u = 0; u < U; u++) {
                if (j0 + u < len) {
#pragma unroll
                    for (int r = 0; r < S; r++)
#pragma unroll
                        for (int cc = 0; cc < S; cc++)
                            acc[r] = fma(blk[u][r * S + cc], fma(bt, pv[u][cc], zv[u][cc]), acc[r]);
                }
            }
        }
        T dot = T(0);
        if (row < A.n_rows) {
#pragma unroll
            for (int r = 0; r < S; r++) {
                const uint64_t i = (uint64_t)row * S + r;
                const T pn = CG ? fma(bt, __ldcg(pold + i), __ldcg(z + i)) : fma(bt, pold[i], z[i]);
                pnew[i] = pn;
                q[i] = acc[r];
                dot = fma(acc[r], pn, dot);
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) dot += __shfl_xor_sync(0xffffffffu, dot, o);
        if (lane == 0) A.slice_dot[sl] = dot;
        uint32_t nx = 0;
        if (lane == 0) nx = atomicAdd(&next_sl, 1u);
        sl = __shfl_sync(0xffffffffu, nx, 0);
    }
    __syncthreads();
    T dot = T(0);
    for (uint32_t i = s_beg + threadIdx.x; i < s_end; i += kVecThreads) dot += A.slice_dot[i];
    finish_pq<T, CG>(dot, part_pq, fin ? ctl : nullptr, sh, &flag, cta);
}


// Asynchronous 16-byte global -> shared copies (completion tracked per thread
// in commit groups; cp.async.wait_group is a hardware wait on those copies).
__device__ __forceinline__ void cp_async16(void *smem, const void *gmem)
{
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait()
{
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// One s x s block of the lane's row from a 32-slot SELL group held in shared memory.
template <int S, typename T>
__device__ __forceinline__ void load_sell_block_sm(const T *group, uint32_t lane, T blk[S * S])
{
    constexpr int V = kSellVec<S, T>;
    if constexpr (S == 2 && V == 4) {
        const float4 a = reinterpret_cast<const float4 *>(group)[lane];
        blk[0] = a.x; blk[1] = a.y; blk[2] = a.z; blk[3] = a.w;
    } else if constexpr (S == 2 && V == 2) {
        const double2 a = reinterpret_cast<const double2 *>(group)[lane];
        const double2 b = reinterpret_cast<const double2 *>(group + 64)[lane];
        blk[0] = a.x; blk[1] = a.y; blk[2] = b.x; blk[3] = b.y;
    } else {
#pragma unroll
        for (int c = 0; c < S * S; c++) blk[c] = group[sell_off<S, T>(c, (int)lane)];
    }
}

// Bytes of one pipeline stage of k_sell_pq_cp: values and columns of U slot groups.
template <int S, int U, typename T>
__host__ __device__ constexpr uint32_t sell_stage_bytes()
{
    return (uint32_t)(U * 32 * S * S * sizeof(T) + U * 32 * 4);
}

// Kernel A on the SELL copy with the matrix streamed through shared memory:
// each warp walks its slices in steps of U slot groups and keeps NST - 1 steps
// of values and columns in flight as cp.async copies (no registers held), so
// the matrix stream continues while the current step's x entries are gathered.
// Same per-row FMA order as k_sell_pq, so q is bitwise the same.  Dynamic
// shared memory: kVecThreads / 32 * NST * sell_stage_bytes<S, U, T>() bytes.
template <int S, int U, int NST, typename T>
__global__ void __launch_bounds__(kVecThreads) k_sell_pq_cp(SellView<T> A, const T *__restrict__ x,
                                                            T *__restrict__ y, double *part_pq, const int32_t *done,
                                                            PcgCtl *fin)
{
    extern __shared__ __align__(16) unsigned char sm_stage[];
    __shared__ double sh[33];
    __shared__ int flag;
    pdl_wait();
    pdl_release();
    if (done && *done) return;
    constexpr uint32_t WPB = kVecThreads / 32;
    constexpr uint32_t VB = (uint32_t)(U * 32 * S * S * sizeof(T));
    constexpr uint32_t SB = sell_stage_bytes<S, U, T>();
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned char *wbase = sm_stage + (size_t)warp * NST * SB;
    const uint32_t sl_step = gridDim.x * WPB;
    const uint32_t n_slices = A.n_slices;

    // issue side: next step whose copies have not been started
    uint32_t i_sl = blockIdx.x * WPB + warp, i_j = 0, i_len = 0;
    uint64_t i_g0 = 0;
    auto i_enter = [&]() {
        for (; i_sl < n_slices; i_sl += sl_step) {
            i_g0 = __ldg(A.slice_ptr + i_sl);
            i_len = (uint32_t)((__ldg(A.slice_ptr + i_sl + 1) - i_g0) >> 5);
            if (i_len) break;
        }
    };
    auto issue = [&](uint32_t stage) {
        if (i_sl < n_slices) {
            const uint32_t cnt = min((uint32_t)U, i_len - i_j);
            const uint64_t gs = i_g0 + (uint64_t)i_j * 32;
            unsigned char *dst = wbase + stage * SB;
            const unsigned char *gv = reinterpret_cast<const unsigned char *>(A.val + gs * (S * S));
            const uint32_t nv = cnt * (uint32_t)(32 * S * S * sizeof(T) / 16);
            for (uint32_t k = lane; k < nv; k += 32) cp_async16(dst + 16 * k, gv + 16 * k);
            const unsigned char *gc = reinterpret_cast<const unsigned char *>(A.col + gs);
            for (uint32_t k = lane; k < cnt * 8; k += 32) cp_async16(dst + VB + 16 * k, gc + 16 * k);
            i_j += U;
            if (i_j >= i_len) {
                i_j = 0;
                i_sl += sl_step;
                i_enter();
            }
        }
        cp_async_commit();   // one group per step, empty past the end, so the counts line up
    };
    i_enter();
#pragma unroll
    for (int k = 0; k < NST - 1; k++) issue(k);

    // consume side
    uint32_t c_sl = blockIdx.x * WPB + warp, c_j = 0, c_len = 0, row = 0;
    auto c_enter = [&]() {
        for (; c_sl < n_slices; c_sl += sl_step) {
            const uint64_t g0 = __ldg(A.slice_ptr + c_sl);
            c_len = (uint32_t)((__ldg(A.slice_ptr + c_sl + 1) - g0) >> 5);
            if (c_len) break;
        }
        if (c_sl < n_slices) row = __ldg(A.perm + (uint64_t)c_sl * 32 + lane);
    };
    c_enter();
    T dot = T(0);
    T acc[S];
#pragma unroll
    for (int r = 0; r < S; r++) acc[r] = T(0);
    uint32_t stage = 0;
    while (c_sl < n_slices) {   // uniform over the warp
        issue(stage == 0 ? NST - 1 : stage - 1);
        cp_async_wait<NST - 1>();
        __syncwarp();
        const unsigned char *src = wbase + stage * SB;
        const T *vals = reinterpret_cast<const T *>(src);
        const uint32_t *cols = reinterpret_cast<const uint32_t *>(src + VB);
        const uint32_t cnt = min((uint32_t)U, c_len - c_j);
        T xv[U][S];
#pragma unroll
        for (int u = 0; u < U; u++)
            if (u < cnt) load_x<S, T>(x, cols[u * 32 + lane], xv[u]);
#pragma unroll
        for (int u = 0; u < U; u++) {
            if (u < cnt) {
                T blk[S * S];
                load_sell_block_sm<S, T>(vals + u * 32 * S * S, lane, blk);
#pragma unroll
                for (int r = 0; r < S; r++)
#pragma unroll
                    for (int cc = 0; cc < S; cc++) acc[r] = fma(blk[r * S + cc], xv[u][cc], acc[r]);
            }
        }
        __syncwarp();   // the stage may be refilled from here on
        stage = stage + 1 == NST ? 0 : stage + 1;
        c_j += U;
        if (c_j >= c_len) {
            if (row < A.n_rows) {
#pragma unroll
                for (int r = 0; r < S; r++) {
                    y[(uint64_t)row * S + r] = acc[r];
                    dot = fma(acc[r], x[(uint64_t)row * S + r], dot);
                }
            }
#pragma unroll
            for (int r = 0; r < S; r++) acc[r] = T(0);
            c_j = 0;
            c_sl += sl_step;
            c_enter();
        }
    }
    cp_async_wait<0>();
    finish_pq<T>(dot, part_pq, fin, sh, &flag, grid_cta());
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

// 16-byte packs of vector entries for the vector kernels.
template <typename T> struct Pack;
template <> struct Pack<float> { using type = float4; static constexpr int n = 4; };
template <> struct Pack<double> { using type = double2; static constexpr int n = 2; };

__device__ __forceinline__ bool aligned16(const void *p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

template <typename T>
__device__ __forceinline__ void ld_pack(const T *p, uint64_t i, T (&o)[Pack<T>::n])
{
    if constexpr (sizeof(T) == 4) {
        const float4 a = reinterpret_cast<const float4 *>(p)[i];
        o[0] = a.x; o[1] = a.y; o[2] = a.z; o[3] = a.w;
    } else {
        const double2 a = reinterpret_cast<const double2 *>(p)[i];
        o[0] = a.x; o[1] = a.y;
    }
}

template <typename T>
__device__ __forceinline__ void ldg_pack(const T *__restrict__ p, uint64_t i, T (&o)[Pack<T>::n])
{
    if constexpr (sizeof(T) == 4) {
        const float4 a = __ldg(reinterpret_cast<const float4 *>(p) + i);
        o[0] = a.x; o[1] = a.y; o[2] = a.z; o[3] = a.w;
    } else {
        const double2 a = __ldg(reinterpret_cast<const double2 *>(p) + i);
        o[0] = a.x; o[1] = a.y;
    }
}

// A pack another CTA may have written during a running persistent kernel
// (CG: through L2 only), else through the read-only path.
template <typename T, bool CG>
__device__ __forceinline__ void ldq_pack(const T *p, uint64_t i, T (&o)[Pack<T>::n])
{
    if constexpr (!CG) {
        ldg_pack<T>(p, i, o);
    } else if constexpr (sizeof(T) == 4) {
        const float4 a = __ldcg(reinterpret_cast<const float4 *>(p) + i);
        o[0] = a.x; o[1] = a.y; o[2] = a.z; o[3] = a.w;
    } else {
        const double2 a = __ldcg(reinterpret_cast<const double2 *>(p) + i);
        o[0] = a.x; o[1] = a.y;
    }
}

template <typename T>
__device__ __forceinline__ void st_pack(T *p, uint64_t i, const T (&o)[Pack<T>::n])
{
    if constexpr (sizeof(T) == 4) reinterpret_cast<float4 *>(p)[i] = make_float4(o[0], o[1], o[2], o[3]);
    else reinterpret_cast<double2 *>(p)[i] = make_double2(o[0], o[1]);
}

// Runs f(i) for every entry i < n of this thread's share: packs of
// Pack<T>::n entries (fpack(k) for pack k) when every vector is 16-byte
// aligned, single entries otherwise and for the tail.
template <typename T, typename FP, typename FS>
__device__ __forceinline__ void for_entries(uint64_t n, bool aligned, Cta cta, FP &&fpack, FS &&fone)
{
    constexpr int W = Pack<T>::n;
    const uint64_t tid = (uint64_t)cta.id * kVecThreads + threadIdx.x;
    const uint64_t stride = (uint64_t)cta.n * kVecThreads;
    uint64_t first = 0;
    if (aligned) {
        const uint64_t npk = n / W;
        for (uint64_t k = tid; k < npk; k += stride) fpack(k);
        first = npk * W;
    }
    for (uint64_t i = first + tid; i < n; i += stride) fone(i);
}

// Kernel B: x += alpha p; r -= alpha q; z = D^-1 r; partials r.z, r.r.
// Last CTA: totals, iteration count, stop test, beta = rz_new / rz.  Each
// thread handles two 16-byte packs per step with all ten loads issued before
// any arithmetic (one memory round trip per step).
template <typename T, bool CG = false>
__device__ __forceinline__ void update_body(const PcgVecs<T> &v, uint64_t n, const PcgParts &parts, PcgCtl *ctl,
                                            double *sh, int *flag, Cta cta)
{
    constexpr int W = Pack<T>::n;
    const T a = (T)ctl_ld<CG>(&ctl->alpha);
    T *__restrict__ x = v.x;
    T *__restrict__ r = v.r;
    T *__restrict__ z = v.z;
    // with two direction buffers the SpMV just wrote this iteration's p into the other one
    const T *__restrict__ p = v.p2 ? (ctl_ld<CG>(&ctl->pcur) ? v.p : v.p2) : v.p;
    const T *__restrict__ q = v.q;
    const T *__restrict__ d = v.dinv;
    T drz = T(0), drr = T(0);   // per-thread partials in the vector precision, CTA sums in FP64
    const bool al = aligned16(x) && aligned16(r) && aligned16(z) && aligned16(p) && aligned16(q) && aligned16(d);
    const uint64_t tid = (uint64_t)cta.id * kVecThreads + threadIdx.x;
    const uint64_t stride = (uint64_t)cta.n * kVecThreads;
    const uint64_t npk = al ? n / W : 0;
    for (uint64_t k = tid; k < npk; k += 2 * stride) {
        const uint64_t k2 = k + stride;
        const bool two = k2 < npk;   // the second pack of the step exists
        T rv[2][W], qv[2][W], xv[2][W], pv[2][W], dv[2][W];
        ld_pack<T>(r, k, rv[0]);
        ldq_pack<T, CG>(q, k, qv[0]);
        ld_pack<T>(x, k, xv[0]);
        ldq_pack<T, CG>(p, k, pv[0]);
        ldg_pack<T>(d, k, dv[0]);
        if (two) {
            ld_pack<T>(r, k2, rv[1]);
            ldq_pack<T, CG>(q, k2, qv[1]);
            ld_pack<T>(x, k2, xv[1]);
            ldq_pack<T, CG>(p, k2, pv[1]);
            ldg_pack<T>(d, k2, dv[1]);
        }
#pragma unroll
        for (int h = 0; h < 2; h++) {
            if (h == 1 && !two) break;
            T zv[W];
#pragma unroll
            for (int c = 0; c < W; c++) {
                rv[h][c] = rv[h][c] - a * qv[h][c];
                xv[h][c] = fma(a, pv[h][c], xv[h][c]);
                zv[c] = rv[h][c] * dv[h][c];
                drz = fma(rv[h][c], zv[c], drz);
                drr = fma(rv[h][c], rv[h][c], drr);
            }
            const uint64_t kk = h ? k2 : k;
            st_pack<T>(r, kk, rv[h]);
            st_pack<T>(x, kk, xv[h]);
            st_pack<T>(z, kk, zv);
        }
    }
    for (uint64_t i = npk * W + tid; i < n; i += stride) {   // tail, or everything when not aligned
        const T qi = CG ? __ldcg(q + i) : q[i];
        const T pi = CG ? __ldcg(p + i) : p[i];
        const T ri = r[i] - a * qi;
        x[i] = fma(a, pi, x[i]);
        r[i] = ri;
        const T zi = ri * d[i];
        z[i] = zi;
        drz = fma(ri, zi, drz);
        drr = fma(ri, ri, drr);
    }
    double brz, brr;
    block_sum2_v<T>(drz, drr, sh, brz, brr);
    if (threadIdx.x == 0) {
        parts.rz[cta.id] = brz;
        parts.rr[cta.id] = brr;
    }
    if (!last_cta(&ctl->ticket, flag, cta.n)) return;
    double rz_new, rr;
    ordered_sum2(parts.rz, parts.rr, cta.n, sh, rz_new, rr);
    if (threadIdx.x == 0) {
        const int64_t it = ctl_ld<CG>(&ctl->iterations) + 1;
        const double rz_old = ctl_ld<CG>(&ctl->rz);
        ctl->iterations = it;
        ctl->rr = rr;
        ctl->rz_prev = rz_old;
        const bool stop = rr <= ctl_ld<CG>(&ctl->tol2) || it >= ctl_ld<CG>(&ctl->maxit) || !(rr == rr);
        if (stop) {
            ctl->done = 1;
        } else {
            ctl->beta = rz_old != 0.0 ? rz_new / rz_old : 0.0;
        }
        ctl->rz = rz_new;
        if (v.p2) ctl->pcur = ctl_ld<CG>(&ctl->pcur) ^ 1;   // this iteration's p is now the latest
        ctl->ticket = 0;
    }
}

// Kernel B of a single solve: update_body's work with its fixed latencies cut.
// The loads of the thread's first step that the SpMV does not produce (x and r,
// last written by the previous update, which finished before the SpMV could
// start; D^-1) are issued before the wait on the SpMV; done, alpha and the
// direction buffer are read in one round; the last CTA fetches the control
// fields together with the partials.  FP32 asks for four resident CTAs per SM
// (FP64 three), so that on the grid of resident CTAs one FP32 step covers
// 1.2 M entries.
template <typename T>
__global__ void __launch_bounds__(kVecThreads, sizeof(T) == 4 ? 4 : 3)
    k_update(PcgVecs<T> v, uint64_t n, PcgParts parts, PcgCtl *ctl)
{
    __shared__ double sh[2 * (kVecThreads >> 5)];
    __shared__ int flag;
    constexpr int W = Pack<T>::n;
    T *__restrict__ x = v.x;
    T *__restrict__ r = v.r;
    T *__restrict__ z = v.z;
    const T *__restrict__ q = v.q;
    const T *__restrict__ d = v.dinv;
    const bool al = aligned16(x) && aligned16(r) && aligned16(z) && aligned16(v.p) && aligned16(q) &&
                    aligned16(d) && (!v.p2 || aligned16(v.p2));
    const uint64_t tid = (uint64_t)blockIdx.x * kVecThreads + threadIdx.x;
    const uint64_t stride = (uint64_t)gridDim.x * kVecThreads;
    const uint64_t npk = al ? n / W : 0;
    T rv[2][W], xv[2][W], dv[2][W];
    if (tid < npk) {
        ld_pack<T>(r, tid, rv[0]);
        ld_pack<T>(x, tid, xv[0]);
        ldg_pack<T>(d, tid, dv[0]);
        if (tid + stride < npk) {
            ld_pack<T>(r, tid + stride, rv[1]);
            ld_pack<T>(x, tid + stride, xv[1]);
            ldg_pack<T>(d, tid + stride, dv[1]);
        }
    }
    // done and pcur are written only by the previous update's last CTA (finished,
    // like x and r); alpha comes from the SpMV this kernel waits on
    const int32_t done = ctl->done;
    const int32_t pcur = ctl->pcur;
    pdl_wait();
    pdl_release();
    if (done) return;
    const T a = (T)ctl->alpha;
    // with two direction buffers the SpMV just wrote this iteration's p into the other one
    const T *__restrict__ p = v.p2 ? (pcur ? v.p : v.p2) : v.p;
    T drz = T(0), drr = T(0);   // per-thread partials in the vector precision, CTA sums in FP64
    for (uint64_t k = tid; k < npk; k += 2 * stride) {
        const uint64_t k2 = k + stride;
        const bool two = k2 < npk;   // the second pack of the step exists
        T qv[2][W], pv[2][W];
        if (k != tid) {
            ld_pack<T>(r, k, rv[0]);
            ld_pack<T>(x, k, xv[0]);
            ldg_pack<T>(d, k, dv[0]);
            if (two) {
                ld_pack<T>(r, k2, rv[1]);
                ld_pack<T>(x, k2, xv[1]);
                ldg_pack<T>(d, k2, dv[1]);
            }
        }
        ld_pack<T>(q, k, qv[0]);
        ld_pack<T>(p, k, pv[0]);
        if (two) {
            ld_pack<T>(q, k2, qv[1]);
            ld_pack<T>(p, k2, pv[1]);
        }
#pragma unroll
        for (int h = 0; h < 2; h++) {
            if (h == 1 && !two) break;
            T zv[W];
#pragma unroll
            for (int c = 0; c < W; c++) {
                rv[h][c] = rv[h][c] - a * qv[h][c];
                xv[h][c] = fma(a, pv[h][c], xv[h][c]);
                zv[c] = rv[h][c] * dv[h][c];
                drz = fma(rv[h][c], zv[c], drz);
                drr = fma(rv[h][c], rv[h][c], drr);
            }
            const uint64_t kk = h ? k2 : k;
            st_pack<T>(r, kk, rv[h]);
            st_pack<T>(x, kk, xv[h]);
            st_pack<T>(z, kk, zv);
        }
    }
    for (uint64_t i = npk * W + tid; i < n; i += stride) {   // tail, or everything when not aligned
        const T ri = r[i] - a * q[i];
        x[i] = fma(a, p[i], x[i]);
        r[i] = ri;
        const T zi = ri * d[i];
        z[i] = zi;
        drz = fma(ri, zi, drz);
        drr = fma(ri, ri, drr);
    }
    double brz, brr;
    block_sum2_v<T>(drz, drr, sh, brz, brr);
    if (threadIdx.x == 0) {
        parts.rz[blockIdx.x] = brz;
        parts.rr[blockIdx.x] = brr;
    }
    if (!last_cta(&ctl->ticket, &flag, gridDim.x)) return;
    // the totals (same order as ordered_sum2) and the control fields in one round
    int64_t it = 0, maxit = 0;
    double rz_old = 0.0, tol2 = 0.0;
    if (threadIdx.x == 0) {
        it = ctl->iterations + 1;
        maxit = ctl->maxit;
        rz_old = ctl->rz;
        tol2 = ctl->tol2;
    }
    double sa = 0.0, sb = 0.0;
    for (uint32_t i = threadIdx.x; i < gridDim.x; i += kVecThreads) {
        sa += __ldcg(parts.rz + i);
        sb += __ldcg(parts.rr + i);
    }
    double rz_new, rr;
    block_sum2_v<double>(sa, sb, sh, rz_new, rr);
    if (threadIdx.x == 0) {
        ctl->iterations = it;
        ctl->rr = rr;
        ctl->rz_prev = rz_old;
        const bool stop = rr <= tol2 || it >= maxit || !(rr == rr);
        if (stop) {
            ctl->done = 1;
        } else {
            ctl->beta = rz_old != 0.0 ? rz_new / rz_old : 0.0;
        }
        ctl->rz = rz_new;
        if (v.p2) ctl->pcur = pcur ^ 1;   // this iteration's p is now the latest
        ctl->ticket = 0;
    }
}

// Kernel C: p = z + beta p, two packs per thread per step.
template <typename T>
__device__ __forceinline__ void direction_body(const PcgVecs<T> &v, uint64_t n, const PcgCtl *ctl, Cta cta)
{
    constexpr int W = Pack<T>::n;
    const T bt = (T)ctl->beta;
    T *__restrict__ p = v.p;
    const T *__restrict__ z = v.z;
    const uint64_t tid = (uint64_t)cta.id * kVecThreads + threadIdx.x;
    const uint64_t stride = (uint64_t)cta.n * kVecThreads;
    const uint64_t npk = aligned16(p) && aligned16(z) ? n / W : 0;
    for (uint64_t k = tid; k < npk; k += 2 * stride) {
        const uint64_t k2 = k + stride;
        const bool two = k2 < npk;
        T pv[2][W], zv[2][W];
        ld_pack<T>(p, k, pv[0]);
        ldg_pack<T>(z, k, zv[0]);
        if (two) {
            ld_pack<T>(p, k2, pv[1]);
            ldg_pack<T>(z, k2, zv[1]);
        }
#pragma unroll
        for (int c = 0; c < W; c++) pv[0][c] = fma(bt, pv[0][c], zv[0][c]);
        st_pack<T>(p, k, pv[0]);
        if (two) {
#pragma unroll
            for (int c = 0; c < W; c++) pv[1][c] = fma(bt, pv[1][c], zv[1][c]);
            st_pack<T>(p, k2, pv[1]);
        }
    }
    for (uint64_t i = npk * W + tid; i < n; i += stride) p[i] = fma(bt, p[i], z[i]);
}

template <typename T>
__global__ void __launch_bounds__(kVecThreads) k_direction(PcgVecs<T> v, uint64_t n, const PcgCtl *ctl)
{
    pdl_wait();
    pdl_release();
    if (ctl->done) return;
    direction_body<T>(v, n, ctl, grid_cta());
}

// z = D^-1 r (and p = z when `set_p`); partials r.z, r.r.  Shared by the start
// and the resume of a run.
template <typename T, bool SET_P>
__device__ __forceinline__ void precond_parts(const PcgVecs<T> &v, uint64_t n, Cta cta, T &drz, T &drr)
{
    constexpr int W = Pack<T>::n;
    const T *__restrict__ r = v.r;
    const T *__restrict__ d = v.dinv;
    T *__restrict__ z = v.z;
    T *__restrict__ p = v.p;
    for_entries<T>(
        n, aligned16(r) && aligned16(d) && aligned16(z) && aligned16(p), cta,
        [&](uint64_t k) {
            T rv[W], dv[W], zv[W];
            ldg_pack<T>(r, k, rv);
            ldg_pack<T>(d, k, dv);
#pragma unroll
            for (int c = 0; c < W; c++) {
                zv[c] = rv[c] * dv[c];
                drz = fma(rv[c], zv[c], drz);
                drr = fma(rv[c], rv[c], drr);
            }
            st_pack<T>(z, k, zv);
            if (SET_P) st_pack<T>(p, k, zv);
        },
        [&](uint64_t i) {
            const T ri = r[i];
            const T zi = ri * d[i];
            z[i] = zi;
            if (SET_P) p[i] = zi;
            drz = fma(ri, zi, drz);
            drr = fma(ri, ri, drr);
        });
}

// Start of a PCG run from the residual r (already holding b - A x):
// z = D^-1 r, p = z; last CTA: rz and rr into the control block.
template <typename T>
__device__ __forceinline__ void start_body(const PcgVecs<T> &v, uint64_t n, const PcgParts &parts, PcgCtl *ctl,
                                           double *sh, int *flag, Cta cta)
{
    T drz = T(0), drr = T(0);
    precond_parts<T, true>(v, n, cta, drz, drr);
    double brz, brr;
    block_sum2_v<T>(drz, drr, sh, brz, brr);
    if (threadIdx.x == 0) {
        parts.rz[cta.id] = brz;
        parts.rr[cta.id] = brr;
    }
    if (!last_cta(&ctl->ticket, flag, cta.n)) return;
    double rz, rr;
    ordered_sum2(parts.rz, parts.rr, cta.n, sh, rz, rr);
    if (threadIdx.x == 0) {
        ctl->rz = rz;
        ctl->rr = rr;
        ctl->ticket = 0;
    }
}

template <typename T>
__global__ void __launch_bounds__(kVecThreads) k_pcg_start(PcgVecs<T> v, uint64_t n, PcgParts parts, PcgCtl *ctl)
{
    __shared__ double sh[33];
    __shared__ int flag;
    start_body<T>(v, n, parts, ctl, sh, &flag, grid_cta());
}

// Resume of a stopped PCG run after its residual r was replaced by the true
// residual, rescaled by `ratio` = old scale / new scale relative to the run's
// vectors: z = D^-1 r, partials r.z, r.r; last CTA: beta = ratio * rz / rz_prev
// so that the following k_direction keeps the previous search direction
// (a reliable update), fresh tol2 / maxit, iterations and done cleared.
template <typename T>
__device__ __forceinline__ void resume_body(const PcgVecs<T> &v, uint64_t n, const PcgParts &parts, PcgCtl *ctl,
                                            double ratio, double tol2, int64_t maxit, double *sh, int *flag, Cta cta)
{
    T drz = T(0), drr = T(0);
    precond_parts<T, false>(v, n, cta, drz, drr);
    double brz, brr;
    block_sum2_v<T>(drz, drr, sh, brz, brr);
    if (threadIdx.x == 0) {
        parts.rz[cta.id] = brz;
        parts.rr[cta.id] = brr;
    }
    if (!last_cta(&ctl->ticket, flag, cta.n)) return;
    double rz, rr;
    ordered_sum2(parts.rz, parts.rr, cta.n, sh, rz, rr);
    if (threadIdx.x == 0) {
        ctl->beta = ctl->rz_prev != 0.0 ? ratio * rz / ctl->rz_prev : 0.0;
        ctl->rz = rz;
        ctl->rr = rr;
        ctl->tol2 = tol2;
        ctl->maxit = maxit;
        ctl->iterations = 0;
        ctl->done = 0;
        ctl->ticket = 0;
    }
}

template <typename T>
__global__ void __launch_bounds__(kVecThreads) k_pcg_resume(PcgVecs<T> v, uint64_t n, PcgParts parts, PcgCtl *ctl,
                                                            double ratio, double tol2, int64_t maxit)
{
    __shared__ double sh[33];
    __shared__ int flag;
    resume_body<T>(v, n, parts, ctl, ratio, tol2, maxit, sh, &flag, grid_cta());
}


// ------------------------------------------------------------------ single-reduction PCG
// Chronopoulos-Gear PCG (A. T. Chronopoulos and C. W. Gear, "s-step iterative
// methods for symmetric linear systems", J. Comput. Appl. Math. 25 (1989)
// 153-168; the s = 1 form): with u = D^-1 r and w = A u,
//   p_i = u_i + beta_i p_(i-1),  s_i = w_i + beta_i s_(i-1)   (s_i = A p_i)
//   x += alpha_i p_i,  r_(i+1) = r_i - alpha_i s_i,  u_(i+1) = D^-1 r_(i+1),  w_(i+1) = A u_(i+1)
//   gamma = r.u, delta = w.u (both of iteration i+1, one reduction),
//   beta_(i+1) = gamma_(i+1) / gamma_i,  alpha_(i+1) = gamma_(i+1) / (delta_(i+1) - beta_(i+1) gamma_(i+1) / alpha_i).
// One kernel per iteration: every warp updates p, s, x, r of its own rows and
// computes w = A u_(i+1) with u_(i+1) of the gathered columns formed from r_i,
// w_i, s_(i-1) and D^-1 by the same expression as for its own rows, so the
// gathered and the stored values agree bit for bit.  r, w and s have two
// buffers each (read one, write the other; ctl->pcur selects), p and x are
// touched by their own rows only.  Dots: per-slice partials in the vector
// precision, summed in slice order per CTA, then in CTA order by the last CTA.
template <typename T>
struct CgcgVecs {
    const T *dinv;
    T *x, *p;
    T *r[2], *w[2], *s[2];
    T *slice3;   // [3 * n_slices]: gamma, delta, r.r partials of each slice
};

// u_(i+1) of one entry from r_i, w_i, s_(i-1), D^-1 (also returns r_(i+1)).
template <typename T>
__device__ __forceinline__ T cgcg_next_u(T r, T w, T sp, T d, T al, T bt, T &rn)
{
    const T sn = fma(bt, sp, w);
    rn = fma(-al, sn, r);
    return d * rn;
}

// Sums of three values per thread over the CTA (warp levels in T, per-warp in
// FP64), valid in thread 0.
template <typename T>
__device__ __forceinline__ void block_sum3_v(T a, T b, T c, double *sh, double &ra, double &rb, double &rc)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_xor_sync(0xffffffffu, a, o);
        b += __shfl_xor_sync(0xffffffffu, b, o);
        c += __shfl_xor_sync(0xffffffffu, c, o);
    }
    constexpr int NW = kVecThreads >> 5;
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) {
        sh[w] = (double)a;
        sh[NW + w] = (double)b;
        sh[2 * NW + w] = (double)c;
    }
    __syncthreads();
    double x = 0.0, y = 0.0, z = 0.0;
    if (w == 0) {
        x = l < NW ? sh[l] : 0.0;
        y = l < NW ? sh[NW + l] : 0.0;
        z = l < NW ? sh[2 * NW + l] : 0.0;
#pragma unroll
        for (int o = NW >> 1; o > 0; o >>= 1) {
            x += __shfl_xor_sync(0xffffffffu, x, o);
            y += __shfl_xor_sync(0xffffffffu, y, o);
            z += __shfl_xor_sync(0xffffffffu, z, o);
        }
    }
    __syncthreads();
    ra = x;
    rb = y;
    rc = z;
}

// One Chronopoulos-Gear iteration (START = false), or the start of a run:
// w = A u for the residual in r[pcur] with p and s[pcur^1] multiplied by
// ctl->pq (the previous run's residual scale over the new one; 0 = fresh start,
// which zeroes them), no update of x or r; its last CTA sets alpha and beta from
// the kept gamma (rescaled by the host) and alpha for a resumed run, or
// alpha = gamma / delta for a fresh one.
template <int S, typename T, int HINT = kMatrixHint, bool START = false>
__global__ void __launch_bounds__(kVecThreads, 2) k_sell_cgcg(SellView<T> A, CgcgVecs<T> v, double *part, PcgCtl *ctl)
{
    constexpr bool start = START;
    __shared__ double sh[3 * (kVecThreads >> 5)];
    __shared__ int flag;
    __shared__ uint32_t next_sl;
    if (A.prefetch_bytes && threadIdx.x == 0) {
        // the matrix does not change during a solve: stream the head of this CTA's
        // slot range into L2 while the predecessor finishes (as k_sell_dir)
        const uint32_t sb = __ldg(A.cta_first + blockIdx.x), se = __ldg(A.cta_first + blockIdx.x + 1);
        const uint64_t g0 = __ldg(A.slice_ptr + sb), g1 = __ldg(A.slice_ptr + se);
        const uint64_t vfull = (g1 - g0) * (S * S * sizeof(T)), cfull = (g1 - g0) * 4;
        const uint64_t vcap = A.prefetch_bytes, ccap = A.prefetch_bytes / (S * S);
        const uint64_t vb = (vfull < vcap ? vfull : vcap) & ~uint64_t(15);
        const uint64_t cbytes = (cfull < ccap ? cfull : ccap) & ~uint64_t(15);
        if (vb) asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(A.val + g0 * (S * S)), "r"((uint32_t)vb) : "memory");
        if (cbytes) asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(A.col + g0), "r"((uint32_t)cbytes) : "memory");
    }
    pdl_wait();
    pdl_release();
    if (!start && ctl->done) return;
    constexpr int U = kSpmvUnroll;
    constexpr uint32_t WPB = kVecThreads / 32;
    const uint32_t lane = threadIdx.x & 31;
    const int cur = ctl->pcur;
    const T al = start ? T(0) : (T)ctl->alpha;
    const T bt = start ? T(0) : (T)ctl->beta;
    const double scale = start ? ctl->pq : 1.0;
    // buffers by parity, selected without indexing (no local copy of the parameter block)
    T *const r0 = cur ? v.r[1] : v.r[0], *const r1 = cur ? v.r[0] : v.r[1];
    T *const w0 = cur ? v.w[1] : v.w[0], *const w1 = cur ? v.w[0] : v.w[1];
    T *const s0 = cur ? v.s[1] : v.s[0], *const s1 = cur ? v.s[0] : v.s[1];
    const T *__restrict__ rc = r0;
    const T *__restrict__ wc = w0;
    T *__restrict__ sp = s1;
    const T *__restrict__ d = v.dinv;
    T *__restrict__ rn_out = r1;
    T *__restrict__ w_out = start ? w0 : w1;
    T *__restrict__ s_out = s0;
    const uint32_t s_beg = __ldg(A.cta_first + blockIdx.x), s_end = __ldg(A.cta_first + blockIdx.x + 1);
    const uint64_t pol = stream_policy<HINT>();
    if (threadIdx.x == 0) next_sl = s_beg + WPB;
    __syncthreads();
    for (uint32_t sl = s_beg + (threadIdx.x >> 5); sl < s_end;) {
        const uint32_t row = __ldg(A.perm + (uint64_t)sl * 32 + lane);
        const uint64_t g0 = __ldg(A.slice_ptr + sl);
        const uint32_t len = (uint32_t)((__ldg(A.slice_ptr + sl + 1) - g0) >> 5);
        T acc[S];
#pragma unroll
        for (int r = 0; r < S; r++) acc[r] = T(0);
        uint32_t c[U];
        T blk[U][S * S];
        for (uint32_t j0 = 0; j0 < len; j0 += U) {
            load_sell_group<S, U, T, HINT>(A, g0, j0, len, lane, c, blk, pol);
            T rv[U][S], wv[U][S], sv[U][S], dv[U][S];
#pragma unroll
            for (int u = 0; u < U; u++) {
                if (j0 + u < len) {
                    load_x<S, T>(rc, c[u], rv[u]);
                    load_x<S, T>(d, c[u], dv[u]);
                    if (!start) {
                        load_x<S, T>(wc, c[u], wv[u]);
                        load_x<S, T>(sp, c[u], sv[u]);
                    }
                }
            }
#pragma unroll
            for (int u = 0; u < U; u++) {
                if (j0 + u < len) {
#pragma unroll
                    for (int cc = 0; cc < S; cc++) {
                        T rn;
                        const T un = start ? dv[u][cc] * rv[u][cc]
                                           : cgcg_next_u<T>(rv[u][cc], wv[u][cc], sv[u][cc], dv[u][cc], al, bt, rn);
#pragma unroll
                        for (int r = 0; r < S; r++) acc[r] = fma(blk[u][r * S + cc], un, acc[r]);
                    }
                }
            }
        }
        T g = T(0), dl = T(0), rr = T(0);
        if (row < A.n_rows) {
#pragma unroll
            for (int r = 0; r < S; r++) {
                const uint64_t i = (uint64_t)row * S + r;
                const T ri = rc[i], di = d[i];
                T un, rnext;
                if (start) {   // the kept direction in the new residual's scale (zero for a fresh start)
                    rnext = ri;
                    un = di * ri;
                    v.p[i] = scale != 0.0 ? (T)(scale * (double)v.p[i]) : T(0);
                    sp[i] = scale != 0.0 ? (T)(scale * (double)sp[i]) : T(0);
                } else {
                    const T wi = wc[i], spi = sp[i];
                    un = cgcg_next_u<T>(ri, wi, spi, di, al, bt, rnext);
                    const T pn = fma(bt, v.p[i], di * ri);
                    v.p[i] = pn;
                    s_out[i] = fma(bt, spi, wi);
                    v.x[i] = fma(al, pn, v.x[i]);
                    rn_out[i] = rnext;
                }
                w_out[i] = acc[r];
                g = fma(rnext, un, g);
                dl = fma(acc[r], un, dl);
                rr = fma(rnext, rnext, rr);
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            g += __shfl_xor_sync(0xffffffffu, g, o);
            dl += __shfl_xor_sync(0xffffffffu, dl, o);
            rr += __shfl_xor_sync(0xffffffffu, rr, o);
        }
        if (lane == 0) {
            v.slice3[3 * (uint64_t)sl] = g;
            v.slice3[3 * (uint64_t)sl + 1] = dl;
            v.slice3[3 * (uint64_t)sl + 2] = rr;
        }
        uint32_t nx = 0;
        if (lane == 0) nx = atomicAdd(&next_sl, 1u);
        sl = __shfl_sync(0xffffffffu, nx, 0);
    }
    __syncthreads();   // the CTA's slice partials are visible to all its threads
    T g = T(0), dl = T(0), rr = T(0);
    for (uint32_t i = s_beg + threadIdx.x; i < s_end; i += kVecThreads) {
        g += v.slice3[3 * (uint64_t)i];
        dl += v.slice3[3 * (uint64_t)i + 1];
        rr += v.slice3[3 * (uint64_t)i + 2];
    }
    double bg, bd, br;
    block_sum3_v<T>(g, dl, rr, sh, bg, bd, br);
    const uint32_t nb = gridDim.x;
    if (threadIdx.x == 0) {
        part[blockIdx.x] = bg;
        part[nb + blockIdx.x] = bd;
        part[2 * nb + blockIdx.x] = br;
    }
    if (!last_cta(&ctl->ticket, &flag, nb)) return;
    double a = 0.0, b = 0.0, c = 0.0;
    for (uint32_t i = threadIdx.x; i < nb; i += kVecThreads) {
        a += __ldcg(part + i);
        b += __ldcg(part + nb + i);
        c += __ldcg(part + 2 * nb + i);
    }
    block_sum3_v<double>(a, b, c, sh, bg, bd, br);
    if (threadIdx.x == 0) {
        const double gamma_old = ctl->rz, alpha_old = ctl->alpha;
        ctl->rr = br;
        ctl->pq = bd;
        if (start) {
            // A kept direction continues, else alpha = gamma / delta.  The stopped run's
            // last iteration moved along p_i and left gamma_(i+1) in rz and gamma_i in
            // rz_prev (both rescaled by the host); the new residual stands in for
            // r_(i+1), so beta = gamma_new / gamma_i.
            const double gamma_i = ctl->rz_prev;
            const double beta = (scale != 0.0 && gamma_i != 0.0) ? bg / gamma_i : 0.0;
            const double den = beta != 0.0 && alpha_old != 0.0 ? bd - beta * bg / alpha_old : bd;
            ctl->beta = beta;
            ctl->alpha = den != 0.0 ? bg / den : 0.0;
            ctl->iterations = 0;
            ctl->done = (br <= ctl->tol2 || !(br == br)) ? 1 : 0;
        } else {
            const int64_t it = ctl->iterations + 1;
            ctl->iterations = it;
            const bool stop = br <= ctl->tol2 || it >= ctl->maxit || !(br == br);
            if (stop) {
                ctl->done = 1;
            } else {
                const double beta = gamma_old != 0.0 ? bg / gamma_old : 0.0;
                const double den = alpha_old != 0.0 ? bd - beta * bg / alpha_old : bd;
                ctl->beta = beta;
                ctl->alpha = den != 0.0 ? bg / den : 0.0;
            }
            ctl->pcur = cur ^ 1;
        }
        ctl->rz_prev = gamma_old;
        ctl->rz = bg;
        ctl->ticket = 0;
    }
}


// ------------------------------------------------------------------ one-kernel PCG iteration
// Standard Jacobi-PCG (alpha = r.z / p.q with the explicit q = A p) in one
// kernel per iteration, k_sell_fused.  Kernel k finishes iteration k-1 for
// the warp's own rows (r_k = r_(k-1) - alpha q_(k-1), x += alpha p_(k-1)),
// forms p_k = z_k + beta_k p_(k-1) for its own rows and for every column it
// gathers, from the stored z_(k-1), w_(k-1) = D^-1 q_(k-1) and p_(k-1):
// z_k = z_(k-1) - alpha w_(k-1), the same expression in every warp, so the
// gathered and the stored p_k agree bit for bit.  It computes q_k = A p_k and
// stores, interleaved per node, z_k = D^-1 r_k and w_k = D^-1 q_k for the next
// kernel (z is re-formed from r every iteration, so it does not drift from
// D^-1 r).  One ordered reduction gives p.q, q.z, q.w, r.z and r.r; the last
// CTA sets alpha_k = r.z / p.q and, since beta_(k+1) is needed before the
// kernel that could reduce r_(k+1).z_(k+1) runs, takes that dot from the
// identity r_(k+1) = r_k - alpha_k q_k:
//   r_(k+1).z_(k+1) = r_k.z_k - 2 alpha_k q_k.z_k + alpha_k^2 q_k.w_k,
// with r_k.z_k the exact dot of this kernel (the expansion's rounding enters
// one beta and does not accumulate).  p and zw are double-buffered (gathered
// while being rewritten); r, q and x are touched by their own rows only.  The
// first kernel of a run (ctl->first) runs with alpha = 0 on the state
// k_fused_prep set up: zw = (D^-1 r, 0), q = 0, p = the kept direction scaled
// (or 0), beta from the residual's r.z.
template <typename T>
struct FusedVecs {
    const T *dinv;
    T *x, *r, *q;   // own rows only
    T *p[2];        // direction (gathered)
    T *zw[2];       // per node: z (S entries), then w (S entries) (gathered)
    double *slice5; // [5 * n_slices]: p.q, q.z, q.w, r.z, r.r partials of each slice
};

// S entries of a node's z and w (2S contiguous values of an interleaved buffer).
template <int S, typename T>
__device__ __forceinline__ void load_zw(const T *__restrict__ zw, uint32_t c, T z[S], T w[S])
{
    if constexpr (S == 2 && sizeof(T) == 4) {
        const float4 a = __ldg(reinterpret_cast<const float4 *>(zw) + c);
        z[0] = a.x; z[1] = a.y; w[0] = a.z; w[1] = a.w;
    } else {
#pragma unroll
        for (int q = 0; q < S; q++) {
            z[q] = __ldg(zw + (uint64_t)c * 2 * S + q);
            w[q] = __ldg(zw + (uint64_t)c * 2 * S + S + q);
        }
    }
}

// p_k of one entry from z_(k-1), w_(k-1), p_(k-1).
template <typename T>
__device__ __forceinline__ T fused_dir(T z, T w, T p, T al, T bt)
{
    return fma(bt, p, fma(-al, w, z));
}

template <int S, typename T, int HINT = kMatrixHint>
__global__ void __launch_bounds__(kVecThreads) k_sell_fused(SellView<T> A, FusedVecs<T> v, double *part, PcgCtl *ctl)
{
    __shared__ double sh[5 * (kVecThreads >> 5)];
    __shared__ int flag;
    __shared__ uint32_t next_sl;
    if (A.prefetch_bytes && threadIdx.x == 0) {
        // the matrix does not change during a solve: stream the head of this CTA's
        // slot range into L2 while the predecessor finishes (as k_sell_dir)
        const uint32_t sb = __ldg(A.cta_first + blockIdx.x), se = __ldg(A.cta_first + blockIdx.x + 1);
        const uint64_t g0 = __ldg(A.slice_ptr + sb), g1 = __ldg(A.slice_ptr + se);
        const uint64_t vfull = (g1 - g0) * (S * S * sizeof(T)), cfull = (g1 - g0) * 4;
        const uint64_t vcap = A.prefetch_bytes, ccap = A.prefetch_bytes / (S * S);
        const uint64_t vb = (vfull < vcap ? vfull : vcap) & ~uint64_t(15);
        const uint64_t cbytes = (cfull < ccap ? cfull : ccap) & ~uint64_t(15);
        if (vb) asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(A.val + g0 * (S * S)), "r"((uint32_t)vb) : "memory");
        if (cbytes) asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(A.col + g0), "r"((uint32_t)cbytes) : "memory");
    }
    pdl_wait();
    pdl_release();
    if (ctl->done) return;
    constexpr int U = kSpmvUnroll;
    constexpr uint32_t WPB = kVecThreads / 32;
    const uint32_t lane = threadIdx.x & 31;
    const int cur = ctl->pcur;
    const T al = (T)ctl->alpha;
    const T bt = (T)ctl->beta;
    const T *__restrict__ pold = cur ? v.p[1] : v.p[0];
    T *__restrict__ pnew = cur ? v.p[0] : v.p[1];
    const T *__restrict__ zwo = cur ? v.zw[1] : v.zw[0];
    T *__restrict__ zwn = cur ? v.zw[0] : v.zw[1];
    const uint32_t s_beg = __ldg(A.cta_first + blockIdx.x), s_end = __ldg(A.cta_first + blockIdx.x + 1);
    const uint64_t pol = stream_policy<HINT>();
    if (threadIdx.x == 0) next_sl = s_beg + WPB;
    __syncthreads();
    for (uint32_t sl = s_beg + (threadIdx.x >> 5); sl < s_end;) {
        const uint32_t row = __ldg(A.perm + (uint64_t)sl * 32 + lane);
        const uint64_t g0 = __ldg(A.slice_ptr + sl);
        const uint32_t len = (uint32_t)((__ldg(A.slice_ptr + sl + 1) - g0) >> 5);
        T acc[S];
#pragma unroll
        for (int r = 0; r < S; r++) acc[r] = T(0);
        uint32_t c[U];
        T blk[U][S * S];
        for (uint32_t j0 = 0; j0 < len; j0 += U) {
            load_sell_group<S, U, T, HINT>(A, g0, j0, len, lane, c, blk, pol);
            T zv[U][S], wv[U][S], pv[U][S];
#pragma unroll
            for (int u = 0; u < U; u++) {
                if (j0 + u < len) {
                    load_zw<S, T>(zwo, c[u], zv[u], wv[u]);
                    load_x<S, T>(pold, c[u], pv[u]);
                }
            }
#pragma unroll
            for (int u = 0; u < U; u++) {
                if (j0 + u < len) {
#pragma unroll
                    for (int cc = 0; cc < S; cc++) {
                        const T pn = fused_dir<T>(zv[u][cc], wv[u][cc], pv[u][cc], al, bt);
#pragma unroll
                        for (int r = 0; r < S; r++) acc[r] = fma(blk[u][r * S + cc], pn, acc[r]);
                    }
                }
            }
        }
        T dpq = T(0), dqz = T(0), dqw = T(0), drz = T(0), drr = T(0);
        if (row < A.n_rows) {
            T zo[S], wo[S];
            load_zw<S, T>(zwo, row, zo, wo);
#pragma unroll
            for (int r = 0; r < S; r++) {
                const uint64_t i = (uint64_t)row * S + r;
                const T po = pold[i];
                const T pn = fused_dir<T>(zo[r], wo[r], po, al, bt);
                const T rk = fma(-al, v.q[i], v.r[i]);
                const T d = v.dinv[i];
                const T qk = acc[r];
                const T zk = d * rk, wk = d * qk;
                pnew[i] = pn;
                v.r[i] = rk;
                v.x[i] = fma(al, po, v.x[i]);
                v.q[i] = qk;
                zwn[(uint64_t)row * 2 * S + r] = zk;
                zwn[(uint64_t)row * 2 * S + S + r] = wk;
                dpq = fma(pn, qk, dpq);
                dqz = fma(qk, zk, dqz);
                dqw = fma(qk, wk, dqw);
                drz = fma(rk, zk, drz);
                drr = fma(rk, rk, drr);
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            dpq += __shfl_xor_sync(0xffffffffu, dpq, o);
            dqz += __shfl_xor_sync(0xffffffffu, dqz, o);
            dqw += __shfl_xor_sync(0xffffffffu, dqw, o);
            drz += __shfl_xor_sync(0xffffffffu, drz, o);
            drr += __shfl_xor_sync(0xffffffffu, drr, o);
        }
        if (lane == 0) {
            double *o5 = v.slice5 + 5 * (uint64_t)sl;
            o5[0] = (double)dpq;
            o5[1] = (double)dqz;
            o5[2] = (double)dqw;
            o5[3] = (double)drz;
            o5[4] = (double)drr;
        }
        uint32_t nx = 0;
        if (lane == 0) nx = atomicAdd(&next_sl, 1u);
        sl = __shfl_sync(0xffffffffu, nx, 0);
    }
    __syncthreads();   // the CTA's slice partials are visible to all its threads
    double a5[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
    for (uint32_t i = s_beg + threadIdx.x; i < s_end; i += kVecThreads) {
#pragma unroll
        for (int k = 0; k < 5; k++) a5[k] += v.slice5[5 * (uint64_t)i + k];
    }
    constexpr int NW = kVecThreads >> 5;
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
#pragma unroll
    for (int k = 0; k < 5; k++) {
        a5[k] = warp_sum(a5[k]);
        if (l == 0) sh[k * NW + w] = a5[k];
    }
    __syncthreads();
    const uint32_t nb = gridDim.x;
    if (threadIdx.x < 5) {
        double t = 0.0;
        for (int k = 0; k < NW; k++) t += sh[threadIdx.x * NW + k];
        part[threadIdx.x * nb + blockIdx.x] = t;
    }
    if (!last_cta(&ctl->ticket, &flag, nb)) return;
#pragma unroll
    for (int k = 0; k < 5; k++) a5[k] = 0.0;
    for (uint32_t i = threadIdx.x; i < nb; i += kVecThreads) {
#pragma unroll
        for (int k = 0; k < 5; k++) a5[k] += __ldcg(part + k * nb + i);
    }
    __syncthreads();   // sh is reused
#pragma unroll
    for (int k = 0; k < 5; k++) {
        a5[k] = warp_sum(a5[k]);
        if (l == 0) sh[k * NW + w] = a5[k];
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double t5[5];
#pragma unroll
        for (int k = 0; k < 5; k++) {
            t5[k] = 0.0;
            for (int j = 0; j < NW; j++) t5[k] += sh[k * NW + j];
        }
        const double pq = t5[0], qz = t5[1], qw = t5[2], rz = t5[3], rr = t5[4];
        const bool first = ctl->first != 0;
        const int64_t it = ctl->iterations + (first ? 0 : 1);
        ctl->first = 0;
        ctl->iterations = it;
        ctl->rr = rr;
        ctl->pq = pq;
        const bool stop = rr <= ctl->tol2 || it >= ctl->maxit || !(rr == rr);
        if (stop) {
            // x, r are those of this step; p[pcur] is the last direction x moved
            // along and ctl->rz its r.z (kept for a resumed run)
            ctl->done = 1;
            ctl->rz_prev = rz;
        } else {
            const double alpha = pq != 0.0 ? rz / pq : 0.0;
            const double rz_next = rz - 2.0 * alpha * qz + alpha * alpha * qw;
            ctl->alpha = alpha;
            ctl->beta = (rz != 0.0 && rz_next > 0.0) ? rz_next / rz : 0.0;
            ctl->rz = rz;
            ctl->pcur = cur ^ 1;
        }
        ctl->ticket = 0;
    }
}

// Set-up of a one-kernel PCG run on the residual in v.r: zw[pcur] = (D^-1 r, 0),
// q = 0, p[pcur] *= scale (0: a fresh run, p = 0).  Partials of r.z; the last
// CTA sets beta = r.z / (ctl->rz scale^2) for a kept direction (ctl->rz: the
// r.z of the previous run's last direction, in that run's scale), else 0.
template <int S, typename T>
__global__ void __launch_bounds__(kVecThreads) k_fused_prep(FusedVecs<T> v, uint64_t n, double scale, double *part,
                                                            PcgCtl *ctl)
{
    __shared__ double sh[33];
    __shared__ int flag;
    const int cur = ctl->pcur;
    T *__restrict__ p = cur ? v.p[1] : v.p[0];
    T *__restrict__ zw = cur ? v.zw[1] : v.zw[0];
    double drz = 0.0;
    for (uint64_t i = (uint64_t)blockIdx.x * kVecThreads + threadIdx.x; i < n; i += (uint64_t)gridDim.x * kVecThreads) {
        const uint64_t node = i / S, comp = i - node * S;
        const T ri = v.r[i];
        const T zi = v.dinv[i] * ri;
        zw[node * 2 * S + comp] = zi;
        zw[node * 2 * S + S + comp] = T(0);
        v.q[i] = T(0);
        p[i] = scale != 0.0 ? (T)(scale * (double)p[i]) : T(0);
        drz += (double)ri * (double)zi;
    }
    const double b = block_sum(drz, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = b;
    if (!last_cta(&ctl->ticket, &flag, gridDim.x)) return;
    const double rz = ordered_sum(part, gridDim.x, sh);
    if (threadIdx.x == 0) {
        const double old = ctl->rz * scale * scale;
        ctl->beta = (scale != 0.0 && old != 0.0) ? rz / old : 0.0;
        ctl->alpha = 0.0;
        ctl->first = 1;
        ctl->ticket = 0;
    }
}

}  // namespace amie
