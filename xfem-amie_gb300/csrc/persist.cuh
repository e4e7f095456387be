// persist.cuh -- Jacobi-PCG runs as one cooperative launch, for systems whose
// matrix and vectors stay in L2.
//
// Reference: ConjugateGradient::solve (solvers/conjugategradient.cpp:69-318),
// the same iteration as the two-kernel graph of solver.cuh (k_sell_dir with
// the direction folded in, then k_update).
//
// On a small system the graph's iteration is latency-bound: every kernel
// boundary costs a launch, the wait for the predecessor, a ticket and the last
// CTA's ordered sum.  Here one CTA per SM runs every iteration of a run (an
// opt-in: on this GPU the grid barriers measured slower than the graph's
// kernel boundaries, see SolverState::persist_mode):
//   phase A  p_new = z + beta p_old for every gathered entry, q = A p_new for
//            the CTA's slot-balanced slice range, per-CTA partial of p_new.q;
//   barrier; every CTA sums the per-CTA partials in index order (the same
//            operations in every CTA, so alpha = rz / pq is the same bits
//            everywhere);
//   phase B  x += alpha p, r -= alpha q, z = D^-1 r over a fixed grid-stride
//            share of the entries, per-CTA partials of r.z and r.r;
//   barrier; every CTA sums them: the stop test, beta, the next iteration.
// Every CTA takes the same decisions from the same sums, so the barrier
// counts stay in step.  Vectors other CTAs rewrite during the launch (z, p,
// q, the partials) are read through L2 (ld.global.cg): an SM's L1 is not
// coherent with the other SMs' stores.  The matrix does not change and is read
// through the read-only path, so a CTA's share can stay in its L1.
//
// Every wait is bounded: a barrier not reached within `polls` polls sets
// *err, and a CTA that sees *err set leaves; the launch always ends and the
// host reports AMIE_TIMEOUT.  `expect` is the number of arrivals a barrier
// waits for: the grid size (a test passes one more, which no barrier reaches).
#pragma once

#include "solver.cuh"

namespace amie {

// CTA size: 24 warps (80 registers) for 2x2 FP32 blocks, 16 warps (128
// registers) otherwise, so that no variant spills.
template <int S, typename T>
__host__ __device__ constexpr int persist_threads() { return (S == 2 && sizeof(T) == 4) ? 768 : 512; }
constexpr uint32_t kPersistPolls = 1u << 22;   // a few seconds of polling: far above any phase's duration

// Sum of one FP64 value per thread over a CTA of NT threads, in a fixed tree;
// the result is broadcast to every thread.  sh: >= NT / 32 + 1 doubles.
template <int NT>
__device__ __forceinline__ double cta_sum_all(double v, double *sh)
{
    constexpr int NW = NT / 32;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) sh[w] = v;
    __syncthreads();
    if (w == 0) {
        double r = l < NW ? sh[l] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) r += __shfl_xor_sync(0xffffffffu, r, o);
        if (l == 0) sh[NW] = r;
    }
    __syncthreads();
    const double r = sh[NW];
    __syncthreads();
    return r;
}

// Two values per thread in the vector precision T (warp levels in T, the
// per-warp sums in FP64, as block_sum2_v); results broadcast.
template <int NT, typename T>
__device__ __forceinline__ void cta_sum2_v(T a, T b, double *sh, double &ra, double &rb)
{
    constexpr int NW = NT / 32;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_xor_sync(0xffffffffu, a, o);
        b += __shfl_xor_sync(0xffffffffu, b, o);
    }
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) {
        sh[w] = (double)a;
        sh[NW + w] = (double)b;
    }
    __syncthreads();
    if (w == 0) {
        double x = l < NW ? sh[l] : 0.0, y = l < NW ? sh[NW + l] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            x += __shfl_xor_sync(0xffffffffu, x, o);
            y += __shfl_xor_sync(0xffffffffu, y, o);
        }
        if (l == 0) {
            sh[2 * NW] = x;
            sh[2 * NW + 1] = y;
        }
    }
    __syncthreads();
    ra = sh[2 * NW];
    rb = sh[2 * NW + 1];
    __syncthreads();
}

// Sum of the G per-CTA partials in index order, the same in every CTA (read
// through L2: other CTAs wrote them during the launch); broadcast.
template <int NT>
__device__ __forceinline__ double parts_sum(const double *parts, uint32_t G, double *sh)
{
    double v = 0.0;
    for (uint32_t i = threadIdx.x; i < G; i += NT) v += __ldcg(parts + i);
    return cta_sum_all<NT>(v, sh);
}

// Grid barrier on a monotone arrival counter: the CTA's stores (ordered
// before thread 0 by the CTA barrier) are released with the arrival and
// acquired with the count; returns false (after setting *err, or on seeing it
// set; *err is checked every 64 polls) if `target` arrivals are not seen
// within `polls` polls.
__device__ __forceinline__ bool grid_arrive_wait(uint32_t *count, uint32_t target, int32_t *err, uint32_t polls,
                                                 int *sh_ok)
{
    __syncthreads();
    if (threadIdx.x == 0) {
        asm volatile("red.release.gpu.global.add.u32 [%0], 1;" ::"l"(count) : "memory");
        int ok = 1;
        for (uint32_t k = 0;; k++) {
            uint32_t v;
            asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(count) : "memory");
            if (v >= target) break;
            if ((k & 63u) == 63u) {
                if (__ldcg(err) != 0) {
                    ok = 0;
                    break;
                }
                if (k >= polls) {
                    atomicExch(err, 1);
                    ok = 0;
                    break;
                }
            }
        }
        *sh_ok = ok;
    }
    __syncthreads();
    return *sh_ok != 0;
}

// Counters of a persistent run: the barrier's arrivals and the error flag
// (zeroed by the host before each launch).
struct PersistSync {
    uint32_t arrivals;
    int32_t err;
};

// The run's scalars, one copy per CTA in shared memory (every CTA holds the
// same values); kept out of registers, which the SpMV phase needs.
struct PersistScalars {
    double rz, beta, rz_prev, rr, pq, alpha, tol2;
    int64_t it, maxit;
    int32_t pcur, stop;
};

template <int S, typename T>
__global__ void __launch_bounds__(persist_threads<S, T>(), 1)
    k_pcg_persist(SellView<T> A, PcgVecs<T> v, uint64_t n, PcgParts parts, PcgCtl *ctl, PersistSync *sync,
                  uint32_t polls, uint32_t expect)
{
    constexpr int NT = persist_threads<S, T>();
    constexpr int NW = NT / 32;
    constexpr int U = kSpmvUnroll;
    constexpr int W = Pack<T>::n;
    __shared__ double sh[2 * NW + 2];
    __shared__ uint32_t next_sl;
    __shared__ int ok;
    __shared__ PersistScalars ps;
    const uint32_t G = gridDim.x, cta = blockIdx.x;
    const uint32_t lane = threadIdx.x & 31;
    // the run's state, the same in every CTA (written by the kernels before this launch)
    if (ctl->done) return;
    if (threadIdx.x == 0) {
        ps.rz = ctl->rz;
        ps.beta = ctl->beta;
        ps.rz_prev = ctl->rz_prev;
        ps.rr = ctl->rr;
        ps.pq = ctl->pq;
        ps.alpha = ctl->alpha;
        ps.tol2 = ctl->tol2;
        ps.it = ctl->iterations;
        ps.maxit = ctl->maxit;
        ps.pcur = ctl->pcur;
        ps.stop = 0;
    }
    const uint32_t s_beg = __ldg(A.cta_first + cta), s_end = __ldg(A.cta_first + cta + 1);
    uint32_t target = 0;
    __syncthreads();
    while (!ps.stop) {
        // ---- phase A: q = A (z + beta p_old), partial p_new.q
        {
            const T bt = (T)ps.beta;
            const T *pold = ps.pcur ? v.p2 : v.p;
            T *pnew = ps.pcur ? v.p : v.p2;
            if (threadIdx.x == 0) next_sl = s_beg + NW;
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
                            load_x_cg<S, T>(v.z, c[u], zv[u]);
                            load_x_cg<S, T>(pold, c[u], pv[u]);
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
                        const T pn = fma(bt, __ldcg(pold + i), __ldcg(v.z + i));
                        pnew[i] = pn;
                        v.q[i] = acc[r];
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
            for (uint32_t i = s_beg + threadIdx.x; i < s_end; i += NT) dot += __ldcg(A.slice_dot + i);
            double part, unused;
            cta_sum2_v<NT, T>(dot, T(0), sh, part, unused);
            if (threadIdx.x == 0) parts.pq[cta] = part;
        }
        target += expect;
        if (!grid_arrive_wait(&sync->arrivals, target, &sync->err, polls, &ok)) return;
        const double pq = parts_sum<NT>(parts.pq, G, sh);
        const double alpha = pq != 0.0 ? ps.rz / pq : 0.0;
        if (threadIdx.x == 0) {
            ps.pq = pq;
            ps.alpha = alpha;
        }

        // ---- phase B: x += alpha p, r -= alpha q, z = D^-1 r, partials r.z, r.r
        {
            const T a = (T)alpha;
            const T *pnew = ps.pcur ? v.p : v.p2;
            const T *__restrict__ d = v.dinv;
            const uint64_t tid = (uint64_t)cta * NT + threadIdx.x, stride = (uint64_t)G * NT;
            const bool al = aligned16(v.x) && aligned16(v.r) && aligned16(v.z) && aligned16(pnew) &&
                            aligned16(v.q) && aligned16(d);
            const uint64_t npk = al ? n / W : 0;
            T drz = T(0), drr = T(0);
            for (uint64_t k = tid; k < npk; k += stride) {
                T rv[W], qv[W], xv[W], pv[W], dv[W], zv[W];
                ld_pack<T>(v.r, k, rv);
                ldq_pack<T, true>(v.q, k, qv);
                ld_pack<T>(v.x, k, xv);
                ldq_pack<T, true>(pnew, k, pv);
                ldg_pack<T>(d, k, dv);
#pragma unroll
                for (int cc = 0; cc < W; cc++) {
                    rv[cc] = rv[cc] - a * qv[cc];
                    xv[cc] = fma(a, pv[cc], xv[cc]);
                    zv[cc] = rv[cc] * dv[cc];
                    drz = fma(rv[cc], zv[cc], drz);
                    drr = fma(rv[cc], rv[cc], drr);
                }
                st_pack<T>(v.r, k, rv);
                st_pack<T>(v.x, k, xv);
                st_pack<T>(v.z, k, zv);
            }
            for (uint64_t i = npk * W + tid; i < n; i += stride) {
                const T ri = v.r[i] - a * __ldcg(v.q + i);
                v.x[i] = fma(a, __ldcg(pnew + i), v.x[i]);
                v.r[i] = ri;
                const T zi = ri * d[i];
                v.z[i] = zi;
                drz = fma(ri, zi, drz);
                drr = fma(ri, ri, drr);
            }
            double brz, brr;
            cta_sum2_v<NT, T>(drz, drr, sh, brz, brr);
            if (threadIdx.x == 0) {
                parts.rz[cta] = brz;
                parts.rr[cta] = brr;
            }
        }
        target += expect;
        if (!grid_arrive_wait(&sync->arrivals, target, &sync->err, polls, &ok)) return;
        double rz_new, rr;
        {
            double a2 = 0.0, b2 = 0.0;
            for (uint32_t i = threadIdx.x; i < G; i += NT) {
                a2 += __ldcg(parts.rz + i);
                b2 += __ldcg(parts.rr + i);
            }
            cta_sum2_v<NT, double>(a2, b2, sh, rz_new, rr);
        }
        if (threadIdx.x == 0) {   // k_update's last-CTA step
            const int64_t it = ps.it + 1;
            const bool stop = rr <= ps.tol2 || it >= ps.maxit || !(rr == rr);
            if (!stop) ps.beta = ps.rz != 0.0 ? rz_new / ps.rz : 0.0;
            ps.it = it;
            ps.rr = rr;
            ps.rz_prev = ps.rz;
            ps.rz = rz_new;
            ps.pcur ^= 1;
            ps.stop = stop ? 1 : 0;
        }
        __syncthreads();
    }
    if (cta == 0 && threadIdx.x == 0) {   // the control block as the graph leaves it
        ctl->iterations = ps.it;
        ctl->rr = ps.rr;
        ctl->rz = ps.rz;
        ctl->rz_prev = ps.rz_prev;
        ctl->beta = ps.beta;
        ctl->pq = ps.pq;
        ctl->alpha = ps.alpha;
        ctl->pcur = ps.pcur;
        ctl->ticket = 0;
        ctl->done = 1;
    }
}

}  // namespace amie
