// server.cuh -- continuous-batching solve server, included by solver.cu.
//
// Requests (independent meshes: microstructure or damage-step solves of
// uneven size) are admitted while others run, as slots and the HBM budget
// allow.  Admission (upload, pattern + scatter map, element matrices, gather,
// Dirichlet elimination) runs on its own stream, overlapping the solves.
// Every admitted solve keeps its matrix, scatter map and warm-start vector on
// the device.  All solves in the batch advance together: one CUDA graph holds
// kBatchIters Jacobi-PCG iterations over every active slot, each kernel
// covering all slots through a CTA -> slot map (CTAs split between slots in
// proportion to their size, so each slot's reductions are its own CTAs'
// partials: deterministic, and the same alone and in a mix).  A slot whose
// inner run has stopped does no more work in the batch; the kernels that end
// each batch replace its residual in FP64 and decide, on the device, whether
// the solve is finished, resumes its FP32 run or restarts it.  Between batch
// launches the host only retires finished solves and joins admitted ones.
// The batch graph has no device-side waiting (the opt-in persistent batch has
// bounded slot barriers).
#pragma once

#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <thread>

namespace amie {

constexpr int kBatchIters = 16;

// State of a slot's whole solve, kept on the device: the host writes it when
// the request joins; afterwards only the last CTA of the slot in the refinement
// kernels (kb_residual, kb_restart) changes it.
struct SlotRun {
    double bnorm;         // |b|
    double target;        // rtol |b|
    double rnorm;         // |b - A x| at the latest residual replacement (the inner run's scale)
    double ratio;         // kRunResume: new / previous residual norm
    int64_t iterations;   // inner iterations of all runs so far
    int64_t maxit;        // cap on them
    int32_t refinements;  // residual replacements (mixed)
    int32_t status;       // AMIE_NOT_READY while the solve runs, then its result
    int32_t mode;         // kRunIterating, or what kb_restart does next
    uint32_t gen;         // join number of the request (the host ignores copies of an earlier one)
};
constexpr int32_t kRunIterating = 0;   // the inner run iterates (or stopped and awaits kb_residual)
constexpr int32_t kRunResume = 1;      // continue the inner run from the replaced residual, direction kept
constexpr int32_t kRunRestart = 2;     // start a fresh inner run from the replaced residual

// Device view of one slot: the slot's SELL copies (CTA table for its own CTA
// count), vectors, control block and its range of the batch's partial sums.
struct SlotDesc {
    SellView<float> A32;
    SellView<double> A64;
    PcgVecs<float> v32;      // inner vectors of the mixed solve (two direction buffers)
    PcgVecs<double> v64;     // FP64 vectors (one direction buffer); v64.A is the FP64 block-CSR matrix
    PcgParts parts;          // the batch partials of CTAs c0 .. c1-1
    PcgCtl *ctl;             // the slot's control block
    SlotRun *run;            // the slot's solve state
    const double *rhs;       // b (after the Dirichlet elimination)
    uint64_t n;
    int32_t c0, c1;          // CTA range in the batch grid
    int32_t active;          // 1 = iterate
    int32_t mixed;
    int32_t s;               // DOF per node: 2 (triangles) or 3 (tetrahedra)
    int32_t pad_;
};

template <typename T>
__device__ __forceinline__ const SellView<T> &slot_A(const SlotDesc &d);
template <>
__device__ __forceinline__ const SellView<float> &slot_A<float>(const SlotDesc &d) { return d.A32; }
template <>
__device__ __forceinline__ const SellView<double> &slot_A<double>(const SlotDesc &d) { return d.A64; }

template <typename T>
__device__ __forceinline__ const PcgVecs<T> &slot_v(const SlotDesc &d);
template <>
__device__ __forceinline__ const PcgVecs<float> &slot_v<float>(const SlotDesc &d) { return d.v32; }
template <>
__device__ __forceinline__ const PcgVecs<double> &slot_v<double>(const SlotDesc &d) { return d.v64; }

// The slot of this CTA and the CTA's place in the slot's group, or null when
// the CTA has no slot, the slot is idle or its run has finished.
__device__ __forceinline__ const SlotDesc *slot_of(const SlotDesc *slots, const int16_t *cta_slot, Cta *c)
{
    const int s = cta_slot[blockIdx.x];
    if (s < 0) return nullptr;
    const SlotDesc *d = slots + s;
    if (!d->active || d->ctl->done) return nullptr;
    *c = Cta{blockIdx.x - (uint32_t)d->c0, (uint32_t)(d->c1 - d->c0)};
    return d;
}

// Batched kernel A (mixed): per slot, p = z + beta p folded into q = A p, p.q,
// alpha -- the single-solve k_sell_dir on the slot's own CTAs.  SMAX = 2: 2D
// slots only; 3: the body of each slot's stride (the batch then has 3D slots;
// a kernel holding both bodies needs more registers, so 2D-only batches keep
// the smaller one).
template <typename T, int SMAX = 2>
__global__ void __launch_bounds__(kVecThreads) kb_sell_dir(const SlotDesc *slots, const int16_t *cta_slot)
{
    // the slot table is the host's, fixed for the whole batch graph: look the
    // slot up before waiting; only its control block depends on the predecessor
    const int s = cta_slot[blockIdx.x];
    const SlotDesc *d = s >= 0 ? slots + s : nullptr;
    const bool live = d && d->active;
    pdl_wait();
    pdl_release();
    if (!live || d->ctl->done) return;
    const Cta c{blockIdx.x - (uint32_t)d->c0, (uint32_t)(d->c1 - d->c0)};
    if (SMAX == 3 && d->s == 3) sell_dir_body<3, T>(slot_A<T>(*d), slot_v<T>(*d), d->parts.pq, d->ctl, true, c);
    else sell_dir_body<2, T>(slot_A<T>(*d), slot_v<T>(*d), d->parts.pq, d->ctl, true, c);
}

// Batched kernel A (FP64): per slot q = A p, p.q, alpha (SMAX as kb_sell_dir).
template <typename T, int SMAX = 2>
__global__ void __launch_bounds__(kVecThreads) kb_sell_pq(const SlotDesc *slots, const int16_t *cta_slot)
{
    __shared__ double sh[33];
    __shared__ int flag;
    __shared__ uint32_t next_sl;
    pdl_wait();
    pdl_release();
    Cta c;
    const SlotDesc *d = slot_of(slots, cta_slot, &c);
    if (!d) return;
    const PcgVecs<T> &v = slot_v<T>(*d);
    if (SMAX == 3 && d->s == 3)
        sell_pq_body<3, kSpmvUnroll, false, T, 0>(slot_A<T>(*d), v.p, v.q, d->parts.pq, d->ctl, sh, &flag, &next_sl, c);
    else
        sell_pq_body<2, kSpmvUnroll, false, T, 0>(slot_A<T>(*d), v.p, v.q, d->parts.pq, d->ctl, sh, &flag, &next_sl, c);
}

// Batched kernel B: per slot x, r, z updates, r.z, r.r; last CTA of the slot:
// stop test and beta (update_body's work).  The slot table is written by the
// host before the batch graph starts, so the slot, its vectors and the loads
// of the CTA's first step that the SpMV does not produce (x and r, last
// written by the previous update, which finished before the SpMV could start;
// D^-1) are issued before the wait on the SpMV, as in k_update.
template <typename T>
__global__ void __launch_bounds__(kVecThreads, 3) kb_update(const SlotDesc *slots, const int16_t *cta_slot)
{
    __shared__ double sh[2 * (kVecThreads >> 5)];
    __shared__ int flag;
    constexpr int W = Pack<T>::n;
    const int s = cta_slot[blockIdx.x];
    const SlotDesc *d = s >= 0 ? slots + s : nullptr;
    const bool live = d && d->active;
    T rv[2][W], xv[2][W], dv[2][W];
    uint64_t tid = 0, stride = 1, npk = 0, n = 0;
    Cta c{0, 1};
    if (live) {
        const PcgVecs<T> &v = slot_v<T>(*d);
        n = d->n;
        c = Cta{blockIdx.x - (uint32_t)d->c0, (uint32_t)(d->c1 - d->c0)};
        const bool al = aligned16(v.x) && aligned16(v.r) && aligned16(v.z) && aligned16(v.p) && aligned16(v.q) &&
                        aligned16(v.dinv) && (!v.p2 || aligned16(v.p2));
        tid = (uint64_t)c.id * kVecThreads + threadIdx.x;
        stride = (uint64_t)c.n * kVecThreads;
        npk = al ? n / W : 0;
        if (tid < npk) {
            ld_pack<T>(v.r, tid, rv[0]);
            ld_pack<T>(v.x, tid, xv[0]);
            ldg_pack<T>(v.dinv, tid, dv[0]);
            if (tid + stride < npk) {
                ld_pack<T>(v.r, tid + stride, rv[1]);
                ld_pack<T>(v.x, tid + stride, xv[1]);
                ldg_pack<T>(v.dinv, tid + stride, dv[1]);
            }
        }
    }
    // done and pcur are written only by the previous update's last CTA (finished);
    // alpha comes from the SpMV this kernel waits on
    PcgCtl *ctl = live ? d->ctl : nullptr;
    const int32_t done = live ? ctl->done : 1;
    const int32_t pcur = live ? ctl->pcur : 0;
    pdl_wait();
    pdl_release();
    if (done) return;
    const T a = (T)ctl->alpha;
    const PcgVecs<T> &v = slot_v<T>(*d);
    T *__restrict__ x = v.x;
    T *__restrict__ r = v.r;
    T *__restrict__ z = v.z;
    const T *__restrict__ q = v.q;
    const T *__restrict__ dinv = v.dinv;
    // with two direction buffers the SpMV just wrote this iteration's p into the other one
    const T *__restrict__ p = v.p2 ? (pcur ? v.p : v.p2) : v.p;
    T drz = T(0), drr = T(0);
    for (uint64_t k = tid; k < npk; k += 2 * stride) {
        const uint64_t k2 = k + stride;
        const bool two = k2 < npk;
        T qv[2][W], pv[2][W];
        if (k != tid) {
            ld_pack<T>(r, k, rv[0]);
            ld_pack<T>(x, k, xv[0]);
            ldg_pack<T>(dinv, k, dv[0]);
            if (two) {
                ld_pack<T>(r, k2, rv[1]);
                ld_pack<T>(x, k2, xv[1]);
                ldg_pack<T>(dinv, k2, dv[1]);
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
            for (int e = 0; e < W; e++) {
                rv[h][e] = rv[h][e] - a * qv[h][e];
                xv[h][e] = fma(a, pv[h][e], xv[h][e]);
                zv[e] = rv[h][e] * dv[h][e];
                drz = fma(rv[h][e], zv[e], drz);
                drr = fma(rv[h][e], rv[h][e], drr);
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
        const T zi = ri * dinv[i];
        z[i] = zi;
        drz = fma(ri, zi, drz);
        drr = fma(ri, ri, drr);
    }
    double brz, brr;
    block_sum2_v<T>(drz, drr, sh, brz, brr);
    const PcgParts &parts = d->parts;
    if (threadIdx.x == 0) {
        parts.rz[c.id] = brz;
        parts.rr[c.id] = brr;
    }
    if (!last_cta(&ctl->ticket, &flag, c.n)) return;
    int64_t it = 0, maxit = 0;
    double rz_old = 0.0, tol2 = 0.0;
    if (threadIdx.x == 0) {
        it = ctl->iterations + 1;
        maxit = ctl->maxit;
        rz_old = ctl->rz;
        tol2 = ctl->tol2;
    }
    double sa = 0.0, sb = 0.0;
    for (uint32_t i = threadIdx.x; i < c.n; i += kVecThreads) {
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

// Batched kernel C (FP64): per slot p = z + beta p.
template <typename T>
__global__ void __launch_bounds__(kVecThreads) kb_direction(const SlotDesc *slots, const int16_t *cta_slot)
{
    pdl_wait();
    pdl_release();
    Cta c;
    const SlotDesc *d = slot_of(slots, cta_slot, &c);
    if (!d) return;
    direction_body<T>(slot_v<T>(*d), d->n, d->ctl, c);
}

// Persistent batch (mixed solver): one cooperative launch runs `iters` PCG
// iterations of every active slot; the CTAs of a slot meet at a slot barrier
// after each phase instead of at kernel boundaries.  Every wait is bounded:
// a barrier that is not reached within `polls` polls (the server's
// barrier_polls, default kBarrierPolls) sets *err, and a CTA that sees *err
// set returns, so the launch always ends.
constexpr uint32_t kBarrierPolls = 1u << 22;   // ~0.3 s at 64 ns per poll

__device__ __forceinline__ bool slot_barrier(uint32_t *count, uint32_t target, int32_t *err, int *sh_ok,
                                             uint32_t max_polls)
{
    __syncthreads();   // the CTA's work of the phase is done
    if (threadIdx.x == 0) {
        __threadfence();   // ... and visible before the arrival
        atomicAdd(count, 1u);
        int ok = 1;
        for (uint32_t polls = 0;; polls++) {
            if (__ldcg(count) >= target) break;
            if (__ldcg(err) != 0) {
                ok = 0;
                break;
            }
            if (polls >= max_polls) {
                atomicExch(err, 1);
                ok = 0;
                break;
            }
            __nanosleep(64);
        }
        __threadfence();
        *sh_ok = ok;
    }
    __syncthreads();
    return *sh_ok != 0;
}

template <typename T>
__global__ void __launch_bounds__(kVecThreads) kb_persistent(const SlotDesc *slots, const int16_t *cta_slot, int iters,
                                                             uint32_t *bar, int32_t *err, uint32_t polls)
{
    __shared__ double sh[2 * (kVecThreads >> 5)];
    __shared__ int flag, ok;
    const int s = cta_slot[blockIdx.x];
    if (s < 0) return;
    const SlotDesc *d = slots + s;
    if (!d->active) return;
    const Cta c{blockIdx.x - (uint32_t)d->c0, (uint32_t)(d->c1 - d->c0)};
    PcgCtl *ctl = d->ctl;
    uint32_t target = 0;
    for (int it = 0; it < iters; it++) {
        // the same for every CTA of the slot: written before the barrier they all passed
        if (ctl_ld<true>(&ctl->done)) break;
        sell_dir_body<2, T, true>(slot_A<T>(*d), slot_v<T>(*d), d->parts.pq, ctl, true, c);
        target += c.n;
        if (!slot_barrier(bar + s, target, err, &ok, polls)) return;
        update_body<T, true>(slot_v<T>(*d), d->n, d->parts, ctl, sh, &flag, c);
        target += c.n;
        if (!slot_barrier(bar + s, target, err, &ok, polls)) return;
    }
}

// ------------------------------------------------------------------ device-side refinement
// Appended to every batch: for each slot whose inner run stopped during the
// batch, the FP64 residual replacement and the decision the single-solve
// driver takes on the host (solve_pcg): retire (converged, NaN, iteration or
// refinement cap), resume the FP32 run with its direction kept (the true
// residual fell by at least half since the previous replacement), or restart
// it.  The host only retires the slots whose SlotRun.status became final.

// The slot of this CTA if its inner run stopped, its solve is open and its
// run is in `mode`.
__device__ __forceinline__ const SlotDesc *slot_stopped(const SlotDesc *slots, const int16_t *cta_slot, int32_t mode,
                                                        Cta *c)
{
    const int s = cta_slot[blockIdx.x];
    if (s < 0) return nullptr;
    const SlotDesc *d = slots + s;
    if (!d->active || !d->ctl->done || d->run->status != AMIE_NOT_READY || d->run->mode != mode) return nullptr;
    *c = Cta{blockIdx.x - (uint32_t)d->c0, (uint32_t)(d->c1 - d->c0)};
    return d;
}

// Mixed: x += rnorm * d (the FP32 run's increment, in the scale of its residual).
__global__ void __launch_bounds__(kVecThreads) kb_accumulate(const SlotDesc *slots, const int16_t *cta_slot)
{
    Cta c;
    const SlotDesc *d = slot_stopped(slots, cta_slot, kRunIterating, &c);
    if (!d) return;
    const double scale = d->run->rnorm;
    const float *__restrict__ dx = d->v32.x;
    double *__restrict__ x = d->v64.x;
    for (uint64_t i = (uint64_t)c.id * kVecThreads + threadIdx.x; i < d->n; i += (uint64_t)c.n * kVecThreads)
        x[i] += scale * (double)dx[i];
}

constexpr int kResidualGroup = 4;   // lanes per block row in kb_residual

// This CTA's part of r = b - A x for a slot of stride S and its partial |r|^2.
template <int S>
__device__ __forceinline__ double residual_rows(const SlotDesc *d, Cta c)
{
    constexpr int G = kResidualGroup;
    constexpr int RPB = kVecThreads / G;
    const BsrView<double> &A = d->v64.A;
    const double *__restrict__ x = d->v64.x;
    const double *__restrict__ b = d->rhs;
    double *__restrict__ r = d->v64.r;
    const int lane = threadIdx.x % G;
    double dot = 0.0;
    for (uint32_t base = c.id * RPB; base < A.n_rows; base += c.n * RPB) {
        const uint32_t row = base + threadIdx.x / G;
        const bool valid = row < A.n_rows;
        const uint32_t rb = valid ? __ldg(A.row_ptr + row) : 0u, re = valid ? __ldg(A.row_ptr + row + 1) : 0u;
        double acc[S];
        row_spmv<S, G, double>(A, x, rb, re, lane, acc);
        if (valid && lane == 0) {
#pragma unroll
            for (int k = 0; k < S; k++) {
                const double y = b[(uint64_t)row * S + k] - acc[k];
                r[(uint64_t)row * S + k] = y;
                dot += y * y;
            }
        }
    }
    return dot;
}

// r = b - A x in FP64 over the slot's CTAs, |r|^2 in CTA order; the slot's last
// CTA counts the run's iterations and decides what follows.
__global__ void __launch_bounds__(kVecThreads) kb_residual(const SlotDesc *slots, const int16_t *cta_slot)
{
    __shared__ double sh[33];
    __shared__ int flag;
    Cta c;
    const SlotDesc *d = slot_stopped(slots, cta_slot, kRunIterating, &c);
    if (!d) return;
    double dot = d->s == 3 ? residual_rows<3>(d, c) : residual_rows<2>(d, c);
    dot = block_sum(dot, sh);
    if (threadIdx.x == 0) d->parts.spare[c.id] = dot;
    PcgCtl *ctl = d->ctl;
    if (!last_cta(&ctl->ticket, &flag, c.n)) return;
    const double rr = ordered_sum(d->parts.spare, c.n, sh);
    if (threadIdx.x == 0) {
        SlotRun *run = d->run;
        run->iterations += ctl->iterations;
        if (d->mixed) run->refinements++;
        const double prev = run->rnorm, rn = sqrt(rr);
        run->rnorm = rn;
        if (!(rr == rr)) {
            run->status = AMIE_NAN;
        } else if (rn <= run->target) {
            run->status = AMIE_OK;
        } else if (run->iterations >= run->maxit || run->refinements > 200) {
            run->status = AMIE_NOT_CONVERGED;
        } else if (d->mixed && rn <= 0.5 * prev) {
            run->mode = kRunResume;
            run->ratio = rn / prev;
        } else {
            run->mode = kRunRestart;
        }
        ctl->ticket = 0;
    }
}

// The next inner run from the replaced residual.  Mixed: r32 = r / |r|, d = 0,
// z = D^-1 r32 (p = z for a restart); FP64: z = D^-1 r, p = z.  Last CTA: the
// control block of the new run (a resume keeps the direction through
// beta = ratio r.z / r.z_prev, as resume_body).
__global__ void __launch_bounds__(kVecThreads) kb_restart(const SlotDesc *slots, const int16_t *cta_slot,
                                                          double inner_reduction, double last_target)
{
    __shared__ double sh[2 * (kVecThreads >> 5)];
    __shared__ int flag;
    const int s = cta_slot[blockIdx.x];
    if (s < 0) return;
    const SlotDesc *d = slots + s;
    if (!d->active || d->run->status != AMIE_NOT_READY) return;
    const int32_t mode = d->run->mode;
    if (mode == kRunIterating) return;
    const Cta c{blockIdx.x - (uint32_t)d->c0, (uint32_t)(d->c1 - d->c0)};
    const SlotRun *run = d->run;
    const uint64_t n = d->n;
    const uint64_t i0 = (uint64_t)c.id * kVecThreads + threadIdx.x, step = (uint64_t)c.n * kVecThreads;
    double brz, brr;
    if (d->mixed) {
        const PcgVecs<float> &v = d->v32;
        const double *__restrict__ r64 = d->v64.r;
        const double inv = 1.0 / run->rnorm;
        float drz = 0.0f, drr = 0.0f;
        for (uint64_t i = i0; i < n; i += step) {
            const float ri = (float)(r64[i] * inv);
            const float zi = ri * v.dinv[i];
            v.r[i] = ri;
            v.x[i] = 0.0f;
            v.z[i] = zi;
            if (mode == kRunRestart) v.p[i] = zi;
            drz = fmaf(ri, zi, drz);
            drr = fmaf(ri, ri, drr);
        }
        block_sum2_v<float>(drz, drr, sh, brz, brr);
    } else {
        const PcgVecs<double> &v = d->v64;
        double drz = 0.0, drr = 0.0;
        for (uint64_t i = i0; i < n; i += step) {
            const double ri = v.r[i];
            const double zi = ri * v.dinv[i];
            v.z[i] = zi;
            v.p[i] = zi;
            drz = fma(ri, zi, drz);
            drr = fma(ri, ri, drr);
        }
        block_sum2_v<double>(drz, drr, sh, brz, brr);
    }
    const PcgParts &parts = d->parts;
    if (threadIdx.x == 0) {
        parts.rz[c.id] = brz;
        parts.rr[c.id] = brr;
    }
    PcgCtl *ctl = d->ctl;
    if (!last_cta(&ctl->ticket, &flag, c.n)) return;
    double rz, rr;
    ordered_sum2(parts.rz, parts.rr, c.n, sh, rz, rr);
    if (threadIdx.x == 0) {
        SlotRun *w = d->run;
        double tol2;
        if (d->mixed) {
            const double need = last_target * w->target / w->rnorm;
            const double inner = fmin(0.5, fmax(inner_reduction, need));
            tol2 = inner * inner;
        } else {
            tol2 = 0.25 * w->target * w->target;
        }
        const int64_t left = w->maxit - w->iterations;
        if (mode == kRunResume) {
            ctl->beta = ctl->rz_prev != 0.0 ? w->ratio * rz / ctl->rz_prev : 0.0;
        } else {
            ctl->alpha = 0.0;
            ctl->beta = 0.0;
            ctl->pq = 0.0;
            ctl->rz_prev = 0.0;
            ctl->pcur = 0;
        }
        ctl->rz = rz;
        ctl->rr = rr;
        ctl->tol2 = tol2;
        ctl->maxit = left > 1 ? left : 1;
        ctl->iterations = 0;
        ctl->done = 0;
        ctl->ticket = 0;
        w->mode = kRunIterating;
    }
}

}  // namespace amie

// ------------------------------------------------------------------ host side

struct amie_server {
    amie_ctx *ctx = nullptr;        // solve stream
    std::vector<amie_ctx *> adms;   // one context (stream) per admission thread
    cudaStream_t xfer = nullptr;    // result copies of retired solves (beside the batches)
    amie_server_config cfg{};
    bool mixed = true;
    int grid = 0, group = 8;
    int rows_per_cta = 512;   // block rows per CTA of a slot
    bool persistent = false;  // mixed batches as one cooperative launch (kb_persistent)
    uint32_t polls = 0;       // slot-barrier poll limit of kb_persistent
    // test hook (AMIE_SERVER_SHORT_SLOT=k): the k-th request to join gets one CTA
    // fewer in the CTA -> slot table than its descriptor claims, so its first
    // slot barrier in a persistent batch cannot be reached and gives up
    int short_slot_at = 0, n_joined = 0;
    uint64_t n_timeouts = 0;  // persistent batches ended by a barrier that gave up
    amie::DevArray<uint32_t> d_bar;   // per slot barrier counters of kb_persistent
    amie::DevArray<int32_t> d_err;    // barrier timeout flag
    int32_t *h_err = nullptr;         // pinned copy
    uint64_t budget = 0;
    std::atomic<uint64_t> in_use{0};

    struct Req {
        uint64_t ticket;
        // deep copies of the request arrays
        std::vector<uint8_t> kind, moved, enr_type, enr_vertex, bc_kinds;
        std::vector<uint32_t> dof_ptr, dof_ids, gp_ptr, mat, enr_ptr, enr_data, bc_ids;
        std::vector<double> gp, jinv, jinv_gp, cmat, cscale, scale, enr_grad, enr_tip, bc_vals, x0;
        std::vector<int8_t> enr_jump;
        amie_mesh mesh{};
        uint64_t footprint = 0;
        double t_submit = 0, t_admit = 0, t_done = 0;
        amie_topo *topo = nullptr;
        int slot = -1;
        uint32_t gen = 0;   // join number
        double bnorm = 0, rnorm = 0;   // rnorm: the true residual the current inner run was scaled by
        int64_t iterations = 0;
        int refinements = 0;
        amie_status status = AMIE_NOT_READY;
        bool cancelled = false;
        std::vector<double> x;   // result
        double relres = 0;
    };

    std::mutex mu;
    std::condition_variable cv;
    std::deque<Req *> pending;
    std::map<uint64_t, Req *> all;
    uint64_t next_ticket = 1;
    bool running = false, stop_flag = false;
    std::thread worker;                   // the batch loop
    std::vector<std::thread> admitters;   // admissions, each on its own context, overlapping the batch
    cudaMemPool_t pool = nullptr;         // the admission contexts' stream-ordered allocations
    uint32_t n_gen = 0;                   // joins so far
    std::deque<Req *> ready;                     // admitted, waiting to join (under mu)
    int admitting = 0, n_active = 0, n_waiting = 0;   // (under mu) inside admit(), in slots, admitted but not joined

    // batch state
    std::vector<Req *> slot_req;                 // per slot
    amie::DevArray<amie::SlotDesc> d_slots;
    amie::DevArray<amie::PcgCtl> d_ctl;         // per slot
    amie::DevArray<int16_t> d_cta_slot;
    amie::DevArray<double> d_parts;              // pq | rz | rr | spare, grid each
    amie::SlotDesc *h_slots = nullptr;           // pinned
    amie::PcgCtl *h_ctl = nullptr;               // pinned: a joining slot's first control block
    amie::DevArray<amie::SlotRun> d_run;         // per slot: the solve's state (device-side refinement)
    amie::SlotRun *h_run = nullptr;              // pinned: a joining slot's first state
    amie::SlotRun *h_ring = nullptr;             // pinned, 2 x slots: d_run after each of two batches in flight
    cudaEvent_t ring_ev[2] = {nullptr, nullptr};
    int16_t *h_cta_slot = nullptr;               // pinned
    cudaGraphExec_t graph = nullptr;    // batch of 2D slots
    cudaGraphExec_t graph3 = nullptr;   // batch with 3D slots (each kernel holds both strides' bodies)
    int n_active3 = 0;                  // active 3D slots (loop thread)
    std::string error;
    amie_server_stats stats{};   // written by the loop thread under `mu`
};

namespace amie {

inline double now_s()
{
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

template <typename T>
static void copy_vec(std::vector<T> &dst, const T *src, size_t n)
{
    if (src) dst.assign(src, src + n);
    else dst.clear();
}

// Device bytes a request needs: staged element blocks, pattern keys and sort
// scratch, matrix (FP64 + FP32), SELL copies, scatter map, vectors, element data.
static uint64_t request_footprint(const amie_mesh &m)
{
    uint64_t blocks = 0;
    for (uint32_t e = 0; e < m.n_elem; e++) {
        const uint64_t nf = m.dof_ptr[e + 1] - m.dof_ptr[e];
        blocks += nf * nf;
    }
    const uint64_t s2 = (uint64_t)m.stride * m.stride;
    const uint64_t rows = m.ndofmax ? m.ndofmax : 1;
    const uint64_t n = rows * m.stride;
    return blocks * (s2 * 8 + 48) + blocks * (s2 * 12 + 8) + blocks * (s2 * 12 + 16) + n * 8 * 18 +
           (uint64_t)m.n_elem * 64 + (uint64_t)m.gp_ptr[m.n_elem] * 64 + (16u << 20);
}

struct ServerOps {
    static amie_status fail_req(amie_server *srv, amie_server::Req *r, amie_status st)
    {
        std::lock_guard<std::mutex> lk(srv->mu);
        r->status = st;
        r->t_done = now_s();
        srv->cv.notify_all();
        return AMIE_OK;
    }

    static amie_status read_sum_on(cudaStream_t st, const double *dev, int n, double *out)
    {
        std::vector<double> h(n);
        AMIE_CUDA(cudaMemcpyAsync(h.data(), dev, n * sizeof(double), cudaMemcpyDeviceToHost, st));
        AMIE_CUDA(cudaStreamSynchronize(st));
        double s = 0.0;
        for (int i = 0; i < n; i++) s += h[i];
        *out = s;
        return AMIE_OK;
    }

    // Upload + pattern + element matrices + gather + elimination on the admission stream,
    // then the initial FP64 residual.
    static amie_status admit(amie_server *srv, amie_server::Req *r, amie_ctx *adm)
    {
        amie_topo *t = nullptr;
        AMIE_TRY(amie_topology_build(adm, &r->mesh, &t));
        r->topo = t;
        if (t->s != 2 && (t->s != 3 || srv->persistent)) {
            set_error(srv->persistent ? "the persistent batch takes 2D meshes only"
                                      : "the server batches 2D and 3D elasticity meshes only");
            return AMIE_BAD_INPUT;
        }
        AMIE_TRY(amie_assemble(t));
        const uint8_t *kinds = r->bc_kinds.empty() ? nullptr : r->bc_kinds.data();
        AMIE_TRY(amie_apply_dirichlet(t, (uint32_t)r->bc_ids.size(), r->bc_ids.data(), r->bc_vals.data(), kinds,
                                      nullptr));
        SolverState *s = nullptr;
        AMIE_TRY(ensure_state(t, srv->mixed, &s));
        if (srv->mixed) AMIE_TRY(finalize_matrix_async(t, true));
        AMIE_TRY(ensure_sell(t, !srv->mixed, srv->mixed));
        AMIE_TRY(ensure_sell_partition(t, ctas_for(srv, t->n_rows)));   // the slot's CTA count
        cudaStream_t st = adm->stream;
        if (!r->x0.empty() && r->x0.size() == t->n)
            AMIE_CUDA(cudaMemcpyAsync(t->x.p, r->x0.data(), t->n * 8, cudaMemcpyHostToDevice, st));
        else
            AMIE_CUDA(cudaMemsetAsync(t->x.p, 0, t->n * 8, st));
        k_norm2_parts<<<s->grid, kVecThreads, 0, st>>>(t->n, t->rhs.p, s->parts.p);
        AMIE_LAUNCHED();
        double bb = 0.0, rr = 0.0;
        AMIE_TRY(read_sum_on(st, s->parts.p, s->grid, &bb));
        launch_spmv<double>(t, s->grid, bsr64(t), t->x.p, t->rhs.p, t->r.p, s->parts.p + 3 * s->stride, st);
        AMIE_TRY(read_sum_on(st, s->parts.p + 3 * s->stride, s->grid, &rr));
        r->bnorm = std::sqrt(bb);
        r->rnorm = std::sqrt(rr);
        return AMIE_OK;
    }

    // CTA allocator over the batch grid: first fit of `count` contiguous CTAs.
    static int alloc_ctas(amie_server *srv, int count)
    {
        int run = 0;
        for (int c = 0; c < srv->grid; c++) {
            run = srv->h_cta_slot[c] < 0 ? run + 1 : 0;
            if (run == count) return c - count + 1;
        }
        return -1;
    }

    // CTAs of a slot: a function of its row count only (so a solve is the same
    // alone and in any mix), srv->rows_per_cta block rows each, at most 128.
    static int ctas_for(const amie_server *srv, uint64_t n_rows)
    {
        const uint64_t per = (uint64_t)srv->rows_per_cta;
        return (int)std::max<uint64_t>(1, std::min<uint64_t>(128, (n_rows + per - 1) / per));
    }

    static void fill_desc(amie_server *srv, int slot, amie_topo *t, int c0, int c1)
    {
        SlotDesc &d = srv->h_slots[slot];
        const uint32_t *first = t->sell_cta_first.at(c1 - c0).p;
        d.A32 = sell_of<float>(t);
        d.A32.cta_first = first;
        d.A64 = sell_of<double>(t);
        d.A64.cta_first = first;
        d.v32 = vecs_of<float>(t);
        d.v64 = vecs_of<double>(t);
        d.v64.p2 = nullptr;   // FP64 batches keep the direction kernel
        const int g = srv->grid;
        double *pp = srv->d_parts.p;
        d.parts = PcgParts{pp + c0, pp + g + c0, pp + 2 * g + c0, pp + 3 * g + c0};
        d.ctl = srv->d_ctl.p + slot;
        d.run = srv->d_run.p + slot;
        d.rhs = t->rhs.p;
        d.n = t->n;
        d.c0 = c0;
        d.c1 = c1;
        d.active = 1;
        d.mixed = srv->mixed ? 1 : 0;
        d.s = t->s;
    }

    // FP32 residual reduction between two FP64 residual replacements of a mixed slot.
    static constexpr double kInnerReduction = 0.1;

    // Start (or restart, with a fresh search direction) the inner run of a slot
    // from its FP64 residual r64 (norm rnorm).
    static amie_status start_inner(amie_server *srv, int slot, amie_server::Req *r)
    {
        cudaStream_t st = srv->ctx->stream;
        amie_topo *t = r->topo;
        const SlotDesc &d = srv->h_slots[slot];
        const int nc = d.c1 - d.c0;
        PcgCtl c{};
        const int64_t maxit = std::max<int64_t>(1000, (int64_t)t->n);
        c.maxit = std::max<int64_t>(1, maxit - r->iterations);
        if (srv->mixed) {
            const double need = kMixedLastTarget * srv->cfg.rtol * r->bnorm / r->rnorm;
            const double inner = std::min(0.5, std::max(kInnerReduction, need));
            c.tol2 = inner * inner;
        } else {
            const double target = srv->cfg.rtol * r->bnorm;
            c.tol2 = 0.25 * target * target;
        }
        srv->h_ctl[slot] = c;
        AMIE_CUDA(cudaMemcpyAsync(srv->d_ctl.p + slot, srv->h_ctl + slot, sizeof(PcgCtl), cudaMemcpyHostToDevice, st));
        AMIE_CUDA(cudaMemcpyAsync(srv->d_slots.p + slot, srv->h_slots + slot, sizeof(SlotDesc), cudaMemcpyHostToDevice, st));
        if (srv->mixed) {
            k_scale_to_f32<<<nc, kVecThreads, 0, st>>>(t->n, t->r.p, 1.0 / r->rnorm, t->r32.p, t->d32.p);
            k_pcg_start<float><<<nc, kVecThreads, 0, st>>>(d.v32, t->n, d.parts, d.ctl);
        } else {
            k_pcg_start<double><<<nc, kVecThreads, 0, st>>>(d.v64, t->n, d.parts, d.ctl);
        }
        g_launches += srv->mixed ? 2 : 1;
        // no synchronisation: the slot's pinned h_ctl / h_slots / h_run entries are
        // written again only when it is retired (which synchronises the stream)
        AMIE_CUDA(cudaGetLastError());
        return AMIE_OK;
    }

    static amie_status join(amie_server *srv, amie_server::Req *r)
    {
        int slot = -1;
        for (size_t i = 0; i < srv->slot_req.size(); i++)
            if (!srv->slot_req[i]) { slot = (int)i; break; }
        if (slot < 0) return AMIE_NOT_READY;
        const int count = ctas_for(srv, r->topo->n_rows);
        const int c0 = alloc_ctas(srv, count);
        if (c0 < 0) return AMIE_NOT_READY;
        for (int c = c0; c < c0 + count; c++) srv->h_cta_slot[c] = (int16_t)slot;
        if (srv->short_slot_at > 0 && ++srv->n_joined == srv->short_slot_at && count > 1)
            srv->h_cta_slot[c0 + count - 1] = -1;   // test hook: one CTA of the slot is not launched
        srv->slot_req[slot] = r;
        r->slot = slot;
        if (r->topo->s == 3) srv->n_active3++;
        {
            std::lock_guard<std::mutex> lk(srv->mu);
            srv->n_active++;
        }
        fill_desc(srv, slot, r->topo, c0, c0 + count);
        cudaStream_t st = srv->ctx->stream;
        AMIE_CUDA(cudaMemcpyAsync(srv->d_cta_slot.p, srv->h_cta_slot, srv->grid * sizeof(int16_t), cudaMemcpyHostToDevice, st));
        if (r->rnorm <= srv->cfg.rtol * r->bnorm || r->bnorm == 0.0) {   // already converged (warm start)
            srv->h_slots[slot].active = 0;
            AMIE_CUDA(cudaMemcpyAsync(srv->d_slots.p + slot, srv->h_slots + slot, sizeof(SlotDesc), cudaMemcpyHostToDevice, st));
            AMIE_CUDA(cudaStreamSynchronize(st));
            return retire(srv, r, AMIE_OK);
        }
        SlotRun &run = srv->h_run[slot];
        run = SlotRun{};
        r->gen = ++srv->n_gen;
        run.gen = r->gen;
        run.bnorm = r->bnorm;
        run.target = srv->cfg.rtol * r->bnorm;
        run.rnorm = r->rnorm;
        run.maxit = std::max<int64_t>(1000, (int64_t)r->topo->n);
        run.status = AMIE_NOT_READY;
        run.mode = kRunIterating;
        AMIE_CUDA(cudaMemcpyAsync(srv->d_run.p + slot, srv->h_run + slot, sizeof(SlotRun), cudaMemcpyHostToDevice, st));
        return start_inner(srv, slot, r);
    }

    // Ends a request.  Its result is copied on the transfer stream (the solve
    // stream may hold a batch in flight, which skips the finished slot); the
    // slot's descriptor and CTAs are released by copies queued on the solve
    // stream (applied before the next batch), and so is the topology's memory
    // (stream-ordered frees into the server's pool, after that batch).
    static amie_status retire(amie_server *srv, amie_server::Req *r, amie_status result)
    {
        cudaStream_t st = srv->ctx->stream;
        amie_topo *t = r->topo;
        if (t && result != AMIE_CANCELLED) {
            r->x.resize(t->n);
            AMIE_CUDA(cudaMemcpyAsync(r->x.data(), t->x.p, t->n * 8, cudaMemcpyDeviceToHost, srv->xfer));
            AMIE_CUDA(cudaStreamSynchronize(srv->xfer));
        }
        if (r->slot >= 0) {
            const int slot = r->slot;
            for (int c = 0; c < srv->grid; c++)
                if (srv->h_cta_slot[c] == slot) srv->h_cta_slot[c] = -1;
            srv->h_slots[slot].active = 0;
            // the pinned sources are rewritten only by later joins and retirements
            // of the loop thread, whose copies follow these on the same stream
            AMIE_CUDA(cudaMemcpyAsync(srv->d_slots.p + slot, srv->h_slots + slot, sizeof(SlotDesc), cudaMemcpyHostToDevice, st));
            AMIE_CUDA(cudaMemcpyAsync(srv->d_cta_slot.p, srv->h_cta_slot, srv->grid * sizeof(int16_t), cudaMemcpyHostToDevice, st));
            srv->slot_req[slot] = nullptr;
            r->slot = -1;
            if (t && t->s == 3) srv->n_active3--;
            std::lock_guard<std::mutex> lk(srv->mu);
            srv->n_active--;
        }
        if (t) {
            set_free_stream(st);
            release_topology(t);
            set_free_stream(nullptr);
            r->topo = nullptr;
        }
        srv->in_use -= r->footprint;
        std::lock_guard<std::mutex> lk(srv->mu);
        r->status = result;
        r->relres = r->bnorm > 0 ? r->rnorm / r->bnorm : 0.0;
        r->t_done = now_s();
        srv->cv.notify_all();
        return AMIE_OK;
    }

    // Kernels that end every batch: the FP64 residual replacement and the
    // decision for the slots whose inner run stopped (device-side refinement).
    static void launch_refine(amie_server *srv, cudaStream_t st)
    {
        const SlotDesc *sl = srv->d_slots.p;
        const int16_t *cs = srv->d_cta_slot.p;
        const int g = srv->grid;
        if (srv->mixed) kb_accumulate<<<g, kVecThreads, 0, st>>>(sl, cs);
        kb_residual<<<g, kVecThreads, 0, st>>>(sl, cs);
        kb_restart<<<g, kVecThreads, 0, st>>>(sl, cs, kInnerReduction, kMixedLastTarget);
    }

    static int refine_kernels(const amie_server *srv) { return srv->mixed ? 3 : 2; }

    // Requests whose solve a batch ended (final SlotRun status in the batch's
    // copy `runs`, of the request's own join): retired.
    static amie_status collect(amie_server *srv, const SlotRun *runs)
    {
        for (size_t i = 0; i < srv->slot_req.size(); i++) {
            amie_server::Req *r = srv->slot_req[i];
            if (!r) continue;
            const SlotRun &run = runs[i];
            if (run.gen != r->gen || run.status == AMIE_NOT_READY) continue;
            r->iterations = run.iterations;
            r->refinements = run.refinements;
            r->rnorm = run.rnorm;
            AMIE_TRY(retire(srv, r, (amie_status)run.status));
        }
        return AMIE_OK;
    }

    // The batch graphs: `iters_per_launch` PCG iterations over every active slot,
    // then the refinement kernels; SMAX = 2 for batches of 2D slots, 3 when 3D
    // slots are active.
    template <int SMAX>
    static amie_status capture_one(amie_server *srv, cudaGraphExec_t *out)
    {
        cudaStream_t st = srv->ctx->stream;
        const SlotDesc *sl = srv->d_slots.p;
        const int16_t *cs = srv->d_cta_slot.p;
        const int g = srv->grid;
        cudaGraph_t graph;
        AMIE_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        for (int it = 0; it < srv->cfg.iters_per_launch; it++) {
            const bool pdl = it > 0;   // the first kernel follows the host's updates in plain stream order
            if (srv->mixed) {
                launch_k(pdl, kb_sell_dir<float, SMAX>, g, 0, st, sl, cs);
                launch_k(true, kb_update<float>, g, 0, st, sl, cs);
            } else {
                launch_k(pdl, kb_sell_pq<double, SMAX>, g, 0, st, sl, cs);
                launch_k(true, kb_update<double>, g, 0, st, sl, cs);
                launch_k(true, kb_direction<double>, g, 0, st, sl, cs);
            }
        }
        launch_refine(srv, st);
        AMIE_CUDA(cudaStreamEndCapture(st, &graph));
        cudaError_t e = cudaGraphInstantiate(out, graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) {
            *out = nullptr;
            set_error("cudaGraphInstantiate: %s", cudaGetErrorString(e));
            return AMIE_CUDA_ERROR;
        }
        return AMIE_OK;
    }

    static amie_status capture(amie_server *srv)
    {
        AMIE_TRY(capture_one<2>(srv, &srv->graph));
        return capture_one<3>(srv, &srv->graph3);
    }

    static bool any_active(amie_server *srv)
    {
        for (auto *r : srv->slot_req)
            if (r) return true;
        return false;
    }

    // Admission thread: takes pending requests while slots allow and admits
    // them (topology, assembly, elimination, SELL copy, first residual) on the
    // admission context, overlapping the batch loop; hands them over in `ready`.
    static void admit_loop(amie_server *srv, amie_ctx *adm)
    {
        cudaSetDevice(srv->ctx->device);
        while (true) {
            amie_server::Req *r = nullptr;
            {
                std::unique_lock<std::mutex> lk(srv->mu);
                while (true) {
                    if (srv->stop_flag && srv->pending.empty()) return;
                    const int used = srv->n_active + srv->n_waiting + (int)srv->ready.size() + srv->admitting;
                    if (!srv->pending.empty() && used < (int)srv->slot_req.size()) {
                        amie_server::Req *c = srv->pending.front();
                        if (c->cancelled) {
                            srv->pending.pop_front();
                            c->status = AMIE_CANCELLED;
                            c->t_done = now_s();
                            srv->cv.notify_all();
                            continue;
                        }
                        if (c->footprint > srv->budget) {   // can never fit
                            srv->pending.pop_front();
                            c->status = AMIE_OOM;
                            c->t_done = now_s();
                            srv->cv.notify_all();
                            continue;
                        }
                        if (srv->in_use + c->footprint <= srv->budget) {
                            srv->pending.pop_front();
                            srv->in_use += c->footprint;
                            srv->admitting++;
                            r = c;
                            break;
                        }
                    }
                    srv->cv.wait_for(lk, std::chrono::milliseconds(2));
                }
            }
            const double ta = now_s();
            r->t_admit = ta;
            const amie_status st = admit(srv, r, adm);
            if (st != AMIE_OK && r->topo) {
                amie_topology_destroy(r->topo);
                r->topo = nullptr;
            }
            std::lock_guard<std::mutex> lk(srv->mu);
            srv->admitting--;
            srv->stats.admit_s += now_s() - ta;
            srv->stats.admitted++;
            if (st != AMIE_OK) {
                srv->in_use -= r->footprint;
                r->status = st;
                r->t_done = now_s();
            } else {
                srv->ready.push_back(r);
            }
            srv->cv.notify_all();
        }
    }

    // One batch on the solve stream (graph, or cooperative launch + refinement),
    // then the copy of every slot's SlotRun into ring buffer `k` and its event.
    static bool launch_batch(amie_server *srv, int k)
    {
        cudaStream_t st = srv->ctx->stream;
        if (srv->persistent) {
            cudaMemsetAsync(srv->d_bar.p, 0, srv->slot_req.size() * sizeof(uint32_t), st);
            const SlotDesc *sl = srv->d_slots.p;
            const int16_t *cs = srv->d_cta_slot.p;
            int iters = srv->cfg.iters_per_launch;
            uint32_t *bar = srv->d_bar.p;
            int32_t *err = srv->d_err.p;
            uint32_t polls = srv->polls;
            void *args[] = {(void *)&sl, (void *)&cs, (void *)&iters, (void *)&bar, (void *)&err, (void *)&polls};
            const cudaError_t le = cudaLaunchCooperativeKernel((const void *)kb_persistent<float>, dim3(srv->grid),
                                                               dim3(kVecThreads), args, 0, st);
            if (le != cudaSuccess) {   // nothing ran: report and stop rather than wait on stale blocks
                srv->error = std::string("cooperative launch: ") + cudaGetErrorString(le);
                std::lock_guard<std::mutex> lk(srv->mu);
                for (auto &kv : srv->all)
                    if (kv.second->status == AMIE_NOT_READY) {
                        kv.second->status = AMIE_CUDA_ERROR;
                        kv.second->t_done = now_s();
                    }
                srv->stop_flag = true;
                srv->cv.notify_all();
                return false;
            }
            g_launches += 1;
            cudaMemcpyAsync(srv->h_err, srv->d_err.p, sizeof(int32_t), cudaMemcpyDeviceToHost, st);
            launch_refine(srv, st);
        } else {
            cudaGraphLaunch(srv->n_active3 > 0 ? srv->graph3 : srv->graph, st);
            g_launches += (srv->mixed ? 2 : 3) * srv->cfg.iters_per_launch;
        }
        g_launches += refine_kernels(srv);
        const size_t ns = srv->slot_req.size();
        cudaMemcpyAsync(srv->h_ring + (size_t)k * ns, srv->d_run.p, ns * sizeof(SlotRun), cudaMemcpyDeviceToHost, st);
        cudaEventRecord(srv->ring_ev[k], st);
        return true;
    }

    // The batch loop.  Two batches stay in flight (one with the persistent
    // kernel): while batch k + 1 runs, the host reads batch k's SlotRun copy,
    // retires the solves it finished (those slots do no work in batch k + 1)
    // and joins admitted requests, whose start kernels and table updates queue
    // behind batch k + 1.
    static void loop(amie_server *srv)
    {
        cudaSetDevice(srv->ctx->device);
        std::vector<amie_server::Req *> admitted;   // handed over, not yet joined
        const int depth = srv->persistent ? 1 : 2;
        int64_t launched = 0, done = 0;             // batches launched / processed
        while (true) {
            const double t_round = now_s();
            // 1. keep `depth` batches in flight while any slot is active
            if (any_active(srv) && launched - done < depth) {
                if (!launch_batch(srv, (int)(launched & 1))) break;
                launched++;
                if (launched - done < depth) continue;   // fill the pipeline first
            }
            // 2. requests the admission threads have finished
            {
                std::unique_lock<std::mutex> lk(srv->mu);
                if (launched == done && srv->ready.empty() && admitted.empty()) {
                    if (srv->stop_flag && srv->pending.empty() && srv->admitting == 0) break;
                    srv->cv.wait_for(lk, std::chrono::milliseconds(2));
                    continue;
                }
                while (!srv->ready.empty()) {
                    admitted.push_back(srv->ready.front());
                    srv->ready.pop_front();
                }
                srv->n_waiting = (int)admitted.size();
            }
            const double tw = now_s();
            // 3. results of the oldest batch in flight
            double t_waited = tw, t_adv = 0.0;
            if (launched > done) {
                const int k = (int)(done & 1);
                cudaEventSynchronize(srv->ring_ev[k]);
                done++;
                t_waited = now_s();
                if (srv->persistent && *srv->h_err) {
                    // a slot barrier gave up and the launch ended: the batch's slots are in
                    // an unknown state, so their requests end with AMIE_TIMEOUT; the flag is
                    // cleared and the server goes on with the next requests
                    srv->n_timeouts++;
                    for (size_t i = 0; i < srv->slot_req.size(); i++)
                        if (srv->slot_req[i]) retire(srv, srv->slot_req[i], AMIE_TIMEOUT);
                    *srv->h_err = 0;
                    cudaMemsetAsync(srv->d_err.p, 0, sizeof(int32_t), srv->ctx->stream);
                }
                for (size_t i = 0; i < srv->slot_req.size(); i++) {
                    amie_server::Req *r = srv->slot_req[i];
                    if (r && r->cancelled) retire(srv, r, AMIE_CANCELLED);
                }
                collect(srv, srv->h_ring + (size_t)k * srv->slot_req.size());
                t_adv = now_s() - t_waited;
            }
            const double tj = now_s();
            // 4. join admitted requests
            std::vector<amie_server::Req *> waiting;
            for (auto *r : admitted) {
                if (r->cancelled) {
                    fail_req(srv, r, AMIE_CANCELLED);
                    continue;
                }
                amie_status st = join(srv, r);
                if (st == AMIE_NOT_READY) waiting.push_back(r);
                else if (st != AMIE_OK) fail_req(srv, r, st);
            }
            admitted.swap(waiting);
            {
                const double te = now_s();
                std::lock_guard<std::mutex> lk(srv->mu);
                srv->n_waiting = (int)admitted.size();
                srv->stats.wait_s += t_waited - tw;
                srv->stats.advance_s += t_adv;
                srv->stats.join_s += te - tj;
                srv->stats.loop_s += te - t_round;
                if (t_waited > tw) srv->stats.batches++;
                srv->cv.notify_all();
            }
            cudaError_t e = cudaGetLastError();
            if (e != cudaSuccess) {
                srv->error = cudaGetErrorString(e);
                std::lock_guard<std::mutex> lk(srv->mu);
                for (auto &kv : srv->all)
                    if (kv.second->status == AMIE_NOT_READY) kv.second->status = AMIE_CUDA_ERROR;
                srv->cv.notify_all();
                break;
            }
        }
        // nothing of this thread's may remain in flight when it ends
        cudaStreamSynchronize(srv->ctx->stream);
    }
};

}  // namespace amie

extern "C" amie_status amie_server_start(amie_ctx *ctx, const amie_server_config *cfg, amie_server **out)
{
    using namespace amie;
    if (!ctx || !out) return AMIE_BAD_INPUT;
    *out = nullptr;
    AMIE_CUDA(cudaSetDevice(ctx->device));
    amie_server *srv = new amie_server();
    srv->ctx = ctx;
    amie_server_config c{AMIE_SOLVER_PCG_MIXED, 1e-10, 0, 256, kBatchIters};
    if (cfg) c = *cfg;
    if (c.rtol <= 0) c.rtol = 1e-10;
    if (c.max_slots <= 0) c.max_slots = 256;
    c.max_slots = std::min(c.max_slots, 1024);
    if (c.iters_per_launch <= 0) c.iters_per_launch = kBatchIters;
    c.iters_per_launch = std::min(c.iters_per_launch, 256);
    if (c.solver != AMIE_SOLVER_PCG_MIXED && c.solver != AMIE_SOLVER_PCG_FP64) {
        delete srv;
        set_error("server solver must be PCG_FP64 or PCG_MIXED");
        return AMIE_BAD_INPUT;
    }
    srv->cfg = c;
    srv->mixed = c.solver == AMIE_SOLVER_PCG_MIXED;
    size_t free_b = 0, total_b = 0;
    cudaMemGetInfo(&free_b, &total_b);
    srv->budget = c.hbm_budget_bytes ? c.hbm_budget_bytes : (uint64_t)(0.9 * free_b);
    // the batch grid: the CTAs of the batch kernels that fit on the GPU at once
    // (a larger grid would run in waves), and at least one CTA per slot
    {
        int occ = 8;
        auto lower = [&](const void *f) {
            int k = 0;
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&k, f, kVecThreads, 0);
            occ = std::min(occ, std::max(1, k));
        };
        if (srv->mixed) {
            lower((const void *)kb_sell_dir<float>);
            lower((const void *)kb_update<float>);
        } else {
            lower((const void *)kb_sell_pq<double>);
            lower((const void *)kb_update<double>);
            lower((const void *)kb_direction<double>);
        }
        int coop = 0;
        cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, ctx->device);
        // opt-in (AMIE_SERVER_PERSISTENT=1): one cooperative launch per batch.  Measured
        // slower than the graph of batched kernels (145 vs 174 solves/s saturated, same
        // 16 ms for a lone request): small slots are bound by dependent memory latency,
        // not by launches, and the kernel's 128 registers leave 2 CTAs per SM.
        srv->persistent = false;
        if (const char *e = std::getenv("AMIE_SERVER_PERSISTENT"))
            srv->persistent = srv->mixed && coop != 0 && std::atoi(e) != 0;
        if (srv->persistent) {
            int k = 0;
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&k, (const void *)kb_persistent<float>, kVecThreads, 0);
            occ = std::max(1, std::min(occ, k));
        }
        // a cooperative launch needs every CTA resident: the grid cannot exceed occ per SM
        srv->grid = srv->persistent ? ctx->num_sms * occ : std::max(ctx->num_sms * occ, c.max_slots);
        // tuning override for measurements: AMIE_SERVER_ROWS_PER_CTA
        if (const char *e = std::getenv("AMIE_SERVER_ROWS_PER_CTA")) {
            const int v = std::atoi(e);
            if (v >= 32 && v <= (1 << 20)) srv->rows_per_cta = v;
        }
        srv->polls = c.barrier_polls ? c.barrier_polls : kBarrierPolls;
        if (const char *e = std::getenv("AMIE_SERVER_SHORT_SLOT")) srv->short_slot_at = std::max(0, std::atoi(e));
    }
    // admission threads (AMIE_SERVER_ADMITTERS, 1-8, default 2), each on its own context
    // (4,096-request mix at 200/s: 1.5 ms of admission per request; one thread and
    // three gave the same latencies)
    int n_adm = 2;
    if (const char *e = std::getenv("AMIE_SERVER_ADMITTERS")) n_adm = std::max(1, std::min(8, std::atoi(e)));
    amie_config ac{ctx->device, 0, 0};
    amie_status rc = AMIE_OK;
    auto fail = [&](amie_status s) {
        for (amie_ctx *a : srv->adms) amie_ctx_destroy(a);
        if (srv->pool) cudaMemPoolDestroy(srv->pool);
        if (srv->xfer) cudaStreamDestroy(srv->xfer);
        for (cudaEvent_t e : srv->ring_ev)
            if (e) cudaEventDestroy(e);
        if (srv->h_slots) cudaFreeHost(srv->h_slots);
        if (srv->h_ctl) cudaFreeHost(srv->h_ctl);
        if (srv->h_err) cudaFreeHost(srv->h_err);
        if (srv->h_run) cudaFreeHost(srv->h_run);
        if (srv->h_ring) cudaFreeHost(srv->h_ring);
        if (srv->h_cta_slot) cudaFreeHost(srv->h_cta_slot);
        delete srv;
        return s;
    };
    {
        // requests' memory comes from a pool of the server's: allocated stream-ordered
        // on an admission stream, freed stream-ordered on the solve stream at retirement
        // (cudaFree would wait for the batch in flight); kept cached, and a free is
        // reused only once it has completed (no cross-stream dependencies inserted)
        cudaMemPoolProps props = {};
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = ctx->device;
        if (cudaMemPoolCreate(&srv->pool, &props) != cudaSuccess) return fail(AMIE_CUDA_ERROR);
        uint64_t keep = UINT64_MAX;
        int no = 0;
        cudaMemPoolSetAttribute(srv->pool, cudaMemPoolAttrReleaseThreshold, &keep);
        cudaMemPoolSetAttribute(srv->pool, cudaMemPoolReuseAllowInternalDependencies, &no);
    }
    for (int i = 0; i < n_adm; i++) {
        amie_ctx *a = nullptr;
        if ((rc = amie_ctx_create(&ac, &a)) != AMIE_OK) return fail(rc);
        a->pool = srv->pool;
        srv->adms.push_back(a);
    }
    if (cudaStreamCreateWithFlags(&srv->xfer, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&srv->ring_ev[0], cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&srv->ring_ev[1], cudaEventDisableTiming) != cudaSuccess)
        return fail(AMIE_CUDA_ERROR);
    srv->slot_req.assign(c.max_slots, nullptr);
    if ((rc = srv->d_slots.alloc(ctx, c.max_slots)) || (rc = srv->d_ctl.alloc(ctx, c.max_slots)) ||
        (rc = srv->d_run.alloc(ctx, c.max_slots)) ||
        (rc = srv->d_bar.alloc(ctx, c.max_slots)) || (rc = srv->d_err.alloc(ctx, 1)) ||
        (rc = srv->d_cta_slot.alloc(ctx, srv->grid)) || (rc = srv->d_parts.alloc(ctx, 4 * (size_t)srv->grid)))
        return fail(rc);
    if (cudaMallocHost((void **)&srv->h_slots, c.max_slots * sizeof(SlotDesc)) != cudaSuccess ||
        cudaMallocHost((void **)&srv->h_ctl, c.max_slots * sizeof(PcgCtl)) != cudaSuccess ||
        cudaMallocHost((void **)&srv->h_err, sizeof(int32_t)) != cudaSuccess ||
        cudaMallocHost((void **)&srv->h_run, c.max_slots * sizeof(SlotRun)) != cudaSuccess ||
        cudaMallocHost((void **)&srv->h_ring, 2 * (size_t)c.max_slots * sizeof(SlotRun)) != cudaSuccess ||
        cudaMallocHost((void **)&srv->h_cta_slot, srv->grid * sizeof(int16_t)) != cudaSuccess)
        return fail(AMIE_OOM);
    std::memset(srv->h_slots, 0, c.max_slots * sizeof(SlotDesc));
    std::memset(srv->h_ctl, 0, c.max_slots * sizeof(PcgCtl));
    std::memset(srv->h_run, 0, c.max_slots * sizeof(SlotRun));
    *srv->h_err = 0;
    cudaMemsetAsync(srv->d_err.p, 0, sizeof(int32_t), ctx->stream);
    for (int i = 0; i < srv->grid; i++) srv->h_cta_slot[i] = -1;
    cudaStream_t st = ctx->stream;
    cudaMemcpyAsync(srv->d_slots.p, srv->h_slots, c.max_slots * sizeof(SlotDesc), cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(srv->d_ctl.p, srv->h_ctl, c.max_slots * sizeof(PcgCtl), cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(srv->d_run.p, srv->h_run, c.max_slots * sizeof(SlotRun), cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(srv->d_cta_slot.p, srv->h_cta_slot, srv->grid * sizeof(int16_t), cudaMemcpyHostToDevice, st);
    cudaMemsetAsync(srv->d_parts.p, 0, 4 * (size_t)srv->grid * 8, st);
    if (cudaStreamSynchronize(st) != cudaSuccess) return fail(AMIE_CUDA_ERROR);
    if ((rc = ServerOps::capture(srv)) != AMIE_OK) return fail(rc);
    srv->running = true;
    srv->worker = std::thread(ServerOps::loop, srv);
    for (amie_ctx *a : srv->adms) srv->admitters.emplace_back(ServerOps::admit_loop, srv, a);
    *out = srv;
    return AMIE_OK;
}

extern "C" amie_status amie_submit(amie_server *srv, const amie_request *req, uint64_t *ticket)
{
    using namespace amie;
    if (!srv || !req || !req->mesh || !ticket) return AMIE_BAD_INPUT;
    const amie_mesh &m = *req->mesh;
    if (m.n_elem == 0 || !m.dof_ptr || !m.kind || !m.gp_ptr) return AMIE_BAD_INPUT;
    auto *r = new amie_server::Req();
    const uint32_t E = m.n_elem;
    const uint64_t ngp = m.gp_ptr[E];
    const uint32_t nenr = m.enr_ptr ? m.enr_ptr[E] : 0;
    const int d = m.dim;
    const int nv = d == 2 ? 3 : 6;
    copy_vec(r->kind, m.kind, E);
    copy_vec(r->dof_ptr, m.dof_ptr, E + 1);
    copy_vec(r->dof_ids, m.dof_ids, m.dof_ptr[E]);
    copy_vec(r->gp_ptr, m.gp_ptr, E + 1);
    copy_vec(r->gp, m.gp, ngp * (d + 1));
    copy_vec(r->jinv, m.jinv, (size_t)E * d * d);
    copy_vec(r->moved, m.moved, m.moved ? E : 0);
    copy_vec(r->jinv_gp, m.jinv_gp, m.jinv_gp ? ngp * d * d : 0);
    copy_vec(r->mat, m.mat, E);
    copy_vec(r->cmat, m.cmat_table, (size_t)m.n_mat * nv * nv);
    copy_vec(r->cscale, m.cscale, m.cscale ? E : 0);
    copy_vec(r->scale, m.scale, m.scale ? E : 0);
    if (m.enr_ptr) {
        copy_vec(r->enr_ptr, m.enr_ptr, E + 1);
        copy_vec(r->enr_type, m.enr_type, nenr);
        copy_vec(r->enr_vertex, m.enr_vertex, nenr);
        copy_vec(r->enr_data, m.enr_data, nenr);
        copy_vec(r->enr_jump, m.enr_jump, m.enr_jump ? m.n_enr_gp : 0);
        copy_vec(r->enr_grad, m.enr_grad, m.enr_grad ? m.n_enr_gp * d : 0);
        copy_vec(r->enr_tip, m.enr_tip, m.enr_tip ? (size_t)m.n_enr_tip * 8 : 0);
    }
    copy_vec(r->bc_ids, req->bc_ids, req->n_bc);
    copy_vec(r->bc_vals, req->bc_values, req->n_bc);
    copy_vec(r->bc_kinds, req->bc_kinds, req->bc_kinds ? req->n_bc : 0);
    r->mesh = m;
    r->mesh.kind = r->kind.data();
    r->mesh.dof_ptr = r->dof_ptr.data();
    r->mesh.dof_ids = r->dof_ids.data();
    r->mesh.gp_ptr = r->gp_ptr.data();
    r->mesh.gp = r->gp.empty() ? nullptr : r->gp.data();
    r->mesh.jinv = r->jinv.data();
    r->mesh.moved = r->moved.empty() ? nullptr : r->moved.data();
    r->mesh.jinv_gp = r->jinv_gp.empty() ? nullptr : r->jinv_gp.data();
    r->mesh.mat = r->mat.data();
    r->mesh.cmat_table = r->cmat.data();
    r->mesh.cscale = r->cscale.empty() ? nullptr : r->cscale.data();
    r->mesh.scale = r->scale.empty() ? nullptr : r->scale.data();
    if (m.enr_ptr) {
        r->mesh.enr_ptr = r->enr_ptr.data();
        r->mesh.enr_type = r->enr_type.data();
        r->mesh.enr_vertex = r->enr_vertex.data();
        r->mesh.enr_data = r->enr_data.data();
        r->mesh.enr_jump = r->enr_jump.empty() ? nullptr : r->enr_jump.data();
        r->mesh.enr_grad = r->enr_grad.empty() ? nullptr : r->enr_grad.data();
        r->mesh.enr_tip = r->enr_tip.empty() ? nullptr : r->enr_tip.data();
    }
    uint32_t max_id = 0;
    for (uint32_t k : r->dof_ids) max_id = std::max(max_id, k);
    if (!r->mesh.ndofmax) r->mesh.ndofmax = max_id + 1;
    if (req->x0) r->x0.assign(req->x0, req->x0 + (size_t)std::max(r->mesh.ndofmax, max_id + 1) * m.stride);
    r->footprint = request_footprint(r->mesh);
    r->t_submit = now_s();
    std::lock_guard<std::mutex> lk(srv->mu);
    r->ticket = srv->next_ticket++;
    srv->all[r->ticket] = r;
    srv->pending.push_back(r);
    srv->cv.notify_all();
    *ticket = r->ticket;
    return AMIE_OK;
}

extern "C" amie_status amie_poll(amie_server *srv, uint64_t ticket, amie_result *res, double *x)
{
    if (!srv) return AMIE_BAD_INPUT;
    std::lock_guard<std::mutex> lk(srv->mu);
    auto it = srv->all.find(ticket);
    if (it == srv->all.end()) return AMIE_BAD_INPUT;
    amie_server::Req *r = it->second;
    if (r->status == AMIE_NOT_READY) return AMIE_NOT_READY;
    if (res) {
        res->status = r->status;
        res->iterations = r->iterations;
        res->relres = r->relres;
        res->latency_s = r->t_done - r->t_submit;
        res->queue_s = (r->t_admit > 0 ? r->t_admit : r->t_done) - r->t_submit;
        res->n = r->x.size();
    }
    if (x && !r->x.empty()) std::memcpy(x, r->x.data(), r->x.size() * sizeof(double));
    return r->status == AMIE_CANCELLED ? AMIE_CANCELLED : AMIE_OK;
}

extern "C" amie_status amie_cancel(amie_server *srv, uint64_t ticket)
{
    if (!srv) return AMIE_BAD_INPUT;
    std::lock_guard<std::mutex> lk(srv->mu);
    auto it = srv->all.find(ticket);
    if (it == srv->all.end()) return AMIE_BAD_INPUT;
    it->second->cancelled = true;
    srv->cv.notify_all();
    return AMIE_OK;
}

extern "C" amie_status amie_server_drain(amie_server *srv, double timeout_s)
{
    if (!srv) return AMIE_BAD_INPUT;
    const double t_end = amie::now_s() + (timeout_s > 0 ? timeout_s : 1e30);
    std::unique_lock<std::mutex> lk(srv->mu);
    while (true) {
        bool busy = false;
        for (auto &kv : srv->all)
            if (kv.second->status == AMIE_NOT_READY) { busy = true; break; }
        if (!busy) return AMIE_OK;
        if (amie::now_s() >= t_end) return AMIE_TIMEOUT;
        srv->cv.wait_for(lk, std::chrono::milliseconds(5));
    }
}

extern "C" amie_status amie_server_stop(amie_server *srv)
{
    if (!srv) return AMIE_OK;
    {
        std::lock_guard<std::mutex> lk(srv->mu);
        srv->stop_flag = true;
        for (auto *r : srv->pending) r->cancelled = true;
        for (auto *r : srv->ready) r->cancelled = true;
        for (auto *r : srv->slot_req)
            if (r) r->cancelled = true;
        srv->cv.notify_all();
    }
    for (std::thread &a : srv->admitters)
        if (a.joinable()) a.join();
    if (srv->worker.joinable()) srv->worker.join();
    cudaSetDevice(srv->ctx->device);
    cudaStreamSynchronize(srv->ctx->stream);
    for (amie_ctx *a : srv->adms) cudaStreamSynchronize(a->stream);
    amie::set_free_stream(srv->ctx->stream);
    for (auto &kv : srv->all) {
        if (kv.second->topo) release_topology(kv.second->topo);
        delete kv.second;
    }
    amie::set_free_stream(nullptr);
    cudaStreamSynchronize(srv->ctx->stream);
    if (srv->graph) cudaGraphExecDestroy(srv->graph);
    if (srv->graph3) cudaGraphExecDestroy(srv->graph3);
    if (srv->h_slots) cudaFreeHost(srv->h_slots);
    if (srv->h_ctl) cudaFreeHost(srv->h_ctl);
    if (srv->h_err) cudaFreeHost(srv->h_err);
    if (srv->h_run) cudaFreeHost(srv->h_run);
    if (srv->h_ring) cudaFreeHost(srv->h_ring);
    if (srv->h_cta_slot) cudaFreeHost(srv->h_cta_slot);
    if (srv->xfer) cudaStreamDestroy(srv->xfer);
    for (cudaEvent_t e : srv->ring_ev)
        if (e) cudaEventDestroy(e);
    srv->d_slots.release();
    srv->d_ctl.release();
    srv->d_run.release();
    srv->d_bar.release();
    srv->d_err.release();
    srv->d_cta_slot.release();
    srv->d_parts.release();
    for (amie_ctx *a : srv->adms) amie_ctx_destroy(a);
    if (srv->pool) cudaMemPoolDestroy(srv->pool);
    delete srv;
    return AMIE_OK;
}

extern "C" amie_status amie_server_query(amie_server *srv, amie_server_stats *stats)
{
    if (!srv || !stats) return AMIE_BAD_INPUT;
    std::lock_guard<std::mutex> lk(srv->mu);
    *stats = srv->stats;
    return AMIE_OK;
}
