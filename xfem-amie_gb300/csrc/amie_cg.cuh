// amie_cg.cuh -- ConjugateGradient::solve semantics on the device
// (solvers/conjugategradient.cpp:69-318), included by solver.cu.
//
// What is reproduced, step by step:
//   * Jacobi preconditioner 1/A_ii (|A_ii| > 1e-12, else 0);
//   * pre-smoothing: up to nssor sweeps x -= D^-1 (A x - b), stopping when
//     ||A x - b|| rises (solvers/conjugategradient.cpp:124-151);
//   * restart step: r = b - A x, z = D^-1 r, p = z, alpha = r.z / q.p, with the
//     |q.p| < 1e-12 r.z exit (:153-210);
//   * inner loop while sqrt|r.z| > max(1e-12, eps) and localnit < n, with the
//     |q.p| < 1e-24 rho break (:218-257);
//   * Kahan-compensated updates of x and r (:198-209, :242-253);
//   * post-smoothing while ||D^-1 (A x - b)|| falls, keeping the best x
//     (:274-302); convergence min(err, sqrt|rho|) < sqrt(realeps) (:305);
//   * outer restarts until n/2 (or maxit) iterations (:93, :121).
// Dot products are tree reductions in FP64 (not sequential Kahan sums), so
// iteration counts match the reference's to within a few and the solution to
// its rounding.
#pragma once

namespace amie {

struct AmieCtl {
    int32_t done;
    int32_t pad;
    int64_t localnit;   // inner-loop iterations of the current restart
    int64_t nit;        // completed CG updates (the reference's nit)
    int64_t nmax;       // localnit cap (n)
    double realeps;
    double last_rho;    // r.z of the last update
    double rho;         // r.z of the current iteration
};

// P1: z = D^-1 r, partial r.z
__global__ void __launch_bounds__(kVecThreads) k_amie_precond(uint64_t n, const double *dinv, const double *r, double *z,
                                                              double *part, const AmieCtl *ctl)
{
    __shared__ double sh[33];
    if (ctl->done) return;
    double a = 0.0;
    for (uint64_t i = (uint64_t)blockIdx.x * kVecThreads + threadIdx.x; i < n; i += (uint64_t)gridDim.x * kVecThreads) {
        const double zi = r[i] * dinv[i];
        z[i] = zi;
        a += r[i] * zi;
    }
    a = block_sum(a, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = a;
}

// P2: loop test on last_rho, then beta = rho / last_rho, p = p beta + z
__global__ void __launch_bounds__(kVecThreads) k_amie_direction(uint64_t n, const double *z, double *p, const double *part_rz,
                                                                AmieCtl *ctl)
{
    __shared__ double sh[33];
    if (ctl->done) return;
    const double last_rho = ctl->last_rho;
    if (!(sqrt(fabs(last_rho)) > ctl->realeps && ctl->localnit < ctl->nmax)) {
        if (blockIdx.x == 0 && threadIdx.x == 0) ctl->done = 1;
        return;
    }
    const double rho = sum_parts(part_rz, gridDim.x, sh);
    const double beta = rho / last_rho;
    for (uint64_t i = (uint64_t)blockIdx.x * kVecThreads + threadIdx.x; i < n; i += (uint64_t)gridDim.x * kVecThreads)
        p[i] = p[i] * beta + z[i];
}

// Kahan-compensated x += alpha p, r -= alpha q (solvers/conjugategradient.cpp:242-253).
__device__ __forceinline__ void kahan_xr(uint64_t i, double alpha, double *x, double *r, double *xc, double *rc,
                                        const double *p, const double *q)
{
    const double yr = -q[i] * alpha - rc[i];
    const double yx = p[i] * alpha - xc[i];
    const double rt = r[i] + yr;
    const double xt = x[i] + yx;
    rc[i] = (rt - r[i]) - yr;
    xc[i] = (xt - x[i]) - yx;
    r[i] = rt;
    x[i] = xt;
}

// P4: pq test, alpha = rho / pq, Kahan update, bookkeeping.
__global__ void __launch_bounds__(kVecThreads) k_amie_update(uint64_t n, double *x, double *r, double *xc, double *rc,
                                                             const double *p, const double *q, const double *part_rz,
                                                             const double *part_pq, AmieCtl *ctl)
{
    __shared__ double sh[33];
    if (ctl->done) return;
    const double rho = sum_parts(part_rz, gridDim.x, sh);
    const double pq = sum_parts(part_pq, gridDim.x, sh);
    if (fabs(pq) < 1e-24 * rho) {
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            ctl->last_rho = rho;
            ctl->rho = rho;
            ctl->localnit += 1;
            ctl->done = 1;
        }
        return;
    }
    const double alpha = rho / pq;
    for (uint64_t i = (uint64_t)blockIdx.x * kVecThreads + threadIdx.x; i < n; i += (uint64_t)gridDim.x * kVecThreads)
        kahan_xr(i, alpha, x, r, xc, rc, p, q);
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        ctl->last_rho = rho;
        ctl->rho = rho;
        ctl->localnit += 1;
        ctl->nit += 1;
    }
}

__global__ void k_amie_first_update(uint64_t n, double alpha, double *x, double *r, double *xc, double *rc,
                                    const double *p, const double *q)
{
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        kahan_xr(i, alpha, x, r, xc, rc, p, q);
}

// Jacobi sweep from y = b - A x: x -= D^-1 (A x - b) with Kahan compensation
// (solvers/conjugategradient.cpp:139-148, 277-285); partial ||D^-1 (A x - b)||^2.
__global__ void __launch_bounds__(kVecThreads) k_amie_jacobi(uint64_t n, const double *y, const double *dinv, double *x,
                                                             double *xc, double *part)
{
    __shared__ double sh[33];
    double a = 0.0;
    for (uint64_t i = (uint64_t)blockIdx.x * kVecThreads + threadIdx.x; i < n; i += (uint64_t)gridDim.x * kVecThreads) {
        const double d = y[i] * dinv[i];          // = -(D^-1 (A x - b))_i
        const double yx = d - xc[i];
        const double xt = x[i] + yx;
        xc[i] = (xt - x[i]) - yx;
        x[i] = xt;
        a += d * d;
    }
    a = block_sum(a, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = a;
}

constexpr int kAmieGraphIters = 16;

amie_status amie_cg_solve(amie_topo *t, const amie_solve_opts *o, amie_solve_stats *st_out)
{
    SolverState *s = nullptr;
    AMIE_TRY(ensure_state(t, false, &s));
    AMIE_TRY(ensure_sell(t, true, false));
    cudaStream_t st = t->ctx->stream;
    const uint64_t n = t->n;
    const int grid = s->grid;
    if (!t->xc.p) {
        AMIE_TRY(t->xc.alloc(t->ctx, n));
        AMIE_TRY(t->rc.alloc(t->ctx, n));
        AMIE_TRY(t->red.alloc(t->ctx, n));   // xmin
    }
    DevArray<AmieCtl> dctl;
    AMIE_TRY(dctl.alloc(t->ctx, 1));
    AmieCtl *hctl = reinterpret_cast<AmieCtl *>(t->ctx->h_scalars);   // pinned, 64 doubles

    const double eps = o && o->eps > 0 ? o->eps : 1e-10;
    const int nssor = o ? o->nssor : 32;
    const double realeps = std::max(1e-12, eps);
    const int64_t Maxit = o && o->maxit > 0 ? o->maxit : (int64_t)(n / 2);
    // partial buffers: pq | rz (restart step and inner loop) | rr (restart step) | norms
    const PcgParts parts0 = parts_of(s);
    double *part_pq = parts0.pq;
    double *part_rz = parts0.rz;
    double *part_a = parts0.spare;
    double *x = t->x.p, *r = t->r.p, *z = t->z.p, *p = t->p.p, *q = t->q.p, *xc = t->xc.p, *rc = t->rc.p;
    double *xmin = t->red.p;
    const BsrView<double> A = bsr64(t);
    PcgVecs<double> v = vecs_of<double>(t);

    st_out->iterations = 0;
    st_out->refinements = 0;
    // homogeneous problem: max|b| < eps^2 (solvers/conjugategradient.cpp:74-78)
    {
        double bb = 0.0;
        k_norm2_parts<<<grid, kVecThreads, 0, st>>>(n, t->rhs.p, part_a);
        AMIE_LAUNCHED();
        AMIE_TRY(read_sum(t, part_a, grid, &bb));
        if (bb == 0.0) {   // (max|b| < eps^2 is implied for the zero vector; other cases proceed)
            AMIE_CUDA(cudaMemsetAsync(x, 0, n * 8, st));
            st_out->status = AMIE_OK;
            st_out->relres = 0.0;
            return AMIE_OK;
        }
    }
    // graph of the inner loop
    cudaGraphExec_t gexec = nullptr;
    {
        cudaGraph_t graph;
        AMIE_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        for (int it = 0; it < kAmieGraphIters; it++) {
            k_amie_precond<<<grid, kVecThreads, 0, st>>>(n, t->invdiag.p, r, z, part_rz, dctl.p);
            k_amie_direction<<<grid, kVecThreads, 0, st>>>(n, z, p, part_rz, dctl.p);
            launch_spmv_pq<double>(t, grid, v, part_pq, &dctl.p->done, nullptr, st);
            k_amie_update<<<grid, kVecThreads, 0, st>>>(n, x, r, xc, rc, p, q, part_rz, part_pq, dctl.p);
        }
        AMIE_CUDA(cudaStreamEndCapture(st, &graph));
        cudaError_t e = cudaGraphInstantiate(&gexec, graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) {
            set_error("cudaGraphInstantiate: %s", cudaGetErrorString(e));
            return AMIE_CUDA_ERROR;
        }
    }
    struct GraphGuard {
        cudaGraphExec_t g;
        ~GraphGuard() { if (g) cudaGraphExecDestroy(g); }
    } guard{gexec};

    int64_t nit = 0;
    double errmin = 0.0;
    amie_status result = AMIE_NOT_CONVERGED;
    AMIE_CUDA(cudaMemcpyAsync(xmin, x, n * 8, cudaMemcpyDeviceToDevice, st));
    while (nit < Maxit) {
        AMIE_CUDA(cudaMemsetAsync(xc, 0, n * 8, st));
        AMIE_CUDA(cudaMemsetAsync(rc, 0, n * 8, st));
        if (nssor) {   // pre-smoothing
            double err = 2.0;
            int iter = 0;
            while (iter++ < nssor && err > realeps) {
                double rr = 0.0;
                launch_spmv<double>(t, grid, A, x, t->rhs.p, r, part_a, st);
                AMIE_TRY(read_sum(t, part_a, grid, &rr));
                const double perr = err;
                err = std::sqrt(rr);
                if (err > perr) break;
                k_amie_jacobi<<<grid, kVecThreads, 0, st>>>(n, r, t->invdiag.p, x, xc, part_a);
                AMIE_LAUNCHED();
            }
            AMIE_CUDA(cudaMemsetAsync(xc, 0, n * 8, st));
        }
        double rr = 0.0;
        launch_spmv<double>(t, grid, A, x, t->rhs.p, r, part_a, st);   // r = b - A x
        AMIE_TRY(read_sum(t, part_a, grid, &rr));
        const double err0 = std::sqrt(rr);
        if (std::isnan(err0)) { result = AMIE_NAN; break; }
        if (nit == 0) errmin = err0;
        if (err0 < realeps) { result = AMIE_OK; break; }
        // z = D^-1 r, p = z, q = A p
        PcgParts parts = parts_of(s);
        AMIE_CUDA(cudaMemsetAsync(s->ctl.p, 0, sizeof(PcgCtl), st));
        k_pcg_start<double><<<grid, kVecThreads, 0, st>>>(v, n, parts, s->ctl.p);   // z, p; partial r.z
        AMIE_LAUNCHED();
        launch_spmv_pq<double>(t, grid, v, part_pq, nullptr, nullptr, st);
        double last_rho = 0.0, pq = 0.0;
        AMIE_TRY(read_sum(t, parts.rz, grid, &last_rho));
        AMIE_TRY(read_sum(t, part_pq, grid, &pq));
        if (std::fabs(pq) < 1e-12 * last_rho) { result = AMIE_OK; break; }
        k_amie_first_update<<<grid, kVecThreads, 0, st>>>(n, last_rho / pq, x, r, xc, rc, p, q);
        AMIE_LAUNCHED();
        // inner loop on the device
        AmieCtl c{};
        c.done = 0;
        c.localnit = 0;
        c.nit = nit;
        c.nmax = (int64_t)n;
        c.realeps = realeps;
        c.last_rho = last_rho;
        c.rho = 0.0;
        *hctl = c;
        AMIE_CUDA(cudaMemcpyAsync(dctl.p, hctl, sizeof(AmieCtl), cudaMemcpyHostToDevice, st));
        AMIE_CUDA(cudaStreamSynchronize(st));
        // host watchdog: localnit <= n, so the device finishes within n / kAmieGraphIters + 2 launches
        const int64_t max_launches = (int64_t)(n / kAmieGraphIters) + 2;
        for (int64_t launch = 0;; launch++) {
            AMIE_CUDA(cudaGraphLaunch(gexec, st));
            g_launches += 4 * kAmieGraphIters;
            AMIE_CUDA(cudaMemcpyAsync(hctl, dctl.p, sizeof(AmieCtl), cudaMemcpyDeviceToHost, st));
            AMIE_CUDA(cudaStreamSynchronize(st));
            if (hctl->done) break;
            if (launch >= max_launches) {
                set_error("CG control block stalled: localnit %lld, nit %lld", (long long)hctl->localnit,
                          (long long)hctl->nit);
                return AMIE_TIMEOUT;
            }
        }
        nit = hctl->nit;
        last_rho = hctl->last_rho;
        const double rho = hctl->rho;
        // r = A x - b (norm only), best x so far
        launch_spmv<double>(t, grid, A, x, t->rhs.p, r, part_a, st);
        AMIE_TRY(read_sum(t, part_a, grid, &rr));
        double err = std::sqrt(rr);
        if (err < errmin) {
            errmin = std::sqrt(std::fabs(rho));
            AMIE_CUDA(cudaMemcpyAsync(xmin, x, n * 8, cudaMemcpyDeviceToDevice, st));
        }
        if (nssor) {   // post-smoothing
            uint64_t iters = 0;
            while (err > realeps && iters++ < n) {
                launch_spmv<double>(t, grid, A, x, t->rhs.p, r, nullptr, st);
                k_amie_jacobi<<<grid, kVecThreads, 0, st>>>(n, r, t->invdiag.p, x, xc, part_a);
                AMIE_LAUNCHED();
                double dd = 0.0;
                AMIE_TRY(read_sum(t, part_a, grid, &dd));
                const double perr = err;
                err = std::sqrt(dd);
                if (err > perr) break;
                AMIE_CUDA(cudaMemcpyAsync(xmin, x, n * 8, cudaMemcpyDeviceToDevice, st));
            }
            if (iters > 2) AMIE_CUDA(cudaMemcpyAsync(x, xmin, n * 8, cudaMemcpyDeviceToDevice, st));
        }
        st_out->refinements++;
        if (std::min(err, std::sqrt(std::fabs(last_rho))) < std::sqrt(realeps)) { result = AMIE_OK; break; }
    }
    // final true relative residual for the statistics
    double rr = 0.0, bb = 0.0;
    launch_spmv<double>(t, grid, A, x, t->rhs.p, r, part_a, st);
    AMIE_TRY(read_sum(t, part_a, grid, &rr));
    k_norm2_parts<<<grid, kVecThreads, 0, st>>>(n, t->rhs.p, part_a);
    AMIE_LAUNCHED();
    AMIE_TRY(read_sum(t, part_a, grid, &bb));
    st_out->iterations = nit;
    st_out->relres = bb > 0 ? std::sqrt(rr / bb) : 0.0;
    st_out->status = result;
    return AMIE_OK;
}

}  // namespace amie
