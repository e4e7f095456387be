// noalloc.cu -- a Jacobi-PCG solve that allocates no device memory.
//
// Who needs it: callers that cannot call cudaMalloc at solve time --
// applications that hand every byte of device memory to their own pool
// allocator at start-up, and real-time loops that cannot afford the implicit
// device synchronisation an allocation may cause.  They keep the matrix, the
// right-hand side and the solution in their own device memory; the work
// vectors of the solve (r, z, p, q, the inverse diagonal, the per-CTA partial
// sums and the control block) live in one file-scope __device__ array of fixed
// size, which every GPU that loads this library reserves until the process
// exits.  The solve is driven from the host: it synchronises the caller's
// stream to read the norms and the control block every 16 iterations.
//
// The array is shared by every call on a device and keeps the last call's
// contents: each call initialises everything it reads before reading it.
// Calls that overlap on the GPU (two host threads, or two streams) race on it.
#include "solver.cuh"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <mutex>

namespace amie {

constexpr uint64_t kNoAllocMaxDof = 262144;   // scalar DOFs (n_rows * stride)
constexpr int kNoAllocMaxCtas = 2048;         // per-CTA partial sums
constexpr uint64_t kNoAllocDoubles = 5 * kNoAllocMaxDof + 4 * (uint64_t)kNoAllocMaxCtas + 16;

// r | z | p | q | D^-1 | partials (pq, rz0, rz1, rr) | control block
static __device__ __align__(256) double g_noalloc_scratch[kNoAllocDoubles];

static_assert(sizeof(PcgCtl) <= 16 * sizeof(double), "control block must fit its reserved slot");

struct NoAllocDevice {
    bool ready = false;
    double *base = nullptr;   // device address of g_noalloc_scratch on this device
    int num_sms = 0;
};

static std::mutex g_noalloc_mu;
static NoAllocDevice g_noalloc_dev[128];

// Inverse diagonal of a block-CSR matrix: 1/A_ii if |A_ii| > 1e-12 else 0
// (sparse/sparse_matrix.cpp:216-231).  The diagonal block is found by a scan of
// the row (10-30 blocks), so the caller's columns need not be sorted; a row
// without a diagonal block gets 0, as the reference's zero diagonal does.
template <int S>
__global__ void k_noalloc_invdiag(uint32_t n_rows, const uint32_t *row_ptr, const uint32_t *col, const double *val,
                                  double *dinv)
{
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n_rows) return;
    const uint32_t end = row_ptr[k + 1];
    uint32_t at = end;
    for (uint32_t j = row_ptr[k]; j < end; j++)
        if (col[j] == k) { at = j; break; }
    for (int r = 0; r < S; r++) {
        const double v = at < end ? val[(uint64_t)at * S * S + r * S + r] : 0.0;
        dinv[(uint64_t)k * S + r] = fabs(v) > 1e-12 ? 1.0 / v : 0.0;
    }
}

__global__ void k_noalloc_norm2(uint64_t n, const double *v, double *part)
{
    __shared__ double sh[33];
    double a = 0.0;
    for (uint64_t i = (uint64_t)blockIdx.x * kVecThreads + threadIdx.x; i < n; i += (uint64_t)gridDim.x * kVecThreads)
        a += v[i] * v[i];
    a = block_sum(a, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = a;
}

namespace {

template <int S, typename F>
void with_group(int group, F &&f)
{
    switch (group) {
    case 4: f(std::integral_constant<int, 4>()); break;
    case 8: f(std::integral_constant<int, 8>()); break;
    case 16: f(std::integral_constant<int, 16>()); break;
    default: f(std::integral_constant<int, 32>()); break;
    }
}

// Sum of n partials read back into a stack buffer (no allocation).
amie_status host_sum(const double *dev, int n, cudaStream_t st, double *out)
{
    double h[kNoAllocMaxCtas];
    AMIE_CUDA(cudaMemcpyAsync(h, dev, n * sizeof(double), cudaMemcpyDeviceToHost, st));
    AMIE_CUDA(cudaStreamSynchronize(st));
    double s = 0.0;
    for (int i = 0; i < n; i++) s += h[i];
    *out = s;
    return AMIE_OK;
}

template <int S>
amie_status noalloc_solve(const NoAllocDevice &dev, uint32_t n_rows, const uint32_t *row_ptr, const uint32_t *col,
                          const double *val, const double *b, double *x, double rtol, int64_t maxit, bool use_x0,
                          cudaStream_t st, amie_solve_stats *stats)
{
    const uint64_t n = (uint64_t)n_rows * S;
    double *base = dev.base;
    double *r = base, *z = base + kNoAllocMaxDof, *p = base + 2 * kNoAllocMaxDof, *q = base + 3 * kNoAllocMaxDof;
    double *dinv = base + 4 * kNoAllocMaxDof;
    double *parts = base + 5 * kNoAllocMaxDof;
    PcgCtl *ctl = reinterpret_cast<PcgCtl *>(parts + 4 * kNoAllocMaxCtas);
    const int grid = std::min(dev.num_sms * 4, kNoAllocMaxCtas);
    PcgParts pp;
    pp.pq = parts;
    pp.rz = parts + kNoAllocMaxCtas;
    pp.rr = parts + 2 * kNoAllocMaxCtas;
    pp.spare = parts + 3 * kNoAllocMaxCtas;
    uint32_t nnzb = 0;
    AMIE_CUDA(cudaMemcpyAsync(&nnzb, row_ptr + n_rows, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    AMIE_CUDA(cudaStreamSynchronize(st));
    const double avg = n_rows ? (double)nnzb / n_rows : 0.0;
    const int group = avg <= 4.5 ? 4 : avg <= 9 ? 8 : avg <= 18 ? 16 : 32;
    const BsrView<double> A{n_rows, row_ptr, col, val};
    PcgVecs<double> v{A, dinv, x, r, z, p, q};

    k_noalloc_invdiag<S><<<(n_rows + 255) / 256, 256, 0, st>>>(n_rows, row_ptr, col, val, dinv);
    AMIE_LAUNCHED();
    if (!use_x0) AMIE_CUDA(cudaMemsetAsync(x, 0, n * sizeof(double), st));
    k_noalloc_norm2<<<grid, kVecThreads, 0, st>>>(n, b, pp.spare);
    AMIE_LAUNCHED();
    double bb = 0.0;
    AMIE_TRY(host_sum(pp.spare, grid, st, &bb));
    const double bnorm = std::sqrt(bb);
    stats->iterations = 0;
    stats->refinements = 0;
    if (bnorm == 0.0) {
        AMIE_CUDA(cudaMemsetAsync(x, 0, n * sizeof(double), st));
        AMIE_CUDA(cudaStreamSynchronize(st));
        stats->relres = 0.0;
        stats->status = AMIE_OK;
        return AMIE_OK;
    }
    auto residual = [&](double *rr) -> amie_status {   // r = b - A x, returns r.r
        with_group<S>(group, [&](auto g) {
            constexpr int G = decltype(g)::value;
            k_spmv<S, G, double><<<grid, kVecThreads, 0, st>>>(A, x, b, r, pp.spare);
        });
        AMIE_LAUNCHED();
        return host_sum(pp.spare, grid, st, rr);
    };
    double rr = 0.0;
    AMIE_TRY(residual(&rr));
    const double target2 = (rtol * bnorm) * (rtol * bnorm);
    int64_t total = 0;
    amie_status result = AMIE_NOT_CONVERGED;
    constexpr int kCheck = 16;   // iterations between host reads of the control block
    for (int outer = 0; outer < 200; outer++) {
        if (!(rr == rr)) { result = AMIE_NAN; break; }
        if (rr <= target2) { result = AMIE_OK; break; }
        if (total >= maxit) break;
        PcgCtl c{};   // done = 0, ticket = 0, iterations = 0
        c.maxit = maxit - total;
        c.tol2 = 0.25 * target2;
        AMIE_CUDA(cudaMemcpyAsync(ctl, &c, sizeof(PcgCtl), cudaMemcpyHostToDevice, st));
        k_pcg_start<double><<<grid, kVecThreads, 0, st>>>(v, n, pp, ctl);
        AMIE_LAUNCHED();
        const int64_t max_rounds = c.maxit / kCheck + 2;
        PcgCtl h{};
        for (int64_t round = 0;; round++) {
            for (int it = 0; it < kCheck; it++) {
                with_group<S>(group, [&](auto g) {
                    constexpr int G = decltype(g)::value;
                    k_spmv_pq<S, G, double><<<grid, kVecThreads, 0, st>>>(v, pp.pq, &ctl->done, ctl);
                });
                k_update<double><<<grid, kVecThreads, 0, st>>>(v, n, pp, ctl);
                k_direction<double><<<grid, kVecThreads, 0, st>>>(v, n, ctl);
                g_launches += 3;
            }
            AMIE_CUDA(cudaMemcpyAsync(&h, ctl, sizeof(PcgCtl), cudaMemcpyDeviceToHost, st));
            AMIE_CUDA(cudaStreamSynchronize(st));
            if (h.done) break;
            if (round >= max_rounds) {
                set_error("no-alloc PCG control block stalled at iteration %lld", (long long)h.iterations);
                return AMIE_TIMEOUT;
            }
        }
        total += h.iterations;
        AMIE_TRY(residual(&rr));
        if (h.iterations == 0) break;
    }
    AMIE_CUDA(cudaGetLastError());
    stats->iterations = total;
    stats->relres = std::sqrt(rr) / bnorm;
    stats->status = result;
    return AMIE_OK;
}

}  // namespace

}  // namespace amie

using namespace amie;

extern "C" amie_status amie_pcg_solve_noalloc(int32_t stride, uint32_t n_rows, const uint32_t *row_ptr_dev,
                                              const uint32_t *col_dev, const double *val_dev, const double *b_dev,
                                              double *x_dev, double rtol, int64_t maxit, int32_t use_x0, void *stream,
                                              amie_solve_stats *stats)
{
    if ((stride != 2 && stride != 3) || !row_ptr_dev || !col_dev || !val_dev || !b_dev || !x_dev || !stats) {
        set_error("amie_pcg_solve_noalloc: stride must be 2 or 3 and every pointer non-null");
        return AMIE_BAD_INPUT;
    }
    if (n_rows == 0 || (uint64_t)n_rows * stride > kNoAllocMaxDof) {
        set_error("amie_pcg_solve_noalloc: %llu scalar DOFs, the static work area holds 1 to %llu",
                  (unsigned long long)n_rows * stride, (unsigned long long)kNoAllocMaxDof);
        return AMIE_BAD_INPUT;
    }
    int device = 0;
    AMIE_CUDA(cudaGetDevice(&device));
    if (device < 0 || device >= 128) {
        set_error("amie_pcg_solve_noalloc: device %d, this library serves devices 0 to 127", device);
        return AMIE_BAD_INPUT;
    }
    NoAllocDevice dev;
    {
        // Set-up, once per device, with that device current: the device address of
        // the static work area.  In host code the array's name is only a host-side
        // stand-in, so kernels receive this address instead.
        std::lock_guard<std::mutex> lk(g_noalloc_mu);
        NoAllocDevice &d = g_noalloc_dev[device];
        if (!d.ready) {
            void *ptr = nullptr;
            cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
            if (e != cudaSuccess || !ptr) {
                set_error("cudaGetSymbolAddress(g_noalloc_scratch): %s", cudaGetErrorString(e));
                cudaGetLastError();
                return AMIE_CUDA_ERROR;
            }
            int sms = 0;
            AMIE_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
            d.base = static_cast<double *>(ptr);
            d.num_sms = sms;
            d.ready = true;
        }
        dev = d;
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const double tol = rtol > 0 ? rtol : 1e-10;
    const int64_t cap = maxit > 0 ? maxit : std::max<int64_t>(1000, (int64_t)n_rows * stride);
    *stats = amie_solve_stats{};
    const auto t0 = std::chrono::steady_clock::now();
    amie_status rc = stride == 2 ? noalloc_solve<2>(dev, n_rows, row_ptr_dev, col_dev, val_dev, b_dev, x_dev, tol, cap,
                                                    use_x0 != 0, st, stats)
                                 : noalloc_solve<3>(dev, n_rows, row_ptr_dev, col_dev, val_dev, b_dev, x_dev, tol, cap,
                                                    use_x0 != 0, st, stats);
    stats->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (rc != AMIE_OK) return rc;
    return (amie_status)stats->status;
}
