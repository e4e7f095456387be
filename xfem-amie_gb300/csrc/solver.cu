// solver.cu -- host drivers of the device-resident solvers and the solve
// entry points of the C-ABI.
//
//   AMIE_SOLVER_PCG_FP64   Jacobi-PCG in FP64, relative-residual stop, restarted
//                          from the true residual b - A x if the recursive one drifted.
//   AMIE_SOLVER_PCG_MIXED  FP32 Jacobi-PCG (FP32 SpMV, preconditioner and vector
//                          updates) with reliable updates: whenever the FP32
//                          recursive residual has dropped by inner_rtol, the FP32
//                          increment is added to x in FP64, r = b - A x is
//                          recomputed in FP64 and the FP32 run continues from it
//                          with its search direction kept (no Krylov restart).
//   AMIE_SOLVER_AMIE_CG    ConjugateGradient::solve semantics (amie_cg.cu).
#include "solver.cuh"
#include "persist.cuh"

#include <chrono>
#include <cstdlib>
#include <cmath>
#include <mutex>
#include <unordered_map>

namespace amie {

amie_status assemble_async(amie_topo *t);
amie_status finalize_matrix_async(amie_topo *t, bool want32);
amie_status amie_cg_solve(amie_topo *t, const amie_solve_opts *o, amie_solve_stats *st);

// k_sell_dir instance for the stride and the matrix-stream hint
template <typename T>
const void *sell_dir_kernel(int s, int hint)
{
    if (s == 2) {
        if (hint == 1) return (const void *)k_sell_dir<2, T, 1>;
        if (hint == 2) return (const void *)k_sell_dir<2, T, 2>;
        return (const void *)k_sell_dir<2, T, 0>;
    }
    if (hint == 1) return (const void *)k_sell_dir<3, T, 1>;
    if (hint == 2) return (const void *)k_sell_dir<3, T, 2>;
    return (const void *)k_sell_dir<3, T, 0>;
}

// k_sell_fused instance for the stride and the matrix-stream hint
const void *sell_fused_kernel(int s, int hint)
{
    if (s == 2) {
        if (hint == 1) return (const void *)k_sell_fused<2, float, 1>;
        if (hint == 2) return (const void *)k_sell_fused<2, float, 2>;
        return (const void *)k_sell_fused<2, float, 0>;
    }
    if (hint == 1) return (const void *)k_sell_fused<3, float, 1>;
    if (hint == 2) return (const void *)k_sell_fused<3, float, 2>;
    return (const void *)k_sell_fused<3, float, 0>;
}

template <bool START>
const void *sell_cgcg_kernel(int s, int hint)
{
    if (s == 2) {
        if (hint == 1) return (const void *)k_sell_cgcg<2, float, 1, START>;
        if (hint == 2) return (const void *)k_sell_cgcg<2, float, 2, START>;
        return (const void *)k_sell_cgcg<2, float, 0, START>;
    }
    if (hint == 1) return (const void *)k_sell_cgcg<3, float, 1, START>;
    if (hint == 2) return (const void *)k_sell_cgcg<3, float, 2, START>;
    return (const void *)k_sell_cgcg<3, float, 0, START>;
}

struct SolverState {
    int grid = 0;                 // block-CSR SpMV, AMIE_CG and server kernels
    int grid_vec[2] = {0, 0};     // PCG vector kernels, FP32 / FP64 (resident CTAs of k_update)
    int grid_sell[2] = {0, 0};    // SELL SpMV, FP32 / FP64 (resident CTAs of that kernel)
    int grid_dir[2] = {0, 0};     // k_sell_dir, FP32 / FP64
    int stride = 0;               // partials per kind in `parts` (the largest grid)
    bool pdl = true;              // programmatic dependent launch inside the PCG graphs
    // FP32 graphs form p = z + beta p inside the SpMV (two kernels per iteration);
    // FP64 graphs keep the direction kernel: folding it costs one FP64 FMA per
    // gathered entry instead of one per vector entry, and FP64 issue is the
    // scarce resource of this GPU (the folded FP64 solve ran 1.4x slower)
    bool fold_dir = true;
    // L2 eviction hint of the matrix stream in k_sell_dir (see ld_stream);
    // AMIE_MATRIX_HINT overrides it for measurements
    int matrix_hint = kMatrixHint;
    // bytes of each CTA's matrix range k_sell_dir prefetches into L2 before its wait
    // (AMIE_PREFETCH_KB; mixed solve of the 1.2 M-DOF P2 problem: 0 KB 686 ms, 16 KB 673 ms,
    // 32-64 KB 674 ms, 128 KB 688 ms)
    uint32_t prefetch_bytes = 16u << 10;
    int graph_kernels[2] = {3, 3};   // kernels per iteration of the FP32 / FP64 graph
    DevArray<double> parts;       // 4 * stride: pq, rz, rr, spare
    DevArray<PcgCtl> ctl;
    PcgCtl *h_ctl = nullptr;      // pinned
    PcgCtl *h_ring = nullptr;     // pinned, 2: control block after each of two graph launches in flight
    cudaEvent_t ring_ev[2] = {nullptr, nullptr};
    cudaGraphExec_t graph64 = nullptr, graph32 = nullptr;
    int graph_iters = 0;
    DevArray<double> x_saved;        // FP64 solve: the first stage's iterate while the second runs
    // FP32 inner runs of the mixed solver as single-reduction (Chronopoulos-Gear)
    // PCG, one kernel per iteration; opt-in (AMIE_CGCG=1).  Measured against the
    // two-kernel standard PCG (mixed, rtol 1e-10): 150 k-DOF P1 11.7 vs 13.5 us per
    // iteration but 2,016 vs 1,584 iterations and a node error of 1.3e-8 vs 3.6e-9;
    // 64^3-voxel tetrahedra 47.0 vs 42.8 us per iteration; 1.2 M-DOF P2 (4,000
    // inclusions, a Heaviside crack) did not converge: the recursively updated
    // s = A p and the alpha recurrence drift in FP32 over its ~18,000 iterations
    bool cgcg = false;
    int grid_cgcg = 0;
    int cg_cur = 0;                  // buffer of r, w holding the current FP32 residual
    DevArray<float> r32b, w32[2], s32[2], slice3;
    cudaGraphExec_t graph_cg = nullptr;
    // FP32 inner runs of the mixed solver as one kernel per iteration of standard
    // PCG (k_sell_fused); opt-in (AMIE_FUSED=1).  Same iterations and accuracy as
    // the two-kernel graph (1.2 M-DOF P2: 18,556 vs 18,619, node error 4.2e-9 vs
    // 3.4e-9), but slower: 48.3 vs 37.0 us per iteration there (51.0 us for the
    // kernel alone against 28.7 us for k_sell_dir), 51.1 vs 42.8 on the 64^3-voxel
    // tetrahedra.  The update's vectors move into the bandwidth-bound SpMV (the
    // warp's rows are SELL-permuted, so their r, q, x, D^-1 accesses scatter), its
    // gathers read 24 instead of 16 bytes per block column, and 80 registers
    // leave 3 CTAs per SM; that costs more than the update kernel it saves.
    bool fused = false;
    int grid_fused = 0;
    int fused_cur = 0;               // direction / zw buffer of the latest run's last direction
    DevArray<float> zw32[2];         // per node: z then w = D^-1 q (2 s floats), double-buffered
    DevArray<double> slice5;
    cudaGraphExec_t graph_fused = nullptr;
    // Runs of the standard PCG as one cooperative launch (k_pcg_persist) instead
    // of graphs of kernels (FP32 runs, whose graphs fold the direction update);
    // opt-in (AMIE_PERSIST=1).  Measured against the graphs
    // (mixed, rtol 1e-10): 44.6 k-DOF P1 23.4 vs 22.6 ms (25.2 ms with an
    // atomicAdd arrival and a sleeping poll), the 250 k-DOF notched beam's
    // 60-step damage loop 35.0 vs 32.0 s, 824 k-DOF voxel tetrahedra 73.1 vs
    // 63.7 ms; same iterations.  A grid barrier with the partial sums after it
    // costs more than a PDL kernel boundary, and the SpMV phase with 24 warps
    // per SM runs slower than k_sell_dir with 32 and its early prefetch.
    int persist_mode = 0;
    int grid_persist[2] = {0, 0};    // FP32 / FP64: one CTA per SM, 0 = not possible
    DevArray<PersistSync> psync;
    PersistSync *h_psync = nullptr;  // pinned
    // AMIE_PERSIST_BARRIER_TEST=1 (tests): the barriers wait for one arrival more
    // than the grid has and give up after 4096 polls
    bool persist_barrier_test = false;
    ~SolverState()
    {
        if (graph64) cudaGraphExecDestroy(graph64);
        if (graph32) cudaGraphExecDestroy(graph32);
        if (graph_cg) cudaGraphExecDestroy(graph_cg);
        if (graph_fused) cudaGraphExecDestroy(graph_fused);
        pinned_put(h_ctl, sizeof(PcgCtl));
        pinned_put(h_ring, 2 * sizeof(PcgCtl));
        pinned_put(h_psync, sizeof(PersistSync));
        for (cudaEvent_t e : ring_ev)
            if (e) cudaEventDestroy(e);
    }
};

template <typename T>
bool fold(const SolverState *s)
{
    return sizeof(T) == 4 && s->fold_dir;
}

static std::mutex g_state_mu;
static std::unordered_map<const amie_topo *, SolverState *> g_states;

SolverState *state_of(amie_topo *t)
{
    std::lock_guard<std::mutex> lk(g_state_mu);
    auto it = g_states.find(t);
    return it == g_states.end() ? nullptr : it->second;
}

void release_solver_state(const amie_topo *t)
{
    std::lock_guard<std::mutex> lk(g_state_mu);
    auto it = g_states.find(t);
    if (it != g_states.end()) {
        delete it->second;
        g_states.erase(it);
    }
}

template <int S, typename T, typename F>
void dispatch_group(int group, F &&f)
{
    switch (group) {
    case 1: f(std::integral_constant<int, 1>()); break;
    case 2: f(std::integral_constant<int, 2>()); break;
    case 4: f(std::integral_constant<int, 4>()); break;
    case 8: f(std::integral_constant<int, 8>()); break;
    case 16: f(std::integral_constant<int, 16>()); break;
    default: f(std::integral_constant<int, 32>()); break;
    }
}

amie_status ensure_sell(amie_topo *t, bool want64, bool want32);
amie_status ensure_sell_partition(amie_topo *t, int grid);

// SELL copy of the current matrix in precision T (val == nullptr if not converted).
template <typename T>
SellView<T> sell_of(amie_topo *t);
template <>
SellView<double> sell_of<double>(amie_topo *t)
{
    return SellView<double>{t->n_rows, t->n_slices, t->sell_perm.p, t->sell_ptr.p, t->sell_col.p,
                            t->sell64_ok ? t->sell_val.p : nullptr, nullptr, t->sell_dot.p};
}
template <>
SellView<float> sell_of<float>(amie_topo *t)
{
    return SellView<float>{t->n_rows, t->n_slices, t->sell_perm.p, t->sell_ptr.p, t->sell_col.p,
                           t->sell32_ok ? t->sell_val32.p : nullptr, nullptr,
                           reinterpret_cast<float *>(t->sell_dot.p)};
}

// Launch with programmatic stream serialization (the kernel calls pdl_wait
// before it reads anything its predecessor wrote) when `pdl`, else plainly.
template <typename... KArgs, typename... Args>
void launch_k(bool pdl, void (*kern)(KArgs...), int grid, size_t smem, cudaStream_t st, Args... args)
{
    if (!pdl) {
        kern<<<grid, kVecThreads, smem, st>>>(args...);
        return;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3(kVecThreads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, kern, args...);
}

template <typename T>
using SellKernel = void (*)(SellView<T>, const T *, T *, double *, const int32_t *, PcgCtl *);

// SELL SpMV kernel for block size s and loop variant (see amie_topo::sell_variant)
// and its dynamic shared memory.
template <typename T>
SellKernel<T> sell_kernel(int s, int variant, size_t *smem)
{
    *smem = 0;
    constexpr size_t W = kVecThreads / 32;
    if (variant == 6) {
        if (s == 2) {
            *smem = W * 4 * sell_stage_bytes<2, 2, T>();
            return k_sell_pq_cp<2, 2, 4, T>;
        }
        *smem = W * 4 * sell_stage_bytes<3, 2, T>();
        return k_sell_pq_cp<3, 2, 4, T>;
    }
    if (variant == 7) {
        if (s == 2) {
            *smem = W * 3 * sell_stage_bytes<2, 4, T>();
            return k_sell_pq_cp<2, 4, 3, T>;
        }
        *smem = W * 3 * sell_stage_bytes<3, 2, T>();
        return k_sell_pq_cp<3, 2, 3, T>;
    }
    if (s == 2) {
        switch (variant) {
        case 1: return k_sell_pq<2, 8, false, 1, T>;
        case 2: return k_sell_pq<2, 2, true, 1, T>;
        case 3: return k_sell_pq<2, 4, true, 1, T>;
        case 4: return k_sell_pq<2, 4, false, 5, T>;
        case 5: return k_sell_pq<2, 2, true, 5, T>;
        default: return k_sell_pq<2, 4, false, 1, T>;
        }
    }
    switch (variant) {
    case 1: return k_sell_pq<3, 8, false, 1, T>;
    case 2: case 5: return k_sell_pq<3, 2, true, 1, T>;
    case 3: return k_sell_pq<3, 4, true, 1, T>;
    default: return k_sell_pq<3, 4, false, 1, T>;
    }
}

// Launch q = A p (+ partial p.q): on the SELL copy when it is current (see
// ensure_sell), else on the block-CSR matrix with the topology's lane group;
// `done` (nullable) stops it, `fin` (nullable) receives pq and alpha.  The
// kernel writes `grid` partials.
template <typename T>
void launch_spmv_pq(amie_topo *t, int grid, const PcgVecs<T> &v, double *part, const int32_t *done, PcgCtl *fin,
                    cudaStream_t st, bool pdl = false)
{
    SellView<T> sv = sell_of<T>(t);
    auto part_it = t->sell_cta_first.find(grid);   // made by ensure_state for every grid it hands out
    if (sv.val && part_it != t->sell_cta_first.end()) {
        sv.cta_first = part_it->second.p;
        size_t smem = 0;
        const SellKernel<T> k = sell_kernel<T>(t->s, t->sell_variant, &smem);
        launch_k(pdl, k, grid, smem, st, sv, (const T *)v.p, v.q, part, done, fin);
        AMIE_LAUNCHED();
        return;
    }
    auto go = [&](auto g) {
        constexpr int G = decltype(g)::value;
        if (t->s == 2) launch_k(pdl, k_spmv_pq<2, G, T>, grid, 0, st, v, part, done, fin);
        else launch_k(pdl, k_spmv_pq<3, G, T>, grid, 0, st, v, part, done, fin);
    };
    dispatch_group<2, T>(t->spmv_group, go);
    AMIE_LAUNCHED();
}

template <typename T>
void launch_spmv(amie_topo *t, int grid, BsrView<T> A, const T *x, const T *b, T *y, double *part, cudaStream_t st)
{
    auto go = [&](auto g) {
        constexpr int G = decltype(g)::value;
        if (t->s == 2) k_spmv<2, G, T><<<grid, kVecThreads, 0, st>>>(A, x, b, y, part);
        else k_spmv<3, G, T><<<grid, kVecThreads, 0, st>>>(A, x, b, y, part);
    };
    dispatch_group<2, T>(t->spmv_group, go);
    AMIE_LAUNCHED();
}

BsrView<double> bsr64(amie_topo *t) { return BsrView<double>{t->n_rows, t->row_ptr.p, t->col.p, t->val.p}; }
BsrView<float> bsr32(amie_topo *t) { return BsrView<float>{t->n_rows, t->row_ptr.p, t->col.p, t->val32.p}; }

amie_status ensure_state(amie_topo *t, bool want32, SolverState **out)
{
    SolverState *s = state_of(t);
    if (!s) {
        s = new SolverState();
        {
            std::lock_guard<std::mutex> lk(g_state_mu);
            g_states[t] = s;
        }
        // Grid: resident CTAs of the SpMV kernel on every SM (a multiple of the SM count).
        int per_sm = 0;
        auto occ = [&](auto g) {
            constexpr int G = decltype(g)::value;
            if (t->s == 2)
                cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_spmv_pq<2, G, double>, kVecThreads, 0);
            else
                cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_spmv_pq<3, G, double>, kVecThreads, 0);
        };
        dispatch_group<2, double>(t->spmv_group, occ);
        per_sm = std::max(1, std::min(per_sm, 8));
        s->grid = t->ctx->num_sms * per_sm;
        auto resident = [&](const void *f, size_t smem) {
            int k = 0;
            if (smem > 48 * 1024) cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&k, f, kVecThreads, smem);
            return t->ctx->num_sms * std::max(1, std::min(k, 8));
        };
        size_t sm32 = 0, sm64 = 0;
        const void *k32 = (const void *)sell_kernel<float>(t->s, t->sell_variant, &sm32);
        const void *k64 = (const void *)sell_kernel<double>(t->s, t->sell_variant, &sm64);
        s->grid_sell[0] = resident(k32, sm32);
        s->grid_sell[1] = resident(k64, sm64);
        s->grid_vec[0] = resident((const void *)k_update<float>, 0);
        s->grid_vec[1] = resident((const void *)k_update<double>, 0);
        if (const char *e = std::getenv("AMIE_MATRIX_HINT")) s->matrix_hint = std::min(2, std::max(0, std::atoi(e)));
        if (const char *e = std::getenv("AMIE_PREFETCH_KB")) s->prefetch_bytes = (uint32_t)std::min(1024, std::max(0, std::atoi(e))) * 1024u;
        s->grid_dir[0] = resident(sell_dir_kernel<float>(t->s, s->matrix_hint), 0);
        s->grid_dir[1] = resident(sell_dir_kernel<double>(t->s, s->matrix_hint), 0);
        // A small system gets grids sized to its work (at least one CTA per SM,
        // a multiple of the SM count): a slice per warp of the SpMV kernels, one
        // two-pack step per thread of the vector kernels, so that fewer CTAs take
        // tickets and fewer partials are summed (AMIE_WORK_GRID=0: the resident
        // grids).  40 k-DOF P1, mixed: 18.4 instead of 22.4 ms per solve.  On the
        // 1.2 M-DOF P2 problem fewer update CTAs than resident cost more in steps
        // per thread than they save in tickets: 37.3 / 37.8 / 38.7 / 41.5 us per
        // FP32 iteration with 4 / 3 / 2 / 1 CTAs per SM.
        bool work_grid = true;
        if (const char *e = std::getenv("AMIE_WORK_GRID")) work_grid = std::atoi(e) != 0;
        if (work_grid) {
            const uint64_t sms = (uint64_t)t->ctx->num_sms;
            auto cap = [&](int g, uint64_t units, uint64_t per_cta) {
                const uint64_t want = (units + per_cta - 1) / per_cta;
                const uint64_t sized = std::max<uint64_t>(sms, (want + sms - 1) / sms * sms);
                return (int)std::min<uint64_t>((uint64_t)g, sized);
            };
            const uint64_t slices = std::max<uint64_t>(((uint64_t)t->n_rows + 31) / 32, 1);
            for (int k = 0; k < 2; k++) {
                s->grid_sell[k] = cap(s->grid_sell[k], slices, kVecThreads / 32);
                s->grid_dir[k] = cap(s->grid_dir[k], slices, kVecThreads / 32);
            }
            s->grid_vec[0] = cap(s->grid_vec[0], t->n, 2 * kVecThreads * Pack<float>::n);
            s->grid_vec[1] = cap(s->grid_vec[1], t->n, 2 * kVecThreads * Pack<double>::n);
        }
        s->grid_cgcg = std::min(resident(sell_cgcg_kernel<false>(t->s, s->matrix_hint), 0),
                                resident(sell_cgcg_kernel<true>(t->s, s->matrix_hint), 0));
        if (const char *e = std::getenv("AMIE_CGCG")) s->cgcg = std::atoi(e) != 0;
        s->grid_fused = resident(sell_fused_kernel(t->s, s->matrix_hint), 0);
        if (const char *e = std::getenv("AMIE_FUSED")) s->fused = std::atoi(e) != 0;
        {
            int coop = 0;
            cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, t->ctx->device);
            auto one_per_sm = [&](const void *f, int threads) {
                int k = 0;
                cudaOccupancyMaxActiveBlocksPerMultiprocessor(&k, f, threads, 0);
                return coop && k >= 1 ? t->ctx->num_sms : 0;
            };
            if (t->s == 2) {
                s->grid_persist[0] = one_per_sm((const void *)k_pcg_persist<2, float>, persist_threads<2, float>());
                s->grid_persist[1] = one_per_sm((const void *)k_pcg_persist<2, double>, persist_threads<2, double>());
            } else {
                s->grid_persist[0] = one_per_sm((const void *)k_pcg_persist<3, float>, persist_threads<3, float>());
                s->grid_persist[1] = one_per_sm((const void *)k_pcg_persist<3, double>, persist_threads<3, double>());
            }
            if (const char *e = std::getenv("AMIE_PERSIST")) s->persist_mode = std::atoi(e) != 0 ? 1 : 0;
            if (const char *e = std::getenv("AMIE_PERSIST_BARRIER_TEST")) s->persist_barrier_test = std::atoi(e) != 0;
            if (s->grid_persist[0] || s->grid_persist[1]) {
                AMIE_TRY(ensure_sell_partition(t, t->ctx->num_sms));
                AMIE_TRY(s->psync.alloc(t->ctx, 1));
                s->h_psync = (PersistSync *)pinned_get(sizeof(PersistSync));
                if (!s->h_psync) {
                    set_error("pinned host allocation failed");
                    return AMIE_OOM;
                }
            }
        }
        AMIE_CUDA(cudaGetLastError());
        AMIE_TRY(ensure_sell_partition(t, s->grid_cgcg));
        AMIE_TRY(ensure_sell_partition(t, s->grid));
        AMIE_TRY(ensure_sell_partition(t, s->grid_sell[0]));
        AMIE_TRY(ensure_sell_partition(t, s->grid_sell[1]));
        AMIE_TRY(ensure_sell_partition(t, s->grid_dir[0]));
        AMIE_TRY(ensure_sell_partition(t, s->grid_dir[1]));
        s->stride = std::max(std::max(std::max(s->grid, std::max(s->grid_vec[0], s->grid_vec[1])),
                                      std::max(s->grid_sell[0], s->grid_sell[1])),
                             std::max(std::max(s->grid_dir[0], s->grid_dir[1]),
                                      std::max(s->grid_cgcg, s->grid_fused)));
        // tuning overrides for measurements: AMIE_PDL=0 launches the PCG graph kernels plainly,
        // AMIE_FOLD_DIR=0 keeps the separate direction kernel (three kernels per iteration)
        if (const char *e = std::getenv("AMIE_PDL")) s->pdl = std::atoi(e) != 0;
        if (const char *e = std::getenv("AMIE_FOLD_DIR")) s->fold_dir = std::atoi(e) != 0;
        AMIE_TRY(s->parts.alloc(t->ctx, 5 * (size_t)s->stride));   // pq | rz | rr | spare (+ the fused kernel's fifth)
        AMIE_TRY(s->ctl.alloc(t->ctx, 1));
        s->h_ctl = (PcgCtl *)pinned_get(sizeof(PcgCtl));
        s->h_ring = (PcgCtl *)pinned_get(2 * sizeof(PcgCtl));
        if (!s->h_ctl || !s->h_ring) {
            set_error("pinned host allocation failed");
            return AMIE_OOM;
        }
        for (cudaEvent_t &e : s->ring_ev) AMIE_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        const uint64_t n = t->n;
        AMIE_TRY(t->r.alloc(t->ctx, n));
        AMIE_TRY(t->z.alloc(t->ctx, n));
        AMIE_TRY(t->p.alloc(t->ctx, n));
        AMIE_TRY(t->q.alloc(t->ctx, n));
        AMIE_TRY(t->p_alt.alloc(t->ctx, n));
    }
    if (want32 && !t->r32.p) {
        const uint64_t n = t->n;
        AMIE_TRY(t->r32.alloc(t->ctx, n));
        AMIE_TRY(t->z32.alloc(t->ctx, n));
        AMIE_TRY(t->p32.alloc(t->ctx, n));
        AMIE_TRY(t->q32.alloc(t->ctx, n));
        AMIE_TRY(t->d32.alloc(t->ctx, n));
        AMIE_TRY(t->p32_alt.alloc(t->ctx, n));
    }
    if (want32 && s->cgcg && !s->r32b.p) {
        const uint64_t n = t->n;
        AMIE_TRY(s->r32b.alloc(t->ctx, n));
        for (int k = 0; k < 2; k++) {
            AMIE_TRY(s->w32[k].alloc(t->ctx, n));
            AMIE_TRY(s->s32[k].alloc(t->ctx, n));
            AMIE_CUDA(cudaMemsetAsync(s->w32[k].p, 0, n * 4, t->ctx->stream));
            AMIE_CUDA(cudaMemsetAsync(s->s32[k].p, 0, n * 4, t->ctx->stream));
        }
        AMIE_TRY(s->slice3.alloc(t->ctx, 3 * (size_t)std::max<uint32_t>(t->n_slices, 1)));
        s->cg_cur = 0;
    }
    *out = s;
    return AMIE_OK;
}

PcgParts parts_of(SolverState *s)
{
    PcgParts p;
    p.pq = s->parts.p;
    p.rz = s->parts.p + s->stride;
    p.rr = s->parts.p + 2 * s->stride;
    p.spare = s->parts.p + 3 * s->stride;
    return p;
}

template <typename T>
PcgVecs<T> vecs_of(amie_topo *t);
template <>
PcgVecs<double> vecs_of<double>(amie_topo *t)
{
    return PcgVecs<double>{bsr64(t), t->invdiag.p, t->x.p, t->r.p, t->z.p, t->p.p, t->q.p, t->p_alt.p};
}
template <>
PcgVecs<float> vecs_of<float>(amie_topo *t)
{
    return PcgVecs<float>{bsr32(t), t->invdiag32.p, t->d32.p, t->r32.p, t->z32.p, t->p32.p, t->q32.p, t->p32_alt.p};
}

// q = A p with p = z + beta p formed inside the SpMV (two direction buffers, see
// k_sell_dir); false when the SELL copy or the CTA table for `grid` is missing.
template <typename T>
bool launch_spmv_dir(amie_topo *t, int grid, const PcgVecs<T> &v, double *part, PcgCtl *ctl, bool fin,
                     cudaStream_t st, bool pdl, int hint, uint32_t prefetch_bytes = 0)
{
    SellView<T> sv = sell_of<T>(t);
    sv.prefetch_bytes = prefetch_bytes;
    auto it = t->sell_cta_first.find(grid);
    if (!sv.val || it == t->sell_cta_first.end() || !v.p2) return false;
    sv.cta_first = it->second.p;
    auto kern = (void (*)(SellView<T>, PcgVecs<T>, double *, PcgCtl *, int))sell_dir_kernel<T>(t->s, hint);
    launch_k(pdl, kern, grid, 0, st, sv, v, part, ctl, fin ? 1 : 0);
    AMIE_LAUNCHED();
    return true;
}

constexpr int kGraphIters = 16;   // PCG iterations per graph launch

CgcgVecs<float> cgcg_vecs(amie_topo *t, SolverState *s)
{
    CgcgVecs<float> v;
    v.dinv = t->invdiag32.p;
    v.x = t->d32.p;
    v.p = t->p32.p;
    v.r[0] = t->r32.p;
    v.r[1] = s->r32b.p;
    v.w[0] = s->w32[0].p;
    v.w[1] = s->w32[1].p;
    v.s[0] = s->s32[0].p;
    v.s[1] = s->s32[1].p;
    v.slice3 = s->slice3.p;
    return v;
}

// One launch of k_sell_cgcg (start: the run's first pass).
void launch_cgcg(amie_topo *t, SolverState *s, bool start, bool pdl, cudaStream_t st)
{
    SellView<float> sv = sell_of<float>(t);
    sv.prefetch_bytes = s->prefetch_bytes;
    sv.cta_first = t->sell_cta_first.find(s->grid_cgcg)->second.p;
    auto kern = (void (*)(SellView<float>, CgcgVecs<float>, double *, PcgCtl *))(
        start ? sell_cgcg_kernel<true>(t->s, s->matrix_hint) : sell_cgcg_kernel<false>(t->s, s->matrix_hint));
    launch_k(pdl, kern, s->grid_cgcg, 0, st, sv, cgcg_vecs(t, s), parts_of(s).pq, s->ctl.p);
    AMIE_LAUNCHED();
}

amie_status graph_cgcg(amie_topo *t, SolverState *s)
{
    if (s->graph_cg) return AMIE_OK;
    cudaStream_t st = t->ctx->stream;
    cudaGraph_t graph = nullptr;
    AMIE_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    const uint64_t before = g_launches.load();
    for (int it = 0; it < kGraphIters; it++) launch_cgcg(t, s, false, s->pdl && it > 0, st);
    g_launches = before;   // captured, not launched: counted per graph launch
    AMIE_CUDA(cudaStreamEndCapture(st, &graph));
    cudaError_t e = cudaGraphInstantiate(&s->graph_cg, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
        s->graph_cg = nullptr;
        set_error("cudaGraphInstantiate: %s", cudaGetErrorString(e));
        return AMIE_CUDA_ERROR;
    }
    return AMIE_OK;
}

// Whether the mixed solver's FP32 runs use k_sell_cgcg (needs the FP32 SELL copy).
bool use_cgcg(amie_topo *t, SolverState *s)
{
    return s->cgcg && s->r32b.p && t->sell32_ok && t->sell_cta_first.count(s->grid_cgcg);
}

FusedVecs<float> fused_vecs(amie_topo *t, SolverState *s)
{
    FusedVecs<float> v;
    v.dinv = t->invdiag32.p;
    v.x = t->d32.p;
    v.r = t->r32.p;
    v.q = t->q32.p;
    v.p[0] = t->p32.p;
    v.p[1] = t->p32_alt.p;
    v.zw[0] = s->zw32[0].p;
    v.zw[1] = s->zw32[1].p;
    v.slice5 = s->slice5.p;
    return v;
}

// Buffers and CTA table of the one-kernel PCG (single solves only: the server's
// requests do not need them); false if it is off or the FP32 SELL copy is missing.
amie_status ensure_fused(amie_topo *t, SolverState *s, bool *on)
{
    *on = false;
    if (!s->fused || !t->sell32_ok || !t->r32.p) return AMIE_OK;
    if (!s->zw32[0].p) {
        const uint64_t n = t->n;
        for (int k = 0; k < 2; k++) {
            AMIE_TRY(s->zw32[k].alloc(t->ctx, 2 * n));
            AMIE_CUDA(cudaMemsetAsync(s->zw32[k].p, 0, 2 * n * 4, t->ctx->stream));
        }
        AMIE_TRY(s->slice5.alloc(t->ctx, 5 * (size_t)std::max<uint32_t>(t->n_slices, 1)));
        AMIE_TRY(ensure_sell_partition(t, s->grid_fused));
    }
    *on = t->sell_cta_first.count(s->grid_fused) != 0;
    return AMIE_OK;
}

// One launch of k_sell_fused.
void launch_fused(amie_topo *t, SolverState *s, bool pdl, cudaStream_t st)
{
    SellView<float> sv = sell_of<float>(t);
    sv.prefetch_bytes = s->prefetch_bytes;
    sv.cta_first = t->sell_cta_first.find(s->grid_fused)->second.p;
    auto kern = (void (*)(SellView<float>, FusedVecs<float>, double *, PcgCtl *))sell_fused_kernel(t->s, s->matrix_hint);
    launch_k(pdl, kern, s->grid_fused, 0, st, sv, fused_vecs(t, s), s->parts.p, s->ctl.p);
    AMIE_LAUNCHED();
}

amie_status graph_fused(amie_topo *t, SolverState *s)
{
    if (s->graph_fused) return AMIE_OK;
    cudaStream_t st = t->ctx->stream;
    cudaGraph_t graph = nullptr;
    AMIE_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    const uint64_t before = g_launches.load();
    for (int it = 0; it < kGraphIters; it++) launch_fused(t, s, s->pdl && it > 0, st);
    g_launches = before;   // captured, not launched: counted per graph launch
    AMIE_CUDA(cudaStreamEndCapture(st, &graph));
    cudaError_t e = cudaGraphInstantiate(&s->graph_fused, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
        s->graph_fused = nullptr;
        set_error("cudaGraphInstantiate: %s", cudaGetErrorString(e));
        return AMIE_CUDA_ERROR;
    }
    return AMIE_OK;
}

template <typename T>
amie_status graph_for(amie_topo *t, SolverState *s, cudaGraphExec_t *g)
{
    if (*g) return AMIE_OK;
    cudaStream_t st = t->ctx->stream;
    PcgVecs<T> v = vecs_of<T>(t);
    PcgParts parts = parts_of(s);
    cudaGraph_t graph = nullptr;
    AMIE_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    const int pi = sizeof(T) == 8 ? 1 : 0;
    const int gs = s->grid_sell[pi];
    const int gd = s->grid_dir[pi];
    const int gv = s->grid_vec[pi];
    const uint64_t n = t->n;
    PcgCtl *ctl = s->ctl.p;
    const uint64_t before = g_launches.load();
    for (int it = 0; it < kGraphIters; it++) {
        // the first kernel follows the previous graph launch in plain stream order
        if (fold<T>(s)) {
            launch_spmv_dir<T>(t, gd, v, parts.pq, ctl, true, st, s->pdl && it > 0, s->matrix_hint, s->prefetch_bytes);
            launch_k(s->pdl, k_update<T>, gv, 0, st, v, n, parts, ctl);
        } else {
            PcgVecs<T> v1 = v;
            v1.p2 = nullptr;   // one direction buffer: k_direction forms p
            launch_spmv_pq<T>(t, gs, v1, parts.pq, &ctl->done, ctl, st, s->pdl && it > 0);
            launch_k(s->pdl, k_update<T>, gv, 0, st, v1, n, parts, ctl);
            launch_k(s->pdl, k_direction<T>, gv, 0, st, v1, n, (const PcgCtl *)ctl);
        }
    }
    s->graph_kernels[pi] = fold<T>(s) ? 2 : 3;
    g_launches = before;   // captured, not launched: counted per graph launch
    AMIE_CUDA(cudaStreamEndCapture(st, &graph));
    cudaError_t e = cudaGraphInstantiate(g, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
        set_error("cudaGraphInstantiate: %s", cudaGetErrorString(e));
        return AMIE_CUDA_ERROR;
    }
    return AMIE_OK;
}

double sum_host(const double *p, int n)
{
    double s = 0.0;
    for (int i = 0; i < n; i++) s += p[i];
    return s;
}

// Sum of the first `n` doubles of a device array (partials), synchronously.
amie_status read_sum(amie_topo *t, const double *dev, int n, double *out)
{
    std::vector<double> h(n);
    AMIE_CUDA(cudaMemcpyAsync(h.data(), dev, n * sizeof(double), cudaMemcpyDeviceToHost, t->ctx->stream));
    AMIE_CUDA(cudaStreamSynchronize(t->ctx->stream));
    *out = sum_host(h.data(), n);
    return AMIE_OK;
}

// The run prepared in the control block as one cooperative launch of
// k_pcg_persist, when it is switched on and the system allows it (*used); the
// control block ends as the graph would leave it.
template <typename T>
amie_status run_persist(amie_topo *t, SolverState *s, int64_t *iters, double *rr_out, bool *used)
{
    *used = false;
    const int pi = sizeof(T) == 8 ? 1 : 0;
    const int grid = s->grid_persist[pi];
    // only runs whose graph folds the direction update (FP32): the others form p in
    // k_direction, on one buffer, and resume_pcg relies on that
    if (s->persist_mode == 0 || !grid || !fold<T>(s)) return AMIE_OK;
    SellView<T> sv = sell_of<T>(t);
    PcgVecs<T> v = vecs_of<T>(t);
    auto it = t->sell_cta_first.find(grid);
    if (!sv.val || !v.p2 || it == t->sell_cta_first.end()) return AMIE_OK;
    sv.cta_first = it->second.p;
    cudaStream_t st = t->ctx->stream;
    AMIE_CUDA(cudaMemsetAsync(s->psync.p, 0, sizeof(PersistSync), st));
    PcgParts parts = parts_of(s);
    uint64_t n = t->n;
    PcgCtl *ctl = s->ctl.p;
    PersistSync *sync = s->psync.p;
    uint32_t polls = s->persist_barrier_test ? 4096u : kPersistPolls;
    uint32_t expect = (uint32_t)grid + (s->persist_barrier_test ? 1u : 0u);
    void *args[] = {&sv, &v, &n, &parts, &ctl, &sync, &polls, &expect};
    const void *k = nullptr;
    int threads = 0;
    if (t->s == 2) {
        k = (const void *)k_pcg_persist<2, T>;
        threads = persist_threads<2, T>();
    } else {
        k = (const void *)k_pcg_persist<3, T>;
        threads = persist_threads<3, T>();
    }
    AMIE_CUDA(cudaLaunchCooperativeKernel(k, dim3((unsigned)grid), dim3((unsigned)threads), args, 0, st));
    AMIE_LAUNCHED();
    AMIE_CUDA(cudaMemcpyAsync(s->h_ctl, s->ctl.p, sizeof(PcgCtl), cudaMemcpyDeviceToHost, st));
    AMIE_CUDA(cudaMemcpyAsync(s->h_psync, s->psync.p, sizeof(PersistSync), cudaMemcpyDeviceToHost, st));
    AMIE_CUDA(cudaStreamSynchronize(st));
    if (s->h_psync->err) {
        set_error("persistent PCG: a grid barrier was not reached within %u polls (iterations %lld)", polls,
                  (long long)s->h_ctl->iterations);
        return AMIE_TIMEOUT;
    }
    *used = true;
    *iters = s->h_ctl->iterations;
    *rr_out = s->h_ctl->rr;
    return AMIE_OK;
}

// Launches the PCG graph until the control block reports done.
// Graphs of the FP32 runs: two-kernel standard PCG, single-reduction, one-kernel PCG.
enum class Graph { standard, cgcg, fused };

template <typename T>
amie_status drive_pcg(amie_topo *t, SolverState *s, int64_t maxit, int64_t *iters, double *rr_out,
                      Graph kind = Graph::standard)
{
    if (kind == Graph::standard) {
        bool used = false;
        AMIE_TRY(run_persist<T>(t, s, iters, rr_out, &used));
        if (used) return AMIE_OK;
    }
    cudaStream_t st = t->ctx->stream;
    cudaGraphExec_t *g = sizeof(T) == 8 ? &s->graph64 : &s->graph32;
    if (kind == Graph::cgcg) {
        AMIE_TRY(graph_cgcg(t, s));
        g = &s->graph_cg;
    } else if (kind == Graph::fused) {
        AMIE_TRY(graph_fused(t, s));
        g = &s->graph_fused;
    } else {
        AMIE_TRY(graph_for<T>(t, s, g));
    }
    // Host watchdog: the device sets `done` by maxit at the latest, so more
    // launches than maxit / kGraphIters + 2 mean the control block is not advancing.
    const int64_t max_launches = maxit / kGraphIters + 2;
    // Two graph launches stay in flight: the host reads the control block copied
    // after launch k while launch k + 1 runs, so the GPU does not idle during the
    // check.  A launch queued after the stop finds `done` set and its kernels
    // return at once.  Each ring slot is read only after its event completed.
    const int pi = sizeof(T) == 8 ? 1 : 0;
    const int per_iter = kind != Graph::standard ? 1 : s->graph_kernels[pi];
    auto launch = [&](int64_t k) -> amie_status {
        AMIE_CUDA(cudaGraphLaunch(*g, st));
        g_launches += per_iter * kGraphIters;
        AMIE_CUDA(cudaMemcpyAsync(s->h_ring + (k & 1), s->ctl.p, sizeof(PcgCtl), cudaMemcpyDeviceToHost, st));
        AMIE_CUDA(cudaEventRecord(s->ring_ev[k & 1], st));
        return AMIE_OK;
    };
    AMIE_TRY(launch(0));
    AMIE_TRY(launch(1));
    for (int64_t k = 0;; k++) {
        AMIE_CUDA(cudaEventSynchronize(s->ring_ev[k & 1]));
        const PcgCtl h = s->h_ring[k & 1];
        if (h.done) {
            *s->h_ctl = h;
            break;
        }
        if (k >= max_launches) {
            set_error("PCG control block stalled: %lld launches, iterations %lld, maxit %lld, rr %g, tol2 %g",
                      (long long)k, (long long)h.iterations, (long long)h.maxit, h.rr, h.tol2);
            return AMIE_TIMEOUT;
        }
        AMIE_TRY(launch(k + 2));
    }
    *iters = s->h_ctl->iterations;
    *rr_out = s->h_ctl->rr;
    return AMIE_OK;
}

// One PCG run from the residual already in v.r; stops when r.r <= tol2 or after maxit iterations.
template <typename T>
amie_status run_pcg(amie_topo *t, SolverState *s, double tol2, int64_t maxit, int64_t *iters, double *rr_out)
{
    cudaStream_t st = t->ctx->stream;
    PcgCtl init{};
    init.done = 0;
    init.ticket = 0;
    init.iterations = 0;
    init.maxit = maxit;
    init.tol2 = tol2;
    init.beta = 0.0;   // with the direction folded into the SpMV, the first p is z + 0 p
    init.pcur = 0;     // k_pcg_start writes p into the first buffer
    *s->h_ctl = init;
    AMIE_CUDA(cudaMemcpyAsync(s->ctl.p, s->h_ctl, sizeof(PcgCtl), cudaMemcpyHostToDevice, st));
    k_pcg_start<T><<<s->grid_vec[sizeof(T) == 8 ? 1 : 0], kVecThreads, 0, st>>>(vecs_of<T>(t), t->n, parts_of(s),
                                                                              s->ctl.p);   // rz, rr
    AMIE_LAUNCHED();
    // The pinned copy is rewritten by drive_pcg only after this copy has completed.
    AMIE_CUDA(cudaStreamSynchronize(st));
    return drive_pcg<T>(t, s, maxit, iters, rr_out);
}

// Continues a stopped run whose residual v.r was replaced (rescaled by
// `ratio`, see k_pcg_resume) with the previous search direction kept.
template <typename T>
amie_status resume_pcg(amie_topo *t, SolverState *s, double ratio, double tol2, int64_t maxit, int64_t *iters,
                       double *rr_out)
{
    cudaStream_t st = t->ctx->stream;
    const PcgVecs<T> v = vecs_of<T>(t);
    const int gv = s->grid_vec[sizeof(T) == 8 ? 1 : 0];
    k_pcg_resume<T><<<gv, kVecThreads, 0, st>>>(v, t->n, parts_of(s), s->ctl.p, ratio, tol2, maxit);
    g_launches += 1;
    if (!fold<T>(s)) {   // else the graph's first SpMV forms p = z + beta p from the latest p
        PcgVecs<T> v1 = v;
        v1.p2 = nullptr;
        k_direction<T><<<gv, kVecThreads, 0, st>>>(v1, t->n, s->ctl.p);
        g_launches += 1;
    }
    AMIE_CUDA(cudaGetLastError());
    return drive_pcg<T>(t, s, maxit, iters, rr_out);
}

// A single-reduction FP32 run from the residual in r[cg_cur]: scale = the
// previous run's residual scale over the new one to keep the search direction
// (reliable update), 0 for a fresh start.
amie_status run_cgcg(amie_topo *t, SolverState *s, double scale, double tol2, int64_t maxit, int64_t *iters,
                     double *rr_out)
{
    cudaStream_t st = t->ctx->stream;
    PcgCtl c = *s->h_ctl;   // the previous run's final state (gamma, alpha)
    c.done = 0;
    c.ticket = 0;
    c.iterations = 0;
    c.maxit = maxit;
    c.tol2 = tol2;
    c.pcur = s->cg_cur;
    c.pq = scale;
    if (scale != 0.0) {
        c.rz = c.rz * scale * scale;
        c.rz_prev = c.rz_prev * scale * scale;
    } else {
        c.rz = 0.0;
        c.rz_prev = 0.0;
        c.alpha = 0.0;
    }
    *s->h_ctl = c;
    AMIE_CUDA(cudaMemcpyAsync(s->ctl.p, s->h_ctl, sizeof(PcgCtl), cudaMemcpyHostToDevice, st));
    launch_cgcg(t, s, true, false, st);
    // the pinned copy is rewritten by drive_pcg only after this copy has completed
    AMIE_CUDA(cudaStreamSynchronize(st));
    AMIE_TRY(drive_pcg<float>(t, s, maxit, iters, rr_out, Graph::cgcg));
    s->cg_cur = s->h_ctl->pcur;
    return AMIE_OK;
}

// A one-kernel FP32 PCG run from the residual in r32: scale = the previous run's
// residual scale over the new one to keep its last direction (reliable update),
// 0 for a fresh start.
amie_status run_fused(amie_topo *t, SolverState *s, double scale, double tol2, int64_t maxit, int64_t *iters,
                      double *rr_out)
{
    cudaStream_t st = t->ctx->stream;
    PcgCtl c = *s->h_ctl;   // the previous run's final state (rz of its last direction)
    c.done = 0;
    c.ticket = 0;
    c.iterations = 0;
    c.maxit = maxit;
    c.tol2 = tol2;
    c.pcur = s->fused_cur;
    if (scale == 0.0) c.rz = 0.0;
    *s->h_ctl = c;
    AMIE_CUDA(cudaMemcpyAsync(s->ctl.p, s->h_ctl, sizeof(PcgCtl), cudaMemcpyHostToDevice, st));
    const int gv = s->grid_vec[0];
    if (t->s == 2) k_fused_prep<2, float><<<gv, kVecThreads, 0, st>>>(fused_vecs(t, s), t->n, scale, s->parts.p, s->ctl.p);
    else k_fused_prep<3, float><<<gv, kVecThreads, 0, st>>>(fused_vecs(t, s), t->n, scale, s->parts.p, s->ctl.p);
    AMIE_LAUNCHED();
    // the pinned copy is rewritten by drive_pcg only after this copy has completed
    AMIE_CUDA(cudaStreamSynchronize(st));
    AMIE_TRY(drive_pcg<float>(t, s, maxit, iters, rr_out, Graph::fused));
    s->fused_cur = s->h_ctl->pcur;
    return AMIE_OK;
}

__global__ void k_scale_to_f32(uint64_t n, const double *r, double inv, float *r32, float *d32)
{
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        r32[i] = (float)(r[i] * inv);
        d32[i] = 0.0f;
    }
}

__global__ void k_accumulate(uint64_t n, const float *d32, double scale, double *x)
{
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        x[i] += scale * (double)d32[i];
}

__global__ void k_norm2_parts(uint64_t n, const double *v, double *part)
{
    __shared__ double sh[33];
    double a = 0.0;
    for (uint64_t i = (uint64_t)blockIdx.x * kVecThreads + threadIdx.x; i < n; i += (uint64_t)gridDim.x * kVecThreads)
        a += v[i] * v[i];
    a = block_sum(a, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = a;
}

// r = b - A x in FP64; returns r.r.
amie_status true_residual(amie_topo *t, SolverState *s, double *rr)
{
    launch_spmv<double>(t, s->grid, bsr64(t), t->x.p, t->rhs.p, t->r.p, s->parts.p + 3 * s->stride, t->ctx->stream);
    AMIE_CUDA(cudaGetLastError());
    return read_sum(t, s->parts.p + 3 * s->stride, s->grid, rr);
}

amie_status solve_pcg(amie_topo *t, const amie_solve_opts *o, amie_solve_stats *st_out, bool mixed)
{
    SolverState *s = nullptr;
    AMIE_TRY(ensure_state(t, mixed, &s));
    if (mixed && !t->have32) AMIE_TRY(finalize_matrix_async(t, true));
    AMIE_TRY(ensure_sell(t, !mixed, mixed));   // before any graph of this topology is captured
    cudaStream_t st = t->ctx->stream;
    const double rtol = o && o->rtol > 0 ? o->rtol : 1e-10;
    const int64_t maxit = o && o->maxit > 0 ? o->maxit : std::max<int64_t>(1000, (int64_t)t->n);
    const bool caller_inner = o && o->inner_rtol > 0;
    double inner_rtol = caller_inner ? o->inner_rtol : kMixedInner;
    k_norm2_parts<<<s->grid, kVecThreads, 0, st>>>(t->n, t->rhs.p, s->parts.p);
    AMIE_LAUNCHED();
    double bb = 0.0;
    AMIE_TRY(read_sum(t, s->parts.p, s->grid, &bb));
    const double bnorm = std::sqrt(bb);
    st_out->iterations = 0;
    st_out->refinements = 0;
    if (bnorm == 0.0) {
        AMIE_CUDA(cudaMemsetAsync(t->x.p, 0, t->n * 8, st));
        AMIE_CUDA(cudaStreamSynchronize(st));
        st_out->relres = 0.0;
        st_out->status = AMIE_OK;
        return AMIE_OK;
    }
    double rr = 0.0;
    AMIE_TRY(true_residual(t, s, &rr));
    int64_t total = 0;
    double prev_norm = 0.0;   // MIXED: scale of the FP32 run's vectors (0 = no run yet)
    // the stop, as a fraction of rtol (mixed: kMixedStopLong once the run shows long
    // segments; AMIE_MIXED_STOP fixes it for measurements)
    double stop_fraction = 1.0;
    const char *stop_env = mixed ? std::getenv("AMIE_MIXED_STOP") : nullptr;
    if (stop_env) stop_fraction = std::min(1.0, std::max(0.01, std::atof(stop_env)));
    double target2 = (stop_fraction * rtol * bnorm) * (stop_fraction * rtol * bnorm);
    amie_status result = AMIE_NOT_CONVERGED;
    for (int outer = 0; outer < 200; outer++) {
        if (!(rr == rr)) { result = AMIE_NAN; break; }
        if (rr <= target2) { result = AMIE_OK; break; }
        if (total >= maxit) break;
        int64_t it = 0;
        double rr_in = 0.0;
        if (!mixed) {
            // recursive residual target a little below the true one (the true residual is re-checked)
            AMIE_TRY(run_pcg<double>(t, s, target2 * 0.25, maxit - total, &it, &rr_in));
        } else {
            // FP32 PCG on the residual scaled to unit norm; at each return the FP32
            // increment is added to x in FP64, r is replaced by the true FP64
            // residual and the FP32 run resumes with its search direction kept.
            const double norm = std::sqrt(rr);
            bool fz = false;
            AMIE_TRY(ensure_fused(t, s, &fz));
            const bool cg = !fz && use_cgcg(t, s);
            float *r32 = cg && s->cg_cur ? s->r32b.p : t->r32.p;
            k_scale_to_f32<<<s->grid, kVecThreads, 0, st>>>(t->n, t->r.p, 1.0 / norm, r32, t->d32.p);
            AMIE_LAUNCHED();
            // reduce by inner_rtol, or by less when that is all the outer target still needs
            const double need = kMixedLastTarget * rtol * bnorm / norm;
            const double inner = std::min(0.5, std::max(inner_rtol, need));
            // keep the search direction only while replacements show real progress; a
            // true residual that fell by less than half means the FP32 recursion has
            // drifted from it, and the run restarts from the new residual instead
            const bool fresh = prev_norm == 0.0 || norm > 0.5 * prev_norm;
            if (fz) AMIE_TRY(run_fused(t, s, fresh ? 0.0 : prev_norm / norm, inner * inner, maxit - total, &it, &rr_in));
            else if (cg) AMIE_TRY(run_cgcg(t, s, fresh ? 0.0 : prev_norm / norm, inner * inner, maxit - total, &it, &rr_in));
            else if (fresh) AMIE_TRY(run_pcg<float>(t, s, inner * inner, maxit - total, &it, &rr_in));
            else AMIE_TRY(resume_pcg<float>(t, s, norm / prev_norm, inner * inner, maxit - total, &it, &rr_in));
            prev_norm = norm;
            k_accumulate<<<s->grid, kVecThreads, 0, st>>>(t->n, t->d32.p, norm, t->x.p);
            AMIE_LAUNCHED();
            st_out->refinements++;
            if (it > kMixedLongSegment && !caller_inner && inner_rtol != kMixedInnerLong) {
                inner_rtol = kMixedInnerLong;   // a long, drift-prone FP32 run: see kMixedLongSegment
                if (!stop_env) {
                    stop_fraction = kMixedStopLong;
                    target2 = (stop_fraction * rtol * bnorm) * (stop_fraction * rtol * bnorm);
                }
            }
        }
        total += it;
        AMIE_TRY(true_residual(t, s, &rr));
        if (!mixed && it == 0) break;
    }
    if (!mixed && result == AMIE_OK && total > 0 && total < maxit &&
        !(rr <= target2 * (kFp64StopFraction * kFp64StopFraction))) {
        // Second stage of the FP64 stop: the same recursion continues (direction
        // kept) towards kFp64StopFraction rtol within a quarter more iterations;
        // its iterate is kept only if the true residual improved (a nearly
        // singular system may not get there, and then the first stage stands).
        if (!s->x_saved.p) AMIE_TRY(s->x_saved.alloc(t->ctx, t->n));
        AMIE_CUDA(cudaMemcpyAsync(s->x_saved.p, t->x.p, t->n * 8, cudaMemcpyDeviceToDevice, st));
        const int64_t extra = std::min<int64_t>(maxit - total, std::max<int64_t>(64, total / 4));
        int64_t it2 = 0;
        double rr_in = 0.0, rr2 = 0.0;
        AMIE_TRY(resume_pcg<double>(t, s, 1.0, target2 * (kFp64StopFraction * kFp64StopFraction), extra, &it2,
                                    &rr_in));
        AMIE_TRY(true_residual(t, s, &rr2));
        total += it2;
        if (rr2 <= rr) {
            rr = rr2;
        } else {
            AMIE_CUDA(cudaMemcpyAsync(t->x.p, s->x_saved.p, t->n * 8, cudaMemcpyDeviceToDevice, st));
        }
    }
    AMIE_CUDA(cudaGetLastError());
    st_out->iterations = total;
    st_out->relres = std::sqrt(rr) / bnorm;
    st_out->status = result;
    if (result != AMIE_OK)
        set_error("%s PCG stopped at relative residual %g (rtol %g) after %lld iterations, %d refinements",
                  mixed ? "mixed" : "FP64", st_out->relres, rtol, (long long)total, (int)st_out->refinements);
    return AMIE_OK;
}

}  // namespace amie

// The AMIE_CG control block starts with the same `done` flag as PcgCtl, so the
// SpMV kernel's early exit works with either.
#include "amie_cg.cuh"
#include "server.cuh"

namespace amie {

amie_status solve_dispatch(amie_topo *t, const amie_solve_opts *o, amie_solve_stats *stats)
{
    if (!t->assembled) {
        set_error("solve before amie_assemble");
        return AMIE_BAD_INPUT;
    }
    const int solver = o ? o->solver : AMIE_SOLVER_PCG_FP64;
    auto t0 = std::chrono::steady_clock::now();
    amie_status rc;
    if (solver == AMIE_SOLVER_PCG_FP64) rc = solve_pcg(t, o, stats, false);
    else if (solver == AMIE_SOLVER_PCG_MIXED) rc = solve_pcg(t, o, stats, true);
    else if (solver == AMIE_SOLVER_AMIE_CG) rc = amie_cg_solve(t, o, stats);
    else {
        set_error("unknown solver %d", solver);
        return AMIE_BAD_INPUT;
    }
    if (rc == AMIE_OK) AMIE_TRY(proportional_solution_async(t));
    AMIE_CUDA(cudaStreamSynchronize(t->ctx->stream));
    stats->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    t->last_solve_s = stats->seconds;
    return rc;
}

}  // namespace amie

using namespace amie;

extern "C" amie_status amie_solve_resident(amie_topo *t, const amie_solve_opts *o, amie_solve_stats *stats)
{
    if (!t) return AMIE_BAD_INPUT;
    AMIE_CUDA(cudaSetDevice(t->ctx->device));
    amie_solve_stats local{};
    amie_solve_stats *sp = stats ? stats : &local;
    if (!(o && o->use_x0)) AMIE_CUDA(cudaMemsetAsync(t->x.p, 0, t->n * 8, t->ctx->stream));
    AMIE_TRY(solve_dispatch(t, o, sp));
    return (amie_status)sp->status;
}

extern "C" amie_status amie_solve(amie_topo *t, const amie_solve_opts *o, double *x_inout, amie_solve_stats *stats)
{
    if (!t || !x_inout) return AMIE_BAD_INPUT;
    AMIE_CUDA(cudaSetDevice(t->ctx->device));
    cudaStream_t st = t->ctx->stream;
    if (o && o->use_x0) AMIE_CUDA(cudaMemcpyAsync(t->x.p, x_inout, t->n * 8, cudaMemcpyHostToDevice, st));
    else AMIE_CUDA(cudaMemsetAsync(t->x.p, 0, t->n * 8, st));
    amie_solve_stats local{};
    amie_solve_stats *sp = stats ? stats : &local;
    AMIE_TRY(solve_dispatch(t, o, sp));
    AMIE_CUDA(cudaMemcpyAsync(x_inout, t->x.p, t->n * 8, cudaMemcpyDeviceToHost, st));
    AMIE_CUDA(cudaStreamSynchronize(st));
    return (amie_status)sp->status;
}

namespace amie {

// x <- 2 x - x_hist, x_hist <- x (a NaN entry of x counts as 0): the
// displacement history step of Assembly::extrapolate with factor 1.
__global__ void k_extrapolate(uint64_t n, double *x, double *hist)
{
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const double u = x[i] == x[i] ? x[i] : 0.0;
        x[i] = u + (u - hist[i]);
        hist[i] = u;
    }
}

}  // namespace amie

extern "C" amie_status amie_extrapolate(amie_topo *t)
{
    if (!t || !t->x.p) return AMIE_BAD_INPUT;
    AMIE_CUDA(cudaSetDevice(t->ctx->device));
    cudaStream_t st = t->ctx->stream;
    if (!t->x_hist.p) {
        AMIE_TRY(t->x_hist.alloc(t->ctx, t->n));
        AMIE_CUDA(cudaMemsetAsync(t->x_hist.p, 0, t->n * 8, st));
    }
    k_extrapolate<<<t->ctx->num_sms * 4, 256, 0, st>>>(t->n, t->x.p, t->x_hist.p);
    AMIE_LAUNCHED();
    AMIE_CUDA(cudaGetLastError());
    return AMIE_OK;
}

extern "C" amie_status amie_solution_download(const amie_topo *t, double *x)
{
    if (!t || !x) return AMIE_BAD_INPUT;
    AMIE_CUDA(cudaSetDevice(t->ctx->device));
    AMIE_CUDA(cudaMemcpyAsync(x, t->x.p, t->n * 8, cudaMemcpyDeviceToHost, t->ctx->stream));
    AMIE_CUDA(cudaStreamSynchronize(t->ctx->stream));
    return AMIE_OK;
}

extern "C" amie_status amie_solution_upload(amie_topo *t, const double *x)
{
    if (!t || !x) return AMIE_BAD_INPUT;
    AMIE_CUDA(cudaSetDevice(t->ctx->device));
    AMIE_CUDA(cudaMemcpyAsync(t->x.p, x, t->n * 8, cudaMemcpyHostToDevice, t->ctx->stream));
    AMIE_CUDA(cudaStreamSynchronize(t->ctx->stream));
    return AMIE_OK;
}

extern "C" amie_status amie_timer_start(amie_ctx *ctx)
{
    if (!ctx) return AMIE_BAD_INPUT;
    AMIE_CUDA(cudaSetDevice(ctx->device));
    AMIE_CUDA(cudaEventRecord(ctx->ev0, ctx->stream));
    return AMIE_OK;
}

extern "C" amie_status amie_timer_stop(amie_ctx *ctx, double *ms)
{
    if (!ctx || !ms) return AMIE_BAD_INPUT;
    AMIE_CUDA(cudaSetDevice(ctx->device));
    AMIE_CUDA(cudaEventRecord(ctx->ev1, ctx->stream));
    AMIE_CUDA(cudaEventSynchronize(ctx->ev1));
    float f = 0.0f;
    AMIE_CUDA(cudaEventElapsedTime(&f, ctx->ev0, ctx->ev1));
    *ms = f;
    return AMIE_OK;
}

extern "C" amie_status amie_profile_spmv(amie_topo *t, int32_t precision, int32_t reps, double *ms_per_launch)
{
    if (!t || !ms_per_launch || reps <= 0 || (precision != 32 && precision != 64)) return AMIE_BAD_INPUT;
    if (!t->assembled) return AMIE_BAD_INPUT;
    AMIE_CUDA(cudaSetDevice(t->ctx->device));
    SolverState *s = nullptr;
    AMIE_TRY(ensure_state(t, precision == 32, &s));
    if (precision == 32 && !t->have32) AMIE_TRY(finalize_matrix_async(t, true));
    AMIE_TRY(ensure_sell(t, precision == 64, precision == 32));
    cudaStream_t st = t->ctx->stream;
    // zeroed inputs keep every value defined; the kernel's cost does not depend on them
    const size_t w = precision == 64 ? 8 : 4;
    void *vz = precision == 64 ? (void *)t->z.p : (void *)t->z32.p;
    void *vp = precision == 64 ? (void *)t->p.p : (void *)t->p32.p;
    void *vp2 = precision == 64 ? (void *)t->p_alt.p : (void *)t->p32_alt.p;
    AMIE_CUDA(cudaMemsetAsync(vz, 0, t->n * w, st));
    AMIE_CUDA(cudaMemsetAsync(vp, 0, t->n * w, st));
    AMIE_CUDA(cudaMemsetAsync(vp2, 0, t->n * w, st));
    // the SpMV kernel of the solver graph: with the direction folded in, beta = 0.5, first buffer current;
    // for the single-reduction iteration (the mixed solver's FP32 kernel when it is on) every
    // vector it touches zeroed and a stop that never triggers
    bool fz = false;
    if (precision == 32) AMIE_TRY(ensure_fused(t, s, &fz));
    const bool cg = precision == 32 && !fz && use_cgcg(t, s);
    PcgCtl c{};
    c.beta = 0.5;
    if (fz) {
        // the one-kernel PCG iteration (the mixed solver's FP32 kernel when it is on)
        const FusedVecs<float> v = fused_vecs(t, s);
        for (float *q : {v.x, v.r, v.q, v.p[0], v.p[1]}) AMIE_CUDA(cudaMemsetAsync(q, 0, t->n * 4, st));
        for (float *q : {v.zw[0], v.zw[1]}) AMIE_CUDA(cudaMemsetAsync(q, 0, 2 * t->n * 4, st));
        c.tol2 = -1.0;
        c.maxit = INT64_MAX;
    }
    if (cg) {
        const CgcgVecs<float> v = cgcg_vecs(t, s);
        for (float *q : {v.x, v.p, v.r[0], v.r[1], v.w[0], v.w[1], v.s[0], v.s[1]})
            AMIE_CUDA(cudaMemsetAsync(q, 0, t->n * 4, st));
        c.tol2 = -1.0;
        c.maxit = INT64_MAX;
    }
    *s->h_ctl = c;
    AMIE_CUDA(cudaMemcpyAsync(s->ctl.p, s->h_ctl, sizeof(PcgCtl), cudaMemcpyHostToDevice, st));
    PcgParts parts = parts_of(s);
    const int pi = precision == 64 ? 1 : 0;
    for (int i = 0; i <= reps; i++) {   // launch 0 is a warm-up
        if (i == 1) AMIE_CUDA(cudaEventRecord(t->ctx->ev0, st));
        if (fz) {
            launch_fused(t, s, false, st);
        } else if (cg) {
            launch_cgcg(t, s, false, false, st);
        } else if (precision == 32 && fold<float>(s)) {
            launch_spmv_dir<float>(t, s->grid_dir[pi], vecs_of<float>(t), parts.pq, s->ctl.p, false, st, false,
                                   s->matrix_hint);
        } else {
            if (precision == 64) launch_spmv_pq<double>(t, s->grid_sell[pi], vecs_of<double>(t), parts.pq, nullptr, nullptr, st);
            else launch_spmv_pq<float>(t, s->grid_sell[pi], vecs_of<float>(t), parts.pq, nullptr, nullptr, st);
        }
    }
    AMIE_CUDA(cudaEventRecord(t->ctx->ev1, st));
    AMIE_CUDA(cudaEventSynchronize(t->ctx->ev1));
    float f = 0.0f;
    AMIE_CUDA(cudaEventElapsedTime(&f, t->ctx->ev0, t->ctx->ev1));
    *ms_per_launch = (double)f / reps;
    return AMIE_OK;
}

namespace amie {

// Streaming read of n4 16-byte words, four independent loads per thread in flight.
__global__ void __launch_bounds__(kVecThreads) k_stream_read(const float4 *__restrict__ a, uint64_t n4, float *sink)
{
    float acc = 0.0f;
    const uint64_t stride = (uint64_t)gridDim.x * kVecThreads;
    uint64_t i = (uint64_t)blockIdx.x * kVecThreads + threadIdx.x;
    for (; i + 3 * stride < n4; i += 4 * stride) {
        float4 v[4];
#pragma unroll
        for (int u = 0; u < 4; u++) v[u] = __ldg(a + i + u * stride);
#pragma unroll
        for (int u = 0; u < 4; u++) acc += v[u].x + v[u].y + v[u].z + v[u].w;
    }
    for (; i < n4; i += stride) {
        const float4 v = __ldg(a + i);
        acc += v.x + v.y + v.z + v.w;
    }
    if (acc == 1234.5f) sink[blockIdx.x] = acc;   // keeps the loads; the buffers hold zeros
}

}  // namespace amie

extern "C" amie_status amie_profile_stream(amie_ctx *ctx, uint64_t bytes, int32_t reps, double *ms_per_launch)
{
    if (!ctx || !ms_per_launch || reps <= 0 || bytes < 16) return AMIE_BAD_INPUT;
    AMIE_CUDA(cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;
    const uint64_t flush_bytes = 512ull << 20;
    DevArray<float4> buf, flush;
    DevArray<float> sink;
    const int grid = ctx->num_sms * 8;
    AMIE_TRY(buf.alloc(ctx, bytes / 16));
    AMIE_TRY(flush.alloc(ctx, flush_bytes / 16));
    AMIE_TRY(sink.alloc(ctx, grid));
    AMIE_CUDA(cudaMemsetAsync(buf.p, 0, (bytes / 16) * 16, st));
    AMIE_CUDA(cudaMemsetAsync(flush.p, 0, flush_bytes, st));
    double total = 0.0;
    for (int i = 0; i <= reps; i++) {   // launch 0 is a warm-up
        k_stream_read<<<grid, kVecThreads, 0, st>>>(flush.p, flush_bytes / 16, sink.p);   // clean lines only
        AMIE_CUDA(cudaEventRecord(ctx->ev0, st));
        k_stream_read<<<grid, kVecThreads, 0, st>>>(buf.p, bytes / 16, sink.p);
        AMIE_CUDA(cudaEventRecord(ctx->ev1, st));
        AMIE_CUDA(cudaEventSynchronize(ctx->ev1));
        float f = 0.0f;
        AMIE_CUDA(cudaEventElapsedTime(&f, ctx->ev0, ctx->ev1));
        if (i > 0) total += f;
    }
    AMIE_CUDA(cudaGetLastError());
    *ms_per_launch = total / reps;
    return AMIE_OK;
}

extern "C" amie_status amie_spmv(amie_topo *t, const double *x, double *y)
{
    if (!t || !x || !y) return AMIE_BAD_INPUT;
    if (!t->assembled) return AMIE_BAD_INPUT;
    AMIE_CUDA(cudaSetDevice(t->ctx->device));
    SolverState *s = nullptr;
    AMIE_TRY(ensure_state(t, false, &s));
    cudaStream_t st = t->ctx->stream;
    AMIE_CUDA(cudaMemcpyAsync(t->p.p, x, t->n * 8, cudaMemcpyHostToDevice, st));
    launch_spmv<double>(t, s->grid, bsr64(t), t->p.p, nullptr, t->q.p, nullptr, st);
    AMIE_CUDA(cudaMemcpyAsync(y, t->q.p, t->n * 8, cudaMemcpyDeviceToHost, st));
    AMIE_CUDA(cudaStreamSynchronize(st));
    return AMIE_OK;
}
