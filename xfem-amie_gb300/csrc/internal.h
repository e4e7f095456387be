// internal.h -- shared definitions of the GB300 FE hot-path library.
#pragma once

#include "amie_gpu.h"

#include <cuda_runtime.h>

#include <atomic>
#include <map>
#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

namespace amie {

constexpr int kSMs = 152;          // GB300: 2 dies x 76 SMs
constexpr int kMaxFunctions = 32;  // shape + enrichment functions per element
constexpr int kMaxGpWarpTile = 8;  // Gauss points staged per tile in the warp quadrature kernel
constexpr int kLongGp = 64;        // enriched elements with more Gauss points are split into chunks
constexpr int kChunkGp = 4;        // Gauss points per chunk of a long element (one warp each)

// One chunk of the Gauss points of a long enriched element and where its
// partial pair sums go; a long element and its chunks.
struct QuadChunk {
    uint32_t elem, gp_begin, gp_end;
    uint64_t out;
};
struct QuadLong {
    uint32_t elem, chunk_first, chunk_count;
};

void set_error(const char *fmt, ...);
extern std::atomic<uint64_t> g_launches;

#define AMIE_CUDA(call)                                                                     \
    do {                                                                                    \
        cudaError_t _e = (call);                                                            \
        if (_e != cudaSuccess) {                                                            \
            ::amie::set_error("%s:%d %s: %s", __FILE__, __LINE__, #call, cudaGetErrorString(_e)); \
            return _e == cudaErrorMemoryAllocation ? AMIE_OOM : AMIE_CUDA_ERROR;             \
        }                                                                                   \
    } while (0)

#define AMIE_TRY(expr)                       \
    do {                                     \
        amie_status _s = (expr);             \
        if (_s != AMIE_OK) return _s;        \
    } while (0)

#define AMIE_LAUNCHED() (::amie::g_launches.fetch_add(1, std::memory_order_relaxed))

// Device allocation tracked against the context's HBM budget.  A context with
// a memory pool allocates stream-ordered on its stream and frees on the
// calling thread's free stream (set_free_stream) or its own: no implicit
// device synchronisation, which matters where solves run beside admissions.
struct Ctx;
amie_status dev_alloc(Ctx *ctx, void **p, size_t bytes);
void dev_free(Ctx *ctx, void *p, size_t bytes);
void set_free_stream(cudaStream_t st);   // this thread's frees of pool memory follow st (nullptr: the context's)

// Small pinned host blocks, recycled instead of freed (cudaFreeHost waits for the device).
void *pinned_get(size_t bytes);
void pinned_put(void *p, size_t bytes);

template <typename T>
struct DevArray {
    T *p = nullptr;
    size_t n = 0;
    Ctx *ctx = nullptr;
    amie_status alloc(Ctx *c, size_t count)
    {
        release();
        ctx = c;
        n = count;
        if (count == 0) return AMIE_OK;
        return dev_alloc(c, (void **)&p, count * sizeof(T));
    }
    void release()
    {
        if (p) dev_free(ctx, p, n * sizeof(T));
        p = nullptr;
        n = 0;
    }
    size_t bytes() const { return n * sizeof(T); }
    ~DevArray() { release(); }
    DevArray() = default;
    DevArray(const DevArray &) = delete;
    DevArray &operator=(const DevArray &) = delete;
};

struct Ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    uint64_t budget = 0;
    std::atomic<uint64_t> allocated{0};
    int verbose = 0;
    int num_sms = kSMs;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    double *h_scalars = nullptr;  // pinned scratch for solver control reads
    cudaMemPool_t pool = nullptr; // stream-ordered allocations (the server's admission contexts)
};

// Device-side view of the element data used by the quadrature kernels.
struct MeshView {
    int dim, s, nv;
    uint32_t n_elem;
    const uint8_t *kind;
    const uint32_t *dof_ptr;
    const uint32_t *dof_ids;
    const uint32_t *gp_ptr;
    const double *gp;
    const double *jinv;
    const uint8_t *moved;
    const double *jinv_gp;
    const uint32_t *mat;
    const double *cmat_table;
    const double *cscale;
    const uint32_t *enr_ptr;
    const uint8_t *enr_type;
    const uint8_t *enr_vertex;
    const uint32_t *enr_data;
    const int8_t *enr_jump;
    const double *enr_grad;
    const double *enr_tip;    // tip branch-function records (8 doubles each)
    const uint64_t *blk_off;  // first staged block of each element (in s*s blocks)
    double *ke;               // staged element matrices: nf*nf blocks of s*s, row-major
    const double *imposed;    // imposed strain per element (Voigt, nv), or null
};

// Block-sparse matrix on the device: CSR over block rows, s x s blocks row-major.
template <typename T>
struct BsrView {
    uint32_t n_rows;
    const uint32_t *row_ptr;
    const uint32_t *col;
    const T *val;
};

// Sliced-ELL copy of a block-CSR matrix (SELL-32-sigma): block rows are
// sorted by length (descending, stable) inside windows of kSellSigma rows and
// cut into slices of 32; slice k holds 32 rows padded to its longest row, its
// slots stored j-major (slot = slice_ptr[k] + 32 j + lane) so a warp reads the
// j-th block of its 32 rows from one contiguous run.  Values of the 32 blocks
// of one j are stored in chunks of kSellVec<S,T> components, each chunk lane
// by lane: chunk k holds components kV .. kV+w-1 (w = min(V, S*S - kV)), and
// component c of lane l sits at val[32*S*S*(group) + 32*V*(c / V) + w*l + c % V]
// (sell_off), so a lane loads a chunk with one 16-byte access.  Padding slots
// have zero values and the row's own column (no effect on the result).
constexpr uint32_t kSellSigma = 128;
constexpr uint32_t kSellNone = 0xffffffffu;
template <int S, typename T>
constexpr int kSellVec = int(16 / sizeof(T)) > S * S ? 1 : (S == 2 || sizeof(T) == 4 ? int(16 / sizeof(T)) : 1);
template <int S, typename T>
__host__ __device__ constexpr int sell_off(int c, int lane)
{
    constexpr int V = kSellVec<S, T>;
    const int k = c / V;
    const int w = (S * S - k * V) < V ? (S * S - k * V) : V;
    return 32 * V * k + w * lane + c % V;
}

template <typename T>
struct SellView {
    uint32_t n_rows, n_slices;
    const uint32_t *perm;        // [32 * n_slices] block row of each lane (n_rows = padding)
    const uint64_t *slice_ptr;   // [n_slices + 1] first slot of each slice
    const uint32_t *col;         // [slots] block column
    const T *val;                // [slots * S * S] chunked as above
    const uint32_t *cta_first;   // [grid + 1] first slice of each CTA of the launch (slot-balanced ranges)
    T *slice_dot;                // [n_slices] per-slice partial of the fused dot product (scratch)
    uint32_t prefetch_bytes = 0; // k_sell_dir: L2 prefetch of the start of each CTA's range before its wait
};

}  // namespace amie

namespace amie {
struct DamageState;
}
void release_damage(amie_topo *t);   // damage.cu
void release_topology(amie_topo *t);   // assemble.cu: frees everything, no synchronisation
namespace amie {
amie_status proportional_solution_async(amie_topo *t);   // assemble.cu: u[id] = offset + sum c u[p]
}

// Opaque handles of the C-ABI.
struct amie_ctx : public amie::Ctx {};

struct amie_topo {
    amie_ctx *ctx = nullptr;
    int dim = 0, s = 0, nv = 0;
    uint32_t n_elem = 0, n_rows = 0, ndofmax = 0, n_mat = 0;
    uint64_t nnzb = 0, n = 0, n_blocks_staged = 0, n_contrib = 0;
    bool has_scale = false, has_cscale = false, has_moved = false;
    std::vector<uint32_t> h_dof_ptr;   // host copy (element matrix export)

    // element data
    amie::DevArray<uint8_t> kind, moved, enr_type, enr_vertex;
    amie::DevArray<uint32_t> dof_ptr, dof_ids, gp_ptr, mat, enr_ptr, enr_data;
    amie::DevArray<double> gp, jinv, jinv_gp, cmat_table, cscale, scale, enr_grad, enr_tip;
    amie::DevArray<int8_t> enr_jump;
    amie::DevArray<uint64_t> blk_off;
    amie::DevArray<uint32_t> simple_list, warp_list;   // elements per quadrature kernel
    uint32_t n_simple = 0, n_warp = 0;
    amie::DevArray<amie::QuadChunk> quad_chunks;         // long enriched elements, split by Gauss points
    amie::DevArray<amie::QuadLong> quad_long;
    amie::DevArray<double> quad_partial;
    uint32_t n_chunks = 0, n_long = 0;

    // staging + scatter map
    amie::DevArray<double> ke;
    amie::DevArray<uint32_t> map;        // staged block index per contribution, slot order
    amie::DevArray<uint64_t> map_ptr;    // [nnzb+1]
    amie::DevArray<uint32_t> blk_elem;   // staged block -> element (only with scale)

    // pattern + matrix
    amie::DevArray<uint32_t> row_ptr, col, diag_pos;
    amie::DevArray<double> val;
    amie::DevArray<float> val32;
    amie::DevArray<double> invdiag;
    amie::DevArray<float> invdiag32;
    bool assembled = false, eliminated = false, have32 = false;
    int spmv_group = 8;
    // SELL-32-sigma copy used by the solver SpMV (values converted on demand
    // after each change of the matrix)
    amie::DevArray<uint32_t> sell_perm, sell_col, sell_blk;   // sell_blk: BSR block per slot or kSellNone
    amie::DevArray<uint64_t> sell_ptr;
    amie::DevArray<double> sell_val;
    amie::DevArray<float> sell_val32;
    uint32_t n_slices = 0;
    uint64_t n_slots = 0;
    std::vector<uint64_t> h_sell_ptr;                          // host copy of sell_ptr
    amie::DevArray<double> sell_dot;                           // [n_slices] SpMV dot partials (FP32 or FP64)
    std::map<int, amie::DevArray<uint32_t>> sell_cta_first;   // per launch grid: slice ranges of the CTAs
    bool sell64_ok = false, sell32_ok = false;
    // SELL SpMV loop: 0 = 4 slots per step, 1 = 8, 2 = 2 pipelined, 3 = 4 pipelined,
    // 4 / 5 = 0 / 2 with registers capped for 5 CTAs per SM (2x2 FP32 blocks),
    // 6 / 7 = matrix streamed through shared memory by cp.async (2 slots x 4 stages / 4 x 3)
    int sell_variant = 0;

    // right-hand side, solution and solver work vectors
    amie::DevArray<double> rhs, x, r, z, p, q, xc, rc, red;
    amie::DevArray<float> r32, z32, p32, q32, d32;
    amie::DevArray<double> p_alt;     // second direction buffers of the PCG graphs
    amie::DevArray<float> p32_alt;
    amie::DevArray<uint8_t> fixed;
    amie::DevArray<double> fixval;
    amie::DevArray<double> strain;    // element strains (field recovery, damage grading)
    amie::DamageState *dmg = nullptr; // damage path (amie_damage_setup)
    amie::DevArray<double> x_hist;    // previous solution for amie_extrapolate (zero until first used)
    // imposed strain (per element) and its induced forces: staged per element
    // function, gathered per block row through fmap (contributions in element order)
    amie::DevArray<double> imposed, fstage;
    amie::DevArray<uint32_t> fmap, fmap_ptr;
    bool has_imposed = false;
    // Dirichlet / force multipliers and initial forces of the last
    // amie_apply_dirichlet; re-applied by every amie_assemble (make_final does
    // scatter + setBoundaryConditions in one call, solvers/assembly.cpp:803-816).
    amie::DevArray<uint32_t> bc_ids;
    amie::DevArray<double> bc_vals, rhs0;
    amie::DevArray<uint8_t> bc_kinds;
    uint32_t n_bc = 0;
    bool bc_set = false, has_rhs0 = false, has_bc_kinds = false;
    amie::DevArray<uint32_t> force_ids;   // the SET_FORCE multipliers among them, in order
    amie::DevArray<double> force_vals;
    uint32_t n_force = 0;
    bool force_unique = true;             // no DOF has two force multipliers
    // proportional displacements (amie_set_proportional), applied after the elimination
    amie::DevArray<uint32_t> prop_ids, prop_ptr, prop_dofs;
    amie::DevArray<double> prop_off, prop_coefs;
    uint32_t n_prop = 0;
    // sorted host copies for the check that no DOF is both fixed and proportional
    // (the reference's setters keep one multiplier per DOF)
    std::vector<uint32_t> fixed_sorted, prop_sorted;
    amie::DevArray<double> scal;   // solver scalars
    amie::DevArray<int32_t> flags; // solver control flags

    double last_solve_s = 0;
};
