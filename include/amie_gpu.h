/* amie_gpu.h -- C-ABI of the GB300 (sm_103a) implementation of AMIE's
 * finite-element hot path:
 *
 *   element stiffness  K_e = sum_g w_g B_i^T C B_j   (incl. XFEM enrichment)
 *   -> scatter into AMIE's block-sparse CoordinateIndexedSparseMatrix
 *   -> Dirichlet elimination
 *   -> Jacobi-preconditioned conjugate gradient (FP64, FP32-inner with FP64
 *      iterative refinement, or AMIE's own ConjugateGradient semantics)
 *
 * plus a continuous-batching solve server.
 *
 * Plain C types only: host pointers unless a name ends in `_dev`.  Every call
 * returns an amie_status.  The library owns all device memory it allocates;
 * callers own every host array they pass (arrays are read during the call
 * only).  Calls on one handle must not overlap; distinct handles may be driven
 * from distinct host threads.
 *
 * Reference interfaces (paths relative to the AMIE source tree) are cited at
 * each entry point.
 */
#ifndef AMIE_GPU_H
#define AMIE_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define AMIE_GPU_ABI_VERSION 2

#if defined(__GNUC__)
#define AMIE_API __attribute__((visibility("default")))
#else
#define AMIE_API
#endif

typedef enum amie_status {
    AMIE_OK = 0,
    AMIE_NOT_CONVERGED = 1,   /* ConjugateGradient::solve returned false (solvers/conjugategradient.cpp:316) */
    AMIE_NAN = 2,             /* NaN residual; the reference exit(0)s (solvers/conjugategradient.cpp:160-165) */
    AMIE_OOM = 3,             /* device allocation failed or would exceed the configured HBM budget */
    AMIE_BAD_INPUT = 4,       /* malformed arrays (ids out of range, counts inconsistent, ...) */
    AMIE_TIMEOUT = 5,         /* a bounded device wait or a server deadline ran out */
    AMIE_CUDA_ERROR = 6,      /* a CUDA runtime call failed; see amie_last_error() */
    AMIE_NOT_READY = 7,       /* amie_poll: the request is still running */
    AMIE_CANCELLED = 8        /* amie_poll: the request was cancelled */
} amie_status;

/* Element kinds (TriElement LINEAR / QUADRATIC, TetrahedralElement LINEAR). */
enum { AMIE_TRI3 = 1, AMIE_TRI6 = 2, AMIE_TET4 = 3 };
/* Enrichment function kinds. */
enum { AMIE_ENR_TABULATED = 0, AMIE_ENR_HEAVISIDE = 1, AMIE_ENR_TIP = 2 };
/* Multiplier kinds: displacement (SET_ALONG_* / FIX_ALONG_*, eliminated) or
 * nodal force (SET_FORCE_*, added to the right-hand side). */
enum { AMIE_BC_DISPLACEMENT = 0, AMIE_BC_FORCE = 1 };
/* Solver algorithms. */
enum {
    AMIE_SOLVER_PCG_FP64 = 0,   /* Jacobi-PCG, FP64 throughout, stop ||b-Ax|| <= rtol ||b|| */
    AMIE_SOLVER_PCG_MIXED = 1,  /* FP32 SpMV/preconditioner/direction updates inside an FP64
                                   iterative-refinement loop (FP64 residual, dots of the outer
                                   loop and solution accumulation) */
    AMIE_SOLVER_AMIE_CG = 2     /* ConjugateGradient::solve semantics: Jacobi smoothing,
                                   absolute stop sqrt(r.D^-1 r) < max(1e-12, eps), restarts */
};

typedef struct amie_ctx amie_ctx;
typedef struct amie_topo amie_topo;
typedef struct amie_server amie_server;

typedef struct amie_config {
    int32_t device;            /* CUDA device ordinal */
    uint64_t hbm_budget_bytes; /* 0 = no limit besides free memory */
    int32_t verbose;
} amie_config;

/* Element data of one mesh, as held by Assembly after FeatureTree::assemble
 * (features/features.cpp:3337-3408).  n_elem elements in Assembly::element2d /
 * element3d order, which is the order the reference scatters in
 * (solvers/assembly.cpp:657). */
typedef struct amie_mesh {
    int32_t dim;                 /* 2 or 3 */
    int32_t stride;              /* DOF per node: equals dim (elasticity) */
    uint32_t n_elem;
    uint32_t ndofmax;            /* Assembly::setMaxDof (solvers/assembly.h:286); 0 = max id + 1 */
    const uint8_t *kind;         /* [n_elem] AMIE_TRI3 / AMIE_TRI6 / AMIE_TET4 */
    const uint32_t *dof_ptr;     /* [n_elem+1] */
    const uint32_t *dof_ids;     /* getDofIds (elements/elements.cpp:204): node ids, then enrichment ids */
    const uint32_t *gp_ptr;      /* [n_elem+1]; an element with 0 points uses its kind's default rule */
    const double *gp;            /* (dim+1) per point: local coordinates, weight * det J */
    const double *jinv;          /* [n_elem*dim*dim] inverse Jacobian at the centroid, row-major */
    const uint8_t *moved;        /* [n_elem] or NULL: 1 = inverse Jacobian per Gauss point */
    const double *jinv_gp;       /* [n_gp*dim*dim], read for moved elements only */
    const uint32_t *mat;         /* [n_elem] row of cmat_table */
    const double *cmat_table;    /* [n_mat*nv*nv], nv = 3 (2D) or 6 (3D): Form::param */
    uint32_t n_mat;
    const double *cscale;        /* [n_elem] or NULL: factor on C ((1-d) damage, per-element modulus) */
    const double *scale;         /* [n_elem] or NULL: Assembly::add scale (solvers/assembly.cpp:106) */
    const uint32_t *enr_ptr;     /* [n_elem+1] or NULL: enrichment functions of element e */
    const uint8_t *enr_type;     /* [n_enr] AMIE_ENR_* */
    const uint8_t *enr_vertex;   /* [n_enr] P1 vertex (0,1,2) of a Heaviside function */
    const uint32_t *enr_data;    /* [n_enr] first per-GP entry of the function */
    uint64_t n_enr_gp;           /* entries of enr_jump / enr_grad (per dim) */
    const int8_t *enr_jump;      /* Heaviside: H(x_g) - H(x_k), per (function, GP) */
    const double *enr_grad;      /* Tabulated: local gradient, dim per (function, GP) */
    /* Tip branch functions of BranchedCrack::enrichTip (features/crack.cpp:898-960):
     * N_v^{P1} (F_j(x) - F_j(x_v)), F = sqrt(r) {sin(t/2), cos(t/2), sin(t/2) sin t,
     * cos(t/2) sin t}, r and t about the tip in the frame of the crack direction
     * (t as the reference's atan2 token gives it, see the implementation), on
     * straight-sided 2D elements; evaluated with their exact gradients at every
     * Gauss point (the reference differentiates them numerically, the two agree
     * to ~2e-9).  enr_data[f] of an AMIE_ENR_TIP function indexes a record of 8
     * doubles in enr_tip: x(0,0) - x_tip (2), dx/dxi (2), dx/deta (2) of the
     * element's map x(xi, eta) = x(0,0) + xi dx/dxi + eta dx/deta, the crack
     * angle at the tip, and the branch j (0..3). */
    const double *enr_tip;       /* [8 * n_enr_tip] or NULL */
    uint32_t n_enr_tip;
} amie_mesh;

typedef struct amie_solve_opts {
    int32_t solver;              /* AMIE_SOLVER_* */
    double rtol;                 /* relative residual target (PCG solvers); default 1e-10 */
    double eps;                  /* AMIE_CG absolute tolerance (Assembly::setEpsilon); default 1e-10 */
    int32_t nssor;               /* AMIE_CG smoothing sweeps (Assembly::setSSORIterations); default 32 */
    int64_t maxit;               /* iteration cap; <= 0 = reference default n/2 (AMIE_CG) / 20 n (PCG) */
    double inner_rtol;           /* MIXED: FP32 residual reduction between two FP64 residual replacements
                                    (reliable updates); <= 0 = 0.1, and 0.3 with the stop at 0.5 rtol
                                    once an FP32 run takes more than 1,000 iterations */
    int32_t use_x0;              /* 1 = start from x_inout (Assembly::extrapolate warm start) */
} amie_solve_opts;

typedef struct amie_solve_stats {
    int64_t iterations;          /* total (inner) CG iterations */
    int32_t refinements;         /* MIXED: outer refinement steps */
    int32_t status;              /* amie_status of the solve */
    double relres;               /* final true relative residual ||b - A x|| / ||b|| */
    double seconds;              /* wall time of the solve on the device */
} amie_solve_stats;

/* ------------------------------------------------------------------ context */
AMIE_API amie_status amie_ctx_create(const amie_config *cfg, amie_ctx **out);
AMIE_API amie_status amie_ctx_destroy(amie_ctx *ctx);
AMIE_API const char *amie_last_error(void);
AMIE_API int32_t amie_abi_version(void);

/* ------------------------------------------------------------------ topology
 * Uploads the element data and builds, on the device, the block sparsity
 * pattern of Assembly::make_final (solvers/assembly.cpp:445-537: every
 * (ids[j], ids[k]) pair, diagonal gap fill, (ndofmax-1, ndofmax-1)) and the
 * scatter map that assembles without atomics.  The pattern is bit-exact with
 * the reference's row_size / column_index. */
AMIE_API amie_status amie_topology_build(amie_ctx *ctx, const amie_mesh *mesh, amie_topo **out);
AMIE_API amie_status amie_topology_destroy(amie_topo *topo);
/* n_rows = block rows, nnzb = stored blocks, n = n_rows * stride scalar DOFs. */
AMIE_API amie_status amie_topology_sizes(const amie_topo *topo, uint32_t *n_rows, uint64_t *nnzb, uint64_t *n);
/* Lanes per block row the block SpMV uses for this topology (1, 2, 4, 8, 16 or 32),
 * chosen from the blocks per row at topology build.  No reference counterpart:
 * a kernel-configuration query for reports. */
AMIE_API amie_status amie_topology_spmv_lanes(const amie_topo *topo, int32_t *lanes);
/* row_size [n_rows] and column_index [nnzb] of CoordinateIndexedSparseMatrix
 * (sparse/sparse_matrix.h:129-179). */
AMIE_API amie_status amie_topology_pattern(const amie_topo *topo, uint32_t *row_size, uint32_t *column_index);

/* ------------------------------------------------------------------ assembly
 * Element matrices (DelaunayTriangle::getElementaryMatrix, mesher/delaunay.cpp:2408;
 * Stiffness::apply, physics/stiffness.cpp:43) and the Kahan-compensated
 * element-order scatter of Assembly::make_final (solvers/assembly.cpp:657-803)
 * into the device-resident block matrix.  Clears any previous Dirichlet
 * elimination and right-hand side. */
AMIE_API amie_status amie_assemble(amie_topo *topo);
/* Imposed strain per element (Voigt, [n_elem * nv]; NULL removes it).  Every
 * assembly then adds its induced forces sum_g w_g B_f^T (C eps0) per element
 * function to the right-hand side before the Dirichlet elimination
 * (StiffnessWithImposedStrain::getBoundaryConditions,
 * physics/stiffness_with_imposed_deformation.cpp:83-110, through
 * DofDefinedBoundaryCondition SET_VOLUMIC_STRESS_*, features/boundarycondition.cpp:542-617,
 * and Assembly::addForceOn, solvers/assembly.cpp:1477), and the recovered
 * stress is C (eps - eps0) (REAL_STRESS_FIELD).  C is the undamaged material
 * matrix in the forces, as in the reference.  Re-assembles an assembled topology. */
AMIE_API amie_status amie_set_imposed_strain(amie_topo *topo, const double *eps0);

/* Re-integrate with new per-element factors on C (damage step:
 * StiffnessAndFracture::apply, physics/stiffness_and_fracture.cpp:75-79). */
AMIE_API amie_status amie_set_cscale(amie_topo *topo, const double *cscale);
/* Element matrices as dense (nf*s)^2 row-major blocks, element after element. */
AMIE_API amie_status amie_element_matrices(const amie_topo *topo, double *ke, uint64_t capacity);

/* Dirichlet elimination of Assembly::setBoundaryConditions
 * (solvers/assembly.cpp:125-283) for multipliers set by Assembly::setPointAlong
 * (solvers/assembly.cpp:1590) or SET_FORCE_*.  rhs0: initial force vector
 * [n] or NULL (zero).  The multipliers stay on the device: every later
 * amie_assemble (a damage step, a new material factor) scatters and
 * eliminates again, as make_final does. */
AMIE_API amie_status amie_apply_dirichlet(amie_topo *topo, uint32_t n_bc, const uint32_t *ids, const double *values,
                                 const uint8_t *kinds, const double *rhs0);

/* Proportional displacements of Assembly::setPointProportional
 * (solvers/assembly.cpp:1636-1760; SET_PROPORTIONAL_DISPLACEMENT multipliers,
 * e.g. the inclined rollers SET_PROPORTIONAL_DISPLACEMENT_XI_ETA of
 * features/boundarycondition.cpp:256-264): u[ids[i]] = offsets[i] +
 * sum_k coefs[k] u[prop_ids[k]], k in [ptr[i], ptr[i+1]).  Stored on the
 * topology and applied after the Dirichlet elimination and the force
 * multipliers of every later elimination, multiplier after multiplier in the
 * order given (setBoundaryConditions, solvers/assembly.cpp:279-318: the DOF's
 * column moves onto its DOFs, its row is added to theirs, it becomes a unit row
 * with a zero right-hand side; an entry outside the pattern is dropped, as the
 * reference's sparse access drops it), and to the solution at the end of every
 * solve (Assembly::cgsolve, solvers/assembly.cpp:1881-1892).  An assembled
 * topology is assembled and eliminated again with every stored multiplier;
 * amie_assemble applies them with or without a Dirichlet list.  n = 0 removes
 * them.  A DOF carries one multiplier, as the reference's setters keep it (each
 * erases an earlier multiplier of its DOF): an id given twice here, or given
 * here and as a displacement to amie_apply_dirichlet (in either order), is
 * AMIE_BAD_INPUT and changes nothing. */
AMIE_API amie_status amie_set_proportional(amie_topo *topo, uint32_t n, const uint32_t *ids, const double *offsets,
                                           const uint32_t *ptr, const uint32_t *prop_ids, const double *coefs);

/* Matrix and right-hand side in AMIE's own layout (CoordinateIndexedSparseMatrix::array,
 * blocks column-major with even-padded columns, sparse/sparse_vector.cpp:50-58):
 * array [nnzb * s * (s + s%2)], rhs [n] (Assembly::getForces, solvers/assembly.h:343). */
AMIE_API amie_status amie_matrix_download(const amie_topo *topo, double *array, double *rhs);

/* y = A x on the device-resident matrix (CoordinateIndexedSparseMatrix::operator*,
 * sparse/sparse_matrix.cpp:505-547).  Host x, y of length n. */
AMIE_API amie_status amie_spmv(amie_topo *topo, const double *x, double *y);

/* ------------------------------------------------------------------ solve
 * Assembly::cgsolve (solvers/assembly.cpp:1829-1953) after make_final: solves
 * A x = rhs on the device.  x_inout [n] (host): warm start in (if use_x0),
 * solution out (Assembly::getDisplacements, solvers/assembly.h:349). */
AMIE_API amie_status amie_solve(amie_topo *topo, const amie_solve_opts *opts, double *x_inout, amie_solve_stats *stats);
/* Same, with the right-hand side and the solution left on the device (no host
 * copies); read the solution with amie_solution_download. */
AMIE_API amie_status amie_solve_resident(amie_topo *topo, const amie_solve_opts *opts, amie_solve_stats *stats);
AMIE_API amie_status amie_solution_download(const amie_topo *topo, double *x);
/* Warm start of the next amie_solve_resident (with use_x0) by the reference's
 * displacement-history extrapolation, Assembly::extrapolate (factor 1,
 * solvers/assembly.cpp:1772-1814) as cgsolve uses it (:1850-1867): the device
 * solution x becomes 2 x - x_prev and x_prev becomes x.  x_prev starts at zero,
 * like the history [0, u1] the reference keeps after its first solve; call it
 * once between consecutive solves of the same topology. */
AMIE_API amie_status amie_extrapolate(amie_topo *topo);

/* Jacobi-PCG (FP64, relative-residual stop) on a block-CSR matrix the caller
 * already holds in device memory, without allocating any device memory.  No
 * counterpart in the reference.  For callers that cannot call cudaMalloc at
 * solve time: applications whose own pool allocator took all device memory at
 * start-up (an allocation here would fail or break their accounting), and
 * real-time loops that cannot take the device-wide synchronisation that
 * cudaMalloc / cudaFree may cause.
 *   Matrix: row_ptr_dev [n_rows+1], col_dev [nnzb], val_dev [nnzb*s*s] (s x s
 *   blocks row-major, this library's device layout; columns of a row in any
 *   order, each at most once), b_dev, x_dev [n_rows*s]; x_dev is the warm
 *   start if use_x0, the solution on return.  stream: a cudaStream_t, or NULL
 *   for the default stream.  The call returns when the solve is finished: it
 *   synchronises `stream` to read the solver's progress.
 *   Limit: n_rows * stride <= 262144 scalar DOFs; larger systems return
 *   AMIE_BAD_INPUT.  The work vectors live in one static device array of about
 *   10.5 MB that every GPU loading this library reserves until exit.
 *   The first call on a device looks up that array's device address (set-up);
 *   make that first call before any stream capture.  Every call shares the
 *   array, so calls that overlap on the GPU race. */
AMIE_API amie_status amie_pcg_solve_noalloc(int32_t stride, uint32_t n_rows, const uint32_t *row_ptr_dev,
                                            const uint32_t *col_dev, const double *val_dev, const double *b_dev,
                                            double *x_dev, double rtol, int64_t maxit, int32_t use_x0, void *stream,
                                            amie_solve_stats *stats);

/* ------------------------------------------------------------------ serving
 * Continuous-batching solve server: independent meshes (2D or 3D elasticity:
 * microstructure or damage-step solves) are admitted while others run, as free
 * HBM allows; all admitted solves advance together in batched PCG iterations
 * captured in a CUDA graph, which also replaces the residuals of the solves
 * whose inner run stopped and decides on the device whether each is finished,
 * resumes or restarts.  Admission runs on two host threads (env
 * AMIE_SERVER_ADMITTERS, 1-8), the batch loop on a third. */
typedef struct amie_server_config {
    int32_t solver;              /* AMIE_SOLVER_PCG_FP64 or AMIE_SOLVER_PCG_MIXED */
    double rtol;                 /* per request relative residual target */
    uint64_t hbm_budget_bytes;   /* admission limit; 0 = 90% of free memory */
    int32_t max_slots;           /* concurrent solves; 0 = 256 */
    int32_t iters_per_launch;    /* PCG iterations per graph launch; 0 = 16 */
    uint32_t barrier_polls;      /* persistent batches (AMIE_SERVER_PERSISTENT=1): polls of a slot barrier
                                    before it gives up, ~64 ns each; 0 = 4,194,304 (~0.3 s).  A barrier that
                                    gives up ends the launch; the batch's requests end with AMIE_TIMEOUT and
                                    the server goes on serving. */
} amie_server_config;

typedef struct amie_request {
    const amie_mesh *mesh;       /* copied at submit */
    uint32_t n_bc;
    const uint32_t *bc_ids;
    const double *bc_values;
    const uint8_t *bc_kinds;
    const double *x0;            /* warm start [n] or NULL */
} amie_request;

typedef struct amie_result {
    int32_t status;              /* amie_status */
    int64_t iterations;
    double relres;
    double latency_s;            /* submit -> completion */
    double queue_s;              /* submit -> admission */
    uint64_t n;                  /* scalar DOFs */
} amie_result;

AMIE_API amie_status amie_server_start(amie_ctx *ctx, const amie_server_config *cfg, amie_server **out);
/* Copies the request; returns a ticket. */
AMIE_API amie_status amie_submit(amie_server *srv, const amie_request *req, uint64_t *ticket);
/* AMIE_NOT_READY while running; on completion fills res and, if x != NULL,
 * copies the solution [n]. */
AMIE_API amie_status amie_poll(amie_server *srv, uint64_t ticket, amie_result *res, double *x);
AMIE_API amie_status amie_cancel(amie_server *srv, uint64_t ticket);
/* Runs the server loop until every submitted request is finished or timeout_s elapses. */
AMIE_API amie_status amie_server_drain(amie_server *srv, double timeout_s);
AMIE_API amie_status amie_server_stop(amie_server *srv);

/* Where the server's host loop spent its time since start (seconds of wall
 * clock): admitting requests (topology, assembly, elimination, SELL copy),
 * waiting for batch graphs, residual replacements, joins; batches launched.
 * No reference counterpart: a report of the serving loop. */
typedef struct amie_server_stats {
    double admit_s, wait_s, advance_s, join_s, loop_s;
    uint64_t batches, admitted;
} amie_server_stats;
AMIE_API amie_status amie_server_query(amie_server *srv, amie_server_stats *stats);

/* ------------------------------------------------------------------ integration rules
 * Integration rules and Heaviside values of triangles crossed by a crack
 * polyline, generated on the device: DelaunayTriangle::getSubTriangulatedGaussPoints
 * (mesher/delaunay.cpp:2801-2985) for the hints BranchedCrack::enrichSegmentedLine
 * gives (features/crack.cpp:1088-1175), and the crack's Heaviside function
 * (PositionOperation::eval, polynomial/vm_token.cpp:258-271).
 * corners [n*6]: the corner vertices (x, y) at reference coordinates (0,1),
 * (0,0), (1,0); line [n_line*2]: the polyline (n_line >= 2, first segment not
 * empty); flags: 0 or AMIE_CUT_REPLACE_MONTE_CARLO.  Out: count [n] (points of
 * the rule, 0 unless status is AMIE_CUT_OK or AMIE_CUT_REPLACED), status [n]
 * (AMIE_CUT_*), rule [n*AMIE_CUT_MAX_POINTS*3] (xi, eta, weight times det J),
 * h_point [n*AMIE_CUT_MAX_POINTS] (Heaviside +-1 at each point), h_vertex [n*3]
 * (Heaviside at the corners, whatever the status).  The jump of the enrichment
 * function of corner k at point g is h_point[g] - h_vertex[k].
 * Without the flag, a status other than AMIE_CUT_OK leaves the element to the
 * caller's own rule (AMIE_CUT_MONTE_CARLO is where the reference falls back to
 * 512 random points).  With AMIE_CUT_REPLACE_MONTE_CARLO those elements, and the
 * order-dependent ones, get a deterministic crack-conforming rule instead
 * (AMIE_CUT_REPLACED): exact for the Heaviside integrand, so the element
 * matrices differ from the reference's Monte-Carlo ones by that method's error. */
#define AMIE_CUT_MAX_HINTS 6
#define AMIE_CUT_MAX_POINTS 52
#define AMIE_CUT_REPLACE_MONTE_CARLO 1u
enum {
    AMIE_CUT_OK = 0,
    AMIE_CUT_NOT_CUT = 1,           /* the polyline neither crosses the element nor ends in it */
    AMIE_CUT_MONTE_CARLO = 2,       /* fewer than three sub-triangles once close hints are dropped */
    AMIE_CUT_ORDER_DEPENDENT = 3,   /* two hints closer than the insertion tolerance 0.05 */
    AMIE_CUT_TOO_MANY_HINTS = 4,    /* more than AMIE_CUT_MAX_HINTS hints */
    AMIE_CUT_REPLACED = 5           /* deterministic rule where the reference uses Monte-Carlo */
};
AMIE_API amie_status amie_cut_rules(amie_ctx *ctx, uint32_t n, const double *corners, uint32_t n_line,
                                    const double *line, uint32_t flags, uint32_t *count, int8_t *status,
                                    double *rule, int8_t *h_point, int8_t *h_vertex);

/* ------------------------------------------------------------------ fields and damage
 * Per-element strain (Voigt, engineering shear: xx yy xy in 2D, xx yy zz yz xz xy
 * in 3D) and stress (C_eff strain) from the device-resident solution, averaged
 * over the element's Gauss points with their weights
 * (FeatureTree::strainFromDisplacements / stressFromDisplacements,
 * features/features.cpp:4223, 3424).  strain, stress: [n_elem * nv] host arrays or NULL. */
AMIE_API amie_status amie_element_fields(amie_topo *topo, double *strain, double *stress);

/* Field averaged over the mesh: sum_e v_e f_e / sum_e v_e with f_e the element's
 * Gauss-point average (as amie_element_fields) and v_e its area (2D: the
 * triangle of its corners, from J^-1 at the centroid) or volume (3D), Kahan
 * sums; FeatureTree::getAverageField (features/features.cpp:6711) through
 * Mesh::getField (mesher/mesh.h:919-960) and ElementState::getAverageField
 * (elements/integrable_entity.cpp:1992).  avg: [nv]; measure (nullable): sum v_e. */
enum { AMIE_FIELD_STRAIN = 0, AMIE_FIELD_STRESS = 1 };
AMIE_API amie_status amie_average_field(amie_topo *topo, int32_t field, double *avg, double *measure);

/* ------------------------------------------------------------------ damage
 * Non-local Mazars damage of StiffnessAndFracture (physics/stiffness_and_fracture.cpp:75-90)
 * on 2D linear triangles in plane stress, stepped the way FeatureTree::step does
 * it (features/features.cpp:6150-6270, stepElements :4875-5360):
 *   grade   FractureCriterion::step of every element (physics/fracturecriteria/fracturecriterion.cpp:534-560):
 *           the strain averaged over a smoothing neighbourhood (Mesh::getSmoothedFields,
 *           mesher/mesh.h:1384-1790, QUARTIC_COMPACT kernel of the material radius,
 *           neighbourhoods of FractureCriterion::initialiseCache, fracturecriterion.cpp:171-196),
 *           the element's damaged stress from it, their principal values, and
 *           NonLocalMazars::gradeAtTime (physics/fracturecriteria/mazars.cpp:73-147) -> score;
 *   update  FiberBasedIsotropicLinearDamage::step of every element in mesh order
 *           (physics/damagemodels/fiberbasedisotropiclineardamage.cpp:59-98): an element
 *           whose criterion is met and whose score is within score_tolerance of the
 *           largest score in its neighbourhood (FractureCriterion::getMaxScoreInNeighbourhood,
 *           fracturecriterion.cpp:251-280) gains fibre_fraction of damage; at cutoff it is
 *           fractured and keeps residual C (fiberbasedisotropiclineardamage.cpp:36-57).
 * The factor on C of every element follows its damage, so the next amie_assemble
 * integrates the damaged stiffness. */
enum { AMIE_DAMAGE_FIBER_ISOTROPIC = 0 };   /* FiberBasedIsotropicLinearDamage */
typedef struct amie_damage_law {
    int32_t model;             /* AMIE_DAMAGE_FIBER_ISOTROPIC */
    double threshold;          /* NonLocalMazars(thresh, E, nu, Gf, radius, PLANE_STRESS), mazars.cpp:27-35 */
    double young;
    double poisson;
    double fracture_energy;
    double radius;             /* material characteristic radius */
    double score_tolerance;    /* FractureCriterion scoreTolerance; <= 0: 2e-3 (fracturecriterion.cpp:77) */
    double fibre_fraction;     /* damage increment per event; <= 0: 0.1 */
    double cutoff;             /* fractured at this damage; <= 0: 0.6 */
    double residual;           /* stiffness fraction of a fractured element; <= 0: 1e-4 */
} amie_damage_law;

/* Geometry (centre, circumradius, area) and smoothing neighbourhoods of every
 * element, built on the device; damage starts at zero.  corners [n_elem*6]:
 * the three vertices (x, y) of each element in its local order.  Every element
 * must be an AMIE_TRI3 with at most one Gauss point and no enrichment. */
AMIE_API amie_status amie_damage_setup(amie_topo *topo, const amie_damage_law *law, const double *corners);
/* Damage of every element [n_elem] (host): set (NULL = zeros) or read. */
AMIE_API amie_status amie_damage_set_state(amie_topo *topo, const double *damage);
AMIE_API amie_status amie_damage_get_state(amie_topo *topo, double *damage);
/* Grade every element from the current solution; score [n_elem] (-1 for a
 * fractured element) and smoothed [n_elem*4] (principal smoothed stress, then
 * principal smoothed strain, each in toPrincipal's order) are optional host outputs.
 * Without `smoothed` (and in amie_damage_load_step) an element is not smoothed
 * where a bound shows its smoothed strain below the threshold: no unfractured
 * element of its neighbourhood's grid cells strains above it (the tensile
 * strain norm is convex, the smoothing an average); its score is then -d, the
 * same bits the smoothing gives. */
AMIE_API amie_status amie_damage_grade(amie_topo *topo, double *score, double *smoothed);
/* Step the damage model of every element from the last grade; n_changed:
 * elements whose damage grew. */
AMIE_API amie_status amie_damage_update(amie_topo *topo, uint32_t *n_changed);
/* Replace the device solution (the state amie_damage_grade reads) by x [n] (host). */
AMIE_API amie_status amie_solution_upload(amie_topo *topo, const double *x);

/* One load step with the multipliers of the last amie_apply_dirichlet: repeat
 * { assemble the damaged stiffness if the damage changed, eliminate, solve
 * (warm-started from the last solution), grade, update } until no element
 * changes or max_sub_iterations passes (FeatureTree::stepInternal's loop,
 * features/features.cpp:6188-6248; the reference solves three times per pass,
 * twice by CG and once by BiCGStab from the CG solution, this solves once). */
typedef struct amie_damage_step_stats {
    int32_t sub_iterations;    /* passes of the loop */
    int32_t status;            /* amie_status: AMIE_NOT_CONVERGED if max_sub_iterations ran out */
    int64_t cg_iterations;     /* solver iterations of all passes */
    uint32_t damaged;          /* elements with damage > 0 at the end */
    uint32_t fractured;        /* elements at the cutoff */
    uint64_t changes;          /* damage increments of all passes */
    uint64_t smoothed;         /* element smoothings of all passes (the others' scores were bounded) */
    double seconds;
} amie_damage_step_stats;
AMIE_API amie_status amie_damage_load_step(amie_topo *topo, const amie_solve_opts *opts, int32_t max_sub_iterations,
                                           amie_damage_step_stats *stats);

/* ------------------------------------------------------------------ timing
 * Device time on the context's stream (CUDA events) between start and stop;
 * stop synchronises the stream.  No counterpart in the reference, which
 * prints wall times only (solvers/assembly.cpp:1851-1853). */
AMIE_API amie_status amie_timer_start(amie_ctx *ctx);
AMIE_API amie_status amie_timer_stop(amie_ctx *ctx, double *ms);
/* Average device duration of the SpMV kernel of one PCG iteration as the solver
 * graph runs it (q = A p with the fused p.q; for precision 32 also the direction
 * update p = z + beta p, unless AMIE_FOLD_DIR=0) over `reps` back-to-back
 * launches on the current matrix; precision 64 (FP64 values) or 32 (FP32
 * values).  Used to report the kernel's achieved bandwidth against the HBM
 * roofline.  Overwrites the solver's work vectors. */
AMIE_API amie_status amie_profile_spmv(amie_topo *topo, int32_t precision, int32_t reps, double *ms_per_launch);

/* Average device duration of one plain streaming read of `bytes` bytes (16-byte
 * loads, one launch, L2 evicted by reading a 512 MB buffer before each launch)
 * over `reps` launches: the bandwidth a single launch of that size can reach,
 * reported beside the SpMV's.  No reference counterpart. */
AMIE_API amie_status amie_profile_stream(amie_ctx *ctx, uint64_t bytes, int32_t reps, double *ms_per_launch);

/* Number of kernels this library has launched (process-wide counter). */
AMIE_API uint64_t amie_kernel_launches(void);

#ifdef __cplusplus
}
#endif
#endif
