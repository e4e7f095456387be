/* amie_oracle.h -- CPU restatement of AMIE's element-stiffness / block-sparse
 * scatter / Dirichlet elimination / Jacobi-preconditioned CG path.
 *
 * TEST INFRASTRUCTURE ONLY: the parity tests, the smoke check and the CPU
 * baseline of the benchmark call this library as the checker.  The GPU library
 * never links or loads it.
 *
 * Every function cites the reference code it restates (paths relative to the
 * AMIE source tree).  Matrices are in AMIE's CoordinateIndexedSparseMatrix
 * layout: block-CSR over node ids, each stride x stride block stored
 * column-major with columns padded to an even length
 * (sparse/sparse_vector.cpp:50-58, sparse/sparse_matrix.cpp:59).
 */
#ifndef AMIE_ORACLE_H
#define AMIE_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { ORACLE_TRI3 = 1, ORACLE_TRI6 = 2, ORACLE_TET4 = 3 };
enum { ORACLE_ENR_TABULATED = 0, ORACLE_ENR_HEAVISIDE = 1 };

/* Element data, same meaning as amie_mesh in include/amie_gpu.h. */
typedef struct oracle_mesh {
    int32_t dim;
    int32_t stride;
    uint32_t n_elem;
    uint32_t ndofmax;
    const uint8_t *kind;
    const uint32_t *dof_ptr;
    const uint32_t *dof_ids;
    const uint32_t *gp_ptr;     /* 0 GPs for an element = default rule of its kind */
    const double *gp;           /* (dim+1) per GP: local coords then weight */
    const double *jinv;         /* dim*dim per element, row-major */
    const uint8_t *moved;       /* per element, or NULL: 1 = use jinv_gp at each Gauss point */
    const double *jinv_gp;      /* dim*dim per Gauss point (read for moved elements only) */
    const uint32_t *mat;        /* material index per element */
    const double *cmat_table;   /* nv*nv per material, nv = 3 (2D) / 6 (3D) */
    const double *cscale;       /* per element factor on C, or NULL */
    const double *scale;        /* per element assembly scale, or NULL */
    const uint32_t *enr_ptr;    /* enrichment functions of element e: [enr_ptr[e], enr_ptr[e+1]) */
    const uint8_t *enr_type;
    const uint8_t *enr_vertex;
    const uint32_t *enr_data;   /* per function: offset of its per-GP entries */
    const int8_t *enr_jump;     /* Heaviside jump per (function, GP) */
    const double *enr_grad;     /* tabulated local gradient, dim per (function, GP) */
} oracle_mesh;

/* Element matrices K_e, dense (nf*s) x (nf*s) row-major, element e at ke + ke_off[e].
 * Restates DelaunayTriangle::getElementaryMatrix (mesher/delaunay.cpp:2408-2535),
 * Stiffness::apply (physics/stiffness.cpp:43-48), VirtualMachine::ieval(GtMtG)
 * (polynomial/vm_base.cpp:2974-2989) and geval (polynomial/vm_base.cpp:2156-2298). */
int oracle_element_matrices(const oracle_mesh *m, const uint64_t *ke_off, double *ke);

/* Sparsity pattern of Assembly::make_final (solvers/assembly.cpp:445-537).
 * Call once with row_size == NULL to get n_rows and nnzb, then with buffers. */
int oracle_induced_forces(const oracle_mesh *m, const double *imposed, double *force);
int oracle_pattern(const oracle_mesh *m, uint32_t *n_rows, uint64_t *nnzb, uint32_t *row_size,
                   uint32_t *column_index);

/* Kahan-compensated scatter of K_e into the padded block array
 * (solvers/assembly.cpp:657-734, 2D; 1060-1206, 3D). array is zeroed first. */
int oracle_scatter(const oracle_mesh *m, const uint64_t *ke_off, const double *ke, uint32_t n_rows,
                   const uint32_t *row_size, const uint32_t *column_index, double *array);

/* Dirichlet elimination of Assembly::setBoundaryConditions (solvers/assembly.cpp:125-260)
 * for SET_ALONG_* / FIX_ALONG_* multipliers (kind 0) and SET_FORCE_* (kind 1, added to rhs
 * afterwards, solvers/assembly.cpp:277-283). ids are scalar DOF ids. */
int oracle_dirichlet(int32_t stride, uint32_t n_rows, const uint32_t *row_size, const uint32_t *column_index,
                     double *array, uint32_t n_bc, const uint32_t *ids, const double *values,
                     const uint8_t *kinds, double *rhs);

/* y = A x (+ y0 if y0 != NULL), Kahan per output component, block order and
 * within-block order of CoordinateIndexedSparseMatrix::inner_product
 * (sparse/sparse_matrix.h:235-333). */
int oracle_spmv(int32_t stride, uint32_t n_rows, const uint32_t *row_size, const uint32_t *column_index,
                const double *array, const double *x, const double *y0, double *y);

/* ConjugateGradient::solve (solvers/conjugategradient.cpp:69-318) as driven by
 * Assembly::cgsolve: Jacobi preconditioner, nssor Jacobi pre/post smoothing,
 * Kahan-compensated updates, absolute stop sqrt(r.D^-1 r) < max(1e-12, eps),
 * outer restarts up to maxit (n/2 when maxit < 0).
 * Returns 0 converged, 1 not converged, 2 NaN residual. */
int oracle_cg_amie(int32_t stride, uint32_t n_rows, const uint32_t *row_size, const uint32_t *column_index,
                   const double *array, const double *b, double *x, double eps, int32_t nssor, int64_t maxit,
                   int64_t *iterations);

/* Textbook Jacobi-PCG with relative-residual stop ||b - A x|| <= rtol ||b||
 * (the GPU library's plain FP64 solver semantics).  Returns 0 converged. */
int oracle_pcg(int32_t stride, uint32_t n_rows, const uint32_t *row_size, const uint32_t *column_index,
               const double *array, const double *b, double *x, double rtol, int64_t maxit,
               int64_t *iterations, double *relres);

/* Per-element strain (Voigt, engineering shear) averaged over the element's Gauss
 * points with their weights, and stress = cscale C strain, from displacements u
 * (FeatureTree::strainFromDisplacements / stressFromDisplacements,
 * features/features.cpp:4223, 3424).  strain, stress: [n_elem * nv]. */
int oracle_element_fields(const oracle_mesh *m, const double *u, double *strain, double *stress);

/* ---- non-local Mazars damage on linear triangles (damage_oracle.cpp) ---- */

/* NonLocalMazars(threshold, young, poisson, fracture_energy, radius, PLANE_STRESS)
 * (physics/fracturecriteria/mazars.cpp:27-35) with a FiberBasedIsotropicLinearDamage
 * (physics/damagemodels/fiberbasedisotropiclineardamage.cpp:17-24): damage grows
 * by `fibre` per event, the element is fractured at `cutoff` and keeps
 * `residual` C; score_tolerance is FractureCriterion's scoreTolerance. */
typedef struct oracle_damage_law {
    double threshold, young, poisson, fracture_energy, radius;
    double score_tolerance, fibre, cutoff, residual;
} oracle_damage_law;

/* Centre, circumradius and area of each triangle from its corners [n*6]
 * (geometry/geometry_2D.cpp:480-515, 653-659). */
int oracle_damage_geometry(uint32_t n, const double *xy, double *centre, double *radius, double *area);
/* Smoothing cache of every element (Mesh::generateCache through
 * FractureCriterion::initialiseCache): CSR ptr [n+1], idx, normalised coef.
 * idx == NULL counts only. */
int oracle_damage_cache(uint32_t n, double R, const double *xy, const double *centre, const double *radius,
                        const double *area, uint64_t *ptr, uint32_t *idx, double *coef);
/* FractureCriterion::step of every element: score [n] (-1 fractured) and the
 * smoothed principal stress and strain [n*4], from element strains [n*3]
 * (Voigt, engineering shear), each element's undamaged C [n*9], damage state,
 * area and one-point Gauss weight gpw (weight times det J). */
int oracle_damage_grade(uint32_t n, const oracle_damage_law *law, const double *strain, const double *cmat,
                        const double *state, const double *area, const double *gpw, const uint64_t *ptr,
                        const uint32_t *idx, const double *coef, double *score, double *smoothed);
/* FiberBasedIsotropicLinearDamage::step of every element from the scores;
 * state updated in place, changed [n] set to 1 where it grew. */
int oracle_damage_update(uint32_t n, const oracle_damage_law *law, const double *centre, const double *radius,
                         const double *score, double *state, uint8_t *changed);

/* Number of OpenMP threads the oracle uses (for reporting). */
int oracle_threads(void);

#ifdef __cplusplus
}
#endif
#endif
