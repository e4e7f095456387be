// ref_harness.cpp -- drives the compiled AMIE reference library through its own
// public API (FeatureTree / Assembly / ConjugateGradient) and exports golden
// vectors for the oracle and the GPU parity tests.
//
// TEST INFRASTRUCTURE ONLY.  This program links the reference library built by
// oracle/Makefile (target `ref`) and is never part of the GPU product.
//
// What it exports, per case (one binary file of named arrays, see Out below):
//   * per element, in Assembly::element2d / element3d order (the order
//     Assembly::make_final scatters in, solvers/assembly.cpp:657):
//       kind, bounding-point coordinates, getDofIds() (elements/elements.cpp:204),
//       Gauss points + weights (already divided by det(J^-1), elements/elements.cpp:939),
//       the cached inverse Jacobian (mesher/delaunay.cpp:2436), the behaviour
//       tensor `param` (physics/stiffness.cpp:43), the assembly scale,
//       and for every enrichment function its P1 vertex, its value and its
//       finite-difference gradient at each Gauss point exactly as
//       VirtualMachine::deval produces them (polynomial/vm_base.cpp:1115);
//     the element matrix K_e returned by getElementaryMatrix
//     (mesher/delaunay.cpp:2408);
//   * the Dirichlet multipliers as Assembly::setPointAlong stored them
//     (solvers/assembly.cpp:1590);
//   * after Assembly::make_final: row_size, column_index and the padded,
//     column-major block array of CoordinateIndexedSparseMatrix
//     (sparse/sparse_matrix.cpp:59), and the right-hand side;
//   * the ConjugateGradient solution driven exactly as Assembly::cgsolve does
//     (solvers/assembly.cpp:1829-1850), its iteration count and wall time.
//
// Case `damage` (config-3 family): a notched beam in three-point bending with
// StiffnessAndFracture (physics/stiffness_and_fracture.cpp) graded by
// NonLocalMazars (physics/fracturecriteria/mazars.cpp:73-147) and damaged by
// FiberBasedIsotropicLinearDamage (the StiffnessAndFracture default,
// physics/damagemodels/fiberbasedisotropiclineardamage.cpp) or
// IsotropicLinearDamage (model=iso); FeatureTree::step per load step.  Exports
// the element data of the undamaged beam, each element's centre, circumradius
// and area, the supports and the load patch, and after every load step the
// displacements, the damage (1 - C_eff/C), the criterion's score and the
// smoothed principal stress and strain of every element.
//
// Usage:  ref_harness <case> <out.bin> [key=value ...]
//   case = incl | crack | voxel | plate | imposed | damage
//   keys: sampling, order (1|2), ninc, seed, E, nu, Einc, disp, size, crack_y,
//         n, nphase, sigma_log, strain

#include "features/features.h"
#include "features/sample.h"
#include "features/sample3d.h"
#include "features/inclusion.h"
#include "features/crack.h"
#include "physics/stiffness.h"
#include "physics/stiffness_with_imposed_deformation.h"
#include "physics/stiffness_and_fracture.h"
#include "physics/fracturecriteria/mazars.h"
#include "physics/damagemodels/isotropiclineardamage.h"
#include "physics/damagemodels/fiberbasedisotropiclineardamage.h"
#include "physics/void_form.h"
#include "utilities/placement.h"
#include "solvers/assembly.h"
#include "solvers/conjugategradient.h"
#include <cstdio>
#include <cstdint>
#include <cstring>
#include <map>
#include <random>
#include <string>
#include <vector>
#include <sys/time.h>

using namespace Amie;

namespace {

double now_s()
{
    timeval t;
    gettimeofday(&t, nullptr);
    return t.tv_sec + 1e-6 * t.tv_usec;
}

// Record stream: [u32 name_len][name][u8 type][u64 count][count * sizeof(type)]
// type: 'd' float64, 'i' int32, 'u' uint32, 'q' int64, 'b' int8.
struct Out {
    FILE *f = nullptr;
    explicit Out(const char *path) { f = std::fopen(path, "wb"); }
    ~Out() { if (f) std::fclose(f); }
    void put(const std::string &name, char type, const void *data, uint64_t count, size_t elsize)
    {
        uint32_t n = (uint32_t)name.size();
        std::fwrite(&n, 4, 1, f);
        std::fwrite(name.data(), 1, n, f);
        uint8_t t = (uint8_t)type;
        std::fwrite(&t, 1, 1, f);
        std::fwrite(&count, 8, 1, f);
        if (count) std::fwrite(data, elsize, count, f);
    }
    void d(const std::string &n, const std::vector<double> &v) { put(n, 'd', v.data(), v.size(), 8); }
    void u(const std::string &n, const std::vector<uint32_t> &v) { put(n, 'u', v.data(), v.size(), 4); }
    void i(const std::string &n, const std::vector<int32_t> &v) { put(n, 'i', v.data(), v.size(), 4); }
    void b(const std::string &n, const std::vector<int8_t> &v) { put(n, 'b', v.data(), v.size(), 1); }
    void scalar(const std::string &n, double x) { put(n, 'd', &x, 1, 8); }
};

std::map<std::string, std::string> parse_kv(int argc, char **argv, int first)
{
    std::map<std::string, std::string> kv;
    for (int a = first; a < argc; a++) {
        const char *eq = std::strchr(argv[a], '=');
        if (eq) kv[std::string(argv[a], eq - argv[a])] = std::string(eq + 1);
    }
    return kv;
}

double getd(std::map<std::string, std::string> &kv, const char *k, double def)
{
    auto it = kv.find(k);
    return it == kv.end() ? def : std::atof(it->second.c_str());
}

// Element kinds shared with the oracle and the GPU library.
enum { KIND_TRI3 = 1, KIND_TRI6 = 2, KIND_TET4 = 3 };

struct ElementExport {
    std::vector<uint32_t> kind, moved, dof_ptr{0}, dof_ids, gp_ptr{0}, enr_ptr{0}, enr_vertex, enr_gp_ptr{0};
    std::vector<double> xy, gp, jinv, jinv_gp, cmat, scale, enr_val, enr_grad, ke, imposed;
    std::vector<uint32_t> ke_ptr{0};
};

// Export one element (2D triangle or 3D tetrahedron).  `vertices` gives the
// Point* of the P1 vertices in shape-function order (first, second, third),
// used to identify which P1 shape function an enrichment function multiplies.
void export_element(IntegrableEntity *e, int dim, double scale, const std::vector<const Point *> &vertices,
                    VirtualMachine &vm, ElementExport &X)
{
    const size_t nshape = e->getShapeFunctions().size();
    const size_t nenr = e->getEnrichmentFunctions().size();
    const int s = dim;  // DOF per node (elasticity)
    std::valarray<std::valarray<Matrix>> &Ke = e->getElementaryMatrix(&vm);

    uint32_t kind = 0;
    if (dim == 2) kind = (nshape == 3) ? KIND_TRI3 : (nshape == 6 ? KIND_TRI6 : 0);
    else kind = (nshape == 4) ? KIND_TET4 : 0;
    X.kind.push_back(kind);

    for (size_t i = 0; i < nshape; i++) {
        const Point &p = e->getBoundingPoint(i);
        X.xy.push_back(p.getX());
        X.xy.push_back(p.getY());
        if (dim == 3) X.xy.push_back(p.getZ());
    }

    std::vector<size_t> ids = e->getDofIds();
    for (size_t id : ids) X.dof_ids.push_back((uint32_t)id);
    X.dof_ptr.push_back((uint32_t)X.dof_ids.size());

    const GaussPointArray &gpa = e->getGaussPoints();
    const size_t ngp = gpa.gaussPoints.size();
    for (size_t g = 0; g < ngp; g++) {
        X.gp.push_back(gpa.gaussPoints[g].first.getX());
        X.gp.push_back(gpa.gaussPoints[g].first.getY());
        if (dim == 3) X.gp.push_back(gpa.gaussPoints[g].first.getZ());
        X.gp.push_back(gpa.gaussPoints[g].second);
    }
    X.gp_ptr.push_back((uint32_t)(X.gp_ptr.back() + ngp));

    const Matrix &J = *e->getState().JinvCache;
    for (int r = 0; r < dim; r++)
        for (int c = 0; c < dim; c++) X.jinv.push_back(J[r][c]);
    // Elements whose nodes were projected on a curved boundary are "moved": their
    // inverse Jacobian is re-evaluated at every Gauss point (mesher/delaunay.cpp:2441-2447).
    X.moved.push_back(e->isMoved() ? 1u : 0u);
    for (size_t g = 0; g < ngp; g++) {
        Matrix Jg(dim, dim);
        if (e->isMoved()) e->getState().getInverseJacobianMatrix(gpa.gaussPoints[g].first, Jg);
        else Jg = J;
        for (int r = 0; r < dim; r++)
            for (int c = 0; c < dim; c++) X.jinv_gp.push_back(Jg[r][c]);
    }

    const Matrix &C = e->getBehaviour()->param;
    for (size_t r = 0; r < C.numRows(); r++)
        for (size_t c = 0; c < C.numCols(); c++) X.cmat.push_back(C[r][c]);
    X.scale.push_back(scale);
    // imposed strain of the behaviour (physics/stiffness_with_imposed_deformation.h), zeros otherwise
    const StiffnessWithImposedStrain *imp = dynamic_cast<const StiffnessWithImposedStrain *>(e->getBehaviour());
    for (size_t k = 0; k < C.numRows(); k++) X.imposed.push_back(imp && k < imp->imposed.size() ? imp->imposed[k] : 0.0);

    for (size_t j = 0; j < nenr; j++) {
        const Function &f = e->getEnrichmentFunction(j);
        uint32_t vtx = 255;
        for (size_t k = 0; k < vertices.size(); k++)
            if (f.getPoint() == vertices[k]) vtx = (uint32_t)k;
        X.enr_vertex.push_back(vtx);
        for (size_t g = 0; g < ngp; g++) {
            const Point &p = gpa.gaussPoints[g].first;
            X.enr_val.push_back(vm.eval(f, p));
            X.enr_grad.push_back(vm.deval(f, XI, p));
            X.enr_grad.push_back(vm.deval(f, ETA, p));
            if (dim == 3) X.enr_grad.push_back(vm.deval(f, ZETA, p));
        }
        X.enr_gp_ptr.push_back((uint32_t)(X.enr_gp_ptr.back() + ngp));
    }
    X.enr_ptr.push_back((uint32_t)X.enr_vertex.size());

    // K_e as a dense (nf*s) x (nf*s) row-major matrix.
    const size_t nf = nshape + nenr;
    const size_t m = nf * s;
    std::vector<double> dense(m * m, 0.0);
    for (size_t a = 0; a < nf; a++)
        for (size_t b = 0; b < nf; b++)
            for (int r = 0; r < s; r++)
                for (int c = 0; c < s; c++) dense[(a * s + r) * m + b * s + c] = Ke[a][b][r][c];
    X.ke.insert(X.ke.end(), dense.begin(), dense.end());
    X.ke_ptr.push_back((uint32_t)X.ke.size());
}

void write_elements(Out &o, ElementExport &X)
{
    o.u("elem_kind", X.kind);
    o.d("elem_xy", X.xy);
    o.u("elem_dof_ptr", X.dof_ptr);
    o.u("elem_dof_ids", X.dof_ids);
    o.u("gp_ptr", X.gp_ptr);
    o.d("gp", X.gp);
    o.d("jinv", X.jinv);
    o.u("elem_moved", X.moved);
    o.d("jinv_gp", X.jinv_gp);
    o.d("cmat", X.cmat);
    o.d("elem_scale", X.scale);
    o.u("enr_ptr", X.enr_ptr);
    o.u("enr_vertex", X.enr_vertex);
    o.u("enr_gp_ptr", X.enr_gp_ptr);
    o.d("enr_val", X.enr_val);
    o.d("enr_grad", X.enr_grad);
    o.u("ke_ptr", X.ke_ptr);
    o.d("ke", X.ke);
    o.d("elem_imposed", X.imposed);
}

// Dirichlet multipliers as stored by the Assembly (before make_final sorts them);
// a SET_PROPORTIONAL_DISPLACEMENT multiplier (u_id = offset + sum coefs u_propid,
// Assembly::setPointProportional, solvers/assembly.cpp:1636-1760) also gives its
// DOFs and coefficients (bc_prop_ptr / bc_prop_ids / bc_prop_coefs).
void write_multipliers(Out &o, Assembly *K)
{
    std::vector<uint32_t> ids, types, pptr{0}, pids;
    std::vector<double> vals, pco;
    for (auto &m : K->multipliers) {
        ids.push_back((uint32_t)m.getId());
        types.push_back((uint32_t)m.type);
        vals.push_back(m.getValue());
        if (m.type == SET_PROPORTIONAL_DISPLACEMENT) {
            const std::valarray<unsigned int> d = m.getDofIds();
            for (size_t k = 0; k < d.size(); k++) {
                pids.push_back(d[k]);
                pco.push_back(m.coefs[k]);
            }
        }
        pptr.push_back((uint32_t)pids.size());
    }
    o.u("bc_ids", ids);
    o.u("bc_types", types);
    o.d("bc_values", vals);
    o.u("bc_prop_ptr", pptr);
    o.u("bc_prop_ids", pids);
    o.d("bc_prop_coefs", pco);
}

// make_final + the ConjugateGradient call of Assembly::cgsolve, then export.
void finish_and_solve(Out &o, Assembly *K)
{
    double t0 = now_s();
    K->make_final();
    double t1 = now_s();
    CoordinateIndexedSparseMatrix &A = K->getMatrix();
    std::vector<uint32_t> rs(std::begin(A.row_size), std::end(A.row_size));
    std::vector<uint32_t> ci(std::begin(A.column_index), std::end(A.column_index));
    std::vector<double> arr(std::begin(A.array), std::end(A.array));
    o.u("row_size", rs);
    o.u("column_index", ci);
    o.d("array", arr);
    o.scalar("stride", (double)A.stride);
    std::vector<double> b(std::begin(K->getForces()), std::end(K->getForces()));
    o.d("rhs", b);

    ConjugateGradient cg(K);
    cg.nssor = K->nssor;
    double t2 = now_s();
    bool ok = cg.solve(K->extrapolate(), nullptr, K->epsilon, -1, false);
    double t3 = now_s();
    std::vector<double> x(std::begin(cg.x), std::end(cg.x));
    o.d("u", x);
    // the displacements Assembly::cgsolve reports: a proportional multiplier's DOF
    // set from its DOFs after the solve, in multiplier order (solvers/assembly.cpp:1881-1892)
    std::vector<double> xp(x);
    for (auto &m : K->multipliersBuffer)   // filled by setBoundaryConditions in multiplier order
        if (m.type == SET_PROPORTIONAL_DISPLACEMENT) {
            const std::valarray<unsigned int> d = m.getDofIds();
            double v = m.getValue();
            for (size_t k = 0; k < d.size(); k++) v += m.coefs[k] * xp[d[k]];
            xp[m.getId()] = v;
        }
    o.d("u_post", xp);
    o.scalar("cg_iterations", (double)cg.nit);
    o.scalar("cg_converged", ok ? 1.0 : 0.0);
    o.scalar("epsilon", K->epsilon);
    o.scalar("nssor", (double)K->nssor);
    o.scalar("time_make_final_s", t1 - t0);
    o.scalar("time_cg_s", t3 - t2);
    std::fprintf(stderr, "harness: n=%zu nnzb=%zu iterations=%zu converged=%d make_final=%.3fs cg=%.3fs\n",
                 x.size(), ci.size(), (size_t)cg.nit, (int)ok, t1 - t0, t3 - t2);
}

int run_2d(const std::string &which, Out &o, std::map<std::string, std::string> &kv)
{
    const double L = getd(kv, "size", 0.04);
    const double E = getd(kv, "E", 30e9), nu = getd(kv, "nu", 0.2);
    const double Einc = getd(kv, "Einc", 60e9);
    const int ninc = (int)getd(kv, "ninc", 0);
    const int seed = (int)getd(kv, "seed", 7);
    const double sampling = getd(kv, "sampling", 16);
    const int order = (int)getd(kv, "order", 1);
    const double disp = getd(kv, "disp", 1e-5);

    RectangularFeature box(nullptr, L, L, 0, 0);
    if (which == "imposed")
        // the behaviour examples/test/test_stiffness_with_imposed_deformation.ini builds through
        // utilities/object_translator.cpp:289-295 (the (E, nu, alpha) constructor)
        box.setBehaviour(new StiffnessWithImposedStrain(E, nu, getd(kv, "imposed", 1e-3), SPACE_TWO_DIMENSIONAL,
                                                        PLANE_STRESS, YOUNG_POISSON));
    else
        box.setBehaviour(new Stiffness(E, nu, SPACE_TWO_DIMENSIONAL, PLANE_STRESS));
    FeatureTree F(&box);

    std::vector<Feature *> placed;
    if (ninc > 0) {
        std::mt19937 gen(seed);
        std::uniform_real_distribution<double> rd(getd(kv, "rmin", 0.3e-3), getd(kv, "rmax", 1.5e-3));
        std::vector<Feature *> incs;
        for (int k = 0; k < ninc; k++) incs.push_back(new Inclusion(rd(gen), 0., 0.));
        placed = placement2D(dynamic_cast<Rectangle *>(&box), incs, 1e-5, 0, 64000, M_PI,
                             std::vector<Geometry *>(), seed);
        for (auto f : placed) {
            f->setBehaviour(new Stiffness(Einc, nu, SPACE_TWO_DIMENSIONAL, PLANE_STRESS));
            F.addFeature(&box, f);
        }
    }
    if (which == "crack") {
        const double y0 = getd(kv, "crack_y", 0.0013);
        BranchedCrack *c = new BranchedCrack(&box, new Point(-L / 2 + 1e-4, y0), new Point(-L / 2 + 0.3 * L, y0));
        F.addFeature(&box, c);
    }
    std::vector<BoundaryCondition *> bcs = {
        new BoundingBoxDefinedBoundaryCondition(FIX_ALONG_XI, BOTTOM),
        new BoundingBoxDefinedBoundaryCondition(FIX_ALONG_ETA, BOTTOM),
        new BoundingBoxDefinedBoundaryCondition(SET_ALONG_ETA, TOP, disp)};
    if (which == "imposed") {
        // examples/main_check_behaviour.cpp with --free: the plate is held by rollers only
        // and expands under its imposed strain; the reference's known answer is
        // strain_yy * 1e3 = 1, stress_yy / 1e6 = 0
        // (examples/test/check_behaviour_test_stiffness_with_imposed_deformation_base).
        bcs = {new BoundingBoxDefinedBoundaryCondition(FIX_ALONG_ETA, BOTTOM),
               new BoundingBoxDefinedBoundaryCondition(FIX_ALONG_XI, BOTTOM_LEFT)};
    }
    if (which == "plate") {
        // examples/main_check_behaviour.cpp with examples/test/test_stiffness.ini:
        // 10 x 10 mm plate, E = 10 GPa, nu = 0.2, 1 MPa imposed as a stress on TOP;
        // the reference's known answer is strain_yy * 1e3 = 0.1, stress_yy / 1e6 = 1
        // (examples/test/check_behaviour_test_stiffness_base).
        bcs = {new BoundingBoxDefinedBoundaryCondition(FIX_ALONG_ETA, BOTTOM),
               new BoundingBoxDefinedBoundaryCondition(FIX_ALONG_XI, BOTTOM_LEFT),
               new BoundingBoxDefinedBoundaryCondition(SET_STRESS_ETA, TOP, getd(kv, "stress", 1e6))};
    }
    if (getd(kv, "prop", 0.0) != 0.0)   // an inclined roller on RIGHT: u_x = prop * u_y
        bcs.push_back(new BoundingBoxDefinedBoundaryCondition(SET_PROPORTIONAL_DISPLACEMENT_XI_ETA, RIGHT,
                                                              getd(kv, "prop", 0.0)));
    F.setSamplingNumber(sampling);
    if (order == 2) F.setOrder(QUADRATIC);

    Assembly *K = F.getAssembly(true);
    VirtualMachine vm;
    ElementExport X;
    for (size_t ie = 0; ie < K->element2d.size(); ie++) {
        ElementarySurface *e = K->element2d[ie];
        DelaunayTriangle *t = dynamic_cast<DelaunayTriangle *>(e);
        std::vector<const Point *> verts;
        if (t) verts = {t->first, t->second, t->third};
        export_element(e, 2, K->scales[ie], verts, vm, X);
        e->applyBoundaryCondition(K, &vm);
    }
    write_elements(o, X);
    for (auto bc : bcs) bc->apply(K, F.get2DMesh(), &vm);
    write_multipliers(o, K);
    o.scalar("ndofmax", (double)K->ndofmax);
    o.scalar("n_inclusions_placed", (double)placed.size());
    o.scalar("dim", 2);
    finish_and_solve(o, K);
    return 0;
}

// Config-2 style 3D case: an n^3 voxel file meshed by AMIE's VoxelFilter
// (6 linear tetrahedra per voxel, filters/voxelfilter.cpp:352-400) through
// FeatureTree(voxelSource, behaviourMap) (features/features.cpp:211).  Each
// voxel gets one of `nphase` phases; phase p has a Young's modulus drawn from a
// seeded lognormal (median E, sigma_log).  The cube spans [0, 1e-4]^3 m.
int run_voxel(Out &o, std::map<std::string, std::string> &kv)
{
    const int n = (int)getd(kv, "n", 4);
    const int nphase = (int)getd(kv, "nphase", 16);
    const double E = getd(kv, "E", 30e9), nu = getd(kv, "nu", 0.2);
    const double sig = getd(kv, "sigma_log", 0.4);
    const double strain = getd(kv, "strain", 1e-4);
    const int seed = (int)getd(kv, "seed", 5);
    const char *path = "/tmp/ref_harness_voxels.txt";

    std::mt19937 gen(seed);
    std::lognormal_distribution<double> lnd(std::log(E), sig);
    std::uniform_int_distribution<int> pick(0, nphase - 1);
    std::map<unsigned char, Form *> behaviours;
    std::vector<double> phaseE;
    for (int p = 0; p < nphase; p++) {
        double Ep = lnd(gen);
        phaseE.push_back(Ep);
        behaviours[(unsigned char)('A' + p)] =
            new Stiffness(Tensor::cauchyGreen(Ep, nu, SPACE_THREE_DIMENSIONAL, PLANE_STRESS, YOUNG_POISSON));
    }
    {
        FILE *f = std::fopen(path, "w");
        std::fprintf(f, "voxels amie %d %d %d\n", n, n, n);
        for (int v = 0; v < n * n * n; v++) std::fputc('A' + pick(gen), f);
        std::fputc('\n', f);
        std::fclose(f);
    }
    FeatureTree F(path, behaviours);
    std::vector<BoundaryCondition *> bcs = {
        new BoundingBoxDefinedBoundaryCondition(FIX_ALONG_XI, LEFT),
        new BoundingBoxDefinedBoundaryCondition(FIX_ALONG_ETA, BOTTOM),
        new BoundingBoxDefinedBoundaryCondition(FIX_ALONG_ZETA, BACK),
        new BoundingBoxDefinedBoundaryCondition(SET_ALONG_XI, RIGHT, strain * 1e-4)};

    Assembly *K = F.getAssembly(true);
    VirtualMachine vm;
    ElementExport X;
    for (size_t ie = 0; ie < K->element3d.size(); ie++) {
        ElementaryVolume *e = K->element3d[ie];
        export_element(e, 3, K->scales[ie], {}, vm, X);
        e->applyBoundaryCondition(K, &vm);
    }
    write_elements(o, X);
    for (auto bc : bcs) bc->apply(K, F.get3DMesh(), &vm);
    write_multipliers(o, K);
    o.d("phase_E", phaseE);
    o.scalar("ndofmax", (double)K->ndofmax);
    o.scalar("dim", 3);
    finish_and_solve(o, K);
    return 0;
}


// Read access to a criterion's cache ids (FractureCriterion::cachecoreID /
// cacheID, protected) for the export of the smoothing neighbourhoods.
struct CriterionCaches : public FractureCriterion {
    static int core(FractureCriterion *f) { return static_cast<CriterionCaches *>(f)->cachecoreID; }
    static int all(FractureCriterion *f) { return static_cast<CriterionCaches *>(f)->cacheID; }
};

// Read access to the smoothing weights of a cache (Mesh::coefs, protected).
struct MeshCoefs : public Mesh<DelaunayTriangle, DelaunayTreeItem> {
    static const std::vector<std::vector<double>> &of(Mesh<DelaunayTriangle, DelaunayTreeItem> *m, int id)
    {
        return static_cast<MeshCoefs *>(m)->coefs[id];
    }
};

// Config-3 family: notched beam, damage by load steps through FeatureTree::step.
int run_damage(Out &o, std::map<std::string, std::string> &kv)
{
    const double Lb = getd(kv, "length", 0.08), Hb = getd(kv, "height", 0.02);
    const double nw = getd(kv, "notch_w", 0.004), nh = getd(kv, "notch_h", 0.002);
    const double E = getd(kv, "E", 35e9), nu = getd(kv, "nu", 0.2);
    const double thr = getd(kv, "eps0", 1e-4), Gf = getd(kv, "Gf", 100.0), R = getd(kv, "radius", 0.002);
    const double patch = getd(kv, "patch", 0.004);
    const double dmax = getd(kv, "deflection", 2e-5);
    const int steps = (int)getd(kv, "steps", 6);
    const int model = (int)getd(kv, "model", 0);   // 0 FiberBasedIsotropicLinearDamage, 1 IsotropicLinearDamage
    const double fibre = getd(kv, "fibre", 0.1), cutoff = getd(kv, "cutoff", 0.6);
    const double sampling = getd(kv, "sampling", 32);
    const int maxit = (int)getd(kv, "maxit", 200);

    RectangularFeature box(nullptr, Lb, Hb, 0, 0);
    DamageModel *dm = model == 1 ? (DamageModel *)new IsotropicLinearDamage()
                                 : (DamageModel *)new FiberBasedIsotropicLinearDamage(fibre, cutoff);
    box.setBehaviour(new StiffnessAndFracture(E, nu, new NonLocalMazars(thr, E, nu, Gf, R, PLANE_STRESS), dm,
                                              SPACE_TWO_DIMENSIONAL, PLANE_STRESS));
    FeatureTree F(&box);
    // the notch: a void rectangle centred on the bottom edge at midspan (examples/main_tension_benchmark.cpp:124-127)
    RectangularFeature *notch = new RectangularFeature(nullptr, nw, 2 * nh, 0., -Hb / 2);
    notch->setBehaviour(new VoidForm());
    F.addFeature(&box, notch);
    F.setSamplingNumber(sampling);
    F.setMaxIterationsPerStep(maxit);
    BoundingBoxAndRestrictionDefinedBoundaryCondition *load = new BoundingBoxAndRestrictionDefinedBoundaryCondition(
        SET_ALONG_ETA, TOP, -patch / 2, patch / 2, -10., 10., 0.);
    std::vector<BoundaryCondition *> bcs = {new BoundingBoxDefinedBoundaryCondition(FIX_ALONG_XI, BOTTOM_LEFT),
                                            new BoundingBoxDefinedBoundaryCondition(FIX_ALONG_ETA, BOTTOM_LEFT),
                                            new BoundingBoxDefinedBoundaryCondition(FIX_ALONG_ETA, BOTTOM_RIGHT), load};
    for (auto bc : bcs) F.addBoundaryCondition(bc);

    // element data of the undamaged beam, in Assembly::element2d order
    Assembly *K = F.getAssembly(true);
    VirtualMachine vm;
    ElementExport X;
    std::vector<DelaunayTriangle *> elems;
    std::vector<double> centre, radius, area;
    for (size_t ie = 0; ie < K->element2d.size(); ie++) {
        DelaunayTriangle *t = dynamic_cast<DelaunayTriangle *>(K->element2d[ie]);
        elems.push_back(t);
        export_element(t, 2, K->scales[ie], {t->first, t->second, t->third}, vm, X);
        centre.push_back(t->getCenter().getX());
        centre.push_back(t->getCenter().getY());
        radius.push_back(t->getRadius());
        area.push_back(t->area());
    }
    write_elements(o, X);
    {
        // the multipliers of one load step, applied to a scratch Assembly with the
        // load patch at -1 (load step k sets it to -deflection * k / steps)
        Assembly A;
        A.add(elems[0]);
        load->setData(-1.0);
        for (auto bc : bcs) bc->apply(&A, F.get2DMesh(), &vm);
        load->setData(0.0);
        write_multipliers(o, &A);
    }
    o.d("elem_centre", centre);
    o.d("elem_radius", radius);
    o.d("elem_area", area);
    o.scalar("ndofmax", (double)K->ndofmax);
    o.scalar("dim", 2);
    o.scalar("eps0", thr);
    o.scalar("Gf", Gf);
    o.scalar("E", E);
    o.scalar("nu", nu);
    o.scalar("radius", R);
    o.scalar("model", model);
    o.scalar("fibre", fibre);
    o.scalar("cutoff", cutoff);
    o.scalar("steps", steps);
    o.scalar("deflection", dmax);

    const size_t ne = elems.size();
    for (int k = 1; k <= steps; k++) {
        load->setData(-dmax * k / steps);
        double t0 = now_s();
        F.step();
        double t1 = now_s();
        const Vector &u = F.getDisplacements();
        std::vector<double> uu(std::begin(u), std::end(u)), dmg(ne), score(ne), sm(4 * ne), eps(3 * ne);
        size_t damaged = 0;
        for (size_t i = 0; i < ne; i++) {
            Form *b = elems[i]->getBehaviour();
            const Matrix Ceff = b->getTensor(Point());
            dmg[i] = 1.0 - Ceff[0][0] / b->param[0][0];
            damaged += dmg[i] > 0;
            FractureCriterion *fc = b->getFractureCriterion();
            score[i] = fc->getScoreAtState();
            std::pair<Vector, Vector> f = fc->getSmoothedFields(PRINCIPAL_REAL_STRESS_FIELD, PRINCIPAL_TOTAL_STRAIN_FIELD,
                                                                 elems[i]->getState(), 0.);
            sm[4 * i] = f.first[0];
            sm[4 * i + 1] = f.first[1];
            sm[4 * i + 2] = f.second[0];
            sm[4 * i + 3] = f.second[1];
            Vector es(3);
            elems[i]->getState().getAverageField(MECHANICAL_STRAIN_FIELD, es, &vm, 0.);
            for (int c = 0; c < 3; c++) eps[3 * i + c] = es[c];
        }
        const std::string sfx = "_" + std::to_string(k);
        o.d("u" + sfx, uu);
        o.d("damage" + sfx, dmg);
        o.d("score" + sfx, score);
        o.d("smoothed" + sfx, sm);
        o.d("strain" + sfx, eps);
        o.scalar("step_time_s" + sfx, t1 - t0);
        o.scalar("average_damage" + sfx, F.averageDamage);
        std::fprintf(stderr, "harness damage: step %d deflection %.3e damaged %zu avg %.3e time %.2fs\n", k,
                     dmax * k / steps, damaged, F.averageDamage, t1 - t0);
    }
    // the smoothing neighbourhood of every element (Mesh::generateCache through
    // FractureCriterion::initialiseCache), as positions in the element order above
    std::map<int, uint32_t> pos;
    for (size_t i = 0; i < ne; i++) pos[elems[i]->index] = (uint32_t)i;
    std::vector<uint32_t> cptr{0}, cidx, aptr{0}, aidx;
    std::vector<double> ccoef;
    for (size_t i = 0; i < ne; i++) {
        FractureCriterion *fc = elems[i]->getBehaviour()->getFractureCriterion();
        for (int id : F.get2DMesh()->getCache(CriterionCaches::core(fc))) cidx.push_back(pos.count(id) ? pos[id] : 0xffffffffu);
        cptr.push_back((uint32_t)cidx.size());
        for (const auto &w : MeshCoefs::of(F.get2DMesh(), CriterionCaches::core(fc))) ccoef.push_back(w.empty() ? -1.0 : w[0]);
        for (int id : F.get2DMesh()->getCache(CriterionCaches::all(fc))) aidx.push_back(pos.count(id) ? pos[id] : 0xffffffffu);
        aptr.push_back((uint32_t)aidx.size());
    }
    o.u("cache_ptr", cptr);
    o.u("cache_idx", cidx);
    o.d("cache_coef", ccoef);
    o.u("cache_all_ptr", aptr);
    o.u("cache_all_idx", aidx);
    o.scalar("n_elem", (double)ne);
    return 0;
}

// Read access to the smoothing weights of a 3D cache (Mesh::coefs, protected).
struct MeshCoefs3D : public Mesh<DelaunayTetrahedron, DelaunayTreeItem3D> {
    static const std::vector<std::vector<double>> &of(Mesh<DelaunayTetrahedron, DelaunayTreeItem3D> *m, int id)
    {
        return static_cast<MeshCoefs3D *>(m)->coefs[id];
    }
};

// 3D damage: an n^3 voxel cube (VoxelFilter, 6 tetrahedra per voxel, [0, 1e-4]^3 m)
// whose voxels take one of `nphase` phases, phase p StiffnessAndFracture with a
// seeded lognormal Young's modulus, NonLocalMazars and
// FiberBasedIsotropicLinearDamage; pulled along x (left face fixed in x, bottom
// in y, back in z, right face displaced) by load steps through FeatureTree::step.
// Exports as the 2D damage case: element data, centres, circumradii, volumes,
// the multipliers of one step with the pull at 1, and per step the
// displacements, damage, scores, smoothed principal stresses and strains (3 + 3)
// and element strains (6), then the smoothing and maximum neighbourhoods.
int run_damage3d(Out &o, std::map<std::string, std::string> &kv)
{
    const int n = (int)getd(kv, "n", 6);
    const int nphase = (int)getd(kv, "nphase", 8);
    const double E = getd(kv, "E", 30e9), nu = getd(kv, "nu", 0.2), sig = getd(kv, "sigma_log", 0.4);
    const double thr = getd(kv, "eps0", 1e-4), Gf = getd(kv, "Gf", 100.0), R = getd(kv, "radius", 2e-5);
    const double fibre = getd(kv, "fibre", 0.1), cutoff = getd(kv, "cutoff", 0.6);
    const double dmax = getd(kv, "displacement", 3e-8);
    const int steps = (int)getd(kv, "steps", 6);
    const int maxit = (int)getd(kv, "maxit", 200);
    const int seed = (int)getd(kv, "seed", 7);
    const char *path = "/tmp/ref_harness_damage3d.txt";

    std::mt19937 gen(seed);
    std::lognormal_distribution<double> lnd(std::log(E), sig);
    std::uniform_int_distribution<int> pick(0, nphase - 1);
    std::map<unsigned char, Form *> behaviours;
    std::vector<double> phaseE;
    for (int p = 0; p < nphase; p++) {
        const double Ep = lnd(gen);
        phaseE.push_back(Ep);
        behaviours[(unsigned char)('A' + p)] = new StiffnessAndFracture(
            Ep, nu, new NonLocalMazars(thr, Ep, nu, Gf, R, PLANE_STRESS), new FiberBasedIsotropicLinearDamage(fibre, cutoff),
            SPACE_THREE_DIMENSIONAL);
    }
    {
        FILE *f = std::fopen(path, "w");
        std::fprintf(f, "voxels amie %d %d %d\n", n, n, n);
        for (int v = 0; v < n * n * n; v++) std::fputc('A' + pick(gen), f);
        std::fputc('\n', f);
        std::fclose(f);
    }
    FeatureTree F(path, behaviours);
    F.setMaxIterationsPerStep(maxit);
    BoundingBoxDefinedBoundaryCondition *pull = new BoundingBoxDefinedBoundaryCondition(SET_ALONG_XI, RIGHT, 0.);
    std::vector<BoundaryCondition *> bcs = {new BoundingBoxDefinedBoundaryCondition(FIX_ALONG_XI, LEFT),
                                            new BoundingBoxDefinedBoundaryCondition(FIX_ALONG_ETA, BOTTOM),
                                            new BoundingBoxDefinedBoundaryCondition(FIX_ALONG_ZETA, BACK), pull};
    for (auto bc : bcs) F.addBoundaryCondition(bc);

    Assembly *K = F.getAssembly(true);
    VirtualMachine vm;
    ElementExport X;
    std::vector<DelaunayTetrahedron *> elems;
    std::vector<double> centre, radius, volume;
    for (size_t ie = 0; ie < K->element3d.size(); ie++) {
        DelaunayTetrahedron *t = dynamic_cast<DelaunayTetrahedron *>(K->element3d[ie]);
        elems.push_back(t);
        export_element(t, 3, K->scales[ie], {}, vm, X);
        centre.push_back(t->getCenter().getX());
        centre.push_back(t->getCenter().getY());
        centre.push_back(t->getCenter().getZ());
        radius.push_back(t->getRadius());
        volume.push_back(t->volume());
    }
    write_elements(o, X);
    {
        Assembly A;
        A.add(elems[0]);
        pull->setData(1.0);
        for (auto bc : bcs) bc->apply(&A, F.get3DMesh(), &vm);
        pull->setData(0.0);
        write_multipliers(o, &A);
    }
    o.d("elem_centre", centre);
    o.d("elem_radius", radius);
    o.d("elem_volume", volume);
    o.d("phase_E", phaseE);
    o.scalar("ndofmax", (double)K->ndofmax);
    o.scalar("dim", 3);
    o.scalar("eps0", thr);
    o.scalar("Gf", Gf);
    o.scalar("nu", nu);
    o.scalar("radius", R);
    o.scalar("fibre", fibre);
    o.scalar("cutoff", cutoff);
    o.scalar("steps", steps);
    o.scalar("displacement", dmax);

    const size_t ne = elems.size();
    std::vector<double> sub;
    for (int k = 1; k <= steps; k++) {
        pull->setData(dmax * k / steps);
        const double t0 = now_s();
        F.step();
        const double t1 = now_s();
        const Vector &u = F.getDisplacements();
        std::vector<double> uu(std::begin(u), std::end(u)), dmg(ne), score(ne), sm(6 * ne), eps(6 * ne);
        size_t damaged = 0;
        for (size_t i = 0; i < ne; i++) {
            Form *b = elems[i]->getBehaviour();
            const Matrix Ceff = b->getTensor(Point());
            dmg[i] = 1.0 - Ceff[0][0] / b->param[0][0];
            damaged += dmg[i] > 0;
            FractureCriterion *fc = b->getFractureCriterion();
            score[i] = fc->getScoreAtState();
            std::pair<Vector, Vector> f = fc->getSmoothedFields(PRINCIPAL_REAL_STRESS_FIELD, PRINCIPAL_TOTAL_STRAIN_FIELD,
                                                                 elems[i]->getState(), 0.);
            for (int c = 0; c < 3; c++) {
                sm[6 * i + c] = f.first.size() > (size_t)c ? f.first[c] : 0.0;
                sm[6 * i + 3 + c] = f.second.size() > (size_t)c ? f.second[c] : 0.0;
            }
            Vector es(6);
            elems[i]->getState().getAverageField(MECHANICAL_STRAIN_FIELD, es, &vm, 0.);
            for (int c = 0; c < 6; c++) eps[6 * i + c] = es[c];
        }
        const std::string sfx = "_" + std::to_string(k);
        o.d("u" + sfx, uu);
        o.d("damage" + sfx, dmg);
        o.d("score" + sfx, score);
        o.d("smoothed" + sfx, sm);
        o.d("strain" + sfx, eps);
        o.scalar("step_time_s" + sfx, t1 - t0);
        std::fprintf(stderr, "harness damage3d: step %d displacement %.3e damaged %zu avg %.3e time %.2fs\n", k,
                     dmax * k / steps, damaged, F.averageDamage, t1 - t0);
    }
    std::map<int, uint32_t> pos;
    for (size_t i = 0; i < ne; i++) pos[elems[i]->index] = (uint32_t)i;
    std::vector<uint32_t> cptr{0}, cidx, aptr{0}, aidx;
    std::vector<double> ccoef;
    for (size_t i = 0; i < ne; i++) {
        FractureCriterion *fc = elems[i]->getBehaviour()->getFractureCriterion();
        for (int id : F.get3DMesh()->getCache(CriterionCaches::core(fc))) cidx.push_back(pos.count(id) ? pos[id] : 0xffffffffu);
        cptr.push_back((uint32_t)cidx.size());
        for (const auto &w : MeshCoefs3D::of(F.get3DMesh(), CriterionCaches::core(fc))) ccoef.push_back(w.empty() ? -1.0 : w[0]);
        for (int id : F.get3DMesh()->getCache(CriterionCaches::all(fc))) aidx.push_back(pos.count(id) ? pos[id] : 0xffffffffu);
        aptr.push_back((uint32_t)aidx.size());
    }
    o.u("cache_ptr", cptr);
    o.u("cache_idx", cidx);
    o.d("cache_coef", ccoef);
    o.u("cache_all_ptr", aptr);
    o.u("cache_all_idx", aidx);
    o.scalar("n_elem", (double)ne);
    return 0;
}

}  // namespace

int main(int argc, char **argv)
{
    if (argc < 3) {
        std::fprintf(stderr, "usage: %s incl|crack|voxel out.bin [key=value ...]\n", argv[0]);
        return 2;
    }
    std::string which = argv[1];
    auto kv = parse_kv(argc, argv, 3);
    Out o(argv[2]);
    if (!o.f) return 3;
    if (which == "incl" || which == "crack" || which == "plate" || which == "imposed") return run_2d(which, o, kv);
    if (which == "voxel") return run_voxel(o, kv);
    if (which == "damage") return run_damage(o, kv);
    if (which == "damage3d") return run_damage3d(o, kv);
    std::fprintf(stderr, "unknown case %s\n", which.c_str());
    return 2;
}
