// gpu_assembly.hpp -- C++ mirror of AMIE's Assembly (solvers/assembly.h:228-450)
// for the element-stiffness -> scatter -> conjugate-gradient path, running on the
// GPU through the C-ABI of amie_gpu.h.
//
// Method names and meaning follow the reference:
//   add(...)                 Assembly::add (solvers/assembly.cpp:106-123), here one
//                            element at a time from plain element data
//   setPointAlong / fixPoint Assembly::setPointAlong / fixPoint (:1590-1634, :1762)
//   setForceOn               Assembly::setForceOn (SET_FORCE_INDEXED_AXIS, :1560-1588)
//   setPointProportional     Assembly::setPointProportional (:1636-1697, :1699-1761): v1 =
//                            sum val_k v_k + offset at one node (SET_PROPORTIONAL_DISPLACEMENT)
//   setMaxDof, setEpsilon, setSSORIterations
//   cgsolve(maxit)           Assembly::cgsolve (:1829-1953): make_final + solve,
//                            warm start from extrapolate() (:1772-1814), keeps the
//                            displacement history
//   getMatrix / getForces / getDisplacements
//   clear / clearElements    (:448-449)
// Errors: cgsolve returns false when the solver did not converge, as the
// reference does; a NaN residual (the reference exit(0)s) and every other
// failure throw gpu::Error carrying the amie_status.
#pragma once

#include "amie_gpu.h"

#include <cstdint>
#include <map>
#include <stdexcept>
#include <string>
#include <vector>

namespace gpu {

enum Variable { XI = 0, ETA = 1, ZETA = 2 };

struct Error : std::runtime_error {
    amie_status status;
    Error(amie_status s, const std::string &what) : std::runtime_error(what), status(s) {}
};

// One element as Assembly holds it when cgsolve runs.
struct Element {
    int kind = AMIE_TRI3;                 // AMIE_TRI3 / AMIE_TRI6 / AMIE_TET4
    std::vector<uint32_t> dofIds;         // getDofIds(): node ids, then enrichment ids
    std::vector<double> gaussPoints;      // (dim+1) per point: local coords, weight*detJ; empty = default rule
    std::vector<double> jinv;             // dim*dim inverse Jacobian (centroid)
    std::vector<double> jinvPerGp;        // dim*dim per Gauss point for moved elements, else empty
    std::vector<double> C;                // behaviour tensor (nv*nv), Form::param
    double cscale = 1.0;                  // damage / modulus factor on C
    double scale = 1.0;                   // Assembly::add scale
    struct Enrichment {
        int type = AMIE_ENR_HEAVISIDE;    // AMIE_ENR_HEAVISIDE or AMIE_ENR_TABULATED
        int vertex = 0;                   // P1 vertex of a Heaviside function
        std::vector<int8_t> jump;         // Heaviside: H(x_g) - H(x_k) per Gauss point
        std::vector<double> grad;         // tabulated: dim per Gauss point
    };
    std::vector<Enrichment> enrichment;
};

class Assembly {
public:
    explicit Assembly(int device = 0);
    ~Assembly();
    Assembly(const Assembly &) = delete;
    Assembly &operator=(const Assembly &) = delete;

    void add(const Element &e);
    void setMaxDof(size_t n) { ndofmax_ = n; }
    void setEpsilon(double e) { epsilon_ = e; }
    double getEpsilon() const { return epsilon_; }
    void setSSORIterations(size_t n) { nssor_ = (int)n; }
    // AMIE_SOLVER_AMIE_CG reproduces ConjugateGradient::solve; PCG_FP64 / PCG_MIXED
    // stop at a relative residual.
    void setSolver(int solver, double rtol = 1e-10) { solver_ = solver; rtol_ = rtol; }

    void setPointAlong(Variable v, double val, size_t id);
    void fixPoint(size_t id, Variable v) { setPointAlong(v, 0.0, id); }
    void setForceOn(Variable v, double val, size_t id);
    void setPointProportional(Variable v1, Variable v2, double val, double offset, size_t id);
    void setPointProportional(Variable v1, const std::vector<std::pair<Variable, double>> &val, double offset,
                              size_t id);

    bool cgsolve(int maxit = -1, bool verbose = false);

    // CoordinateIndexedSparseMatrix pieces: row_size, column_index, array (AMIE layout).
    void getMatrix(std::vector<uint32_t> &row_size, std::vector<uint32_t> &column_index,
                   std::vector<double> &array) const;
    std::vector<double> getForces() const;
    const std::vector<double> &getDisplacements() const { return displacements_; }
    std::vector<double> extrapolate() const;
    const amie_solve_stats &lastStats() const { return stats_; }

    void clear();
    void clearElements();

private:
    void make_final();
    void check(amie_status s, const char *where) const;

    int dim_ = 0;
    amie_ctx *ctx_ = nullptr;
    amie_topo *topo_ = nullptr;
    bool topologyDirty_ = true;
    bool topoHasProportional_ = false;   // the topology holds proportional multipliers
    size_t ndofmax_ = 0;
    double epsilon_ = 1e-10;
    double rtol_ = 1e-10;
    int nssor_ = 32;
    int solver_ = AMIE_SOLVER_AMIE_CG;
    std::vector<Element> elements_;
    std::map<uint32_t, std::pair<double, uint8_t>> multipliers_;
    struct Proportional {
        double offset;
        std::vector<uint32_t> dofs;
        std::vector<double> coefs;
    };
    std::map<uint32_t, Proportional> proportional_;   // by constrained DOF, as make_final sorts them
    std::vector<double> displacements_;
    std::vector<std::vector<double>> history_;
    amie_solve_stats stats_{};
};

}  // namespace gpu
