// amie_bridge.cpp -- the AMIE-side adapter: feeds gpu::Assembly from AMIE's own
// elements and multipliers, as a drop-in for Assembly::cgsolve inside
// FeatureTree::solve (features/features.cpp:4764).  It is built inside the AMIE
// tree (it includes AMIE's headers and links libamie_gpu.so); this repository
// only compile-checks it against the reference headers (oracle/Makefile,
// target `bridge`).
#include "features/features.h"
#include "gpu_assembly.hpp"

namespace Amie {

// Element data of one AMIE element in the form gpu::Assembly takes.
gpu::Element toGpuElement(IntegrableEntity *e, int dim, double scale, VirtualMachine &vm)
{
    gpu::Element g;
    const size_t ns = e->getShapeFunctions().size();
    g.kind = dim == 3 ? AMIE_TET4 : (ns == 3 ? AMIE_TRI3 : AMIE_TRI6);
    for (size_t id : e->getDofIds()) g.dofIds.push_back((uint32_t)id);           // elements/elements.cpp:204
    const GaussPointArray &gp = e->getGaussPoints();                               // weights x det J
    if (!e->getState().JinvCache) e->getState().updateInverseJacobianCache(Point(1. / 3., 1. / 3.));
    const Matrix &J = *e->getState().JinvCache;                                    // mesher/delaunay.cpp:2436
    for (int r = 0; r < dim; r++)
        for (int c = 0; c < dim; c++) g.jinv.push_back(J[r][c]);
    for (size_t k = 0; k < gp.gaussPoints.size(); k++) {
        g.gaussPoints.push_back(gp.gaussPoints[k].first.getX());
        g.gaussPoints.push_back(gp.gaussPoints[k].first.getY());
        if (dim == 3) g.gaussPoints.push_back(gp.gaussPoints[k].first.getZ());
        g.gaussPoints.push_back(gp.gaussPoints[k].second);
        if (e->isMoved()) {                                                        // mesher/delaunay.cpp:2441
            Matrix Jg(dim, dim);
            e->getState().getInverseJacobianMatrix(gp.gaussPoints[k].first, Jg);
            for (int r = 0; r < dim; r++)
                for (int c = 0; c < dim; c++) g.jinvPerGp.push_back(Jg[r][c]);
        }
    }
    const Matrix &C = e->getBehaviour()->param;                                    // physics/stiffness.cpp:43
    for (size_t r = 0; r < C.numRows(); r++)
        for (size_t c = 0; c < C.numCols(); c++) g.C.push_back(C[r][c]);
    g.scale = scale;
    for (size_t j = 0; j < e->getEnrichmentFunctions().size(); j++) {             // tabulated gradients
        const Function &f = e->getEnrichmentFunction(j);
        gpu::Element::Enrichment en;
        en.type = AMIE_ENR_TABULATED;
        for (size_t k = 0; k < gp.gaussPoints.size(); k++) {
            en.grad.push_back(vm.deval(f, XI, gp.gaussPoints[k].first));         // polynomial/vm_base.cpp:1115
            en.grad.push_back(vm.deval(f, ETA, gp.gaussPoints[k].first));
            if (dim == 3) en.grad.push_back(vm.deval(f, ZETA, gp.gaussPoints[k].first));
        }
        g.enrichment.push_back(en);
    }
    return g;
}

// Drop-in for K->cgsolve(): the elements and multipliers AMIE's Assembly holds
// are handed to the GPU, the solution comes back into K's displacement vector.
bool gpuCgsolve(Assembly *K, gpu::Assembly &G, bool reuseTopology)
{
    VirtualMachine vm;
    if (!reuseTopology) {
        G.clearElements();
        for (size_t i = 0; i < K->element2d.size(); i++) G.add(toGpuElement(K->element2d[i], 2, K->scales[i], vm));
        for (size_t i = 0; i < K->element3d.size(); i++) G.add(toGpuElement(K->element3d[i], 3, K->scales[i], vm));
        G.setMaxDof(K->ndofmax);
    }
    for (auto &m : K->multipliers) {                                               // solvers/assembly.cpp:1590
        if (m.type == SET_PROPORTIONAL_DISPLACEMENT) {                             // :1636-1760
            const std::valarray<unsigned int> dofs = m.getDofIds();
            std::vector<std::pair<gpu::Variable, double>> val;
            for (size_t k = 0; k < dofs.size(); k++)
                val.emplace_back((gpu::Variable)(dofs[k] % K->ndof), m.coefs[k]);
            G.setPointProportional((gpu::Variable)(m.getId() % K->ndof), val, m.getValue(), m.getId() / K->ndof);
        } else if (m.type == SET_FORCE_XI || m.type == SET_FORCE_ETA || m.type == SET_FORCE_ZETA)
            G.setForceOn((gpu::Variable)(m.getId() % K->ndof), m.getValue(), m.getId() / K->ndof);
        else
            G.setPointAlong((gpu::Variable)(m.getId() % K->ndof), m.getValue(), m.getId() / K->ndof);
    }
    G.setEpsilon(K->epsilon);
    G.setSSORIterations(K->nssor);
    const bool ok = G.cgsolve();
    const std::vector<double> &u = G.getDisplacements();
    K->displacements.resize(u.size());
    for (size_t i = 0; i < u.size(); i++) K->displacements[i] = u[i];
    return ok;
}

}  // namespace Amie
