// gpu_assembly.cpp -- see gpu_assembly.hpp.
#include "gpu_assembly.hpp"

#include <cmath>

#include <algorithm>

namespace gpu {

namespace {
int nshape(int kind) { return kind == AMIE_TRI3 ? 3 : kind == AMIE_TRI6 ? 6 : kind == AMIE_TET4 ? 4 : 0; }
}  // namespace

Assembly::Assembly(int device)
{
    amie_config cfg{device, 0, 0};
    check(amie_ctx_create(&cfg, &ctx_), "amie_ctx_create");
}

Assembly::~Assembly()
{
    if (topo_) amie_topology_destroy(topo_);
    if (ctx_) amie_ctx_destroy(ctx_);
}

void Assembly::check(amie_status s, const char *where) const
{
    if (s != AMIE_OK) throw Error(s, std::string(where) + ": " + amie_last_error());
}

void Assembly::add(const Element &e)
{
    const int d = e.kind == AMIE_TET4 ? 3 : 2;
    if (dim_ && d != dim_) throw Error(AMIE_BAD_INPUT, "mixed 2D and 3D elements");
    dim_ = d;
    elements_.push_back(e);
    topologyDirty_ = true;
}

void Assembly::setPointAlong(Variable v, double val, size_t id)
{
    const int s = dim_ ? dim_ : 2;
    proportional_.erase((uint32_t)(id * s + (int)v));   // a later multiplier on a DOF replaces the earlier one
    multipliers_[(uint32_t)(id * s + (int)v)] = {val, (uint8_t)AMIE_BC_DISPLACEMENT};
}

void Assembly::setPointProportional(Variable v1, Variable v2, double val, double offset, size_t id)
{
    if (v1 == v2) return;
    const int s = dim_ ? dim_ : 2;
    const uint32_t dof = (uint32_t)(id * s + (int)v1);
    multipliers_.erase(dof);
    proportional_[dof] = Proportional{offset, {(uint32_t)(id * s + (int)v2)}, {val}};
}

void Assembly::setPointProportional(Variable v1, const std::vector<std::pair<Variable, double>> &val, double offset,
                                    size_t id)
{
    const int s = dim_ ? dim_ : 2;
    Proportional p{offset, {}, {}};
    for (const auto &vc : val) {
        p.dofs.push_back((uint32_t)(id * s + (int)vc.first));
        p.coefs.push_back(vc.second);
    }
    const uint32_t dof = (uint32_t)(id * s + (int)v1);
    multipliers_.erase(dof);
    proportional_[dof] = std::move(p);
}

void Assembly::setForceOn(Variable v, double val, size_t id)
{
    const int s = dim_ ? dim_ : 2;
    auto &m = multipliers_[(uint32_t)(id * s + (int)v)];
    if (m.second != AMIE_BC_FORCE) m = {0.0, (uint8_t)AMIE_BC_FORCE};
    m.first += val;   // duplicates accumulate (solvers/assembly.cpp:1560-1588)
}

void Assembly::clear()
{
    clearElements();
    multipliers_.clear();
    proportional_.clear();
    history_.clear();
    displacements_.clear();
}

void Assembly::clearElements()
{
    elements_.clear();
    if (topo_) amie_topology_destroy(topo_);
    topo_ = nullptr;
    topologyDirty_ = true;
}

// make_final: pattern + scatter map (first call or new topology), element
// matrices + scatter, Dirichlet elimination (solvers/assembly.cpp:425-1223).
void Assembly::make_final()
{
    if (elements_.empty()) throw Error(AMIE_BAD_INPUT, "no elements in assembly");
    if (topologyDirty_ || !topo_) {
        const int s = dim_, nv = dim_ == 2 ? 3 : 6;
        const uint32_t E = (uint32_t)elements_.size();
        std::vector<uint8_t> kind(E), moved(E, 0), enr_type, enr_vertex;
        std::vector<uint32_t> dof_ptr(E + 1, 0), dof_ids, gp_ptr(E + 1, 0), mat(E), enr_ptr(E + 1, 0), enr_data;
        std::vector<double> gp, jinv, jinv_gp, cmat, cscale(E), scale(E), enr_grad;
        std::vector<int8_t> enr_jump;
        std::map<std::vector<double>, uint32_t> materials;
        bool any_moved = false;
        uint64_t cursor = 0;
        for (uint32_t i = 0; i < E; i++) {
            const Element &e = elements_[i];
            kind[i] = (uint8_t)e.kind;
            dof_ids.insert(dof_ids.end(), e.dofIds.begin(), e.dofIds.end());
            dof_ptr[i + 1] = (uint32_t)dof_ids.size();
            const uint32_t ngp = (uint32_t)(e.gaussPoints.size() / (s + 1));
            gp.insert(gp.end(), e.gaussPoints.begin(), e.gaussPoints.end());
            gp_ptr[i + 1] = gp_ptr[i] + ngp;
            jinv.insert(jinv.end(), e.jinv.begin(), e.jinv.end());
            if (!e.jinvPerGp.empty()) {
                moved[i] = 1;
                any_moved = true;
                jinv_gp.insert(jinv_gp.end(), e.jinvPerGp.begin(), e.jinvPerGp.end());
            } else {
                for (uint32_t g = 0; g < ngp; g++) jinv_gp.insert(jinv_gp.end(), e.jinv.begin(), e.jinv.end());
            }
            auto it = materials.find(e.C);
            if (it == materials.end()) it = materials.emplace(e.C, (uint32_t)materials.size()).first;
            mat[i] = it->second;
            cscale[i] = e.cscale;
            scale[i] = e.scale;
            const uint32_t ngp_eff = ngp ? ngp : (e.kind == AMIE_TRI6 ? 4 : 1);
            for (const auto &f : e.enrichment) {
                enr_type.push_back((uint8_t)f.type);
                enr_vertex.push_back((uint8_t)f.vertex);
                enr_data.push_back((uint32_t)cursor);
                if (f.type == AMIE_ENR_HEAVISIDE) {
                    enr_jump.insert(enr_jump.end(), f.jump.begin(), f.jump.end());
                    enr_jump.resize(cursor + ngp_eff, 0);
                    enr_grad.resize((cursor + ngp_eff) * s, 0.0);
                } else {
                    enr_grad.insert(enr_grad.end(), f.grad.begin(), f.grad.end());
                    enr_grad.resize((cursor + ngp_eff) * s, 0.0);
                    enr_jump.resize(cursor + ngp_eff, 0);
                }
                cursor += ngp_eff;
            }
            enr_ptr[i + 1] = (uint32_t)enr_type.size();
            if ((int)e.dofIds.size() != nshape(e.kind) + (int)e.enrichment.size())
                throw Error(AMIE_BAD_INPUT, "element dof count != shape + enrichment functions");
        }
        cmat.resize(materials.size() * nv * nv);
        for (const auto &kv : materials) std::copy(kv.first.begin(), kv.first.end(), cmat.begin() + kv.second * nv * nv);
        amie_mesh m{};
        m.dim = s;
        m.stride = s;
        m.n_elem = E;
        m.ndofmax = (uint32_t)ndofmax_;
        m.kind = kind.data();
        m.dof_ptr = dof_ptr.data();
        m.dof_ids = dof_ids.data();
        m.gp_ptr = gp_ptr.data();
        m.gp = gp.empty() ? nullptr : gp.data();
        m.jinv = jinv.data();
        m.moved = any_moved ? moved.data() : nullptr;
        m.jinv_gp = any_moved ? jinv_gp.data() : nullptr;
        m.mat = mat.data();
        m.cmat_table = cmat.data();
        m.n_mat = (uint32_t)materials.size();
        m.cscale = cscale.data();
        m.scale = scale.data();
        if (!enr_type.empty()) {
            m.enr_ptr = enr_ptr.data();
            m.enr_type = enr_type.data();
            m.enr_vertex = enr_vertex.data();
            m.enr_data = enr_data.data();
            m.n_enr_gp = cursor;
            m.enr_jump = enr_jump.data();
            m.enr_grad = enr_grad.data();
        }
        if (topo_) amie_topology_destroy(topo_);
        topo_ = nullptr;
        check(amie_topology_build(ctx_, &m, &topo_), "amie_topology_build");
        topoHasProportional_ = false;
        topologyDirty_ = false;
    }
    check(amie_assemble(topo_), "amie_assemble");
    std::vector<uint32_t> ids;
    std::vector<double> vals;
    std::vector<uint8_t> kinds;
    for (const auto &kv : multipliers_) {   // sorted by id, as make_final sorts them
        ids.push_back(kv.first);
        vals.push_back(kv.second.first);
        kinds.push_back(kv.second.second);
    }
    std::vector<uint32_t> pids, pptr{0}, pdofs;
    std::vector<double> poff, pco;
    for (const auto &kv : proportional_) {
        pids.push_back(kv.first);
        poff.push_back(kv.second.offset);
        pdofs.insert(pdofs.end(), kv.second.dofs.begin(), kv.second.dofs.end());
        pco.insert(pco.end(), kv.second.coefs.begin(), kv.second.coefs.end());
        pptr.push_back((uint32_t)pdofs.size());
    }
    // a DOF may have moved between the two lists since the last make_final: the
    // old proportional multipliers go first, so that no DOF is in both at once
    if (topoHasProportional_) {
        const uint32_t zero = 0;
        check(amie_set_proportional(topo_, 0, nullptr, nullptr, &zero, nullptr, nullptr), "amie_set_proportional");
        topoHasProportional_ = false;
    }
    check(amie_apply_dirichlet(topo_, (uint32_t)ids.size(), ids.data(), vals.data(), kinds.data(), nullptr),
          "amie_apply_dirichlet");
    if (!pids.empty()) {
        check(amie_set_proportional(topo_, (uint32_t)pids.size(), pids.data(), poff.data(), pptr.data(),
                                    pdofs.data(), pco.data()),
              "amie_set_proportional");
        topoHasProportional_ = true;
    }
}

std::vector<double> Assembly::extrapolate() const
{
    if (history_.size() < 2) return displacements_;
    const auto &a = history_[history_.size() - 2], &b = history_.back();
    std::vector<double> x(b.size());
    for (size_t i = 0; i < b.size(); i++) {
        const double u = std::isnan(b[i]) ? 0.0 : b[i];
        x[i] = u + (u - a[i]);
    }
    return x;
}

bool Assembly::cgsolve(int maxit, bool verbose)
{
    (void)verbose;
    make_final();
    uint64_t n = 0;
    check(amie_topology_sizes(topo_, nullptr, nullptr, &n), "amie_topology_sizes");
    std::vector<double> x = extrapolate();
    amie_solve_opts o{};
    o.solver = solver_;
    o.rtol = rtol_;
    o.eps = epsilon_;
    o.nssor = nssor_;
    o.maxit = maxit > 0 ? maxit : 0;
    o.inner_rtol = 0.0;   // library default
    o.use_x0 = x.size() == n ? 1 : 0;
    x.resize(n, 0.0);
    amie_status s = amie_solve(topo_, &o, x.data(), &stats_);
    if (s != AMIE_OK && s != AMIE_NOT_CONVERGED) check(s, "amie_solve");
    displacements_ = x;
    // the reference keeps two entries and starts them as [0, u1] (solvers/assembly.cpp:1859-1867)
    if (history_.size() == 2) {
        history_[0] = history_[1];
        history_[1] = x;
    } else {
        history_.assign({std::vector<double>(x.size(), 0.0), x});
    }
    return s == AMIE_OK;
}

void Assembly::getMatrix(std::vector<uint32_t> &row_size, std::vector<uint32_t> &column_index,
                         std::vector<double> &array) const
{
    uint32_t nr = 0;
    uint64_t nnzb = 0;
    check(amie_topology_sizes(topo_, &nr, &nnzb, nullptr), "amie_topology_sizes");
    row_size.resize(nr);
    column_index.resize(nnzb);
    const int s = dim_;
    array.resize(nnzb * s * (s + s % 2));
    check(amie_topology_pattern(topo_, row_size.data(), column_index.data()), "amie_topology_pattern");
    check(amie_matrix_download(topo_, array.data(), nullptr), "amie_matrix_download");
}

std::vector<double> Assembly::getForces() const
{
    uint64_t n = 0;
    check(amie_topology_sizes(topo_, nullptr, nullptr, &n), "amie_topology_sizes");
    std::vector<double> f(n);
    check(amie_matrix_download(topo_, nullptr, f.data()), "amie_matrix_download");
    return f;
}

}  // namespace gpu
