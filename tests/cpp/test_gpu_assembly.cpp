// C++ driver of gpu::Assembly (the mirror of AMIE's Assembly) for the GPU tests.
//
// Reads one case as raw arrays from a directory (written by
// tests/test_cpp_assembly.py), adds the elements one by one, sets the Dirichlet
// multipliers with setPointAlong (and the proportional ones, when the case has
// them, with setPointProportional), runs cgsolve with the requested solver and
// writes the displacements and the matrix back as raw arrays.
//
//   test_gpu_assembly <dir> <solver: 0 fp64 | 1 mixed | 2 amie_cg>
#include "gpu_assembly.hpp"

#include <cstdio>
#include <string>
#include <vector>

template <typename T>
static std::vector<T> load(const std::string &path)
{
    std::vector<T> v;
    FILE *f = std::fopen(path.c_str(), "rb");
    if (!f) return v;
    std::fseek(f, 0, SEEK_END);
    const long bytes = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    v.resize(bytes / sizeof(T));
    if (!v.empty() && std::fread(v.data(), sizeof(T), v.size(), f) != v.size()) v.clear();
    std::fclose(f);
    return v;
}

template <typename T>
static void save(const std::string &path, const std::vector<T> &v)
{
    FILE *f = std::fopen(path.c_str(), "wb");
    if (!f) return;
    std::fwrite(v.data(), sizeof(T), v.size(), f);
    std::fclose(f);
}

int main(int argc, char **argv)
{
    if (argc < 3) return 2;
    const std::string dir = argv[1];
    const int solver = std::atoi(argv[2]);
    auto kind = load<uint8_t>(dir + "/kind.bin");
    auto dof_ptr = load<uint32_t>(dir + "/dof_ptr.bin");
    auto dof_ids = load<uint32_t>(dir + "/dof_ids.bin");
    auto gp_ptr = load<uint32_t>(dir + "/gp_ptr.bin");
    auto gp = load<double>(dir + "/gp.bin");
    auto jinv = load<double>(dir + "/jinv.bin");
    auto cmat = load<double>(dir + "/cmat.bin");
    auto bc_ids = load<uint32_t>(dir + "/bc_ids.bin");
    auto bc_vals = load<double>(dir + "/bc_vals.bin");
    auto meta = load<double>(dir + "/meta.bin");   // dim, ndofmax, eps, nssor
    auto prop_ids = load<uint32_t>(dir + "/prop_ids.bin");   // u[prop_ids] = coefs u[prop_dofs] + offsets
    auto prop_dofs = load<uint32_t>(dir + "/prop_dofs.bin");
    auto prop_offsets = load<double>(dir + "/prop_offsets.bin");
    auto prop_coefs = load<double>(dir + "/prop_coefs.bin");
    if (kind.empty() || meta.size() < 4) return 3;
    const int dim = (int)meta[0];
    const int nv = dim == 2 ? 3 : 6;
    try {
        gpu::Assembly K(0);
        for (size_t e = 0; e < kind.size(); e++) {
            gpu::Element el;
            el.kind = kind[e];
            el.dofIds.assign(dof_ids.begin() + dof_ptr[e], dof_ids.begin() + dof_ptr[e + 1]);
            el.gaussPoints.assign(gp.begin() + (size_t)gp_ptr[e] * (dim + 1), gp.begin() + (size_t)gp_ptr[e + 1] * (dim + 1));
            el.jinv.assign(jinv.begin() + e * dim * dim, jinv.begin() + (e + 1) * dim * dim);
            el.C.assign(cmat.begin() + e * nv * nv, cmat.begin() + (e + 1) * nv * nv);
            K.add(el);
        }
        K.setMaxDof((size_t)meta[1]);
        K.setEpsilon(meta[2]);
        K.setSSORIterations((size_t)meta[3]);
        for (size_t i = 0; i < bc_ids.size(); i++)
            K.setPointAlong((gpu::Variable)(bc_ids[i] % dim), bc_vals[i], bc_ids[i] / dim);
        for (size_t i = 0; i < prop_ids.size(); i++) {
            if (prop_dofs[i] / dim != prop_ids[i] / dim) return 5;   // one node per setPointProportional
            K.setPointProportional((gpu::Variable)(prop_ids[i] % dim), (gpu::Variable)(prop_dofs[i] % dim), prop_coefs[i],
                                   prop_offsets[i], prop_ids[i] / dim);
        }
        K.setSolver(solver, 1e-12);
        const bool ok = K.cgsolve();
        save(dir + "/u.bin", K.getDisplacements());
        std::vector<uint32_t> rs, ci;
        std::vector<double> arr;
        K.getMatrix(rs, ci, arr);
        save(dir + "/row_size.bin", rs);
        save(dir + "/column_index.bin", ci);
        save(dir + "/array.bin", arr);
        save(dir + "/rhs.bin", K.getForces());
        std::printf("{\"converged\": %d, \"iterations\": %lld, \"relres\": %.3e}\n", ok ? 1 : 0,
                    (long long)K.lastStats().iterations, K.lastStats().relres);
        return ok ? 0 : 1;
    } catch (const gpu::Error &e) {
        std::fprintf(stderr, "gpu::Error %d: %s\n", (int)e.status, e.what());
        return 4;
    }
}
