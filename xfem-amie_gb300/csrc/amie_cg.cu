// amie_cg.cu -- ConjugateGradient::solve semantics on the device (see amie_gpu.h).
#include "solver.cuh"

namespace amie {

amie_status amie_cg_solve(amie_topo *t, const amie_solve_opts *o, amie_solve_stats *st)
{
    (void)t; (void)o; (void)st;
    set_error("AMIE_SOLVER_AMIE_CG is not available in this build");
    return AMIE_BAD_INPUT;
}

}  // namespace amie
