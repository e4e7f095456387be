"""The damage path on the GPU (xfem-amie_gb300/csrc/damage.cu) against the
reference's notched beam (fixture damage_p1) and the oracle.

* grading: from the reference's displacements and damage after each load step,
  the device scores and smoothed principal fields equal the reference's to 1e-12,
  and the bounded grading (no smoothed fields wanted) gives the same score bits;
* update: on a state with elements about to fracture, the device step equals
  the oracle's (same damage, same number of changes), including the rule that
  an element fractured earlier in a pass leaves the neighbourhood maxima of the
  elements after it;
* load steps: the six load steps replayed on the device (assembly of the
  damaged stiffness, elimination, solve, grading, update until nothing changes)
  give the reference's number of passes and damage field at every step, and
  its displacements to 1e-9 (FP64 solver at rtol 1e-12) or 1e-8 (mixed solver
  at rtol 1e-10).
"""
import numpy as np
import pytest

from conftest import load_golden
from test_damage_oracle import exported, law_of, state_of

import amie_mesh as am
import oracle as O

pytestmark = pytest.mark.gpu


def device_law(d):
    import amie_gpu
    return amie_gpu.DamageLaw(amie_gpu.DAMAGE_FIBER_ISOTROPIC, float(d["eps0"][0]), float(d["E"][0]),
                              float(d["nu"][0]), float(d["Gf"][0]), float(d["radius"][0]), 2e-3,
                              float(d["fibre"][0]), float(d["cutoff"][0]), 1e-4)


def damage_topology(ctx, d):
    import amie_gpu
    m = am.from_golden(d, "auto")
    t = amie_gpu.Topology(ctx, m)
    t.assemble()
    t.damage_setup(device_law(d), d["elem_xy"])
    return t, m


def test_device_grade_matches_reference(gpu_ctx):
    d = load_golden("damage_p1")
    n = int(d["n_elem"][0])
    t, m = damage_topology(gpu_ctx, d)
    try:
        for k in range(1, int(d["steps"][0]) + 1):
            t.damage_set_state(state_of(d[f"damage_{k}"]))
            t.solution_upload(d[f"u_{k}"])
            score, sm = t.damage_grade()
            bounded, none = t.damage_grade(smoothed=False)
            assert none is None
            assert np.array_equal(bounded.view(np.uint64), score.view(np.uint64)), k
            ref = d[f"score_{k}"]
            assert np.array_equal(score == -1.0, ref == -1.0), k
            assert np.abs(score - ref).max() <= 1e-12, k
            live = ref > -1
            ref_sm = d[f"smoothed_{k}"].reshape(n, 4)
            for cols in (slice(0, 2), slice(2, 4)):
                scale = np.abs(ref_sm[live, cols]).max()
                assert np.abs(sm[live, cols] - ref_sm[live, cols]).max() <= 1e-12 * scale, (k, cols)
    finally:
        t.close()


def test_device_update_matches_oracle(gpu_ctx):
    """A pass far from equilibrium: the step-2 displacements quadrupled, on the
    step-2 damage with the criterion-meeting elements raised to 0.5, so that
    their increments fracture them in this pass."""
    d = load_golden("damage_p1")
    n = int(d["n_elem"][0])
    law = law_of(d)
    xy = d["elem_xy"].reshape(n, 6)
    c, r, a = O.damage_geometry(xy)
    cache = O.damage_cache(law.radius, xy, c, r, a)
    state = state_of(d["damage_2"])
    u = 4.0 * d["u_2"]
    t, m = damage_topology(gpu_ctx, d)
    try:
        t.damage_set_state(state)
        t.solution_upload(u)
        met = t.damage_grade()[0] > 0
        state = np.where(met, state_of(np.full(n, 0.5)), state)
        t.damage_set_state(state)
        score, _ = t.damage_grade()
        eps, _ = O.element_fields(m, u)
        score_o, _ = O.damage_grade(law, eps, d["cmat"].reshape(n, 9), state, a, d["gp"].reshape(-1, 3)[:, 2], cache)
        assert np.abs(score - score_o).max() <= 1e-12
        assert (score > 0).sum() > 5
        changed = t.damage_update()
        new_o, ch_o = O.damage_update(law, c, r, score_o, state)
        assert changed == int(ch_o.sum()) and changed > 0
        new = t.damage_state()
        assert np.array_equal(new, new_o)
        assert ((new >= law.cutoff) & (state < law.cutoff)).sum() > 0   # some elements fractured in the pass
    finally:
        t.close()


@pytest.mark.parametrize("solver,rtol,utol", [("fp64", 1e-12, 1e-9), ("mixed", 1e-10, 1e-8)])
def test_device_load_steps_match_reference(gpu_ctx, solver, rtol, utol):
    """FP64 at rtol 1e-12, and the mixed FP32/FP64 solver at rtol 1e-10: the damage
    decisions are the reference's in both."""
    import amie_gpu
    sv = amie_gpu.SOLVER_PCG_FP64 if solver == "fp64" else amie_gpu.SOLVER_PCG_MIXED
    d = load_golden("damage_p1")
    t, m = damage_topology(gpu_ctx, d)
    ids = d["bc_ids"].astype(np.uint32)
    kinds = np.zeros(len(ids), np.uint8)
    nsteps = int(d["steps"][0])
    try:
        for k in range(1, nsteps + 1):
            t.apply_dirichlet(ids, d["bc_values"] * (float(d["deflection"][0]) * k / nsteps), kinds)
            st = t.damage_load_step(sv, rtol=rtol, warm=k > 1)
            assert st["sub_iterations"] == int(d["sub_iterations"][k - 1]), (k, st)
            assert st["smoothed"] <= st["sub_iterations"] * m.n_elem, (k, st)
            if k > 1:   # damage grows: the elements that meet the criterion were smoothed
                assert st["smoothed"] > 0, (k, st)
            else:   # below the threshold away from the notch: most elements skip the smoothing
                assert st["smoothed"] < m.n_elem, st
            state = t.damage_state()
            assert np.abs(exported(state) - d[f"damage_{k}"]).max() <= 1e-12, k
            assert st["damaged"] == int((d[f"damage_{k}"] > 0).sum())
            u = t.solution()
            ref_u = d[f"u_{k}"]
            assert np.abs(u - ref_u).max() <= utol * np.abs(ref_u).max(), k
    finally:
        t.close()
