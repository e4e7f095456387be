"""The damage oracle (oracle/damage_oracle.cpp) pinned to the reference.

The fixture damage_p1 is the reference's own notched beam in three-point
bending (StiffnessAndFracture + NonLocalMazars + FiberBasedIsotropicLinearDamage,
six load steps through FeatureTree::step, tests/golden/make_golden.py).  It
carries, per element, the reference's centre, circumradius, area and smoothing
neighbourhood (members and weights), and after every load step its
displacements, element strains, smoothed principal fields, criterion scores
and damage, and the number of passes of FeatureTree::stepInternal.

Checked here on the CPU: geometry and neighbourhoods; the grading of every
element from the reference's displacements and damage (scores and smoothed
fields to 1e-12); and a replay of the six load steps by the oracle alone
(assembly with the damaged stiffness, Dirichlet elimination, PCG, grading,
update), which must reproduce the reference's pass counts and damage fields
exactly and its displacements to 1e-9.
"""
import numpy as np
import pytest

from conftest import load_golden

import amie_mesh as am
import oracle as O


def fixture():
    d = load_golden("damage_p1")
    n = int(d["n_elem"][0])
    return d, n, d["elem_xy"].reshape(n, 6)


def law_of(d):
    return O.DamageLaw(threshold=float(d["eps0"][0]), young=float(d["E"][0]), poisson=float(d["nu"][0]),
                       fracture_energy=float(d["Gf"][0]), radius=float(d["radius"][0]), score_tolerance=2e-3,
                       fibre=float(d["fibre"][0]), cutoff=float(d["cutoff"][0]), residual=1e-4)


def state_of(damage, fibre=0.1, cutoff=0.6):
    """The damage model's state behind the reference's exported damage (1 - C_eff / C): a
    number of fibre increments added one by one; a fractured element (C_eff = 1e-4 C) sits
    at the cutoff."""
    out = np.zeros(len(damage))
    for e, dmg in enumerate(damage):
        k = int(round(cutoff / fibre)) if dmg > 0.99 else int(round(dmg / fibre))
        s = 0.0
        for _ in range(k):
            s = min(s + fibre, 1.0)
        out[e] = s
    return out


def exported(state, cutoff=0.6, residual=1e-4):
    return np.where(state >= cutoff, 1.0 - residual, state)


def test_geometry_and_neighbourhoods():
    d, n, xy = fixture()
    c, r, a = O.damage_geometry(xy)
    assert np.abs(c.ravel() - d["elem_centre"]).max() <= 1e-15 * np.abs(c).max()
    assert np.abs(r - d["elem_radius"]).max() <= 1e-11 * r.max()
    assert np.abs(a - d["elem_area"]).max() <= 1e-15 * a.max()
    ptr, idx, coef = O.damage_cache(float(d["radius"][0]), xy, c, r, a)
    cp, ci, cc = d["cache_ptr"], d["cache_idx"], d["cache_coef"]
    for e in range(n):
        ref = dict(zip(ci[cp[e]:cp[e + 1]].tolist(), cc[cp[e]:cp[e + 1]].tolist()))
        mine = dict(zip(idx[ptr[e]:ptr[e + 1]].tolist(), coef[ptr[e]:ptr[e + 1]].tolist()))
        assert ref.keys() == mine.keys(), e
        assert max(abs(ref[j] - mine[j]) for j in ref) <= 1e-14, e
    # neighbourhood of the maxima: every element whose centre is within
    # max(6 R_e, 4 r_e) 2.5 + r_e of the element's centre
    R = float(d["radius"][0])
    ap, ai = d["cache_all_ptr"], d["cache_all_idx"]
    for e in range(n):
        Re = max(R, 1.1 * r[e])
        rho = max(Re * 6.0, r[e] * 4.0) * 2.5 + r[e]
        dx, dy = c[:, 0] - c[e, 0], c[:, 1] - c[e, 1]
        inside = np.nonzero(dx * dx + dy * dy < rho * rho)[0]
        assert set(inside.tolist()) == set(ai[ap[e]:ap[e + 1]].tolist()), e


def test_grade_matches_reference():
    d, n, xy = fixture()
    law = law_of(d)
    c, r, a = O.damage_geometry(xy)
    cache = O.damage_cache(law.radius, xy, c, r, a)
    m = am.from_golden(d, "auto")
    cm = d["cmat"].reshape(n, 9)
    gpw = d["gp"].reshape(-1, 3)[:, 2]
    for k in range(1, int(d["steps"][0]) + 1):
        eps, _ = O.element_fields(m, d[f"u_{k}"])
        ref_eps = d[f"strain_{k}"].reshape(n, 3)
        assert np.abs(eps - ref_eps).max() <= 1e-12 * np.abs(ref_eps).max()
        state = state_of(d[f"damage_{k}"])
        score, sm = O.damage_grade(law, eps, cm, state, a, gpw, cache)
        ref_score = d[f"score_{k}"]
        assert np.array_equal(score == -1.0, ref_score == -1.0)
        assert np.abs(score - ref_score).max() <= 1e-12
        live = ref_score > -1
        ref_sm = d[f"smoothed_{k}"].reshape(n, 4)
        for cols in (slice(0, 2), slice(2, 4)):
            scale = np.abs(ref_sm[live, cols]).max()
            assert np.abs(sm[live, cols] - ref_sm[live, cols]).max() <= 1e-12 * scale, (k, cols)


def replay(d, steps=None, rtol=1e-13):
    """The reference's load steps on the oracle: (passes, state, u) per step."""
    n = int(d["n_elem"][0])
    xy = d["elem_xy"].reshape(n, 6)
    law = law_of(d)
    c, r, a = O.damage_geometry(xy)
    cache = O.damage_cache(law.radius, xy, c, r, a)
    m = am.from_golden(d, "auto")
    cm = d["cmat"].reshape(n, 9)
    gpw = d["gp"].reshape(-1, 3)[:, 2]
    ids = d["bc_ids"].astype(np.uint32)
    kinds = np.zeros(len(ids), np.uint8)
    nsteps = int(d["steps"][0])
    state = np.zeros(n)
    out = []
    for k in range(1, (steps or nsteps) + 1):
        vals = d["bc_values"] * (float(d["deflection"][0]) * k / nsteps)   # the load patch carries -1 per unit
        passes = 0
        while True:
            passes += 1
            m.cscale = np.where(state >= law.cutoff, law.residual, 1.0 - state)
            R = O.assemble(m, ids, vals, kinds)
            u, _, _, rc = O.pcg(2, R["row_size"], R["column_index"], R["array"], R["rhs"], rtol=rtol)
            assert rc == 0
            eps, _ = O.element_fields(m, u)
            score, _ = O.damage_grade(law, eps, cm, state, a, gpw, cache)
            state, changed = O.damage_update(law, c, r, score, state)
            if not changed.any():
                break
        out.append((passes, state.copy(), u))
    return out


def test_replay_matches_reference():
    d = load_golden("damage_p1")
    for k, (passes, state, u) in enumerate(replay(d), start=1):
        assert passes == int(d["sub_iterations"][k - 1]), (k, passes)
        assert np.abs(exported(state) - d[f"damage_{k}"]).max() <= 1e-12, k
        ref_u = d[f"u_{k}"]
        assert np.abs(u - ref_u).max() <= 1e-9 * np.abs(ref_u).max(), k


def test_fracture_leaves_later_maxima():
    """Elements are stepped in mesh order: a neighbour that fractured earlier in the
    same pass no longer counts in the neighbourhood maximum (the rule the reference's
    loop follows; without it the replay's second load step diverges)."""
    law = O.DamageLaw(threshold=1e-4, young=35e9, poisson=0.2, fracture_energy=100.0, radius=0.002,
                      score_tolerance=2e-3, fibre=0.1, cutoff=0.6, residual=1e-4)
    centre = np.array([[0.0, 0.0], [0.001, 0.0], [0.002, 0.0]])
    radius = np.full(3, 0.0005)
    # element 0 is about to fracture and has the largest score; element 2 is within
    # tolerance of element 1 only once element 0 no longer counts
    score = np.array([0.9, 0.5, 0.499])
    state = np.array([0.5, 0.0, 0.0])
    new, changed = O.damage_update(law, centre, radius, score, state)
    assert new[0] >= law.cutoff and changed.tolist() == [True, True, True]
    # with element 0 not fracturing (state 0.3 -> 0.4) elements 1 and 2 stay below its maximum
    new, changed = O.damage_update(law, centre, radius, score, np.array([0.3, 0.0, 0.0]))
    assert changed.tolist() == [True, False, False]
