"""The premise of the bounded damage grading (k_dmg_grade with a cell bound,
xfem-amie_gb300/csrc/damage.cu), checked on the oracle's own arithmetic
(oracle/damage_oracle.cpp, NonLocalMazars::gradeAtTime): the tensile strain
norm sqrt(<e1>+^2 + <e2>+^2 + <ezz>+^2) of a smoothed (weighted-average) strain
is at most the largest norm among the averaged strains, and an element whose
neighbourhood stays at or below the threshold gets the score -d."""
import numpy as np

import oracle as O
import workloads as W


def _norm(pe, nu):
    ezz = -nu * (pe[:, 0] + pe[:, 1]) / (1.0 - nu)
    pos = lambda v: 0.5 * (np.abs(v) + v)
    return np.sqrt(pos(pe[:, 0]) ** 2 + pos(pe[:, 1]) ** 2 + pos(ezz) ** 2)


def test_smoothed_norm_bounded_by_neighbours():
    rng = np.random.default_rng(11)
    n, k, nu, thr = 600, 24, 0.2, 1e-4
    law = O.DamageLaw(thr, 30e9, nu, 100.0, 0.005, 2e-3, 0.1, 0.6, 1e-4)
    strain = rng.normal(0.0, 6e-5, (n, 3))
    strain[: n // 3] *= 0.3                      # a third of the elements well below the threshold
    strain[2 * (n // 3):] += [2e-4, 1e-4, 0.0]   # and a third pulled past it
    cmat = np.tile(W.plane_stress(30e9, nu).ravel(), (n, 1))
    state = rng.uniform(0.0, 0.5, n)
    area = rng.uniform(0.5, 2.0, n) * 1e-6
    gpw = rng.uniform(0.2, 1.0, n)
    # neighbourhoods: the element and k - 1 others of its third, positive weights summing to one
    idx, ptr = [], [0]
    for e in range(n):
        lo = (e // (n // 3)) * (n // 3)
        nb = np.concatenate([[e], rng.choice(np.setdiff1d(np.arange(lo, lo + n // 3), [e]), k - 1, replace=False)])
        idx.extend(sorted(nb.tolist()))
        ptr.append(len(idx))
    idx = np.array(idx, np.uint32)
    ptr = np.array(ptr, np.uint64)
    coef = rng.uniform(0.1, 1.0, len(idx))
    for e in range(n):
        coef[ptr[e]:ptr[e + 1]] /= coef[ptr[e]:ptr[e + 1]].sum()
    score, sm = O.damage_grade(law, strain, cmat, state, area, gpw, (ptr, idx, coef))
    # each element's own norm, through the same arithmetic (a neighbourhood of itself)
    selfc = (np.arange(n + 1, dtype=np.uint64), np.arange(n, dtype=np.uint32), np.ones(n))
    _, sm_self = O.damage_grade(law, strain, cmat, state, area, gpw, selfc)
    f_self = _norm(sm_self[:, 2:4], nu)
    f_smooth = _norm(sm[:, 2:4], nu)
    bound = np.array([f_self[idx[ptr[e]:ptr[e + 1]]].max() for e in range(n)])
    assert (f_smooth <= bound * (1 + 1e-12) + 1e-300).all()
    below = bound * (1 + 1e-6) <= thr
    assert below.sum() >= 50 and (f_smooth > thr).sum() >= 50
    assert np.array_equal(score[below], -state[below])
