"""Device integration rules of crack-crossed triangles (amie_cut_rules) against
the CPU restatement (oracle/cut_rules.py) and the reference's fixtures.

* golden crack cases: the same status and number of points as the
  restatement for every Heaviside-enriched element, the points and weights to
  1e-13, the Heaviside values equal; the element matrices computed on the
  device from the device rules match the reference's K_e to 1e-9 (its
  Heaviside gradients are finite differences) and the oracle's K_e on the same
  rules to 1e-13;
* seeded random triangles around a kinked polyline (crossed, tip, kink, not
  cut, hints near corners): status, points and Heaviside values as the
  restatement's;
* a known answer: the right triangle cut at half height;
* with AMIE_CUT_REPLACE_MONTE_CARLO: the same as the restatement, the elements
  the reference integrated by Monte-Carlo replaced by conforming rules whose
  device element matrices equal an independent exact rule's to 1e-12.
"""
import numpy as np
import pytest

from conftest import load_golden

import amie_mesh as am
import crack_cases as CC
import cut_rules as CR
import oracle as O

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def assert_same_rules(dev, ref, scale):
    """Equal status, count and Heaviside values; points matched one to one
    (reference coordinates to 1e-13, weights to 1e-13 of the element's scale)."""
    cnt, st, rule, hp, hv = dev
    rcnt, rst, rrule, rhp, rhv = ref
    assert np.array_equal(st, rst)
    assert np.array_equal(cnt, rcnt)
    assert np.array_equal(hv, rhv)
    for e in np.nonzero(np.isin(st, (CR.OK, CR.REPLACED)))[0]:
        n = int(cnt[e])
        a, b = rule[e, :n], rrule[e, :n]
        d = np.abs(a[:, None, :2] - b[None, :, :2]).max(axis=2)
        j = d.argmin(axis=1)
        assert d[np.arange(n), j].max() <= 1e-13, e
        assert len(set(j.tolist())) == n, e
        assert np.abs(a[:, 2] - b[j, 2]).max() <= 1e-13 * scale[e], e
        assert np.array_equal(hp[e, :n], rhp[e, j]), e


@pytest.mark.parametrize("name", ["crack_p1", "crack_p2"])
def test_cut_rules_golden(gpu_ctx, name):
    import amie_gpu
    d = load_golden(name)
    m = am.from_golden(d, "auto")
    elems = CC.heaviside_elements(m)
    corners = CC.corners(d, m, elems)
    line = CC.crack_line(d)
    dev = gpu_ctx.cut_rules(corners, line)
    ref = CR.cut_rules(corners, line)
    area = np.array([m.gp[3 * m.gp_ptr[e] + 2:3 * m.gp_ptr[e + 1]:3].sum() for e in elems])
    assert_same_rules(dev, ref, area)
    cnt, st, rule, hp, hv = dev
    ok = np.nonzero(st == amie_gpu.CUT_OK)[0]
    ngp = np.diff(m.gp_ptr.astype(np.int64))[elems]
    assert np.array_equal(cnt[ok], ngp[ok])
    sub = CC.submesh(m, elems[ok], cnt[ok], rule[ok], hp[ok], hv[ok])
    t = amie_gpu.Topology(gpu_ctx, sub)
    try:
        t.assemble()
        off, ke = t.element_matrices()
    finally:
        t.close()
    _, ko = O.element_matrices(sub)
    for i, e in enumerate(elems[ok]):
        a, b = int(off[i]), int(off[i + 1])
        assert rel(ke[a:b], ko[a:b]) <= 1e-13, e
        assert rel(ke[a:b], CC.golden_ke(d, e)) <= 1e-9, e


def random_cases(n, seed):
    """Triangles of random shape and orientation near a 4-point polyline."""
    rng = np.random.default_rng(seed)
    line = np.array([[0.0, 0.0], [1.0, 0.15], [1.8, -0.2], [2.5, 0.3]])
    seg = rng.integers(0, 3, n)
    t = rng.uniform(-0.15, 1.15, n)
    centre = line[seg] + t[:, None] * (line[seg + 1] - line[seg]) + rng.normal(0, 0.05, (n, 2))
    size = rng.uniform(0.05, 0.3, n)
    ang = rng.uniform(0, 2 * np.pi, (n, 3)) + np.array([0, 2.1, 4.2])
    rad = size[:, None] * rng.uniform(0.4, 1.0, (n, 3))
    pts = centre[:, None, :] + rad[..., None] * np.stack([np.cos(ang), np.sin(ang)], -1)
    flip = rng.random(n) < 0.5
    pts[flip] = pts[flip][:, ::-1]
    return pts.reshape(n, 6), line


def test_cut_rules_random(gpu_ctx):
    corners, line = random_cases(3000, 7)
    dev = gpu_ctx.cut_rules(corners, line)
    ref = CR.cut_rules(corners, line)
    X = corners.reshape(-1, 3, 2)
    area = 0.5 * np.abs((X[:, 1, 0] - X[:, 0, 0]) * (X[:, 2, 1] - X[:, 0, 1])
                        - (X[:, 1, 1] - X[:, 0, 1]) * (X[:, 2, 0] - X[:, 0, 0]))
    assert_same_rules(dev, ref, area)
    st = dev[1]
    # every outcome occurs
    for code in (CR.OK, CR.NOT_CUT, CR.MONTE_CARLO, CR.ORDER_DEPENDENT):
        assert (st == code).sum() > 0, code
    # the rules integrate the element's area
    ok = st == CR.OK
    assert rel(dev[2][ok, :, 2].sum(axis=1), area[ok]) <= 1e-12


def test_cut_rules_known_answer(gpu_ctx):
    """Corners at reference positions scaled by 2: the line y = 1 (half height)
    cuts off the top triangle (area 0.5) from the trapezoid below (area 1.5);
    the witness lies above, so points below are +1 and the top corner -1."""
    corners = np.array([[0.0, 2.0, 0.0, 0.0, 2.0, 0.0]])
    line = np.array([[-1.0, 1.0], [3.0, 1.0]])
    cnt, st, rule, hp, hv = gpu_ctx.cut_rules(corners, line)
    assert st[0] == CR.OK and cnt[0] == 12
    assert hv[0].tolist() == [-1, 1, 1]
    n = int(cnt[0])
    w, h = rule[0, :n, 2], hp[0, :n]
    eta = rule[0, :n, 1]
    assert np.all((eta > 0.5) == (h == -1))
    assert abs(w[h == -1].sum() - 0.5) <= 1e-14 and abs(w[h == 1].sum() - 1.5) <= 1e-14


@pytest.mark.parametrize("name", ["crack_p1", "crack_p2"])
def test_cut_rules_replacement_golden(gpu_ctx, name):
    import amie_gpu
    d = load_golden(name)
    m = am.from_golden(d, "auto")
    elems = CC.heaviside_elements(m)
    corners = CC.corners(d, m, elems)
    line = CC.crack_line(d)
    dev = gpu_ctx.cut_rules(corners, line, amie_gpu.CUT_REPLACE_MONTE_CARLO)
    ref = CR.cut_rules(corners, line, CR.REPLACE_MONTE_CARLO)
    area = np.array([m.gp[3 * m.gp_ptr[e] + 2:3 * m.gp_ptr[e + 1]:3].sum() for e in elems])
    assert_same_rules(dev, ref, area)
    cnt, st, rule, hp, hv = dev
    ngp = np.diff(m.gp_ptr.astype(np.int64))[elems]
    assert np.array_equal(st == amie_gpu.CUT_REPLACED, ngp == 512)
    for i in np.nonzero(st == amie_gpu.CUT_REPLACED)[0]:
        split = CR.split_rule_degree4(corners[i], line)
        assert split is not None
        e = elems[i:i + 1]
        sub = CC.submesh(m, e, cnt[i:i + 1], rule[i:i + 1], hp[i:i + 1], hv[i:i + 1])
        t = amie_gpu.Topology(gpu_ctx, sub)
        try:
            t.assemble()
            _, ke = t.element_matrices()
        finally:
            t.close()
        n = len(split)
        srule = np.array([[(p[0], p[1], p[2]) for p in split]])
        shp = np.array([[p[3] for p in split]], np.int8)
        _, ks = O.element_matrices(CC.submesh(m, e, np.array([n]), srule, shp, hv[i:i + 1]))
        assert rel(ke, ks) <= 1e-12, int(elems[i])


def test_cut_rules_replacement_random(gpu_ctx):
    import amie_gpu
    corners, line = random_cases(3000, 7)
    base = gpu_ctx.cut_rules(corners, line)
    dev = gpu_ctx.cut_rules(corners, line, amie_gpu.CUT_REPLACE_MONTE_CARLO)
    ref = CR.cut_rules(corners, line, CR.REPLACE_MONTE_CARLO)
    X = corners.reshape(-1, 3, 2)
    area = 0.5 * np.abs((X[:, 1, 0] - X[:, 0, 0]) * (X[:, 2, 1] - X[:, 0, 1])
                        - (X[:, 1, 1] - X[:, 0, 1]) * (X[:, 2, 0] - X[:, 0, 0]))
    assert_same_rules(dev, ref, area)
    fell_back = np.isin(base[1], (CR.MONTE_CARLO, CR.ORDER_DEPENDENT))
    assert (dev[1] == CR.REPLACED).sum() > 0
    assert np.all(dev[1][~fell_back] == base[1][~fell_back])
    assert np.all(np.isin(dev[1][fell_back], (CR.REPLACED, CR.MONTE_CARLO)))
    ok = np.isin(dev[1], (CR.OK, CR.REPLACED))
    assert rel(dev[2][ok, :, 2].sum(axis=1), area[ok]) <= 1e-12
