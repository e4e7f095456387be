"""Element data of the AMIE FE hot path, as plain numpy arrays.

``MeshData`` carries exactly what ``amie_mesh`` (include/amie_gpu.h) carries
across the C-ABI: what AMIE's ``Assembly`` holds per element when
``Assembly::cgsolve`` runs (solvers/assembly.h:228-450):

* the DOF ids of ``ElementarySurface::getDofIds`` (elements/elements.cpp:204):
  node ids first, then enrichment ids (>= number of mesh nodes);
* the Gauss points with weights already multiplied by det J
  (elements/elements.cpp:939-945); an element with no Gauss points uses its
  kind's default rule;
* the inverse Jacobian cached at the centroid (mesher/delaunay.cpp:2436), or,
  for elements whose nodes were moved onto a curved boundary, one inverse
  Jacobian per Gauss point (mesher/delaunay.cpp:2441-2447);
* the behaviour tensor C (``Form::param``, physics/stiffness.cpp:43) through a
  material table, times a per-element factor (damage 1-d, or a per-element
  modulus), and the ``Assembly::add`` scale;
* enrichment functions: Heaviside ``N_k^{P1} (H - H_k)`` (features/crack.cpp:1316)
  as an int8 jump per Gauss point, or any other function as its local-coordinate
  gradient tabulated per Gauss point (what ``VirtualMachine::deval`` returns,
  polynomial/vm_base.cpp:1115).
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import Optional

import numpy as np

TRI3, TRI6, TET4 = 1, 2, 3
ENR_TABULATED, ENR_HEAVISIDE, ENR_TIP = 0, 1, 2
NSHAPE = {TRI3: 3, TRI6: 6, TET4: 4}

# Multiplier kinds accepted by the Dirichlet step.
BC_DISPLACEMENT, BC_FORCE = 0, 1


@dataclass
class MeshData:
    dim: int
    stride: int
    kind: np.ndarray            # uint8 [n_elem]
    dof_ptr: np.ndarray         # uint32 [n_elem+1]
    dof_ids: np.ndarray         # uint32
    gp_ptr: np.ndarray          # uint32 [n_elem+1]
    gp: np.ndarray              # float64 [(dim+1) * n_gp]
    jinv: np.ndarray            # float64 [n_elem*dim*dim]
    mat: np.ndarray             # uint32 [n_elem]
    cmat_table: np.ndarray      # float64 [n_mat*nv*nv]
    ndofmax: int = 0
    moved: Optional[np.ndarray] = None    # uint8 [n_elem]: 1 = per-GP inverse Jacobian
    jinv_gp: Optional[np.ndarray] = None  # float64 [n_gp*dim*dim]
    cscale: Optional[np.ndarray] = None   # float64 [n_elem]
    scale: Optional[np.ndarray] = None    # float64 [n_elem]
    enr_ptr: Optional[np.ndarray] = None  # uint32 [n_elem+1]
    enr_type: Optional[np.ndarray] = None     # uint8 [n_enr]
    enr_vertex: Optional[np.ndarray] = None   # uint8 [n_enr]
    enr_data: Optional[np.ndarray] = None     # uint32 [n_enr]
    enr_jump: Optional[np.ndarray] = None     # int8 [n_enr_gp]
    enr_grad: Optional[np.ndarray] = None     # float64 [dim*n_enr_gp]
    enr_tip: Optional[np.ndarray] = None      # float64 [8*n_enr_tip]: tip branch-function records
    extra: dict = field(default_factory=dict)

    @property
    def n_elem(self) -> int:
        return int(len(self.kind))

    @property
    def nv(self) -> int:
        return 3 if self.dim == 2 else 6

    def __post_init__(self):
        self.kind = np.ascontiguousarray(self.kind, dtype=np.uint8)
        for name in ("dof_ptr", "dof_ids", "gp_ptr", "mat"):
            setattr(self, name, np.ascontiguousarray(getattr(self, name), dtype=np.uint32))
        for name in ("gp", "jinv", "cmat_table"):
            setattr(self, name, np.ascontiguousarray(getattr(self, name), dtype=np.float64))
        n = self.n_elem
        if self.enr_ptr is None:
            self.enr_ptr = np.zeros(n + 1, np.uint32)
            self.enr_type = np.zeros(0, np.uint8)
            self.enr_vertex = np.zeros(0, np.uint8)
            self.enr_data = np.zeros(0, np.uint32)
            self.enr_jump = np.zeros(0, np.int8)
            self.enr_grad = np.zeros(0, np.float64)
        self.enr_ptr = np.ascontiguousarray(self.enr_ptr, dtype=np.uint32)
        self.enr_type = np.ascontiguousarray(self.enr_type, dtype=np.uint8)
        self.enr_vertex = np.ascontiguousarray(self.enr_vertex, dtype=np.uint8)
        self.enr_data = np.ascontiguousarray(self.enr_data, dtype=np.uint32)
        self.enr_jump = np.ascontiguousarray(self.enr_jump, dtype=np.int8)
        self.enr_grad = np.ascontiguousarray(self.enr_grad, dtype=np.float64)
        if self.enr_tip is not None:
            self.enr_tip = np.ascontiguousarray(self.enr_tip, dtype=np.float64)
        if self.moved is not None:
            self.moved = np.ascontiguousarray(self.moved, dtype=np.uint8)
            self.jinv_gp = np.ascontiguousarray(self.jinv_gp, dtype=np.float64)
        if self.cscale is not None:
            self.cscale = np.ascontiguousarray(self.cscale, dtype=np.float64)
        if self.scale is not None:
            self.scale = np.ascontiguousarray(self.scale, dtype=np.float64)
        if not self.ndofmax:
            self.ndofmax = int(self.dof_ids.max()) + 1 if len(self.dof_ids) else 0

    # ---------------------------------------------------------------- helpers
    def nf(self) -> np.ndarray:
        """Functions (shape + enrichment) per element."""
        return np.diff(self.dof_ptr.astype(np.int64))

    def ke_offsets(self) -> np.ndarray:
        """Offsets (in doubles) of each dense (nf*s)^2 element matrix."""
        sz = (self.nf() * self.stride) ** 2
        off = np.zeros(self.n_elem + 1, np.uint64)
        np.cumsum(sz, out=off[1:])
        return off

    def validate(self) -> None:
        n = self.n_elem
        assert self.dim in (2, 3) and self.stride == self.dim
        assert len(self.dof_ptr) == n + 1 and len(self.gp_ptr) == n + 1
        assert len(self.enr_ptr) == n + 1
        assert len(self.jinv) == n * self.dim * self.dim
        assert len(self.mat) == n
        nsh = np.array([NSHAPE.get(int(k), 0) for k in np.unique(self.kind)])
        assert (nsh > 0).all(), "unknown element kind"
        shape = np.vectorize(lambda k: NSHAPE[int(k)])(self.kind) if n else np.zeros(0)
        assert np.array_equal(self.nf(), shape + np.diff(self.enr_ptr.astype(np.int64))), \
            "dof count must equal shape + enrichment functions"
        assert int(self.mat.max(initial=0)) < len(self.cmat_table) // (self.nv * self.nv)


def tip_record(first, second, third, tip, angle, branch):
    """The 8 doubles of an AMIE_ENR_TIP function of a straight-sided triangle with
    corners first (local (0,1)), second (0,0), third (1,0): x(0,0) - tip,
    dx/dxi, dx/deta, the crack angle at the tip, the branch index."""
    o = np.asarray(second, float) - np.asarray(tip, float)
    a = np.asarray(third, float) - np.asarray(second, float)
    b = np.asarray(first, float) - np.asarray(second, float)
    return np.array([o[0], o[1], a[0], a[1], b[0], b[1], float(angle), float(branch)])


def tip_values(rec, vertex, xi, eta):
    """Values of the tip branch function of `rec` attached to P1 vertex `vertex` at
    local points (xi, eta): N_v (F_j(x) - F_j(x_v)) (BranchedCrack::enrichTip,
    features/crack.cpp:898-960; t as the reference's atan2 token gives it)."""
    xi = np.asarray(xi, float)
    eta = np.asarray(eta, float)
    a, j = rec[6], int(rec[7])

    def F(s0, s1):
        dx = rec[0] + s0 * rec[2] + s1 * rec[4]
        dy = rec[1] + s0 * rec[3] + s1 * rec[5]
        t = -np.arctan2(-np.sin(a) * dx + np.cos(a) * dy, np.cos(a) * dx + np.sin(a) * dy)
        g = [np.sin(t / 2), np.cos(t / 2), np.sin(t / 2) * np.sin(t), np.cos(t / 2) * np.sin(t)][j]
        return np.sqrt(np.hypot(dx, dy)) * g

    vx, vy = [(0.0, 1.0), (0.0, 0.0), (1.0, 0.0)][vertex]
    N = [eta, 1 - xi - eta, xi][vertex]
    return N * (F(xi, eta) - F(vx, vy))


def from_golden(d, enrichment: str = "auto", tips=()) -> MeshData:
    """Build MeshData from a reference fixture (tests/golden/*.npz).

    enrichment = "tabulated": every enrichment function carries the gradients
    the reference's VM produced (finite differences included); "auto": functions
    whose values are exactly N_k^{P1} * {-2, 0, 2} become Heaviside jumps, the
    rest stay tabulated; "tip": as "auto", and functions whose values are those
    of a tip branch function of one of `tips` ((x, y), angle) to 1e-12 on a
    straight-sided triangle become AMIE_ENR_TIP records.
    """
    dim = int(d["dim"][0])
    kind = d["elem_kind"].astype(np.uint8)
    n = len(kind)
    nv = 3 if dim == 2 else 6
    cm = d["cmat"].reshape(n, nv * nv)
    table, mat = np.unique(cm, axis=0, return_inverse=True)
    gp = d["gp"]
    gp_ptr = d["gp_ptr"]
    enr_ptr = d["enr_ptr"]
    egp = d["enr_gp_ptr"]
    nenr = len(d["enr_vertex"])
    enr_type = np.zeros(nenr, np.uint8)
    enr_jump = np.zeros(int(egp[-1]) if nenr else 0, np.int8)
    enr_grad = d["enr_grad"].copy()
    enr_data = egp[:-1].astype(np.uint32) if nenr else np.zeros(0, np.uint32)
    tip_recs = []
    if nenr and enrichment in ("auto", "tip"):
        g2 = gp.reshape(-1, dim + 1)
        for e in np.nonzero(np.diff(enr_ptr))[0]:
            pts = g2[gp_ptr[e]:gp_ptr[e + 1], :dim]
            N = [pts[:, 1], 1 - pts[:, 0] - pts[:, 1], pts[:, 0]]
            for j in range(enr_ptr[e], enr_ptr[e + 1]):
                k = int(d["enr_vertex"][j])
                if k > 2:
                    continue
                vals = d["enr_val"][egp[j]:egp[j + 1]]
                with np.errstate(divide="ignore", invalid="ignore"):
                    q = np.where(np.abs(N[k]) > 1e-14, vals / N[k], 0.0)
                r = np.round(q / 2) * 2
                if np.all(np.abs(q - r) < 1e-9) and np.all(np.isin(r, (-2, 0, 2))):
                    enr_type[j] = ENR_HEAVISIDE
                    enr_jump[egp[j]:egp[j + 1]] = r.astype(np.int8)
                    continue
                if enrichment != "tip" or dim != 2 or ("elem_moved" in d and d["elem_moved"][e]):
                    continue
                ns = 6 if kind[e] == TRI6 else 3
                xy0 = int(np.sum(np.where(kind[:e] == TRI6, 6, 3))) * 2
                pts_xy = d["elem_xy"][xy0:xy0 + 2 * ns].reshape(ns, 2)
                first, second, third = pts_xy[[0, 2, 4]] if ns == 6 else pts_xy
                scale = max(np.abs(vals).max(), 1e-300)
                for tip, angle in tips:
                    hit = None
                    for br in range(4):
                        rec = tip_record(first, second, third, tip, angle, br)
                        if np.abs(tip_values(rec, k, pts[:, 0], pts[:, 1]) - vals).max() <= 1e-12 * scale:
                            hit = rec
                            break
                    if hit is not None:
                        enr_type[j] = ENR_TIP
                        enr_data[j] = len(tip_recs)
                        tip_recs.append(hit)
                        break
    vert = d["enr_vertex"].astype(np.int64)
    vert[vert > 2] = 0
    m = MeshData(dim=dim, stride=dim, kind=kind, dof_ptr=d["elem_dof_ptr"], dof_ids=d["elem_dof_ids"],
                 gp_ptr=gp_ptr, gp=gp, jinv=d["jinv"],
                 moved=d["elem_moved"].astype(np.uint8) if "elem_moved" in d else None,
                 jinv_gp=d["jinv_gp"] if "jinv_gp" in d else None, mat=mat.reshape(-1).astype(np.uint32),
                 cmat_table=table.reshape(-1), ndofmax=int(d["ndofmax"][0]),
                 scale=d["elem_scale"], enr_ptr=enr_ptr, enr_type=enr_type,
                 enr_vertex=vert.astype(np.uint8), enr_data=enr_data, enr_jump=enr_jump,
                 enr_grad=enr_grad, enr_tip=np.concatenate(tip_recs) if tip_recs else None)
    return m


# LagrangeMultiplierType values (solvers/assembly.h:36-96): the force types are
# added to the right-hand side after elimination, SET_PROPORTIONAL_DISPLACEMENT
# multipliers are substituted after it (golden_proportional), GENERAL is not
# supported, every other type is an eliminated displacement
# (solvers/assembly.cpp:163-169).
LM_FORCE_TYPES = (34, 35, 36, 37)          # SET_FORCE_XI, _ETA, _ZETA, _INDEXED_AXIS
LM_PROPORTIONAL = 23                       # SET_PROPORTIONAL_DISPLACEMENT
LM_UNSUPPORTED = (0,)                      # GENERAL


def golden_bcs(d):
    """Displacement and force multipliers of a fixture as (ids, values, kinds), sorted by
    id as make_final sorts them (proportional ones: golden_proportional)."""
    ids = d["bc_ids"].astype(np.uint32)
    vals = d["bc_values"].astype(np.float64)
    types = d["bc_types"].astype(np.int64)
    if np.isin(types, LM_UNSUPPORTED).any():
        raise ValueError("GENERAL multipliers are not supported")
    keep = types != LM_PROPORTIONAL
    ids, vals, types = ids[keep], vals[keep], types[keep]
    kinds = np.where(np.isin(types, LM_FORCE_TYPES), BC_FORCE, BC_DISPLACEMENT).astype(np.uint8)
    order = np.argsort(ids, kind="stable")
    return ids[order], vals[order], kinds[order]


def golden_proportional(d):
    """SET_PROPORTIONAL_DISPLACEMENT multipliers of a fixture, sorted by id as
    make_final sorts them: (ids, offsets, ptr, prop_ids, coefs)."""
    types = d["bc_types"].astype(np.int64)
    sel = np.nonzero(types == LM_PROPORTIONAL)[0]
    if not len(sel) or "bc_prop_ptr" not in d:
        return (np.zeros(0, np.uint32), np.zeros(0), np.zeros(1, np.uint32), np.zeros(0, np.uint32), np.zeros(0))
    pp = d["bc_prop_ptr"].astype(np.int64)
    sel = sel[np.argsort(d["bc_ids"][sel], kind="stable")]
    ids = d["bc_ids"][sel].astype(np.uint32)
    offs = d["bc_values"][sel].astype(np.float64)
    ptr = [0]
    pids, coefs = [], []
    for i in sel:
        pids.extend(d["bc_prop_ids"][pp[i]:pp[i + 1]].tolist())
        coefs.extend(d["bc_prop_coefs"][pp[i]:pp[i + 1]].tolist())
        ptr.append(len(pids))
    return ids, offs, np.array(ptr, np.uint32), np.array(pids, np.uint32), np.array(coefs)
