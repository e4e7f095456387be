"""ctypes binding of libamie_gpu.so (include/amie_gpu.h) and a host-side
mirror of AMIE's ``Assembly`` for the element-stiffness -> scatter -> CG path.

``Assembly`` keeps the reference's method names and meaning
(solvers/assembly.h:228-450): elements are added, Dirichlet multipliers set with
``setPointAlong``, ``cgsolve`` solves, ``getMatrix`` / ``getForces`` /
``getDisplacements`` return the results.  Everything runs on the GPU through the
C-ABI; there is no CPU fallback: loading fails loudly if the library or a GPU is
missing.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Optional

import numpy as np

import amie_mesh as am

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libamie_gpu.so")

AMIE_OK, AMIE_NOT_CONVERGED, AMIE_NAN, AMIE_OOM, AMIE_BAD_INPUT, AMIE_TIMEOUT, AMIE_CUDA_ERROR, \
    AMIE_NOT_READY, AMIE_CANCELLED = range(9)
STATUS_NAMES = ["OK", "NOT_CONVERGED", "NAN", "OOM", "BAD_INPUT", "TIMEOUT", "CUDA_ERROR", "NOT_READY",
                "CANCELLED"]
SOLVER_PCG_FP64, SOLVER_PCG_MIXED, SOLVER_AMIE_CG = 0, 1, 2

EXPORTED = [
    "amie_ctx_create", "amie_ctx_destroy", "amie_last_error", "amie_abi_version", "amie_topology_build",
    "amie_topology_destroy", "amie_topology_sizes", "amie_topology_pattern", "amie_assemble", "amie_set_cscale",
    "amie_element_matrices", "amie_apply_dirichlet", "amie_matrix_download", "amie_spmv", "amie_solve",
    "amie_solve_resident", "amie_solution_download", "amie_server_start", "amie_submit", "amie_poll",
    "amie_cancel", "amie_server_drain", "amie_server_stop", "amie_kernel_launches", "amie_timer_start",
    "amie_timer_stop", "amie_profile_spmv", "amie_element_fields", "amie_pcg_solve_noalloc",
    "amie_topology_spmv_lanes", "amie_profile_stream", "amie_average_field", "amie_set_imposed_strain",
    "amie_server_query", "amie_cut_rules", "amie_extrapolate", "amie_damage_setup", "amie_damage_set_state",
    "amie_damage_get_state", "amie_damage_grade", "amie_damage_update", "amie_damage_load_step",
    "amie_solution_upload", "amie_set_proportional",
]


class ServerStats(C.Structure):
    _fields_ = [("admit_s", C.c_double), ("wait_s", C.c_double), ("advance_s", C.c_double), ("join_s", C.c_double),
                ("loop_s", C.c_double), ("batches", C.c_uint64), ("admitted", C.c_uint64)]
FIELD_STRAIN, FIELD_STRESS = 0, 1
# amie_cut_rules: points per element at most, and the per-element status codes
CUT_MAX_POINTS = 52
CUT_OK, CUT_NOT_CUT, CUT_MONTE_CARLO, CUT_ORDER_DEPENDENT, CUT_TOO_MANY_HINTS, CUT_REPLACED = 0, 1, 2, 3, 4, 5
CUT_REPLACE_MONTE_CARLO = 1


DAMAGE_FIBER_ISOTROPIC = 0


class DamageLaw(C.Structure):
    """amie_damage_law: NonLocalMazars(threshold, young, poisson, fracture_energy, radius, PLANE_STRESS)
    with FiberBasedIsotropicLinearDamage(fibre_fraction, cutoff), residual stiffness fraction."""
    _fields_ = [("model", C.c_int32), ("threshold", C.c_double), ("young", C.c_double), ("poisson", C.c_double),
                ("fracture_energy", C.c_double), ("radius", C.c_double), ("score_tolerance", C.c_double),
                ("fibre_fraction", C.c_double), ("cutoff", C.c_double), ("residual", C.c_double)]


class DamageStepStats(C.Structure):
    _fields_ = [("sub_iterations", C.c_int32), ("status", C.c_int32), ("cg_iterations", C.c_int64),
                ("damaged", C.c_uint32), ("fractured", C.c_uint32), ("changes", C.c_uint64),
                ("smoothed", C.c_uint64), ("seconds", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class AmieError(RuntimeError):
    def __init__(self, status: int, where: str, detail: str = ""):
        self.status = status
        name = STATUS_NAMES[status] if 0 <= status < len(STATUS_NAMES) else str(status)
        super().__init__(f"{where}: {name} {detail}".strip())


class _Config(C.Structure):
    _fields_ = [("device", C.c_int32), ("hbm_budget_bytes", C.c_uint64), ("verbose", C.c_int32)]


class _Mesh(C.Structure):
    _fields_ = [
        ("dim", C.c_int32), ("stride", C.c_int32), ("n_elem", C.c_uint32), ("ndofmax", C.c_uint32),
        ("kind", C.c_void_p), ("dof_ptr", C.c_void_p), ("dof_ids", C.c_void_p), ("gp_ptr", C.c_void_p),
        ("gp", C.c_void_p), ("jinv", C.c_void_p), ("moved", C.c_void_p), ("jinv_gp", C.c_void_p),
        ("mat", C.c_void_p), ("cmat_table", C.c_void_p), ("n_mat", C.c_uint32), ("cscale", C.c_void_p),
        ("scale", C.c_void_p), ("enr_ptr", C.c_void_p), ("enr_type", C.c_void_p), ("enr_vertex", C.c_void_p),
        ("enr_data", C.c_void_p), ("n_enr_gp", C.c_uint64), ("enr_jump", C.c_void_p), ("enr_grad", C.c_void_p),
        ("enr_tip", C.c_void_p), ("n_enr_tip", C.c_uint32),
    ]


class SolveOpts(C.Structure):
    _fields_ = [("solver", C.c_int32), ("rtol", C.c_double), ("eps", C.c_double), ("nssor", C.c_int32),
                ("maxit", C.c_int64), ("inner_rtol", C.c_double), ("use_x0", C.c_int32)]


class SolveStats(C.Structure):
    _fields_ = [("iterations", C.c_int64), ("refinements", C.c_int32), ("status", C.c_int32),
                ("relres", C.c_double), ("seconds", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class ServerConfig(C.Structure):
    _fields_ = [("solver", C.c_int32), ("rtol", C.c_double), ("hbm_budget_bytes", C.c_uint64),
                ("max_slots", C.c_int32), ("iters_per_launch", C.c_int32), ("barrier_polls", C.c_uint32)]


class Request(C.Structure):
    _fields_ = [("mesh", C.c_void_p), ("n_bc", C.c_uint32), ("bc_ids", C.c_void_p), ("bc_values", C.c_void_p),
                ("bc_kinds", C.c_void_p), ("x0", C.c_void_p)]


class Result(C.Structure):
    _fields_ = [("status", C.c_int32), ("iterations", C.c_int64), ("relres", C.c_double),
                ("latency_s", C.c_double), ("queue_s", C.c_double), ("n", C.c_uint64)]


_lib = None


def lib():
    """Load libamie_gpu.so (build it first with build.py / __graft_entry__.build)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: run `python xfem-amie_gb300/build.py` first")
        L = C.CDLL(LIB_PATH)
        L.amie_last_error.restype = C.c_char_p
        L.amie_kernel_launches.restype = C.c_uint64
        for name in EXPORTED:
            if name not in ("amie_last_error", "amie_kernel_launches", "amie_abi_version"):
                getattr(L, name).restype = C.c_int
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def check(rc: int, where: str, ok=(AMIE_OK,)):
    if rc not in ok:
        raise AmieError(rc, where, lib().amie_last_error().decode(errors="replace"))
    return rc


def kernel_launches() -> int:
    return int(lib().amie_kernel_launches())


def mesh_struct(m: am.MeshData):
    """ctypes amie_mesh over the arrays of a MeshData (which must outlive it)."""
    s = _Mesh(m.dim, m.stride, m.n_elem, m.ndofmax)
    for name in ("kind", "dof_ptr", "dof_ids", "gp_ptr", "gp", "jinv", "moved", "jinv_gp", "mat", "cmat_table",
                 "cscale", "scale", "enr_ptr", "enr_type", "enr_vertex", "enr_data", "enr_jump", "enr_grad"):
        setattr(s, name, _p(getattr(m, name)))
    s.n_mat = len(m.cmat_table) // (m.nv * m.nv)
    s.n_enr_gp = len(m.enr_jump) if len(m.enr_jump) else (len(m.enr_grad) // m.dim)
    if len(m.enr_grad) // m.dim > s.n_enr_gp:
        s.n_enr_gp = len(m.enr_grad) // m.dim
    if m.enr_tip is not None and len(m.enr_tip):
        s.enr_tip = _p(m.enr_tip)
        s.n_enr_tip = len(m.enr_tip) // 8
    if m.enr_ptr is not None and int(m.enr_ptr[-1]) == 0:
        s.enr_ptr = None
    return s


class Context:
    def __init__(self, device: int = 0, hbm_budget_bytes: int = 0, verbose: int = 0):
        self.ptr = C.c_void_p()
        check(lib().amie_ctx_create(C.byref(_Config(device, hbm_budget_bytes, verbose)), C.byref(self.ptr)),
              "amie_ctx_create")

    def timer_start(self):
        check(lib().amie_timer_start(self.ptr), "amie_timer_start")

    def cut_rules(self, corners, line, flags=0):
        """Rules of triangles crossed by the crack polyline `line` [(x, y), ...]:
        (count [n], status [n], rule [n, CUT_MAX_POINTS, 3], h_point [n, CUT_MAX_POINTS], h_vertex [n, 3]).
        flags = CUT_REPLACE_MONTE_CARLO: deterministic rules where the reference uses Monte-Carlo."""
        c = np.ascontiguousarray(corners, np.float64).reshape(-1, 6)
        ln = np.ascontiguousarray(line, np.float64).reshape(-1, 2)
        n = c.shape[0]
        cnt = np.zeros(n, np.uint32)
        status = np.zeros(n, np.int8)
        rule = np.zeros((n, CUT_MAX_POINTS, 3), np.float64)
        hp = np.zeros((n, CUT_MAX_POINTS), np.int8)
        hv = np.zeros((n, 3), np.int8)
        check(lib().amie_cut_rules(self.ptr, C.c_uint32(n), _p(c), C.c_uint32(ln.shape[0]), _p(ln),
                                   C.c_uint32(flags), _p(cnt), _p(status), _p(rule), _p(hp), _p(hv)),
              "amie_cut_rules")
        return cnt, status, rule, hp, hv
        return cnt, rule, side

    def profile_stream(self, nbytes: int, reps: int = 10) -> float:
        """Milliseconds of one plain streaming read of `nbytes` (L2 evicted before each launch)."""
        ms = C.c_double()
        check(lib().amie_profile_stream(self.ptr, C.c_uint64(nbytes), C.c_int32(reps), C.byref(ms)),
              "amie_profile_stream")
        return ms.value

    def timer_stop(self) -> float:
        """Milliseconds of device time on the context's stream since timer_start."""
        ms = C.c_double()
        check(lib().amie_timer_stop(self.ptr, C.byref(ms)), "amie_timer_stop")
        return ms.value

    def close(self):
        if self.ptr:
            lib().amie_ctx_destroy(self.ptr)
            self.ptr = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Topology:
    """Device-resident mesh: element data, pattern, scatter map, matrix, vectors."""

    def __init__(self, ctx: Context, m: am.MeshData):
        self.ctx = ctx
        self.mesh = m
        self._ms = mesh_struct(m)
        self.ptr = C.c_void_p()
        check(lib().amie_topology_build(ctx.ptr, C.byref(self._ms), C.byref(self.ptr)), "amie_topology_build")
        nr, nz, n = C.c_uint32(), C.c_uint64(), C.c_uint64()
        lib().amie_topology_sizes(self.ptr, C.byref(nr), C.byref(nz), C.byref(n))
        self.n_rows, self.nnzb, self.n = nr.value, nz.value, n.value

    def close(self):
        if self.ptr:
            lib().amie_topology_destroy(self.ptr)
            self.ptr = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def spmv_lanes(self):
        g = C.c_int32()
        check(lib().amie_topology_spmv_lanes(self.ptr, C.byref(g)), "amie_topology_spmv_lanes")
        return g.value

    def pattern(self):
        rs = np.zeros(self.n_rows, np.uint32)
        ci = np.zeros(self.nnzb, np.uint32)
        check(lib().amie_topology_pattern(self.ptr, _p(rs), _p(ci)), "amie_topology_pattern")
        return rs, ci

    def assemble(self):
        check(lib().amie_assemble(self.ptr), "amie_assemble")

    def set_cscale(self, cscale):
        cs = np.ascontiguousarray(cscale, np.float64)
        check(lib().amie_set_cscale(self.ptr, _p(cs)), "amie_set_cscale")

    def element_matrices(self):
        off = self.mesh.ke_offsets()
        ke = np.zeros(int(off[-1]), np.float64)
        check(lib().amie_element_matrices(self.ptr, _p(ke), C.c_uint64(len(ke))), "amie_element_matrices")
        return off, ke

    def apply_dirichlet(self, ids, values, kinds=None, rhs0=None):
        ids = np.ascontiguousarray(ids, np.uint32)
        values = np.ascontiguousarray(values, np.float64)
        kinds = None if kinds is None else np.ascontiguousarray(kinds, np.uint8)
        rhs0 = None if rhs0 is None else np.ascontiguousarray(rhs0, np.float64)
        check(lib().amie_apply_dirichlet(self.ptr, C.c_uint32(len(ids)), _p(ids), _p(values), _p(kinds), _p(rhs0)),
              "amie_apply_dirichlet")

    def set_proportional(self, ids, offsets, ptr, prop_ids, coefs):
        """Proportional displacements u[ids[i]] = offsets[i] + sum coefs[k] u[prop_ids[k]],
        k in [ptr[i], ptr[i+1]) (Assembly::setPointProportional), applied after every
        elimination and to every solution; empty arrays remove them."""
        ids = np.ascontiguousarray(ids, np.uint32)
        offsets = np.ascontiguousarray(offsets, np.float64)
        ptr = np.ascontiguousarray(ptr, np.uint32)
        prop_ids = np.ascontiguousarray(prop_ids, np.uint32)
        coefs = np.ascontiguousarray(coefs, np.float64)
        check(lib().amie_set_proportional(self.ptr, C.c_uint32(len(ids)), _p(ids), _p(offsets), _p(ptr), _p(prop_ids),
                                          _p(coefs)), "amie_set_proportional")

    def matrix(self):
        """(array in AMIE's padded column-major block layout, rhs)."""
        s = self.mesh.stride
        arr = np.zeros(self.nnzb * s * (s + s % 2), np.float64)
        rhs = np.zeros(self.n, np.float64)
        check(lib().amie_matrix_download(self.ptr, _p(arr), _p(rhs)), "amie_matrix_download")
        return arr, rhs

    def spmv(self, x):
        x = np.ascontiguousarray(x, np.float64)
        y = np.zeros(self.n, np.float64)
        check(lib().amie_spmv(self.ptr, _p(x), _p(y)), "amie_spmv")
        return y

    def solve(self, solver=SOLVER_PCG_FP64, rtol=1e-10, x0=None, maxit=0, eps=1e-10, nssor=32,
              inner_rtol=0.0, accept=(AMIE_OK,)):
        x = np.zeros(self.n, np.float64) if x0 is None else np.array(x0, np.float64, copy=True)
        opts = SolveOpts(solver, rtol, eps, nssor, maxit, inner_rtol, 1 if x0 is not None else 0)
        st = SolveStats()
        rc = lib().amie_solve(self.ptr, C.byref(opts), _p(x), C.byref(st))
        check(rc, "amie_solve", ok=accept)
        return x, st.as_dict()

    def solve_resident(self, solver=SOLVER_PCG_FP64, rtol=1e-10, maxit=0, inner_rtol=0.0, use_x0=False,
                       accept=(AMIE_OK,)):
        opts = SolveOpts(solver, rtol, 1e-10, 32, maxit, inner_rtol, 1 if use_x0 else 0)
        st = SolveStats()
        rc = lib().amie_solve_resident(self.ptr, C.byref(opts), C.byref(st))
        check(rc, "amie_solve_resident", ok=accept)
        return st.as_dict()

    def extrapolate(self):
        """Device warm start 2 x - x_prev for the next resident solve (Assembly::extrapolate)."""
        check(lib().amie_extrapolate(self.ptr), "amie_extrapolate")

    def solution(self):
        x = np.zeros(self.n, np.float64)
        check(lib().amie_solution_download(self.ptr, _p(x)), "amie_solution_download")
        return x

    def element_fields(self):
        """(strain, stress) per element, Voigt, from the device solution."""
        nv = self.mesh.nv
        eps = np.zeros(self.mesh.n_elem * nv, np.float64)
        sig = np.zeros(self.mesh.n_elem * nv, np.float64)
        check(lib().amie_element_fields(self.ptr, _p(eps), _p(sig)), "amie_element_fields")
        return eps.reshape(-1, nv), sig.reshape(-1, nv)

    def set_imposed_strain(self, eps0):
        """Imposed strain per element ([n_elem, nv] Voigt, None removes it): induced forces in the RHS."""
        if eps0 is None:
            check(lib().amie_set_imposed_strain(self.ptr, None), "amie_set_imposed_strain")
            return
        e = np.ascontiguousarray(eps0, np.float64).reshape(-1)
        if e.size != self.mesh.n_elem * self.mesh.nv:
            raise ValueError("eps0 must have n_elem * nv entries")
        check(lib().amie_set_imposed_strain(self.ptr, _p(e)), "amie_set_imposed_strain")

    def average_field(self, field=FIELD_STRAIN):
        """(mesh average of the strain or stress, total area or volume) from the device solution."""
        avg = np.zeros(self.mesh.nv, np.float64)
        w = C.c_double()
        check(lib().amie_average_field(self.ptr, C.c_int32(field), _p(avg), C.byref(w)), "amie_average_field")
        return avg, w.value

    def solution_upload(self, x):
        x = np.ascontiguousarray(x, np.float64)
        check(lib().amie_solution_upload(self.ptr, _p(x)), "amie_solution_upload")

    def damage_setup(self, law: DamageLaw, corners):
        """Non-local Mazars damage of the (P1, 2D) mesh; corners [n_elem, 6] vertex coordinates."""
        cr = np.ascontiguousarray(corners, np.float64).reshape(-1)
        check(lib().amie_damage_setup(self.ptr, C.byref(law), _p(cr)), "amie_damage_setup")
        self._law = law

    def damage_set_state(self, damage=None):
        dm = None if damage is None else np.ascontiguousarray(damage, np.float64)
        check(lib().amie_damage_set_state(self.ptr, _p(dm)), "amie_damage_set_state")

    def damage_state(self):
        dm = np.zeros(self.mesh.n_elem, np.float64)
        check(lib().amie_damage_get_state(self.ptr, _p(dm)), "amie_damage_get_state")
        return dm

    def damage_grade(self, smoothed=True):
        """(score [n_elem], smoothed principal stress and strain [n_elem, 4]) from the device solution;
        with smoothed=False only the scores (bounded grading, the same scores), smoothed None."""
        sc = np.zeros(self.mesh.n_elem, np.float64)
        sm = np.zeros(self.mesh.n_elem * 4, np.float64) if smoothed else None
        check(lib().amie_damage_grade(self.ptr, _p(sc), _p(sm) if smoothed else None), "amie_damage_grade")
        return sc, (sm.reshape(-1, 4) if smoothed else None)

    def damage_update(self) -> int:
        n = C.c_uint32()
        check(lib().amie_damage_update(self.ptr, C.byref(n)), "amie_damage_update")
        return n.value

    def damage_load_step(self, solver=SOLVER_PCG_FP64, rtol=1e-10, max_sub_iterations=0, inner_rtol=0.0,
                         warm=True, accept=(AMIE_OK,)):
        """Solve-grade-update passes until no element changes (FeatureTree::stepInternal); returns stats.
        warm: the first pass starts from the current device solution (else from zero)."""
        opts = SolveOpts(solver, rtol, 1e-10, 32, 0, inner_rtol, 1 if warm else 0)
        st = DamageStepStats()
        rc = lib().amie_damage_load_step(self.ptr, C.byref(opts), C.c_int32(max_sub_iterations), C.byref(st))
        check(rc, "amie_damage_load_step", ok=accept)
        return st.as_dict()

    def profile_spmv(self, precision: int = 64, reps: int = 20) -> float:
        """Average device milliseconds of one q = A p (+ p.q) launch."""
        ms = C.c_double()
        check(lib().amie_profile_spmv(self.ptr, C.c_int32(precision), C.c_int32(reps), C.byref(ms)),
              "amie_profile_spmv")
        return ms.value


class Server:
    """Continuous-batching solve server (amie_server_* of the C-ABI)."""

    def __init__(self, ctx: Context, solver=SOLVER_PCG_MIXED, rtol=1e-10, hbm_budget_bytes=0, max_slots=0,
                 iters_per_launch=0, barrier_polls=0):
        self.ctx = ctx
        self.ptr = C.c_void_p()
        cfg = ServerConfig(solver, rtol, hbm_budget_bytes, max_slots, iters_per_launch, barrier_polls)
        check(lib().amie_server_start(ctx.ptr, C.byref(cfg), C.byref(self.ptr)), "amie_server_start")
        self._keep = {}
        self._n = {}

    def submit(self, m: am.MeshData, bc_ids, bc_values, bc_kinds=None, x0=None) -> int:
        ms = mesh_struct(m)
        ids = np.ascontiguousarray(bc_ids, np.uint32)
        vals = np.ascontiguousarray(bc_values, np.float64)
        kinds = None if bc_kinds is None else np.ascontiguousarray(bc_kinds, np.uint8)
        x0a = None if x0 is None else np.ascontiguousarray(x0, np.float64)
        req = Request(C.cast(C.pointer(ms), C.c_void_p), len(ids), _p(ids), _p(vals), _p(kinds), _p(x0a))
        t = C.c_uint64()
        check(lib().amie_submit(self.ptr, C.byref(req), C.byref(t)), "amie_submit")
        self._n[t.value] = (int(max(m.ndofmax, int(m.dof_ids.max()) + 1)) * m.stride)
        return t.value

    def stats(self) -> dict:
        """Host-loop time split since start (admission, batch waits, residual replacements, joins)."""
        st = ServerStats()
        check(lib().amie_server_query(self.ptr, C.byref(st)), "amie_server_query")
        return {k: getattr(st, k) for k, _ in ServerStats._fields_}

    def poll(self, ticket: int, want_x: bool = True):
        """None while running; else (result dict, solution or None)."""
        res = Result()
        x = np.zeros(self._n.get(ticket, 0), np.float64) if want_x else None
        rc = lib().amie_poll(self.ptr, C.c_uint64(ticket), C.byref(res), _p(x) if want_x else None)
        if rc == AMIE_NOT_READY:
            return None
        if rc not in (AMIE_OK, AMIE_CANCELLED):
            check(rc, "amie_poll")
        d = {k: getattr(res, k) for k, _ in Result._fields_}
        if x is not None and res.n:
            x = x[:res.n]
        return d, x

    def cancel(self, ticket: int):
        check(lib().amie_cancel(self.ptr, C.c_uint64(ticket)), "amie_cancel")

    def drain(self, timeout_s: float = 0.0) -> int:
        return int(lib().amie_server_drain(self.ptr, C.c_double(timeout_s)))

    def stop(self):
        if self.ptr:
            lib().amie_server_stop(self.ptr)
            self.ptr = C.c_void_p()

    def __del__(self):
        try:
            self.stop()
        except Exception:
            pass


class Assembly:
    """Mirror of AMIE's ``Assembly`` (solvers/assembly.h:228-450) on the GPU path.

    Elements arrive as a ``MeshData`` batch (``add``), Dirichlet multipliers
    through ``setPointAlong`` / ``fixPoint``, nodal forces through
    ``setForceOn``; ``cgsolve`` runs make_final (pattern, scatter, elimination)
    and the solve, and keeps the displacement history used by ``extrapolate``
    (solvers/assembly.cpp:1772-1814) as the next warm start.
    """

    XI, ETA, ZETA = 0, 1, 2

    def __init__(self, ctx: Optional[Context] = None):
        self.ctx = ctx or Context()
        self.mesh: Optional[am.MeshData] = None
        self.topo: Optional[Topology] = None
        self.multipliers = {}        # dof id -> (value, kind)
        self.proportional = {}       # dof id -> (offset, [dof ids], [coefficients])
        self._topo_has_proportional = False
        self.epsilon = 1e-10
        self.nssor = 32
        self.solver = SOLVER_PCG_FP64
        self.rtol = 1e-10
        self.ndofmax = 0
        self.displacements = np.zeros(0)
        self.history = []
        self.last_stats = {}
        self._dirty_topology = True

    # element side ------------------------------------------------------
    def add(self, mesh: am.MeshData):
        self.mesh = mesh
        self._dirty_topology = True

    def setMaxDof(self, n: int):
        self.ndofmax = n

    def setEpsilon(self, e: float):
        self.epsilon = e

    def setSSORIterations(self, n: int):
        self.nssor = n

    def setSolver(self, solver: int, rtol: float = 1e-10):
        self.solver = solver
        self.rtol = rtol

    def setCScale(self, cscale):
        """New per-element factor on C (damage step), keeps the topology."""
        self.mesh.cscale = np.ascontiguousarray(cscale, np.float64)
        if self.topo is not None:
            self.topo.set_cscale(self.mesh.cscale)

    # multipliers -------------------------------------------------------
    def setPointAlong(self, axis: int, value: float, node_id: int):
        dof = node_id * self.mesh.stride + axis
        self.proportional.pop(dof, None)   # one multiplier per DOF, the last one set
        self.multipliers[dof] = (float(value), am.BC_DISPLACEMENT)

    def setPointProportional(self, axis: int, other, value, offset: float, node_id: int):
        """Assembly::setPointProportional (solvers/assembly.cpp:1636-1761): u_axis = value u_other
        + offset at one node; `other` may instead be a list of (axis, coefficient) pairs (value
        then unused), the reference's second overload."""
        s = self.mesh.stride
        pairs = list(other) if isinstance(other, (list, tuple)) else [(other, value)]
        if len(pairs) == 1 and pairs[0][0] == axis:
            return   # v1 == v2 is ignored by the reference
        dof = node_id * s + axis
        self.multipliers.pop(dof, None)
        self.proportional[dof] = (float(offset), [node_id * s + int(a) for a, _ in pairs],
                                  [float(c) for _, c in pairs])

    def fixPoint(self, node_id: int, axis: int):
        self.setPointAlong(axis, 0.0, node_id)

    def setForceOn(self, axis: int, value: float, node_id: int):
        key = node_id * self.mesh.stride + axis
        old = self.multipliers.get(key)
        base = old[0] if old is not None and old[1] == am.BC_FORCE else 0.0   # forces on a DOF accumulate
        self.multipliers[key] = (base + float(value), am.BC_FORCE)

    def setMultipliers(self, ids, values, kinds=None):
        kinds = np.zeros(len(ids), np.uint8) if kinds is None else kinds
        for i, v, k in zip(ids, values, kinds):
            self.multipliers[int(i)] = (float(v), int(k))

    def clear(self):
        self.multipliers.clear()
        self.proportional.clear()
        self.topo = None
        self.history.clear()

    # solve -------------------------------------------------------------
    def make_final(self):
        if self.topo is None or self._dirty_topology:
            if self.ndofmax:
                self.mesh.ndofmax = self.ndofmax
            self.topo = Topology(self.ctx, self.mesh)
            self._dirty_topology = False
            self._topo_has_proportional = False
        self.topo.assemble()
        ids = np.array(sorted(self.multipliers), np.uint32)
        vals = np.array([self.multipliers[i][0] for i in ids], np.float64)
        kinds = np.array([self.multipliers[i][1] for i in ids], np.uint8)
        if self._topo_has_proportional:   # a DOF may have moved between the lists: old ones go first
            self.topo.set_proportional(np.zeros(0, np.uint32), np.zeros(0), np.zeros(1, np.uint32),
                                       np.zeros(0, np.uint32), np.zeros(0))
            self._topo_has_proportional = False
        self.topo.apply_dirichlet(ids, vals, kinds)
        if self.proportional:
            pids = sorted(self.proportional)
            ptr = np.cumsum([0] + [len(self.proportional[i][1]) for i in pids]).astype(np.uint32)
            self.topo.set_proportional(np.array(pids, np.uint32),
                                       np.array([self.proportional[i][0] for i in pids], np.float64), ptr,
                                       np.array([d for i in pids for d in self.proportional[i][1]], np.uint32),
                                       np.array([c for i in pids for c in self.proportional[i][2]], np.float64))
            self._topo_has_proportional = True

    def extrapolate(self):
        """Assembly::extrapolate (factor 1): 2 u_k - u_(k-1) from the two-entry
        history, which the reference starts as [0, u_1] after its first solve."""
        if len(self.history) < 2:
            return self.displacements if len(self.displacements) else None
        a, b = self.history[-2], np.nan_to_num(self.history[-1], nan=0.0)
        return b + (b - a)

    def _record(self, x):
        """Displacements and history after a solve (solvers/assembly.cpp:1856-1867):
        two entries, starting as [0, u_1]."""
        self.displacements = x
        self.history = [self.history[-1], x] if len(self.history) == 2 else [np.zeros_like(x), x]

    def cgsolve(self, maxit: int = -1) -> bool:
        self.make_final()
        x0 = self.extrapolate()
        if x0 is not None and len(x0) != self.topo.n:
            x0 = None
        x, st = self.topo.solve(self.solver, rtol=self.rtol, x0=x0, maxit=max(maxit, 0), eps=self.epsilon,
                                nssor=self.nssor, accept=(AMIE_OK, AMIE_NOT_CONVERGED))
        self._record(x)
        self.last_stats = st
        return st["status"] == AMIE_OK

    def getMatrix(self):
        rs, ci = self.topo.pattern()
        arr, _ = self.topo.matrix()
        return rs, ci, arr

    def getForces(self):
        return self.topo.matrix()[1]

    def getDisplacements(self):
        return self.displacements
