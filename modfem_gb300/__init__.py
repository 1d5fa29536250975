"""GB300-native integrate / assemble / SpMV / GMRES path for ModFEM.

The compute lives in ``libmodfem_gb300.so`` (CUDA, sm_103a) behind the C ABI
in ``include/modfem_gb300.h``.  This module is a thin ctypes binding used by
the tests, the benchmark and the serving loop; there is no CPU fallback: if
the library is missing or cannot reach a GPU, the calls raise.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libmodfem_gb300.so")

ELEMENT, FACE = 4, 3
COMP_SM, COMP_RHS, COMP_BOTH = 1, 2, 3
SCATTER_ATOMIC, SCATTER_COLOR, SCATTER_GATHER = 0, 1, 2
OPT_CACHE_TABLES = 1
OPT_STD_ARITH = 2
OPT_DG_SPMV_ARITH = 3
OPT_DG_RESIDUAL = 4
OPT_STD_SPMV_ARITH = 5
STD_FP64, STD_DWORD = 0, 1
RESIDUAL_FP64, RESIDUAL_COMPENSATED = 0, 1
DG_VOLUME_FP64, DG_VOLUME_TC, DG_VOLUME_TF32, DG_VOLUME_DWORD, DG_VOLUME_TC_DWORD = 0, 1, 2, 3, 4
DG_FACE_FP64, DG_FACE_TC, DG_FACE_DWORD, DG_FACE_TC_DWORD = 0, 1, 2, 3

# (name, restype, argtypes) of every symbol include/modfem_gb300.h declares
_vp, _ci, _cd, _cll = ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_longlong
_pi, _pd, _pll, _pvp = (ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double),
                        ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_void_p))
SIGNATURES = [
    ("gbfem_version", _ci, []),
    ("gbfem_last_error", ctypes.c_char_p, []),
    ("gbfem_create", _ci, [_pvp, _ci]),
    ("gbfem_destroy", _ci, [_vp]),
    ("gbfem_device_bytes", _cll, [_vp]),
    ("gbfem_set_option", _ci, [_vp, _ci, _cll]),
    ("gbfem_invalidate_tables", _ci, [_vp]),
    ("gbfem_table_cache_stats", _ci, [_vp, _pll, _pll]),
    ("gbfem_set_mesh", _ci, [_vp, _ci, _vp, _ci, _ci, _vp, _ci, _vp, _vp, _vp, _vp]),
    ("gbfem_set_mesh_mixed", _ci, [_vp, _ci, _vp, _ci, _vp, _vp]),
    ("gbfem_set_node_coords", _ci, [_vp, _vp]),
    ("gbfem_set_coefficients", _ci, [_vp, _vp, _vp, _cd, _cd, _cd]),
    ("gbfem_set_constraints", _ci, [_vp, _ci, _vp, _vp, _vp]),
    ("gbfem_set_crs_structure", _ci, [_vp, _ci, _vp, _cll, _vp, _vp]),
    ("gbfem_build_structure", _ci, [_vp, _pi, _pll, _pi]),
    ("gbfem_build_structure_device", _ci, [_vp, _pi, _pll]),
    ("gbfem_get_crs_structure", _ci, [_vp, _vp, _vp, _vp]),
    ("gbfem_get_element_tables", _ci, [_vp, _vp]),
    ("gbfem_create_assemble_stiff_mat", _ci,
     [_vp, _ci, _ci, _pi, _ci, _vp, _vp, _ci, _vp, _ci, _vp, _vp, _vp, _ci, _vp, _vp]),
    ("gbfem_assemble", _ci, [_vp, _ci]),
    ("gbfem_get_matrix", _ci, [_vp, _vp, _vp]),
    ("gbfem_set_matrix", _ci, [_vp, _vp, _vp]),
    ("gbfem_dg_set_degrees", _ci, [_vp, _vp]),
    ("gbfem_dg_set_faces", _ci, [_vp, _ci, _vp, _vp, _vp, _vp, _vp]),
    ("gbfem_dg_set_penalty", _ci, [_vp, _cd]),
    ("gbfem_dg_set_volume_kernel", _ci, [_vp, _ci]),
    ("gbfem_dg_set_face_kernel", _ci, [_vp, _ci]),
    ("gbfem_dg_build_structure", _ci, [_vp, _pi, _pll]),
    ("gbfem_dg_get_structure", _ci, [_vp, _vp, _vp, _vp, _vp]),
    ("gbfem_dg_assemble", _ci, [_vp]),
    ("gbfem_dg_last_timing", _ci, [_vp, _pd, _pd, _pd, _pi]),
    ("gbfem_dg_autotune", _ci, [_vp, _ci, _vp, _vp, _vp]),
    ("gbfem_dg_set_variants", _ci, [_vp, _vp, _vp]),
    ("gbfem_dg_get_matrix", _ci, [_vp, _vp, _vp]),
    ("gbfem_dg_set_matrix", _ci, [_vp, _vp, _vp]),
    ("gbfem_dg_compute_residual", _ci, [_vp, _ci, _ci, _ci, _vp, _vp, _vp]),
    ("gbfem_dg_solve", _ci, [_vp, _ci, _ci, _cd, _ci, _vp, _pd, _pd]),
    ("gbfem_dg_solve_ir", _ci, [_vp, _ci, _ci, _cd, _cd, _vp, _pi, _pd]),
    ("gbfem_compute_residual", _ci, [_vp, _ci, _ci, _ci, _vp, _vp, _vp]),
    ("gbfem_compute_residual_noalloc", _ci, [_vp, _ci, _ci, _ci, _vp, _vp, _vp]),
    ("gbfem_solve", _ci, [_vp, _ci, _ci, _cd, _ci, _vp, _pd, _pd]),
    ("gbfem_last_assembly_timing", _ci, [_vp, _pd, _pd, _pi]),
    ("gbfem_last_solve_timing", _ci, [_vp, _pd, _pd, _pi, _pi]),
    ("gbfem_host_alloc", _vp, [_cll]),
    ("gbfem_host_free", _ci, [_vp]),
    ("gbfem_measure_fp64_peak", _ci, [_vp, _pd]),
    ("gbfem_read_jk", _ci, [ctypes.c_char_p, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    ("gbfem_write_field_std", _ci, [ctypes.c_char_p, _ci, _vp, _vp]),
    ("gbfem_write_field_dg", _ci, [ctypes.c_char_p, _ci, _vp, _vp, _vp, _ci]),
    ("gbfem_batch_create", _ci, [_pvp, _ci]),
    ("gbfem_batch_destroy", _ci, [_vp]),
    ("gbfem_batch_set", _ci, [_vp, _ci, _vp, _vp, _vp, _ci, _vp, _vp, _vp, _cd, _pll, _pll]),
    ("gbfem_batch_set_layout", _ci, [_vp, _vp, _vp, _cll, _cll]),
    ("gbfem_batch_set_variants", _ci, [_vp, _vp, _vp]),
    ("gbfem_batch_set_arith", _ci, [_vp, _ci]),
    ("gbfem_batch_autotune", _ci, [_vp, _ci, _vp, _vp, _vp]),
    ("gbfem_batch_run", _ci, [_vp, _pd]),
    ("gbfem_batch_get", _ci, [_vp, _vp, _vp]),
    ("gbfem_server_create", _ci, [_pvp, _ci, _cll, _ci, _ci]),
    ("gbfem_server_destroy", _ci, [_vp]),
    ("gbfem_server_submit", _cll, [_vp, _vp]),
    ("gbfem_server_wait", _ci, [_vp, _cll, _cd]),
    ("gbfem_server_result", _ci, [_vp, _cll, _vp, _cll, _pi, _pd, _vp]),
    ("gbfem_server_release", _ci, [_vp, _cll]),
    ("gbfem_server_cancel", _ci, [_vp, _cll]),
    ("gbfem_server_set_option", _ci, [_vp, _ci, _cll]),
    ("gbfem_server_stats", _ci, [_vp, _vp]),
    ("gbfem_serve_footprint", _cll, [_vp]),
]

_LIB = None


class GbFemError(RuntimeError):
    pass


def load_library(path=LIB_PATH):
    """Loads libmodfem_gb300.so and binds every declared entry point."""
    global _LIB
    if _LIB is not None and path == LIB_PATH:
        return _LIB
    if not os.path.exists(path):
        raise GbFemError(f"{path} is missing: build it with modfem_gb300.build.build()")
    lib = ctypes.CDLL(path)
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path == LIB_PATH:
        _LIB = lib
    return lib


def _p(a):
    return None if a is None else ctypes.c_void_p(a.ctypes.data)


def _i32(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.int32)


def _f64(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.float64)


class Context:
    """One problem on one GPU (see include/modfem_gb300.h)."""

    def __init__(self, device=0):
        self.L = load_library()
        self._h = ctypes.c_void_p()
        self._check(self.L.gbfem_create(ctypes.byref(self._h), device))
        self._keep = {}

    def _check(self, rc):
        if rc < 0:
            raise GbFemError(self.L.gbfem_last_error().decode())
        return rc

    def close(self):
        if self._h:
            self.L.gbfem_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def device_bytes(self):
        return self.L.gbfem_device_bytes(self._h)

    def set_option(self, opt, value):
        self._check(self.L.gbfem_set_option(self._h, opt, value))

    def invalidate_tables(self):
        """gbfem_invalidate_tables: the next drop-in call uploads its lists and table again."""
        self._check(self.L.gbfem_invalidate_tables(self._h))

    def table_cache_stats(self):
        """(generation, uploads) of the drop-in table cache."""
        g, u = ctypes.c_longlong(), ctypes.c_longlong()
        self._check(self.L.gbfem_table_cache_stats(self._h, ctypes.byref(g), ctypes.byref(u)))
        return g.value, u.value

    # ---------------- problem data ----------------
    def set_mesh(self, mesh):
        xyz = _f64(mesh.coords)
        el = _i32(mesh.el_nodes)
        nv = el.shape[1]
        fid = _i32(getattr(mesh, "bc_face_id", np.zeros(0)))
        fel = _i32(getattr(mesh, "bc_face_el", np.zeros(0)))
        fsd = _i32(getattr(mesh, "bc_face_side", np.zeros(0)))
        fbc = _i32(getattr(mesh, "bc_face_bc", np.zeros(0)))
        self._check(self.L.gbfem_set_mesh(self._h, xyz.shape[0], _p(xyz), el.shape[0], nv, _p(el), fel.size,
                                          _p(fid), _p(fel), _p(fsd), _p(fbc)))
        self.nno, self.nel, self.nv, self.nfa = xyz.shape[0], el.shape[0], nv, fel.size

    def set_mesh_mixed(self, mesh):
        """gbfem_set_mesh_mixed: a mesh of prisms and tetrahedra together (DG
        only); mesh.el_nodes has 6 slots per element, mesh.el_nv the vertex
        count (modfem_gb300.mesh.structured_mixed_mesh)."""
        xyz = _f64(mesh.coords)
        el = _i32(mesh.el_nodes)
        nv = _i32(mesh.el_nv)
        self._check(self.L.gbfem_set_mesh_mixed(self._h, xyz.shape[0], _p(xyz), el.shape[0], _p(nv), _p(el)))
        self.nno, self.nel, self.nv, self.nfa = xyz.shape[0], el.shape[0], 6, 0

    def set_node_coords(self, xyz):
        xyz = _f64(xyz)
        self._keep["xyz"] = xyz
        self._check(self.L.gbfem_set_node_coords(self._h, _p(xyz)))

    def set_coefficients(self, k=None, D=None, f=1.0, g=0.0, penalty=1.0e7):
        k = _f64(k)
        D = _f64(D)
        self._keep["k"], self._keep["D"] = k, D
        self._check(self.L.gbfem_set_coefficients(self._h, _p(k), _p(D), f, g, penalty))

    def set_constraints(self, vertex, nr_constr, constr_id):
        """gbfem_set_constraints: constrained (hanging) vertices with their 2
        or 4 constraining vertices (constr_id: 4 per vertex, -1 padded)."""
        v, n = _i32(vertex), _i32(nr_constr)
        p = _i32(np.asarray(constr_id).reshape(-1, 4)) if len(v) else np.zeros((0, 4), np.int32)
        self._check(self.L.gbfem_set_constraints(self._h, v.size, _p(v), _p(n), _p(p)))

    def set_crs_structure(self, dof_of_node, row_ptr, col_ind):
        dn, rp, ci = _i32(dof_of_node), _i32(row_ptr), _i32(col_ind)
        self._check(self.L.gbfem_set_crs_structure(self._h, rp.size - 1, _p(dn), ci.size, _p(rp), _p(ci)))
        self.ndof, self.nnz = rp.size - 1, ci.size

    def build_structure(self):
        nd, nnz, nc = ctypes.c_int(), ctypes.c_longlong(), ctypes.c_int()
        self._check(self.L.gbfem_build_structure(self._h, ctypes.byref(nd), ctypes.byref(nnz), ctypes.byref(nc)))
        self.ndof, self.nnz = nd.value, nnz.value
        return nd.value, nnz.value, nc.value

    def build_structure_device(self):
        """gbfem_build_structure_device: the same arrays built by kernels (no colouring)."""
        nd, nnz = ctypes.c_int(), ctypes.c_longlong()
        self._check(self.L.gbfem_build_structure_device(self._h, ctypes.byref(nd), ctypes.byref(nnz)))
        self.ndof, self.nnz = nd.value, nnz.value
        return nd.value, nnz.value

    def get_crs_structure(self):
        dn = np.zeros(self.nno, np.int32)
        rp = np.zeros(self.ndof + 1, np.int32)
        ci = np.zeros(self.nnz, np.int32)
        self._check(self.L.gbfem_get_crs_structure(self._h, _p(dn), _p(rp), _p(ci)))
        return dn, rp, ci

    def get_element_tables(self):
        t = np.zeros(self.nel * (self.nv * self.nv + self.nv), np.int32)
        self._check(self.L.gbfem_get_element_tables(self._h, _p(t)))
        return t

    # ---------------- hot path ----------------
    def create_assemble_stiff_mat(self, int_ent_type, int_ent_id, color_elems, color_faces, asse_pos,
                                  assembly_table, comp_type=COMP_BOTH, crs_val=None, rhs=None, level_id=0,
                                  max_dofs=None):
        """ModFEM pdr_create_assemble_stiff_mat through the C ABI (host arrays)."""
        t, i = _i32(int_ent_type), _i32(int_ent_id)
        ce, cf = _i32(color_elems), _i32(color_faces)
        ap, at = _i32(asse_pos), _i32(assembly_table)
        self._keep["dropin"] = (t, i, ce, cf, ap, at)
        pdeg = ctypes.c_int(-10)
        self._check(self.L.gbfem_create_assemble_stiff_mat(
            self._h, level_id, comp_type, ctypes.byref(pdeg), i.size, _p(t), _p(i),
            0 if ce is None else ce.size - 1, _p(ce), 0 if cf is None else cf.size - 1, _p(cf), _p(ap), _p(at),
            self.nv if max_dofs is None else max_dofs, _p(crs_val), _p(rhs)))

    # ---------------- DG prisms ----------------
    def dg_set_degrees(self, p_el):
        p = _i32(p_el)
        self._keep["dgp"] = p
        self._check(self.L.gbfem_dg_set_degrees(self._h, _p(p)))

    def dg_set_faces(self, faces, penalty=None):
        """faces: a FaceTable (modfem_gb300.mesh.prism_faces) or any object with
        type, bc, el1, el2, side1 and nodes (n x 4) arrays."""
        t = _i32(faces.type)
        bc = _i32(faces.bc)
        el = _i32(np.stack([faces.el1, faces.el2], axis=1))
        sd = _i32(faces.side1)
        nd = _i32(faces.nodes)
        self._keep["dgfaces"] = (t, bc, el, sd, nd)
        self._check(self.L.gbfem_dg_set_faces(self._h, t.size, _p(t), _p(bc), _p(el), _p(sd), _p(nd)))
        if penalty is not None:
            self._check(self.L.gbfem_dg_set_penalty(self._h, float(penalty)))

    def dg_set_volume_kernel(self, mode):
        """DG_VOLUME_FP64, DG_VOLUME_TC (tensor cores, split BF16, FP64-equivalent)
        or DG_VOLUME_TF32 (tensor cores, TF32 hi/lo, FP32 accumulation)."""
        self._check(self.L.gbfem_dg_set_volume_kernel(self._h, mode))

    def dg_set_face_kernel(self, mode):
        """DG_FACE_FP64, DG_FACE_TC (tensor cores, split BF16, FP64-equivalent), DG_FACE_DWORD (double-word
        sums on the FP32 pipes) or DG_FACE_TC_DWORD (tensor cores where they apply, double word elsewhere)."""
        self._check(self.L.gbfem_dg_set_face_kernel(self._h, mode))

    def dg_build_structure(self):
        nd, nv = ctypes.c_int(), ctypes.c_longlong()
        self._check(self.L.gbfem_dg_build_structure(self._h, ctypes.byref(nd), ctypes.byref(nv)))
        self.dg_ndof, self.dg_nval = nd.value, nv.value
        return nd.value, nv.value

    def dg_get_structure(self):
        nblk = self._check(self.L.gbfem_dg_get_structure(self._h, None, None, None, None))
        off = np.zeros(self.nel + 1, np.int32)
        bptr = np.zeros(self.nel + 1, np.int32)
        bcol = np.zeros(nblk, np.int32)
        boff = np.zeros(nblk + 1, np.int64)
        self._check(self.L.gbfem_dg_get_structure(self._h, _p(off), _p(bptr), _p(bcol), _p(boff)))
        return off, bptr, bcol, boff

    def dg_assemble(self):
        self._check(self.L.gbfem_dg_assemble(self._h))

    def dg_get_matrix(self):
        vals = np.zeros(self.dg_nval)
        rhs = np.zeros(self.dg_ndof)
        self._check(self.L.gbfem_dg_get_matrix(self._h, _p(vals), _p(rhs)))
        return vals, rhs

    def dg_set_matrix(self, vals=None, rhs=None):
        self._check(self.L.gbfem_dg_set_matrix(self._h, _p(_f64(vals)), _p(_f64(rhs))))

    def dg_autotune(self, sample=16384):
        """Chooses the fastest launch shapes per degree; returns (vol[5], face[5], ms[4, 5])."""
        vol = np.zeros(5, np.int32)
        face = np.zeros(5, np.int32)
        ms = np.zeros(20)
        self._check(self.L.gbfem_dg_autotune(self._h, sample, _p(vol), _p(face), _p(ms)))
        return vol, face, ms.reshape(4, 5)

    def dg_set_variants(self, vol=None, face=None):
        self._check(self.L.gbfem_dg_set_variants(self._h, _p(_i32(vol)), _p(_i32(face))))

    def dg_last_timing(self):
        """(total ms, volume-kernel ms, face-kernel ms, launches) of the last DG assembly."""
        t, v, f, n = ctypes.c_double(), ctypes.c_double(), ctypes.c_double(), ctypes.c_int()
        self._check(self.L.gbfem_dg_last_timing(self._h, ctypes.byref(t), ctypes.byref(v), ctypes.byref(f),
                                                ctypes.byref(n)))
        return t.value, v.value, f.value, n.value

    def dg_compute_residual(self, x, b=None, use_rhs=1, ini_zero=0):
        x = _f64(x)
        b = _f64(b)
        v = np.zeros(self.dg_ndof)
        self._check(self.L.gbfem_dg_compute_residual(self._h, use_rhs, ini_zero, self.dg_ndof, _p(x), _p(b),
                                                     _p(v)))
        return v

    def dg_solve_ir(self, krylov=50, max_iter=100000, tol_rel=1e-10, inner_tol=1e-4):
        """Mixed precision: FP64 refinement around FP32-operator GMRES.
        Returns (x, inner iterations, refinement steps, relative true residual)."""
        x = np.zeros(self.dg_ndof)
        k, rel = ctypes.c_int(), ctypes.c_double()
        it = self._check(self.L.gbfem_dg_solve_ir(self._h, krylov, max_iter, tol_rel, inner_tol, _p(x),
                                                  ctypes.byref(k), ctypes.byref(rel)))
        return x, it, k.value, rel.value

    def dg_solve(self, krylov=50, max_iter=1000, tol_rel=1e-8, x0=None):
        x = np.zeros(self.dg_ndof) if x0 is None else np.array(x0, dtype=np.float64)
        res, rel = ctypes.c_double(), ctypes.c_double()
        it = self._check(self.L.gbfem_dg_solve(self._h, krylov, max_iter, tol_rel, 1 if x0 is None else 0, _p(x),
                                               ctypes.byref(res), ctypes.byref(rel)))
        return x, it, res.value, rel.value

    def assemble(self, mode=SCATTER_ATOMIC):
        self._check(self.L.gbfem_assemble(self._h, mode))

    def get_matrix(self, val=None, rhs=None):
        val = np.zeros(self.nnz) if val is None else val
        rhs = np.zeros(self.ndof) if rhs is None else rhs
        self._check(self.L.gbfem_get_matrix(self._h, _p(val), _p(rhs)))
        return val, rhs

    def set_matrix(self, val=None, rhs=None):
        self._check(self.L.gbfem_set_matrix(self._h, _p(_f64(val)), _p(_f64(rhs))))

    def compute_residual(self, x, b=None, use_rhs=1, ini_zero=0):
        x = _f64(x)
        b = _f64(b)
        v = np.zeros(self.ndof)
        self._check(self.L.gbfem_compute_residual(self._h, use_rhs, ini_zero, self.ndof, _p(x), _p(b), _p(v)))
        return v

    def compute_residual_noalloc(self, x, b=None, use_rhs=1, ini_zero=0):
        """gbfem_compute_residual_noalloc: same result, no device allocation."""
        x = _f64(x)
        b = _f64(b)
        v = np.zeros(self.ndof)
        self._check(self.L.gbfem_compute_residual_noalloc(self._h, use_rhs, ini_zero, self.ndof, _p(x), _p(b),
                                                          _p(v)))
        return v

    def solve(self, krylov=30, max_iter=1000, tol_rel=1e-8, x0=None):
        x = np.zeros(self.ndof) if x0 is None else np.array(x0, dtype=np.float64)
        res, rel = ctypes.c_double(), ctypes.c_double()
        it = self._check(self.L.gbfem_solve(self._h, krylov, max_iter, tol_rel, 1 if x0 is None else 0, _p(x),
                                            ctypes.byref(res), ctypes.byref(rel)))
        return x, it, res.value, rel.value

    def last_timing(self):
        """(total ms, element-kernel ms, kernel launches) of the last assembly call."""
        ms, el, nl = ctypes.c_double(), ctypes.c_double(), ctypes.c_int()
        self._check(self.L.gbfem_last_assembly_timing(self._h, ctypes.byref(ms), ctypes.byref(el),
                                                      ctypes.byref(nl)))
        return ms.value, el.value, nl.value

    def last_solve_timing(self):
        """(total ms, SpMV ms, SpMV count, kernel launches) of the last solve."""
        t, sp, n, k = ctypes.c_double(), ctypes.c_double(), ctypes.c_int(), ctypes.c_int()
        self._check(self.L.gbfem_last_solve_timing(self._h, ctypes.byref(t), ctypes.byref(sp), ctypes.byref(n),
                                                   ctypes.byref(k)))
        return t.value, sp.value, n.value, k.value

    def measure_fp64_peak(self):
        v = ctypes.c_double()
        self._check(self.L.gbfem_measure_fp64_peak(self._h, ctypes.byref(v)))
        return v.value


PRISM_NS = {1: 6, 2: 18, 3: 40, 4: 75}
TET_NS = {1: 4, 2: 10, 3: 20, 4: 35}


class Batch:
    """Batched DG volume integrals of mixed prisms and tetrahedra of degrees
    1..4 in one persistent launch (gbfem_batch_*)."""

    def __init__(self, device=0):
        self.L = load_library()
        self._h = ctypes.c_void_p()
        self._check(self.L.gbfem_batch_create(ctypes.byref(self._h), device))

    def _check(self, rc):
        if rc < 0:
            raise GbFemError(self.L.gbfem_last_error().decode())
        return rc

    def set(self, prism_xyz, prism_A, prism_p, tet_xyz, tet_A, tet_p, f=1.0):
        """prism_xyz (np, 6, 3), prism_A (np, 3, 3), prism_p (np,); tets
        likewise with (nt, 4, 3).  Returns (nval, nrhs) of the default
        layout (prism blocks, then tetrahedron blocks)."""
        self._in = [_f64(prism_xyz), _f64(prism_A), _i32(prism_p), _f64(tet_xyz), _f64(tet_A), _i32(tet_p)]
        self.pp, self.tp = self._in[2].ravel(), self._in[5].ravel()
        nv, nr = ctypes.c_longlong(), ctypes.c_longlong()
        self._check(self.L.gbfem_batch_set(self._h, self.pp.size, _p(self._in[0]), _p(self._in[1]), _p(self._in[2]),
                                           self.tp.size, _p(self._in[3]), _p(self._in[4]), _p(self._in[5]), f,
                                           ctypes.byref(nv), ctypes.byref(nr)))
        self.nval, self.nrhs = nv.value, nr.value
        self.layout = None
        return self.nval, self.nrhs

    def set_layout(self, val_off, rhs_off, nval, nrhs):
        """Write element e's block at val_off[e] and load vector at rhs_off[e]."""
        vo = np.ascontiguousarray(val_off, dtype=np.int64)
        ro = _i32(rhs_off)
        self._check(self.L.gbfem_batch_set_layout(self._h, _p(vo), _p(ro), nval, nrhs))
        self.nval, self.nrhs, self.layout = nval, nrhs, (vo, ro)

    def set_arith(self, dword):
        """Prism stiffness sums in FP64 (False) or double-word arithmetic (True)."""
        self._check(self.L.gbfem_batch_set_arith(self._h, 1 if dword else 0))

    def set_variants(self, prism=None, tet=None):
        """Variants per degree, dicts or length-5 sequences indexed by p."""
        def arr(v):
            if v is None:
                return None
            a = np.zeros(5, np.int32)
            for p in range(1, 5):
                a[p] = v[p]
            return a
        pv, tv = arr(prism), arr(tet)
        self._check(self.L.gbfem_batch_set_variants(self._h, _p(pv), _p(tv)))

    def autotune(self, sample=0):
        """Returns (prism variants[5], tet variants[5], ms[2, 5, 5])."""
        pv, tv, ms = np.zeros(5, np.int32), np.zeros(5, np.int32), np.zeros(50)
        self._check(self.L.gbfem_batch_autotune(self._h, sample, _p(pv), _p(tv), _p(ms)))
        return pv, tv, ms.reshape(2, 5, 5)

    def run(self):
        """Runs the batch; returns the device time in ms."""
        ms = ctypes.c_double()
        self._check(self.L.gbfem_batch_run(self._h, ctypes.byref(ms)))
        return ms.value

    def get(self):
        """(vals, rhs) flat, blocks in input order: prisms, then tetrahedra."""
        vals, rhs = np.empty(self.nval), np.empty(self.nrhs)
        self._check(self.L.gbfem_batch_get(self._h, _p(vals), _p(rhs)))
        return vals, rhs

    def blocks(self):
        """Lists of (ns, ns) element matrices and (ns,) load vectors."""
        vals, rhs = self.get()
        mats, loads, v, r = [], [], 0, 0
        nss = [PRISM_NS[int(p)] for p in self.pp] + [TET_NS[int(p)] for p in self.tp]
        for e, ns in enumerate(nss):
            if self.layout is not None:
                v, r = int(self.layout[0][e]), int(self.layout[1][e])
            mats.append(vals[v:v + ns * ns].reshape(ns, ns).T)
            loads.append(rhs[r:r + ns])
            v += ns * ns
            r += ns
        return mats, loads

    def close(self):
        if self._h:
            self.L.gbfem_batch_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class PinnedArray:
    """numpy view of page-locked host memory from gbfem_host_alloc."""

    def __init__(self, shape, dtype=np.float64):
        self.L = load_library()
        dtype = np.dtype(dtype)
        nbytes = int(np.prod(shape)) * dtype.itemsize
        self.ptr = self.L.gbfem_host_alloc(max(nbytes, 8))
        if not self.ptr:
            raise GbFemError(self.L.gbfem_last_error().decode())
        buf = (ctypes.c_char * max(nbytes, 8)).from_address(self.ptr)
        self.array = np.frombuffer(buf, dtype=dtype, count=int(np.prod(shape))).reshape(shape)

    def free(self):
        if self.ptr:
            self.array = None
            self.L.gbfem_host_free(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass
