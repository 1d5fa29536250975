"""Test infrastructure only: ctypes access to the reference ModFEM CPU path.

``oracle/ref/Makefile`` compiles the reference's own C sources (mesh module
mmd_prism, approximation modules apd_std_lin / apd_dg_prism, the conv-diff
weak forms, sid_mkb, lsd_mkb and utd_util/uts_ls_intf.c) together with
``oracle/ref/harness.c`` into ``oracle/_ref/libmodfem_ref_{std,dg}.so``.  This
module wraps those libraries for the golden-fixture generator and for the
parity tests that run in this container.  The library keeps ModFEM's global
state, so one process can hold one mesh/field/solver per library; the fixture
generator therefore runs each case in a fresh subprocess.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")

APC_ELEMENT = 4
APC_FACE = 3
APC_VERTEX = 1


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def lib_path(kind):
    return os.path.join(REF_DIR, f"libmodfem_ref_{kind}.so")


def available(kind="std"):
    return os.path.exists(lib_path(kind))


MKB_TEMPLATE = """FINE_LEVEL       (the only level for single-level solvers)
1 1 {krylov}    single-level GMRES, number of levels, number of Krylov vectors
1 1 {block_type}  \t\ttype of preconditioner (block Jacobi), sweeps, block type (negative: -storage type)
{max_iter} {conv_type} {tol:.3e}   \tmax_iter, convergence type, convergence treshold
{monitor} 1 0   \toutput level, nr_pre and post_smooth steps

COARSE_LEVEL\t(the coarsest level solver)
1 -1 100  \tsingle/multi-level GMRES, dummy=0, number of Krylov vectors
2 1 2  \t\ttype of preconditioner,  number of internal sweeps,  block type
100 1 1e-12   \tmax_iter, convergence type, convergence treshold
0    \t\toutput level
"""


class RefModfem:
    """One reference problem: jk mesh, field, coefficients, MKB solver."""

    def __init__(self, kind="std"):
        self.kind = kind
        self.L = ctypes.CDLL(lib_path(kind))
        L = self.L
        L.refh_set_coeffs.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                      ctypes.c_double, ctypes.c_double, ctypes.c_int]
        L.refh_assemble.restype = ctypes.c_double
        L.refh_set_dg_penalty.argtypes = [ctypes.c_double]
        L.refh_solve.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_void_p,
                                 ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
        L.refh_residual.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                                    ctypes.c_void_p, ctypes.c_void_p]

    # ---------------- mesh ----------------
    def load_jk(self, path):
        mid = self.L.refh_load_jk(path.encode())
        s = [ctypes.c_int() for _ in range(6)]
        self.L.refh_mesh_sizes(*[ctypes.byref(x) for x in s])
        (self.nno, self.max_node, self.nel, self.max_el, self.nfa, self.max_fa) = [x.value for x in s]
        return mid

    def node_coords(self):
        xyz = np.zeros(3 * self.max_node)
        self.L.refh_node_coords(_p(xyz))
        return xyz.reshape(-1, 3)

    def set_node_coords(self, xyz):
        xyz = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1)
        self.L.refh_set_node_coords(_p(xyz))

    def el_nodes(self, nv=6):
        a = np.zeros(nv * self.max_el, dtype=np.int32)
        self.L.refh_el_nodes(nv, _p(a))
        return a.reshape(-1, nv)

    def bc_faces(self):
        n = self.L.refh_bc_faces(None, None, None)
        fid = np.zeros(n, np.int32)
        fbc = np.zeros(n, np.int32)
        fel = np.zeros(n, np.int32)
        self.L.refh_bc_faces(_p(fid), _p(fbc), _p(fel))
        return fid, fbc, fel

    # ---------------- field / coefficients ----------------
    def init_field(self, field_type="s", pdeg=1):
        return self.L.refh_init_field(ord(field_type), pdeg)

    def set_coeffs(self, k=None, D=None, f=1.0, g=0.0):
        nel = self.max_el
        kk = None if k is None else np.ascontiguousarray(k, dtype=np.float64)
        DD = None if D is None else np.ascontiguousarray(D, dtype=np.float64).reshape(-1)
        self._keep = (kk, DD)
        self.L.refh_set_coeffs(nel, None if kk is None else kk.ctypes.data,
                               None if DD is None else DD.ctypes.data, f, g, 0 if D is None else 1)

    def set_dg_penalty(self, p):
        self.L.refh_set_dg_penalty(p)

    def int_ent_stiff(self, ent_type, ent_id, maxn=130):
        sm = np.zeros(maxn * maxn)
        rhs = np.zeros(maxn)
        nd = ctypes.c_int()
        ne = ctypes.c_int()
        dt = np.zeros(40, np.int32)
        di = np.zeros(40, np.int32)
        dn = np.zeros(40, np.int32)
        self.L.refh_int_ent_stiff(ent_type, ent_id, _p(sm), _p(rhs), ctypes.byref(nd),
                                  ctypes.byref(ne), _p(dt), _p(di), _p(dn))
        n = nd.value
        # column-major storage: Stiff_mat[u*n + w], u = column (trial), w = row (test)
        return (sm[:n * n].reshape(n, n).T.copy(), rhs[:n].copy(), di[:ne.value].copy())

    # ---------------- solver ----------------
    def solver_create(self, mkb_path):
        sid = self.L.refh_solver_create(mkb_path.encode())
        v = [ctypes.c_int() for _ in range(8)]
        self.table_len = self.L.refh_level_sizes(*[ctypes.byref(x) for x in v])
        (self.ndof, self.nr_int_ent, self.nr_dof_ent, self.nr_colors_elems, self.nr_colors_faces,
         _, self.max_dofs_int_ent, self.nnz) = [x.value for x in v]
        return sid

    def level_lists(self):
        n = self.nr_int_ent
        out = dict(
            int_ent_type=np.zeros(n, np.int32), int_ent_id=np.zeros(n, np.int32),
            color_elems=np.zeros(self.nr_colors_elems + 1, np.int32),
            color_faces=np.zeros(self.nr_colors_faces + 1, np.int32),
            asse_pos=np.zeros(n, np.int32), assembly_table=np.zeros(self.table_len, np.int32),
            dof_ent_type=np.zeros(self.nr_dof_ent, np.int32), dof_ent_id=np.zeros(self.nr_dof_ent, np.int32),
            dof_posglob=np.zeros(self.nr_dof_ent, np.int32), dof_block_id=np.zeros(self.nr_dof_ent, np.int32))
        self.L.refh_level_lists(_p(out["int_ent_type"]), _p(out["int_ent_id"]), _p(out["color_elems"]),
                                _p(out["color_faces"]), _p(out["asse_pos"]), _p(out["assembly_table"]),
                                self.table_len, _p(out["dof_ent_type"]), _p(out["dof_ent_id"]),
                                _p(out["dof_posglob"]), _p(out["dof_block_id"]))
        return out

    def assemble(self):
        return self.L.refh_assemble()

    def crs(self):
        rp = np.zeros(self.ndof + 1, np.int32)
        ci = np.zeros(self.nnz, np.int32)
        val = np.zeros(self.nnz)
        rhs = np.zeros(self.ndof)
        self.L.refh_crs_get(_p(rp), _p(ci), _p(val), _p(rhs))
        return rp, ci, val, rhs

    def block_crs(self, matrix_id=0):
        """The block-storage (lad_block) matrix of a DG solver expanded to a
        scalar CRS over global dofs with sorted columns (harness_block.c)."""
        L = self.L
        L.refh_block_crs.argtypes = [ctypes.c_int] + [ctypes.c_void_p] * 5
        nd = ctypes.c_int()
        nnz = L.refh_block_crs(matrix_id, ctypes.addressof(nd), None, None, None, None)
        if nnz < 0:
            raise RuntimeError("no block matrix")
        rp = np.zeros(nd.value + 1, np.int32)
        ci = np.zeros(nnz, np.int32)
        val = np.zeros(nnz)
        rhs = np.zeros(nd.value)
        L.refh_block_crs(matrix_id, None, _p(rp), _p(ci), _p(val), _p(rhs))
        return rp, ci, val, rhs

    def residual(self, x, b=None, use_rhs=1):
        x = np.ascontiguousarray(x, dtype=np.float64)
        v = np.zeros(self.ndof)
        bb = np.zeros(self.ndof) if b is None else np.ascontiguousarray(b, dtype=np.float64)
        self.L.refh_residual(use_rhs, 0, self.ndof, _p(x), _p(bb) if b is not None else None, _p(v))
        return v

    def solve(self, max_iter, tol, monitor=0, stride=1):
        cap = max(self.max_node, self.max_el) + 1
        sol = np.zeros(cap * stride)
        meas = ctypes.c_double()
        times = np.zeros(2)
        nit = self.L.refh_solve(max_iter, tol, monitor, _p(sol), cap, stride, ctypes.byref(meas) and
                                ctypes.cast(ctypes.pointer(meas), ctypes.c_void_p), _p(times))
        return sol, nit, meas.value, times


def write_mkb(path, krylov=30, max_iter=1000, conv_type=0, tol=1e-8, monitor=0, block_type=-2):
    """conv_type: 0 relative to the initial residual (REL_RES_INI), 1 absolute
    (ABS_RES), 2 relative to the rhs (lsd_mkb_core/lsh_mkb_core.h:111-113).
    block_type < 0 enforces storage -block_type (lss_mkb_core.c:459-464):
    -2 CRS (one dof per block: std), -4 generic CRS (variable blocks: DG)."""
    with open(path, "w") as f:
        f.write(MKB_TEMPLATE.format(krylov=krylov, max_iter=max_iter, conv_type=conv_type,
                                    tol=tol, monitor=monitor, block_type=block_type))
