"""ModFEM file formats through the library: jk prism meshes in, field dumps
out (gbfem_read_jk, gbfem_write_field_std / _dg)."""
import ctypes

import numpy as np

from . import GbFemError, load_library
from .mesh import FaceTable, PrismMesh


def _p(a):
    return None if a is None else ctypes.c_void_p(a.ctypes.data)


def _check(L, r):
    if r < 0:
        raise GbFemError(L.gbfem_last_error().decode())
    return r


def read_jk(path):
    """(PrismMesh, FaceTable) of a jk file, numbered as the reference's
    mmr_import_mesh_grad numbers it; the boundary faces with a Dirichlet
    flag (0 < bc < 10) are the mesh's bc_face_* lists."""
    L = load_library()
    sizes = np.zeros(3, np.int32)
    _check(L, L.gbfem_read_jk(path.encode(), _p(sizes), None, None, None, None, None, None, None))
    nno, nel, nfa = (int(v) for v in sizes)
    xyz = np.zeros((nno, 3))
    el = np.zeros((nel, 6), np.int32)
    ft, fb, fs = (np.zeros(nfa, np.int32) for _ in range(3))
    fe = np.zeros((nfa, 2), np.int32)
    fn = np.zeros((nfa, 4), np.int32)
    _check(L, L.gbfem_read_jk(path.encode(), _p(sizes), _p(xyz), _p(el), _p(ft), _p(fb), _p(fe), _p(fs), _p(fn)))
    F = FaceTable(id=np.arange(1, nfa + 1, dtype=np.int32), type=ft, bc=fb, el1=fe[:, 0].copy(),
                  el2=fe[:, 1].copy(), side1=fs, side2=np.zeros(nfa, np.int32), nodes=fn)
    bnd = (F.el2 < 0) & (F.bc > 0) & (F.bc < 10)
    m = PrismMesh(n=None, coords=xyz, el_nodes=el, bc_face_id=F.id[bnd], bc_face_el=F.el1[bnd],
                  bc_face_side=F.side1[bnd], bc_face_bc=F.bc[bnd], ntri=None, nlay=None)
    return m, F


def write_field_std(path, dof_of_node, x):
    L = load_library()
    dn = np.ascontiguousarray(dof_of_node, dtype=np.int32)
    xx = np.ascontiguousarray(x, dtype=np.float64)
    return _check(L, L.gbfem_write_field_std(path.encode(), dn.size, _p(dn), _p(xx)))


def write_field_dg(path, p_el, dof_off, x, uniform=None):
    """uniform: one degree line (the reference's form for a field created
    with one degree); default: when every element has the same degree."""
    L = load_library()
    pe = np.ascontiguousarray(p_el, dtype=np.int32)
    off = np.ascontiguousarray(dof_off, dtype=np.int32)
    xx = np.ascontiguousarray(x, dtype=np.float64)
    if uniform is None:
        uniform = bool(np.all(pe == pe[0]))
    return _check(L, L.gbfem_write_field_dg(path.encode(), pe.size, _p(pe), _p(off), _p(xx), int(uniform)))
