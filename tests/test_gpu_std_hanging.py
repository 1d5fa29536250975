"""GPU parity of the drop-in on a refined mesh with hanging vertices
(gbfem_set_constraints + gbfem_create_assemble_stiff_mat): the reference's
own refinement, entity lists, tables and assembled system
(tests/golden/std_n9_hang.npz), the oracle for the anisotropic and
double-word variants, GMRES against the reference's, and the refusals."""
import numpy as np
import pytest

import oracle as O
from _util import REL_TOL, RefinedMesh, crs_rel_err, load, vec_rel_err

pytestmark = pytest.mark.gpu

LISTS = ("int_ent_type", "int_ent_id", "color_elems", "color_faces", "asse_pos", "assembly_table")


@pytest.fixture(scope="module")
def gb():
    from modfem_gb300 import build
    build.build(verbose=False)
    import modfem_gb300
    return modfem_gb300


@pytest.fixture(scope="module")
def case():
    g = load("std_n9_hang")
    m = RefinedMesh(g)
    args = (m.coords, m.el_nodes, g["k"], g["int_ent_type"], g["int_ent_id"], g["asse_pos"], g["assembly_table"],
            g["row_ptr"].size - 1, g["col_ind"].size, m.fa_of_id)
    kw = dict(con_cnt=g["con_cnt"], con_par=g["con_par"])
    sv, sr = O.std_dropin_assemble(*args, absolute=True, **kw)
    return g, m, args, kw, sv, sr


def _ctx(gb, g, m, D=None):
    c = gb.Context(0)
    c.set_mesh(m)
    if D is None:
        c.set_coefficients(k=g["k"], f=1.0, g=0.0, penalty=1e7)
    else:
        c.set_coefficients(D=D, f=1.0, g=0.0, penalty=1e7)
    c.set_constraints(m.con_vertex, m.con_nr, m.con_par)
    c.set_crs_structure(g["dof_of_node"], g["row_ptr"], g["col_ind"])
    return c


def _err(val, ref, scale):
    return float(np.max(np.abs(val - ref) / np.where(scale > 0, scale, 1.0)))


def _assemble(c, g):
    val = np.zeros(g["col_ind"].size)
    rhs = np.zeros(g["row_ptr"].size - 1)
    c.create_assemble_stiff_mat(*[g[k] for k in LISTS], crs_val=val, rhs=rhs, max_dofs=int(g["max_dofs_int_ent"]))
    return val, rhs


@pytest.mark.parametrize("cache", [0, 1])
def test_dropin_on_refined_mesh_matches_reference(gb, case, cache):
    """The reference's sir_create lists and n x n + n tables of a mesh with
    63 mid-edge and 17 mid-face hanging vertices; the assembled CRS values
    and rhs against the reference's, each entry within 1e-12 of the sum of
    the magnitudes of its contributions (twice: the second call clears)."""
    g, m, args, kw, sv, sr = case
    c = _ctx(gb, g, m)
    c.set_option(gb.OPT_CACHE_TABLES, cache)
    for _ in range(2):
        val, rhs = _assemble(c, g)
        assert _err(val, g["crs_val"], sv) < REL_TOL
        assert _err(rhs, g["crs_rhs"], sr) < REL_TOL
    _, _, launches = c.last_timing()
    assert launches == 4  # plain faces, plain elements, constrained elements, constrained faces
    c.close()


def test_dropin_refined_double_word_and_anisotropic(gb, case):
    """Plain elements in double-word arithmetic (the entities with hanging
    vertices stay FP64) against the reference; a full coefficient tensor
    against the oracle's rewrite of the anisotropic element."""
    from modfem_gb300.mesh import anisotropic_tensors
    g, m, args, kw, sv, sr = case
    c = _ctx(gb, g, m)
    c.set_option(gb.OPT_STD_ARITH, gb.STD_DWORD)
    val, rhs = _assemble(c, g)
    assert _err(val, g["crs_val"], sv) < REL_TOL
    assert _err(rhs, g["crs_rhs"], sr) < REL_TOL
    c.close()
    D = anisotropic_tensors(m.nel, seed=4).reshape(-1, 9)
    c = _ctx(gb, g, m, D=D)
    val, rhs = _assemble(c, g)
    Dm = D.reshape(-1, 3, 3)
    ref, rref = O.std_dropin_assemble(*args, D_el=Dm, **kw)
    sva, sra = O.std_dropin_assemble(*args, D_el=Dm, absolute=True, **kw)
    assert _err(val, ref, sva) < REL_TOL
    assert _err(rhs, rref, sra) < REL_TOL
    c.close()


def test_gmres_on_refined_mesh_vs_reference(gb, case):
    """gbfem_solve on the assembled constrained system: the reference's
    iteration count (GMRES(30), point Jacobi, 1e-8) and its solution."""
    g, m, *_ = case
    c = _ctx(gb, g, m)
    _assemble(c, g)
    x, it, res, rel = c.solve(30, 5000, 1e-8)
    assert abs(it - int(g["gmres_iters"])) <= 1
    assert rel < 1e-8
    assert vec_rel_err(x, g["gmres_x"]) < 1e-5
    c.close()


def test_constraint_refusals(gb, case):
    """Bad constraint data, a hanging vertex nobody named, a constrained
    vertex with a dof, and the library's own structure builds on a mesh with
    constraints are refused with an error."""
    g, m, *_ = case
    c = gb.Context(0)
    c.set_mesh(m)
    c.set_coefficients(k=g["k"], f=1.0, g=0.0, penalty=1e7)
    bad_nr = m.con_nr.copy()
    bad_nr[0] = 3
    with pytest.raises(gb.GbFemError, match="2 \\(mid-edge\\) or 4"):
        c.set_constraints(m.con_vertex, bad_nr, m.con_par)
    chain = m.con_par.copy()
    chain[0, 0] = m.con_vertex[1]
    with pytest.raises(gb.GbFemError, match="itself constrained"):
        c.set_constraints(m.con_vertex, m.con_nr, chain)
    # without constraints the structure's dof-less vertices are refused
    with pytest.raises(gb.GbFemError, match="hanging"):
        c.set_crs_structure(g["dof_of_node"], g["row_ptr"], g["col_ind"])
    c.set_constraints(m.con_vertex, m.con_nr, m.con_par)
    dn = g["dof_of_node"].copy()
    dn[m.con_vertex[0]] = 0
    with pytest.raises(gb.GbFemError, match="carries a dof"):
        c.set_crs_structure(dn, g["row_ptr"], g["col_ind"])
    with pytest.raises(gb.GbFemError, match="structure and tables come from the caller"):
        c.build_structure()
    # a new mesh clears the constraints
    c.set_mesh(m)
    with pytest.raises(gb.GbFemError, match="hanging"):
        c.set_crs_structure(g["dof_of_node"], g["row_ptr"], g["col_ind"])
    c.close()
