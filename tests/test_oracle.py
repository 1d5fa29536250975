"""The C restatement (oracle/) against golden fixtures made by the reference.

CPU only.  These tests pin the oracle that the GPU parity tests then trust.
"""
import numpy as np
import pytest

import oracle as O
from _util import FixtureMesh, REL_TOL, crs_rel_err, face_rel_err, load, mat_rel_err, vec_rel_err


@pytest.fixture(scope="module", params=["std_n4", "std_n10", "std_n3_flat"])
def case(request):
    g = load(request.param)
    return request.param, g, FixtureMesh(g)


def test_element_matrices_bit_exact(case):
    name, g, m = case
    if "el_sm" not in g:
        pytest.skip("fixture keeps no element matrices")
    for e in range(m.nel):
        A = np.diag([g["k"][e]] * 3)
        K, r = O.std_prism_element(m.coords[m.el_nodes[e]], A, 1.0)
        # the restatement follows the reference's operation order: identical bits
        assert np.array_equal(K, g["el_sm"][e]), (name, e)
        assert np.array_equal(r, g["el_rhs"][e]), (name, e)


def test_face_matrices(case):
    name, g, m = case
    if "fa_sm" not in g:
        pytest.skip("fixture keeps no face matrices")
    for i in range(m.bc_face_id.size):
        X = m.coords[m.el_nodes[m.bc_face_el[i]]]
        K, r = O.std_prism_face(X, int(m.bc_face_side[i]), 1e7, 0.0)
        # face points are mapped through a different formula than the
        # reference's mmr_fa_elem_coor: equal up to rounding
        assert mat_rel_err(K, g["fa_sm"][i]) < REL_TOL, (name, i)
        assert np.array_equal(r, g["fa_rhs"][i])


def test_dof_order_and_crs_structure_bit_exact(case):
    name, g, m = case
    d, nd = O.dof_order(m.el_nodes, m.nno)
    assert np.array_equal(d, g["dof_of_node"])
    rp, ci = O.crs_structure(m.el_nodes, d, nd)
    assert np.array_equal(rp, g["row_ptr"])
    assert np.array_equal(ci, g["col_ind"])


def test_assembly_tables_bit_exact(case):
    name, g, m = case
    if g["color_elems"].size <= 2:
        pytest.skip("reference builds tables only with colouring (more than 1000 dofs)")
    rp, ci, d = g["row_ptr"], g["col_ind"], g["dof_of_node"]
    fa_of_id = {int(f): i for i, f in enumerate(m.bc_face_id)}
    for i, (t, eid) in enumerate(zip(g["int_ent_type"], g["int_ent_id"])):
        e = eid - 1 if t == 4 else m.bc_face_el[fa_of_id[int(eid)]]
        tab = O.crs_table(d[m.el_nodes[e]], rp, ci)
        p = g["asse_pos"][i]
        assert np.array_equal(tab, g["assembly_table"][p:p + 42]), (name, i)


def test_colouring_is_valid(case):
    name, g, m = case
    d = g["dof_of_node"]
    ed = d[m.el_nodes]
    col, nc = O.color_entities(ed, int(d.max()) + 1)
    for c in range(nc):
        dofs = ed[col == c].reshape(-1)
        assert np.unique(dofs).size == dofs.size, "two elements of one colour share a dof"


def test_assembled_values(case):
    name, g, m = case
    val, rhs, _ = O.std_prism_assemble(m, g["k"], g["dof_of_node"], g["row_ptr"], g["col_ind"])
    assert crs_rel_err(g["row_ptr"], val, g["crs_val"]) < REL_TOL
    assert vec_rel_err(rhs, g["crs_rhs"]) < REL_TOL


def test_residual(case):
    name, g, m = case
    v = O.crs_residual(g["row_ptr"], g["col_ind"], g["crs_val"], g["resid_x"], g["crs_rhs"])
    assert vec_rel_err(v, g["resid_v"]) < 1e-12


def test_gmres_matches_reference(case):
    name, g, m = case
    x, it, res, rel = O.gmres_jacobi(g["row_ptr"], g["col_ind"], g["crs_val"], g["crs_rhs"],
                                     int(g["krylov"]), 5000, float(g["tol"]))
    assert it == int(g["gmres_iters"])
    assert vec_rel_err(x, g["gmres_x"]) < 1e-10


def test_tet_elements_bit_exact():
    """Std tetrahedra: oracle equals the reference's apr_elem_calc_3D-based integral."""
    g = load("std_tet_n2")
    for e in range(g["el_nodes"].shape[0]):
        K, r = O.std_tet_element(g["coords"][g["el_nodes"][e]], np.diag([g["k"][e]] * 3), 1.0)
        assert np.array_equal(K, g["el_sm"][e]) and np.array_equal(r, g["el_rhs"][e]), e


@pytest.mark.parametrize("name", ["dg_el_n2", "dg_el_aniso_n2"])
def test_dg_elements_vs_reference(name):
    """DG tensor prisms (p = 1..4 mixed), isotropic and full-tensor coefficients."""
    g = load(name)
    for e in range(g["el_nodes"].shape[0]):
        p = int(g["pdeg"][e])
        A = g["D"][e] if g["D"].size else np.diag([g["k"][e]] * 3)
        K, r = O.dg_prism_element(g["coords"][g["el_nodes"][e]], A, p)
        ns = K.shape[0]
        Kr = g["sm"][g["sm_off"][e]:g["sm_off"][e + 1]].reshape(ns, ns)
        rr = g["rhs"][g["rhs_off"][e]:g["rhs_off"][e + 1]]
        assert mat_rel_err(K, Kr) < 1e-14, (e, p)
        assert vec_rel_err(r, rr) < 1e-14


@pytest.mark.parametrize("name", ["dg_el_n2", "dg_el_aniso_n2"])
def test_dg_faces_vs_reference(name):
    """DG faces: interior-penalty coupling of both neighbours (interior faces)
    and the Dirichlet boundary form, every face of the mixed-p mesh."""
    from modfem_gb300.mesh import prism_faces, structured_prism_mesh
    g = load(name)
    m = structured_prism_mesh(2, jitter=0.2, seed=21)
    assert np.array_equal(m.coords, g["coords"]) and np.array_equal(m.el_nodes, g["el_nodes"])
    F = prism_faces(m)
    A = g["D"] if g["D"].size else np.array([np.diag([k] * 3).reshape(-1) for k in g["k"]])
    assert F.n == g["fa_sm_off"].size - 1
    for i in range(F.n):
        K, r = O.dg_face(m, F, i, g["pdeg"], A, pen=float(g["pen"]), g=float(g["g"]))
        n = K.shape[0]
        Kr = g["fa_sm"][g["fa_sm_off"][i]:g["fa_sm_off"][i + 1]].reshape(n, n)
        rr = g["fa_rhs"][g["fa_rhs_off"][i]:g["fa_rhs_off"][i + 1]]
        assert face_rel_err(K, Kr) < 1e-14, (i, int(F.type[i]), int(F.el2[i]))
        assert vec_rel_err(r, rr) < 1e-14 if np.any(rr) else not np.any(r), i


@pytest.mark.parametrize("name", ["dg_asm_p2", "dg_asm_mixed", "dg_asm_aniso"])
def test_dg_assembled_system_vs_reference(name):
    """The whole DG system (elements + interior-penalty and Dirichlet faces,
    block storage) against the reference MKB solver's lad_block matrix:
    dof order and block pattern identical, values within 1e-12."""
    from _util import sparse_rel_err
    from modfem_gb300.mesh import prism_faces, structured_prism_mesh
    g = load(name)
    m = structured_prism_mesh(int(g["n"]), jitter=float(g["jitter"]), seed=int(g["seed"]))
    assert np.array_equal(m.coords, g["coords"])
    F = prism_faces(m)
    A = g["D"].reshape(-1, 9) if g["D"].size else np.array([np.diag([k] * 3).reshape(-1) for k in g["k"]])
    rp, ci, val, rhs, off = O.dg_assemble(m, F, g["pdeg"], A, pen=float(g["pen"]), g=float(g["g"]),
                                          f=float(g["f"]))
    assert np.array_equal(g["dof_ent_id"], np.arange(1, m.nel + 1))
    assert np.array_equal(g["dof_posglob"], off[:-1])
    assert np.array_equal(rp, g["row_ptr"]) and np.array_equal(ci, g["col_ind"])
    assert sparse_rel_err(rp, ci, val, g["val"]) < REL_TOL
    assert vec_rel_err(rhs, g["rhs"]) < REL_TOL
