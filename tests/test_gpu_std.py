"""GPU parity of the std-linear integrate / assemble / SpMV / GMRES path.

All calls go through the C ABI (libmodfem_gb300.so via ctypes).  References:
golden fixtures made by the reference ModFEM compiled in-tree
(tests/golden/make_golden.py) and, for sizes without fixtures, the C oracle
pinned by tests/test_oracle.py.
"""
import ctypes

import numpy as np
import pytest

import oracle as O
from _util import FixtureMesh, REL_TOL, crs_rel_err, energy_scale, load, mat_rel_err, vec_rel_err

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gb():
    from modfem_gb300 import build
    build.build(verbose=False)
    import modfem_gb300
    return modfem_gb300


def make_ctx(gb, m, k, structure=None, f=1.0, penalty=1e7):
    c = gb.Context(0)
    c.set_mesh(m)
    c.set_coefficients(k=k, f=f, g=0.0, penalty=penalty)
    if structure is not None:
        c.set_crs_structure(*structure)
    return c


# ---------------------------------------------------------------- element level
def block_tables(nent, n):
    """Assembly tables into a block-diagonal CRS: entity i owns values
    [i*n*n, (i+1)*n*n) and rhs [i*n, (i+1)*n), so the assembled values are the
    local matrices themselves."""
    t = np.zeros((nent, n * n + n), np.int32)
    t[:, :n * n] = np.arange(nent)[:, None] * n * n + np.arange(n * n)[None, :]
    t[:, n * n:] = np.arange(nent)[:, None] * n + np.arange(n)[None, :]
    return t.reshape(-1), (np.arange(nent) * (n * n + n)).astype(np.int32)


def block_structure(nent, n):
    rp = (np.arange(nent * n + 1) * n).astype(np.int32)
    ci = np.tile(np.arange(n), nent * n).astype(np.int32)  # column values unused by the kernels
    return np.zeros(1, np.int32), rp, ci


@pytest.mark.parametrize("name", ["std_n4", "std_n3_flat"])
def test_element_matrices_vs_reference(gb, name):
    g = load(name)
    m = FixtureMesh(g)
    nel = m.nel
    dn, rp, ci = block_structure(nel, 6)
    c = make_ctx(gb, m, g["k"])
    c.set_crs_structure(np.zeros(m.nno, np.int32), rp, ci)
    tab, pos = block_tables(nel, 6)
    types = np.full(nel, gb.ELEMENT, np.int32)
    ids = np.arange(1, nel + 1, dtype=np.int32)
    val = np.zeros(36 * nel)
    rhs = np.zeros(6 * nel)
    c.create_assemble_stiff_mat(types, ids, np.array([0, nel], np.int32), None, pos, tab, crs_val=val, rhs=rhs)
    for e in range(nel):
        K = val[36 * e:36 * e + 36].reshape(6, 6).T  # column-major -> (row w, column u)
        assert mat_rel_err(K, g["el_sm"][e]) < REL_TOL, e
        assert vec_rel_err(rhs[6 * e:6 * e + 6], g["el_rhs"][e]) < REL_TOL, e


def test_face_matrices_vs_reference(gb):
    g = load("std_n4")
    m = FixtureMesh(g)
    nfa = m.bc_face_id.size
    c = make_ctx(gb, m, g["k"])
    dn, rp, ci = block_structure(nfa, 6)
    c.set_crs_structure(np.zeros(m.nno, np.int32), rp, ci)
    tab, pos = block_tables(nfa, 6)
    types = np.full(nfa, gb.FACE, np.int32)
    val = np.zeros(36 * nfa)
    rhs = np.zeros(6 * nfa)
    c.create_assemble_stiff_mat(types, m.bc_face_id, None, np.array([0, nfa], np.int32), pos, tab, crs_val=val,
                                rhs=rhs)
    for i in range(nfa):
        K = val[36 * i:36 * i + 36].reshape(6, 6).T
        assert mat_rel_err(K, g["fa_sm"][i]) < REL_TOL, i


# ------------------------------------------------------------- drop-in boundary
def test_dropin_create_assemble_matches_reference(gb):
    """pdr_create_assemble_stiff_mat drop-in fed with the reference's own
    entity lists, colours and assembly tables (sir_create output)."""
    g = load("std_n10")
    m = FixtureMesh(g)
    c = make_ctx(gb, m, g["k"], (g["dof_of_node"], g["row_ptr"], g["col_ind"]))
    val = np.zeros(g["col_ind"].size)
    rhs = np.zeros(g["row_ptr"].size - 1)
    sc = energy_scale(g["row_ptr"], g["col_ind"], g["crs_val"])
    for _ in range(2):  # the second call must clear and give the same values
        c.create_assemble_stiff_mat(g["int_ent_type"], g["int_ent_id"], g["color_elems"], g["color_faces"],
                                    g["asse_pos"], g["assembly_table"], crs_val=val, rhs=rhs)
        assert crs_rel_err(g["row_ptr"], val, g["crs_val"], sc) < REL_TOL
        assert vec_rel_err(rhs, g["crs_rhs"]) < REL_TOL
    ms, el_ms, launches = c.last_timing()
    assert launches == 2 and ms > 0


@pytest.mark.parametrize("cache", [0, 1])
def test_dropin_comp_types_and_empty_lists(gb, cache):
    """Comp_type SM only and RHS only clear and fill just their part (the
    other keeps what the caller's array held, as MKB's matrix does between
    the calls); an empty entity list clears the matrix and rhs; entity ids
    outside the mesh are refused."""
    g = load("std_n10")
    m = FixtureMesh(g)
    c = make_ctx(gb, m, g["k"], (g["dof_of_node"], g["row_ptr"], g["col_ind"]))
    c.set_option(gb.OPT_CACHE_TABLES, cache)
    args = [np.ascontiguousarray(g[k], dtype=np.int32) for k in
            ("int_ent_type", "int_ent_id", "color_elems", "color_faces", "asse_pos", "assembly_table")]
    nnz, nd = g["col_ind"].size, g["row_ptr"].size - 1
    sc = energy_scale(g["row_ptr"], g["col_ind"], g["crs_val"])
    val, rhs = np.full(nnz, 3.5), np.full(nd, 3.5)
    c.create_assemble_stiff_mat(*args, comp_type=gb.COMP_SM, crs_val=val, rhs=None)
    assert crs_rel_err(g["row_ptr"], val, g["crs_val"], sc) < REL_TOL
    assert np.all(rhs == 3.5)
    c.create_assemble_stiff_mat(*args, comp_type=gb.COMP_RHS, crs_val=None, rhs=rhs)
    assert vec_rel_err(rhs, g["crs_rhs"]) < REL_TOL
    # both again through the device copy
    v2, r2 = c.get_matrix()
    assert crs_rel_err(g["row_ptr"], v2, g["crs_val"], sc) < REL_TOL and vec_rel_err(r2, g["crs_rhs"]) < REL_TOL
    # no entities: a cleared matrix
    e = np.zeros(0, np.int32)
    val0, rhs0 = np.full(nnz, 1.0), np.full(nd, 1.0)
    c.create_assemble_stiff_mat(e, e, np.array([0, 0], np.int32), None, e, args[5], crs_val=val0, rhs=rhs0)
    assert not np.any(val0) and not np.any(rhs0)
    # an element id beyond the mesh
    bad = args[1].copy()
    bad[3] = m.nel + 5
    with pytest.raises(gb.GbFemError, match="outside the mesh"):
        c.create_assemble_stiff_mat(args[0], bad, *args[2:], crs_val=val, rhs=rhs)
    c.close()


def test_dropin_table_cache(gb):
    g = load("std_n10")
    m = FixtureMesh(g)
    c = make_ctx(gb, m, g["k"], (g["dof_of_node"], g["row_ptr"], g["col_ind"]))
    c.set_option(gb.OPT_CACHE_TABLES, 1)
    args = [np.ascontiguousarray(g[k], dtype=np.int32) for k in
            ("int_ent_type", "int_ent_id", "color_elems", "color_faces", "asse_pos", "assembly_table")]
    val = np.zeros(g["col_ind"].size)
    rhs = np.zeros(g["row_ptr"].size - 1)
    k2 = g["k"] * 2.0
    c.create_assemble_stiff_mat(*args, crs_val=val, rhs=rhs)
    c.set_coefficients(k=k2)
    c.create_assemble_stiff_mat(*args, crs_val=val, rhs=rhs)  # cached tables, new coefficients
    vo, ro, _ = O.std_prism_assemble(m, k2, g["dof_of_node"], g["row_ptr"], g["col_ind"])
    sc = energy_scale(g["row_ptr"], g["col_ind"], vo)
    assert crs_rel_err(g["row_ptr"], val, vo, sc) < REL_TOL


GUARD = 16


def _guarded(n):
    """A host array of n doubles followed by GUARD sentinel entries; returns
    (the whole buffer, its first n entries as a view)."""
    buf = np.full(n + GUARD, 7.25)
    return buf, buf[:n]


def _own_dropin_problem(gb, n, seed):
    """A jittered n^3 x 2 prism mesh with the library's own structure and
    element tables laid out as the drop-in's entity lists (elements, then
    the boundary faces with their element's table), and the oracle's
    assembled values."""
    from modfem_gb300.mesh import lognormal_k, structured_prism_mesh
    m = structured_prism_mesh(n, jitter=0.2, seed=seed)
    k = lognormal_k(m.nel, seed=seed)
    c = make_ctx(gb, m, k)
    c.build_structure()
    tables = c.get_element_tables()
    dn, rp, ci = c.get_crs_structure()
    c.close()
    nf = m.bc_face_id.size
    lists = {"int_ent_type": np.concatenate([np.full(m.nel, gb.ELEMENT), np.full(nf, gb.FACE)]),
             "int_ent_id": np.concatenate([np.arange(1, m.nel + 1), m.bc_face_id]),
             "color_elems": np.array([0, m.nel]), "color_faces": np.array([m.nel, m.nel + nf]),
             "asse_pos": np.arange(m.nel + nf) * 42,
             "assembly_table": np.concatenate([tables, tables.reshape(m.nel, 42)[m.bc_face_el].reshape(-1)])}
    vo, ro, _ = O.std_prism_assemble(m, k, dn, rp, ci)
    return m, k, (dn, rp, ci), lists, vo, ro


LIST_NAMES = ("int_ent_type", "int_ent_id", "color_elems", "color_faces", "asse_pos", "assembly_table")


@pytest.mark.parametrize("cache", [0, 1])
def test_smaller_structure_in_a_live_context(gb, cache):
    """A large structure, then a smaller one in the same context: the device
    buffers keep their larger capacity, but every copy to or from the host is
    sized by the current structure (guard entries past the end stay as they
    were), and the drop-in, gbfem_get_matrix and gbfem_set_matrix give the
    small problem's values.  With the table cache on, the small problem's
    lists and tables sit at the same host addresses as the large one's."""
    big, small = _own_dropin_problem(gb, 12, 21), _own_dropin_problem(gb, 5, 22)
    bufs = {k: np.zeros(big[3][k].size + 64, np.int32) for k in LIST_NAMES}
    c = gb.Context(0)
    c.set_option(gb.OPT_CACHE_TABLES, cache)
    for m, k, st, lists, vo, ro in (big, small):
        c.set_mesh(m)
        c.set_coefficients(k=k, f=1.0, g=0.0, penalty=1e7)
        c.set_crs_structure(*st)
        rp, ci = st[1], st[2]
        nnz, nd = ci.size, rp.size - 1
        args = []
        for name in LIST_NAMES:
            a = lists[name].astype(np.int32)
            bufs[name][:a.size] = a
            args.append(bufs[name][:a.size])
        vb, val = _guarded(nnz)
        rb, rhs = _guarded(nd)
        c.create_assemble_stiff_mat(*args, crs_val=val, rhs=rhs)
        assert np.all(vb[nnz:] == 7.25) and np.all(rb[nd:] == 7.25)
        sc = energy_scale(rp, ci, vo)
        assert crs_rel_err(rp, val, vo, sc) < REL_TOL
        assert vec_rel_err(rhs, ro) < REL_TOL
        # download into exactly-sized views of guarded buffers
        vb2, val2 = _guarded(nnz)
        rb2, rhs2 = _guarded(nd)
        c.get_matrix(val2, rhs2)
        assert np.all(vb2[nnz:] == 7.25) and np.all(rb2[nd:] == 7.25)
        assert np.array_equal(val2, val) and np.array_equal(rhs2, rhs)
        # upload reads nnz / ndof entries only: the guard values must not arrive
        c.set_matrix(vb2[:nnz] * 2.0, rb2[:nd] * 2.0)
        val3, rhs3 = c.get_matrix()
        assert np.array_equal(val3, 2.0 * val) and np.array_equal(rhs3, 2.0 * rhs)
    c.close()


def test_dropin_cache_sees_new_tables_at_the_same_address(gb):
    """With cached tables, the entity order changed in place (same host
    pointers, same lengths): the sampled contents differ, so the call
    uploads the lists again and rebuilds its chunked download plan; setting
    the option again or gbfem_invalidate_tables voids the cache too.  Each
    call matches a one-shot call without the cache."""
    from modfem_gb300.mesh import lognormal_k, structured_prism_mesh
    m = structured_prism_mesh(50, jitter=0.2, seed=7)
    k = lognormal_k(m.nel, seed=7)
    ref = make_ctx(gb, m, k)
    nd, nnz, _ = ref.build_structure()
    tables = ref.get_element_tables()
    fa_tab = tables.reshape(m.nel, 42)[m.bc_face_el].reshape(-1)
    tab = np.concatenate([tables, fa_tab]).astype(np.int32)
    nf = m.bc_face_id.size
    types = np.concatenate([np.full(m.nel, gb.ELEMENT), np.full(nf, gb.FACE)]).astype(np.int32)
    ce = np.array([0, m.nel], np.int32)
    cf = np.array([m.nel, m.nel + nf], np.int32)
    ids = np.zeros(m.nel + nf, np.int32)
    pos = np.zeros(m.nel + nf, np.int32)

    def fill(order):
        ids[:m.nel] = order + 1
        ids[m.nel:] = m.bc_face_id
        pos[:m.nel] = order * 42
        pos[m.nel:] = 42 * m.nel + np.arange(nf) * 42

    fill(np.arange(m.nel))
    v0, r0 = np.zeros(nnz), np.zeros(nd)
    ref.create_assemble_stiff_mat(types, ids, ce, cf, pos, tab, crs_val=v0, rhs=r0)
    sc = np.abs(v0) + 1e-300

    c = make_ctx(gb, m, k)
    c.build_structure()
    c.set_option(gb.OPT_CACHE_TABLES, 1)
    val, rhs = np.zeros(nnz), np.zeros(nd)

    def run():
        val[:] = 0
        rhs[:] = 0
        c.create_assemble_stiff_mat(types, ids, ce, cf, pos, tab, crs_val=val, rhs=rhs)
        assert np.max(np.abs(val - v0) / np.maximum(sc, 1e-3 * np.max(sc))) < 1e-12
        assert np.max(np.abs(rhs - r0)) <= 1e-12 * np.max(np.abs(r0))

    run()
    gen0, up0 = c.table_cache_stats()
    run()  # cache hit: nothing uploaded
    assert c.table_cache_stats() == (gen0, up0)
    fill(np.random.default_rng(1).permutation(m.nel))  # same addresses, new order
    run()
    gen1, up1 = c.table_cache_stats()
    assert up1 == up0 + 2  # ids and positions again; the assembly table is unchanged
    fill(np.arange(m.nel)[::-1].copy())
    c.set_option(gb.OPT_CACHE_TABLES, 1)  # voids the cache: all three arrays again
    run()
    gen2, up2 = c.table_cache_stats()
    assert gen2 > gen1 and up2 == up1 + 3
    c.invalidate_tables()
    run()
    assert c.table_cache_stats()[1] == up2 + 3
    # a new structure voids the cache as well
    c.set_crs_structure(*ref.get_crs_structure())
    run()
    assert c.table_cache_stats()[1] == up2 + 6
    ref.close()
    c.close()


def test_constrained_vertices_are_refused(gb):
    """A once-refined ModFEM mesh has constrained (hanging) vertices: they
    carry no dof, and the dof lists of their elements name the constraining
    vertices instead (apr_get_stiff_mat_data, aps_std_lin_intf.c:2995-3170),
    so sir_create reports more dofs per entity than vertices.  Without the
    constraint data (gbfem_set_constraints) both signs of it are refused
    with an error instead of assembling a wrong matrix."""
    g = load("std_n10")
    m = FixtureMesh(g)
    c = make_ctx(gb, m, g["k"])
    dn = g["dof_of_node"].astype(np.int32).copy()
    hanging = int(m.el_nodes[7, 4])
    dn[hanging] = -1  # a vertex without a dof
    with pytest.raises(gb.GbFemError, match="hanging"):
        c.set_crs_structure(dn, g["row_ptr"], g["col_ind"])
    # the conforming structure is accepted; a dof list longer than the
    # element's vertex count is refused by the drop-in
    c.set_crs_structure(g["dof_of_node"], g["row_ptr"], g["col_ind"])
    val, rhs = np.zeros(g["col_ind"].size), np.zeros(g["row_ptr"].size - 1)
    args = [g[k] for k in ("int_ent_type", "int_ent_id", "color_elems", "color_faces", "asse_pos",
                           "assembly_table")]
    with pytest.raises(gb.GbFemError, match="hanging"):
        c.create_assemble_stiff_mat(*args, crs_val=val, rhs=rhs, max_dofs=9)
    c.create_assemble_stiff_mat(*args, crs_val=val, rhs=rhs)
    assert crs_rel_err(g["row_ptr"], val, g["crs_val"], energy_scale(g["row_ptr"], g["col_ind"], g["crs_val"])) \
        < REL_TOL
    c.close()


@pytest.mark.parametrize("shuffle", [False, True])
def test_dropin_pipelined_download(gb, shuffle):
    """With cached tables the drop-in runs the elements in chunks and copies
    each chunk's finished rows while the next runs: 250,000 prisms (three
    chunks) give the values of the one-shot call, also with the elements in
    shuffled order (rows then finish late) and with the rhs alone."""
    from modfem_gb300.mesh import lognormal_k, structured_prism_mesh
    m = structured_prism_mesh(50, jitter=0.2, seed=3)
    k = lognormal_k(m.nel, seed=3)
    c = make_ctx(gb, m, k)
    nd, nnz, _ = c.build_structure()
    tables = c.get_element_tables()
    order = np.random.default_rng(5).permutation(m.nel) if shuffle else np.arange(m.nel)
    fa_tab = tables.reshape(m.nel, 42)[m.bc_face_el].reshape(-1)
    ids = np.concatenate([order + 1, m.bc_face_id]).astype(np.int32)
    types = np.concatenate([np.full(m.nel, gb.ELEMENT), np.full(m.bc_face_id.size, gb.FACE)]).astype(np.int32)
    table = np.concatenate([tables.reshape(m.nel, 42)[order].reshape(-1), fa_tab]).astype(np.int32)
    pos = (np.arange(ids.size) * 42).astype(np.int32)
    ce = np.array([0, m.nel], np.int32)
    cf = np.array([m.nel, ids.size], np.int32)
    args = (types, ids, ce, cf, pos, table)
    v1, r1 = np.zeros(nnz), np.zeros(nd)
    c.create_assemble_stiff_mat(*args, crs_val=v1, rhs=r1)  # one shot
    c.set_option(gb.OPT_CACHE_TABLES, 1)
    for _ in range(2):  # plan built on the first call, reused on the second
        v2, r2 = np.full(nnz, np.nan), np.full(nd, np.nan)
        c.create_assemble_stiff_mat(*args, crs_val=v2, rhs=r2)
        sc = np.max(np.abs(v1))
        assert np.max(np.abs(v2 - v1)) <= 1e-12 * sc
        assert np.max(np.abs(r2 - r1)) <= 1e-12 * np.max(np.abs(r1))
    _, _, launches = c.last_timing()
    assert launches == 1 + 3
    r3 = np.full(nd, np.nan)
    c.create_assemble_stiff_mat(*args, crs_val=None, rhs=r3)
    assert np.max(np.abs(r3 - r1)) <= 1e-12 * np.max(np.abs(r1))
    dn, rp, ci = c.get_crs_structure()
    vo, ro, _ = O.std_prism_assemble(m, k, dn, rp, ci, nthreads=8)
    assert crs_rel_err(rp, v2, vo, energy_scale(rp, ci, vo)) < REL_TOL
    assert vec_rel_err(r2, ro) < REL_TOL


@pytest.mark.parametrize("shuffle", [False, True])
def test_dropin_overlaps_coordinate_and_coefficient_uploads(gb, shuffle):
    """With cached tables, new node coordinates and coefficients set before
    each call go up in pieces while the element chunks that do not read the
    rest already run: over three calls with different coordinates, k or a
    full tensor, every result equals the oracle's (in element order and
    shuffled, where a chunk reads nodes all over the mesh), and so do the
    library's own assembly and a residual right after (the context stream
    waits for every piece)."""
    from modfem_gb300.mesh import anisotropic_tensors, lognormal_k, structured_prism_mesh
    n = 50
    c = None
    order = np.random.default_rng(6).permutation(n ** 3 * 2) if shuffle else np.arange(n ** 3 * 2)
    for it, seed in enumerate((3, 4, 5)):
        m = structured_prism_mesh(n, jitter=0.2, seed=seed)
        k = lognormal_k(m.nel, seed=seed)
        D = anisotropic_tensors(m.nel, seed=seed).reshape(-1, 9) if it == 2 else None
        if c is None:
            c = make_ctx(gb, m, k)
            nd, nnz, _ = c.build_structure()
            tables = c.get_element_tables().reshape(m.nel, 42)
            fa_tab = tables[m.bc_face_el].reshape(-1)
            ids = np.concatenate([order + 1, m.bc_face_id]).astype(np.int32)
            types = np.concatenate([np.full(m.nel, gb.ELEMENT), np.full(m.bc_face_id.size, gb.FACE)]).astype(np.int32)
            table = np.concatenate([tables[order].reshape(-1), fa_tab]).astype(np.int32)
            pos = (np.arange(ids.size) * 42).astype(np.int32)
            args = (types, ids, np.array([0, m.nel], np.int32), np.array([m.nel, ids.size], np.int32), pos, table)
            c.set_option(gb.OPT_CACHE_TABLES, 1)
            dn, rp, ci = c.get_crs_structure()
        c.set_node_coords(m.coords)
        if D is None:
            c.set_coefficients(k=k, f=1.0, g=0.0, penalty=1e7)
        else:
            c.set_coefficients(D=D, f=1.0, g=0.0, penalty=1e7)
        v, r = np.full(nnz, np.nan), np.full(nd, np.nan)
        c.create_assemble_stiff_mat(*args, crs_val=v, rhs=r)
        kw = dict(D_el=D) if D is not None else {}
        vo, ro, _ = O.std_prism_assemble(m, k, dn, rp, ci, nthreads=8, **kw)
        assert crs_rel_err(rp, v, vo, energy_scale(rp, ci, vo)) < REL_TOL, it
        assert vec_rel_err(r, ro) < REL_TOL, it
    # the library's own assembly after piece uploads
    m = structured_prism_mesh(n, jitter=0.2, seed=7)
    k = lognormal_k(m.nel, seed=7)
    c.set_node_coords(m.coords)
    c.set_coefficients(k=k, f=1.0, g=0.0, penalty=1e7)
    c.assemble(gb.SCATTER_ATOMIC)
    v, r = c.get_matrix()
    vo, ro, _ = O.std_prism_assemble(m, k, dn, rp, ci, nthreads=8)
    assert crs_rel_err(rp, v, vo, energy_scale(rp, ci, vo)) < REL_TOL
    assert vec_rel_err(r, ro) < REL_TOL
    c.close()


def test_double_word_assembly_vs_reference_and_oracle(gb):
    """Element matrices in double-word arithmetic (float pairs on the FP32
    pipe): the reference's own assembled matrix (golden, std_n10), and on a
    jittered 40^3 x 2 mesh with lognormal k the oracle's stiffness without
    penalty, both within the 1e-12 energy-scale bound; atomic, colour and
    drop-in paths agree."""
    g = load("std_n10")
    m = FixtureMesh(g)
    c = make_ctx(gb, m, g["k"], (g["dof_of_node"], g["row_ptr"], g["col_ind"]))
    c.set_option(gb.OPT_STD_ARITH, gb.STD_DWORD)
    val = np.zeros(g["col_ind"].size)
    rhs = np.zeros(g["row_ptr"].size - 1)
    c.create_assemble_stiff_mat(g["int_ent_type"], g["int_ent_id"], g["color_elems"], g["color_faces"],
                                g["asse_pos"], g["assembly_table"], crs_val=val, rhs=rhs)
    sc = energy_scale(g["row_ptr"], g["col_ind"], g["crs_val"])
    assert crs_rel_err(g["row_ptr"], val, g["crs_val"], sc) < REL_TOL
    assert vec_rel_err(rhs, g["crs_rhs"]) < REL_TOL

    from modfem_gb300.mesh import lognormal_k, structured_prism_mesh
    m = structured_prism_mesh(40, jitter=0.2, seed=11)
    k = lognormal_k(m.nel, seed=11)
    c = make_ctx(gb, m, k, penalty=0.0)
    c.build_structure()
    dn, rp, ci = c.get_crs_structure()
    c.assemble(gb.SCATTER_ATOMIC)
    v64, r64 = c.get_matrix()
    c.set_option(gb.OPT_STD_ARITH, gb.STD_DWORD)
    c.assemble(gb.SCATTER_ATOMIC)
    vdw, rdw = c.get_matrix()
    c.assemble(gb.SCATTER_COLOR)
    vdc, rdc = c.get_matrix()
    vo, ro, _ = O.std_prism_assemble(m, k, dn, rp, ci, penalty=0.0, nthreads=8)
    es = energy_scale(rp, ci, vo)
    assert crs_rel_err(rp, vdw, vo, es) < REL_TOL
    assert crs_rel_err(rp, vdc, vo, es) < REL_TOL
    assert vec_rel_err(rdw, ro) < REL_TOL
    # the double-word entries sit within 1e-13 of the FP64 kernel's
    assert crs_rel_err(rp, vdw, v64, es) < 1e-13
    assert vec_rel_err(rdw, r64) < 1e-13
    # constants stay in the kernel of the stiffness
    rows_sum = np.add.reduceat(vdw, rp[:-1])
    assert np.max(np.abs(rows_sum)) < 1e-12 * np.max(np.abs(vdw))


def test_dropin_rejects_bad_entities_and_recovers(gb):
    g = load("std_n4")
    m = FixtureMesh(g)
    d, nd = O.dof_order(m.el_nodes, m.nno)
    rp, ci = O.crs_structure(m.el_nodes, d, nd)
    c = make_ctx(gb, m, g["k"], (d, rp, ci))
    nel = m.nel
    tab = np.concatenate([O.crs_table(d[m.el_nodes[e]], rp, ci) for e in range(nel)])
    pos = (np.arange(nel) * 42).astype(np.int32)
    ids = np.arange(1, nel + 1, dtype=np.int32)
    bad = ids.copy()
    bad[5] = nel + 7  # not an element of the mesh
    types = np.full(nel, gb.ELEMENT, np.int32)
    with pytest.raises(gb.GbFemError, match="outside the mesh"):
        c.create_assemble_stiff_mat(types, bad, np.array([0, nel], np.int32), None, pos, tab)
    with pytest.raises(gb.GbFemError):
        c.create_assemble_stiff_mat(types, ids, np.array([0, nel], np.int32), None, pos, tab, level_id=1)
    # the context stays usable
    val = np.zeros(ci.size)
    rhs = np.zeros(nd)
    c.create_assemble_stiff_mat(types, ids, np.array([0, nel], np.int32), None, pos, tab, crs_val=val, rhs=rhs)
    vo = np.zeros(ci.size)
    ro = np.zeros(nd)
    for e in range(nel):
        K, r = O.std_prism_element(m.coords[m.el_nodes[e]], np.diag([g["k"][e]] * 3))
        t = tab[42 * e:42 * e + 42]
        np.add.at(vo, t[:36], K.T.reshape(-1))
        np.add.at(ro, t[36:], r)
    assert crs_rel_err(rp, val, vo, energy_scale(rp, ci, vo)) < REL_TOL


# -------------------------------------------------- library-built structure
@pytest.mark.parametrize("name", ["std_n4", "std_n10"])
def test_built_structure_and_assembly_vs_reference(gb, name):
    g = load(name)
    m = FixtureMesh(g)
    c = make_ctx(gb, m, g["k"])
    nd, nnz, ncol = c.build_structure()
    dn, rp, ci = c.get_crs_structure()
    assert np.array_equal(dn, g["dof_of_node"])
    assert np.array_equal(rp, g["row_ptr"])
    assert np.array_equal(ci, g["col_ind"])
    sc = energy_scale(rp, ci, g["crs_val"])
    for mode in (gb.SCATTER_ATOMIC, gb.SCATTER_COLOR, gb.SCATTER_GATHER):
        c.assemble(mode)
        val, rhs = c.get_matrix()
        assert crs_rel_err(rp, val, g["crs_val"], sc) < REL_TOL, mode
        assert vec_rel_err(rhs, g["crs_rhs"]) < REL_TOL, mode


@pytest.mark.parametrize("mode", ["color", "gather"])
def test_color_and_gather_modes_are_deterministic(gb, mode):
    from modfem_gb300.mesh import lognormal_k, structured_prism_mesh
    md = gb.SCATTER_COLOR if mode == "color" else gb.SCATTER_GATHER
    m = structured_prism_mesh(16, jitter=0.2, seed=9)
    k = lognormal_k(m.nel, seed=9)
    c = make_ctx(gb, m, k)
    c.build_structure()
    c.assemble(md)
    v1, r1 = c.get_matrix()
    c.assemble(md)
    v2, r2 = c.get_matrix()
    assert np.array_equal(v1, v2) and np.array_equal(r1, r2)


def test_gather_scatter_after_device_build(gb):
    """The gather scatter (one thread a row over the incident elements in
    element order) on a device-built structure, isotropic and anisotropic,
    against the oracle; bit-identical on a second context (no dependence on
    thread scheduling); the tetrahedron and double-word forms refused."""
    from modfem_gb300.mesh import anisotropic_tensors, lognormal_k, structured_prism_mesh, structured_tet_mesh
    m = structured_prism_mesh(14, jitter=0.2, seed=12)
    k = lognormal_k(m.nel, seed=12)
    D = anisotropic_tensors(m.nel, seed=13).reshape(-1, 9)
    for coef in ("k", "D"):
        outs = []
        for _ in range(2):
            c = gb.Context(0)
            c.set_mesh(m)
            if coef == "k":
                c.set_coefficients(k=k, f=1.0, g=0.3, penalty=1e7)
            else:
                c.set_coefficients(D=D, f=1.0, g=0.3, penalty=1e7)
            c.build_structure_device()
            c.assemble(gb.SCATTER_GATHER)
            outs.append(c.get_matrix())
            dn, rp, ci = c.get_crs_structure()
            c.close()
        assert np.array_equal(outs[0][0], outs[1][0]) and np.array_equal(outs[0][1], outs[1][1])
        kw = dict(D_el=D) if coef == "D" else {}
        vo, ro, _ = O.std_prism_assemble(m, k, dn, rp, ci, f=1.0, penalty=1e7, g=0.3, **kw)
        assert crs_rel_err(rp, outs[0][0], vo, energy_scale(rp, ci, vo)) < REL_TOL, coef
        assert vec_rel_err(outs[0][1], ro) < REL_TOL, coef
    c = gb.Context(0)
    c.set_mesh(m)
    c.set_coefficients(k=k, f=1.0, g=0.0)
    c.set_option(gb.OPT_STD_ARITH, gb.STD_DWORD)
    c.build_structure_device()
    with pytest.raises(gb.GbFemError, match="gather scatter"):
        c.assemble(gb.SCATTER_GATHER)
    c.close()
    t = structured_tet_mesh(3, jitter=0.1, seed=2)
    c = make_ctx(gb, t, lognormal_k(t.nel, seed=2))
    c.build_structure()
    with pytest.raises(gb.GbFemError, match="gather scatter"):
        c.assemble(gb.SCATTER_GATHER)
    c.close()


# ------------------------------------------------------------ SpMV and GMRES
def test_residual_vs_reference(gb):
    g = load("std_n10")
    m = FixtureMesh(g)
    c = make_ctx(gb, m, g["k"], (g["dof_of_node"], g["row_ptr"], g["col_ind"]))
    c.set_matrix(g["crs_val"], g["crs_rhs"])
    v = c.compute_residual(g["resid_x"])
    assert vec_rel_err(v, g["resid_v"]) < 1e-12
    v0 = c.compute_residual(g["resid_x"], ini_zero=1)
    assert np.array_equal(v0, g["crs_rhs"])
    b = np.cos(np.arange(v.size))
    v2 = c.compute_residual(g["resid_x"], b=b)
    assert vec_rel_err(v2, O.crs_residual(g["row_ptr"], g["col_ind"], g["crs_val"], g["resid_x"], b)) < 1e-12


@pytest.mark.parametrize("name", ["std_n4", "std_n10", "std_n3_flat"])
def test_gmres_vs_reference(gb, name):
    g = load(name)
    m = FixtureMesh(g)
    c = make_ctx(gb, m, g["k"], (g["dof_of_node"], g["row_ptr"], g["col_ind"]))
    c.set_matrix(g["crs_val"], g["crs_rhs"])
    x, it, res, rel = c.solve(int(g["krylov"]), 5000, float(g["tol"]))
    assert abs(it - int(g["gmres_iters"])) <= 1
    assert rel < float(g["tol"])
    # both stop at the same relative preconditioned residual; solutions agree
    # to the accuracy that tolerance allows
    assert vec_rel_err(x, g["gmres_x"]) < 1e3 * float(g["tol"])


def test_gmres_tight_tolerance_vs_oracle(gb):
    from modfem_gb300.mesh import lognormal_k, structured_prism_mesh
    m = structured_prism_mesh(8, jitter=0.2, seed=2)
    k = lognormal_k(m.nel, seed=2)
    c = make_ctx(gb, m, k)
    c.build_structure()
    c.assemble(gb.SCATTER_ATOMIC)
    val, rhs = c.get_matrix()
    dn, rp, ci = c.get_crs_structure()
    x, it, res, rel = c.solve(30, 20000, 1e-13)
    xo, ito, _, _ = O.gmres_jacobi(rp, ci, val, rhs, 30, 20000, 1e-13)
    assert vec_rel_err(x, xo) < 1e-9
    # the stopping measure is the Jacobi-preconditioned residual (the 1e7
    # penalty rows dominate the unpreconditioned one)
    rows = np.repeat(np.arange(rp.size - 1), np.diff(rp))
    diag = val[rows == ci]
    r = O.crs_residual(rp, ci, val, x, rhs) / diag
    # GMRES stops at max(1e-13 * initial, 1e-12 absolute): here the absolute floor
    assert np.linalg.norm(r) < 1.1 * max(1e-12, 1e-13 * np.linalg.norm(rhs / diag))


@pytest.mark.parametrize("spmv", ["fp64", "dword"])
def test_gmres_sliced_ell_column_forms(gb, spmv):
    """gbfem_solve's SpMV runs on a sliced-ELL copy with 16-bit column
    offsets where every column lies within 32767 of its row, 32-bit indices
    otherwise.  The same system in the first-appearance dof order (16-bit
    form) and under a random symmetric permutation of the dofs (32-bit form:
    columns up to 68,920 away) gives the same iterations (Jacobi-
    preconditioned GMRES is invariant under symmetric permutations up to
    rounding) and the same solution; both match the oracle's GMRES."""
    from modfem_gb300.mesh import lognormal_k, structured_prism_mesh
    m = structured_prism_mesh(40, jitter=0.2, seed=6)
    k = lognormal_k(m.nel, seed=6)
    c = make_ctx(gb, m, k)
    nd, nnz, _ = c.build_structure()
    c.assemble(gb.SCATTER_ATOMIC)
    val, rhs = c.get_matrix()
    dn, rp, ci = c.get_crs_structure()
    rows = np.repeat(np.arange(nd), np.diff(rp))
    assert np.max(np.abs(ci - rows)) < 32767
    c.set_option(gb.OPT_STD_SPMV_ARITH, gb.STD_DWORD if spmv == "dword" else gb.STD_FP64)
    x, it, _, rel = c.solve(30, 3000, 1e-10)
    # the permuted system: new dof q = perm[old]
    perm = np.random.default_rng(8).permutation(nd)
    inv = np.argsort(perm)
    cols_new = perm[ci]
    order = np.lexsort((cols_new, perm[rows]))  # by new row, then new column
    rp2 = np.concatenate([[0], np.cumsum(np.bincount(perm[rows], minlength=nd))]).astype(np.int32)
    ci2 = cols_new[order].astype(np.int32)
    assert np.max(np.abs(ci2 - np.repeat(np.arange(nd), np.diff(rp2)))) > 32767
    c2 = gb.Context(0)
    c2.set_mesh(m)
    c2.set_coefficients(k=k)
    c2.set_crs_structure(perm[dn].astype(np.int32), rp2, ci2)
    c2.set_matrix(val[order], rhs[inv])
    c2.set_option(gb.OPT_STD_SPMV_ARITH, gb.STD_DWORD if spmv == "dword" else gb.STD_FP64)
    x2, it2, _, rel2 = c2.solve(30, 3000, 1e-10)
    assert abs(it - it2) <= 1 and rel < 1e-10 and rel2 < 1e-10
    assert vec_rel_err(x2[perm], x) < 1e-8
    xo, ito, _, _ = O.gmres_jacobi(rp, ci, val, rhs, 30, 3000, 1e-10)
    assert abs(it - ito) <= 1
    assert vec_rel_err(x, xo) < 1e-8
    c.close()
    c2.close()


# ------------------------------------------------------------ larger sizes
def test_stiffness_without_penalty_vs_oracle(gb):
    """Stiffness alone (penalty 0): every entry against the oracle in the
    energy scale sqrt(a_rr a_cc), and the diagonal entrywise."""
    from modfem_gb300.mesh import lognormal_k, structured_prism_mesh
    m = structured_prism_mesh(30, jitter=0.2, seed=6)
    k = lognormal_k(m.nel, seed=6)
    c = make_ctx(gb, m, k, penalty=0.0)
    c.build_structure()
    c.assemble(gb.SCATTER_ATOMIC)
    val, rhs = c.get_matrix()
    dn, rp, ci = c.get_crs_structure()
    vo, ro, _ = O.std_prism_assemble(m, k, dn, rp, ci, penalty=0.0)
    assert crs_rel_err(rp, val, vo, energy_scale(rp, ci, vo)) < REL_TOL
    rows = np.repeat(np.arange(rp.size - 1), np.diff(rp))
    d = rows == ci
    assert np.max(np.abs(val[d] - vo[d]) / np.abs(vo[d])) < REL_TOL
    assert vec_rel_err(rhs, ro) < REL_TOL


def test_config1_size_vs_oracle(gb):
    """20^3 x 2 = 16,000 prisms (the reference's CPU-runnable configuration)."""
    from modfem_gb300.mesh import structured_prism_mesh
    m = structured_prism_mesh(20)
    k = np.ones(m.nel)
    c = make_ctx(gb, m, k)
    nd, nnz, _ = c.build_structure()
    assert (nd, nnz) == (9261, 178181)
    c.assemble(gb.SCATTER_ATOMIC)
    val, rhs = c.get_matrix()
    dn, rp, ci = c.get_crs_structure()
    vo, ro, _ = O.std_prism_assemble(m, k, dn, rp, ci)
    assert crs_rel_err(rp, val, vo, energy_scale(rp, ci, vo)) < REL_TOL
    assert vec_rel_err(rhs, ro) < REL_TOL
    x, it, res, rel = c.solve(30, 5000, 1e-8)
    xo, ito, _, _ = O.gmres_jacobi(rp, ci, vo, ro, 30, 5000, 1e-8)
    assert abs(it - ito) <= 1
    assert vec_rel_err(x, xo) < 1e-5


@pytest.mark.slow
def test_full_size_properties():
    """100^3 x 2 = 2,000,000 jittered prisms with lognormal k (the benchmark
    workload): structure identical to the oracle's, colour and atomic
    scatter agree, rhs sums to f*|cube| = 1, the matrix is symmetric, and a
    sample of rows matches the oracle."""
    import modfem_gb300 as gb
    from modfem_gb300 import build
    from modfem_gb300.mesh import lognormal_k, structured_prism_mesh
    build.build(verbose=False)
    m = structured_prism_mesh(100, jitter=0.2, seed=1)
    k = lognormal_k(m.nel, seed=1)
    c = make_ctx(gb, m, k)
    nd, nnz, ncol = c.build_structure()
    assert (nd, nnz) == (1030301, 21250901)
    dn, rp, ci = c.get_crs_structure()
    d2, _ = O.dof_order(m.el_nodes, m.nno)
    assert np.array_equal(dn, d2)
    rp2, ci2 = O.crs_structure(m.el_nodes, d2, nd)
    assert np.array_equal(rp, rp2) and np.array_equal(ci, ci2)
    c.assemble(gb.SCATTER_ATOMIC)
    va, ra = c.get_matrix()
    c.assemble(gb.SCATTER_COLOR)
    vc, rc = c.get_matrix()
    sc = energy_scale(rp, ci, va)
    assert crs_rel_err(rp, va, vc, sc) < REL_TOL
    assert abs(ra.sum() - 1.0) < 1e-12
    # symmetry: A[r, c] == A[c, r]
    rows = np.repeat(np.arange(nd), np.diff(rp))
    key = rows.astype(np.int64) * nd + ci
    keyt = ci.astype(np.int64) * nd + rows
    order = np.argsort(key)
    post = np.searchsorted(key[order], keyt)
    assert crs_rel_err(rp, va, va[order[post]], sc) < REL_TOL
    vo, ro, _ = O.std_prism_assemble(m, k, dn, rp, ci, nthreads=8)
    assert crs_rel_err(rp, va, vo, energy_scale(rp, ci, vo)) < REL_TOL
    # stiffness alone (no penalty on the diagonal to hide behind)
    c.set_coefficients(k=k, f=1.0, g=0.0, penalty=0.0)
    c.assemble(gb.SCATTER_ATOMIC)
    vs, _ = c.get_matrix()
    vso, _, _ = O.std_prism_assemble(m, k, dn, rp, ci, penalty=0.0, nthreads=8)
    assert crs_rel_err(rp, vs, vso, energy_scale(rp, ci, vso)) < REL_TOL
    # constants are in the kernel of the stiffness: A 1 = 0 to rounding
    rows_sum = np.add.reduceat(vs, rp[:-1])
    assert np.max(np.abs(rows_sum)) < 1e-12 * np.max(np.abs(vs))
    assert vec_rel_err(ra, ro) < REL_TOL
    # the double-word element kernel (the benchmark's headline form) against
    # the oracle at the same size and tolerance: stiffness alone, then with
    # the penalty faces, through gbfem_assemble and through the drop-in with
    # cached tables and the chunked download the benchmark times
    c.set_option(gb.OPT_STD_ARITH, gb.STD_DWORD)
    c.assemble(gb.SCATTER_ATOMIC)
    vsd, _ = c.get_matrix()
    assert crs_rel_err(rp, vsd, vso, energy_scale(rp, ci, vso)) < REL_TOL
    assert np.max(np.abs(np.add.reduceat(vsd, rp[:-1]))) < 1e-12 * np.max(np.abs(vsd))
    c.set_coefficients(k=k, f=1.0, g=0.0, penalty=1e7)
    c.assemble(gb.SCATTER_ATOMIC)
    vdw, rdw = c.get_matrix()
    sco = energy_scale(rp, ci, vo)
    assert crs_rel_err(rp, vdw, vo, sco) < REL_TOL
    assert vec_rel_err(rdw, ro) < REL_TOL
    tables = c.get_element_tables()
    nf = m.bc_face_id.size
    tab = np.concatenate([tables, tables.reshape(m.nel, 42)[m.bc_face_el].reshape(-1)]).astype(np.int32)
    types = np.concatenate([np.full(m.nel, gb.ELEMENT), np.full(nf, gb.FACE)]).astype(np.int32)
    ids = np.concatenate([np.arange(1, m.nel + 1), m.bc_face_id]).astype(np.int32)
    pos = (np.arange(m.nel + nf) * 42).astype(np.int32)
    c.set_option(gb.OPT_CACHE_TABLES, 1)
    val, rhs = np.zeros(nnz), np.zeros(nd)
    for _ in range(2):
        c.create_assemble_stiff_mat(types, ids, np.array([0, m.nel], np.int32),
                                    np.array([m.nel, m.nel + nf], np.int32), pos, tab, crs_val=val, rhs=rhs)
        assert crs_rel_err(rp, val, vo, sco) < REL_TOL
        assert vec_rel_err(rhs, ro) < REL_TOL


# ------------------------------------------------------------- tetrahedra
def test_tet_element_matrices_vs_reference(gb):
    g = load("std_tet_n2")
    from modfem_gb300.mesh import TetMesh
    m = TetMesh(2, g["coords"], g["el_nodes"])
    nel = m.nel
    c = make_ctx(gb, m, g["k"])
    dn, rp, ci = block_structure(nel, 4)
    c.set_crs_structure(np.zeros(m.nno, np.int32), rp, ci)
    tab, pos = block_tables(nel, 4)
    val = np.zeros(16 * nel)
    rhs = np.zeros(4 * nel)
    c.create_assemble_stiff_mat(np.full(nel, gb.ELEMENT, np.int32), np.arange(1, nel + 1, dtype=np.int32),
                                np.array([0, nel], np.int32), None, pos, tab, crs_val=val, rhs=rhs)
    for e in range(nel):
        K = val[16 * e:16 * e + 16].reshape(4, 4).T
        assert mat_rel_err(K, g["el_sm"][e]) < REL_TOL, e
        assert vec_rel_err(rhs[4 * e:4 * e + 4], g["el_rhs"][e]) < REL_TOL, e


def test_tet_mesh_structure_and_assembly_vs_oracle(gb):
    from modfem_gb300.mesh import lognormal_k, structured_tet_mesh
    m = structured_tet_mesh(12, jitter=0.1, seed=4)
    k = lognormal_k(m.nel, seed=4)
    c = make_ctx(gb, m, k)
    nd, nnz, ncol = c.build_structure()
    dn, rp, ci = c.get_crs_structure()
    d2, nd2 = O.dof_order(m.el_nodes, m.nno)
    rp2, ci2 = O.crs_structure(m.el_nodes, d2, nd2)
    assert np.array_equal(dn, d2) and np.array_equal(rp, rp2) and np.array_equal(ci, ci2)
    vo = np.zeros(nnz)
    ro = np.zeros(nd)
    for e in range(m.nel):
        K, r = O.std_tet_element(m.coords[m.el_nodes[e]], np.diag([k[e]] * 3), 1.0)
        t = O.crs_table(dn[m.el_nodes[e]], rp, ci)
        np.add.at(vo, t[:16], K.T.reshape(-1))
        np.add.at(ro, t[16:], r)
    for mode in (gb.SCATTER_ATOMIC, gb.SCATTER_COLOR):
        c.assemble(mode)
        val, rhs = c.get_matrix()
        assert crs_rel_err(rp, val, vo, energy_scale(rp, ci, vo)) < REL_TOL
        assert vec_rel_err(rhs, ro) < REL_TOL


# ------------------------------------------------ structure built on the device
@pytest.mark.parametrize("name", ["std_n4", "std_n10"])
def test_device_structure_vs_reference(gb, name):
    """gbfem_build_structure_device: DOF order, CRS and tables identical to
    the reference's (and to the host build); atomic assembly on it."""
    g = load(name)
    m = FixtureMesh(g)
    c = make_ctx(gb, m, g["k"])
    c.build_structure()
    host = (c.get_crs_structure(), c.get_element_tables())
    nd, nnz = c.build_structure_device()
    dn, rp, ci = c.get_crs_structure()
    assert np.array_equal(dn, g["dof_of_node"])
    assert np.array_equal(rp, g["row_ptr"]) and np.array_equal(ci, g["col_ind"])
    assert np.array_equal(c.get_element_tables(), host[1])
    c.assemble(gb.SCATTER_ATOMIC)
    val, rhs = c.get_matrix()
    assert crs_rel_err(rp, val, g["crs_val"], energy_scale(rp, ci, g["crs_val"])) < REL_TOL
    assert vec_rel_err(rhs, g["crs_rhs"]) < REL_TOL
    # the device colouring: colour-batched plain adds give the reference's
    # matrix (a colour holding two elements with a shared dof would race)
    c.assemble(gb.SCATTER_COLOR)
    val, rhs = c.get_matrix()
    assert crs_rel_err(rp, val, g["crs_val"], energy_scale(rp, ci, g["crs_val"])) < REL_TOL
    assert vec_rel_err(rhs, g["crs_rhs"]) < REL_TOL


@pytest.mark.parametrize("kind", ["prism", "tet"])
def test_device_structure_vs_host_larger(gb, kind):
    """Jittered 2M-free sizes: 30^3 x 2 prisms / 12^3 x 6 tetrahedra, host and
    device builds bit-identical."""
    from modfem_gb300.mesh import lognormal_k, structured_prism_mesh, structured_tet_mesh
    m = structured_prism_mesh(30, jitter=0.2, seed=2) if kind == "prism" else structured_tet_mesh(12, jitter=0.2, seed=2)
    c = make_ctx(gb, m, lognormal_k(m.nel, seed=2))
    c.build_structure()
    h = c.get_crs_structure() + (c.get_element_tables(),)
    c.assemble(gb.SCATTER_COLOR)
    vh, rh = c.get_matrix()
    c.build_structure_device()
    d = c.get_crs_structure() + (c.get_element_tables(),)
    for a, b in zip(h, d):
        assert np.array_equal(a, b)
    # colour-batched assembly on the device colouring: repeatable bit for bit
    # and equal to the host colouring's to rounding
    c.assemble(gb.SCATTER_COLOR)
    v1, r1 = c.get_matrix()
    c.assemble(gb.SCATTER_COLOR)
    v2, r2 = c.get_matrix()
    assert np.array_equal(v1, v2) and np.array_equal(r1, r2)
    rp, ci = d[1], d[2]
    assert crs_rel_err(rp, v1, vh, energy_scale(rp, ci, vh)) < REL_TOL
    assert vec_rel_err(r1, rh) < REL_TOL


def test_device_structure_smaller_in_a_live_context(gb):
    """Device builds of a large mesh, then of a smaller one, in the same
    context: the host copies of the structure are sized by the current
    structure, not by the device buffers' grown capacity (the element tables
    land in an exactly-sized view of a guarded buffer, guards untouched), and
    equal a fresh context's."""
    from modfem_gb300.mesh import lognormal_k, structured_prism_mesh
    big, small = structured_prism_mesh(10, jitter=0.2, seed=5), structured_prism_mesh(4, jitter=0.2, seed=6)
    c = gb.Context(0)
    for m in (big, small):
        c.set_mesh(m)
        c.set_coefficients(k=lognormal_k(m.nel, seed=7), f=1.0, g=0.0, penalty=1e7)
        c.build_structure_device()
    ref = make_ctx(gb, small, lognormal_k(small.nel, seed=7))
    ref.build_structure_device()
    n = small.nel * (6 * 6 + 6)
    buf = np.full(n + 64, -7, np.int32)
    c._check(c.L.gbfem_get_element_tables(c._h, ctypes.c_void_p(buf[:n].ctypes.data)))
    assert np.all(buf[n:] == -7)
    assert np.array_equal(buf[:n], ref.get_element_tables())
    for a, b in zip(c.get_crs_structure(), ref.get_crs_structure()):
        assert np.array_equal(a, b)
    c.close()
    ref.close()
