"""The constraint rewrite for hanging vertices in the oracle
(oracle.std_constraint_rewrite, oracle.std_dropin_assemble) against the
reference itself: a jittered 9^3 x 2 prism mesh refined by the reference's
own apr_refine / apr_proj_dof_ref (two passes, generations up to 2), whose
sir_create lists and tables and apr_get_stiff_mat_data matrices are in
tests/golden/std_n9_hang.npz.  CPU only."""
import numpy as np

import oracle as O
from _util import RefinedMesh, load


def _case():
    g = load("std_n9_hang")
    return g, RefinedMesh(g)


def test_fixture_has_both_kinds_of_constraint():
    g, m = _case()
    assert set(np.unique(m.con_nr)) == {2, 4}
    assert int(g["max_dofs_int_ent"]) > 6
    # a hanging vertex carries no dof, its constraining vertices do
    assert np.all(g["dof_of_node"][m.con_vertex] < 0)
    par = m.con_par[m.con_par >= 0]
    assert np.all(g["dof_of_node"][par] >= 0)


def test_rewritten_local_matrices_match_reference():
    """Every element and boundary face whose dof list the reference expanded:
    the same list (constraining vertices in place of each hanging vertex)
    and the same rewritten matrix and load vector."""
    g, m = _case()
    off = offr = 0
    worst = 0.0
    for (t, i), n in zip(g["con_ent"], g["con_ns"]):
        Kg = g["con_sm"][off:off + n * n].reshape(n, n)
        Rg = g["con_rhs"][offr:offr + n]
        dg = g["con_dofs"][offr:offr + n]
        off += n * n
        offr += n
        if t == 4:
            e = int(i) - 1
            K, R = O.std_prism_element(m.coords[m.el_nodes[e]], g["k"][e] * np.eye(3))
        else:
            e, side = m.fa_of_id[int(i)]
            K, R = O.std_prism_face(m.coords[m.el_nodes[e]], side)
        Kc, Rc, ids = O.std_constraint_rewrite(K, R, m.el_nodes[e], g["con_cnt"], g["con_par"])
        assert np.array_equal(ids, dg), (t, i)
        worst = max(worst, np.max(np.abs(Kc - Kg)) / np.max(np.abs(Kg)))
        if np.any(Rg):
            worst = max(worst, np.max(np.abs(Rc - Rg)) / np.max(np.abs(Rg)))
        else:
            assert not np.any(Rc)
    assert worst < 1e-14


def test_assembled_system_matches_reference():
    """The table-driven assembly over the reference's entity lists with the
    rewrite: every CRS entry and rhs row within 1e-14 of the sum of the
    magnitudes of its contributions."""
    g, m = _case()
    args = (m.coords, m.el_nodes, g["k"], g["int_ent_type"], g["int_ent_id"], g["asse_pos"], g["assembly_table"],
            g["row_ptr"].size - 1, g["col_ind"].size, m.fa_of_id)
    kw = dict(con_cnt=g["con_cnt"], con_par=g["con_par"])
    val, rhs = O.std_dropin_assemble(*args, **kw)
    sv, sr = O.std_dropin_assemble(*args, absolute=True, **kw)
    assert np.max(np.abs(val - g["crs_val"]) / np.where(sv > 0, sv, 1.0)) < 1e-14
    assert np.max(np.abs(rhs - g["crs_rhs"]) / np.where(sr > 0, sr, 1.0)) < 1e-14


def test_planted_coefficient_mistake_is_caught(monkeypatch):
    """A planted mistake in the oracle: every constraining vertex taken with
    coefficient 1 (no interpolation) leaves the reference's numbers far
    behind, so the pin above does test the rewrite."""
    g, m = _case()
    expand = O.std_constraint_expand

    def wrong(nodes, con_cnt, con_par):
        src, coef, ids = expand(nodes, con_cnt, con_par)
        return src, np.ones_like(coef), ids

    monkeypatch.setattr(O, "std_constraint_expand", wrong)
    args = (m.coords, m.el_nodes, g["k"], g["int_ent_type"], g["int_ent_id"], g["asse_pos"], g["assembly_table"],
            g["row_ptr"].size - 1, g["col_ind"].size, m.fa_of_id)
    val, rhs = O.std_dropin_assemble(*args, con_cnt=g["con_cnt"], con_par=g["con_par"])
    assert np.max(np.abs(val - g["crs_val"])) > 1e-3 * np.max(np.abs(g["crs_val"]))


def test_table_blocks_follow_the_expanded_lists():
    """The reference's assembly table gives every entity a block of n x n + n
    positions, n its expanded dof count (an element's constrained vertices
    replaced by their constraining vertices; a boundary face takes its
    element's list): the sizes the drop-in derives from the constraint data
    for the table length and for each entity's block."""
    g, m = _case()
    pos = g["asse_pos"]
    sizes = np.diff(np.concatenate([pos, [g["assembly_table"].size]]))
    for i, (t, ent) in enumerate(zip(g["int_ent_type"], g["int_ent_id"])):
        e = int(ent) - 1 if t == 4 else m.fa_of_id[int(ent)][0]
        _, _, ids = O.std_constraint_expand(m.el_nodes[e], g["con_cnt"], g["con_par"])
        n = ids.size
        assert sizes[i] == n * n + n, (i, t, ent)
        # the rhs rows of the block are the dofs of the expanded list
        assert np.array_equal(g["assembly_table"][pos[i] + n * n:pos[i] + n * n + n], g["dof_of_node"][ids])
