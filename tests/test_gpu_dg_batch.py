"""GPU parity of the batched mixed-type DG volume kernel (persistent launch
over prism and tetrahedron tiles of degrees 1..4)."""
import numpy as np
import pytest

import oracle as O
from _util import REL_TOL, mat_rel_err, vec_rel_err

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gb():
    from modfem_gb300 import build
    build.build(verbose=False)
    import modfem_gb300
    return modfem_gb300


def _prisms(n, seed):
    from modfem_gb300.mesh import anisotropic_tensors, structured_prism_mesh
    m = structured_prism_mesh(n, jitter=0.2, seed=seed)
    D = anisotropic_tensors(m.nel, seed=seed).reshape(-1, 3, 3)
    p = np.random.default_rng(seed).integers(1, 5, m.nel).astype(np.int32)
    return m, D, p


def _tets(n, seed):
    from modfem_gb300.mesh import anisotropic_tensors, structured_tet_mesh
    t = structured_tet_mesh(n, jitter=0.2, seed=seed)
    D = anisotropic_tensors(t.nel, seed=seed + 1).reshape(-1, 3, 3)
    p = np.random.default_rng(seed + 2).integers(1, 5, t.nel).astype(np.int32)
    return t, D, p


def test_tets_vs_oracle(gb):
    t, D, p = _tets(2, 3)
    b = gb.Batch(0)
    b.set(np.zeros((0, 6, 3)), np.zeros((0, 3, 3)), np.zeros(0, np.int32), t.coords[t.el_nodes], D, p, f=1.7)
    b.run()
    mats, loads = b.blocks()
    for e in range(t.nel):
        Ko, Ro = O.dg_tet_element(t.coords[t.el_nodes[e]], D[e], int(p[e]), f=1.7)
        assert mat_rel_err(mats[e], Ko) < REL_TOL, (e, int(p[e]))
        assert vec_rel_err(loads[e], Ro) < REL_TOL


def test_tet_p1_equals_reference_linear_tet(gb):
    t, D, _ = _tets(2, 5)
    b = gb.Batch(0)
    b.set(np.zeros((0, 6, 3)), np.zeros((0, 3, 3)), np.zeros(0, np.int32), t.coords[t.el_nodes], D,
          np.ones(t.nel, np.int32), f=1.0)
    b.run()
    mats, loads = b.blocks()
    B = np.array([[1, -1, -1, -1], [0, 1, 0, 0], [0, 0, 1, 0], [0, 0, 0, 1]], float)
    for e in range(t.nel):
        Ks, Rs = O.std_tet_element(t.coords[t.el_nodes[e]], D[e])
        assert mat_rel_err(B @ mats[e] @ B.T, Ks) < REL_TOL
        assert vec_rel_err(B @ loads[e], Rs) < REL_TOL


def test_prisms_bitwise_equal_per_degree_kernel(gb):
    m, D, p = _prisms(3, 7)
    c = gb.Context(0)
    c.set_mesh(m)
    c.set_coefficients(D=D.reshape(-1, 9), f=1.0)
    c.dg_set_degrees(p)
    c.dg_build_structure()
    c.dg_assemble()
    off, bptr, bcol, boff = c.dg_get_structure()
    vals, rhs = c.dg_get_matrix()
    t, Dt, pt = _tets(1, 8)
    b = gb.Batch(0)
    b.set(m.coords[m.el_nodes], D, p, t.coords[t.el_nodes], Dt, pt, f=1.0)
    b.run()
    mats, loads = b.blocks()
    for e in range(m.nel):
        ns = off[e + 1] - off[e]
        K = vals[boff[bptr[e]]:boff[bptr[e]] + ns * ns].reshape(ns, ns).T
        assert np.array_equal(mats[e], K), e
        assert np.array_equal(loads[e], rhs[off[e]:off[e + 1]]), e
    for e in range(t.nel):
        Ko, Ro = O.dg_tet_element(t.coords[t.el_nodes[e]], Dt[e], int(pt[e]))
        assert mat_rel_err(mats[m.nel + e], Ko) < REL_TOL


def test_double_word_prisms_vs_fp64(gb):
    """Prism blocks of the batch with double-word stiffness sums against the
    FP64 batch (degrees 1..4, anisotropic tensors): within 1e-13 of each
    block's energy scale; loads and tetrahedra unchanged (FP64 in both);
    every prism variant within the same bound."""
    m, D, p = _prisms(3, 17)
    t, Dt, pt = _tets(1, 18)
    b = gb.Batch(0)
    b.set(m.coords[m.el_nodes], D, p, t.coords[t.el_nodes], Dt, pt, f=1.0)
    b.run()
    m64, l64 = b.blocks()
    b.set_arith(True)
    for pv in range(3):
        b.set_variants([0] + [pv] * 4, None)
        b.run()
        mdw, ldw = b.blocks()
        worst = max(mat_rel_err(mdw[e], m64[e]) for e in range(m.nel))
        assert worst < 1e-13, (pv, worst)
        for e in range(m.nel + t.nel):
            assert np.array_equal(ldw[e], l64[e])
        for e in range(m.nel, m.nel + t.nel):
            assert np.array_equal(mdw[e], m64[e])
    b.set_arith(False)
    b.run()
    mb, _ = b.blocks()
    assert all(np.array_equal(mb[e], m64[e]) for e in range(m.nel + t.nel))


def test_variants_and_replays_identical(gb):
    m, D, p = _prisms(2, 11)
    t, Dt, pt = _tets(3, 12)
    b = gb.Batch(0)
    b.set(m.coords[m.el_nodes], D, p, t.coords[t.el_nodes], Dt, pt, f=0.5)
    ref = None
    for pv in range(3):
        for tv in range(5):
            b.set_variants([0] + [pv] * 4, [0] + [tv] * 4)
            for _ in range(2):
                b.run()
                v, r = b.get()
                if ref is None:
                    ref = (v, r)
                assert np.array_equal(v, ref[0]) and np.array_equal(r, ref[1]), (pv, tv)
    pv, tv, ms = b.autotune(sample=64)
    assert all(0 <= pv[q] < 3 and 0 <= tv[q] < 5 for q in range(1, 5))
    assert (ms[0, 1:, :3] > 0).all() and (ms[1, 1:, :] > 0).all()
    b.run()
    v, r = b.get()
    assert np.array_equal(v, ref[0]) and np.array_equal(r, ref[1])


def test_layout_scatters_into_block_crs(gb):
    """Diagonal blocks of the prism mesh's block-CRS structure, then a
    second (tetrahedron) matrix appended after it."""
    m, D, p = _prisms(2, 13)
    c = gb.Context(0)
    c.set_mesh(m)
    c.set_coefficients(D=D.reshape(-1, 9), f=1.0)
    c.dg_set_degrees(p)
    nd, nv = c.dg_build_structure()
    off, bptr, bcol, boff = c.dg_get_structure()
    c.dg_assemble()
    vals, rhs = c.dg_get_matrix()
    t, Dt, pt = _tets(1, 14)
    diag = [boff[bptr[e] + int(np.nonzero(bcol[bptr[e]:bptr[e + 1]] == e)[0][0])] for e in range(m.nel)]
    tns = np.array([gb.TET_NS[int(q)] for q in pt])
    toff = nv + np.concatenate([[0], np.cumsum(tns * tns)[:-1]])
    troff = nd + np.concatenate([[0], np.cumsum(tns)[:-1]])
    b = gb.Batch(0)
    b.set(m.coords[m.el_nodes], D, p, t.coords[t.el_nodes], Dt, pt, f=1.0)
    NV, NR = nv + int((tns * tns).sum()), nd + int(tns.sum())
    b.set_layout(np.concatenate([diag, toff]), np.concatenate([off[:-1], troff]), NV, NR)
    b.run()
    v, r = b.get()
    isdiag = np.zeros(nv, bool)
    for e in range(m.nel):
        ns = off[e + 1] - off[e]
        isdiag[diag[e]:diag[e] + ns * ns] = True
    assert np.array_equal(v[:nv][isdiag], vals[isdiag])
    assert not v[:nv][~isdiag].any()
    assert np.array_equal(r[:nd], rhs)
    mats, loads = b.blocks()
    for e in range(t.nel):
        Ko, Ro = O.dg_tet_element(t.coords[t.el_nodes[e]], Dt[e], int(pt[e]))
        assert mat_rel_err(mats[m.nel + e], Ko) < REL_TOL
        assert vec_rel_err(loads[m.nel + e], Ro) < REL_TOL


def test_errors(gb):
    b = gb.Batch(0)
    with pytest.raises(gb.GbFemError):
        b.set(np.zeros((0, 6, 3)), np.zeros((0, 3, 3)), np.zeros(0, np.int32), np.zeros((0, 4, 3)),
              np.zeros((0, 3, 3)), np.zeros(0, np.int32))
    with pytest.raises(gb.GbFemError):
        b.set(np.zeros((1, 6, 3)), np.zeros((1, 3, 3)), np.array([5], np.int32), np.zeros((0, 4, 3)),
              np.zeros((0, 3, 3)), np.zeros(0, np.int32))
    with pytest.raises(gb.GbFemError):
        b.run()
