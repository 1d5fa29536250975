"""The oracle of DG systems on meshes of prisms and tetrahedra together
(no reference counterpart: the reference's DG module is prism-only).

The face integral between a prism and a tetrahedron (oracle.dg_mixed_face)
is one generic routine: each side's local points from the face-vertex
weights and its own basis.  It is pinned here on the faces whose integrals
are pinned already: between two prisms against the reference-pinned
oracle.dg_face, between two tetrahedra against the tetrahedral oracle; and
the whole mixed system reproduces constants and, on affine meshes, linear
functions.
"""
import numpy as np
import pytest

import oracle as O
from modfem_gb300.mesh import (anisotropic_tensors, mixed_faces, prism_faces, structured_mixed_mesh,
                               structured_prism_mesh, structured_tet_mesh, tet_faces)


def _face_scale_err(a, b):
    R = np.abs(b).max(axis=1)
    C = np.abs(b).max(axis=0)
    return float(np.max(np.abs(a - b) / np.sqrt(np.outer(R, C))))


@pytest.mark.parametrize("p1,p2", [(1, 1), (2, 3), (3, 1), (4, 2)])
def test_generic_face_matches_pinned_prism_face(p1, p2):
    m = structured_prism_mesh(3, jitter=0.2, seed=2)
    F = prism_faces(m)
    D = anisotropic_tensors(m.nel, seed=2).reshape(-1, 9)
    nv = np.full(m.nel, 6, np.int32)
    k = next(i for i in range(F.n) if F.type[i] == 3 and F.el2[i] >= 0)  # an interior triangle
    e1, e2 = int(F.el1[k]), int(F.el2[k])
    pdeg = np.ones(m.nel, int)
    pdeg[e1], pdeg[e2] = p1, p2
    K, _ = O.dg_face(m, F, k, pdeg, D, pen=10.0)
    fb = O.dg_mixed_face(m.coords, m.el_nodes, nv, F, k, pdeg, D, pen=10.0)
    n1 = O.DG_NS[p1]
    G = np.block([[fb[(e1, e1)], fb[(e1, e2)]], [fb[(e2, e1)], fb[(e2, e2)]]])
    assert _face_scale_err(G, K) < 1e-12, (p1, p2)
    assert G.shape == K.shape and n1 < G.shape[0]


@pytest.mark.parametrize("p1,p2", [(1, 1), (2, 4), (3, 2)])
def test_generic_face_matches_tet_face(p1, p2):
    t = structured_tet_mesh(2, jitter=0.2, seed=4)
    F = tet_faces(t)
    D = anisotropic_tensors(t.nel, seed=4).reshape(-1, 9)
    el6 = np.full((t.nel, 6), -1, np.int32)
    el6[:, :4] = t.el_nodes
    nv = np.full(t.nel, 4, np.int32)
    k = next(i for i in range(F.n) if F.el2[i] >= 0)
    e1, e2 = int(F.el1[k]), int(F.el2[k])
    pdeg = np.ones(t.nel, int)
    pdeg[e1], pdeg[e2] = p1, p2
    X = t.coords[t.el_nodes]
    ref, _ = O._tet_face(X, D.reshape(-1, 3, 3), pdeg, t.coords[F.nodes[k, :3]], e1, e2, 10.0, 0.0)
    fb = O.dg_mixed_face(t.coords, el6, nv, F, k, pdeg, D, pen=10.0)
    for key in ref:
        # against the block's largest entry: complete-basis functions that
        # vanish on the face leave rows of rounding-level values
        assert np.max(np.abs(fb[key] - ref[key])) < 1e-13 * np.max(np.abs(ref[key])), key


def _system(m, F, pdeg, A, f=1.0, g=0.0):
    blocks, rhs = O.dg_mixed_assemble(m, F, pdeg, A, pen=10.0, g=g, f=f)
    ns = np.array([(O.DG_NS if m.el_nv[e] == 6 else O.DG_TET_NS)[int(pdeg[e])] for e in range(m.nel)])
    off = np.concatenate([[0], np.cumsum(ns)])
    K = np.zeros((off[-1], off[-1]))
    for (a, b), v in blocks.items():
        K[off[a]:off[a + 1], off[b]:off[b + 1]] = v
    return K, np.concatenate(rhs), off


def test_mixed_system_reproduces_constants():
    """f = 0 and Dirichlet value c: the constant c is the discrete solution
    (the constant is the first function of both bases)."""
    m = structured_mixed_mesh(3, 1, jitter=0.2, seed=5)
    F = mixed_faces(m)
    pdeg = np.random.default_rng(5).integers(1, 4, m.nel)
    D = anisotropic_tensors(m.nel, seed=5).reshape(-1, 9)
    K, b, off = _system(m, F, pdeg, D, f=0.0, g=0.7)
    x = np.zeros(off[-1])
    x[off[:-1]] = 0.7
    r = b - K @ x
    assert np.max(np.abs(r)) < 1e-12 * np.max(np.abs(b))


def test_mixed_system_consistent_for_linear_functions():
    """On an affine mixed mesh (no jitter) with A = I, every integrand is a
    polynomial the rules integrate exactly, so for a linear u the rows of the
    elements away from the boundary give B(u, v) = -int Laplace(u) v = 0: the
    interface faces between prisms and tetrahedra are consistent (normals,
    side signs, each side's local points)."""
    m = structured_mixed_mesh(4, 2, jitter=0.0)
    F = mixed_faces(m)
    pdeg = np.random.default_rng(6).integers(1, 4, m.nel)
    A = np.tile(np.eye(3).reshape(1, 9), (m.nel, 1))
    K, _, off = _system(m, F, pdeg, A, f=0.0)
    a, b0 = np.array([0.3, -1.1, 0.7]), 0.25
    x = np.zeros(off[-1])
    for e in range(m.nel):
        nv = int(m.el_nv[e])
        X = m.coords[m.el_nodes[e, :nv]]
        rng = np.random.default_rng(e)
        if nv == 6:
            loc = np.column_stack([rng.uniform(0, 0.5, 40), rng.uniform(0, 0.5, 40), rng.uniform(-1, 1, 40)])
        else:
            loc = rng.dirichlet(np.ones(4), 40)[:, 1:]
        phi, _ = O._basis_at_local(X, nv, int(pdeg[e]), loc)
        if nv == 6:
            xs = np.einsum("qi,ij->qj", O._prism_shape(loc), X)
        else:
            xs = X[0] + loc @ np.stack([X[1] - X[0], X[2] - X[0], X[3] - X[0]])
        x[off[e]:off[e + 1]] = np.linalg.lstsq(phi, xs @ a + b0, rcond=None)[0]
    r = K @ x
    interior = np.ones(m.nel, bool)
    interior[F.el1[F.el2 < 0]] = False
    rows = np.concatenate([np.arange(off[e], off[e + 1]) for e in range(m.nel) if interior[e]])
    mixed_rows = [e for e in range(m.nel) if interior[e] and any(
        (F.el1[i] == e or F.el2[i] == e) and F.el2[i] >= 0 and m.el_nv[F.el1[i]] != m.el_nv[F.el2[i]]
        for i in range(F.n))]
    assert len(mixed_rows) > 0
    assert np.max(np.abs(r[rows])) < 1e-11 * np.max(np.abs(K))


def _faces_by_loop(mesh):
    """The face table by a plain loop over element sides (the definition
    mixed_faces vectorises)."""
    from modfem_gb300.mesh import PRISM_SIDES, TET_SIDES
    rows = []
    for e in range(mesh.nel):
        sides = PRISM_SIDES if mesh.el_nv[e] == 6 else TET_SIDES
        for s, loc in enumerate(sides):
            verts = [int(mesh.el_nodes[e, i]) for i in loc]
            rows.append((tuple(sorted(verts)), e, s, verts))
    rows.sort(key=lambda r: (r[0], r[1]))
    out, i = [], 0
    while i < len(rows):
        key, e1, s1, verts = rows[i]
        if i + 1 < len(rows) and rows[i + 1][0] == key:
            e2, s2 = rows[i + 1][1], rows[i + 1][2]
            i += 2
        else:
            e2, s2 = -1, 0
            i += 1
        out.append((e1, s1, e2, s2, len(verts), verts + [-1] * (4 - len(verts))))
    out.sort(key=lambda r: (r[0], r[1]))
    return out


@pytest.mark.parametrize("n,layers", [(2, 1), (4, 3)])
def test_mixed_faces_matches_loop_definition(n, layers):
    m = structured_mixed_mesh(n, layers, jitter=0.1, seed=1)
    F = mixed_faces(m)
    ref = _faces_by_loop(m)
    assert F.n == len(ref)
    for k, (e1, s1, e2, s2, t, v) in enumerate(ref):
        assert (F.el1[k], F.side1[k], F.el2[k], F.side2[k], F.type[k]) == (e1, s1, e2, s2, t)
        assert list(F.nodes[k]) == v
        assert F.bc[k] == (-1 if e2 >= 0 else 1)
    # interface triangles between the two element types exist
    assert np.any((F.el2 >= 0) & (m.el_nv[F.el1] != m.el_nv[np.maximum(F.el2, 0)]))
