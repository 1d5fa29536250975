"""CPU checks of the DG tetrahedron oracle (no reference counterpart: the
reference's DG module is prism-only, so this restatement is pinned by the
reference's linear tetrahedron at p = 1 and by exact monomial moments)."""
from fractions import Fraction
from math import factorial

import numpy as np
import pytest

import oracle as O
from _util import REL_TOL, mat_rel_err, vec_rel_err


def _tet(seed):
    rng = np.random.default_rng(seed)
    X = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]], float) + rng.uniform(-0.2, 0.2, (4, 3))
    if np.linalg.det(np.stack([X[1] - X[0], X[2] - X[0], X[3] - X[0]], 1)) < 0:
        X[[2, 3]] = X[[3, 2]]
    from modfem_gb300.mesh import anisotropic_tensors
    return X, anisotropic_tensors(1, seed=seed).reshape(3, 3)


def test_basis_sizes():
    for p, ns in zip(range(1, 5), (4, 10, 20, 35)):
        E = O.tet_basis_exponents(p)
        assert len(E) == ns and len(set(E)) == ns and max(sum(e) for e in E) == p
        assert E[0] == (0, 0, 0) and E[1:4] == [(1, 0, 0), (0, 1, 0), (0, 0, 1)]


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_p1_equals_reference_linear_tet(seed):
    """span{1, xi, eta, zeta} is the linear space of the reference's std
    tetrahedron: with its hat functions N = B phi, K_std = B K_dg B^T."""
    X, A = _tet(seed)
    K, R = O.dg_tet_element(X, A, 1, f=1.3)
    Ks, Rs = O.std_tet_element(X, A, f=1.3)
    B = np.array([[1, -1, -1, -1], [0, 1, 0, 0], [0, 0, 1, 0], [0, 0, 0, 1]], float)
    assert mat_rel_err(B @ K @ B.T, Ks) < REL_TOL
    assert vec_rel_err(B @ R, Rs) < REL_TOL


def _exact(p, X, A, f):
    """Element matrix from the exact monomial moments a! b! c! / (a+b+c+3)!."""
    E = O.tet_basis_exponents(p)
    mom = lambda a, b, c: Fraction(factorial(a) * factorial(b) * factorial(c), factorial(a + b + c + 3))
    ns = len(E)
    S = np.zeros((3, 3, ns, ns))
    for a in range(3):
        for b in range(3):
            for i, ei in enumerate(E):
                for j, ej in enumerate(E):
                    if ei[a] == 0 or ej[b] == 0:
                        continue
                    ea, eb = list(ei), list(ej)
                    ea[a] -= 1
                    eb[b] -= 1
                    S[a, b, i, j] = float(ei[a] * ej[b] * mom(*(x + y for x, y in zip(ea, eb))))
    J = np.stack([X[1] - X[0], X[2] - X[0], X[3] - X[0]], 1)
    det = abs(np.linalg.det(J))
    Ji = np.linalg.inv(J)
    G = det * Ji @ A @ Ji.T
    K = np.einsum("ab,abij->ij", G, S)
    R = f * det * np.array([float(mom(*e)) for e in E])
    return K, R


@pytest.mark.parametrize("p", [1, 2, 3, 4])
def test_quadrature_matches_exact_moments(p):
    X, A = _tet(10 + p)
    K, R = O.dg_tet_element(X, A, p, f=0.7)
    Ke, Re = _exact(p, X, A, 0.7)
    assert mat_rel_err(K, Ke) < REL_TOL
    assert vec_rel_err(R, Re) < REL_TOL


@pytest.mark.parametrize("p", [2, 4])
def test_constant_and_linear_reproduction(p):
    X, A = _tet(20 + p)
    K, R = O.dg_tet_element(X, A, p)
    scale = np.abs(K).max()
    assert np.abs(K[:, 0]).max() < 1e-13 * scale  # grad of a constant
    vol = abs(np.linalg.det(np.stack([X[1] - X[0], X[2] - X[0], X[3] - X[0]], 1))) / 6.0
    assert abs(R[0] - vol) < 1e-14
    # u = x: coefficients x0 + J xi on (1, xi, eta, zeta); a(phi_w, u) = int grad phi_w . A e_x
    J = np.stack([X[1] - X[0], X[2] - X[0], X[3] - X[0]], 1)
    c = np.zeros(K.shape[0])
    c[0], c[1:4] = X[0, 0], J[0]
    lin = K @ c
    K1, _ = O.dg_tet_element(X, A, 1)
    assert np.allclose(lin[:4], K1 @ c[:4], rtol=0, atol=1e-13 * scale)


def _tet_system(n, seed, pmax=4):
    from modfem_gb300.mesh import anisotropic_tensors, structured_tet_mesh, tet_faces
    t = structured_tet_mesh(n, jitter=0.2, seed=seed)
    F = tet_faces(t)
    p = np.random.default_rng(seed).integers(1, pmax + 1, t.nel)
    A = anisotropic_tensors(t.nel, seed=seed + 1).reshape(-1, 3, 3)
    return t, F, p, A


def test_tet_face_table():
    from modfem_gb300.mesh import TET_SIDES, structured_tet_mesh, tet_faces
    n = 3
    t = structured_tet_mesh(n)
    F = tet_faces(t)
    assert F.n == (4 * t.nel + 12 * n * n) // 2           # every face twice but the 12 n^2 boundary ones
    assert int((F.el2 < 0).sum()) == 12 * n * n
    for k in range(F.n):                                     # nodes: el1's face, and el2's too
        assert sorted(F.nodes[k, :3]) == sorted(t.el_nodes[F.el1[k], list(TET_SIDES[F.side1[k]])])
        if F.el2[k] >= 0:
            assert set(F.nodes[k, :3]) <= set(t.el_nodes[F.el2[k]])


def test_tet_dg_oracle_reproduces_constants():
    """With f = 0 and Dirichlet value c the constant solves the interior-
    penalty system exactly (consistency of the face terms)."""
    t, F, p, A = _tet_system(2, 3)
    B, R = O.dg_tet_assemble(t, F, p, A, pen=10.0, g=0.7, f=0.0)
    ns = [(q + 1) * (q + 2) * (q + 3) // 6 for q in p]
    scale = max(np.abs(r).max() for r in R)
    for e in range(t.nel):
        acc = -R[e].copy()
        for (i, j), K in B.items():
            if i == e:
                x = np.zeros(ns[j])
                x[0] = 0.7
                acc += K @ x
        assert np.abs(acc).max() < 1e-12 * scale
