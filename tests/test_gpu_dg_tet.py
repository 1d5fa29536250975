"""GPU DG tetrahedra as a full system: volume and interior-penalty face
integrals into the variable-block storage, block SpMV and GMRES (no
reference counterpart: the reference's DG module is prism-only; checked
against the numpy oracle oracle.dg_tet_assemble and by constant
reproduction)."""
import numpy as np
import pytest

import oracle as O
from _util import REL_TOL, dg_blocks_to_crs, sparse_rel_err, vec_rel_err

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gb():
    from modfem_gb300 import build
    build.build(verbose=False)
    import modfem_gb300
    return modfem_gb300


def _system(gb, n, seed, pmax=4, aniso=True, pen=10.0, g=0.3, f=1.2):
    from modfem_gb300.mesh import anisotropic_tensors, lognormal_k, structured_tet_mesh, tet_faces
    t = structured_tet_mesh(n, jitter=0.2, seed=seed)
    F = tet_faces(t)
    p = np.random.default_rng(seed).integers(1, pmax + 1, t.nel)
    A = anisotropic_tensors(t.nel, seed=seed + 1).reshape(-1, 9) if aniso else None
    k = None if aniso else lognormal_k(t.nel, seed=seed + 1)
    c = gb.Context(0)
    c.set_mesh(t)
    c.set_coefficients(k=k, D=A, f=f, g=g)
    c.dg_set_degrees(p)
    c.dg_set_faces(F, penalty=pen)
    c.dg_build_structure()
    c.dg_assemble()
    return c, t, F, p, (A if aniso else k[:, None] * np.eye(3).reshape(1, 9))


def test_tet_system_vs_oracle(gb):
    c, t, F, p, A = _system(gb, 2, 5)
    off, bptr, bcol, boff = c.dg_get_structure()
    vals, rhs = c.dg_get_matrix()
    rp, ci, v = dg_blocks_to_crs(off, bptr, bcol, boff, vals)
    B, R = O.dg_tet_assemble(t, F, p, A, pen=10.0, g=0.3, f=1.2)
    nd = off[-1]
    dense = np.zeros((nd, nd))
    for (i, j), K in B.items():
        dense[off[i]:off[i + 1], off[j]:off[j + 1]] = K
    ref = dense[np.repeat(np.arange(nd), np.diff(rp)), ci]
    assert np.count_nonzero(dense) <= ci.size  # the pattern holds every oracle block
    err = sparse_rel_err(rp, ci, v, ref)
    print(f"tetrahedral DG system vs oracle {err:.2e}")
    assert err < REL_TOL
    assert vec_rel_err(rhs, np.concatenate(R)) < REL_TOL


def test_tet_double_word_faces(gb):
    """Tetrahedral faces summed in double-word arithmetic: against the oracle
    to the FP64 tolerance and within 1e-13 of the FP64 face kernel (p 1..4,
    anisotropic tensors)."""
    c, t, F, p, A = _system(gb, 3, 9)
    off, bptr, bcol, boff = c.dg_get_structure()
    v64, r64 = c.dg_get_matrix()
    c.dg_set_face_kernel(gb.DG_FACE_DWORD)
    c.dg_assemble()
    vdw, rdw = c.dg_get_matrix()
    rp, ci, a64 = dg_blocks_to_crs(off, bptr, bcol, boff, v64)
    _, _, adw = dg_blocks_to_crs(off, bptr, bcol, boff, vdw)
    err = sparse_rel_err(rp, ci, adw, a64)
    print(f"tetrahedral double-word faces vs FP64 faces {err:.2e}")
    assert err < 1e-13
    assert vec_rel_err(rdw, r64) < 1e-13
    B, R = O.dg_tet_assemble(t, F, p, A, pen=10.0, g=0.3, f=1.2)
    nd = off[-1]
    dense = np.zeros((nd, nd))
    for (i, j), K in B.items():
        dense[off[i]:off[i + 1], off[j]:off[j + 1]] = K
    ref = dense[np.repeat(np.arange(nd), np.diff(rp)), ci]
    assert sparse_rel_err(rp, ci, adw, ref) < REL_TOL
    assert vec_rel_err(rdw, np.concatenate(R)) < REL_TOL


@pytest.mark.parametrize("n,aniso", [(4, True), (8, False)])
def test_tet_constant_reproduction(gb, n, aniso):
    c, t, F, p, A = _system(gb, n, 7, aniso=aniso, g=0.7, f=0.0)
    off = c.dg_get_structure()[0]
    x = np.zeros(off[-1])
    x[off[:-1]] = 0.7
    r = c.dg_compute_residual(x)
    vals, rhs = c.dg_get_matrix()
    assert np.max(np.abs(r)) < 1e-11 * np.max(np.abs(rhs))


def test_tet_gmres_and_residual(gb):
    c, t, F, p, A = _system(gb, 4, 9, pmax=2, aniso=False)
    x, it, res, rel = c.dg_solve(krylov=50, max_iter=20000, tol_rel=1e-10)
    r = c.dg_compute_residual(x)
    vals, rhs = c.dg_get_matrix()
    assert rel < 1e-10 and it > 0
    assert np.linalg.norm(r) < 1e-6 * np.linalg.norm(rhs)
    # the same system solved with iterative refinement
    x2, it2, outer, rel2 = c.dg_solve_ir(krylov=50, max_iter=20000, tol_rel=1e-11)
    assert rel2 < 1e-11
    assert np.linalg.norm(x2 - x) < 1e-5 * np.linalg.norm(x)
