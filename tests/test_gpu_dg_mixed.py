"""GPU parity of DG systems on meshes of prisms and tetrahedra together
(gbfem_set_mesh_mixed): the assembled block system against the oracle
oracle.dg_mixed_assemble (parity unpinned: the reference's DG module is
prism-only; the oracle's prism-prism faces are the reference-pinned ones),
every volume and face kernel mode, constant reproduction at a larger size,
and block-Jacobi GMRES against a dense solve of the oracle's system."""
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


def _problem(n, layers, seed, pmax=4, aniso=True, jitter=0.2):
    from modfem_gb300.mesh import anisotropic_tensors, lognormal_k, mixed_faces, structured_mixed_mesh
    m = structured_mixed_mesh(n, layers, jitter=jitter, seed=seed)
    F = mixed_faces(m)
    p = np.random.default_rng(seed).integers(1, pmax + 1, m.nel)
    if aniso:
        A = anisotropic_tensors(m.nel, seed=seed + 1).reshape(-1, 9)
        k = None
    else:
        k = lognormal_k(m.nel, seed=seed + 1)
        A = None
    return m, F, p, A, k


def _context(gb, m, F, p, A, k, pen=10.0, g=0.3, f=1.2, vol=None, face=None):
    c = gb.Context(0)
    c.set_mesh_mixed(m)
    c.set_coefficients(k=k, D=A, f=f, g=g)
    c.dg_set_degrees(p)
    c.dg_set_faces(F, penalty=pen)
    if vol is not None:
        c.dg_set_volume_kernel(vol)
    if face is not None:
        c.dg_set_face_kernel(face)
    c.dg_build_structure()
    c.dg_assemble()
    return c


def _oracle_dense(m, F, p, A, k, pen=10.0, g=0.3, f=1.2):
    At = A if A is not None else k[:, None] * np.eye(3).reshape(1, 9)
    B, R = O.dg_mixed_assemble(m, F, p, At, pen=pen, g=g, f=f)
    ns = np.array([(O.DG_NS if m.el_nv[e] == 6 else O.DG_TET_NS)[int(p[e])] for e in range(m.nel)])
    off = np.concatenate([[0], np.cumsum(ns)])
    dense = np.zeros((off[-1], off[-1]))
    for (i, j), K in B.items():
        dense[off[i]:off[i + 1], off[j]:off[j + 1]] = K
    return dense, np.concatenate(R), off


def _crs(c):
    off, bptr, bcol, boff = c.dg_get_structure()
    vals, rhs = c.dg_get_matrix()
    rp, ci, v = dg_blocks_to_crs(off, bptr, bcol, boff, vals)
    return rp, ci, v, rhs, off


@pytest.mark.parametrize("aniso", [True, False])
def test_mixed_system_vs_oracle(gb, aniso):
    m, F, p, A, k = _problem(3, 1, 5, aniso=aniso)
    c = _context(gb, m, F, p, A, k)
    rp, ci, v, rhs, off = _crs(c)
    dense, R, ooff = _oracle_dense(m, F, p, A, k)
    assert np.array_equal(off, ooff)
    ref = dense[np.repeat(np.arange(off[-1]), np.diff(rp)), ci]
    assert np.count_nonzero(dense) <= ci.size  # the block pattern holds every oracle block
    err = sparse_rel_err(rp, ci, v, ref)
    print(f"mixed prism-tetrahedron DG system vs oracle {err:.2e}")
    assert err < REL_TOL
    assert vec_rel_err(rhs, R) < REL_TOL


@pytest.mark.parametrize("vol,face", [(0, 2), (1, 1), (3, 2), (4, 3)])
def test_mixed_kernel_modes_vs_oracle(gb, vol, face):
    """Tensor-core (split BF16) and double-word volume / face kernels on the
    prisms and tetrahedra of a mixed mesh; the prism-tetrahedron faces stay
    FP64 in every mode."""
    m, F, p, A, k = _problem(4, 2, 11)
    c = _context(gb, m, F, p, A, k, vol=vol, face=face)
    rp, ci, v, rhs, off = _crs(c)
    dense, R, _ = _oracle_dense(m, F, p, A, k)
    ref = dense[np.repeat(np.arange(off[-1]), np.diff(rp)), ci]
    err = sparse_rel_err(rp, ci, v, ref)
    print(f"mode vol={vol} face={face}: {err:.2e}")
    assert err < REL_TOL
    assert vec_rel_err(rhs, R) < REL_TOL


def test_mixed_mesh_of_prisms_only_is_the_prism_mesh(gb):
    """A mixed mesh whose elements are all prisms assembles bit-identically
    to the same mesh given as a prism mesh."""
    from modfem_gb300.mesh import MixedMesh, anisotropic_tensors, prism_faces, structured_prism_mesh
    pm = structured_prism_mesh(4, jitter=0.2, seed=3)
    F = prism_faces(pm)
    p = np.random.default_rng(3).integers(1, 5, pm.nel)
    A = anisotropic_tensors(pm.nel, seed=4).reshape(-1, 9)
    mm = MixedMesh(4, pm.coords, pm.el_nodes.astype(np.int32), np.full(pm.nel, 6, np.int32), 4)
    c1 = gb.Context(0)
    c1.set_mesh(pm)
    c2 = gb.Context(0)
    c2.set_mesh_mixed(mm)
    out = []
    for c in (c1, c2):
        c.set_coefficients(D=A, f=1.0, g=0.2)
        c.dg_set_degrees(p)
        c.dg_set_faces(F, penalty=10.0)
        c.dg_build_structure()
        c.dg_assemble()
        out.append(c.dg_get_matrix())
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])


@pytest.mark.parametrize("aniso", [True, False])
def test_mixed_constant_reproduction(gb, aniso):
    """f = 0 and Dirichlet value c: the constant c (the first function of
    every element) leaves a zero residual, on 12^3 hexahedra split into
    prisms (7 layers) and tetrahedra (5 layers)."""
    m, F, p, A, k = _problem(12, 7, 7, aniso=aniso)
    c = _context(gb, m, F, p, A, k, g=0.7, f=0.0)
    off = c.dg_get_structure()[0]
    x = np.zeros(off[-1])
    x[off[:-1]] = 0.7
    r = c.dg_compute_residual(x)
    vals, rhs = c.dg_get_matrix()
    assert np.max(np.abs(r)) < 1e-11 * np.max(np.abs(rhs))


def test_mixed_gmres_vs_dense_oracle(gb):
    m, F, p, A, k = _problem(3, 1, 9, pmax=3, aniso=False)
    c = _context(gb, m, F, p, A, k)
    x, it, res, rel = c.dg_solve(krylov=50, max_iter=20000, tol_rel=1e-12)
    assert rel < 1e-12 and it > 0
    dense, R, _ = _oracle_dense(m, F, p, A, k)
    xr = np.linalg.solve(dense, R)
    assert vec_rel_err(x, xr) < 1e-7
    x2, it2, outer, rel2 = c.dg_solve_ir(krylov=50, max_iter=20000, tol_rel=1e-12)
    assert rel2 < 1e-12
    assert vec_rel_err(x2, xr) < 1e-7


def test_mixed_mesh_refuses_std_path_and_bad_faces(gb):
    from modfem_gb300 import GbFemError
    from modfem_gb300.mesh import mixed_faces, structured_mixed_mesh
    m = structured_mixed_mesh(2, 1)
    c = gb.Context(0)
    c.set_mesh_mixed(m)
    with pytest.raises(GbFemError, match="DG path"):
        c.build_structure()
    F = mixed_faces(m)
    k = int(np.nonzero((F.el2 >= 0) & (m.el_nv[F.el1] != m.el_nv[np.maximum(F.el2, 0)]))[0][0])
    F.nodes = F.nodes.copy()
    F.nodes[k, 0] = int(np.setdiff1d(np.arange(m.coords.shape[0]), m.el_nodes[[F.el1[k], F.el2[k]]].ravel())[0])
    c.dg_set_degrees(np.ones(m.nel, np.int32))
    with pytest.raises(GbFemError, match="not a vertex"):
        c.dg_set_faces(F)
    bad = np.full(m.nel, 6, np.int32)
    bad[0] = 5
    from modfem_gb300.mesh import MixedMesh
    with pytest.raises(GbFemError, match="vertex count"):
        c.set_mesh_mixed(MixedMesh(2, m.coords, m.el_nodes, bad, 1))


def test_mixed_solves_double_word_operator_and_refinement(gb):
    """On a mixed mesh: GMRES with the double-word Arnoldi operator (block
    SpMV classes of both element types) and compensated-residual refinement,
    both against a dense solve of the oracle's system."""
    m, F, p, A, k = _problem(3, 1, 13, pmax=2, aniso=True)
    dense, R, _ = _oracle_dense(m, F, p, A, k)
    xr = np.linalg.solve(dense, R)
    c = _context(gb, m, F, p, A, k)
    c.set_option(gb.OPT_DG_SPMV_ARITH, gb.STD_DWORD)
    x, it, res, rel = c.dg_solve(krylov=50, max_iter=20000, tol_rel=1e-12)
    assert rel < 1e-12
    assert vec_rel_err(x, xr) < 1e-7
    c.set_option(gb.OPT_DG_RESIDUAL, gb.RESIDUAL_COMPENSATED)
    x2, it2, outer, rel2 = c.dg_solve_ir(krylov=50, max_iter=20000, tol_rel=1e-300)
    assert vec_rel_err(x2, xr) < 1e-9


def test_mixed_autotuned_shapes_are_bit_identical(gb):
    """The launch-shape autotuner on a mixed mesh (it times the prism
    kernels); every variant gives the same matrix bit for bit."""
    m, F, p, A, k = _problem(4, 2, 17)
    c = _context(gb, m, F, p, A, k)
    v0, r0 = c.dg_get_matrix()
    vol, face, ms = c.dg_autotune(sample=256)
    c.dg_assemble()
    v1, r1 = c.dg_get_matrix()
    assert np.array_equal(v0, v1) and np.array_equal(r0, r1)
    c.dg_set_variants(vol=[0, 1, 1, 1, 1], face=[0, 1, 1, 1, 1])
    c.dg_assemble()
    v2, r2 = c.dg_get_matrix()
    assert np.array_equal(v0, v2) and np.array_equal(r0, r2)
