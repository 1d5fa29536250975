"""GPU parity of the whole DG system: volume and face integrals assembled
into the variable-block storage, the block residual and block-Jacobi GMRES,
against the reference's assembled lad_block matrices and solutions and the
oracle."""
import numpy as np
import pytest

import oracle as O
from _util import REL_TOL, dg_blocks_to_crs, load, sparse_rel_err, vec_rel_err

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gb():
    from modfem_gb300 import build
    build.build(verbose=False)
    import modfem_gb300
    return modfem_gb300


def _tensors(g):
    return g["D"].reshape(-1, 9) if g["D"].size else None


def _context(gb, m, F, pdeg, k=None, D=None, pen=10.0, g=0.0, f=1.0):
    c = gb.Context(0)
    c.set_mesh(m)
    c.set_coefficients(k=k, D=D, f=f, g=g)
    c.dg_set_degrees(pdeg)
    c.dg_set_faces(F, penalty=pen)
    c.dg_build_structure()
    return c


def _expand(c):
    off, bptr, bcol, boff = c.dg_get_structure()
    vals, rhs = c.dg_get_matrix()
    rp, ci, v = dg_blocks_to_crs(off, bptr, bcol, boff, vals)
    return rp, ci, v, rhs, off


def _fixture_problem(name):
    from modfem_gb300.mesh import prism_faces, structured_prism_mesh
    g = load(name)
    m = structured_prism_mesh(int(g["n"]), jitter=float(g["jitter"]), seed=int(g["seed"]))
    assert np.array_equal(m.coords, g["coords"])
    return g, m, prism_faces(m)


@pytest.mark.parametrize("name", ["dg_asm_p2", "dg_asm_mixed", "dg_asm_aniso"])
def test_dg_system_vs_reference(gb, name):
    g, m, F = _fixture_problem(name)
    D = _tensors(g)
    c = _context(gb, m, F, g["pdeg"], k=None if D is not None else g["k"], D=D, pen=float(g["pen"]),
                 g=float(g["g"]), f=float(g["f"]))
    c.dg_assemble()
    rp, ci, v, rhs, off = _expand(c)
    # dof order and block pattern identical to the reference's block storage
    assert np.array_equal(off[:-1], g["dof_posglob"])
    assert np.array_equal(rp, g["row_ptr"]) and np.array_equal(ci, g["col_ind"])
    assert sparse_rel_err(rp, ci, v, g["val"]) < REL_TOL
    assert vec_rel_err(rhs, g["rhs"]) < REL_TOL


@pytest.mark.parametrize("name", ["dg_asm_p2", "dg_asm_mixed", "dg_asm_aniso"])
def test_dg_gmres_vs_reference(gb, name):
    """GMRES(50) with block Jacobi to 1e-10 on the reference's problem: the
    iteration count of lsr_mkb_core_gmres within 2, the solution within the
    accuracy the stopping test guarantees."""
    g, m, F = _fixture_problem(name)
    D = _tensors(g)
    c = _context(gb, m, F, g["pdeg"], k=None if D is not None else g["k"], D=D, pen=float(g["pen"]),
                 g=float(g["g"]), f=float(g["f"]))
    c.dg_assemble()
    x, it, res, rel = c.dg_solve(krylov=int(g["krylov"]), max_iter=5000, tol_rel=float(g["tol"]))
    assert abs(it - int(g["gmres_iters"])) <= 2, (it, int(g["gmres_iters"]))
    assert rel < float(g["tol"])
    assert vec_rel_err(x, g["gmres_x"]) < 1e-7


@pytest.mark.parametrize("name", ["dg_asm_p2", "dg_asm_mixed", "dg_asm_aniso"])
def test_dg_gmres_double_word_operator_vs_reference(gb, name):
    """GMRES with the Arnoldi products on double-word copies of the matrix
    and the block-Jacobi inverse: the reference's iteration count within 2 and
    its solution to the same accuracy as the FP64 operator."""
    g, m, F = _fixture_problem(name)
    D = _tensors(g)
    c = _context(gb, m, F, g["pdeg"], k=None if D is not None else g["k"], D=D, pen=float(g["pen"]),
                 g=float(g["g"]), f=float(g["f"]))
    c.dg_assemble()
    c.set_option(gb.OPT_DG_SPMV_ARITH, gb.STD_DWORD)
    x, it, res, rel = c.dg_solve(krylov=int(g["krylov"]), max_iter=5000, tol_rel=float(g["tol"]))
    assert abs(it - int(g["gmres_iters"])) <= 2, (it, int(g["gmres_iters"]))
    assert rel < float(g["tol"])
    assert vec_rel_err(x, g["gmres_x"]) < 1e-7
    # the FP64 operator on the same problem: iteration counts within one,
    # solutions as close as the stopping test allows (different rounding,
    # different iterates: about cond x tol)
    c.set_option(gb.OPT_DG_SPMV_ARITH, gb.STD_FP64)
    x64, it64, _, _ = c.dg_solve(krylov=int(g["krylov"]), max_iter=5000, tol_rel=float(g["tol"]))
    assert abs(it - it64) <= 1
    assert vec_rel_err(x, x64) < 1e-7


def test_dg_residual_vs_numpy(gb):
    g, m, F = _fixture_problem("dg_asm_mixed")
    c = _context(gb, m, F, g["pdeg"], k=g["k"], pen=float(g["pen"]), g=float(g["g"]))
    c.dg_assemble()
    rp, ci, v, rhs, off = _expand(c)
    x = np.sin(np.arange(off[-1]) * 0.37)
    rows = np.repeat(np.arange(off[-1]), np.diff(rp))
    ax = np.zeros(off[-1])
    np.add.at(ax, rows, v * x[ci])
    r = c.dg_compute_residual(x)
    assert vec_rel_err(r, rhs - ax) < 1e-13
    r0 = c.dg_compute_residual(x, use_rhs=0)
    assert vec_rel_err(r0, -ax) < 1e-13


@pytest.mark.parametrize("aniso", [False, True])
def test_dg_system_vs_oracle_larger(gb, aniso):
    """n = 4 (128 prisms, 416 faces), mixed p = 1..4, against the oracle's
    assembly of the same problem."""
    from modfem_gb300.mesh import anisotropic_tensors, lognormal_k, prism_faces, structured_prism_mesh
    m = structured_prism_mesh(4, jitter=0.2, seed=9)
    F = prism_faces(m)
    pdeg = np.random.default_rng(9).integers(1, 5, m.nel)
    k = lognormal_k(m.nel, seed=9)
    D = anisotropic_tensors(m.nel, seed=9).reshape(m.nel, 9) if aniso else None
    A = D if aniso else np.array([np.diag([kk] * 3).reshape(-1) for kk in k])
    c = _context(gb, m, F, pdeg, k=None if aniso else k, D=D, pen=7.5, g=0.4, f=1.3)
    c.dg_assemble()
    rp, ci, v, rhs, off = _expand(c)
    rpo, cio, vo, rhso, offo = O.dg_assemble(m, F, pdeg, A, pen=7.5, g=0.4, f=1.3)
    assert np.array_equal(rp, rpo) and np.array_equal(ci, cio)
    assert sparse_rel_err(rp, ci, v, vo) < REL_TOL
    assert vec_rel_err(rhs, rhso) < REL_TOL


def test_dg_assembly_deterministic(gb):
    """Every block entry is written by one thread in a fixed order: two
    assemblies are bit-identical."""
    from modfem_gb300.mesh import lognormal_k, prism_faces, structured_prism_mesh
    m = structured_prism_mesh(6, jitter=0.2, seed=4)
    F = prism_faces(m)
    pdeg = np.random.default_rng(4).integers(1, 5, m.nel)
    c = _context(gb, m, F, pdeg, k=lognormal_k(m.nel, seed=4), g=0.2)
    c.dg_assemble()
    v1, r1 = c.dg_get_matrix()
    c.dg_assemble()
    v2, r2 = c.dg_get_matrix()
    assert np.array_equal(v1, v2) and np.array_equal(r1, r2)


@pytest.mark.parametrize("n,pmax", [(12, 4), (40, 2)])
def test_dg_constant_reproduction_full_size(gb, n, pmax):
    """Size-independent property of the interior-penalty system: with f = 0
    and Dirichlet value c the constant function (coefficient c on each
    element's first monomial, 1) satisfies A x = b exactly, so the block
    residual vanishes to rounding.  Exercises every volume and face block at
    sizes the oracle cannot check entry by entry."""
    from modfem_gb300.mesh import lognormal_k, prism_faces, structured_prism_mesh
    m = structured_prism_mesh(n, jitter=0.2, seed=n)
    F = prism_faces(m)
    pdeg = np.random.default_rng(n).integers(1, pmax + 1, m.nel)
    cval = 0.7
    c = _context(gb, m, F, pdeg, k=lognormal_k(m.nel, seed=n), g=cval, f=0.0)
    c.dg_assemble()
    off = c.dg_get_structure()[0]
    x = np.zeros(off[-1])
    x[off[:-1]] = cval
    r = c.dg_compute_residual(x)
    vals, rhs = c.dg_get_matrix()
    assert np.max(np.abs(r)) < 1e-11 * np.max(np.abs(rhs))


@pytest.mark.parametrize("name", ["dg_asm_p2", "dg_asm_aniso"])
def test_dg_tensor_core_volume_vs_reference(gb, name):
    """The tensor-core volume kernel (split BF16 products, FP64 recombination)
    gives the reference's system to the same FP64 tolerance (p = 4 elements of
    the mixed mesh stay on the FP64 kernel)."""
    g, m, F = _fixture_problem(name)
    D = _tensors(g)
    c = _context(gb, m, F, g["pdeg"], k=None if D is not None else g["k"], D=D, pen=float(g["pen"]),
                 g=float(g["g"]), f=float(g["f"]))
    c.dg_set_volume_kernel(gb.DG_VOLUME_TC)
    c.dg_assemble()
    rp, ci, v, rhs, off = _expand(c)
    assert np.array_equal(rp, g["row_ptr"]) and np.array_equal(ci, g["col_ind"])
    assert sparse_rel_err(rp, ci, v, g["val"]) < REL_TOL
    assert vec_rel_err(rhs, g["rhs"]) < REL_TOL


@pytest.mark.parametrize("name", ["dg_asm_p2", "dg_asm_mixed", "dg_asm_aniso"])
def test_dg_tensor_core_faces_vs_reference(gb, name):
    """The tensor-core face kernel (and volume kernel) give the reference's
    assembled system to the FP64 tolerance; owners with a degree-4 neighbour
    stay on the FP64 face kernel."""
    g, m, F = _fixture_problem(name)
    D = _tensors(g)
    c = _context(gb, m, F, g["pdeg"], k=None if D is not None else g["k"], D=D, pen=float(g["pen"]),
                 g=float(g["g"]), f=float(g["f"]))
    c.dg_set_volume_kernel(gb.DG_VOLUME_TC)
    c.dg_set_face_kernel(gb.DG_FACE_TC)
    c.dg_assemble()
    rp, ci, v, rhs, off = _expand(c)
    assert np.array_equal(rp, g["row_ptr"]) and np.array_equal(ci, g["col_ind"])
    err = sparse_rel_err(rp, ci, v, g["val"])
    print(f"{name}: tensor-core faces vs reference {err:.2e}")
    assert err < REL_TOL
    assert vec_rel_err(rhs, g["rhs"]) < REL_TOL


@pytest.mark.parametrize("n,pmax,aniso", [(6, 1, False), (6, 2, True), (7, 3, True), (8, 3, False), (8, 4, False)])
def test_dg_tensor_core_faces_vs_fp64_kernel(gb, n, pmax, aniso):
    """Whole block matrix with tensor-core faces against the FP64 face kernel
    on jittered meshes larger than the fixtures (uniform and mixed degrees,
    isotropic lognormal and anisotropic tensors)."""
    from modfem_gb300.mesh import anisotropic_tensors, lognormal_k, prism_faces, structured_prism_mesh
    m = structured_prism_mesh(n, jitter=0.2, seed=n + pmax)
    F = prism_faces(m)
    rng = np.random.default_rng(n)
    pdeg = np.full(m.nel, pmax) if n % 2 else rng.integers(1, pmax + 1, m.nel)
    kw = {"D": anisotropic_tensors(m.nel, seed=n).reshape(m.nel, 9)} if aniso else {"k": lognormal_k(m.nel, seed=n)}
    out = []
    for mode in (gb.DG_FACE_FP64, gb.DG_FACE_TC):
        c = _context(gb, m, F, pdeg, g=0.3, f=1.0, **kw)
        c.dg_set_face_kernel(mode)
        c.dg_assemble()
        out.append(_expand(c))
        c.close()
    (rp, ci, v64, r64, _), (rp2, ci2, vtc, rtc, _) = out
    assert np.array_equal(rp, rp2) and np.array_equal(ci, ci2)
    err = sparse_rel_err(rp, ci, vtc, v64)
    print(f"n={n} pmax={pmax}: tensor-core faces vs FP64 faces {err:.2e}")
    assert err < REL_TOL
    assert vec_rel_err(rtc, r64) < REL_TOL


def test_dg_tensor_core_faces_constant_reproduction(gb):
    """With f = 0 and Dirichlet value c, the constant is an exact discrete
    solution of the system the tensor-core kernels assemble."""
    from modfem_gb300.mesh import lognormal_k, prism_faces, structured_prism_mesh
    m = structured_prism_mesh(16, jitter=0.2, seed=3)
    F = prism_faces(m)
    pdeg = np.random.default_rng(3).integers(1, 4, m.nel)
    c = _context(gb, m, F, pdeg, k=lognormal_k(m.nel, seed=3), g=0.7, f=0.0)
    c.dg_set_volume_kernel(gb.DG_VOLUME_TC)
    c.dg_set_face_kernel(gb.DG_FACE_TC)
    c.dg_assemble()
    off = c.dg_get_structure()[0]
    x = np.zeros(off[-1])
    x[off[:-1]] = 0.7
    r = c.dg_compute_residual(x)
    vals, rhs = c.dg_get_matrix()
    assert np.max(np.abs(r)) < 1e-11 * np.max(np.abs(rhs))


@pytest.mark.parametrize("name", ["dg_asm_p2", "dg_asm_mixed", "dg_asm_aniso"])
def test_dg_double_word_faces_vs_reference(gb, name):
    """Face integrals summed in double-word arithmetic give the reference's
    assembled system to the FP64 tolerance (all degrees, p = 4 included)."""
    g, m, F = _fixture_problem(name)
    D = _tensors(g)
    c = _context(gb, m, F, g["pdeg"], k=None if D is not None else g["k"], D=D, pen=float(g["pen"]),
                 g=float(g["g"]), f=float(g["f"]))
    c.dg_set_face_kernel(gb.DG_FACE_DWORD)
    c.dg_assemble()
    rp, ci, v, rhs, off = _expand(c)
    assert np.array_equal(rp, g["row_ptr"]) and np.array_equal(ci, g["col_ind"])
    err = sparse_rel_err(rp, ci, v, g["val"])
    print(f"{name}: double-word faces vs reference {err:.2e}")
    assert err < REL_TOL
    assert vec_rel_err(rhs, g["rhs"]) < REL_TOL


@pytest.mark.parametrize("tc", [False, True])
@pytest.mark.parametrize("n,pmax,aniso", [(6, 1, False), (6, 2, True), (7, 3, True), (8, 4, False), (7, 4, True)])
def test_dg_double_word_faces_vs_fp64_kernel(gb, n, pmax, aniso, tc):
    """Whole block matrix with double-word faces (alone, or behind the tensor
    cores for the owners they do not cover) against the FP64 face kernel
    (uniform and mixed degrees up to 4, isotropic and anisotropic), within
    1e-13 of the FP64 kernel's own entries."""
    from modfem_gb300.mesh import anisotropic_tensors, lognormal_k, prism_faces, structured_prism_mesh
    m = structured_prism_mesh(n, jitter=0.2, seed=n + pmax)
    F = prism_faces(m)
    rng = np.random.default_rng(n)
    pdeg = np.full(m.nel, pmax) if n % 2 else rng.integers(1, pmax + 1, m.nel)
    kw = {"D": anisotropic_tensors(m.nel, seed=n).reshape(m.nel, 9)} if aniso else {"k": lognormal_k(m.nel, seed=n)}
    out = []
    for mode in (gb.DG_FACE_FP64, gb.DG_FACE_TC_DWORD if tc else gb.DG_FACE_DWORD):
        c = _context(gb, m, F, pdeg, g=0.3, f=1.0, **kw)
        c.dg_set_face_kernel(mode)
        c.dg_assemble()
        out.append(_expand(c))
        c.close()
    (rp, ci, v64, r64, _), (rp2, ci2, vdw, rdw, _) = out
    assert np.array_equal(rp, rp2) and np.array_equal(ci, ci2)
    err = sparse_rel_err(rp, ci, vdw, v64)
    print(f"n={n} pmax={pmax}: double-word faces vs FP64 faces {err:.2e}")
    assert err < 1e-13
    assert vec_rel_err(rdw, r64) < 1e-13


def test_dg_double_word_faces_constant_reproduction(gb):
    """With f = 0 and Dirichlet value c, the constant solves the system with
    double-word faces (p 1..4)."""
    from modfem_gb300.mesh import lognormal_k, prism_faces, structured_prism_mesh
    m = structured_prism_mesh(14, jitter=0.2, seed=4)
    F = prism_faces(m)
    pdeg = np.random.default_rng(4).integers(1, 5, m.nel)
    c = _context(gb, m, F, pdeg, k=lognormal_k(m.nel, seed=4), g=0.7, f=0.0)
    c.dg_set_face_kernel(gb.DG_FACE_DWORD)
    c.dg_assemble()
    off = c.dg_get_structure()[0]
    x = np.zeros(off[-1])
    x[off[:-1]] = 0.7
    r = c.dg_compute_residual(x)
    vals, rhs = c.dg_get_matrix()
    assert np.max(np.abs(r)) < 1e-11 * np.max(np.abs(rhs))


@pytest.mark.parametrize("name", ["dg_asm_p2", "dg_asm_mixed", "dg_asm_aniso"])
def test_dg_double_word_assembly_vs_reference(gb, name):
    """Volume and face entries summed in double-word arithmetic give the
    reference's assembled system to the FP64 tolerance; likewise the tensor
    cores with double words behind them."""
    g, m, F = _fixture_problem(name)
    D = _tensors(g)
    for vmode, fmode in ((gb.DG_VOLUME_DWORD, gb.DG_FACE_DWORD), (gb.DG_VOLUME_TC_DWORD, gb.DG_FACE_TC_DWORD)):
        c = _context(gb, m, F, g["pdeg"], k=None if D is not None else g["k"], D=D, pen=float(g["pen"]),
                     g=float(g["g"]), f=float(g["f"]))
        c.dg_set_volume_kernel(vmode)
        c.dg_set_face_kernel(fmode)
        c.dg_assemble()
        rp, ci, v, rhs, off = _expand(c)
        assert np.array_equal(rp, g["row_ptr"]) and np.array_equal(ci, g["col_ind"])
        err = sparse_rel_err(rp, ci, v, g["val"])
        print(f"{name} modes {vmode}/{fmode}: vs reference {err:.2e}")
        assert err < REL_TOL
        assert vec_rel_err(rhs, g["rhs"]) < REL_TOL
        c.close()


@pytest.mark.parametrize("p", [1, 2, 3, 4])
def test_dg_double_word_volume_vs_fp64_kernel(gb, p):
    """Element blocks summed in double-word arithmetic against the FP64
    volume kernel (jittered anisotropic mesh, every degree): within 1e-13 of
    the FP64 blocks (energy scale of each block)."""
    from modfem_gb300.mesh import anisotropic_tensors, structured_prism_mesh
    m = structured_prism_mesh(7, jitter=0.2, seed=20 + p)
    D = anisotropic_tensors(m.nel, seed=p).reshape(m.nel, 9)
    out = []
    for mode in (gb.DG_VOLUME_FP64, gb.DG_VOLUME_DWORD):
        c = gb.Context(0)
        c.set_mesh(m)
        c.set_coefficients(D=D, f=1.0, g=0.0)
        c.dg_set_degrees(np.full(m.nel, p))
        c.dg_build_structure()
        c.dg_set_volume_kernel(mode)
        c.dg_assemble()
        out.append(c.dg_get_matrix())
        off, bptr, bcol, boff = c.dg_get_structure()
        c.close()
    from _util import mat_rel_err
    ns = [0, 6, 18, 40, 75][p]
    worst = 0.0
    for e in range(m.nel):
        K64 = out[0][0][boff[e]:boff[e] + ns * ns].reshape(ns, ns)
        Kdw = out[1][0][boff[e]:boff[e] + ns * ns].reshape(ns, ns)
        worst = max(worst, mat_rel_err(Kdw, K64))
    print(f"p={p}: double-word volume vs FP64 {worst:.2e}")
    assert worst < 1e-13, worst
    assert np.array_equal(out[1][1], out[0][1])  # the load vector is the FP64 kernel's


@pytest.mark.parametrize("p", [1, 2, 3])
def test_dg_tensor_core_volume_vs_fp64_kernel(gb, p):
    """Element blocks of the tensor-core kernel against the FP64 kernel on a
    jittered anisotropic mesh with more elements than one CTA batch."""
    from modfem_gb300.mesh import anisotropic_tensors, structured_prism_mesh
    m = structured_prism_mesh(5, jitter=0.25, seed=p + 40)
    D = anisotropic_tensors(m.nel, seed=p + 40).reshape(m.nel, 9)
    out = []
    for mode in (gb.DG_VOLUME_FP64, gb.DG_VOLUME_TC):
        c = gb.Context(0)
        c.set_mesh(m)
        c.set_coefficients(D=D, f=1.3)
        c.dg_set_degrees(np.full(m.nel, p))
        c.dg_build_structure()
        c.dg_set_volume_kernel(mode)
        c.dg_assemble()
        out.append(c.dg_get_matrix())
        off, bptr, bcol, boff = c.dg_get_structure()
        c.close()
    from _util import mat_rel_err
    ns = [0, 6, 18, 40, 75][p]
    worst = 0.0
    for e in range(m.nel):
        K64 = out[0][0][boff[e]:boff[e] + ns * ns].reshape(ns, ns)
        Ktc = out[1][0][boff[e]:boff[e] + ns * ns].reshape(ns, ns)
        worst = max(worst, mat_rel_err(Ktc, K64))
    assert worst < 1e-13, worst
    assert vec_rel_err(out[1][1], out[0][1]) < 1e-14


@pytest.mark.parametrize("p", [1, 2, 3])
def test_dg_tf32_volume_vs_fp64_kernel(gb, p):
    """TF32 hi/lo tensor-core contraction with FP32 accumulation: an
    approximate element matrix, within 5e-5 of the FP64 kernel's in the
    entry-scale measure (and not bit-equal: it is a different precision);
    the load vector stays FP64."""
    from modfem_gb300.mesh import anisotropic_tensors, structured_prism_mesh
    m = structured_prism_mesh(5, jitter=0.25, seed=p + 50)
    D = anisotropic_tensors(m.nel, seed=p + 50).reshape(m.nel, 9)
    out = []
    for mode in (gb.DG_VOLUME_FP64, gb.DG_VOLUME_TF32):
        c = gb.Context(0)
        c.set_mesh(m)
        c.set_coefficients(D=D, f=1.3)
        c.dg_set_degrees(np.full(m.nel, p))
        c.dg_build_structure()
        c.dg_set_volume_kernel(mode)
        c.dg_assemble()
        out.append(c.dg_get_matrix())
        off, bptr, bcol, boff = c.dg_get_structure()
        c.close()
    from _util import mat_rel_err
    ns = [0, 6, 18, 40, 75][p]
    worst = 0.0
    for e in range(m.nel):
        K64 = out[0][0][boff[e]:boff[e] + ns * ns].reshape(ns, ns)
        Ktf = out[1][0][boff[e]:boff[e] + ns * ns].reshape(ns, ns)
        worst = max(worst, mat_rel_err(Ktf, K64))
    print(f"TF32 p={p}: worst energy-scale deviation {worst:.3e}")
    assert 0.0 < worst < 5e-5, worst  # measured 1.3e-6 / 3.5e-6 / 8.9e-6 for p = 1 / 2 / 3
    assert vec_rel_err(out[1][1], out[0][1]) < 1e-14


@pytest.mark.parametrize("name", ["dg_asm_mixed", "dg_asm_aniso"])
def test_dg_iterative_refinement_vs_reference(gb, name):
    """Mixed precision (FP64 refinement around FP32-operator GMRES) drives the
    true relative residual to 1e-13; its solution then agrees with a dense
    direct solve of the same system to the accuracy the conditioning allows
    and with the reference's (which stopped at 1e-10 on the preconditioned
    residual, so is accurate to ~1e-7) to 1e-6."""
    g, m, F = _fixture_problem(name)
    D = _tensors(g)
    c = _context(gb, m, F, g["pdeg"], k=None if D is not None else g["k"], D=D, pen=float(g["pen"]),
                 g=float(g["g"]), f=float(g["f"]))
    c.dg_assemble()
    x, inner, outer, rel = c.dg_solve_ir(krylov=50, max_iter=20000, tol_rel=1e-13, inner_tol=1e-6)
    assert rel <= 1e-13 and outer >= 2
    r = c.dg_compute_residual(x)
    assert np.linalg.norm(r) <= 1.01e-13 * np.linalg.norm(c.dg_get_matrix()[1])
    # dense direct solve of the same (small) system as the exact answer
    rp, ci, v, rhs, off = _expand(c)
    A = np.zeros((off[-1], off[-1]))
    A[np.repeat(np.arange(off[-1]), np.diff(rp)), ci] = v
    xd = np.linalg.solve(A, rhs)
    # condition number ~1e5 (penalty-dominated, mixed degree): a 1e-13 true
    # residual bounds the solution error by ~1e-8
    assert vec_rel_err(x, xd) < 1e-7
    assert vec_rel_err(x, g["gmres_x"]) < 1e-6


def _p3_aniso_form(n, seed=44):
    """The p = 3 anisotropic DG problem (432k prisms at full size) at a
    small size: DG p = 3 prisms on a
    jittered n^3 x 2 mesh, the anisotropic tensor R diag(1, 0.1, 0.01) R^T per
    element, Dirichlet value 0.3."""
    from modfem_gb300.mesh import anisotropic_tensors, prism_faces, structured_prism_mesh
    m = structured_prism_mesh(n, jitter=0.2, seed=seed)
    return m, prism_faces(m), anisotropic_tensors(m.nel, seed=seed).reshape(m.nel, 9)


def _accurate_dense_solution(rp, ci, v, rhs):
    """Dense LU of the oracle's matrix, then refinement with residuals in
    extended precision (numpy longdouble): LU alone is off by up to 1e-9 on
    these systems (1-norm condition ~5e8), the refined solution is accurate
    to ~1e-15."""
    N = rhs.size
    A = np.zeros((N, N))
    A[np.repeat(np.arange(N), np.diff(rp)), ci] = v
    x = np.linalg.solve(A, rhs)
    Al, bl = A.astype(np.longdouble), rhs.astype(np.longdouble)
    for _ in range(3):
        d = np.linalg.solve(A, (bl - Al @ x.astype(np.longdouble)).astype(np.float64))
        x = x + d
    assert np.linalg.norm(d) <= 1e-14 * np.linalg.norm(x)
    return x


def _refined_solution(gb, m, F, D, volume, face):
    c = _context(gb, m, F, np.full(m.nel, 3), D=D, g=0.3)
    c.dg_set_volume_kernel(volume)
    c.dg_set_face_kernel(face)
    c.dg_assemble()
    c.set_option(gb.OPT_DG_RESIDUAL, gb.RESIDUAL_COMPENSATED)
    x, inner, outer, rel = c.dg_solve_ir(krylov=50, max_iter=200000, tol_rel=1e-300, inner_tol=1e-6)
    c.close()
    assert outer >= 3 and rel < 1e-12
    return x


def _l2_rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


MIXED_FORMS = {"fp64": (0, 0), "tc_volume_tc_faces": (1, 1), "dword_volume_tc_faces": (3, 1)}


@pytest.mark.parametrize("n", [3, 4])
def test_mixed_precision_solution_error_vs_oracle(gb, n):
    """Config 4's mixed forms against the FP64 oracle at <= 1e-10 relative
    solution error.  The oracle's assembled matrix is solved densely to
    ~1e-15; each GPU assembly (plain FP64, split-BF16 tensor-core volume and
    faces, double-word volume with tensor-core faces) is solved by FP64
    iterative refinement around FP32-operator GMRES(50) with compensated
    residuals until the corrections reach FP64 rounding.  These systems
    amplify entry perturbations strongly (a random 1e-16 relative change of
    every entry moves the solution by ~1e-11), so the GPU FP64 matrix itself
    (within ~1.4e-15 of the oracle's on the entry scale) lands 3-5e-11 from
    the oracle's solution; the mixed forms land as close."""
    m, F, D = _p3_aniso_form(n)
    rp, ci, v, rhs, off = O.dg_assemble(m, F, np.full(m.nel, 3), D, pen=10.0, g=0.3, f=1.0)
    xo = _accurate_dense_solution(rp, ci, v, rhs)
    for name, (vol, face) in MIXED_FORMS.items():
        x = _refined_solution(gb, m, F, D, vol, face)
        err = _l2_rel(x, xo)
        print(f"n={n} {name}: relative solution error vs oracle {err:.2e}")
        assert err <= 1e-10, (name, err)  # measured 2.6e-11 .. 5.2e-11


def test_mixed_precision_solution_error_vs_fp64_larger(gb):
    """The same at 2,000 prisms (80,000 dofs; beyond a dense solve): the
    mixed forms' refined solutions against the plain FP64 assembly's refined
    solution (measured 6.4e-11 for both).  The double-word faces (4e-14 of
    the largest entry) move the solution by ~1.5e-9 on this system, which is
    why the mixed p = 3 form takes the tensor-core faces."""
    m, F, D = _p3_aniso_form(10)
    x64 = _refined_solution(gb, m, F, D, 0, 0)
    for name in ("tc_volume_tc_faces", "dword_volume_tc_faces"):
        x = _refined_solution(gb, m, F, D, *MIXED_FORMS[name])
        err = _l2_rel(x, x64)
        print(f"{name}: relative solution error vs FP64 {err:.2e}")
        assert err <= 1e-10, (name, err)
    xdw = _refined_solution(gb, m, F, D, gb.DG_VOLUME_DWORD, gb.DG_FACE_DWORD)
    assert _l2_rel(xdw, x64) <= 5e-9


def test_compensated_residual(gb):
    """The compensated DG residual against an exact rational evaluation of
    b - A x for a sample of rows, and against the FP64 residual."""
    from fractions import Fraction
    m, F, D = _p3_aniso_form(3)
    c = _context(gb, m, F, np.full(m.nel, 3), D=D, g=0.3)
    c.dg_assemble()
    rp, ci, v, rhs, off = _expand(c)
    x = np.random.default_rng(9).standard_normal(rhs.size)
    r64 = c.dg_compute_residual(x)
    c.set_option(gb.OPT_DG_RESIDUAL, gb.RESIDUAL_COMPENSATED)
    rc = c.dg_compute_residual(x)
    c.close()
    worst_c, worst_64 = 0.0, 0.0
    for i in np.random.default_rng(10).choice(rhs.size, 60, replace=False):
        row, cols = v[rp[i]:rp[i + 1]], x[ci[rp[i]:rp[i + 1]]]
        exact = Fraction(rhs[i]) - sum(Fraction(a) * Fraction(xv) for a, xv in zip(row, cols))
        scale = float(np.sum(np.abs(row * cols))) + abs(rhs[i])
        # Dot2's bound: one rounding of the exact value plus a term of order
        # (n eps)^2 of the summed magnitudes
        bound_c = 1.2e-16 * abs(float(exact)) + 1e-26 * scale
        worst_c = max(worst_c, abs(float(Fraction(rc[i]) - exact)) / bound_c)
        worst_64 = max(worst_64, abs(float(Fraction(r64[i]) - exact)) / scale)
    assert worst_c <= 1.0, worst_c
    assert worst_64 <= 1e-14


def test_dg_autotune_choices_do_not_change_results(gb):
    """Every launch shape gives the same bits; the tuner's choice is one of them."""
    from modfem_gb300.mesh import anisotropic_tensors, prism_faces, structured_prism_mesh
    m = structured_prism_mesh(5, jitter=0.2, seed=3)
    F = prism_faces(m)
    pdeg = np.random.default_rng(3).integers(1, 5, m.nel)
    c = _context(gb, m, F, pdeg, D=anisotropic_tensors(m.nel, seed=3).reshape(m.nel, 9), g=0.2)
    ref = None
    for v in range(3):
        for fv in range(2):
            c.dg_set_variants(vol=[0, v, v, v, v], face=[0, fv, fv, fv, fv])
            c.dg_assemble()
            out = c.dg_get_matrix()
            if ref is None:
                ref = out
            else:
                assert np.array_equal(out[0], ref[0]) and np.array_equal(out[1], ref[1]), (v, fv)
    vol, face, ms = c.dg_autotune(sample=1000)
    assert all(0 <= v < 3 for v in vol[1:]) and all(0 <= f < 2 for f in face[1:])
    assert np.all(ms[:, :3] > 0)
    c.dg_assemble()
    out = c.dg_get_matrix()
    assert np.array_equal(out[0], ref[0])
