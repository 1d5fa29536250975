"""gbfem_compute_residual_noalloc against gbfem_compute_residual.

The no-alloc entry point serves callers that cannot let the library allocate
device memory (their own memory manager owns the GPU, or a cudaMalloc's
implicit synchronisation is not acceptable on their path).  It stages X, B
and V in a file-scope __device__ array shared by all calls on a device; these
tests check that two calls in a row give the allocating entry point's result
(the second call sees the array the first one left behind) and that sizes
above the array's capacity are refused.  The file sorts last so that a run
stopping at its first failure has run every other test before it.
"""
import numpy as np
import pytest

from _util import load, vec_rel_err

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gb():
    from modfem_gb300 import build
    build.build(verbose=False)
    import modfem_gb300
    return modfem_gb300


def test_noalloc_residual_matches_allocating_entry_point_twice(gb):
    from _util import FixtureMesh
    g = load("std_n10")
    m = FixtureMesh(g)
    c = gb.Context(0)
    c.set_mesh(m)
    c.set_coefficients(k=g["k"])
    c.set_crs_structure(g["dof_of_node"], g["row_ptr"], g["col_ind"])
    c.set_matrix(g["crs_val"], g["crs_rhs"])
    n = g["row_ptr"].size - 1
    x1 = g["resid_x"]
    x2 = np.cos(np.arange(n) * 0.11)
    b2 = np.sin(np.arange(n) * 0.7)
    # call 1: assembled rhs; call 2: explicit B and a different X
    ref1 = c.compute_residual(x1)
    got1 = c.compute_residual_noalloc(x1)
    assert vec_rel_err(got1, ref1) < 1e-12
    ref2 = c.compute_residual(x2, b=b2)
    got2 = c.compute_residual_noalloc(x2, b=b2)
    assert vec_rel_err(got2, ref2) < 1e-12
    # zero initial guess after a call that left a non-zero X in the array
    got3 = c.compute_residual_noalloc(x2, ini_zero=1)
    assert np.array_equal(got3, c.compute_residual(x2, ini_zero=1))
    # both results also agree with the reference's lar_compute_residual
    assert vec_rel_err(got1, g["resid_v"]) < 1e-12
    c.close()


def _device_free_bytes():
    """cuMemGetInfo on the calling thread's current context (the runtime's
    primary context, made current by the library's calls)."""
    import ctypes
    cu = ctypes.CDLL("libcuda.so.1")
    free, total = ctypes.c_size_t(), ctypes.c_size_t()
    assert cu.cuMemGetInfo_v2(ctypes.byref(free), ctypes.byref(total)) == 0
    return free.value


def test_noalloc_allocates_nothing_on_a_fresh_context(gb):
    """First residual of a fresh context through the no-alloc call: the
    context's device buffers do not grow, and once the first call has looked
    up the scratch array, further calls leave the device's free memory as it
    was.  The allocating call afterwards grows the context, as a contrast."""
    from _util import FixtureMesh
    g = load("std_n10")
    m = FixtureMesh(g)
    c = gb.Context(0)
    c.set_mesh(m)
    c.set_coefficients(k=g["k"])
    c.set_crs_structure(g["dof_of_node"], g["row_ptr"], g["col_ind"])
    c.set_matrix(g["crs_val"], g["crs_rhs"])
    n = g["row_ptr"].size - 1
    x = np.cos(np.arange(n) * 0.3)
    held = c.device_bytes()
    v1 = c.compute_residual_noalloc(x)
    assert c.device_bytes() == held
    free1 = _device_free_bytes()
    v2 = c.compute_residual_noalloc(x, b=np.ones(n))
    v3 = c.compute_residual_noalloc(x)
    assert _device_free_bytes() == free1
    assert c.device_bytes() == held
    assert np.array_equal(v1, v3)
    ref = c.compute_residual(x)
    assert vec_rel_err(v1, ref) < 1e-12
    assert vec_rel_err(v2, c.compute_residual(x, b=np.ones(n))) < 1e-12
    assert c.device_bytes() > held  # the allocating entry point grew its staging buffers
    c.close()


def test_noalloc_rejects_sizes_beyond_scratch(gb):
    from modfem_gb300.mesh import structured_prism_mesh
    m = structured_prism_mesh(64)  # 65^3 = 274,625 dofs > 262,144
    c = gb.Context(0)
    c.set_mesh(m)
    c.set_coefficients(k=np.ones(m.nel))
    nd, nnz, _ = c.build_structure()
    assert nd > 262144
    c.assemble(gb.SCATTER_ATOMIC)
    x = np.ones(nd)
    with pytest.raises(gb.GbFemError, match="GBFEM_NOALLOC_MAX_NDOF"):
        c.compute_residual_noalloc(x)
    # the allocating entry point still serves this size
    v = c.compute_residual(x)
    assert v.shape == (nd,)
    c.close()
