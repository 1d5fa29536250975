"""GPU parity of the DG prism volume integrals (tensor monomial basis, p=1..4)."""
import numpy as np
import pytest

import oracle as O
from _util import REL_TOL, load, mat_rel_err, vec_rel_err

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gb():
    from modfem_gb300 import build
    build.build(verbose=False)
    import modfem_gb300
    return modfem_gb300


class _Mesh:
    def __init__(self, coords, el_nodes):
        self.coords = coords
        self.el_nodes = el_nodes.astype(np.int32)
        self.bc_face_id = self.bc_face_el = self.bc_face_side = self.bc_face_bc = np.zeros(0, np.int32)


def dg_blocks(c, nel):
    off, bptr, bcol, boff = c.dg_get_structure()
    vals, rhs = c.dg_get_matrix()
    return off, bptr, bcol, boff, vals, rhs


def test_dg_element_blocks_vs_reference(gb):
    g = load("dg_el_n2")
    m = _Mesh(g["coords"], g["el_nodes"])
    c = gb.Context(0)
    c.set_mesh(m)
    c.set_coefficients(k=g["k"], f=1.0)
    c.dg_set_degrees(g["pdeg"])
    nd, nv = c.dg_build_structure()
    c.dg_assemble()
    off, bptr, bcol, boff, vals, rhs = dg_blocks(c, m.el_nodes.shape[0])
    for e in range(m.el_nodes.shape[0]):
        ns = off[e + 1] - off[e]
        blk = bptr[e]
        assert bcol[blk] == e
        K = vals[boff[blk]:boff[blk] + ns * ns].reshape(ns, ns).T
        Kr = g["sm"][g["sm_off"][e]:g["sm_off"][e + 1]].reshape(ns, ns)
        assert mat_rel_err(K, Kr) < REL_TOL, (e, int(g["pdeg"][e]))
        rr = g["rhs"][g["rhs_off"][e]:g["rhs_off"][e + 1]]
        assert vec_rel_err(rhs[off[e]:off[e + 1]], rr) < REL_TOL


@pytest.mark.parametrize("p", [1, 2, 3, 4])
def test_dg_anisotropic_vs_oracle(gb, p):
    from modfem_gb300.mesh import anisotropic_tensors, structured_prism_mesh
    m = structured_prism_mesh(3, jitter=0.2, seed=p)
    D = anisotropic_tensors(m.nel, seed=p)
    c = gb.Context(0)
    c.set_mesh(m)
    c.set_coefficients(D=D, f=1.0)
    c.dg_set_degrees(np.full(m.nel, p))
    c.dg_build_structure()
    c.dg_assemble()
    off, bptr, bcol, boff, vals, rhs = dg_blocks(c, m.nel)
    for e in range(m.nel):
        ns = off[e + 1] - off[e]
        K = vals[boff[e]:boff[e] + ns * ns].reshape(ns, ns).T
        Ko, ro = O.dg_prism_element(m.coords[m.el_nodes[e]], D[e], p)
        assert mat_rel_err(K, Ko) < REL_TOL, e
        assert vec_rel_err(rhs[off[e]:off[e + 1]], ro) < REL_TOL
