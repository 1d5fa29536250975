"""CPU checks: mesh generator numbering, and the C-ABI library surface."""
import os
import re

import numpy as np
import pytest

from _util import load

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.parametrize("name", ["std_n4", "std_n10", "std_n3_flat"])
def test_generator_reproduces_reference_numbering(name):
    """The generator's nodes, elements and boundary faces equal what the
    reference's jk reader (mmr_import_mesh_grad) and mmr_el_node_coor give."""
    from modfem_gb300.mesh import structured_prism_mesh
    g = load(name)
    m = structured_prism_mesh(int(g["n"]), jitter=float(g["jitter"]), seed=int(g["seed"]))
    assert np.array_equal(m.coords, g["coords"])
    assert np.array_equal(m.el_nodes, g["el_nodes"])
    assert np.array_equal(m.bc_face_id, g["bc_face_id"])
    assert np.array_equal(m.bc_face_el, g["bc_face_el"])
    assert np.array_equal(m.bc_face_bc, g["bc_face_bc"])


def test_jitter_keeps_boundary_and_positive_jacobians():
    from modfem_gb300.mesh import prism_min_detj, structured_prism_mesh
    m = structured_prism_mesh(12, jitter=0.2, seed=11)
    assert prism_min_detj(m) > 0
    for axis in range(3):
        c = m.coords[:, axis]
        on = (np.abs(c) < 1e-14) | (np.abs(c - 1) < 1e-14)
        assert on.sum() == 2 * 13 * 13  # both boundary planes stay fully populated


def declared_symbols():
    txt = open(os.path.join(ROOT, "include", "modfem_gb300.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(gbfem_[a-z_0-9]+)\s*\(", txt)))


def test_header_and_binding_agree():
    import modfem_gb300 as gb
    bound = sorted(n for n, _, _ in gb.SIGNATURES)
    assert bound == declared_symbols()


def test_library_loads_and_exports_every_declared_symbol():
    from modfem_gb300 import build
    import modfem_gb300 as gb
    build.build(verbose=False)
    lib = gb.load_library()
    for name in declared_symbols():
        assert hasattr(lib, name), name
    assert lib.gbfem_version() >= 1


def test_oracle_symbols_export():
    import oracle as O
    L = O.lib()
    for name in ["orc_std_prism_element", "orc_std_prism_face", "orc_std_tet_element", "orc_std_dof_order",
                 "orc_std_crs_structure", "orc_crs_table", "orc_color_entities", "orc_std_prism_assemble",
                 "orc_crs_residual", "orc_gmres_jacobi"]:
        assert hasattr(L, name)
