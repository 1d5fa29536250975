"""ModFEM file formats (CPU only): the jk reader against the reference's
mesh numbering, and the field dumps against files written by the
reference's own apr_write_field."""
import os

import numpy as np
import pytest

from _util import GOLDEN, load


@pytest.fixture(scope="module")
def io():
    from modfem_gb300 import build, io as gio
    build.build(verbose=False)
    return gio


@pytest.mark.parametrize("n", [2, 4, 7])
def test_read_jk_numbering(io, tmp_path, n):
    from modfem_gb300.mesh import prism_faces, structured_prism_mesh, write_jk
    path = str(tmp_path / "mesh.jk")
    write_jk(path, n)
    m, F = io.read_jk(path)
    ref = structured_prism_mesh(n)
    Fr = prism_faces(ref)
    assert np.array_equal(m.coords, ref.coords) and np.array_equal(m.el_nodes, ref.el_nodes)
    for k in ("type", "bc", "el1", "el2", "side1", "nodes"):
        assert np.array_equal(getattr(F, k), getattr(Fr, k)), k
    assert np.array_equal(m.bc_face_id, ref.bc_face_id) and np.array_equal(m.bc_face_el, ref.bc_face_el)
    assert np.array_equal(m.bc_face_side, ref.bc_face_side)


def test_read_jk_matches_reference_reader(io, tmp_path):
    """Coordinates and connectivity as the reference's own jk import left
    them (kept in the std_n4 fixture)."""
    from modfem_gb300.mesh import write_jk
    g = load("std_n4")
    path = str(tmp_path / "mesh.jk")
    write_jk(path, int(g["n"]))
    m, F = io.read_jk(path)
    assert np.array_equal(m.coords, g["coords_unjittered"])
    assert np.array_equal(m.el_nodes, g["el_nodes"])
    assert np.array_equal(np.sort(m.bc_face_id), np.sort(g["bc_face_id"]))


def test_read_jk_rejects_malformed(io, tmp_path):
    from modfem_gb300 import GbFemError
    path = tmp_path / "bad.jk"
    path.write_text("0 0 0 0\n3 0.0 1.0 1 1 1\n0 0\n1 0\n")
    with pytest.raises(GbFemError):
        io.read_jk(str(path))


def test_field_dump_std_matches_reference_writer(io, tmp_path):
    g = load("std_n4")
    out = str(tmp_path / "field.dmp")
    io.write_field_std(out, g["dof_of_node"], g["gmres_x"])
    assert open(out).read() == open(os.path.join(GOLDEN, "field_std_n4.dmp")).read()


def test_field_dump_dg_matches_reference_writer(io, tmp_path):
    g = load("dg_asm_mixed")
    out = str(tmp_path / "field.dmp")
    off = np.concatenate([g["dof_posglob"], [g["gmres_x"].size]])
    # the reference's field was created with one degree: one degree line
    io.write_field_dg(out, g["pdeg"], off, g["gmres_x"], uniform=True)
    assert open(out).read() == open(os.path.join(GOLDEN, "field_dg_mixed_n2.dmp")).read()
    io.write_field_dg(out, g["pdeg"], off, g["gmres_x"], uniform=False)
    lines = open(out).read().splitlines()
    assert lines[1:1 + g["pdeg"].size] == [str(-101 * int(p)) for p in g["pdeg"]]
