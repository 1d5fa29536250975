"""The ModFEM-side shim (modfem_gb300/modfem_side/pds_gb300_ls_intf.c)
compiled against the reference's own headers and linked with the
reference's solver chain in place of its CPU assembly driver
(oracle/ref/Makefile, target shim).

Runs where the ModFEM sources are present (they are needed to build the
reference objects).  On a machine with a GPU the reference's sir_create,
assembly call and residual run through the shim and match the reference's
own assembly; without one the shim's first call reports the library's
failure (no device) and returns < 0, which shows the call reaching it.
"""
import os
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def _ref_src():
    import __graft_entry__ as g
    return g._ref_src()


def _build():
    ref = _ref_src()
    if not ref:
        pytest.skip("ModFEM sources not present")
    lib = os.path.join(ROOT, "modfem_gb300", "libmodfem_gb300.so")
    if not os.path.exists(lib):
        pytest.skip("libmodfem_gb300.so not built")
    subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "oracle", "ref"), f"REF={ref}", "all", "shim"])
    return os.path.join(ROOT, "oracle", "_ref", "libmodfem_ref_std_gb300.so")


RUN = r"""
import sys, json, os, tempfile
sys.path.insert(0, {root!r}); sys.path.insert(0, os.path.join({root!r}, "oracle"))
import numpy as np
import refmod
from modfem_gb300.mesh import lognormal_k, structured_prism_mesh, write_jk
m = structured_prism_mesh(10, jitter=0.2, seed=5)
k = lognormal_k(m.nel, seed=5)
tmp = tempfile.mkdtemp()
jk, mkb = os.path.join(tmp, "mesh.jk"), os.path.join(tmp, "mkb.dat")
write_jk(jk, 10)
refmod.write_mkb(mkb, krylov=30, max_iter=5000, tol=1e-8)
R = refmod.RefModfem({kind!r})
R.load_jk(jk)
R.set_node_coords(m.coords)
R.init_field("s", 1)
R.set_coeffs(k=k, f=1.0, g=0.0)
R.solver_create(mkb)
R.assemble()
rp, ci, val, rhs = R.crs()
np.savez(os.path.join({out!r}), row_ptr=rp, col_ind=ci, val=val, rhs=rhs)
"""


def _run(kind, out):
    code = RUN.format(root=ROOT, kind=kind, out=out)
    return subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600)


def test_shim_links_against_the_reference(tmp_path):
    lib = _build()
    syms = subprocess.run(["nm", "-D", "--defined-only", lib], capture_output=True, text=True).stdout
    assert " T pdr_create_assemble_stiff_mat" in syms and " T gbfem_shim_reset" in syms
    # the harness object of this build leaves the function to the shim
    hobj = os.path.join(ROOT, "oracle", "_ref", "obj_std", "harness_shim.o")
    assert "pdr_create_assemble_stiff_mat" not in subprocess.run(
        ["nm", "--defined-only", hobj], capture_output=True, text=True).stdout
    undefined = subprocess.run(["nm", "-D", "--undefined-only", lib], capture_output=True, text=True).stdout
    assert "gbfem_create_assemble_stiff_mat" in undefined  # resolved from libmodfem_gb300.so at load


def test_reference_assembly_call_goes_through_the_shim(tmp_path):
    _build()
    ref = _run("std", str(tmp_path / "ref.npz"))
    assert ref.returncode == 0, ref.stderr[-2000:]
    shim = _run("std_gb300", str(tmp_path / "shim.npz"))
    assert shim.returncode == 0, shim.stderr[-2000:]
    if "gbfem shim: gbfem_create" in shim.stderr:
        # no GPU here: the reference's assembly reached the shim, which
        # reported the library's error instead of assembling
        assert "gbfem_create" in shim.stderr
        return
    from _util import REL_TOL, crs_rel_err, energy_scale
    a, b = np.load(tmp_path / "shim.npz"), np.load(tmp_path / "ref.npz")
    assert np.array_equal(a["row_ptr"], b["row_ptr"]) and np.array_equal(a["col_ind"], b["col_ind"])
    sc = energy_scale(b["row_ptr"], b["col_ind"], b["val"])
    assert crs_rel_err(b["row_ptr"], a["val"], b["val"], sc) < REL_TOL
    assert np.max(np.abs(a["rhs"] - b["rhs"])) <= 1e-12 * np.max(np.abs(b["rhs"]))
