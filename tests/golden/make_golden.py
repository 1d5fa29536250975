"""Generates the golden fixtures in this directory from the reference ModFEM.

Runs the reference C path compiled in-tree (``make -C oracle/ref REF=...``,
which needs the ModFEM sources: $MODFEM_REF_SRC, or a checkout named
``reference`` beside this repository) through ``oracle/refmod.py``: the reference's own jk
mesh reader, approximation module, weak forms, sir_create, the table-driven
assembly driver and GMRES.  Each case runs in a fresh process because the
reference keeps its meshes, fields and solvers in global arrays.

    python tests/golden/make_golden.py            # all cases
    python tests/golden/make_golden.py std_n4     # one case

Fixtures are small .npz files; the GPU machine never needs the reference.
"""
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

# name: (n, jitter, seed, keep element matrices, krylov, tol)
CASES = {
    "std_n4": (4, 0.2, 3, True, 30, 1e-8),
    "std_n10": (10, 0.2, 5, False, 30, 1e-8),
    "std_n3_flat": (3, 0.0, 0, True, 30, 1e-10),
}


def run_case(name):
    import refmod
    from modfem_gb300.mesh import lognormal_k, structured_prism_mesh, write_jk

    n, jitter, seed, keep_el, krylov, tol = CASES[name]
    m = structured_prism_mesh(n, jitter=jitter, seed=seed)
    k = lognormal_k(m.nel, seed=seed) if jitter > 0 else np.ones(m.nel)
    tmp = tempfile.mkdtemp()
    jk = os.path.join(tmp, "mesh.jk")
    mkb = os.path.join(tmp, "mkb.dat")
    write_jk(jk, n)
    refmod.write_mkb(mkb, krylov=krylov, max_iter=5000, tol=tol)
    R = refmod.RefModfem("std")
    R.load_jk(jk)
    ref_xyz0 = R.node_coords()
    R.set_node_coords(m.coords)
    R.init_field("s", 1)
    R.set_coeffs(k=k, f=1.0, g=0.0)
    out = dict(n=n, jitter=jitter, seed=seed, krylov=krylov, tol=tol,
               coords=R.node_coords(), coords_unjittered=ref_xyz0, el_nodes=R.el_nodes() - 1, k=k)
    fid, fbc, fel = R.bc_faces()
    out.update(bc_face_id=fid, bc_face_bc=fbc, bc_face_el=fel - 1)
    if keep_el:
        sms, rhss = [], []
        for e in range(R.max_el):
            K, r, _ = R.int_ent_stiff(refmod.APC_ELEMENT, e + 1)
            sms.append(K)
            rhss.append(r)
        out.update(el_sm=np.array(sms), el_rhs=np.array(rhss))
        fsm, frhs = [], []
        for f in fid:
            K, r, _ = R.int_ent_stiff(refmod.APC_FACE, int(f))
            fsm.append(K)
            frhs.append(r)
        out.update(fa_sm=np.array(fsm), fa_rhs=np.array(frhs))
    R.solver_create(mkb)
    ll = R.level_lists()
    R.assemble()
    rp, ci, val, rhs = R.crs()
    dof_of_node = np.full(R.max_node, -1, np.int32)
    dof_of_node[ll["dof_ent_id"] - 1] = ll["dof_posglob"]
    out.update(row_ptr=rp, col_ind=ci, crs_val=val, crs_rhs=rhs, dof_of_node=dof_of_node,
               int_ent_type=ll["int_ent_type"], int_ent_id=ll["int_ent_id"], color_elems=ll["color_elems"],
               color_faces=ll["color_faces"], asse_pos=ll["asse_pos"], assembly_table=ll["assembly_table"])
    # residual of a deterministic vector through lar_compute_residual
    x = np.sin(np.arange(R.ndof) * 0.37)
    out.update(resid_x=x, resid_v=R.residual(x, None, 1))
    sol, nit, meas, _ = R.solve(-1, -1.0)
    xs = np.zeros(R.ndof)
    has = dof_of_node >= 0
    xs[dof_of_node[has]] = sol[1:R.max_node + 1][has]
    out.update(gmres_x=xs, gmres_iters=nit, gmres_meas=meas)
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)
    print(f"{name}: nel {R.max_el} ndof {R.ndof} nnz {R.nnz} colours {R.nr_colors_elems}/{R.nr_colors_faces} "
          f"gmres {nit} it", file=sys.stderr)


# name: (n, jitter, seed, passes of 1-based element ids to refine, max generation)
HANG_CASES = {
    "std_n9_hang": (9, 0.2, 8, [[1, 200, 731], [1459, 1000]], 2),
}


def run_hanging(name):
    """A std prism mesh after the reference's own refinement (apr_refine with
    the 1-irregular rule, apr_proj_dof_ref creating the constraint data): the
    active elements' dof lists hold the constraining vertices of their
    hanging vertices, and the reference's apr_get_stiff_mat_data rewrites
    their element and face matrices.  Records the refined mesh, the
    constraint data, the rewritten local matrices of the constrained
    entities, the solver lists and tables and the assembled system."""
    import ctypes
    import refmod
    from refmod import _p
    from modfem_gb300.mesh import lognormal_k, structured_prism_mesh, write_jk

    n, jitter, seed, passes, max_gen = HANG_CASES[name]
    m = structured_prism_mesh(n, jitter=jitter, seed=seed)
    tmp = tempfile.mkdtemp()
    jk = os.path.join(tmp, "mesh.jk")
    mkb = os.path.join(tmp, "mkb.dat")
    write_jk(jk, n, capacity=(20000, 60000, 60000, 20000))
    refmod.write_mkb(mkb, krylov=30, max_iter=5000, tol=1e-8)
    R = refmod.RefModfem("std")
    R.load_jk(jk)
    R.set_node_coords(m.coords)
    R.init_field("s", 1)
    for ids in passes:
        ids = np.array(ids, np.int32)
        R.L.refh_refine(ids.size, _p(ids), max_gen)
    s = [ctypes.c_int() for _ in range(6)]
    R.L.refh_mesh_sizes(*[ctypes.byref(x) for x in s])
    R.nno, R.max_node, R.nel, R.max_el = s[0].value, s[1].value, s[2].value, s[3].value
    status = np.zeros(R.max_el, np.int32)
    R.L.refh_el_status(_p(status))
    cnt = np.zeros(R.max_node, np.int32)
    par = np.zeros(4 * R.max_node, np.int32)
    R.L.refh_constr(_p(cnt), _p(par))
    k = lognormal_k(R.max_el, seed=seed)
    R.set_coeffs(k=k, f=1.0, g=0.0)
    fid, fbc, fel = R.bc_faces()
    side = np.zeros(fid.size, np.int32)
    R.L.refh_bc_face_sides(fid.size, _p(fid), _p(fel), _p(side))
    out = dict(n=n, jitter=jitter, seed=seed, coords=R.node_coords(), el_nodes=R.el_nodes() - 1,
               el_status=status, k=k, con_cnt=cnt, con_par=par.reshape(-1, 4) - 1,
               bc_face_id=fid, bc_face_bc=fbc, bc_face_el=fel - 1, bc_face_side=side)
    # rewritten local matrices of every active element and boundary face
    # whose dof list holds constraining vertices, with that list
    ents, sms, rhss, dofs = [], [], [], []
    for e in np.nonzero(status == 1)[0]:
        K, r, d = R.int_ent_stiff(refmod.APC_ELEMENT, int(e) + 1, maxn=30)
        if K.shape[0] > 6:
            ents.append((refmod.APC_ELEMENT, int(e) + 1))
            sms.append(K)
            rhss.append(r)
            dofs.append(d)
    for f in fid:
        K, r, d = R.int_ent_stiff(refmod.APC_FACE, int(f), maxn=30)
        if K.shape[0] > 6:
            ents.append((refmod.APC_FACE, int(f)))
            sms.append(K)
            rhss.append(r)
            dofs.append(d)
    ns = np.array([K.shape[0] for K in sms], np.int32)
    out.update(con_ent=np.array(ents, np.int32).reshape(-1, 2), con_ns=ns,
               con_sm=np.concatenate([K.ravel() for K in sms]), con_rhs=np.concatenate(rhss),
               con_dofs=np.concatenate(dofs) - 1)
    R.solver_create(mkb)
    ll = R.level_lists()
    R.assemble()
    rp, ci, val, rhs = R.crs()
    dof_of_node = np.full(R.max_node, -1, np.int32)
    dof_of_node[ll["dof_ent_id"] - 1] = ll["dof_posglob"]
    out.update(row_ptr=rp, col_ind=ci, crs_val=val, crs_rhs=rhs, dof_of_node=dof_of_node,
               int_ent_type=ll["int_ent_type"], int_ent_id=ll["int_ent_id"], color_elems=ll["color_elems"],
               color_faces=ll["color_faces"], asse_pos=ll["asse_pos"], assembly_table=ll["assembly_table"],
               max_dofs_int_ent=R.max_dofs_int_ent)
    sol, nit, meas, _ = R.solve(-1, -1.0)
    xs = np.zeros(R.ndof)
    has = dof_of_node >= 0
    xs[dof_of_node[has]] = sol[1:R.max_node + 1][has]
    out.update(gmres_x=xs, gmres_iters=nit, gmres_meas=meas)
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)
    print(f"{name}: {R.nel} active of {R.max_el} elements, {int((cnt > 0).sum())} constrained vertices "
          f"({int((cnt == 2).sum())} mid-edge, {int((cnt == 4).sum())} mid-face), {len(ents)} rewritten "
          f"entities, ndof {R.ndof} nnz {R.nnz} max dofs {R.max_dofs_int_ent}, gmres {nit} it", file=sys.stderr)


def run_tets(name="std_tet_n2"):
    """Std linear tetrahedra through the reference's apr_elem_calc_3D (tetra
    base) and quadrature; no tet mesh module is linked, so the elements come
    from the structured Kuhn split with jitter."""
    import refmod
    from modfem_gb300.mesh import lognormal_k, structured_tet_mesh
    import ctypes
    m = structured_tet_mesh(2, jitter=0.15, seed=8)
    k = lognormal_k(m.nel, seed=8)
    L = ctypes.CDLL(refmod.lib_path("std"))
    L.refh_tet_element.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_double, ctypes.c_void_p,
                                   ctypes.c_void_p]
    sms, rhss = [], []
    for e in range(m.nel):
        X = np.ascontiguousarray(m.coords[m.el_nodes[e]]).reshape(-1)
        A = np.ascontiguousarray(np.diag([k[e]] * 3)).reshape(-1)
        sm = np.zeros(16)
        r = np.zeros(4)
        L.refh_tet_element(X.ctypes.data, A.ctypes.data, 1.0, sm.ctypes.data, r.ctypes.data)
        sms.append(sm.reshape(4, 4).T.copy())
        rhss.append(r)
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), coords=m.coords, el_nodes=m.el_nodes, k=k,
                        el_sm=np.array(sms), el_rhs=np.array(rhss))
    print(f"{name}: {m.nel} tets", file=sys.stderr)


# Dirichlet value on the DG boundary faces (enters the face load vectors)
DG_G = 0.3


def run_dg_elements(name="dg_el_n2"):
    """DG tensor prisms of mixed degree p in 1..4 through the reference's DG
    module (apr_num_int_el of apd_dg_prism via the DG weak form); the
    "aniso" case uses a full symmetric tensor R diag(1, 0.1, 0.01) R^T."""
    import refmod
    from modfem_gb300.mesh import anisotropic_tensors, lognormal_k, structured_prism_mesh, write_jk
    n, seed = 2, 21
    m = structured_prism_mesh(n, jitter=0.2, seed=seed)
    k = lognormal_k(m.nel, seed=seed)
    D = anisotropic_tensors(m.nel, seed=seed) if "aniso" in name else None
    pdeg = np.random.default_rng(seed).integers(1, 5, m.nel)
    tmp = tempfile.mkdtemp()
    jk = os.path.join(tmp, "mesh.jk")
    write_jk(jk, n)
    R = refmod.RefModfem("dg")
    R.load_jk(jk)
    R.set_node_coords(m.coords)
    R.init_field("t", 101)
    if D is None:
        R.set_coeffs(k=k, f=1.0, g=DG_G)
    else:
        R.set_coeffs(D=D, f=1.0, g=DG_G)
    R.set_dg_penalty(10.0)
    sms, rhss = [], []
    for e in range(m.nel):
        R.L.refh_set_el_pdeg(e + 1, int(101 * pdeg[e]))
    for e in range(m.nel):
        K, r, _ = R.int_ent_stiff(refmod.APC_ELEMENT, e + 1)
        sms.append(K.reshape(-1))
        rhss.append(r)
    off = np.concatenate([[0], np.cumsum([x.size for x in sms])])
    roff = np.concatenate([[0], np.cumsum([x.size for x in rhss])])
    # every face (interior and Dirichlet boundary), in mmr face order
    from modfem_gb300.mesh import prism_faces
    F = prism_faces(m)
    fsm, frhs = [], []
    for fid in F.id:
        K, r, _ = R.int_ent_stiff(refmod.APC_FACE, int(fid), maxn=200)
        fsm.append(K.reshape(-1))
        frhs.append(r)
    foff = np.concatenate([[0], np.cumsum([x.size for x in fsm])])
    froff = np.concatenate([[0], np.cumsum([x.size for x in frhs])])
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), coords=m.coords, el_nodes=m.el_nodes, k=k,
                        D=np.zeros(0) if D is None else D, pdeg=pdeg, sm=np.concatenate(sms), sm_off=off,
                        rhs=np.concatenate(rhss), rhs_off=roff, fa_sm=np.concatenate(fsm), fa_sm_off=foff,
                        fa_rhs=np.concatenate(frhs), fa_rhs_off=froff, pen=10.0, g=DG_G)
    print(f"{name}: {m.nel} DG prisms, p counts {np.bincount(pdeg, minlength=5)[1:]}", file=sys.stderr)


# assembled DG systems: (n, degree mode, anisotropic)
DG_ASM_CASES = {"dg_asm_p2": (2, 2, False), "dg_asm_mixed": (2, "mixed", False), "dg_asm_aniso": (2, "mixed", True)}


def run_dg_assembly(name):
    """Whole DG system from the reference: every element and face integrated
    and assembled by the MKB solver into its block storage (lad_block), the
    rhs, and the GMRES(50) solution with block Jacobi to 1e-10 relative."""
    import refmod
    from modfem_gb300.mesh import anisotropic_tensors, lognormal_k, structured_prism_mesh, write_jk
    n, mode, aniso = DG_ASM_CASES[name]
    seed = 21
    m = structured_prism_mesh(n, jitter=0.2, seed=seed)
    k = lognormal_k(m.nel, seed=seed)
    D = anisotropic_tensors(m.nel, seed=seed) if aniso else None
    pdeg = np.random.default_rng(seed).integers(1, 5, m.nel) if mode == "mixed" else np.full(m.nel, mode)
    krylov, tol = 50, 1e-10
    tmp = tempfile.mkdtemp()
    jk = os.path.join(tmp, "mesh.jk")
    mkb = os.path.join(tmp, "mkb.dat")
    write_jk(jk, n)
    refmod.write_mkb(mkb, krylov=krylov, max_iter=5000, tol=tol)
    R = refmod.RefModfem("dg")
    R.load_jk(jk)
    R.set_node_coords(m.coords)
    R.init_field("t", 101 * int(pdeg.max()))
    if D is None:
        R.set_coeffs(k=k, f=1.0, g=DG_G)
    else:
        R.set_coeffs(D=D, f=1.0, g=DG_G)
    R.set_dg_penalty(10.0)
    for e in range(m.nel):
        R.L.refh_set_el_pdeg(e + 1, int(101 * pdeg[e]))
    R.solver_create(mkb)
    ll = R.level_lists()
    R.assemble()
    rp, ci, val, rhs = R.block_crs()
    stride = 75
    sol, nit, meas, _ = R.solve(-1, -1.0, stride=stride)
    off = ll["dof_posglob"]
    x = np.zeros(R.ndof)
    for ent, pos in zip(ll["dof_ent_id"], off):
        e = int(ent) - 1
        ns = [0, 6, 18, 40, 75][int(pdeg[e])]
        x[pos:pos + ns] = sol[(e + 1) * stride:(e + 1) * stride + ns]
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), n=n, jitter=0.2, seed=seed, coords=m.coords,
                        el_nodes=m.el_nodes, k=k, D=np.zeros(0) if D is None else D, pdeg=pdeg, pen=10.0, g=DG_G,
                        f=1.0, dof_ent_id=ll["dof_ent_id"], dof_posglob=off, row_ptr=rp, col_ind=ci, val=val,
                        rhs=rhs, krylov=krylov, tol=tol, gmres_iters=nit, gmres_meas=meas, gmres_x=x)
    print(f"{name}: {m.nel} DG prisms, ndof {R.ndof}, nnz {ci.size}, gmres {nit} it", file=sys.stderr)


def run_fields(name="fields"):
    """field.dmp files written by the reference's apr_write_field for the
    std_n4 solution (std module) and for the dg_asm_mixed solution (DG
    module), with the values the fixtures hold."""
    import ctypes
    import refmod
    from modfem_gb300.mesh import structured_prism_mesh, write_jk
    tmp = tempfile.mkdtemp()
    g = dict(np.load(os.path.join(HERE, "std_n4.npz")))
    jk = os.path.join(tmp, "mesh4.jk")
    write_jk(jk, int(g["n"]))
    R = refmod.RefModfem("std")
    R.load_jk(jk)
    R.set_node_coords(g["coords"])
    R.init_field("s", 1)
    vals = np.full(g["dof_of_node"].size, np.nan)
    has = g["dof_of_node"] >= 0
    vals[has] = g["gmres_x"][g["dof_of_node"][has]]
    out = os.path.join(HERE, "field_std_n4.dmp")
    R.L.refh_write_field.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
    R.L.refh_write_field(out.encode(), refmod.APC_VERTEX, vals.size, vals.ctypes.data, None)
    gd = dict(np.load(os.path.join(HERE, "dg_asm_mixed.npz")))
    jk = os.path.join(tmp, "mesh2.jk")
    write_jk(jk, int(gd["n"]))
    R = refmod.RefModfem("dg")
    R.load_jk(jk)
    R.set_node_coords(gd["coords"])
    R.init_field("t", 101 * int(gd["pdeg"].max()))
    for e, p in enumerate(gd["pdeg"]):
        R.L.refh_set_el_pdeg(e + 1, int(101 * p))
    off = np.concatenate([gd["dof_posglob"], [gd["gmres_x"].size]]).astype(np.int32)
    out = os.path.join(HERE, "field_dg_mixed_n2.dmp")
    R.L.refh_write_field.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
    R.L.refh_write_field(out.encode(), refmod.APC_ELEMENT, gd["pdeg"].size, gd["gmres_x"].ctypes.data,
                         off.ctypes.data)
    print("fields: field_std_n4.dmp, field_dg_mixed_n2.dmp", file=sys.stderr)


def main(argv):
    ref = os.environ.get("MODFEM_REF_SRC") or os.path.normpath(
        os.path.join(ROOT, "..", "reference", "modfem2017", "src"))
    subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "oracle", "ref"), f"REF={ref}"])
    names = argv or list(CASES) + list(HANG_CASES) + ["std_tet_n2", "dg_el_n2", "dg_el_aniso_n2"] + list(DG_ASM_CASES) + ["fields"]
    if len(names) == 1 and os.environ.get("MAKE_GOLDEN_CHILD"):
        with open(os.devnull, "w") as dn:
            # the reference prints progress on stdout; keep only our stderr summary
            os.dup2(dn.fileno(), 1)
            if names[0] == "std_tet_n2":
                run_tets(names[0])
            elif names[0].startswith("dg_el_"):
                run_dg_elements(names[0])
            elif names[0] in DG_ASM_CASES:
                run_dg_assembly(names[0])
            elif names[0] == "fields":
                run_fields()
            elif names[0] in HANG_CASES:
                run_hanging(names[0])
            else:
                run_case(names[0])
        return
    for nm in names:
        env = dict(os.environ, MAKE_GOLDEN_CHILD="1")
        subprocess.check_call([sys.executable, __file__, nm], env=env)


if __name__ == "__main__":
    main(sys.argv[1:])
