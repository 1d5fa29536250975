"""Test infrastructure only: ctypes access to the C restatement (liboracle.so).

Used by tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg,
always as the checker or the timed CPU baseline, never as the product.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")

_L = None


def build():
    subprocess.check_call(["make", "-s", "-C", HERE, "liboracle.so"])


def lib():
    global _L
    if _L is None:
        if not os.path.exists(LIB):
            build()
        L = ctypes.CDLL(LIB)
        vp, ci, cd = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
        L.orc_std_prism_element.argtypes = [vp, vp, cd, vp, vp]
        L.orc_std_prism_face.argtypes = [vp, ci, cd, cd, vp, vp]
        L.orc_std_tet_element.argtypes = [vp, vp, cd, vp, vp]
        L.orc_std_dof_order.argtypes = [ci, ci, vp, ci, vp]
        L.orc_std_crs_structure.argtypes = [ci, ci, vp, vp, ci, vp, vp]
        L.orc_std_crs_structure.restype = ctypes.c_long
        L.orc_crs_table.argtypes = [ci, vp, vp, vp, vp]
        L.orc_color_entities.argtypes = [ci, ci, vp, ci, vp]
        L.orc_std_prism_assemble.argtypes = [ci, vp, vp, vp, vp, cd, ci, vp, vp, cd, cd, vp, vp, vp,
                                             vp, vp, ci, vp, vp]
        L.orc_std_prism_assemble.restype = cd
        L.orc_set_accumulate_abs.argtypes = [ci]
        L.orc_dg_prism_element.argtypes = [vp, vp, cd, ci, vp, vp]
        L.orc_dg_face.argtypes = [ci, vp, vp, ci, vp, ci, vp, vp, ci, vp, cd, cd, vp, vp]
        L.orc_crs_residual.argtypes = [ci, vp, vp, vp, ci, vp, vp, vp]
        L.orc_gmres_jacobi.argtypes = [ci, vp, vp, vp, vp, vp, ci, ci, cd, vp, vp]
        _L = L
    return _L


def _p(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def _c(a, dt):
    return None if a is None else np.ascontiguousarray(a, dtype=dt)


def std_prism_element(X, A, f=1.0):
    X = _c(X, np.float64).reshape(-1)
    A = _c(A, np.float64).reshape(-1)
    sm = np.zeros(36)
    rhs = np.zeros(6)
    lib().orc_std_prism_element(_p(X), _p(A), f, _p(sm), _p(rhs))
    return sm.reshape(6, 6).T.copy(), rhs  # (row w, column u)


def std_prism_face(X, side, penalty=1e7, g=0.0):
    X = _c(X, np.float64).reshape(-1)
    sm = np.zeros(36)
    rhs = np.zeros(6)
    lib().orc_std_prism_face(_p(X), side, penalty, g, _p(sm), _p(rhs))
    return sm.reshape(6, 6).T.copy(), rhs


def std_tet_element(X, A, f=1.0):
    X = _c(X, np.float64).reshape(-1)
    A = _c(A, np.float64).reshape(-1)
    sm = np.zeros(16)
    rhs = np.zeros(4)
    lib().orc_std_tet_element(_p(X), _p(A), f, _p(sm), _p(rhs))
    return sm.reshape(4, 4).T.copy(), rhs


def dg_prism_element(X, A, p, f=1.0):
    """DG tensor prism of degree p: (ns x ns matrix (row w, column u), rhs)."""
    X = _c(X, np.float64).reshape(-1)
    A = _c(A, np.float64).reshape(-1)
    ns = lib().orc_dg_nshape(p)
    sm = np.zeros(ns * ns)
    rhs = np.zeros(ns)
    lib().orc_dg_prism_element(_p(X), _p(A), f, p, _p(sm), _p(rhs))
    return sm.reshape(ns, ns).T.copy(), rhs


def face_local_vertices(el_nodes_e, face_nodes):
    """Local vertex index in an element of each face vertex (face order)."""
    return np.array([int(np.nonzero(el_nodes_e == v)[0][0]) for v in face_nodes if v >= 0], np.int32)


def dg_face(mesh, faces, i, pdeg, A, pen=10.0, g=0.0):
    """DG face matrix ((ns1+ns2)^2 as (row, column)) and rhs of face i of a
    FaceTable; A: (nel, 9) coefficient tensors; pdeg per element."""
    e1, e2 = int(faces.el1[i]), int(faces.el2[i])
    fn = faces.nodes[i]
    X1 = _c(mesh.coords[mesh.el_nodes[e1]], np.float64).reshape(-1)
    l1 = face_local_vertices(mesh.el_nodes[e1], fn)
    A1 = _c(A[e1], np.float64)
    p1 = int(pdeg[e1])
    n = lib().orc_dg_nshape(p1)
    X2 = l2 = A2 = None
    p2 = 1
    if e2 >= 0:
        X2 = _c(mesh.coords[mesh.el_nodes[e2]], np.float64).reshape(-1)
        l2 = face_local_vertices(mesh.el_nodes[e2], fn)
        A2 = _c(A[e2], np.float64)
        p2 = int(pdeg[e2])
        n += lib().orc_dg_nshape(p2)
    sm = np.zeros(n * n)
    rhs = np.zeros(n)
    lib().orc_dg_face(int(faces.type[i]), _p(X1), _p(l1), p1, _p(A1), int(faces.side1[i]), _p(X2), _p(l2), p2,
                      _p(A2), pen, g, _p(sm), _p(rhs))
    return sm.reshape(n, n).T.copy(), rhs


DG_NS = (0, 6, 18, 40, 75)


def dg_block_structure(nel, faces, pdeg):
    """Dof offsets of the DG blocks (one per element, element order:
    utr_get_list_ent, utd_util/uts_ls_intf.c:640-700) and the column blocks
    of each block row: the element and its face neighbours, ascending (the
    sorted neighbour lists of sir_create, sid_mkb/sis_mkb_intf.c:1100-1146)."""
    off = np.concatenate([[0], np.cumsum([DG_NS[int(p)] for p in pdeg])]).astype(np.int64)
    nb = [[e] for e in range(nel)]
    if faces is not None:
        for e1, e2 in zip(faces.el1, faces.el2):
            if e2 >= 0:
                nb[int(e1)].append(int(e2))
                nb[int(e2)].append(int(e1))
    return off, [sorted(x) for x in nb]


def dg_assemble(mesh, faces, pdeg, A, pen=10.0, g=0.0, f=1.0):
    """The whole DG system: element integrals, then face integrals in face
    order, summed block by block as lar_assemble_SM_and_LV_block does
    (lsd_mkb/lad_block/las_block_intf.c:362-520).  A: (nel, 9) tensors.
    Returns the scalar expansion of the block storage (every entry of every
    block, columns ascending: row_ptr, col_ind, val), the rhs and the dof
    offsets."""
    nel = mesh.nel
    off, cols = dg_block_structure(nel, faces, pdeg)
    B = {}
    rhs = np.zeros(int(off[-1]))
    for e in range(nel):
        K, r = dg_prism_element(mesh.coords[mesh.el_nodes[e]], A[e], int(pdeg[e]), f)
        B[(e, e)] = K
        rhs[off[e]:off[e + 1]] += r
    if faces is not None:
        for i in range(faces.n):
            K, r = dg_face(mesh, faces, i, pdeg, A, pen, g)
            e1, e2 = int(faces.el1[i]), int(faces.el2[i])
            n1 = DG_NS[int(pdeg[e1])]
            B[(e1, e1)] = B[(e1, e1)] + K[:n1, :n1]
            rhs[off[e1]:off[e1 + 1]] += r[:n1]
            if e2 >= 0:
                B[(e1, e2)] = B.get((e1, e2), 0.0) + K[:n1, n1:]
                B[(e2, e1)] = B.get((e2, e1), 0.0) + K[n1:, :n1]
                B[(e2, e2)] = B[(e2, e2)] + K[n1:, n1:]
    rp = [0]
    ci, val = [], []
    for e in range(nel):
        row = np.concatenate([B[(e, c)] for c in cols[e]], axis=1)
        cidx = np.concatenate([np.arange(off[c], off[c + 1]) for c in cols[e]])
        for i in range(row.shape[0]):
            ci.append(cidx)
            val.append(row[i])
            rp.append(rp[-1] + cidx.size)
    return (np.array(rp, np.int64), np.concatenate(ci).astype(np.int64), np.concatenate(val), rhs, off)


def dof_order(el_nodes, nno):
    el = _c(el_nodes, np.int32)
    d = np.zeros(nno, np.int32)
    nd = lib().orc_std_dof_order(el.shape[0], el.shape[1], _p(el), nno, _p(d))
    return d, nd


def crs_structure(el_nodes, dof_of_node, ndof):
    el = _c(el_nodes, np.int32)
    dn = _c(dof_of_node, np.int32)
    rp = np.zeros(ndof + 1, np.int32)
    nnz = lib().orc_std_crs_structure(el.shape[0], el.shape[1], _p(el), _p(dn), ndof, _p(rp), None)
    ci = np.zeros(nnz, np.int32)
    lib().orc_std_crs_structure(el.shape[0], el.shape[1], _p(el), _p(dn), ndof, _p(rp), _p(ci))
    return rp, ci


def crs_table(dofs, row_ptr, col_ind):
    d = _c(dofs, np.int32)
    n = d.size
    t = np.zeros(n * n + n, np.int32)
    lib().orc_crs_table(n, _p(d), _p(row_ptr), _p(col_ind), _p(t))
    return t


def color_entities(ent_dofs, ndof):
    e = _c(ent_dofs, np.int32)
    col = np.zeros(e.shape[0], np.int32)
    nc = lib().orc_color_entities(e.shape[0], e.shape[1], _p(e), ndof, _p(col))
    return col, nc


def std_prism_assemble(mesh, k_el, dof_of_node, row_ptr, col_ind, f=1.0, penalty=1e7, g=0.0,
                       D_el=None, color_ptr=None, perm=None, nthreads=1):
    nnz = col_ind.size
    val = np.zeros(nnz)
    rhs = np.zeros(row_ptr.size - 1)
    el = _c(mesh.el_nodes, np.int32)
    xyz = _c(mesh.coords, np.float64)
    k = _c(k_el, np.float64)
    D = _c(D_el, np.float64)
    fe = _c(mesh.bc_face_el, np.int32)
    fs = _c(mesh.bc_face_side, np.int32)
    cp = _c(color_ptr, np.int32)
    pm = _c(perm, np.int32)
    t = lib().orc_std_prism_assemble(el.shape[0], _p(el), _p(xyz), _p(k), _p(D), f, fe.size, _p(fe),
                                     _p(fs), penalty, g, _p(_c(dof_of_node, np.int32)),
                                     _p(_c(row_ptr, np.int32)), _p(_c(col_ind, np.int32)), _p(cp),
                                     _p(pm), nthreads, _p(val), _p(rhs))
    return val, rhs, t


def std_prism_assemble_abs(mesh, k_el, dof_of_node, row_ptr, col_ind, **kw):
    """Sum of |contributions| per CRS entry and rhs row: the scale against
    which assembled values are compared (each contribution carries its own
    relative rounding error, so a sum with cancellation cannot be matched to
    a relative tolerance of the sum itself)."""
    lib().orc_set_accumulate_abs(1)
    try:
        return std_prism_assemble(mesh, k_el, dof_of_node, row_ptr, col_ind, **kw)
    finally:
        lib().orc_set_accumulate_abs(0)


def std_constraint_expand(nodes, con_cnt, con_par):
    """The dof entity list of a std element whose vertices may be hanging,
    with the coefficients of its rewrite (apr_get_stiff_mat_data,
    apd_std_lin/aps_std_lin_intf.c:2978-3035): in vertex order, a real vertex
    stands for itself with coefficient 1, a constrained vertex for its
    constraining vertices (apr_get_constr_data order) with coefficient 1/2
    (2 of them: mid-edge) or 1/4 (4: mid-face).  Returns (local vertex of
    each entry, coefficient, vertex id)."""
    src, coef, ids = [], [], []
    for ino, v in enumerate(nodes):
        c = int(con_cnt[v])
        if c == 0:
            src.append(ino)
            coef.append(1.0)
            ids.append(int(v))
        else:
            cv = 0.5 if c == 2 else 0.25
            for j in range(c):
                src.append(ino)
                coef.append(cv)
                ids.append(int(con_par[v][j]))
    return np.array(src), np.array(coef), np.array(ids, np.int32)


def std_constraint_rewrite(K, R, nodes, con_cnt, con_par):
    """The rewrite of a local matrix (row w, column u) and load vector for
    hanging vertices (aps_std_lin_intf.c:3077-3160): entry (a, b) of the
    rewritten matrix is c_b c_a K[i(a), i(b)], entry a of the load vector
    c_a R[i(a)], over the expanded list of std_constraint_expand."""
    src, coef, ids = std_constraint_expand(nodes, con_cnt, con_par)
    Kc = (coef[None, :] * coef[:, None]) * K[np.ix_(src, src)]
    return Kc, coef * R[src], ids


def std_dropin_assemble(coords, el_nodes, k_el, int_ent_type, int_ent_id, asse_pos, table, ndof, nnz,
                        fa_of_id, f=1.0, penalty=1e7, g=0.0, con_cnt=None, con_par=None, D_el=None,
                        absolute=False):
    """The table-driven assembly of utr_create_assemble_stiff_mat
    (utd_util/uts_ls_intf.c:3629-3858) over the reference's entity lists:
    each element (type 4, 1-based id) and boundary face (type 3, id mapped by
    ``fa_of_id`` to (element, side)) computes its local matrix
    (std_prism_element / std_prism_face), rewritten through
    std_constraint_rewrite when constraint data is given, and adds entry
    (a, b) at table[pos + a + n b], rhs row a at table[pos + n n + a].
    ``absolute``: sums of |contribution| instead (the comparison scale)."""
    val = np.zeros(nnz)
    rhs = np.zeros(ndof)
    for t, i, pos in zip(int_ent_type, int_ent_id, asse_pos):
        if t == 4:
            e = int(i) - 1
            A = D_el[e] if D_el is not None else k_el[e] * np.eye(3)
            K, R = std_prism_element(coords[el_nodes[e]], A, f)
        else:
            e, side = fa_of_id[int(i)]
            K, R = std_prism_face(coords[el_nodes[e]], side, penalty, g)
        if con_cnt is not None:
            K, R, _ = std_constraint_rewrite(K, R, el_nodes[e], con_cnt, con_par)
        n = K.shape[0]
        tb = table[pos:pos + n * n + n]
        KK = np.abs(K) if absolute else K
        RR = np.abs(R) if absolute else R
        np.add.at(val, tb[:n * n], KK.T.ravel())
        np.add.at(rhs, tb[n * n:], RR)
    return val, rhs


def crs_residual(row_ptr, col_ind, val, x, b=None):
    n = row_ptr.size - 1
    v = np.zeros(n)
    bb = _c(b, np.float64)
    lib().orc_crs_residual(n, _p(row_ptr), _p(col_ind), _p(_c(val, np.float64)), 0 if b is None else 1,
                           _p(bb), _p(_c(x, np.float64)), _p(v))
    return v


def gmres_jacobi(row_ptr, col_ind, val, b, krylov=30, max_iter=1000, tol_rel=1e-8, x0=None):
    n = row_ptr.size - 1
    x = np.zeros(n) if x0 is None else np.array(x0, dtype=np.float64)
    res = ctypes.c_double()
    rel = ctypes.c_double()
    it = lib().orc_gmres_jacobi(n, _p(row_ptr), _p(col_ind), _p(_c(val, np.float64)),
                                _p(_c(b, np.float64)), _p(x), krylov, max_iter, tol_rel,
                                ctypes.cast(ctypes.pointer(res), ctypes.c_void_p),
                                ctypes.cast(ctypes.pointer(rel), ctypes.c_void_p))
    return x, it, res.value, rel.value


def tet_basis_exponents(p):
    """Complete monomial basis xi^a eta^b zeta^c, a+b+c <= p, ordered by total
    degree d, then a descending, then b descending (the library's DG
    tetrahedron order; no reference counterpart)."""
    return [(a, b, d - a - b) for d in range(p + 1) for a in range(d, -1, -1) for b in range(d - a, -1, -1)]


def _collapsed_tet_rule(n):
    """n^3-point rule on the reference tetrahedron by the collapsed (Duffy)
    map xi = u, eta = v (1-u), zeta = w (1-u)(1-v) of Gauss-Legendre points
    on [0,1]^3; exact for polynomials of degree <= 2n - 3."""
    g, w = np.polynomial.legendre.leggauss(n)
    g, w = 0.5 * (g + 1.0), 0.5 * w
    U, V, W = np.meshgrid(g, g, g, indexing="ij")
    WU, WV, WW = np.meshgrid(w, w, w, indexing="ij")
    xi = U
    eta = V * (1.0 - U)
    zeta = W * (1.0 - U) * (1.0 - V)
    wt = WU * WV * WW * (1.0 - U) ** 2 * (1.0 - V)
    return np.stack([xi.ravel(), eta.ravel(), zeta.ravel()], 1), wt.ravel()


def dg_tet_element(X, A, p, f=1.0):
    """DG affine tetrahedron of degree p by quadrature (independent of the
    library's exact moment tables): K[w][u] = int a_ij d_i phi_w d_j phi_u,
    R[w] = int f phi_w.  Returns (K (row w, column u), R)."""
    X = np.asarray(X, np.float64).reshape(4, 3)
    A = np.asarray(A, np.float64).reshape(3, 3)
    J = np.stack([X[1] - X[0], X[2] - X[0], X[3] - X[0]], 1)  # dx/dxi columns
    det = abs(np.linalg.det(J))
    Jit = np.linalg.inv(J).T
    E = np.array(tet_basis_exponents(p), float)
    pts, wts = _collapsed_tet_rule(p + 3)
    phi = np.prod(pts[:, None, :] ** E[None, :, :], axis=2)  # (q, ns)
    dphi = np.zeros((len(pts), len(E), 3))
    for a in range(3):
        Ea = E.copy()
        Ea[:, a] = np.maximum(Ea[:, a] - 1, 0)
        dphi[:, :, a] = E[:, a] * np.prod(pts[:, None, :] ** Ea[None, :, :], axis=2)
    grad = dphi @ Jit.T  # physical gradients (q, ns, 3)
    K = np.einsum("q,qwi,ij,quj->wu", wts * det, grad, A, grad)
    R = f * det * (wts @ phi)
    return K, R


def _collapsed_tri_rule(n):
    """n^2-point rule on the reference triangle (0,0), (1,0), (0,1) by the
    collapsed map s = u, t = v (1 - u) of Gauss-Legendre points on [0,1]^2;
    weights sum to 1/2; exact for degree <= 2n - 2."""
    g, w = np.polynomial.legendre.leggauss(n)
    g, w = 0.5 * (g + 1.0), 0.5 * w
    U, V = np.meshgrid(g, g, indexing="ij")
    WU, WV = np.meshgrid(w, w, indexing="ij")
    return np.stack([U.ravel(), (V * (1.0 - U)).ravel()], 1), (WU * WV * (1.0 - U)).ravel()


def _tet_basis_at(X, p, xs):
    """Values (q, ns) and physical gradients (q, ns, 3) of the complete
    monomial basis of the affine tetrahedron X (4 x 3) at physical points xs."""
    J = np.stack([X[1] - X[0], X[2] - X[0], X[3] - X[0]], 1)
    xi = np.linalg.solve(J, (xs - X[0]).T).T  # reference coordinates
    E = np.array(tet_basis_exponents(p), float)
    phi = np.prod(xi[:, None, :] ** E[None, :, :], axis=2)
    d = np.zeros((len(xi), len(E), 3))
    for a in range(3):
        Ea = E.copy()
        Ea[:, a] = np.maximum(Ea[:, a] - 1, 0)
        d[:, :, a] = E[:, a] * np.prod(xi[:, None, :] ** Ea[None, :, :], axis=2)
    return phi, d @ np.linalg.inv(J)  # grad_x = J^-T grad_xi (row vectors: d J^-1)


def dg_tet_assemble(mesh, faces, pdeg, A, pen=10.0, g=0.0, f=1.0):
    """DG system of an affine tetrahedral mesh with the interior-penalty form
    of the prism DG weak form (pds_conv_diff_weakform_dg.c:232-1140): volume
    blocks from dg_tet_element; per face, rows i (test, side s_i) and columns
    j (trial, side s_j): a [ s_j phi_j (f g_i + s_i c phi_i) - s_i f phi_i g_j ]
    with g = n . (A grad phi), f = 1/2 inside and 1 on (Dirichlet) boundary
    faces, c = pen min(p1, p2) / sqrt(area) (pen p1 / sqrt(area) on the
    boundary), n the unit normal out of el1; boundary rhs g_D a (g_i + c phi_i).
    Quadrature: the collapsed rule above, exact at these degrees.  Returns
    (blocks {(row el, col el): ns_r x ns_c}, rhs list per element)."""
    X = np.asarray(mesh.coords)[np.asarray(mesh.el_nodes)]
    A = np.asarray(A, float).reshape(-1, 3, 3)
    blocks, rhs = {}, []
    for e in range(X.shape[0]):
        K, R = dg_tet_element(X[e], A[e], int(pdeg[e]), f=f)
        blocks[(e, e)] = K
        rhs.append(R.copy())
    for k in range(faces.n):
        e1, e2 = int(faces.el1[k]), int(faces.el2[k])
        V = np.asarray(mesh.coords)[faces.nodes[k, :3]]
        fb, r1 = _tet_face(X, A, pdeg, V, e1, e2, pen, g)
        for key, v in fb.items():
            blocks[key] = blocks.get(key, 0.0) + v
        if r1 is not None:
            rhs[e1] += r1
    return blocks, rhs


def _tet_face(X, A, pdeg, V, e1, e2, pen, g):
    """One face of dg_tet_assemble: blocks {(row el, col el)} and, on the
    boundary, el1's rhs (else None).  X[e]: vertices, A[e]: 3 x 3 tensor."""
    nrm = np.cross(V[1] - V[0], V[2] - V[0])
    area = 0.5 * np.linalg.norm(nrm)
    n = nrm / np.linalg.norm(nrm)
    if np.dot(n, V.mean(0) - X[e1].mean(0)) < 0:
        n = -n
    sides = [e1] + ([e2] if e2 >= 0 else [])
    pmax = max(int(pdeg[s]) for s in sides)
    st, w = _collapsed_tri_rule(pmax + 2)
    xs = V[0] + st[:, :1] * (V[1] - V[0]) + st[:, 1:] * (V[2] - V[0])
    aw = w * 2.0 * area
    if e2 >= 0:
        fac, c = 0.5, pen * min(int(pdeg[e1]), int(pdeg[e2])) / np.sqrt(area)
    else:
        fac, c = 1.0, pen * int(pdeg[e1]) / np.sqrt(area)
    val = {}
    for s, e in enumerate(sides):
        phi, grad = _tet_basis_at(X[e], int(pdeg[e]), xs)
        gg = np.einsum("qjk,lk,l->qj", grad, A[e], n)  # n . (A grad phi)
        val[e] = (1.0 if s == 0 else -1.0, phi, gg)
    blocks = {}
    for ei in sides:
        si, phi_i, g_i = val[ei]
        for ej in sides:
            sj, phi_j, g_j = val[ej]
            blocks[(ei, ej)] = np.einsum("q,qi,qj->ij", aw * sj, fac * g_i + si * c * phi_i, phi_j) \
                - np.einsum("q,qi,qj->ij", aw * si * fac, phi_i, g_j)
    r1 = None
    if e2 < 0:
        _, phi1, g1 = val[e1]
        r1 = g * np.einsum("q,qi->i", aw, g1 + c * phi1)
    return blocks, r1


# ----------------------------------------------------------------------------
# DG systems on meshes of prisms and tetrahedra together.  No reference
# counterpart (the reference's DG module is prism-only): the volume blocks are
# the pinned prism element (dg_prism_element) and the independent tetrahedron
# element (dg_tet_element); prism-prism faces the pinned dg_face,
# tetrahedron-tetrahedron faces the form of dg_tet_assemble, and the faces
# between a prism and a tetrahedron the same form with each side's own basis.
# ----------------------------------------------------------------------------
PRISM_VLOC = np.array([(0, 0, -1), (1, 0, -1), (0, 1, -1), (0, 0, 1), (1, 0, 1), (0, 1, 1)], float)
TET_VLOC = np.array([(0, 0, 0), (1, 0, 0), (0, 1, 0), (0, 0, 1)], float)
DG_TET_NS = (0, 4, 10, 20, 35)


def dg_face_rule(p, ti):
    """The DG module's face rule of degree p (ti 0 triangle, 1 quadrilateral):
    points (s, t) and weights."""
    out = np.zeros(3 * 64)
    nq = lib().orc_dg_face_rule(p, ti, _p(out))
    r = out[:3 * nq].reshape(nq, 3)
    return r[:, :2].copy(), r[:, 2].copy()


def dg_exponents(p):
    """Exponents (a, b, c) of the tensor prism basis of degree p, reference order."""
    out = np.zeros(3 * 128, np.int32)
    ns = lib().orc_dg_exponents(p, _p(out))
    return out[:3 * ns].reshape(ns, 3).copy()


def _monomials(E, e):
    """Values (q, ns) and local gradients (q, ns, 3) of xi^a eta^b zeta^c."""
    E = np.asarray(E, float)
    phi = np.prod(e[:, None, :] ** E[None, :, :], axis=2)
    d = np.zeros((e.shape[0], E.shape[0], 3))
    for a in range(3):
        Ea = E.copy()
        Ea[:, a] = np.maximum(Ea[:, a] - 1, 0)
        d[:, :, a] = E[:, a] * np.prod(e[:, None, :] ** Ea[None, :, :], axis=2)
    return phi, d


def _prism_jacobians(X, e):
    """dx/dxi columns of the linear prism at local points e (q, 3): (q, 3, 3)."""
    xi, eta, z = e[:, 0], e[:, 1], e[:, 2]
    lo, hi, l0 = (1 - z) / 2, (1 + z) / 2, 1 - xi - eta
    dN = np.zeros((e.shape[0], 6, 3))
    dN[:, :, 0] = np.stack([-lo, lo, 0 * z, -hi, hi, 0 * z], 1)
    dN[:, :, 1] = np.stack([-lo, 0 * z, lo, -hi, 0 * z, hi], 1)
    dN[:, :, 2] = 0.5 * np.stack([-l0, -xi, -eta, l0, xi, eta], 1)
    return np.einsum("ia,qib->qab", X, dN)


def _basis_at_local(X, nv, p, e):
    """Values (q, ns) and physical gradients (q, ns, 3) of an element's DG
    basis at local points e: the prism tensor basis (reference order) or the
    tetrahedron's complete basis (tet_basis_exponents)."""
    if nv == 6:
        phi, d = _monomials(dg_exponents(p), e)
        J = _prism_jacobians(X, e)
    else:
        phi, d = _monomials(tet_basis_exponents(p), e)
        J0 = np.stack([X[1] - X[0], X[2] - X[0], X[3] - X[0]], 1)
        J = np.broadcast_to(J0, (e.shape[0], 3, 3))
    return phi, np.einsum("qja,qab->qjb", d, np.linalg.inv(J))


def dg_mixed_face(coords, el_nodes, el_nv, faces, k, pdeg, A, pen=10.0):
    """Blocks {(row el, col el)} of interior triangle face k between any two
    elements: the interior-penalty form of dg_tet_assemble, at the DG
    module's triangle rule of degree max(p1, p2); each side's local point from
    the face-vertex weights (barycentric), n the unit normal out of el1,
    weights 2 area w_q, penalty pen min(p1, p2) / sqrt(area)."""
    e1, e2 = int(faces.el1[k]), int(faces.el2[k])
    assert e2 >= 0 and faces.type[k] == 3
    nodes = faces.nodes[k, :3]
    V = coords[nodes]
    nrm = np.cross(V[1] - V[0], V[2] - V[0])
    area = 0.5 * np.linalg.norm(nrm)
    n = nrm / np.linalg.norm(nrm)
    X1 = coords[el_nodes[e1, :el_nv[e1]]]
    if np.dot(n, V.mean(0) - X1.mean(0)) < 0:
        n = -n
    p1, p2 = int(pdeg[e1]), int(pdeg[e2])
    st, w = dg_face_rule(max(p1, p2), 0)
    bary = np.stack([1 - st[:, 0] - st[:, 1], st[:, 0], st[:, 1]], 1)
    aw = w * 2.0 * area
    fac, c = 0.5, pen * min(p1, p2) / np.sqrt(area)
    val = {}
    for s, e in enumerate((e1, e2)):
        nv = int(el_nv[e])
        X = coords[el_nodes[e, :nv]]
        loc = [int(np.nonzero(el_nodes[e, :nv] == v)[0][0]) for v in nodes]
        vloc = PRISM_VLOC if nv == 6 else TET_VLOC
        el = bary @ vloc[loc]
        phi, grad = _basis_at_local(X, nv, int(pdeg[e]), el)
        gg = grad @ (A[e].reshape(3, 3).T @ n)
        val[e] = (1.0 if s == 0 else -1.0, phi, gg)
    blocks = {}
    for ei in (e1, e2):
        si, phi_i, g_i = val[ei]
        for ej in (e1, e2):
            sj, phi_j, g_j = val[ej]
            blocks[(ei, ej)] = np.einsum("q,qi,qj->ij", aw * sj, fac * g_i + si * c * phi_i, phi_j) \
                - np.einsum("q,qi,qj->ij", aw * si * fac, phi_i, g_j)
    return blocks


def dg_mixed_assemble(mesh, faces, pdeg, A, pen=10.0, g=0.0, f=1.0):
    """The DG system of a MixedMesh (prisms and tetrahedra): blocks {(row el,
    col el)} and the rhs list per element."""
    coords = np.asarray(mesh.coords, float)
    el, nv = np.asarray(mesh.el_nodes), np.asarray(mesh.el_nv)
    A = np.asarray(A, float).reshape(-1, 9)
    blocks, rhs = {}, []
    for e in range(mesh.nel):
        X = coords[el[e, :nv[e]]]
        K, R = (dg_prism_element(X, A[e], int(pdeg[e]), f) if nv[e] == 6 else
                dg_tet_element(X, A[e], int(pdeg[e]), f))
        blocks[(e, e)] = K
        rhs.append(R.copy())

    class _PM:  # the prism-only view dg_face reads
        pass
    pm = _PM()
    pm.coords, pm.el_nodes = coords, el
    for k in range(faces.n):
        e1, e2 = int(faces.el1[k]), int(faces.el2[k])
        if e2 >= 0 and nv[e1] != nv[e2]:
            fb = dg_mixed_face(coords, el, nv, faces, k, pdeg, A, pen)
            for key, v in fb.items():
                blocks[key] = blocks.get(key, 0.0) + v
            continue
        if nv[e1] == 6:
            K, r = dg_face(pm, faces, k, pdeg, A, pen, g)
            n1 = DG_NS[int(pdeg[e1])]
            blocks[(e1, e1)] = blocks[(e1, e1)] + K[:n1, :n1]
            rhs[e1] += r[:n1]
            if e2 >= 0:
                blocks[(e1, e2)] = blocks.get((e1, e2), 0.0) + K[:n1, n1:]
                blocks[(e2, e1)] = blocks.get((e2, e1), 0.0) + K[n1:, :n1]
                blocks[(e2, e2)] = blocks[(e2, e2)] + K[n1:, n1:]
            continue

        Xt = {e1: coords[el[e1, :4]]}
        At = {e1: A[e1].reshape(3, 3)}
        if e2 >= 0:
            Xt[e2], At[e2] = coords[el[e2, :4]], A[e2].reshape(3, 3)
        fb, r1 = _tet_face(Xt, At, pdeg, coords[faces.nodes[k, :3]], e1, e2, pen, g)
        for key, v in fb.items():
            blocks[key] = blocks.get(key, 0.0) + v
        if r1 is not None:
            rhs[e1] += r1
    return blocks, rhs


def _prism_shape(e):
    """Linear prism shape functions (q, 6) at local points e (q, 3)."""
    xi, eta, z = e[:, 0], e[:, 1], e[:, 2]
    lo, hi, l0 = (1 - z) / 2, (1 + z) / 2, 1 - xi - eta
    return np.stack([l0 * lo, xi * lo, eta * lo, l0 * hi, xi * hi, eta * hi], 1)
