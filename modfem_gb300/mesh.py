"""Structured prism meshes in ModFEM's numbering, and the jk ("gradmesh") writer.

ModFEM's prism mesh module reads a 2D triangulation plus a layer count
(``mmr_import_mesh_grad``, mmd_prism/mms_prism_input_gradmesh.c:30-560) and
numbers the 3D entities from it:

* node ``istr + lay*N2`` (1-based) sits above 2D node ``istr`` at layer
  ``lay`` (mms_prism_input_gradmesh.c:95-104);
* element ``itri + lay*T`` (1-based) is the prism over 2D triangle ``itri`` in
  layer ``lay`` (:180-190); its vertices, as returned by ``mmr_el_node_coor``
  (mmd_prism/mms_prism_datstr.c:365), are the triangle's three jk nodes on the
  bottom level followed by the same three on the top level;
* horizontal face ``itri + lev*T`` lies at level ``lev`` (0..nlay) (:193-245);
  vertical faces get ids ``T*(nlay+1) + (k-1)*nlay + lay + 1`` for the k-th
  triangle edge met while scanning triangles in order and their edges
  0,1,2, an interior edge being created by the first of its two triangles
  (:258-330).

This module generates the unit-cube mesh of n^3 hexahedra, each split into two
prisms along the same diagonal, directly in that numbering (no file round
trip), and also writes the jk file so the reference can read the same mesh.
"""
import numpy as np

# element sides (reference element coordinates): 0 bottom (zeta=-1),
# 1 top (zeta=+1), 2+i lateral face over triangle edge i (node i -> node i+1)
SIDE_BOTTOM, SIDE_TOP = 0, 1


class PrismMesh:
    """Flat structure-of-arrays prism mesh (0-based indices)."""

    def __init__(self, n, coords, el_nodes, bc_face_id, bc_face_el, bc_face_side, bc_face_bc,
                 ntri, nlay):
        self.n = n
        self.coords = coords            # (nno, 3) float64, row = reference node id - 1
        self.el_nodes = el_nodes        # (nel, 6) int32, 0-based, reference local order
        self.bc_face_id = bc_face_id    # (nbc,) reference face ids (1-based), ascending
        self.bc_face_el = bc_face_el    # (nbc,) 0-based element of each bc face
        self.bc_face_side = bc_face_side
        self.bc_face_bc = bc_face_bc
        self.ntri = ntri
        self.nlay = nlay

    @property
    def nno(self):
        return self.coords.shape[0]

    @property
    def nel(self):
        return self.el_nodes.shape[0]


def _tri_grid(n):
    """2D triangulation of the unit square: (n+1)^2 nodes, 2n^2 triangles.

    Returns node xy, triangle vertex ids (1-based, counter-clockwise) and the
    jk neighbour list (triangle id or -bc) for edges (v0,v1), (v1,v2), (v2,v0).
    """
    N = n + 1
    i, j = np.meshgrid(np.arange(N), np.arange(N), indexing="xy")
    xy = np.stack([i.reshape(-1) / n, j.reshape(-1) / n], axis=1)
    tri = np.zeros((2 * n * n, 3), np.int64)
    nb = np.zeros((2 * n * n, 3), np.int64)
    ii, jj = np.meshgrid(np.arange(n), np.arange(n), indexing="xy")
    ii = ii.reshape(-1)
    jj = jj.reshape(-1)
    a = ii + jj * N + 1
    b = a + 1
    c = a + N + 1
    d = a + N
    t1 = 2 * (ii + jj * n) + 1
    t2 = t1 + 1
    tri[t1 - 1] = np.stack([a, b, c], 1)
    tri[t2 - 1] = np.stack([a, c, d], 1)
    # neighbours of t1: bottom edge a-b, right edge b-c, diagonal c-a
    nb[t1 - 1, 0] = np.where(jj > 0, 2 * (ii + (jj - 1) * n) + 2, -1)
    nb[t1 - 1, 1] = np.where(ii < n - 1, 2 * (ii + 1 + jj * n) + 2, -1)
    nb[t1 - 1, 2] = t2
    # neighbours of t2: diagonal a-c, top edge c-d, left edge d-a
    nb[t2 - 1, 0] = t1
    nb[t2 - 1, 1] = np.where(jj < n - 1, 2 * (ii + (jj + 1) * n) + 1, -1)
    nb[t2 - 1, 2] = np.where(ii > 0, 2 * (ii - 1 + jj * n) + 1, -1)
    return xy, tri, nb


def write_jk(path, n, bc=1, capacity=(0, 0, 0, 0)):
    """Writes the jk file of the n^3-hexahedra unit cube split into prisms.
    ``capacity``: the first line's node, edge, face and element array sizes
    (0: exactly the mesh read; refinement needs room for the new entities)."""
    xy, tri, nb = _tri_grid(n)
    nbj = np.where(nb < 0, -bc, nb)
    with open(path, "w") as f:
        f.write("%d %d %d %d\n" % tuple(capacity))
        f.write(f"{xy.shape[0]} 0.0 1.0 {n} {bc} {bc}\n")
        for x, y in xy:
            f.write(f"{x:.17g} {y:.17g}\n")
        f.write(f"{tri.shape[0]}\n")
        for t in range(tri.shape[0]):
            f.write("1 %d %d %d %d %d %d\n" % (tri[t, 0], tri[t, 1], tri[t, 2],
                                                  nbj[t, 0], nbj[t, 1], nbj[t, 2]))


def structured_prism_mesh(n, jitter=0.0, seed=0, bc=1):
    """Unit cube, n^3 hexahedra x 2 prisms, in ModFEM's numbering.

    ``jitter`` moves every node by U(-jitter*h, +jitter*h) per coordinate
    (h = 1/n), keeping boundary nodes on their boundary planes.
    """
    xy, tri, nb = _tri_grid(n)
    N2 = xy.shape[0]
    T = tri.shape[0]
    nlay = n
    # z = z_bottom + lay*dz with dz = (z_top - z_bottom)/nlay, as the jk reader computes it
    z = 0.0 + np.arange(nlay + 1) * ((1.0 - 0.0) / nlay)
    coords = np.zeros(((nlay + 1) * N2, 3))
    for lay in range(nlay + 1):
        coords[lay * N2:(lay + 1) * N2, 0:2] = xy
        coords[lay * N2:(lay + 1) * N2, 2] = z[lay]
    if jitter > 0.0:
        rng = np.random.default_rng(seed)
        h = 1.0 / n
        d = rng.uniform(-jitter * h, jitter * h, size=coords.shape)
        on_bnd = (np.abs(coords) < 1e-12) | (np.abs(coords - 1.0) < 1e-12)
        d[on_bnd] = 0.0
        coords = coords + d
    tri0 = (tri - 1).astype(np.int64)
    el_nodes = np.zeros((T * nlay, 6), np.int32)
    for lay in range(nlay):
        el_nodes[lay * T:(lay + 1) * T, 0:3] = tri0 + lay * N2
        el_nodes[lay * T:(lay + 1) * T, 3:6] = tri0 + (lay + 1) * N2

    # boundary faces (bc > 0) in ascending reference face id
    fid, fel, fside, fbc = [], [], [], []
    # bottom level: face ids 1..T, element = itri (layer 0), side 0
    fid.append(np.arange(1, T + 1))
    fel.append(np.arange(T))
    fside.append(np.full(T, SIDE_BOTTOM))
    fbc.append(np.full(T, bc))
    # top level: ids nlay*T+1..(nlay+1)*T, element in the last layer, side 1
    fid.append(nlay * T + np.arange(1, T + 1))
    fel.append((nlay - 1) * T + np.arange(T))
    fside.append(np.full(T, SIDE_TOP))
    fbc.append(np.full(T, bc))
    # vertical faces in creation order
    nr_hor = T * (nlay + 1)
    creator = []  # (itri0, edge) for each created vertical face column
    is_bnd = []
    for t in range(T):
        for e in range(3):
            g = nb[t, e]
            if g < 0 or g > t + 1:
                creator.append((t, e))
                is_bnd.append(g < 0)
    creator = np.array(creator, np.int64).reshape(-1, 2)
    is_bnd = np.array(is_bnd, bool)
    k = np.nonzero(is_bnd)[0]  # 0-based creation index of boundary columns
    lay = np.arange(nlay)
    ids = nr_hor + (k[:, None]) * nlay + lay[None, :] + 1
    els = creator[k, 0][:, None] + lay[None, :] * T
    sides = 2 + creator[k, 1][:, None] + 0 * lay[None, :]
    fid.append(ids.reshape(-1))
    fel.append(els.reshape(-1))
    fside.append(sides.reshape(-1))
    fbc.append(np.full(ids.size, bc))
    fid = np.concatenate(fid).astype(np.int32)
    order = np.argsort(fid, kind="stable")
    return PrismMesh(n, coords, el_nodes, fid[order],
                     np.concatenate(fel)[order].astype(np.int32),
                     np.concatenate(fside)[order].astype(np.int32),
                     np.concatenate(fbc)[order].astype(np.int32), T, nlay)


def lognormal_k(nel, seed=0, mu=0.0, sigma=1.0):
    """Per-element diffusion coefficient k ~ lognormal(mu, sigma) from a seed."""
    return np.random.default_rng(seed + 7919).lognormal(mu, sigma, nel)


def prism_min_detj(mesh):
    """Smallest Jacobian determinant over the 6 std quadrature points."""
    X = mesh.coords[mesh.el_nodes]  # (nel, 6, 3)
    a0, a1, a2, b0, b1, b2 = [X[:, i, :] for i in range(6)]
    m1 = 0.5 * ((a1 - a0) + (b1 - b0))
    d1 = 0.5 * ((b1 - b0) - (a1 - a0))
    m2 = 0.5 * ((a2 - a0) + (b2 - b0))
    d2 = 0.5 * ((b2 - b0) - (a2 - a0))
    c0 = 0.5 * (b0 - a0)
    g = 0.577350269189626
    pts = [(1 / 6, 1 / 6), (1 / 6, 2 / 3), (2 / 3, 1 / 6)]
    dmin = np.inf
    for zeta in (-g, g):
        for (xi, eta) in pts:
            jx = m1 + zeta * d1
            jy = m2 + zeta * d2
            jz = c0 + xi * d1 + eta * d2
            det = np.einsum("ij,ij->i", jx, np.cross(jy, jz))
            dmin = min(dmin, det.min())
    return dmin


class TetMesh:
    """Flat tetrahedral mesh (0-based), vertices in positive orientation."""

    def __init__(self, n, coords, el_nodes):
        self.n = n
        self.coords = coords
        self.el_nodes = el_nodes
        self.bc_face_id = np.zeros(0, np.int32)
        self.bc_face_el = np.zeros(0, np.int32)
        self.bc_face_side = np.zeros(0, np.int32)
        self.bc_face_bc = np.zeros(0, np.int32)

    @property
    def nno(self):
        return self.coords.shape[0]

    @property
    def nel(self):
        return self.el_nodes.shape[0]


# the six tetrahedra of a cube around its main diagonal (corner b = dx + 2 dy + 4 dz)
_KUHN = np.array([[0, 1, 3, 7], [0, 1, 5, 7], [0, 2, 3, 7], [0, 2, 6, 7], [0, 4, 5, 7], [0, 4, 6, 7]])


def structured_tet_mesh(n, jitter=0.0, seed=0):
    """Unit cube, n^3 hexahedra x 6 tetrahedra (Kuhn split), nodes numbered
    x fastest, then y, then z; jitter keeps boundary nodes on their planes."""
    N = n + 1
    i, j, k = np.meshgrid(np.arange(N), np.arange(N), np.arange(N), indexing="ij")
    coords = np.stack([i.T.reshape(-1), j.T.reshape(-1), k.T.reshape(-1)], 1) / n
    if jitter > 0.0:
        rng = np.random.default_rng(seed)
        d = rng.uniform(-jitter / n, jitter / n, size=coords.shape)
        on_bnd = (np.abs(coords) < 1e-12) | (np.abs(coords - 1.0) < 1e-12)
        d[on_bnd] = 0.0
        coords = coords + d
    ci, cj, ck = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    ci, cj, ck = ci.T.reshape(-1), cj.T.reshape(-1), ck.T.reshape(-1)
    corner = np.zeros((ci.size, 8), np.int64)
    for b in range(8):
        dx, dy, dz = b & 1, (b >> 1) & 1, (b >> 2) & 1
        corner[:, b] = (ci + dx) + (cj + dy) * N + (ck + dz) * N * N
    el = corner[:, _KUHN].reshape(-1, 4)
    X = coords[el]
    det = np.einsum("ij,ij->i", X[:, 1] - X[:, 0], np.cross(X[:, 2] - X[:, 0], X[:, 3] - X[:, 0]))
    flip = det < 0
    el[flip, 2], el[flip, 3] = el[flip, 3].copy(), el[flip, 2].copy()
    return TetMesh(n, coords, el.astype(np.int32))


def random_rotations(n, seed=0):
    """n seeded random rotation matrices (QR of Gaussian matrices, det +1)."""
    rng = np.random.default_rng(seed + 104729)
    Q, R = np.linalg.qr(rng.standard_normal((n, 3, 3)))
    Q = Q * np.sign(np.diagonal(R, axis1=1, axis2=2))[:, None, :]
    det = np.linalg.det(Q)
    Q[det < 0, :, 0] *= -1.0
    return Q


def anisotropic_tensors(n, seed=0, eig=(1.0, 0.1, 0.01)):
    """D = R diag(eig) R^T per element with seeded random rotations R,
    row-major 9 values per element."""
    Q = random_rotations(n, seed)
    D = np.einsum("nij,j,nkj->nik", Q, np.asarray(eig, float), Q)
    return D.reshape(n, 9)


class FaceTable:
    """All faces of a structured prism mesh in the reference's numbering.

    id (1-based), type (3 triangle, 4 quadrilateral), bc flag (> 0 boundary
    condition, 0 / -1 interior), el1 / el2 (0-based, el2 = -1 on the
    boundary), side1 / side2 (element sides), nodes (4 vertex indices, 0-based,
    -1 padded) in the order of mmr_fa_node_coor (mmd_prism/
    mms_prism_datstr.c:1488), which fixes the diagonal mmr_fa_area
    (mms_prism_datstr.c:1732-1790) splits a quadrilateral along.
    """

    def __init__(self, **kw):
        self.__dict__.update(kw)

    @property
    def n(self):
        return self.id.size


def prism_faces(mesh, bc=1):
    """Full face table of structured_prism_mesh(n) (see mmr_import_mesh_grad,
    mms_prism_input_gradmesh.c:193-330, for the numbering)."""
    n = mesh.n
    _, tri, nb = _tri_grid(n)
    T = tri.shape[0]
    nlay = mesh.nlay
    N2 = (n + 1) ** 2
    tri0 = tri - 1
    rows = []
    # horizontal faces, level by level
    for lev in range(nlay + 1):
        for t in range(T):
            fid = t + 1 + lev * T
            v = tri0[t] + lev * N2
            if lev == 0:
                rows.append((fid, 3, bc, t, -1, 0, 0, v[0], v[2], v[1], -1))
            elif lev == nlay:
                rows.append((fid, 3, bc, t + (nlay - 1) * T, -1, 1, 0, v[0], v[1], v[2], -1))
            else:
                rows.append((fid, 3, 0, t + (lev - 1) * T, t + lev * T, 1, 0, v[0], v[1], v[2], -1))
    # vertical faces in creation order
    nr_hor = T * (nlay + 1)
    k = 0
    for t in range(T):
        for e in range(3):
            g = nb[t, e]
            if not (g < 0 or g > t + 1):
                continue
            a, b = tri0[t, e], tri0[t, (e + 1) % 3]
            if g < 0:
                el2s = None
            else:
                gi = g - 1
                back = [j for j in range(3) if nb[gi, j] == t + 1][0]
                el2s = (gi, 2 + back)
            for lay in range(nlay):
                fid = nr_hor + k * nlay + lay + 1
                v = np.array([a, b, b + N2, a + N2]) + lay * N2
                if el2s is None:
                    rows.append((fid, 4, bc, t + lay * T, -1, 2 + e, 0, *v))
                else:
                    rows.append((fid, 4, -1, t + lay * T, el2s[0] + lay * T, 2 + e, el2s[1], *v))
            k += 1
    arr = np.array(rows, dtype=np.int64)
    arr = arr[np.argsort(arr[:, 0], kind="stable")]
    return FaceTable(id=arr[:, 0].astype(np.int32), type=arr[:, 1].astype(np.int32),
                     bc=arr[:, 2].astype(np.int32), el1=arr[:, 3].astype(np.int32),
                     el2=arr[:, 4].astype(np.int32), side1=arr[:, 5].astype(np.int32),
                     side2=arr[:, 6].astype(np.int32), nodes=arr[:, 7:11].astype(np.int32))


# local faces of a tetrahedron: side k is the face opposite local vertex k
TET_SIDES = ((1, 2, 3), (0, 2, 3), (0, 1, 3), (0, 1, 2))


def tet_faces(mesh, bc=1):
    """Face table of a tetrahedral mesh in the format of prism_faces: every
    face once, el1 the lower-numbered neighbour and side1 its local face
    (opposite vertex side1), nodes in el1's local order of that face; type 3;
    bc on the boundary, -1 inside.  Faces ordered by (el1, side1)."""
    el = np.asarray(mesh.el_nodes, np.int64)
    nel = el.shape[0]
    sides = np.array(TET_SIDES)
    verts = el[:, sides]                        # (nel, 4, 3) in local face order
    key = np.sort(verts, axis=2).reshape(-1, 3)
    owner = np.repeat(np.arange(nel), 4)
    side = np.tile(np.arange(4), nel)
    order = np.lexsort((owner, key[:, 2], key[:, 1], key[:, 0]))
    ks = key[order]
    same = np.all(ks[1:] == ks[:-1], axis=1)
    first = np.ones(len(order), bool)
    first[1:] = ~same
    second = np.zeros(len(order), bool)
    second[:-1] = same                          # the next entry is this face's second neighbour
    idx1 = order[first]
    has2 = second[first]
    idx2 = np.full(idx1.size, -1)
    pos_first = np.nonzero(first)[0]
    idx2[has2] = order[pos_first[has2] + 1]
    e1, s1 = owner[idx1], side[idx1]
    e2 = np.where(idx2 >= 0, owner[np.maximum(idx2, 0)], -1)
    s2 = np.where(idx2 >= 0, side[np.maximum(idx2, 0)], 0)
    srt = np.lexsort((s1, e1))
    e1, s1, e2, s2 = e1[srt], s1[srt], e2[srt], s2[srt]
    nodes = np.full((e1.size, 4), -1, np.int64)
    nodes[:, :3] = verts[e1, s1]
    n = e1.size
    return FaceTable(id=np.arange(1, n + 1, dtype=np.int32), type=np.full(n, 3, np.int32),
                     bc=np.where(e2 >= 0, -1, bc).astype(np.int32), el1=e1.astype(np.int32),
                     el2=e2.astype(np.int32), side1=s1.astype(np.int32), side2=s2.astype(np.int32),
                     nodes=nodes.astype(np.int32))


# local faces of a prism in the orientation of prism_faces (side 0 bottom
# seen from below, 1 top, 2 + e the lateral face over triangle edge e)
PRISM_SIDES = ((0, 2, 1), (3, 4, 5), (0, 1, 4, 3), (1, 2, 5, 4), (2, 0, 3, 5))


class MixedMesh:
    """Prisms and tetrahedra in one mesh (0-based): el_nodes (nel, 6) with a
    tetrahedron's 4 vertices first and -1 after them, el_nv (nel,) 6 or 4."""

    def __init__(self, n, coords, el_nodes, el_nv, n_prism_layers):
        self.n = n
        self.coords = coords
        self.el_nodes = el_nodes
        self.el_nv = el_nv
        self.n_prism_layers = n_prism_layers
        self.bc_face_id = np.zeros(0, np.int32)
        self.bc_face_el = np.zeros(0, np.int32)
        self.bc_face_side = np.zeros(0, np.int32)
        self.bc_face_bc = np.zeros(0, np.int32)

    @property
    def nno(self):
        return self.coords.shape[0]

    @property
    def nel(self):
        return self.el_nodes.shape[0]


def structured_mixed_mesh(n, prism_layers, jitter=0.0, seed=0):
    """Unit cube of n^3 hexahedra: the lower `prism_layers` layers split into
    two prisms each (structured_prism_mesh), the layers above into six
    tetrahedra each (structured_tet_mesh's Kuhn split).  Both splits cut the
    horizontal squares along the same diagonal, so the prisms' top triangles
    are the tetrahedra's bottom faces.  One node grid (x fastest, then y,
    then z), prisms first, then tetrahedra; jitter keeps boundary nodes on
    their planes."""
    assert 0 < prism_layers < n
    pm = structured_prism_mesh(n, jitter=jitter, seed=seed)
    tm = structured_tet_mesh(n, jitter=0.0)
    T = 2 * n * n
    prisms = pm.el_nodes[:prism_layers * T]
    per_layer = 6 * n * n
    tets = tm.el_nodes[prism_layers * per_layer:]
    # the tetrahedra's orientation check on the jittered coordinates
    X = pm.coords[tets]
    det = np.einsum("ij,ij->i", X[:, 1] - X[:, 0], np.cross(X[:, 2] - X[:, 0], X[:, 3] - X[:, 0]))
    tets = tets.copy()
    flip = det < 0
    tets[flip, 2], tets[flip, 3] = tets[flip, 3].copy(), tets[flip, 2].copy()
    el = np.full((prisms.shape[0] + tets.shape[0], 6), -1, np.int32)
    el[:prisms.shape[0]] = prisms
    el[prisms.shape[0]:, :4] = tets
    nv = np.concatenate([np.full(prisms.shape[0], 6), np.full(tets.shape[0], 4)]).astype(np.int32)
    return MixedMesh(n, pm.coords, el, nv, prism_layers)


def mixed_faces(mesh, bc=1):
    """Face table of a MixedMesh in the format of prism_faces: every face
    once, el1 the lower-numbered neighbour and side1 its local face (prisms:
    PRISM_SIDES, tetrahedra: TET_SIDES), nodes in el1's local order of that
    face; type 3 or 4; bc on the boundary, -1 inside.  Ordered by (el1,
    side1).  Faces are matched by their sorted vertex sets (numpy sorts, no
    per-face loop)."""
    el, nv = np.asarray(mesh.el_nodes), np.asarray(mesh.el_nv)
    parts_e, parts_s, parts_v = [], [], []
    for typ, sides in ((6, PRISM_SIDES), (4, TET_SIDES)):
        es = np.nonzero(nv == typ)[0]
        for s, loc in enumerate(sides):
            v = np.full((es.size, 4), -1, np.int64)
            v[:, :len(loc)] = el[es][:, list(loc)]
            parts_e.append(es)
            parts_s.append(np.full(es.size, s, np.int64))
            parts_v.append(v)
    E, S, V = np.concatenate(parts_e), np.concatenate(parts_s), np.concatenate(parts_v)
    K = np.sort(np.where(V >= 0, V, np.iinfo(np.int64).max), axis=1)
    order = np.lexsort((E, K[:, 3], K[:, 2], K[:, 1], K[:, 0]))
    Ks = K[order]
    first = np.nonzero(np.all(Ks[1:] == Ks[:-1], axis=1))[0]  # a face met twice: rows i, i + 1
    paired = np.zeros(order.size, bool)
    paired[first] = True
    paired[first + 1] = True
    single = np.nonzero(~paired)[0]
    i1 = np.concatenate([order[first], order[single]])
    i2 = np.concatenate([order[first + 1], np.full(single.size, -1)])
    e1, s1 = E[i1], S[i1]
    e2 = np.where(i2 >= 0, E[np.maximum(i2, 0)], -1)
    s2 = np.where(i2 >= 0, S[np.maximum(i2, 0)], 0)
    srt = np.lexsort((s1, e1))
    e1, s1, e2, s2, nodes = e1[srt], s1[srt], e2[srt], s2[srt], V[i1][srt]
    nf = e1.size
    return FaceTable(id=np.arange(1, nf + 1, dtype=np.int32), type=(nodes >= 0).sum(1).astype(np.int32),
                     bc=np.where(e2 >= 0, -1, bc).astype(np.int32), el1=e1.astype(np.int32),
                     el2=e2.astype(np.int32), side1=s1.astype(np.int32), side2=s2.astype(np.int32),
                     nodes=nodes.astype(np.int32))
