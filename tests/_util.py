"""Shared helpers for the parity tests: golden fixtures and error measures."""
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")

# Parity tolerance for FP64 values: relative to the entry, with entries that
# are cancellation-dominated (below 1e-3 of their row's largest magnitude)
# measured against that floor instead.
REL_TOL = 1e-12
FLOOR = 1e-3


def load(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))


class FixtureMesh:
    """Mesh object with the attributes the library binding and oracle use."""

    def __init__(self, g):
        self.coords = g["coords"]
        self.el_nodes = g["el_nodes"].astype(np.int32)
        self.bc_face_id = g["bc_face_id"].astype(np.int32)
        self.bc_face_el = g["bc_face_el"].astype(np.int32)
        self.bc_face_bc = g["bc_face_bc"].astype(np.int32)
        # side from the numbering rule (checked against the generator in test_mesh)
        from modfem_gb300.mesh import structured_prism_mesh
        m = structured_prism_mesh(int(g["n"]), jitter=float(g["jitter"]), seed=int(g["seed"]))
        self.bc_face_side = m.bc_face_side

    @property
    def nno(self):
        return self.coords.shape[0]

    @property
    def nel(self):
        return self.el_nodes.shape[0]


class RefinedMesh:
    """A refined std prism mesh of a fixture made by the reference's own
    refinement (tests/golden/make_golden.py run_hanging): every element id
    the mesh module holds (refined parents included, only active ones are
    in the entity lists), the active boundary faces with their sides, and
    the constraint data of the hanging vertices."""

    def __init__(self, g):
        self.coords = g["coords"]
        self.el_nodes = g["el_nodes"].astype(np.int32)
        self.bc_face_id = g["bc_face_id"].astype(np.int32)
        self.bc_face_el = g["bc_face_el"].astype(np.int32)
        self.bc_face_bc = g["bc_face_bc"].astype(np.int32)
        self.bc_face_side = g["bc_face_side"].astype(np.int32)
        cnt = g["con_cnt"]
        self.con_vertex = np.nonzero(cnt > 0)[0].astype(np.int32)
        self.con_nr = cnt[self.con_vertex].astype(np.int32)
        self.con_par = g["con_par"][self.con_vertex].astype(np.int32)
        self.fa_of_id = {int(i): (int(e), int(s)) for i, e, s in
                         zip(self.bc_face_id, self.bc_face_el, self.bc_face_side)}

    @property
    def nno(self):
        return self.coords.shape[0]

    @property
    def nel(self):
        return self.el_nodes.shape[0]


def crs_rel_err(row_ptr, a, b, scale=None):
    """Assembled-value error.

    With ``scale`` (the per-entry sum of absolute element contributions,
    oracle.std_prism_assemble_abs): max |a-b| / scale.  An assembled value is
    a sum of element contributions, each exact to FP64 rounding relative to
    itself; where the sum cancels, no two summation orders agree relative to
    the sum, so the sum of magnitudes is the scale the 1e-12 applies to.  For
    entries without cancellation (scale == |b|) this is the plain relative
    error.  Without ``scale``: max |a-b| / max(|b|, FLOOR * max|row of b|)."""
    if scale is not None:
        den = np.where(scale > 0, scale, 1.0)
        return float(np.max(np.abs(a - b) / den)) if a.size else 0.0
    n = row_ptr.size - 1
    rows = np.repeat(np.arange(n), np.diff(row_ptr))
    rowmax = np.zeros(n)
    np.maximum.at(rowmax, rows, np.abs(b))
    den = np.maximum(np.abs(b), FLOOR * rowmax[rows])
    den[den == 0] = 1.0
    return float(np.max(np.abs(a - b) / den)) if a.size else 0.0


def mat_rel_err(a, b):
    """Local (element or face) matrices: max |a_ij - b_ij| / sqrt(|b_ii| |b_jj|),
    the energy-scale measure of crs_rel_err / energy_scale applied to one
    local matrix (plain relative error on the diagonal).  Rows without a
    diagonal (vertices off a boundary face) are compared against |b_ij|."""
    d = np.sqrt(np.abs(np.diag(b)))
    den = np.outer(d, d)
    den = np.where(den > 0, den, np.abs(b))
    err = np.abs(a - b)
    ok = den > 0
    if np.any(err[~ok] != 0):
        return float("inf")
    return float(np.max(err[ok] / den[ok])) if np.any(ok) else 0.0


def vec_rel_err(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def abs_scale(mesh, k, dof_of_node, row_ptr, col_ind, **kw):
    """Per-entry sum of |element contributions| from the oracle."""
    import oracle as O
    sv, sr, _ = O.std_prism_assemble_abs(mesh, k, dof_of_node, row_ptr, col_ind, **kw)
    return sv


def energy_scale(row_ptr, col_ind, b):
    """sqrt(|b_rr| |b_cc|) per CRS entry: the Cauchy-Schwarz bound of an entry
    of a symmetric positive semi-definite matrix, i.e. the size of the entry in
    the energy inner product.  Entry (r, c) of a stiffness matrix is an
    integral of k grad(phi_r).grad(phi_c), a sum of dot products whose
    rounding error is proportional to |grad phi_r||grad phi_c|, so this is the
    scale a relative tolerance applies to; for diagonal entries it is the
    entry itself."""
    n = row_ptr.size - 1
    rows = np.repeat(np.arange(n), np.diff(row_ptr))
    diag = np.zeros(n)
    isd = rows == col_ind
    diag[rows[isd]] = np.abs(b[isd])
    return np.sqrt(diag[rows] * diag[col_ind])


def face_rel_err(a, b):
    """Non-symmetric local matrices (DG face blocks): max |a_ij - b_ij| /
    sqrt(R_i C_j) with R_i, C_j the largest magnitudes of row i and column j
    of b (the scale of the dot products entry (i, j) sums).  Functions that
    vanish on the face make some diagonals zero, so the energy scale of
    mat_rel_err does not apply; rows and columns that are zero in b must be
    zero in a."""
    R = np.abs(b).max(axis=1)
    C = np.abs(b).max(axis=0)
    den = np.sqrt(np.outer(R, C))
    err = np.abs(a - b)
    ok = den > 0
    if np.any(err[~ok] != 0):
        return float("inf")
    return float(np.max(err[ok] / den[ok])) if np.any(ok) else 0.0


def dg_blocks_to_crs(off, bptr, bcol, boff, vals):
    """Scalar expansion (sorted columns, every block entry) of the library's
    variable-block storage: column-major blocks, leading dimension the row
    block's size."""
    rp = [0]
    ci, out = [], []
    for e in range(off.size - 1):
        ns = off[e + 1] - off[e]
        blocks, cidx = [], []
        for k in range(bptr[e], bptr[e + 1]):
            c = bcol[k]
            nc = off[c + 1] - off[c]
            blocks.append(vals[boff[k]:boff[k + 1]].reshape(nc, ns).T)
            cidx.append(np.arange(off[c], off[c + 1]))
        row = np.concatenate(blocks, axis=1)
        cidx = np.concatenate(cidx)
        for i in range(ns):
            ci.append(cidx)
            out.append(row[i])
            rp.append(rp[-1] + cidx.size)
    return np.array(rp, np.int64), np.concatenate(ci).astype(np.int64), np.concatenate(out)


def sparse_rel_err(row_ptr, col_ind, a, b):
    """Assembled matrices without a usable diagonal scale (DG blocks):
    max |a_ij - b_ij| / sqrt(R_i C_j) with R_i, C_j the largest magnitudes in
    row i and column j of b."""
    n = row_ptr.size - 1
    rows = np.repeat(np.arange(n), np.diff(row_ptr))
    R = np.zeros(n)
    C = np.zeros(n)
    np.maximum.at(R, rows, np.abs(b))
    np.maximum.at(C, col_ind, np.abs(b))
    den = np.sqrt(R[rows] * C[col_ind])
    err = np.abs(a - b)
    ok = den > 0
    if np.any(err[~ok] != 0):
        return float("inf")
    return float(np.max(err[ok] / den[ok])) if np.any(ok) else 0.0
