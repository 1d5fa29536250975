"""Writes dg_tables.h: the DG prism basis ordering and quadrature rules.

The tensor-product DG basis of ModFEM's apd_dg_prism (apr_shape_fun_3D,
aps_dg_util.c:408-995) consists of monomials xi^a eta^b zeta^c in a fixed
order, and its volume / face quadratures (apr_set_quadr_3D / _2D,
aps_dg_util.c:1415-1560, Gauss-Legendre line rules and Dunavant triangle
rules from aps_gauss_util.c) are fixed point sets.  The CUDA kernels and the
oracle must use exactly the same ordering and points, so this script takes
them from the reference module itself (the harness library built by
``make -C oracle/ref``) and writes them as constant tables:

    python modfem_gb300/csrc/gen_dg_tables.py

Only needed when the tables change; the generated header is committed.
"""
import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

PMAX = 4
MMC_TRIA, MMC_QUAD = 3, 4


def table(out, ctype, name, dims, init):
    """A host table plus its initialiser as a macro (name_INIT), so that CUDA
    code can declare the same values as a __device__ array."""
    out.append("#define %s_INIT \\\n  " % name + init.replace("\n", " \\\n"))
    out.append("static const %s %s%s = %s_INIT;" % (ctype, name, dims, name))


def main():
    import refmod
    L = ctypes.CDLL(refmod.lib_path("dg"))
    vp = ctypes.c_void_p
    L.refh_dg_basis.argtypes = [ctypes.c_int, vp, vp, vp, vp, vp]
    L.refh_dg_quadrature.argtypes = [ctypes.c_int, vp, vp]
    L.refh_dg_face_quadrature.argtypes = [ctypes.c_int, ctypes.c_int, vp, vp]
    rng = np.random.default_rng(0)
    pts = rng.uniform(0.1, 0.4, (4, 3))
    exps, ns, qps, fq = {}, {}, {}, {}
    for p in range(1, PMAX + 1):
        pdeg = 101 * p
        vals = []
        for pt in pts:
            e = np.ascontiguousarray(pt)
            phi = np.zeros(200)
            d = [np.zeros(200) for _ in range(3)]
            n = L.refh_dg_basis(pdeg, e.ctypes.data, phi.ctypes.data, d[0].ctypes.data, d[1].ctypes.data,
                                d[2].ctypes.data)
            vals.append(phi[:n].copy())
        vals = np.array(vals)
        ex = []
        for i in range(n):
            cand = [(a, b, c) for a in range(p + 1) for b in range(p + 1 - a) for c in range(p + 1)
                    if np.allclose(vals[:, i], pts[:, 0] ** a * pts[:, 1] ** b * pts[:, 2] ** c, rtol=1e-13,
                                   atol=0)]
            assert len(cand) == 1, (p, i, cand)
            ex.append(cand[0])
        exps[p], ns[p] = ex, n
        xg = np.zeros(3000)
        wg = np.zeros(1000)
        nq = L.refh_dg_quadrature(pdeg, xg.ctypes.data, wg.ctypes.data)
        qps[p] = (xg[:3 * nq].reshape(nq, 3).copy(), wg[:nq].copy())
        for ft in (MMC_TRIA, MMC_QUAD):
            xg2 = np.zeros(3000)
            wg2 = np.zeros(1000)
            nf = L.refh_dg_face_quadrature(ft, pdeg, xg2.ctypes.data, wg2.ctypes.data)
            fq[(p, ft)] = (xg2[:2 * nf].reshape(nf, 2).copy(), wg2[:nf].copy())
    maxq = max(len(qps[p][1]) for p in qps)
    maxf = max(len(v[1]) for v in fq.values())
    out = []
    out.append("// Generated by gen_dg_tables.py from the reference DG prism module; do not edit.")
    out.append("// Tensor DG prism basis (pdeg = 101 p): monomial exponents (xi, eta, zeta) in the")
    out.append("// reference's order; volume rules (xi, eta, zeta, w); face rules (s, t, w) for")
    out.append("// triangle (0) and quadrilateral (1) faces, coordinates as the reference returns them.")
    out.append("// Each table X also exists as the initialiser macro X_INIT.")
    out.append("#pragma once")
    out.append(f"#define GB_DG_PMAX {PMAX}")
    out.append(f"#define GB_DG_MAXNS {max(ns.values())}")
    out.append(f"#define GB_DG_MAXNQ {maxq}")
    out.append(f"#define GB_DG_MAXNQF {maxf}")
    table(out, "int", "GB_DG_NS", "[GB_DG_PMAX + 1]",
          "{0, " + ", ".join(str(ns[p]) for p in range(1, PMAX + 1)) + "}")
    table(out, "int", "GB_DG_NQ", "[GB_DG_PMAX + 1]",
          "{0, " + ", ".join(str(len(qps[p][1])) for p in range(1, PMAX + 1)) + "}")
    table(out, "int", "GB_DG_NQF", "[GB_DG_PMAX + 1][2]", "{{0, 0}, " + ", ".join(
        "{%d, %d}" % (len(fq[(p, MMC_TRIA)][1]), len(fq[(p, MMC_QUAD)][1])) for p in range(1, PMAX + 1)) + "}")
    rows = []
    for p in range(1, PMAX + 1):
        ex = exps[p] + [(0, 0, 0)] * (max(ns.values()) - ns[p])
        rows.append("  {" + ", ".join("{%d, %d, %d}" % e for e in ex) + "}")
    table(out, "unsigned char", "GB_DG_EXP", "[GB_DG_PMAX][GB_DG_MAXNS][3]", "{\n" + ",\n".join(rows) + "}")
    rows = []
    for p in range(1, PMAX + 1):
        xg, wg = qps[p]
        ent = ["{%.17g, %.17g, %.17g, %.17g}" % (x[0], x[1], x[2], w) for x, w in zip(xg, wg)]
        ent += ["{0, 0, 0, 0}"] * (maxq - len(ent))
        rows.append("  {" + ",\n   ".join(ent) + "}")
    table(out, "double", "GB_DG_QP", "[GB_DG_PMAX][GB_DG_MAXNQ][4]", "{\n" + ",\n".join(rows) + "}")
    rows = []
    for p in range(1, PMAX + 1):
        sub = []
        for ft in (MMC_TRIA, MMC_QUAD):
            xg, wg = fq[(p, ft)]
            ent = ["{%.17g, %.17g, %.17g}" % (x[0], x[1], w) for x, w in zip(xg, wg)]
            ent += ["{0, 0, 0}"] * (maxf - len(ent))
            sub.append("   {" + ",\n    ".join(ent) + "}")
        rows.append("  {\n" + ",\n".join(sub) + "}")
    table(out, "double", "GB_DG_FQ", "[GB_DG_PMAX][2][GB_DG_MAXNQF][3]", "{\n" + ",\n".join(rows) + "}")
    open(os.path.join(HERE, "dg_tables.h"), "w").write("\n".join(out) + "\n")
    print("wrote dg_tables.h", {p: (ns[p], len(qps[p][1])) for p in ns},
          {k: len(v[1]) for k, v in fq.items()}, file=sys.stderr)


if __name__ == "__main__":
    main()
