"""The element math of the CUDA kernels (host+device header), compiled for the
host with nvcc and checked against the oracle on the CPU."""
import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

import oracle as O
from _util import mat_rel_err

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "hostcheck", "prism_math_host.cu")
HDRS = [os.path.join(HERE, "..", "modfem_gb300", "csrc", h) for h in ("prism_std.cuh", "prism_dw.cuh", "dword.cuh")]
LIB = os.path.join(HERE, "hostcheck", "libprism_math_host.so")


@pytest.fixture(scope="module")
def hostlib():
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(f) for f in [SRC] + HDRS):
        subprocess.check_call([nvcc, "-O2", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off", "-shared", "-o",
                               LIB, SRC])
    L = ctypes.CDLL(LIB)
    for fn in (L.host_prism_std_element, L.host_prism_std_element_dw):
        fn.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p]
    L.host_dw_roundtrip.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
    L.host_dw_ops.argtypes = [ctypes.c_int, ctypes.c_int] + [ctypes.c_void_p] * 5
    L.host_dwacc_dot.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
    L.host_dwacc_dot.restype = ctypes.c_double
    return L


def unpack(K21):
    K = np.zeros((6, 6))
    k = 0
    for u in range(6):
        for w in range(u, 6):
            K[u, w] = K[w, u] = K21[k]
            k += 1
    return K


def test_prism_element_math_vs_oracle(hostlib):
    from modfem_gb300.mesh import lognormal_k, structured_prism_mesh
    m = structured_prism_mesh(6, jitter=0.25, seed=12)
    k = lognormal_k(m.nel, seed=12)
    worst = 0.0
    for e in range(m.nel):
        X = np.ascontiguousarray(m.coords[m.el_nodes[e]]).reshape(-1)
        K21 = np.zeros(21)
        R = np.zeros(6)
        hostlib.host_prism_std_element(X.ctypes.data, k[e], 1.3, K21.ctypes.data, R.ctypes.data)
        Ko, Ro = O.std_prism_element(X, np.diag([k[e]] * 3), 1.3)
        worst = max(worst, mat_rel_err(unpack(K21), Ko))
        assert np.max(np.abs(R - Ro)) <= 1e-13 * np.max(np.abs(Ro))
    assert worst < 1e-13, worst


def test_prism_element_math_double_word(hostlib):
    """The double-word form of the same element math (float pairs): within
    1e-13 of the oracle's FP64 matrix on jittered elements of a fine mesh
    (h = 1/200, determinants near 1e-7) with lognormal k, and on distorted
    elements over four decades of size."""
    from modfem_gb300.mesh import lognormal_k, structured_prism_mesh
    m = structured_prism_mesh(200, jitter=0.25, seed=7)
    k = lognormal_k(m.nel, seed=7)
    rng = np.random.default_rng(7)
    worst = worst_r = 0.0
    for e in rng.choice(m.nel, 400, replace=False):
        X = np.ascontiguousarray(m.coords[m.el_nodes[e]]).reshape(-1)
        K21, R = np.zeros(21), np.zeros(6)
        hostlib.host_prism_std_element_dw(X.ctypes.data, k[e], 1.3, K21.ctypes.data, R.ctypes.data)
        Ko, Ro = O.std_prism_element(X, np.diag([k[e]] * 3), 1.3)
        worst = max(worst, mat_rel_err(unpack(K21), Ko))
        worst_r = max(worst_r, np.max(np.abs(R - Ro)) / np.max(np.abs(Ro)))
    assert worst < 1e-13 and worst_r < 1e-13, (worst, worst_r)
    base = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1], [1, 0, 1], [0, 1, 1]], float)
    for _ in range(200):
        X = (base + rng.uniform(-0.2, 0.2, base.shape)) * 10.0 ** rng.uniform(-3, 1)
        X = np.ascontiguousarray(X).reshape(-1)
        K21, R = np.zeros(21), np.zeros(6)
        hostlib.host_prism_std_element_dw(X.ctypes.data, 2.5, 1.0, K21.ctypes.data, R.ctypes.data)
        Ko, Ro = O.std_prism_element(X, np.diag([2.5] * 3), 1.0)
        assert mat_rel_err(unpack(K21), Ko) < 1e-13
        assert np.max(np.abs(R - Ro)) <= 1e-13 * np.max(np.abs(Ro))
        # far from the origin the FP64 vertex differences (shared by both
        # forms) dominate the error: compare with the FP64 form
        X = np.ascontiguousarray(X + np.tile(rng.uniform(-5, 5, 3), 6))
        K64, R64 = np.zeros(21), np.zeros(6)
        hostlib.host_prism_std_element(X.ctypes.data, 2.5, 1.0, K64.ctypes.data, R64.ctypes.data)
        hostlib.host_prism_std_element_dw(X.ctypes.data, 2.5, 1.0, K21.ctypes.data, R.ctypes.data)
        assert mat_rel_err(unpack(K21), unpack(K64)) < 1e-13
        assert np.max(np.abs(R - R64)) <= 1e-13 * np.max(np.abs(R64))


def test_double_word_conversions(hostlib):
    """double -> float pair keeps 47+ bits (the pair's sum differs from the
    double by at most 2^-47 of it) on [2^-74, 2^127), the high word alone
    down to 2^-126; float pair -> double is exact when the pair's bits fit
    53; zero maps to zero."""
    rng = np.random.default_rng(1)
    x = np.concatenate([rng.standard_normal(2000) * 10.0 ** rng.uniform(-20, 20, 2000),
                        [0.0, -0.0, 1.0, -1.0, 2.0 ** -80, 3e-30, -7e35, 1e-3]])
    hl = np.zeros(2 * x.size, np.float32)
    back = np.zeros(x.size)
    hostlib.host_dw_roundtrip(x.ctypes.data, x.size, hl.ctypes.data, back.ctypes.data)
    h, l = hl[0::2].astype(np.float64), hl[1::2].astype(np.float64)
    nz = x != 0
    fit = nz & (np.abs(x) >= 2.0 ** -74) & (np.abs(x) < 2.0 ** 127)  # pairs of normal floats
    small = nz & ~fit & (np.abs(x) >= 2.0 ** -126)                    # high word only
    assert np.all(np.abs((h + l - x)[fit]) <= 2.0 ** -47 * np.abs(x[fit]))
    assert np.all(np.abs((h + l - x)[small]) <= 2.0 ** -23 * np.abs(x[small]))
    assert np.all(back[~nz] == 0)
    assert np.all(np.abs((back - (h + l))[fit]) <= 2.0 ** -52 * np.abs(x[fit]))
    assert np.all(np.abs((back - x)[fit | small]) <= 2.0 ** -23 * np.abs(x[fit | small]))


def test_prism_element_math_distorted(hostlib):
    rng = np.random.default_rng(3)
    base = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1], [1, 0, 1], [0, 1, 1]], float)
    for _ in range(200):
        X = (base + rng.uniform(-0.2, 0.2, base.shape)) * rng.uniform(1e-3, 10)
        X = np.ascontiguousarray(X).reshape(-1)
        K21 = np.zeros(21)
        R = np.zeros(6)
        hostlib.host_prism_std_element(X.ctypes.data, 2.5, 1.0, K21.ctypes.data, R.ctypes.data)
        Ko, Ro = O.std_prism_element(X, np.diag([2.5] * 3), 1.0)
        assert mat_rel_err(unpack(K21), Ko) < 1e-13
        assert np.max(np.abs(R - Ro)) <= 1e-13 * np.max(np.abs(Ro))


DG_SRC = os.path.join(HERE, "hostcheck", "dg_face_host.cu")
DG_HDR = os.path.join(HERE, "..", "modfem_gb300", "csrc", "dg_face.cuh")
DG_LIB = os.path.join(HERE, "hostcheck", "libdg_face_host.so")


@pytest.fixture(scope="module")
def dghost():
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    if not os.path.exists(DG_LIB) or os.path.getmtime(DG_LIB) < max(os.path.getmtime(DG_SRC),
                                                                     os.path.getmtime(DG_HDR)):
        subprocess.check_call([nvcc, "-O2", "-std=c++17", "-Xcompiler", "-fPIC", "-shared", "-o", DG_LIB, DG_SRC])
    L = ctypes.CDLL(DG_LIB)
    vp = ctypes.c_void_p
    L.host_dg_face.argtypes = [ctypes.c_int, vp, vp, ctypes.c_int, vp, ctypes.c_int, vp, vp, ctypes.c_int, vp,
                               ctypes.c_double, ctypes.c_double, vp, vp]
    return L


def _host_face(L, m, F, i, pdeg, A, pen, g):
    e1, e2 = int(F.el1[i]), int(F.el2[i])
    fn = F.nodes[i]
    X1 = np.ascontiguousarray(m.coords[m.el_nodes[e1]]).reshape(-1)
    l1 = O.face_local_vertices(m.el_nodes[e1], fn)
    A1 = np.ascontiguousarray(A[e1], dtype=np.float64)
    p1 = int(pdeg[e1])
    n = O.lib().orc_dg_nshape(p1)
    X2 = l2 = A2 = None
    p2 = 1
    if e2 >= 0:
        X2 = np.ascontiguousarray(m.coords[m.el_nodes[e2]]).reshape(-1)
        l2 = O.face_local_vertices(m.el_nodes[e2], fn)
        A2 = np.ascontiguousarray(A[e2], dtype=np.float64)
        p2 = int(pdeg[e2])
        n += O.lib().orc_dg_nshape(p2)
    sm = np.zeros(n * n)
    rhs = np.zeros(n)
    ptr = lambda a: None if a is None else a.ctypes.data
    L.host_dg_face(int(F.type[i]), ptr(X1), ptr(l1), p1, ptr(A1), int(F.side1[i]), ptr(X2), ptr(l2), p2, ptr(A2),
                   pen, g, sm.ctypes.data, rhs.ctypes.data)
    return sm.reshape(n, n).T.copy(), rhs


@pytest.mark.parametrize("aniso", [False, True])
def test_dg_face_row_form_vs_oracle(dghost, aniso):
    """The per-owner row form of the DG face kernel against the oracle's
    term-by-term face integral, every face of a jittered mixed-degree mesh."""
    from _util import face_rel_err, vec_rel_err
    from modfem_gb300.mesh import anisotropic_tensors, lognormal_k, prism_faces, structured_prism_mesh
    m = structured_prism_mesh(3, jitter=0.25, seed=5)
    F = prism_faces(m)
    pdeg = np.random.default_rng(5).integers(1, 5, m.nel)
    if aniso:
        A = anisotropic_tensors(m.nel, seed=5).reshape(m.nel, 9)
    else:
        A = np.array([np.diag([k] * 3).reshape(-1) for k in lognormal_k(m.nel, seed=5)])
    worst = 0.0
    for i in range(F.n):
        K, r = _host_face(dghost, m, F, i, pdeg, A, 10.0, 0.7)
        Ko, ro = O.dg_face(m, F, i, pdeg, A, pen=10.0, g=0.7)
        worst = max(worst, face_rel_err(K, Ko))
        if F.el2[i] < 0:
            assert vec_rel_err(r, ro) < 1e-13
    assert worst < 1e-13, worst


def test_double_word_operations_error_bounds(hostlib):
    """Each double-word operation against exact rational arithmetic on the
    converted operands: relative error within 2^-44 of the result (products,
    reciprocals) or of the operands' magnitude (sums, fused forms), the order
    of the published bounds for these algorithms."""
    from fractions import Fraction
    rng = np.random.default_rng(5)
    n = 400
    a, b, c, d = (rng.standard_normal(n) * 10.0 ** rng.uniform(-6, 6, n) for _ in range(4))
    out = np.zeros(n)
    conv = np.zeros(2 * n, np.float32)
    back = np.zeros(n)
    exact_in = []
    for v in (a, b, c, d):  # the operands as the kernels hold them (h + l)
        hostlib.host_dw_roundtrip(np.ascontiguousarray(v).ctypes.data, n, conv.ctypes.data, back.ctypes.data)
        exact_in.append([Fraction(float(h)) + Fraction(float(l)) for h, l in zip(conv[0::2], conv[1::2])])
    A, B, C, D = exact_in
    u = 2.0 ** -44
    ptr = [np.ascontiguousarray(v).ctypes.data for v in (a, b, c, d)]
    for op, exact, scale in (
            (0, [x * y for x, y in zip(A, B)], None),
            (1, [x + y for x, y in zip(A, B)], [abs(x) + abs(y) for x, y in zip(A, B)]),
            (2, [x * y + z for x, y, z in zip(A, B, C)], [abs(x * y) + abs(z) for x, y, z in zip(A, B, C)]),
            (3, [x * y - z * w for x, y, z, w in zip(A, B, C, D)],
             [abs(x * y) + abs(z * w) for x, y, z, w in zip(A, B, C, D)]),
            (4, [1 / x for x in A], None),
            (5, [(x + y + z) * w for x, y, z, w in zip(A, B, C, D)],
             [(abs(x) + abs(y) + abs(z)) * abs(w) for x, y, z, w in zip(A, B, C, D)])):
        hostlib.host_dw_ops(op, n, *ptr, out.ctypes.data)
        sc = scale if scale is not None else [abs(e) for e in exact]
        err = max(abs(Fraction(float(o)) - e) / s for o, e, s in zip(out, exact, sc))
        assert err < u, (op, float(err))


def test_double_word_long_sums(hostlib):
    """The long-sum accumulator of the DG kernels (exact products, TwoSum
    chain, rounding errors folded every few terms) on dot products of length
    48 with cancellation: error within 2^-46 of the summed magnitudes."""
    from fractions import Fraction
    rng = np.random.default_rng(9)
    worst = 0.0
    for _ in range(200):
        n = 48
        x = rng.standard_normal(n) * 10.0 ** rng.uniform(-3, 3)
        y = rng.standard_normal(n)
        y[-1] = -float(np.dot(x[:-1], y[:-1]) / x[-1])  # strong cancellation
        conv = np.zeros(2 * n, np.float32)
        back = np.zeros(n)
        xs, ys = [], []
        for v, acc in ((x, xs), (y, ys)):
            hostlib.host_dw_roundtrip(np.ascontiguousarray(v).ctypes.data, n, conv.ctypes.data, back.ctypes.data)
            acc.extend(Fraction(float(h)) + Fraction(float(l)) for h, l in zip(conv[0::2], conv[1::2]))
        exact = sum(p * q for p, q in zip(xs, ys))
        mag = sum(abs(p * q) for p, q in zip(xs, ys))
        for fold in (2, 4):
            got = hostlib.host_dwacc_dot(n, np.ascontiguousarray(x).ctypes.data, np.ascontiguousarray(y).ctypes.data,
                                         fold)
            worst = max(worst, float(abs(Fraction(got) - exact) / mag))
    assert worst < 2.0 ** -46, worst
