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
HDR = os.path.join(HERE, "..", "modfem_gb300", "csrc", "prism_std.cuh")
LIB = os.path.join(HERE, "hostcheck", "libprism_math_host.so")


@pytest.fixture(scope="module")
def hostlib():
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(SRC), os.path.getmtime(HDR)):
        subprocess.check_call([nvcc, "-O2", "-std=c++17", "-Xcompiler", "-fPIC", "-shared", "-o", LIB, SRC])
    L = ctypes.CDLL(LIB)
    L.host_prism_std_element.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_double, ctypes.c_void_p,
                                         ctypes.c_void_p]
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
