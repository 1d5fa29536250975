"""Python front end of the serving engine (gbfem_server_*): request
construction from the library's mesh objects, submission, results, and a
Poisson-arrival load driver reporting latency percentiles."""
import ctypes
import threading
import time

import numpy as np

from . import GbFemError, load_library

STD, DG = 0, 1


class Request(ctypes.Structure):
    """Mirror of gbfem_serve_request (include/modfem_gb300.h)."""
    _fields_ = [
        ("kind", ctypes.c_int), ("dg_p", ctypes.c_int),
        ("nno", ctypes.c_int), ("node_xyz", ctypes.c_void_p),
        ("nel", ctypes.c_int), ("el_nodes", ctypes.c_void_p),
        ("k_el", ctypes.c_void_p), ("f", ctypes.c_double), ("g", ctypes.c_double),
        ("nbf", ctypes.c_int), ("bf_el", ctypes.c_void_p), ("bf_side", ctypes.c_void_p),
        ("nfa", ctypes.c_int), ("fa_type", ctypes.c_void_p), ("fa_bc", ctypes.c_void_p),
        ("fa_el", ctypes.c_void_p), ("fa_side", ctypes.c_void_p), ("fa_nodes", ctypes.c_void_p),
        ("dg_penalty", ctypes.c_double),
        ("krylov", ctypes.c_int), ("max_iter", ctypes.c_int), ("tol_rel", ctypes.c_double),
    ]


class Problem:
    """A heat problem ready for submission: keeps the arrays the request
    points to alive.  kind STD (linear prisms, penalty Dirichlet on the
    boundary faces) or DG (degree p, interior penalty, full face table)."""

    def __init__(self, mesh, k, kind=STD, p=1, faces=None, f=1.0, g=0.0, krylov=30, max_iter=20000, tol=1e-8,
                 penalty=10.0):
        self.kind, self.p, self.nel = kind, p, mesh.nel
        self.xyz = np.ascontiguousarray(mesh.coords, dtype=np.float64)
        self.el = np.ascontiguousarray(mesh.el_nodes, dtype=np.int32)
        self.k = np.ascontiguousarray(k, dtype=np.float64)
        r = Request()
        r.kind, r.dg_p = kind, p
        r.nno, r.node_xyz = self.xyz.shape[0], self.xyz.ctypes.data
        r.nel, r.el_nodes = self.el.shape[0], self.el.ctypes.data
        r.k_el, r.f, r.g = self.k.ctypes.data, f, g
        r.krylov, r.max_iter, r.tol_rel = krylov, max_iter, tol
        r.dg_penalty = penalty
        if kind == STD:
            self.bf_el = np.ascontiguousarray(mesh.bc_face_el, dtype=np.int32)
            self.bf_side = np.ascontiguousarray(mesh.bc_face_side, dtype=np.int32)
            r.nbf, r.bf_el, r.bf_side = self.bf_el.size, self.bf_el.ctypes.data, self.bf_side.ctypes.data
        else:
            if faces is None:
                from .mesh import prism_faces
                faces = prism_faces(mesh)
            self.fa = [np.ascontiguousarray(a, dtype=np.int32) for a in (
                faces.type, faces.bc, np.stack([faces.el1, faces.el2], axis=1), faces.side1, faces.nodes)]
            r.nfa = self.fa[0].size
            r.fa_type, r.fa_bc, r.fa_el, r.fa_side, r.fa_nodes = [a.ctypes.data for a in self.fa]
        self.req = r

    def footprint(self):
        return load_library().gbfem_serve_footprint(ctypes.byref(self.req))


class Server:
    def __init__(self, device=0, hbm_budget=0, max_active=32, prep_threads=4, steps_per_poll=None):
        self.L = load_library()
        h = ctypes.c_void_p()
        self._check(self.L.gbfem_server_create(ctypes.byref(h), device, int(hbm_budget), max_active, prep_threads))
        self._h = h
        self._lock = threading.Lock()
        if steps_per_poll is not None:
            self._check(self.L.gbfem_server_set_option(self._h, 1, int(steps_per_poll)))

    def _check(self, r):
        if r < 0:
            raise GbFemError(self.L.gbfem_last_error().decode())
        return r

    def submit(self, problem):
        with self._lock:
            return self._check(self.L.gbfem_server_submit(self._h, ctypes.byref(problem.req)))

    def wait(self, rid, timeout=-1.0):
        return self._check(self.L.gbfem_server_wait(self._h, rid, float(timeout)))

    def result(self, rid, n_max):
        x = np.zeros(n_max)
        it = ctypes.c_int()
        rel = ctypes.c_double()
        t = np.zeros(5)
        n = self._check(self.L.gbfem_server_result(self._h, rid, x.ctypes.data, n_max, ctypes.byref(it),
                                                   ctypes.byref(rel), t.ctypes.data))
        return x[:n], it.value, rel.value, t

    def release(self, rid):
        self._check(self.L.gbfem_server_release(self._h, rid))

    def cancel(self, rid):
        """gbfem_server_cancel: 0 cancelled, 1 already finished or failed."""
        return self._check(self.L.gbfem_server_cancel(self._h, rid))

    def inject_preparation_failures(self, count):
        """The next `count` preparations fail as a device allocation would
        (GBFEM_SERVE_OPT_FAIL_PREPARATIONS; host-side fault injection)."""
        self._check(self.L.gbfem_server_set_option(self._h, 2, int(count)))

    def set_std_precedence(self, on):
        """GBFEM_SERVE_OPT_STD_PRECEDENCE: no new DG steps while a solo-sized
        std request is prepared or solved (default on)."""
        self._check(self.L.gbfem_server_set_option(self._h, 4, int(bool(on))))

    def set_solo_dofs(self, n):
        """GBFEM_SERVE_OPT_SOLO_DOFS: the size from which std requests are
        solved alone on their own stream (0: never)."""
        self._check(self.L.gbfem_server_set_option(self._h, 3, int(n)))

    def stats(self):
        st = np.zeros(8, np.int64)
        self._check(self.L.gbfem_server_stats(self._h, st.ctypes.data))
        keys = ("steps", "launches", "peak_active", "peak_bytes", "budget", "bytes", "queued", "active")
        return dict(zip(keys, (int(v) for v in st)))

    def close(self):
        if self._h:
            self.L.gbfem_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def dof_count(problem):
    """Upper bound of the solution length of a problem (std: nodes; DG:
    functions per element times elements)."""
    if problem.kind == STD:
        return problem.xyz.shape[0]
    return [0, 6, 18, 40, 75][problem.p] * problem.nel


def poisson_stream(server, problems, rate, count, seed=0):
    """Submits `count` problems drawn round-robin from `problems` at Poisson
    arrival times of the given rate (requests/s) and waits for all of them.
    Returns per-request (latency s, times[5], iterations) and the makespan."""
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate, count)
    t0 = time.perf_counter()
    arrivals = t0 + np.cumsum(gaps)
    ids = []
    for i in range(count):
        dt = arrivals[i] - time.perf_counter()
        if dt > 0:
            time.sleep(dt)
        pr = problems[i % len(problems)]
        ids.append((server.submit(pr), pr))
    out = []
    for rid, pr in ids:
        server.wait(rid)
        x, it, rel, t = server.result(rid, dof_count(pr))
        out.append({"latency": t[4], "times": t, "iters": it, "rel": rel, "nel": pr.nel, "kind": pr.kind})
        server.release(rid)
    return out, time.perf_counter() - t0
