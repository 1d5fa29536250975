"""GPU tests of the serving engine: results bit-identical alone and in a
mix, equal to the plain one-problem path within the solver tolerance, and
admission bounded by the HBM budget."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gb():
    from modfem_gb300 import build
    build.build(verbose=False)
    import modfem_gb300
    return modfem_gb300


def _problems():
    from modfem_gb300.mesh import lognormal_k, prism_faces, structured_prism_mesh
    from modfem_gb300.serve import DG, STD, Problem
    out = []
    for n, kind, p in ((5, STD, 1), (8, STD, 1), (11, STD, 1), (4, DG, 1), (3, DG, 2), (6, STD, 1), (5, DG, 1)):
        m = structured_prism_mesh(n, jitter=0.2, seed=n)
        k = lognormal_k(m.nel, seed=n + 100)
        F = prism_faces(m) if kind == DG else None
        out.append((m, k, F, Problem(m, k, kind=kind, p=p, faces=F, f=1.0, g=0.0, krylov=30, max_iter=20000,
                                     tol=1e-8)))
    return out


def _serve(srv, probs, together):
    from modfem_gb300.serve import dof_count
    res = []
    if together:
        ids = [srv.submit(pr) for (_, _, _, pr) in probs]
        for rid, (_, _, _, pr) in zip(ids, probs):
            assert srv.wait(rid, 120.0) == 1
            res.append(srv.result(rid, dof_count(pr)))
            srv.release(rid)
    else:
        for (_, _, _, pr) in probs:
            rid = srv.submit(pr)
            assert srv.wait(rid, 120.0) == 1
            res.append(srv.result(rid, dof_count(pr)))
            srv.release(rid)
    return res


def test_served_results_same_alone_and_in_mix(gb):
    from modfem_gb300.serve import Server
    probs = _problems()
    srv = Server(0, max_active=16, prep_threads=4)
    try:
        mix = _serve(srv, probs, True)
        alone = _serve(srv, probs, False)
        st = srv.stats()
    finally:
        srv.close()
    assert st["peak_active"] > 1
    for (xm, im, rm, _), (xa, ia, ra, _) in zip(mix, alone):
        assert im == ia and np.array_equal(xm, xa)
        assert rm < 1e-8


def test_served_matches_plain_solver(gb):
    """Same assembly and GMRES as the one-problem path: iteration counts
    within 2 and solutions equal to the solver tolerance."""
    from modfem_gb300.serve import DG, Server
    probs = _problems()
    srv = Server(0, max_active=16)
    try:
        served = _serve(srv, probs, True)
    finally:
        srv.close()
    for (m, k, F, pr), (x, it, rel, _) in zip(probs, served):
        c = gb.Context(0)
        c.set_mesh(m)
        c.set_coefficients(k=k, f=1.0, g=0.0)
        if pr.kind == DG:
            c.dg_set_degrees(np.full(m.nel, pr.p))
            c.dg_set_faces(F, penalty=10.0)
            c.dg_build_structure()
            c.dg_assemble()
            xp, itp, _, _ = c.dg_solve(krylov=30, max_iter=20000, tol_rel=1e-8)
        else:
            c.build_structure()
            c.assemble()
            xp, itp, _, _ = c.solve(krylov=30, max_iter=20000, tol_rel=1e-8)
        c.close()
        assert abs(it - itp) <= 2, (pr.kind, m.nel, it, itp)
        assert np.max(np.abs(x - xp)) <= 1e-6 * np.max(np.abs(xp))


def test_admission_respects_budget(gb):
    """A budget that holds one large request at a time: every request still
    finishes, and the bytes charged never exceed the budget."""
    from modfem_gb300.serve import Server
    probs = _problems()
    big = max(pr.footprint() for (_, _, _, pr) in probs)
    srv = Server(0, hbm_budget=int(1.5 * big), max_active=16)
    try:
        res = _serve(srv, probs, True)
        st = srv.stats()
    finally:
        srv.close()
    assert len(res) == len(probs)
    assert st["peak_bytes"] <= st["budget"]
