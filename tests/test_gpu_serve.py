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


# ----------------------------------------------------------- failure handling
# Failures are made on the host (an injected allocation failure, a malformed
# request, a cancellation); no GPU fault is provoked.

def test_injected_preparation_failure_is_contained(gb):
    """The next preparation fails as if its device allocation had failed: that
    request reports the failure, the others are served as usual, and the
    admission accounting returns to zero."""
    from modfem_gb300.serve import Server, dof_count
    probs = [pr for (_, _, _, pr) in _problems()[:4]]
    srv = Server(0, max_active=1, prep_threads=1)  # one at a time: the failure hits the first request
    try:
        srv.inject_preparation_failures(1)
        ids = [srv.submit(pr) for pr in probs]
        with pytest.raises(gb.GbFemError, match="injected allocation failure"):
            srv.wait(ids[0], 120.0)
        for rid, pr in zip(ids[1:], probs[1:]):
            assert srv.wait(rid, 120.0) == 1
            x, it, rel, _ = srv.result(rid, dof_count(pr))
            assert rel < 1e-8 and np.all(np.isfinite(x))
        for rid in ids:
            srv.release(rid)
        st = srv.stats()
        assert st["bytes"] == 0 and st["active"] == 0 and st["queued"] == 0
    finally:
        srv.close()


def test_malformed_request_fails_alone(gb):
    """A request whose element names a node that does not exist is refused
    by its preparation (gbfem_set_mesh's range check) with a message; a
    request without elements is refused at submission; the server keeps
    serving."""
    from modfem_gb300.mesh import lognormal_k, structured_prism_mesh
    from modfem_gb300.serve import STD, Problem, Server, dof_count
    m = structured_prism_mesh(4, jitter=0.1, seed=3)
    k = lognormal_k(m.nel, seed=3)
    bad = Problem(m, k, kind=STD)
    bad.el[5, 2] = m.nno + 7  # out of range, in the array the request points to
    good = _problems()[0][3]
    srv = Server(0, max_active=4, prep_threads=2)
    try:
        rb = srv.submit(bad)
        rg = srv.submit(good)
        with pytest.raises(gb.GbFemError, match="out of range"):
            srv.wait(rb, 120.0)
        assert srv.wait(rg, 120.0) == 1
        assert srv.result(rg, dof_count(good))[2] < 1e-8
        empty = Problem(m, k, kind=STD)
        empty.req.nel = 0
        with pytest.raises(gb.GbFemError, match="empty request"):
            srv.submit(empty)
        srv.release(rb)
        srv.release(rg)
        assert srv.stats()["bytes"] == 0
    finally:
        srv.close()


def test_cancel_queued_and_running_requests(gb):
    """Cancelling a queued request removes it before it is prepared; a
    request already admitted is retired at the end of its preparation or at
    the engine's next poll.  Cancelled requests report "cancelled", their
    memory returns to the budget, and the requests not cancelled give the
    same solutions as when served alone."""
    from modfem_gb300.mesh import lognormal_k, structured_prism_mesh
    from modfem_gb300.serve import STD, Problem, Server, dof_count
    big = []
    for n in (30, 31, 32):  # long enough solves that a cancellation finds them running
        m = structured_prism_mesh(n, jitter=0.2, seed=n)
        big.append(Problem(m, lognormal_k(m.nel, seed=n), kind=STD, krylov=30, max_iter=20000, tol=1e-10))
    small = _problems()[0][3]
    srv = Server(0, max_active=2, prep_threads=1)
    try:
        ref_id = srv.submit(small)
        assert srv.wait(ref_id, 120.0) == 1
        x_ref = srv.result(ref_id, dof_count(small))[0]
        srv.release(ref_id)
        ids = [srv.submit(pr) for pr in big] + [srv.submit(small)]
        # the third big request is still queued (two slots): cancelled at once
        assert srv.cancel(ids[2]) == 0
        with pytest.raises(gb.GbFemError, match="cancelled"):
            srv.wait(ids[2], 120.0)
        # the first one is being prepared or solved
        assert srv.cancel(ids[0]) == 0
        with pytest.raises(gb.GbFemError, match="cancelled"):
            srv.wait(ids[0], 120.0)
        assert srv.wait(ids[1], 300.0) == 1
        assert srv.wait(ids[3], 300.0) == 1
        assert np.array_equal(srv.result(ids[3], dof_count(small))[0], x_ref)
        assert srv.cancel(ids[3]) == 1  # finished: nothing to cancel
        for rid in ids:
            srv.release(rid)
        st = srv.stats()
        assert st["bytes"] == 0 and st["active"] == 0
    finally:
        srv.close()


def test_large_std_request_solved_alone_on_its_stream(gb):
    """A std request with at least GBFEM_SERVE_OPT_SOLO_DOFS dofs (default
    40,000) is solved by its preparation worker with the device-resident
    GMRES on its own stream: the same bits alone and beside a mix of small
    requests, and the plain one-problem path's solution within the solver
    tolerance."""
    from modfem_gb300.mesh import lognormal_k, structured_prism_mesh
    from modfem_gb300.serve import STD, Problem, Server, dof_count
    m = structured_prism_mesh(36, jitter=0.2, seed=36)
    k = lognormal_k(m.nel, seed=36)
    big = Problem(m, k, kind=STD, krylov=30, max_iter=20000, tol=1e-8)
    assert dof_count(big) >= 40000
    small = [pr for (_, _, _, pr) in _problems()]
    srv = Server(0, max_active=16, prep_threads=4)
    try:
        rid = srv.submit(big)
        assert srv.wait(rid, 300.0) == 1
        xa, ia, ra, _ = srv.result(rid, dof_count(big))
        srv.release(rid)
        ids = [srv.submit(pr) for pr in small[:3]] + [srv.submit(big)] + [srv.submit(pr) for pr in small[3:]]
        for i in ids:
            assert srv.wait(i, 300.0) == 1
        xm, im, rm, _ = srv.result(ids[3], dof_count(big))
        for i in ids:
            srv.release(i)
    finally:
        srv.close()
    assert ia == im and np.array_equal(xa, xm)
    assert ra < 1e-8
    c = gb.Context(0)
    c.set_mesh(m)
    c.set_coefficients(k=k, f=1.0, g=0.0)
    c.build_structure_device()
    c.assemble(gb.SCATTER_COLOR)
    x, it, _, rel = c.solve(30, 20000, 1e-8)
    c.close()
    assert abs(it - ia) <= 1
    assert np.max(np.abs(x - xa)) <= 1e-6 * np.max(np.abs(x))


def test_std_precedence_and_solo_threshold_keep_results(gb):
    """Scheduling policies change when work runs, not what it computes: a
    mix with a solo-sized std request (threshold lowered so that the 11^3
    mesh qualifies) gives every request the same bits with the DG lane held
    back during the solo windows (default) and without."""
    from modfem_gb300.serve import Server
    probs = _problems()
    out = []
    for prec in (1, 0):
        srv = Server(0, max_active=16, prep_threads=4)
        try:
            srv.set_solo_dofs(1500)  # the 11^3 x 2 request (1,728 dofs) is solved alone
            srv.set_std_precedence(prec)
            out.append(_serve(srv, probs, True))
        finally:
            srv.close()
    for (xa, ia, ra, _), (xb, ib, rb, _) in zip(*out):
        assert ia == ib and np.array_equal(xa, xb)
        assert ra < 1e-8
