"""Serving loop: many mixed-precision CG solves on different operators,
admitted by HBM budget and advanced together. Each result is the same alone
and in the mix (bit for bit: requests share no state and every kernel is
deterministic) and meets its FP64-checked tolerance."""
import time

import numpy as np
import pytest

import oracle
from amat_gb300 import Maps, aMatFree
from amat_gb300 import problems as P
from amat_gb300.serve import Server

pytestmark = pytest.mark.gpu

RTOL = 1e-8
CASES = [(P.HEX8_POISSON, 10, 1), (P.HEX8_ELASTIC, 6, 2), (P.HEX20_ELASTIC, 4, 3), (P.TET10_POISSON, 6, 4),
         (P.HEX8_POISSON, 16, 5), (P.HEX8_ELASTIC, 8, 6)]


def request(kind, n, seed):
    """Operator with maps, BCs and element matrices set (not finalised) and a random load. (The
    elastic bar's six constraints sit on centre nodes: even edges only.)"""
    m = P.Mesh(kind, n, jitter=0.1, seed=seed)
    ke = m.element_matrices(ngt=3 if kind == P.HEX20_ELASTIC else 2)
    dofs, vals = m.boundary_conditions()
    maps = Maps()
    maps.set_map(m.n_elem, m.dof_map(), m.ndpe, m.n_dofs)
    maps.set_bdr_map(dofs, vals)
    A = aMatFree(maps)
    A.set_element_matrices(0, ke)
    b = np.random.default_rng(seed).normal(size=m.n_dofs)
    b[dofs.astype(np.int64)] = vals
    return A, b, oracle.Problem(m.n_dofs, m.dof_map(), ke, dofs, vals)


def drain(srv, ids, timeout=120.0):
    out, t0 = {}, time.time()
    while len(out) < len(ids):
        srv.poll()
        for i in ids:
            if i not in out:
                r = srv.take(i)
                if r is not None:
                    out[i] = r
        assert time.time() - t0 < timeout, "serving loop made no progress"
    return out


def test_results_alone_and_in_the_mix(gpu):
    srv = Server(0)
    alone = []
    for case in CASES:
        A, b, pr = request(*case)
        rid = srv.submit(A, b, rtol=RTOL)
        x, st, t = drain(srv, [rid])[rid]
        assert st.status == 0 and st.rel_residual <= RTOL
        assert np.linalg.norm(b - pr.matmult_bc(x)) <= 1.01 * RTOL * np.linalg.norm(b)
        assert t[0] <= t[1] <= t[2] <= t[3]
        alone.append(x)
    # all at once: admitted together, advanced together
    ids = []
    for case in CASES:
        A, b, _ = request(*case)
        ids.append(srv.submit(A, b, rtol=RTOL))
    q, a = srv.poll()
    assert q + a == len(CASES)
    res = drain(srv, ids)
    for x0, rid in zip(alone, ids):
        assert np.array_equal(res[rid][0], x0)
    assert srv.info()["lane_max_batch"] >= 2  # the mix shared serving-lane launches
    srv.close()


def test_arrivals_while_others_run(gpu):
    """Continuous batching: requests submitted while an earlier one is mid-solve are admitted and started
    before it finishes, run beside it, and every result, the long one's included, equals the one computed
    alone, bit for bit."""
    long_case = (P.HEX20_ELASTIC, 12, 7)
    cases = CASES[:4]
    srv = Server(0)
    alone = {}
    for case in [long_case] + cases:
        A, b, _ = request(*case)
        rid = srv.submit(A, b, rtol=RTOL)
        alone[case] = drain(srv, [rid])[rid][0]
    pending = [(case, request(*case)) for case in cases]  # built before, submitted while the long one runs
    A, b, _ = request(*long_case)
    first = srv.submit(A, b, rtol=RTOL)
    t0 = time.time()
    while True:  # until the long request runs (admitted and its solve started)
        q, a = srv.poll()
        if q == 0 and a == 1 and time.time() - t0 > 0.02:
            break
        assert time.time() - t0 < 60
    assert srv.take(first) is None, "the long request finished before the others arrived"
    ids = {}
    for case, (A, b, _) in pending:
        ids[srv.submit(A, b, rtol=RTOL)] = case
        srv.poll()
    res = drain(srv, [first] + list(ids))
    t_done_first = res[first][2][3]
    assert np.array_equal(res[first][0], alone[long_case])
    for rid, case in ids.items():
        x, st, t = res[rid]
        assert np.array_equal(x, alone[case])
        assert t[2] < t_done_first  # started while the long one was still running
    info = srv.info()  # the long request on its own stream, the small ones in the lane
    assert info["stream_requests"] >= 2 and info["lane_requests"] >= 2 * len(cases)
    srv.close()


def test_admission_waits_for_memory(gpu):
    """A budget below any two requests admits one at a time; arrivals wait in
    the queue and every one finishes with the same result as alone."""
    srv = Server(0, hbm_budget=1)
    reqs = [request(*c) for c in CASES[:3]]
    ids = [srv.submit(A, b, rtol=RTOL) for A, b, _ in reqs]
    seen_max = 0
    out, t0 = {}, time.time()
    while len(out) < len(ids):
        q, a = srv.poll()
        seen_max = max(seen_max, a)
        for i in ids:
            if i not in out:
                r = srv.take(i)
                if r is not None:
                    out[i] = r
        assert time.time() - t0 < 120
    assert seen_max == 1
    for (A, b, pr), i in zip(reqs, ids):
        x = out[i][0]
        assert np.linalg.norm(b - pr.matmult_bc(x)) <= 1.01 * RTOL * np.linalg.norm(b)
    srv.close()


def test_failed_request_is_reported(gpu):
    """A request whose mixed-precision solve cannot run (FP64 arena) fails
    alone; the server keeps serving the others."""
    from amat_gb300 import AfmError, PRECISION
    srv = Server(0)
    A, b, _ = request(*CASES[0])
    A.set_precision(PRECISION.FP64)
    bad = srv.submit(A, b)
    A2, b2, pr2 = request(*CASES[1])
    good = srv.submit(A2, b2)
    t0 = time.time()
    done = {}
    while len(done) < 2:
        srv.poll()
        for i in (bad, good):
            if i in done:
                continue
            try:
                r = srv.take(i)
                if r is not None:
                    done[i] = r
            except AfmError as e:
                done[i] = e
        assert time.time() - t0 < 60
    assert isinstance(done[bad], AfmError) and done[bad].name == "ERR_STATE"
    x = done[good][0]
    assert np.linalg.norm(b2 - pr2.matmult_bc(x)) <= 1.01 * RTOL * np.linalg.norm(b2)
    srv.close()


def _solve_all(srv, cases):
    reqs = [request(*c) for c in cases]
    ids = [srv.submit(A, b, rtol=RTOL) for A, b, _ in reqs]
    res = drain(srv, ids)
    return [(res[i], pr, b) for i, (_, b, pr) in zip(ids, reqs)]


def test_lane_batches_the_small_requests(gpu):
    """The serving lane: every request of CASES is small enough for it, so their FP32 iterations run in
    shared launches (one cluster per request); launches carry several requests at once, every result meets
    its FP64-checked tolerance, and the number of iterations per launch does not change a single bit."""
    out = {}
    for iters in (8, 32):
        srv = Server(0)
        srv.set_lane(8 << 20, iters)
        out[iters] = _solve_all(srv, CASES)
        info = srv.info()
        srv.close()
        assert info["lane_requests"] == len(CASES) and info["stream_requests"] == 0
        assert info["lane_max_batch"] >= 2
        assert info["lane_solve_launches"] > info["lane_launches"]
        for (x, st, _), pr, b in out[iters]:
            assert st.status == 0 and st.rel_residual <= RTOL
            assert np.linalg.norm(b - pr.matmult_bc(x)) <= 1.01 * RTOL * np.linalg.norm(b)
    for a, b in zip(out[8], out[32]):
        assert np.array_equal(a[0][0], b[0][0])


def test_lane_off_runs_every_request_on_its_stream(gpu):
    srv = Server(0)
    srv.set_lane(0, 32)
    res = _solve_all(srv, CASES[:3])
    info = srv.info()
    srv.close()
    assert info["lane_requests"] == 0 and info["stream_requests"] == 3 and info["lane_launches"] == 0
    for (x, st, _), pr, b in res:
        assert st.status == 0
        assert np.linalg.norm(b - pr.matmult_bc(x)) <= 1.01 * RTOL * np.linalg.norm(b)


def test_lane_arguments(gpu):
    from amat_gb300 import AfmError
    srv = Server(0)
    for bad in (0, 5000):
        with pytest.raises(AfmError) as e:
            srv.set_lane(1 << 20, bad)
        assert e.value.name == "ERR_INVALID_ARG"
    srv.close()
