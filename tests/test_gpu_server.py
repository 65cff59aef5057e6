"""GPU tests of the request server (cp_server_*): propagate, SAC and MAC-solve
requests submitted together are batched by the server; each request's result
must equal the same request run alone (and, for propagation, the oracle)."""
import numpy as np
import pytest

import cpim_gb300 as cp
from oracle import pyoracle as O
from tests.golden_cases import oracle_view_of

pytestmark = pytest.mark.gpu


def _requests(count=36, seed=11):
    """(type, handle) pairs: types 0 propagate, 1 SAC, 2 MAC solve."""
    reqs = []
    for i in range(count):
        t = (0, 0, 1, 0, 2, 1)[i % 6]
        if t == 2:
            h = cp.InstanceHandle.uneven(seed * 7919 + i, 12, 30, 16)
        else:
            h = cp.InstanceHandle.uneven(seed * 7919 + i, 20, 90, 128)
        reqs.append((t, h))
    # Tight members: AC/SAC wipe-outs and a MAC refutation.
    reqs.append((0, cp.InstanceHandle.binary(30, 8, 120, 0.45, 0.45, 0.1, 2)))
    reqs.append((1, cp.InstanceHandle.binary(30, 8, 120, 0.35, 0.35, 0.1, 4)))
    reqs.append((2, cp.InstanceHandle.binary(20, 8, 90, 0.45, 0.45, 0.0, 5)))
    return reqs


def _alone(eng, rtype, h):
    inst = h.export()
    net = eng.upload(inst, max_levels=2 if rtype < 2 else 0)
    try:
        if rtype == 0:
            st = net.enforce_ac(0)
            return {"inc": bool(st.inconsistent), "dom": net.dom_get(0), "inst": inst}
        if rtype == 1:
            st = net.enforce_sac1(0)
            return {"inc": bool(st.inconsistent), "dom": net.dom_get(0), "inst": inst}
        return net.mac_solve(cp.VarHeuristic.VRH_DOM_MIN, cp.ValHeuristic.VLH_MIN)
    finally:
        net.close()


def _check(srv, eng, reqs, tickets):
    for k, ((t, h), tk) in enumerate(zip(reqs, tickets)):
        r = srv.wait(tk, 120000)
        assert r.status == 2, (k, r.status)
        assert r.type == t
        ref = _alone(eng, t, h)
        if t < 2:
            assert bool(r.inconsistent) == ref["inc"], k
            if not ref["inc"]:
                assert np.array_equal(srv.domains(tk, h.n, h.W), ref["dom"]), k
            if t == 0:
                ok, d, _ = O.ac3bit(oracle_view_of(ref["inst"]))
                assert ok == (not ref["inc"]), k
        else:
            assert r.mac_status == ref["status"], k
            assert (r.num_positive, r.num_negative) == (ref["num_positive"], ref["num_negative"]), k
            if ref["status"] == 1:
                assert srv.solution(tk, h.n) == ref["solution"], k
        assert r.latency_ms >= r.queue_ms >= 0.0
        srv.release(tk)


@pytest.mark.parametrize("batching", [True, False])
def test_server_mixed_requests_match_single_runs(batching):
    reqs = _requests()
    with cp.Engine(0) as eng, cp.Server(budget_bytes=8 * 10**9, max_batch=16, batching=batching,
                                        solvers=2) as srv:
        tickets = [srv.submit(t, h) for t, h in reqs]
        _check(srv, eng, reqs, tickets)


def test_server_tiny_budget_admits_one_at_a_time():
    # A budget below every footprint admits one request whenever nothing runs.
    reqs = _requests(12, 3)
    with cp.Engine(0) as eng, cp.Server(budget_bytes=1, max_batch=64) as srv:
        tickets = [srv.submit(t, h) for t, h in reqs]
        _check(srv, eng, reqs, tickets)


def test_server_trace_replay():
    reqs = _requests(24, 5)
    arrivals = np.cumsum(np.full(len(reqs), 0.0005))
    with cp.Server(budget_bytes=8 * 10**9, max_batch=32) as srv:
        lat, st, stats = srv.run_trace(arrivals, [(t, h, ()) for t, h in reqs])
        assert (st == 2).all(), st
        assert (lat > 0).all()
        assert stats[0] >= 1          # ticks
        assert stats[1] >= 1          # batched requests
        assert 0 < stats[3] <= 8 * 10**9  # peak admitted bytes within the budget


def test_server_rejects_bad_calls():
    with cp.Server(budget_bytes=10**9) as srv:
        with pytest.raises(cp.CPError):
            srv.wait(12345, 10)
        with pytest.raises(cp.CPError):
            srv.release(12345)
        h = cp.InstanceHandle.uneven(1, 20, 30, 16)
        with pytest.raises(cp.CPError):
            srv.submit(7, h)


def _choices(h, rng, count):
    n = h.n
    inst = h.export()
    out = []
    for _ in range(count):
        x = int(rng.integers(0, n))
        out.append((x, int(rng.integers(0, int(inst.dom[x])))))
    return out


def _alone_with_choices(eng, rtype, h, choices):
    inst = h.export()
    net = eng.upload(inst, max_levels=2 if rtype < 2 else 0)
    try:
        for x, a in choices:
            net.reduce_to(0, x, a)
        if rtype == 0:
            st = net.enforce_ac(0)
            return {"inc": bool(st.inconsistent), "dom": net.dom_get(0)}
        if rtype == 1:
            st = net.enforce_sac1(0)
            return {"inc": bool(st.inconsistent), "dom": net.dom_get(0)}
        return net.mac_solve(cp.VarHeuristic.VRH_DOM_MIN, cp.ValHeuristic.VLH_MIN)
    finally:
        net.close()


@pytest.mark.parametrize("batching", [True, False])
def test_resident_networks_with_choices_match_single_runs(batching):
    """Requests on registered networks (several per network at once, each on
    its own working level, with random variable choices) equal the same
    choices and propagation run alone."""
    rng = np.random.default_rng(23)
    nets = [cp.InstanceHandle.uneven(900 + i, 20, 70, 64) for i in range(3)]
    small = cp.InstanceHandle.uneven(77, 12, 24, 16)  # MAC requests
    with cp.Engine(0) as eng, cp.Server(budget_bytes=8 * 10**9, max_batch=16, batching=batching,
                                        solvers=2) as srv:
        ids = [srv.register(h, slots=3) for h in nets]
        sid = srv.register(small, slots=1)
        reqs = []
        for k in range(30):
            t = (0, 1, 0, 2, 0)[k % 5]
            if t == 2:
                reqs.append((t, sid, small, _choices(small, rng, k % 2)))
            else:
                j = k % 3
                reqs.append((t, ids[j], nets[j], _choices(nets[j], rng, k % 3)))
        # Two different values for one variable: inconsistent as posed.
        x0 = 0
        reqs.append((0, ids[0], nets[0], [(x0, 0), (x0, 1)]))
        tickets = [srv.submit(t, nid, ch) for t, nid, _, ch in reqs]
        for k, ((t, nid, h, ch), tk) in enumerate(zip(reqs, tickets)):
            r = srv.wait(tk, 120000)
            assert r.status == 2, (k, r.status)
            if len({x for x, _ in ch}) < len(ch) and len(set(ch)) == len(ch):
                assert r.inconsistent == 1, k
                srv.release(tk)
                continue
            ref = _alone_with_choices(eng, t, h, ch)
            if t < 2:
                assert bool(r.inconsistent) == ref["inc"], k
                if not ref["inc"]:
                    assert np.array_equal(srv.domains(tk, h.n, h.W), ref["dom"]), k
            else:
                assert r.mac_status == ref["status"], k
                assert (r.num_positive, r.num_negative) == (ref["num_positive"], ref["num_negative"]), k
                if ref["status"] == 1:
                    assert srv.solution(tk, h.n) == ref["solution"], k
            srv.release(tk)
        for i in ids + [sid]:
            srv.unregister(i)
        with pytest.raises(cp.CPError):
            srv.submit(0, ids[0])


def test_server_cancel_and_unregister_rules():
    h = cp.InstanceHandle.uneven(4242, 150, 200, 128)
    with cp.Server(budget_bytes=8 * 10**9, max_batch=1) as srv:
        nid = srv.register(h, slots=1)
        tickets = [srv.submit(1, nid) for _ in range(12)]
        with pytest.raises(cp.CPError):
            srv.unregister(nid)  # requests queued or running on it
        cancelled = 0
        for tk in tickets[6:]:
            try:
                srv.cancel(tk)
                cancelled += 1
            except cp.CPError:
                pass  # already admitted
        assert cancelled >= 1
        statuses = [srv.wait(tk, 120000).status for tk in tickets]
        assert statuses.count(-7) == cancelled
        assert all(s in (2, -7) for s in statuses)
        for tk in tickets:
            srv.release(tk)
        srv.unregister(nid)


def test_server_register_over_budget():
    h = cp.InstanceHandle.uneven(4242, 150, 200, 128)
    with cp.Server(budget_bytes=1 << 20) as srv:
        with pytest.raises(cp.CPError):
            srv.register(h, slots=4)


def test_server_poll_matches_wait():
    # cp_poll answers 1 (pending) until a request is done, then fills the same
    # result as cp_wait; an unknown ticket is an argument error.
    import time
    reqs = _requests(count=12, seed=5)
    with cp.Server(budget_bytes=8 * 10**9) as srv, cp.Engine(0) as eng:
        tickets = [srv.submit(t, h) for t, h in reqs]
        polled = {}
        deadline = time.time() + 120
        while len(polled) < len(tickets) and time.time() < deadline:
            for tk in tickets:
                if tk not in polled:
                    r = srv.poll(tk)
                    if r is not None:
                        polled[tk] = (r.status, r.inconsistent, r.num_positive, r.num_negative, r.mac_status)
            time.sleep(0.001)
        assert len(polled) == len(tickets)
        for tk in tickets:
            r = srv.wait(tk, 1000)
            assert polled[tk] == (r.status, r.inconsistent, r.num_positive, r.num_negative, r.mac_status)
        _check(srv, eng, reqs, tickets)
        with pytest.raises(cp.CPError):
            srv.poll(10**9)
