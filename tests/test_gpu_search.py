"""GPU tests of the device-resident MAC search (k_mac): a whole search per
CTA must give the host-driven search's node counts and solutions, alone and
batched, with and without variable choices."""
import numpy as np
import pytest

import cpim_gb300 as cp
from tests.golden_cases import make_engine_instance

pytestmark = pytest.mark.gpu


def _host_driven(inst, choices, var_h=cp.VarHeuristic.VRH_DOM_MIN):
    with cp.Engine(0) as e:
        e.set_search_mode(1)
        net = e.upload(inst)
        for x, a in choices:
            net.reduce_to(0, x, a)
        r = net.mac_solve(var_h, cp.ValHeuristic.VLH_MIN, time_limit_ms=120000)
        net.close()
    return r


def _same(a, b, tag):
    assert a["status"] == b["status"], tag
    assert (a["num_positive"], a["num_negative"]) == (b["num_positive"], b["num_negative"]), tag
    if a["status"] == 1:
        assert a["solution"] == b["solution"], tag


def _choices(inst, rng, k):
    out = []
    for _ in range(k):
        x = int(rng.integers(0, inst.n))
        out.append((x, int(rng.integers(0, int(inst.dom[x])))))
    # keep the first choice per variable (the server answers conflicting ones
    # without a search)
    seen, keep = set(), []
    for x, a in out:
        if x not in seen:
            seen.add(x)
            keep.append((x, a))
    return keep


def test_mac_batch_matches_host_driven(golden):
    rng = np.random.default_rng(3)
    insts = [make_engine_instance(c["args"]) for c in golden if c["op"] == "mac"][:10]
    insts += [cp.gen_uneven(700 + i, 12, 40, 64) for i in range(8)]
    insts += [cp.gen_mixed(30, 8, 60, 0.3, 0.5, 40, 60, 0.2, s) for s in (1, 2)]
    with cp.Engine(0) as up, cp.Engine(0) as eng:
        nets = [up.upload(i) for i in insts]
        jobs, refs = [], []
        for inst, net in zip(insts, nets):
            for rep in range(2):
                ch = _choices(inst, rng, rep * 2)
                jobs.append((net, ch))
                refs.append(_host_driven(inst, ch))
        mb = cp.MacBatch(eng, jobs, time_limit_ms=120000)
        got = mb.wait()
        for k, (g, r) in enumerate(zip(got, refs)):
            _same(g, r, k)
        mb.close()
        for n in nets:
            n.close()


def test_mac_batch_poll_reports_each_search_once():
    insts = [cp.gen_uneven(800 + i, 12, 30, 16) for i in range(12)]
    with cp.Engine(0) as eng:
        nets = [eng.upload(i) for i in insts]
        mb = cp.MacBatch(eng, [(n, []) for n in nets], time_limit_ms=120000)
        seen = {}
        for _ in range(200000):
            done, res = mb.poll()
            for i, r in enumerate(res):
                if r is not None and i not in seen:
                    seen[i] = r
            if done.all():
                break
        assert len(seen) == len(nets)
        final = mb.wait()
        for i, r in enumerate(final):
            _same(r, seen[i], i)
        mb.close()
        for n in nets:
            n.close()


def _lex(inst, mode):
    with cp.Engine(0) as eng:
        eng.set_search_mode(mode)
        net = eng.upload(inst)
        try:
            return net.mac_solve(cp.VarHeuristic.VRH_LEX, cp.ValHeuristic.VLH_MIN)
        except cp.CPError as ex:
            return {"error": ex.code}
        finally:
            net.close()


@pytest.mark.parametrize("p", [0.3, 0.55])
def test_mac_lex_order_device_equals_host(p):
    """VRH_LEX takes vars[|I| + 1] (src/MAC.cpp:366-368): it never branches on
    variable 0 and runs off the end once |I| + 1 = n, which both paths report
    as an error; an unsatisfiable network is refuted with equal counts."""
    inst = cp.gen_binary(20, 8, 60, p, p, 0.0, 9)
    d, h = _lex(inst, 0), _lex(inst, 1)
    if "error" in h:
        assert d.get("error") == h["error"]
    else:
        _same(d, h, "lex")


def _gsolve(inst, mode):
    with cp.Engine(0) as eng:
        eng.set_search_mode(mode)
        net = eng.upload(inst)
        r = net.gsolver_solve(time_limit_ms=120000)
        net.close()
    return r


@pytest.mark.parametrize("args", [("binary", 50, 16, 250, 0.3, 0.3, 0.0, 1), ("binary", 50, 16, 250, 0.3, 0.3, 0.0, 2),
                                  ("binary", 24, 8, 110, 0.42, 0.42, 0.0, 5), ("binary", 30, 100, 60, 0.5, 0.5, 0.1, 3),
                                  ("binary", 14, 200, 30, 0.6, 0.6, 0.0, 4),
                                  ("mixed", 30, 8, 60, 0.3, 0.5, 40, 60, 0.2, 2)])
def test_gsolver_device_equals_host_driven(args):
    """The d-way search of GModelSolver run whole on the device gives the
    host-driven search's node counts, verdict and solution."""
    inst = cp.gen_binary(*args[1:]) if args[0] == "binary" else cp.gen_mixed(*args[1:])
    d, h = _gsolve(inst, 0), _gsolve(inst, 1)
    _same(d, h, args)
    if d["status"] == 1:
        from tests.golden_cases import oracle_view_of
        from oracle import pyoracle as O
        assert O.check_solution(oracle_view_of(inst), d["solution"])


def test_gsolver_matches_oracle_dway(golden):
    """cp_gsolver_solve against the oracle's restatement of GModelSolver's
    d-way search (src/GModelSolver.cu:104-189, GetMinDomainVar
    src/GModel.cu:1553-1572) on the networks of the MAC golden cases: the same
    positive and negative node counts, verdict and first solution, in both
    search modes."""
    from oracle import pyoracle as O
    from tests.golden_cases import oracle_view_of
    seen, cases = set(), []
    for c in golden:
        if c["op"] == "mac" and tuple(c["args"]) not in seen:
            seen.add(tuple(c["args"]))
            cases.append(c["args"])
    assert len(cases) >= 20
    for mode in (0, 1):
        with cp.Engine(0) as eng:
            eng.set_search_mode(mode)
            for args in cases:
                inst = make_engine_instance(args)
                ref = O.dway(oracle_view_of(inst), time_limit_ms=120000)
                assert ref["status"] in (0, 1), args
                net = eng.upload(inst)
                r = net.gsolver_solve(time_limit_ms=120000)
                net.close()
                assert r["status"] == ref["status"], (args, mode)
                assert (r["num_positive"], r["num_negative"]) == (ref["num_positive"], ref["num_negative"]), \
                    (args, mode)
                if r["status"] == 1:
                    assert r["solution"] == ref["solution"], (args, mode)


@pytest.mark.parametrize("which", ["queens8", "mixed"])
def test_xcsp_instances_on_the_device(which):
    """Networks read from XCSP text: device GAC and MAC equal the oracle's."""
    from cpim_gb300.xcsp import read_xcsp
    from oracle import pyoracle as O
    from tests.golden_cases import oracle_view_of
    from tests.test_xcsp import MIXED, _queens_xml
    m = read_xcsp(_queens_xml(8) if which == "queens8" else MIXED)
    ov = oracle_view_of(m.inst)
    ok, d, _ = O.gac(ov)
    ref = O.mac(ov)
    with cp.Engine(0) as eng:
        net = eng.upload(m.inst)
        st = net.enforce_ac(0)
        assert bool(st.inconsistent) == (not ok)
        if ok:
            assert np.array_equal(net.dom_get(0), d)
        net.close()
        net = eng.upload(m.inst)
        r = net.mac_solve()
        net.close()
    assert r["status"] == ref["status"]
    assert (r["num_positive"], r["num_negative"]) == (ref["num_positive"], ref["num_negative"])
    if r["status"] == 1:
        assert r["solution"] == ref["solution"]


@pytest.mark.parametrize("mode", [0, 1])
def test_mac_domdeg_matches_reference(golden, mode):
    # VRH_DOM_DEG_MIN (src/MAC.cpp:371-386): chosen inside the device search
    # (mode 0) or on the host from the device's domain sizes (mode 1);
    # decision counts and first solutions equal the reference's own MAC runs.
    cases = [c for c in golden if c["op"] == "mac_domdeg"]
    assert len(cases) >= 20
    with cp.Engine(0) as e:
        e.set_search_mode(mode)
        for c in cases:
            net = e.upload(make_engine_instance(c["args"]))
            m = net.mac_solve(cp.VarHeuristic.VRH_DOM_DEG_MIN, cp.ValHeuristic.VLH_MIN, time_limit_ms=120000)
            r = c["result"]
            assert (m["status"] == 1) == (r["num_sol"] == 1), c["args"]
            assert (m["num_positive"], m["num_negative"]) == (r["num_positive"], r["num_negative"]), c["args"]
            if m["status"] == 1:
                assert m["solution"] == r["solution"], c["args"]
            net.close()


def test_mac_domdeg_batched_matches_reference(golden):
    """All dom/deg golden networks as one batched device search."""
    cases = [c for c in golden if c["op"] == "mac_domdeg"]
    with cp.Engine(0) as e:
        nets = [e.upload(make_engine_instance(c["args"])) for c in cases]
        mb = cp.MacBatch(e, [(n, []) for n in nets], var_h=cp.VarHeuristic.VRH_DOM_DEG_MIN, time_limit_ms=120000)
        res = mb.wait()
        mb.close()
        for c, m in zip(cases, res):
            r = c["result"]
            assert (m["num_positive"], m["num_negative"]) == (r["num_positive"], r["num_negative"]), c["args"]
            if r["num_sol"] == 1:
                assert m["solution"] == r["solution"], c["args"]
        for n in nets:
            n.close()


@pytest.mark.parametrize("mode", [0, 1])
def test_mac_domwdeg_matches_reference(golden, mode):
    # VRH_DOM_WDEG_MIN (src/MAC.cpp:387-408): weights from replays of the
    # failing nodes in the reference's AC3 order; decision counts and first
    # solutions equal the reference's own MAC runs (search mode does not
    # matter: dom/wdeg always runs host-driven).
    cases = [c for c in golden if c["op"] == "mac_domwdeg"]
    assert len(cases) >= 20
    with cp.Engine(0) as e:
        e.set_search_mode(mode)
        for c in cases:
            net = e.upload(make_engine_instance(c["args"]))
            m = net.mac_solve(cp.VarHeuristic.VRH_DOM_WDEG_MIN, cp.ValHeuristic.VLH_MIN, time_limit_ms=120000)
            r = c["result"]
            assert (m["status"] == 1) == (r["num_sol"] == 1), c["args"]
            assert (m["num_positive"], m["num_negative"]) == (r["num_positive"], r["num_negative"]), c["args"]
            if m["status"] == 1:
                assert m["solution"] == r["solution"], c["args"]
            net.close()


def test_search_block_sizes_give_the_same_search():
    # cp_engine_set_search_block: any CTA size (a multiple of 32 up to 512)
    # runs the same search; other sizes are refused.
    inst = cp.gen_binary(50, 16, 250, 0.3, 0.3, 0.0, 4)
    with cp.Engine(0) as eng:
        for bad in (-32, 16, 33, 544):
            with pytest.raises(cp.CPError):
                eng.set_search_block(bad)
        want = None
        for block in (0, 32, 64, 128, 256, 512):
            eng.set_search_block(block)
            net = eng.upload(inst)
            r = net.mac_solve()
            net.close()
            got = (r["status"], r["num_positive"], r["num_negative"], r["solution"])
            want = want or got
            assert got == want, block
