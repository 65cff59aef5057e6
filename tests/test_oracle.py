"""CPU tests: the oracle restatement against the reference's own outputs
(golden fixtures generated by tests/golden/make_golden.py from the reference
sources), and the oracle's GAC against the literal definition of the
reference's verifier (samples/verify_gac.cpp) and against brute force."""
import numpy as np
import pytest

from oracle import pyoracle as O
from tests.golden_cases import make_oracle_instance


def _cases(golden, op, names=None):
    return [c for c in golden if c["op"] == op and (names is None or c["name"] in names)]


def test_fixture_fingerprints(golden):
    seen = {}
    for c in golden:
        key = tuple(c["args"])
        if key in seen or c["args"][0] == "mixedbin":
            # mixedbin fingerprints cover the table-less copy; the full mixed
            # instance is checked through its own case.
            continue
        inst = make_oracle_instance(c["args"])
        seen[key] = inst.fingerprint
        assert inst.fingerprint == c["result"]["fingerprint"], c["args"]


def test_ac3bit_matches_reference(golden):
    cases = _cases(golden, "ac3bit")
    assert len(cases) >= 40
    for c in cases:
        inst = make_oracle_instance(c["args"])
        ok, d, dels = O.ac3bit(inst)
        r = c["result"]
        assert ok == r["consistent"], c["args"]
        assert dels == r["deletions"], c["args"]
        if ok:
            assert O.dom_hex(d) == r["domains"], c["args"]


def test_sac1_matches_reference(golden):
    cases = _cases(golden, "sac1")
    assert len(cases) >= 40
    for c in cases:
        inst = make_oracle_instance(c["args"])
        ok, d, dels = O.sac1(inst)
        r = c["result"]
        assert ok == r["consistent"], c["args"]
        assert dels == r["deletions"], c["args"]
        if ok:
            assert O.dom_hex(d) == r["domains"], c["args"]


def test_mac_matches_reference(golden):
    cases = _cases(golden, "mac")
    assert len(cases) >= 20
    for c in cases:
        inst = make_oracle_instance(c["args"])
        m = O.mac(inst)
        r = c["result"]
        assert m["num_positive"] == r["num_positive"], c["args"]
        assert m["num_negative"] == r["num_negative"], c["args"]
        assert (m["status"] == 1) == (r["num_sol"] == 1), c["args"]
        if m["status"] == 1:
            assert m["solution"] == r["solution"], c["args"]
            assert O.check_solution(inst, m["solution"])


def test_mac_domdeg_matches_reference(golden):
    # VRH_DOM_DEG_MIN (src/MAC.cpp:371-386): integer size / |neighbourhood|,
    # the first strict minimum; decision counts and first solution exact.
    cases = _cases(golden, "mac_domdeg")
    assert len(cases) >= 20
    for c in cases:
        inst = make_oracle_instance(c["args"])
        m = O.mac(inst, varh=4)
        r = c["result"]
        assert m["num_positive"] == r["num_positive"], c["args"]
        assert m["num_negative"] == r["num_negative"], c["args"]
        assert (m["status"] == 1) == (r["num_sol"] == 1), c["args"]
        if m["status"] == 1:
            assert m["solution"] == r["solution"], c["args"]
            assert O.check_solution(inst, m["solution"])


def test_mac_domwdeg_matches_reference(golden):
    # VRH_DOM_WDEG_MIN (src/MAC.cpp:387-408) with the weights AC3::enforce
    # raises on the constraint whose revision wipes a domain out first
    # (src/AC3.cpp:122-128): decision counts and first solution exact.
    cases = _cases(golden, "mac_domwdeg")
    assert len(cases) >= 20
    for c in cases:
        inst = make_oracle_instance(c["args"])
        m = O.mac(inst, varh=6)
        r = c["result"]
        assert (m["num_positive"], m["num_negative"]) == (r["num_positive"], r["num_negative"]), c["args"]
        assert (m["status"] == 1) == (r["num_sol"] == 1), c["args"]
        if m["status"] == 1:
            assert m["solution"] == r["solution"], c["args"]


def test_mac_rejects_unknown_heuristic(golden):
    inst = make_oracle_instance(_cases(golden, "mac")[0]["args"])
    with pytest.raises(ValueError):
        O.mac(inst, varh=5)


def test_gac_equals_ac3bit_on_binary(golden):
    # The GAC worklist restatement gives the AC3bit closure on binary networks.
    for c in _cases(golden, "ac3bit"):
        inst = make_oracle_instance(c["args"])
        ok1, d1, _ = O.ac3bit(inst)
        ok2, d2, _ = O.gac(inst)
        assert ok1 == ok2
        if ok1:
            assert np.array_equal(d1, d2)


@pytest.mark.parametrize("seed", range(1, 9))
def test_gac_matches_definition_mixed(seed):
    inst = O.gen_mixed(12, 8, 20, 0.3, 0.6, 10, 40, 0.2, seed)
    ok1, d1, _ = O.gac(inst)
    ok2, d2 = O.gac_definitional(inst)
    assert ok1 == ok2
    if ok1:
        assert np.array_equal(d1, d2)


def _nary_instance(seed, n=14, d=4, n_tab=5, arities=(5, 6), ntup=(14, 48)):
    # Positive tables of arity 5 and 6 over small domains (no binary rows);
    # over seeds 1..8 GAC deletes values in most, wipes one out, and one has
    # a solution.
    rng = np.random.default_rng(seed)
    ar, sc, nt, tu = [], [], [], []
    for _ in range(n_tab):
        r = int(rng.choice(arities))
        scope = rng.choice(n, size=r, replace=False)
        k = int(rng.integers(*ntup))
        space = rng.choice(d ** r, size=k, replace=False)
        tuples = [[(int(code) // d ** i) % d for i in range(r)] for code in space]
        ar.append(r)
        sc.extend(int(v) for v in scope)
        nt.append(k)
        tu.extend(v for t in tuples for v in t)
    init = np.full(n, (1 << d) - 1, dtype=np.uint64)
    for x in rng.choice(n, size=3, replace=False):  # a few values removed up front
        init[x] &= ~np.uint64(1 << int(rng.integers(0, d)))
    z = np.zeros(0, np.int32)
    return O.Instance(n=n, W=1, dom=np.full(n, d, np.int32), init=init, bx=z, by=z.copy(),
                      brows=np.zeros(0, np.uint64), tarity=np.array(ar, np.int32), tscope=np.array(sc, np.int32),
                      tntup=np.array(nt, np.int32), ttup=np.array(tu, np.int32))


@pytest.mark.parametrize("seed", range(1, 9))
def test_gac_nary_matches_definition(seed):
    # Tables beyond arity 4 (the device's wide-table path): the oracle's
    # worklist GAC equals the literal definition of samples/verify_gac.cpp,
    # every solution's values survive it, and a wipe-out has no solution.
    inst = _nary_instance(seed)
    ok1, d1, _ = O.gac(inst)
    ok2, d2 = O.gac_definitional(inst)
    assert ok1 == ok2
    if ok1:
        assert np.array_equal(d1, d2)
        m = O.mac(inst)
        if m["status"] == 1:
            assert O.check_solution(inst, m["solution"])
            for x, a in enumerate(m["solution"]):
                assert (int(d1[x]) >> a) & 1
    else:
        assert O.mac(inst)["status"] == 0


def test_gac_mixed_binary_part_pinned(golden):
    # The binary sub-network of each mixed instance matches the reference
    # AC3bit, and adding the tables only removes more.
    for c in _cases(golden, "ac3bit", {"mixedbin"}):
        binonly = make_oracle_instance(c["args"])
        ok, d, _ = O.gac(binonly)
        assert ok == c["result"]["consistent"]
        assert O.dom_hex(d) == c["result"]["domains"]
        mixed = make_oracle_instance(["mixed"] + c["args"][1:])
        okm, dm, _ = O.gac(mixed)
        if okm:
            assert np.all((dm & ~d) == 0)


def test_reference_ac3_mixed_arity_defect_recorded(golden):
    # The reference's generic AC3 reports wipe-outs on mixed-arity networks
    # whose GAC closure is not empty (src/AC.cpp:5 sizes its probe tuple to
    # the maximum arity); the oracle does not follow it there.
    cases = _cases(golden, "ac3", {"mixed_ref_ac3"})
    assert cases
    disagree = 0
    for c in cases:
        inst = make_oracle_instance(c["args"])
        ok, _, _ = O.gac(inst)
        ok_def, _ = O.gac_definitional(inst)
        assert ok == ok_def
        assert ok, c["args"]
        disagree += int(not c["result"]["consistent"])
    assert disagree == len(cases)


@pytest.mark.parametrize("seed", range(1, 13))
def test_mac_agrees_with_brute_force(seed):
    inst = O.gen_binary(10, 4, 25, 0.45, 0.45, 0.0, seed)
    m = O.mac(inst)
    b = O.brute_solve(inst, 1e7)
    assert b in (0, 1)
    assert (m["status"] == 1) == (b == 1)
    if m["status"] == 1:
        assert O.check_solution(inst, m["solution"])


@pytest.mark.parametrize("seed", range(1, 7))
def test_sac_values_pass_singletons(seed):
    # Every value left by SAC1 passes its singleton test on the SAC domains,
    # and SAC1 is idempotent.
    inst = O.gen_binary(20, 6, 60, 0.4, 0.4, 0.1, seed)
    ok, d, _ = O.sac1(inst)
    if not ok:
        return
    for x in range(inst.n):
        for a in range(int(inst.dom[x])):
            if (int(d[x * inst.W + (a >> 6)]) >> (a & 63)) & 1:
                assert O.singleton(inst, d, x, a)
    ok2, d2, dels2 = O.sac1(inst, d)
    assert ok2 and dels2 == 0 and np.array_equal(d, d2)


def test_dway_verdicts_and_solutions(golden):
    """The d-way restatement of GModelSolver agrees with the reference MAC's
    verdict on every MAC golden network, and its solutions satisfy every
    constraint."""
    seen = set()
    for c in golden:
        if c["op"] != "mac" or tuple(c["args"]) in seen:
            continue
        seen.add(tuple(c["args"]))
        inst = make_oracle_instance(c["args"])
        r = O.dway(inst, time_limit_ms=60000)
        assert r["status"] == (1 if c["result"]["num_sol"] == 1 else 0), c["args"]
        if r["status"] == 1:
            assert O.check_solution(inst, r["solution"])
        assert r["num_negative"] <= r["num_positive"]


def test_sac_jacobi_matches_reference_sac1(golden):
    """The Jacobi-order SAC closure on host threads equals the reference's
    sequential SAC1 on every SAC1 golden case (the closure is unique)."""
    cases = [c for c in golden if c["op"] == "sac1"]
    assert len(cases) >= 40
    for c in cases:
        inst = make_oracle_instance(c["args"])
        ok, d, _, _ = O.sac_jacobi(inst, threads=4)
        assert ok == c["result"]["consistent"], c["args"]
        if ok:
            assert O.dom_hex(d) == c["result"]["domains"], c["args"]


def test_singleton_verdicts_match_reference(golden):
    """Every singleton verdict over the root AC closure equals the reference's
    own singleton test (the verdicts golden cases)."""
    cases = [c for c in golden if c["op"] == "verdicts"]
    assert len(cases) >= 8
    for c in cases:
        inst = make_oracle_instance(c["args"])
        ok, d, _ = O.ac3bit(inst)
        assert ok == c["result"]["consistent"], c["args"]
        if not ok:
            continue
        ver, failed = O.singleton_verdicts(inst, d, threads=4)
        got = set()
        for x in range(inst.n):
            for a in range(int(inst.dom[x])):
                w = x * inst.W + a // 64
                if (int(d[w]) >> (a % 64)) & 1 and not (int(ver[w]) >> (a % 64)) & 1:
                    got.add((x, a))
        assert got == set(map(tuple, c["result"]["failed"])), c["args"]
        assert failed == len(got)


def test_nary_cases_pinned_by_definition():
    # Every n-ary case the GPU tests compare against (tables of arity up to
    # 40, domains up to 512 values, grid-sized networks of 8 values): the
    # oracle's worklist GAC equals the literal definition, and its SAC1
    # closure only removes more. (The literal definition takes minutes on the
    # grid-sized network of 400 values, which is left out here.)
    from tests.nary_cases import CASES, GRID_CASES, SEEDS, nary_arrays, to_oracle
    cases = [(name, kw, SEEDS) for name, kw in CASES] + \
            [(name, kw, (1, 2)) for name, kw in GRID_CASES if kw["d"] <= 64]
    for name, kw, seeds in cases:
        for seed in seeds:
            inst = to_oracle(nary_arrays(seed, **kw))
            ok1, d1, _ = O.gac(inst)
            ok2, d2 = O.gac_definitional(inst)
            assert ok1 == ok2, (name, seed)
            if ok1:
                assert np.array_equal(d1, d2), (name, seed)
                if inst.n <= 48:
                    oks, ds, _ = O.sac1(inst)
                    assert not oks or np.all((ds & ~d1) == 0), (name, seed)


def _nary_reference_cases():
    import json
    import os
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "nary_reference_cases.json")
    with open(path) as f:
        cases = json.load(f)["cases"]
    for c in cases:
        c["kwargs"] = {k: tuple(v) if isinstance(v, list) else v for k, v in c["kwargs"].items()}
    return cases


def test_nary_gac_pinned_by_reference_ac3():
    # Networks whose tables all have one arity (2 .. 12, domains up to 300
    # values): the reference's own generic AC3 (run by
    # tests/golden/make_nary_golden.py) and the oracle's GAC agree on the
    # verdict, the deletions and every domain word.
    from tests.nary_cases import nary_arrays, to_oracle
    for c in _nary_reference_cases():
        inst = to_oracle(nary_arrays(c["seed"], **c["kwargs"]))
        ok, d, dels = O.gac(inst)
        ref = c["result"]
        assert ok == ref["consistent"], (c["name"], c["seed"])
        if ok:
            assert dels == ref["deletions"], (c["name"], c["seed"])
            assert O.dom_hex(d) == ref["domains"], (c["name"], c["seed"])


def test_nary_sac1_pinned_by_reference():
    # The same one-arity networks (domains of at most 16 values): the
    # reference's SAC1 over its generic AC3 and the oracle's SAC1 agree on the
    # verdict and, when consistent, on the deletions and every domain word.
    from tests.nary_cases import nary_arrays, to_oracle
    n = 0
    for c in _nary_reference_cases():
        if "sac1" not in c:
            continue
        ok, d, dels = O.sac1(to_oracle(nary_arrays(c["seed"], **c["kwargs"])))
        ref = c["sac1"]
        assert ok == ref["consistent"], (c["name"], c["seed"])
        if ok:
            assert dels == ref["deletions"], (c["name"], c["seed"])
            assert O.dom_hex(d) == ref["domains"], (c["name"], c["seed"])
        n += 1
    assert n >= 30


def test_nary_mac_pinned_by_reference():
    # The same one-arity networks: the reference's MAC over its generic AC3
    # (dom/min and dom/deg, min value) and the oracle's MAC agree on the node
    # counts and the first solution.
    from tests.nary_cases import nary_arrays, to_oracle
    n = 0
    for c in _nary_reference_cases():
        for key, varh in (("mac", 1), ("mac_domdeg", 4)):
            if key not in c:
                continue
            ref = c[key]
            assert not ref["time_out"]
            m = O.mac(to_oracle(nary_arrays(c["seed"], **c["kwargs"])), varh=varh)
            assert (m["num_positive"], m["num_negative"]) == (ref["num_positive"], ref["num_negative"]), (c["name"], key)
            assert m["solution"] == (ref["solution"] if ref["num_sol"] else []), (c["name"], key)
            n += 1
    assert n >= 60
