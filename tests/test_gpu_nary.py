"""Positive tables of any arity, and tables over domains of more than 256
values, on the device against the oracle's GAC (the generic table revise of
src/AC3.cpp:195-209, checked against the definition of
samples/verify_gac.cpp:121-164), SAC1 and MAC."""
import numpy as np
import pytest

import cpim_gb300 as cp
from oracle import pyoracle as O
from tests.nary_cases import CASES, GRID_CASES, SEEDS, nary_arrays, to_engine, to_oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def engine():
    with cp.Engine(0) as e:
        yield e


def _ids(cases):
    return [c[0] for c in cases]


@pytest.mark.parametrize("name,kw", CASES, ids=_ids(CASES))
def test_nary_gac_matches_oracle(engine, name, kw):
    for seed in SEEDS:
        a = nary_arrays(seed, **kw)
        ok, d, dels = O.gac(to_oracle(a))
        net = engine.upload(to_engine(a))
        st = net.enforce_ac(0)
        assert bool(st.inconsistent) == (not ok), (name, seed)
        if ok:
            assert st.deletions == dels, (name, seed)
            assert np.array_equal(net.dom_get(0), d), (name, seed)
            st2 = net.enforce_ac(0)
            assert st2.deletions == 0 and not st2.inconsistent
        net.close()


@pytest.mark.parametrize("name,kw", CASES, ids=_ids(CASES))
def test_nary_sac1_matches_oracle(engine, name, kw):
    for seed in SEEDS:
        a = nary_arrays(seed, **kw)
        ok, d, dels = O.sac1(to_oracle(a))
        net = engine.upload(to_engine(a))
        st = net.enforce_sac1(0)
        assert bool(st.inconsistent) == (not ok), (name, seed)
        if ok:
            assert st.deletions == dels, (name, seed)
            assert np.array_equal(net.dom_get(0), d), (name, seed)
        net.close()


@pytest.mark.parametrize("varh", [cp.VarHeuristic.VRH_DOM_MIN, cp.VarHeuristic.VRH_DOM_DEG_MIN])
@pytest.mark.parametrize("name,kw", CASES, ids=_ids(CASES))
def test_nary_mac_matches_oracle(engine, name, kw, varh):
    for seed in SEEDS:
        a = nary_arrays(seed, **kw)
        o = O.mac(to_oracle(a), varh=int(varh))
        net = engine.upload(to_engine(a))
        r = net.mac_solve(var_h=varh)
        assert r["status"] == o["status"], (name, seed)
        assert (r["num_positive"], r["num_negative"]) == (o["num_positive"], o["num_negative"]), (name, seed)
        assert r["solution"] == o["solution"], (name, seed)
        net.close()


@pytest.mark.parametrize("name,kw", GRID_CASES, ids=_ids(GRID_CASES))
def test_nary_grid_gac_matches_oracle(engine, name, kw):
    for seed in (1, 2):
        a = nary_arrays(seed, **kw)
        ok, d, dels = O.gac(to_oracle(a))
        net = engine.upload(to_engine(a))
        st = net.enforce_ac(0)
        assert bool(st.inconsistent) == (not ok), (name, seed)
        if ok:
            assert st.deletions == dels, (name, seed)
            assert np.array_equal(net.dom_get(0), d), (name, seed)
        net.close()


def test_nary_batch_matches_oracle(engine):
    # Wide tables of several shapes in one multi-instance batch: AC, then SAC1.
    arrays = [nary_arrays(seed, **kw) for _, kw in CASES[:8] for seed in SEEDS[:2]]
    nets = [engine.upload(to_engine(a)) for a in arrays]
    b = cp.Batch(engine, nets, level=1)   # level 0 keeps the initial domains
    b.copy_level(0)
    _, inc = b.ac()
    doms = b.dom_get()
    for i, a in enumerate(arrays):
        ok, d, _ = O.gac(to_oracle(a))
        assert bool(inc[i]) == (not ok), i
        if ok:
            assert np.array_equal(doms[i], d), i
    b.copy_level(0)
    _, inc = b.sac1()
    doms = b.dom_get()
    for i, a in enumerate(arrays):
        ok, d, _ = O.sac1(to_oracle(a))
        assert bool(inc[i]) == (not ok), i
        if ok:
            assert np.array_equal(doms[i], d), i
    b.close()
    for n in nets:
        n.close()


def test_nary_gac_matches_reference_runs(engine):
    # The device's GAC against the reference's own generic AC3 on networks
    # whose tables all have one arity (tests/golden/nary_reference_cases.json).
    import json
    import os
    from tests.golden_cases import dom_hex
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "nary_reference_cases.json")
    with open(path) as f:
        cases = json.load(f)["cases"]
    for c in cases:
        kw = {k: tuple(v) if isinstance(v, list) else v for k, v in c["kwargs"].items()}
        net = engine.upload(to_engine(nary_arrays(c["seed"], **kw)))
        st = net.enforce_ac(0)
        ref = c["result"]
        assert bool(st.inconsistent) == (not ref["consistent"]), (c["name"], c["seed"])
        if ref["consistent"]:
            assert st.deletions == ref["deletions"], (c["name"], c["seed"])
            assert dom_hex(net.dom_get(0)) == ref["domains"], (c["name"], c["seed"])
        net.close()


def test_nary_sac1_and_mac_match_reference_runs(engine):
    # The device's SAC1 and MAC (dom/min, dom/deg) against the reference's own
    # SAC1 and MAC over its generic AC3 on the one-arity networks of at most
    # 16 values (tests/golden/nary_reference_cases.json).
    import json
    import os
    from tests.golden_cases import dom_hex
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "nary_reference_cases.json")
    with open(path) as f:
        cases = [c for c in json.load(f)["cases"] if "sac1" in c]
    assert len(cases) >= 30
    for c in cases:
        kw = {k: tuple(v) if isinstance(v, list) else v for k, v in c["kwargs"].items()}
        arrays = nary_arrays(c["seed"], **kw)
        net = engine.upload(to_engine(arrays))
        st = net.enforce_sac1(0)
        ref = c["sac1"]
        assert bool(st.inconsistent) == (not ref["consistent"]), (c["name"], c["seed"])
        if ref["consistent"]:
            assert st.deletions == ref["deletions"], (c["name"], c["seed"])
            assert dom_hex(net.dom_get(0)) == ref["domains"], (c["name"], c["seed"])
        net.close()
        for key, varh in (("mac", cp.VarHeuristic.VRH_DOM_MIN), ("mac_domdeg", cp.VarHeuristic.VRH_DOM_DEG_MIN)):
            ref = c[key]
            net = engine.upload(to_engine(arrays))
            r = net.mac_solve(var_h=varh)
            net.close()
            assert (r["num_positive"], r["num_negative"]) == (ref["num_positive"], ref["num_negative"]), (c["name"], key)
            assert r["solution"] == (ref["solution"] if ref["num_sol"] else []), (c["name"], key)
