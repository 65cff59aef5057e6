"""GPU parity at the benchmark sizes, against the reference's own runs.

tests/golden/large_cases.json holds the reference's results (its AC3bit and
SAC1 compiled from its sources, oracle/ref/) on the benchmarked SAC sweep
network (n=500, d=128, e=10000, p=0.40, seed 7), on a network of the same n
and d tight enough that singleton tests fail, round two of a branch removes
values (the deep list of the tiled kernel is not empty) and SAC deletes values
over several sweeps, on mid-size networks with SAC deletions or an empty SAC
closure, and on 64 uneven-batch members over the whole configured range (n in
[20, 400], d up to 256; members whose tuple lists are too large for the
reference's in-memory model here come from the oracle, as each case records).
Final domains are compared through the SHA-256 of their hex string; the
first-sweep verdicts as the exact set of failed (x, a) pairs.
"""
import hashlib
import json
import os

import numpy as np
import pytest

import cpim_gb300 as cp
from tests.golden_cases import dom_hex, make_engine_instance

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
_PATH = os.path.join(HERE, "golden", "large_cases.json")
if not os.path.exists(_PATH):
    pytest.skip("large golden cases not generated (tests/golden/make_golden.py --large)", allow_module_level=True)
with open(_PATH) as f:
    LARGE = json.load(f)["cases"]


def _sha(words):
    return hashlib.sha256(dom_hex(words).encode()).hexdigest()


def _case(name, op, args=None):
    for c in LARGE:
        if c["name"] == name and c["op"] == op and (args is None or c["args"] == args):
            return c
    raise KeyError((name, op))


def _failed_pairs(live, verdict, W):
    """(x, a) pairs live in `live` whose verdict bit is clear."""
    out = set()
    gone = np.asarray(live, np.uint64) & ~np.asarray(verdict, np.uint64)
    for i in np.nonzero(gone)[0]:
        w = int(gone[i])
        x, k = divmod(int(i), W)
        while w:
            b = (w & -w).bit_length() - 1
            out.add((x, k * 64 + b))
            w &= w - 1
    return out


SWEEP_CASES = [(c["name"], c["args"]) for c in LARGE if c["op"] == "verdicts"]


@pytest.mark.parametrize("name,args", SWEEP_CASES, ids=["%s-%s" % (n, a[-1]) for n, a in SWEEP_CASES])
@pytest.mark.parametrize("sac_mode", [0, 1], ids=["tiled", "general"])
def test_first_sweep_verdicts_match_reference(engine, name, args, sac_mode):
    """Every singleton verdict of one Jacobi sweep over the root AC closure
    equals the reference's singleton test (src/SAC1.cpp:70-79) of that value,
    through the tiled kernels and through the general fixpoint kernel alone."""
    ref = _case(name, "verdicts", args)["result"]
    ac = _case(name, "ac3bit", args)["result"]
    inst = make_engine_instance(args)
    assert inst.fingerprint == ref["fingerprint"]
    net = engine.upload(inst, max_levels=2)
    try:
        engine.set_sac_mode(sac_mode)
        verdict, deep, st = net.sac_sweep(0)
    finally:
        engine.set_sac_mode(0)
    assert bool(st.inconsistent) == (not ref["consistent"])
    if ref["consistent"]:
        live = net.dom_get(0)
        assert _sha(live) == ac["domains_sha256"], "root AC closure differs from the reference AC3bit"
        got = _failed_pairs(live, verdict, inst.W)
        want = set(map(tuple, ref["failed"]))
        assert got == want, "failed-test sets differ: %d extra, %d missing" % (len(got - want), len(want - got))
        assert st.branches == ref["live"]
        if name == "tight500" and sac_mode == 0:
            assert deep > 0, "the tight network should hand branches to the general kernel"
    net.close()


SAC_CASES = [(c["name"], c["args"]) for c in LARGE if c["op"] == "sac1" and c["name"] != "uneven_full"]


@pytest.mark.parametrize("name,args", SAC_CASES, ids=["%s-%s" % (n, a[-1]) for n, a in SAC_CASES])
def test_sac_closure_matches_reference(engine, name, args):
    """cp_enforce_sac1 at full size ends at the reference SAC1's closure
    (src/SAC1.cpp:57-103), or wipes out where it does."""
    ref = _case(name, "sac1", args)["result"]
    inst = make_engine_instance(args)
    assert inst.fingerprint == ref["fingerprint"]
    net = engine.upload(inst, max_levels=2)
    st = net.enforce_sac1(0)
    assert bool(st.inconsistent) == (not ref["consistent"])
    if ref["consistent"]:
        assert _sha(net.dom_get(0)) == ref["domains_sha256"]
        assert st.deletions == ref["deletions"]
    net.close()


UNEVEN = [c for c in LARGE if c["name"] == "uneven_full" and c["op"] == "sac1"]


def test_uneven_full_range_batch_matches_reference():
    """64 uneven-batch members drawn over the whole configured range (n up to
    400, d up to 256), AC + SAC1 of all of them in one batch, each member
    against the reference's SAC1 run of that member."""
    insts = [make_engine_instance(c["args"]) for c in UNEVEN]
    for c, inst in zip(UNEVEN, insts):
        assert inst.fingerprint == c["result"]["fingerprint"]
    assert max(i.n for i in insts) > 300 and max(i.W for i in insts) == 4
    with cp.Engine(0) as eng:
        nets = [eng.upload(i, max_levels=2) for i in insts]
        b = cp.Batch(eng, nets, level=0)
        b.tune()
        st, inc = b.sac1()
        doms = b.dom_get()
        for k, c in enumerate(UNEVEN):
            ref = c["result"]
            assert bool(inc[k]) == (not ref["consistent"]), k
            if ref["consistent"]:
                assert _sha(doms[k]) == ref["domains_sha256"], k
        b.close()
        for n in nets:
            n.close()


def test_uneven_full_range_single_matches_reference(engine):
    """The same members one at a time through cp_enforce_sac1."""
    for c in UNEVEN[::4]:
        inst = make_engine_instance(c["args"])
        net = engine.upload(inst, max_levels=2)
        st = net.enforce_sac1(0)
        ref = c["result"]
        assert bool(st.inconsistent) == (not ref["consistent"]), c["args"]
        if ref["consistent"]:
            assert _sha(net.dom_get(0)) == ref["domains_sha256"], c["args"]
        net.close()
