"""The reference's own benchmark instances (its samples/bench XCSP files:
queens, composed-25-1-2, rand-2-23, haystacks) on the GPU: MAC with dom/min
and min value order to the first solution, the device-resident search and
the host-driven one, against the reference's own MAC run on the same network
(tests/golden/xcsp_reference_cases.json, made by
tests/golden/make_xcsp_golden.py): equal positive and negative decision
counts, verdict and first solution; the root AC closure against the
reference's AC3bit. Needs the instance files: $CPIM_SAMPLES (a copy of the
samples/bench directory) or the reference checkout; skipped without them."""
import json
import os

import numpy as np
import pytest

import cpim_gb300 as cp
from cpim_gb300.xcsp import read_xcsp
from tests.golden_cases import dom_hex, reference_root

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def _samples():
    d = os.environ.get("CPIM_SAMPLES")
    if d and os.path.isdir(d):
        return d
    ref = reference_root()
    return os.path.join(ref, "samples", "bench") if ref else None


SAMPLES = _samples()
if SAMPLES is None:
    pytest.skip("reference sample instances absent", allow_module_level=True)
with open(os.path.join(HERE, "golden", "xcsp_reference_cases.json")) as f:
    CASES = json.load(f)["cases"]
SOLVED = [c for c in CASES if not c["mac"]["time_out"]]


@pytest.mark.parametrize("case", SOLVED, ids=[c["file"] for c in SOLVED])
def test_mac_matches_reference(engine, case):
    m = read_xcsp(os.path.join(SAMPLES, case["file"]))
    ref = case["mac"]
    modes = (0, 1) if ref["num_positive"] < 5000 else (0,)
    for mode in modes:
        engine.set_search_mode(mode)
        try:
            net = engine.upload(m.inst)
            r = net.mac_solve(time_limit_ms=300000)
            net.close()
        finally:
            engine.set_search_mode(0)
        assert r["status"] == (1 if ref["num_sol"] == 1 else 0), (case["file"], mode)
        assert (r["num_positive"], r["num_negative"]) == (ref["num_positive"], ref["num_negative"]), (case["file"], mode)
        if r["status"] == 1:
            assert r["solution"] == ref["solution"], (case["file"], mode)


@pytest.mark.parametrize("case", CASES, ids=[c["file"] for c in CASES])
def test_root_ac_matches_reference(engine, case):
    m = read_xcsp(os.path.join(SAMPLES, case["file"]))
    ref = case["ac3bit"]
    net = engine.upload(m.inst)
    st = net.enforce_ac(0)
    assert bool(st.inconsistent) == (not ref["consistent"])
    if ref["consistent"]:
        assert dom_hex(net.dom_get(0)) == ref["domains"]
    net.close()


def test_all_solved_instances_in_one_batch():
    """Every solved instance as one batched device search (one launch for all),
    each result equal to the reference's."""
    ms = [read_xcsp(os.path.join(SAMPLES, c["file"])) for c in SOLVED]
    with cp.Engine(0) as eng:
        nets = [eng.upload(m.inst) for m in ms]
        mb = cp.MacBatch(eng, [(n, []) for n in nets], time_limit_ms=300000)
        res = mb.wait()
        mb.close()
        for c, r in zip(SOLVED, res):
            ref = c["mac"]
            assert (r["num_positive"], r["num_negative"]) == (ref["num_positive"], ref["num_negative"]), c["file"]
            if ref["num_sol"] == 1:
                assert r["solution"] == ref["solution"], c["file"]
        for n in nets:
            n.close()
