"""The oracle against the reference's own runs at larger sizes
(tests/golden/large_cases.json): root AC3bit closures, the singleton verdicts
over them, and the SAC closure by Jacobi sweeps on host threads, on the
mid-size networks (n = 200-300) and the root AC of the benchmark network."""
import hashlib
import json
import os

import numpy as np
import pytest

from oracle import pyoracle as O
from tests.golden_cases import make_oracle_instance

HERE = os.path.dirname(os.path.abspath(__file__))
_PATH = os.path.join(HERE, "golden", "large_cases.json")
if not os.path.exists(_PATH):
    pytest.skip("large golden cases not generated", allow_module_level=True)
with open(_PATH) as f:
    LARGE = json.load(f)["cases"]


def _sha(d):
    return hashlib.sha256(O.dom_hex(d).encode()).hexdigest()


@pytest.mark.parametrize("c", [c for c in LARGE if c["op"] == "ac3bit"], ids=lambda c: "%s-%s" % (c["name"], c["args"][1]))
def test_ac3bit_closure(c):
    inst = make_oracle_instance(c["args"])
    assert inst.fingerprint == c["result"]["fingerprint"]
    ok, d, dels = O.ac3bit(inst)
    assert ok == c["result"]["consistent"]
    if ok:
        assert _sha(d) == c["result"]["domains_sha256"]
        assert dels == c["result"]["deletions"]


MID = [c for c in LARGE if c["name"] == "mid"]


@pytest.mark.parametrize("c", [c for c in MID if c["op"] == "verdicts"], ids=lambda c: str(c["args"][1:]))
def test_singleton_verdicts(c):
    inst = make_oracle_instance(c["args"])
    ok, d, _ = O.ac3bit(inst)
    ver, failed = O.singleton_verdicts(inst, d)
    gone = d & ~ver
    got = set()
    for i in np.nonzero(gone)[0]:
        x, k = divmod(int(i), inst.W)
        w = int(gone[i])
        while w:
            b = (w & -w).bit_length() - 1
            got.add((x, 64 * k + b))
            w &= w - 1
    assert got == set(map(tuple, c["result"]["failed"]))


@pytest.mark.parametrize("c", [c for c in MID if c["op"] == "sac1"], ids=lambda c: str(c["args"][1:]))
def test_sac_closure(c):
    inst = make_oracle_instance(c["args"])
    ok, d, dels, _ = O.sac_jacobi(inst)
    assert ok == c["result"]["consistent"]
    if ok:
        assert _sha(d) == c["result"]["domains_sha256"]
        assert dels == c["result"]["deletions"]
