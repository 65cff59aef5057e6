"""GPU test of the C++ facade (include/cpim_gb300.hpp): a C++ program that
uses the reference-shaped API (Network, AC3bit, SAC1, MAC with AC_3bit /
VRH_DOM_MIN / VLH_MIN, GModel + GModelSolver) is compiled against the engine
library and its results are compared with the reference's golden outputs."""
import json
import os
import subprocess

import pytest

from tests.golden_cases import make_oracle_instance

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def demo(tmp_path_factory):
    from cpim_gb300 import build
    build.build()
    out = str(tmp_path_factory.mktemp("facade") / "facade_demo")
    lib_dir = os.path.join(ROOT, "cpim_gb300", "_build")
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-I" + os.path.join(ROOT, "include"),
                           os.path.join(ROOT, "tests", "cpp", "facade_demo.cpp"), "-L" + lib_dir, "-lcpgpu",
                           "-Wl,-rpath," + lib_dir, "-o", out])
    return out


def _golden(golden, name, seed, op):
    for c in golden:
        if c["name"] == name and c["op"] == op and c["args"][-1] == seed:
            return c
    raise KeyError((name, seed, op))


@pytest.mark.parametrize("name,seed", [("cfg1", 1), ("cfg1", 5), ("tight", 1), ("tight", 4), ("tighter", 2)])
def test_facade_matches_reference(demo, golden, name, seed):
    c = _golden(golden, name, seed, "mac")
    _, n, d, e, p, _, rm, s = c["args"]
    res = subprocess.run([demo, str(n), str(d), str(e), str(p), str(rm), str(s)], capture_output=True, text=True,
                         timeout=120)
    assert res.returncode == 0, res.stderr
    runs = {r["op"]: r for r in map(json.loads, res.stdout.strip().splitlines())}
    ac = _golden(golden, name, seed, "ac3bit")["result"]
    assert runs["ac3bit"]["consistent"] == ac["consistent"]
    if ac["consistent"]:
        assert runs["ac3bit"]["domains"] == ac["domains"]
        assert runs["ac3bit"]["deletions"] == ac["deletions"]
    sac = _golden(golden, name, seed, "sac1")["result"]
    assert runs["sac1"]["consistent"] == sac["consistent"]
    if sac["consistent"]:
        assert runs["sac1"]["domains"] == sac["domains"]
        assert runs["sac1"]["deletions"] == sac["deletions"]
    mac = c["result"]
    assert runs["mac"]["num_positive"] == mac["num_positive"]
    assert runs["mac"]["num_negative"] == mac["num_negative"]
    assert runs["mac"]["solution"] == mac["solution"]
    g = runs["gsolver"]
    assert (g["num_solutions"] == 1) == (mac["num_sol"] == 1)
    if g["num_solutions"]:
        from oracle import pyoracle as O
        assert O.check_solution(make_oracle_instance(c["args"]), g["solution"])
