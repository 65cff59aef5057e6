"""XCSP 2.x reader: hand-written instances whose solutions are checked by
brute force in Python, and the reference's own sample files when they are
present (solutions checked against the XML constraints themselves)."""
import itertools
import os
import xml.etree.ElementTree as ET

import pytest

from cpim_gb300.xcsp import read_xcsp
from oracle import pyoracle as O
from tests.golden_cases import oracle_view_of, reference_root


def _queens_xml(k):
    """k-queens with one conflicts relation per distance (own text)."""
    rels, cons = [], []
    for dist in range(1, k):
        bad = [(a, b) for a in range(1, k + 1) for b in range(1, k + 1) if a == b or abs(a - b) == dist]
        rels.append('<relation name="R%d" arity="2" nbTuples="%d" semantics="conflicts">%s</relation>'
                    % (dist, len(bad), "|".join("%d %d" % t for t in bad)))
    ci = 0
    for i in range(k):
        for j in range(i + 1, k):
            cons.append('<constraint name="C%d" arity="2" scope="Q%d Q%d" reference="R%d"/>' % (ci, i, j, j - i))
            ci += 1
    return ("<instance><presentation format=\"XCSP 2.1\"/><domains><domain name=\"D\">1..%d</domain></domains>"
            "<variables>%s</variables><relations>%s</relations><constraints>%s</constraints></instance>"
            % (k, "".join('<variable name="Q%d" domain="D"/>' % i for i in range(k)), "".join(rels), "".join(cons)))


def _ok_queens(sol):
    k = len(sol)
    return all(sol[i] != sol[j] and abs(sol[i] - sol[j]) != j - i for i in range(k) for j in range(i + 1, k))


@pytest.mark.parametrize("k", [4, 6, 8])
def test_queens_text(k):
    m = read_xcsp(_queens_xml(k))
    assert m.inst.n == k and m.inst.n_bin == k * (k - 1) // 2
    r = O.mac(oracle_view_of(m.inst))
    assert r["status"] == 1
    vals = m.solution_values(r["solution"])
    assert _ok_queens([vals["Q%d" % i] for i in range(k)])


MIXED = """<instance><presentation format="XCSP 2.1"/>
<domains><domain name="A">0 2 5..7</domain><domain name="B">-1..1</domain></domains>
<variables><variable name="x" domain="A"/><variable name="y" domain="B"/><variable name="z" domain="A"/>
<variable name="w" domain="B"/></variables>
<relations>
<relation name="U" arity="1" nbTuples="1" semantics="conflicts">6</relation>
<relation name="T" arity="3" nbTuples="5" semantics="supports">0 -1 2|5 0 7|7 1 0|2 1 5|6 0 6</relation>
<relation name="N" arity="3" nbTuples="3" semantics="conflicts">-1 0 5|0 1 7|1 -1 0</relation>
<relation name="E" arity="2" nbTuples="3" semantics="supports">-1 1|0 0|1 -1</relation>
</relations>
<constraints>
<constraint name="c0" arity="1" scope="x" reference="U"/>
<constraint name="c1" arity="3" scope="x y z" reference="T"/>
<constraint name="c2" arity="3" scope="y w z" reference="N"/>
<constraint name="c3" arity="2" scope="y w" reference="E"/>
</constraints></instance>"""


def _brute(xml):
    root = ET.fromstring(xml)
    doms = {d.get("name"): d.text for d in root.iter("domain")}

    def vals(t):
        out = []
        for p in t.split():
            if ".." in p:
                a, b = map(int, p.split(".."))
                out += range(a, b + 1)
            else:
                out.append(int(p))
        return sorted(set(out))
    names = [v.get("name") for v in root.iter("variable")]
    dv = [vals(doms[v.get("domain")]) for v in root.iter("variable")]
    rels = {}
    for r in root.iter("relation"):
        ar = int(r.get("arity"))
        flat = [int(t) for t in r.text.replace("|", " ").split()]
        rels[r.get("name")] = (r.get("semantics"), {tuple(flat[i:i + ar]) for i in range(0, len(flat), ar)})
    cons = [(c.get("scope").split(), c.get("reference")) for c in root.iter("constraint")]

    def ok(assign):
        for scope, ref in cons:
            sem, ts = rels[ref]
            if (tuple(assign[s] for s in scope) in ts) != (sem == "supports"):
                return False
        return True
    sols = [dict(zip(names, t)) for t in itertools.product(*dv) if ok(dict(zip(names, t)))]
    return sols, ok


def test_mixed_arity_unary_and_conflicts():
    m = read_xcsp(MIXED)
    assert m.inst.n_bin == 1 and len(m.inst.tab_arity) == 2
    sols, ok = _brute(MIXED)
    r = O.mac(oracle_view_of(m.inst))
    assert (r["status"] == 1) == bool(sols)
    if sols:
        assert ok(m.solution_values(r["solution"]))
    # GAC keeps exactly the values that appear in some solution of each single
    # constraint; at least every solution's values survive.
    okg, d, _ = O.gac(oracle_view_of(m.inst))
    assert okg  # the instance has solutions
    if okg:
        for s in sols:
            for x, nm in enumerate(m.names):
                a = m.values[x].index(s[nm])
                assert (int(d[x * m.inst.W + a // 64]) >> (a % 64)) & 1


WIDE = """<instance><presentation format="XCSP 2.1"/>
<domains><domain name="D">1..3</domain></domains>
<variables><variable name="a" domain="D"/><variable name="b" domain="D"/><variable name="c" domain="D"/>
<variable name="d" domain="D"/><variable name="e" domain="D"/><variable name="f" domain="D"/></variables>
<relations>
<relation name="S" arity="5" nbTuples="6" semantics="supports">1 2 3 1 2|2 2 2 2 2|3 1 2 3 1|1 1 1 1 1|2 3 1 3 2|3 3 3 1 1</relation>
<relation name="K" arity="5" nbTuples="3" semantics="conflicts">2 2 2 2 2|1 1 1 1 1|3 3 3 1 1</relation>
<relation name="L" arity="2" nbTuples="2" semantics="conflicts">1 1|2 3</relation>
</relations>
<constraints>
<constraint name="c0" arity="5" scope="a b c d e" reference="S"/>
<constraint name="c1" arity="5" scope="b c d e f" reference="K"/>
<constraint name="c2" arity="2" scope="a f" reference="L"/>
</constraints></instance>"""


def test_arity_five_supports_and_conflicts():
    # Constraints above arity 4 become positive tables (a conflicts relation
    # as the rest of its Cartesian product); the oracle's MAC on them agrees
    # with brute force over the XCSP semantics.
    m = read_xcsp(WIDE)
    assert m.inst.n_bin == 1 and m.inst.tab_arity.tolist() == [5, 5]
    assert m.inst.tab_ntup.tolist() == [6, 3 ** 5 - 3]
    sols, ok = _brute(WIDE)
    r = O.mac(oracle_view_of(m.inst))
    assert (r["status"] == 1) == bool(sols)
    if sols:
        assert ok(m.solution_values(r["solution"]))
    okg, d, _ = O.gac(oracle_view_of(m.inst))
    assert okg == bool(sols) or okg
    for sol in sols:
        for x, nm in enumerate(m.names):
            a = m.values[x].index(sol[nm])
            assert (int(d[x * m.inst.W + a // 64]) >> (a % 64)) & 1


_REF = reference_root()
SAMPLES = os.path.join(_REF, "samples", "bench") if _REF else ""


@pytest.mark.skipif(not os.path.isdir(SAMPLES), reason="reference samples absent")
@pytest.mark.parametrize("name", ["queens-4_ext.xml", "test.xml"])
def test_reference_samples(name):
    path = os.path.join(SAMPLES, name)
    m = read_xcsp(path)
    text = open(path).read()
    sols, ok = _brute(text) if m.inst.n <= 6 else (None, None)
    r = O.mac(oracle_view_of(m.inst))
    if sols is not None:
        assert (r["status"] == 1) == bool(sols)
        if r["status"] == 1:
            assert ok(m.solution_values(r["solution"]))
