"""XCSP 2.x extensional instances into the engine's network format, without
libxml2 (Python's own XML parser).

Covers what the reference's samples use (the structure its libxml2 reader
walks, include/model/libxml2_parser.h:57-76): <domain> value lists with
`a..b` ranges, <variable> with a domain reference, <relation> tuple lists
`v1 v2|v3 v4` with `supports` or `conflicts` semantics, and <constraint> with
a scope and a relation reference. Values are mapped to indices 0..d-1 per
variable in increasing order. Unary constraints filter the initial domains;
binary ones become support rows; those of higher arity become positive
tables (a `conflicts` table is turned into the supports of the rest of its
Cartesian product, which must stay below `max_table`)."""
from __future__ import annotations

import itertools
import xml.etree.ElementTree as ET
from dataclasses import dataclass

import numpy as np

from . import Instance


@dataclass
class XcspModel:
    inst: Instance
    names: list          # variable names, in index order
    values: list         # values[x][a] = the XCSP value of index a of variable x

    def solution_values(self, solution):
        """Engine solution (value indices) as the instance's own values."""
        return {self.names[x]: self.values[x][a] for x, a in enumerate(solution)}


def _values(text):
    out = []
    for part in (text or "").split():
        if ".." in part:
            lo, hi = part.split("..")
            out.extend(range(int(lo), int(hi) + 1))
        else:
            out.append(int(part))
    return sorted(set(out))


def _tuples(text, arity):
    flat = [int(t) for t in (text or "").replace("|", " ").split()]
    if len(flat) % arity:
        raise ValueError("tuple list length is not a multiple of the arity")
    return [tuple(flat[i:i + arity]) for i in range(0, len(flat), arity)]


def read_xcsp(source, max_table=200000) -> XcspModel:
    """source: a file path or the XML text itself."""
    src = source.strip()
    root = ET.fromstring(src) if src.startswith("<") else ET.parse(source).getroot()
    domains = {d.get("name"): _values(d.text) for d in root.iter("domain")}
    names, values = [], []
    for v in root.iter("variable"):
        names.append(v.get("name"))
        values.append(domains[v.get("domain")])
    index = {nm: i for i, nm in enumerate(names)}
    n = len(names)
    if n == 0:
        raise ValueError("no variables")
    dom = np.array([len(v) for v in values], np.int32)
    if (dom < 1).any() or dom.max() > 512:
        raise ValueError("domain sizes must be 1..512")
    W = (int(dom.max()) + 63) // 64
    pos = [{val: a for a, val in enumerate(v)} for v in values]
    init = np.zeros(n * W, np.uint64)
    for x in range(n):
        for a in range(dom[x]):
            init[x * W + a // 64] |= np.uint64(1 << (a % 64))
    relations = {r.get("name"): (r.get("semantics", "supports"), int(r.get("arity")), r.text)
                 for r in root.iter("relation")}
    scopes, rows, t_ar, t_sc, t_nt, t_tu = [], [], [], [], [], []
    for c in root.iter("constraint"):
        scope = [index[s] for s in c.get("scope").split()]
        sem, arity, text = relations[c.get("reference")]
        if arity != len(scope):
            raise ValueError("constraint %s: scope and relation arity differ" % c.get("name"))
        tuples = []
        for t in _tuples(text, arity):
            idx = [pos[x].get(v) for x, v in zip(scope, t)]
            if None not in idx:  # tuples with values outside a domain never apply
                tuples.append(tuple(idx))
        if arity == 1:
            x = scope[0]
            keep = {t[0] for t in tuples}
            for a in range(dom[x]):
                if (a in keep) != (sem == "supports"):
                    init[x * W + a // 64] &= ~np.uint64(1 << (a % 64))
        elif arity == 2:
            x, y = scope
            if x == y:
                raise ValueError("binary constraint on one variable")
            allowed = set(tuples)
            r = np.zeros(dom[x] * W, np.uint64)
            for a in range(dom[x]):
                for b in range(dom[y]):
                    if ((a, b) in allowed) == (sem == "supports"):
                        r[a * W + b // 64] |= np.uint64(1 << (b % 64))
            scopes += [x, y]
            rows.append(r)
        else:
            if sem == "conflicts":
                size = int(np.prod([dom[x] for x in scope]))
                if size > max_table:
                    raise ValueError("conflicts table too large to complement: %d tuples" % size)
                banned = set(tuples)
                tuples = [t for t in itertools.product(*[range(dom[x]) for x in scope]) if t not in banned]
            t_ar.append(arity)
            t_sc += scope
            t_nt.append(len(tuples))
            t_tu += [v for t in tuples for v in t]
    inst = Instance(n=n, W=W, dom=dom, init=init, bin_scope=np.array(scopes, np.int32),
                    bin_rows=np.concatenate(rows) if rows else np.zeros(0, np.uint64),
                    tab_arity=np.array(t_ar, np.int32), tab_scope=np.array(t_sc, np.int32),
                    tab_ntup=np.array(t_nt, np.int32), tab_tuples=np.array(t_tu, np.int32))
    return XcspModel(inst=inst, names=names, values=values)


def read_benchmark_list(path):
    """The instance files a reference benchmark list names (<BenchMark>
    <BMFiles><BMFile>path</BMFile>..., the list the reference's driver reads;
    commented entries are not elements): each path as given, else resolved
    against the list's own directory, else its file name in that directory;
    type="dir" entries expand to the .xml files of the directory."""
    import os
    base = os.path.dirname(os.path.abspath(path))
    out = []
    for f in ET.parse(path).getroot().iter("BMFile"):
        raw = (f.text or "").strip()
        cands = [raw, os.path.join(base, raw), os.path.join(base, os.path.basename(raw))]
        hit = next((c for c in cands if os.path.exists(c)), None)
        if hit is None:
            raise FileNotFoundError(raw)
        if f.get("type") == "dir" or os.path.isdir(hit):
            out.extend(sorted(os.path.join(hit, n) for n in os.listdir(hit) if n.endswith(".xml")))
        else:
            out.append(hit)
    return out


def dump_network(inst, path):
    """A network as the text format of the reference driver's `file` mode:
    "n W", domain sizes, initial words, "nb", scope pairs, rows, then (with
    tables) "nt" and per table its arity, scope, tuple count and tuples."""
    with open(path, "w") as f:
        f.write("%d %d\n" % (inst.n, inst.W))
        f.write(" ".join(str(int(d)) for d in inst.dom) + "\n")
        f.write(" ".join(str(int(w)) for w in inst.init) + "\n")
        f.write("%d\n" % inst.n_bin)
        f.write(" ".join(str(int(v)) for v in inst.bin_scope) + "\n")
        f.write(" ".join(str(int(w)) for w in inst.bin_rows) + "\n")
        if inst.n_tab:
            f.write("%d\n" % inst.n_tab)
            so = to = 0
            for t in range(inst.n_tab):
                r, k = int(inst.tab_arity[t]), int(inst.tab_ntup[t])
                f.write("%d %s %d\n" % (r, " ".join(str(int(v)) for v in inst.tab_scope[so:so + r]), k))
                f.write(" ".join(str(int(v)) for v in inst.tab_tuples[to:to + k * r]) + "\n")
                so += r
                to += k * r
