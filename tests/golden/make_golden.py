"""Generates tests/golden/reference_cases.json by running the reference's own
CPU propagators (Network + AC3bit / AC3 / SAC1 / MAC of leezear2022/cpim,
compiled unmodified from its sources by oracle/ref/Makefile into
oracle/_ref/ref_driver) on seeded instances from cpim_gb300/csrc/cp_gen.h.

Run from the repository root in a container that has the reference sources:
    make -C oracle/ref && python tests/golden/make_golden.py

Each case stores the generator arguments, the instance fingerprint (FNV-1a of
every instance array, so a generator change is caught) and the reference's
result: consistency verdict, deletion count and final domain words (hex, n*W
u64 words) for AC3bit / SAC1; positive and negative decision counts and the
first solution for MAC with dom/min variable order and min value order.

    python tests/golden/make_golden.py --large

writes tests/golden/large_cases.json instead: the same reference runs at the
benchmark sizes (n up to 500, d up to 256), with the final domains stored as
the SHA-256 of their hex string, plus "verdicts" cases: the reference's
singleton test of every live (x, a) of the root AC closure, all against the
same domains, listed as the failed pairs (split over processes by slices of
the reference's loop order).
"""
import hashlib
import json
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
DRIVER = os.path.join(ROOT, "oracle", "_ref", "ref_driver")


def cases():
    out = []
    # Model-B networks of the plain CPU-runnable shape: n=50, d=16, e=250, p=0.30.
    for s in range(1, 11):
        for op in ("ac3bit", "sac1", "mac"):
            out.append(("cfg1", ["binary", 50, 16, 250, 0.3, 0.3, 0.0, s], op))
    # MAC with the dom/deg variable order (VRH_DOM_DEG_MIN), same networks.
    for s in range(1, 11):
        out.append(("cfg1", ["binary", 50, 16, 250, 0.3, 0.3, 0.0, s], "mac_domdeg"))
        out.append(("tight", ["binary", 30, 8, 120, 0.35, 0.35, 0.1, s], "mac_domdeg"))
    # MAC with the dom/wdeg variable order (VRH_DOM_WDEG_MIN), same networks.
    for s in range(1, 11):
        out.append(("cfg1", ["binary", 50, 16, 250, 0.3, 0.3, 0.0, s], "mac_domwdeg"))
        out.append(("tight", ["binary", 30, 8, 120, 0.35, 0.35, 0.1, s], "mac_domwdeg"))
    # Tight small networks: AC and SAC delete values, MAC backtracks.
    for s in range(1, 11):
        for op in ("ac3bit", "sac1", "mac"):
            out.append(("tight", ["binary", 30, 8, 120, 0.35, 0.35, 0.1, s], op))
    for s in range(1, 6):
        for op in ("ac3bit", "sac1", "mac"):
            out.append(("tighter", ["binary", 30, 8, 120, 0.45, 0.45, 0.1, s], op))
    # Multi-word domains with a ragged last word (d=100: W=2) and d=256 (W=4).
    for s in range(1, 4):
        for op in ("ac3bit", "sac1", "mac"):
            out.append(("wide100", ["binary", 40, 100, 160, 0.8, 0.8, 0.2, s], op))
        for op in ("ac3bit", "sac1"):
            out.append(("wide256", ["binary", 24, 256, 60, 0.9, 0.9, 0.3, s], op))
    # Singleton verdicts over the root AC closure (every live value tested
    # against the same domains).
    for s in range(1, 4):
        out.append(("cfg1", ["binary", 50, 16, 250, 0.3, 0.3, 0.0, s], "verdicts"))
        out.append(("tight", ["binary", 30, 8, 120, 0.35, 0.35, 0.1, s], "verdicts"))
        out.append(("tighter", ["binary", 30, 8, 120, 0.45, 0.45, 0.1, s], "verdicts"))
    out.append(("wide100", ["binary", 40, 100, 160, 0.8, 0.8, 0.2, 1], "verdicts"))
    out.append(("wide256", ["binary", 24, 256, 60, 0.9, 0.9, 0.3, 1], "verdicts"))
    # Config-3 shape scaled down: n=100, d=128, e=1000, p=0.40.
    for op in ("ac3bit", "sac1"):
        out.append(("cfg3_small", ["binary", 100, 128, 1000, 0.4, 0.4, 0.0, 7], op))
    # Uneven batch members (n in [20, 60], d in {8..256}).
    for i in range(16):
        seed = 1 * 1000003 + i
        for op in ("ac3bit", "sac1"):
            out.append(("uneven", ["uneven", seed, 20, 60, 256], op))
    # Binary sub-networks of mixed-arity instances (pins the binary part of the
    # GAC oracle), and the reference's generic AC3 on the mixed instance
    # itself, recorded to document its mixed-arity defect.
    for s in range(1, 4):
        for args in ([60, 8, 150, 0.2, 0.4, 20, 300, 0.1, s], [60, 16, 200, 0.2, 0.4, 30, 2000, 0.1, s]):
            out.append(("mixedbin", ["mixedbin"] + args, "ac3bit"))
            out.append(("mixed_ref_ac3", ["mixed"] + args, "ac3"))
    return out


def large_cases():
    out = []
    # The benchmarked SAC sweep shape: n=500, d=128, e=10000, p=0.40, seed 7.
    cfg3 = ["binary", 500, 128, 10000, 0.4, 0.4, 0.0, 7]
    # Full n and d, tight enough that singleton tests fail and SAC deletes
    # values over several sweeps (and round two of a branch removes values).
    tight = ["binary", 500, 128, 2500, 0.9, 0.9, 0.0, 7]
    for name, args in (("cfg3", cfg3), ("tight500", tight)):
        out += [(name, args, "ac3bit"), (name, args, "sac1"), (name, args, "verdicts")]
    # Mid-size networks with SAC deletions or an empty SAC closure.
    for args in (["binary", 200, 64, 2000, 0.77, 0.77, 0.0, 1], ["binary", 200, 64, 2000, 0.77, 0.77, 0.0, 2],
                 ["binary", 300, 128, 1500, 0.9, 0.9, 0.0, 1]):
        out += [("mid", args, "ac3bit"), ("mid", args, "sac1"), ("mid", args, "verdicts")]
    # Uneven-batch members over the whole configured range: n in [20, 400],
    # d in {8, ..., 256}, seeds 11*1000003 + i.
    for i in range(64):
        out.append(("uneven_full", ["uneven", 11 * 1000003 + i, 20, 400, 256], "sac1"))
    return out


# The reference's Network keeps every allowed tuple of every constraint
# (about 90 bytes each once built); cases whose estimate passes this limit are
# computed by the oracle restatement instead (pinned against the reference on
# the smaller cases), and say so.
REF_BYTES_LIMIT = 16e9
MEM_BUDGET = float(os.environ.get("GOLDEN_MEM_BUDGET", 36e9))


def _estimate_bytes(args):
    sys.path.insert(0, ROOT)
    from tests.golden_cases import make_oracle_instance
    inst = make_oracle_instance(args)
    tuples = int(np.unpackbits(inst.brows.view(np.uint8)).sum())
    return 90.0 * tuples + 64e6, inst


def _oracle_case(args, op, inst):
    from oracle import pyoracle as O
    threads = os.cpu_count() or 4
    if op == "sac1":
        ok, d, dels, _ = O.sac_jacobi(inst, threads=threads)
    elif op == "ac3bit":
        ok, d, dels = O.ac3bit(inst)
    else:
        raise ValueError(op)
    res = {"fingerprint": inst.fingerprint, "n": inst.n, "W": inst.W, "consistent": bool(ok), "deletions": int(dels),
           "source": "oracle"}
    if ok:
        res["domains_sha256"] = hashlib.sha256(O.dom_hex(d).encode()).hexdigest()
    return res


class _MemGate:
    """Admits jobs while the estimated memory of running jobs stays in budget
    (a job larger than the budget runs alone)."""

    def __init__(self, budget):
        import threading
        self.budget, self.used, self.cv = budget, 0.0, threading.Condition()

    def take(self, b):
        with self.cv:
            while self.used > 0 and self.used + b > self.budget:
                self.cv.wait()
            self.used += b

    def give(self, b):
        with self.cv:
            self.used -= b
            self.cv.notify_all()


def main_large():
    import threading
    sys.path.insert(0, ROOT)
    from oracle import pyoracle as O
    out_path = os.path.join(HERE, "large_cases.json")
    part_path = out_path + ".partial"
    done = {}
    if os.path.exists(part_path):
        for line in open(part_path):
            r = json.loads(line)
            done[(r["name"], json.dumps(r["args"]), r["op"])] = r
    lock = threading.Lock()
    gate = _MemGate(MEM_BUDGET)

    def save(rec):
        with lock:
            done[(rec["name"], json.dumps(rec["args"]), rec["op"])] = rec
            with open(part_path, "a") as f:
                f.write(json.dumps(rec) + "\n")

    def ref_job(cmd, est):
        gate.take(est)
        try:
            return json.loads(subprocess.check_output([DRIVER] + cmd, timeout=14400))
        finally:
            gate.give(est)

    def case_job(case):
        name, args, op = case
        if (name, json.dumps(args), op) in done:
            return
        est, inst = _estimate_bytes(args)
        if est > REF_BYTES_LIMIT:
            save({"name": name, "args": args, "op": op, "result": _oracle_case(args, op, inst)})
            return
        base = [str(a) for a in args]
        if op != "verdicts":
            res = ref_job(base + [op], est)
            if "domains" in res:
                res["domains_sha256"] = hashlib.sha256(res.pop("domains").encode()).hexdigest()
            res["source"] = "reference"
            save({"name": name, "args": args, "op": op, "result": res})
            return
        # Verdicts: slices of the live pairs of the root AC closure, whose size
        # the oracle's AC3bit gives (it equals the reference's).
        ok, d, _ = O.ac3bit(inst)
        if not ok:
            res = ref_job(base + ["verdicts", "0", "0"], est)
            res["source"] = "reference"
            save({"name": name, "args": args, "op": op, "result": res})
            return
        live = int(np.unpackbits(d.view(np.uint8)).sum())
        k = max(1, min(16, int(MEM_BUDGET // est)))
        cuts = [live * j // k for j in range(k + 1)]
        parts = [None] * k

        def one(j):
            parts[j] = ref_job(base + ["verdicts", str(cuts[j]), str(cuts[j + 1] - cuts[j])], est)

        ths = [threading.Thread(target=one, args=(j,)) for j in range(k)]
        for t in ths:
            t.start()
        for t in ths:
            t.join()
        assert sum(p["tested"] for p in parts) == live and all(p["live"] == live for p in parts)
        res = dict(parts[0], failed=[q for p in parts for q in p["failed"]], tested=live, source="reference")
        save({"name": name, "args": args, "op": op, "result": res})

    cs = large_cases()
    # Longest first: the full-size SAC1 runs, then the rest.
    order = sorted(cs, key=lambda c: (c[2] != "sac1", c[1][0] != "binary"))
    with ThreadPoolExecutor(max_workers=max(2, os.cpu_count() or 4)) as ex:
        list(ex.map(case_job, order))
    results = [done[(n, json.dumps(a), o)] for n, a, o in cs]
    with open(out_path, "w") as f:
        json.dump({"generator": "cpim_gb300/csrc/cp_gen.h", "driver": "oracle/ref/ref_driver.cpp",
                   "domains": "sha256 of the lowercase hex string of the n*W u64 domain words",
                   "source": "reference: the reference's own code (oracle/ref); oracle: the restatement in oracle/, "
                             "for networks whose tuple lists do not fit the reference's in-memory model here",
                   "cases": results}, f, indent=0, separators=(",", ":"))
        f.write("\n")
    os.remove(part_path)
    print("wrote %d cases to %s" % (len(results), out_path))


def run(case):
    name, args, op = case
    cmd = [DRIVER] + [str(a) for a in args] + [op]
    res = json.loads(subprocess.check_output(cmd, timeout=600))
    res.pop("solve_ms", None)  # timings are not fixtures
    return {"name": name, "args": args, "op": op, "result": res}


def main():
    if not os.path.exists(DRIVER):
        sys.exit("build the reference driver first: make -C oracle/ref")
    if "--large" in sys.argv:
        return main_large()
    cs = cases()
    with ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        results = list(ex.map(run, cs))
    path = os.path.join(HERE, "reference_cases.json")
    with open(path, "w") as f:
        json.dump({"generator": "cpim_gb300/csrc/cp_gen.h", "driver": "oracle/ref/ref_driver.cpp",
                   "cases": results}, f, indent=0, separators=(",", ":"))
        f.write("\n")
    print("wrote %d cases to %s" % (len(results), path))


if __name__ == "__main__":
    main()
