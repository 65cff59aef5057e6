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
        args = ["uneven", 11 * 1000003 + i, 20, 400, 256]
        out += [("uneven_full", args, "ac3bit"), ("uneven_full", args, "sac1")]
    return out


def run(case):
    name, args, op = case
    cmd = [DRIVER] + [str(a) for a in args] + [op]
    res = json.loads(subprocess.check_output(cmd, timeout=600))
    return {"name": name, "args": args, "op": op, "result": res}


def run_large(case):
    name, args, op = case
    base = [DRIVER] + [str(a) for a in args]
    if op != "verdicts":
        res = json.loads(subprocess.check_output(base + [op], timeout=7200))
        if "domains" in res:
            res["domains_sha256"] = hashlib.sha256(res.pop("domains").encode()).hexdigest()
        return {"name": name, "args": args, "op": op, "result": res}
    head = json.loads(subprocess.check_output(base + ["verdicts", "0", "0"], timeout=600))
    if not head["consistent"]:
        return {"name": name, "args": args, "op": op, "result": head}
    live, k = head["live"], 16
    cuts = [live * j // k for j in range(k + 1)]
    with ThreadPoolExecutor(max_workers=k) as ex:
        parts = list(ex.map(lambda j: json.loads(subprocess.check_output(
            base + ["verdicts", str(cuts[j]), str(cuts[j + 1] - cuts[j])], timeout=7200)), range(k)))
    failed = [p for part in parts for p in part["failed"]]
    assert sum(part["tested"] for part in parts) == live
    res = dict(head, failed=failed, tested=live)
    return {"name": name, "args": args, "op": op, "result": res}


def main_large():
    cs = large_cases()
    # Verdict cases fan out over processes themselves; the others run
    # single-threaded side by side, the longest first.
    order = sorted(range(len(cs)), key=lambda j: (cs[j][2] != "sac1", cs[j][1][0] != "binary"))
    with ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        done = dict(zip(order, ex.map(lambda j: run_large(cs[j]), order)))
    results = [done[j] for j in range(len(cs))]
    path = os.path.join(HERE, "large_cases.json")
    with open(path, "w") as f:
        json.dump({"generator": "cpim_gb300/csrc/cp_gen.h", "driver": "oracle/ref/ref_driver.cpp",
                   "domains": "sha256 of the lowercase hex string of the n*W u64 domain words",
                   "cases": results}, f, indent=0, separators=(",", ":"))
        f.write("\n")
    print("wrote %d cases to %s" % (len(results), path))


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
