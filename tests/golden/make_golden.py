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
"""
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


def run(case):
    name, args, op = case
    cmd = [DRIVER] + [str(a) for a in args] + [op]
    res = json.loads(subprocess.check_output(cmd, timeout=600))
    return {"name": name, "args": args, "op": op, "result": res}


def main():
    if not os.path.exists(DRIVER):
        sys.exit("build the reference driver first: make -C oracle/ref")
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
