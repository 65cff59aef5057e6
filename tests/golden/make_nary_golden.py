"""Golden fixtures for positive tables of one arity per network, from the
reference's own generic AC3 (src/AC3.cpp:99-141, 195-209), compiled from its
sources by oracle/ref/Makefile into oracle/_ref/ref_driver: each network
(tests/nary_cases.py's seeded generator) is written in the driver's `file`
format and propagated by AC3 there. On networks whose tables all have the
same arity the reference's generic revise is exact (its defect needs mixed
arities), so these pin the oracle's GAC and, through it, the device's; on the
small-domain ones the reference's SAC1 and MAC (dom/min, dom/deg) over that
AC3 pin the oracle's SAC1 and MAC.

    python tests/golden/make_nary_golden.py   # writes nary_reference_cases.json
"""
import json
import os
import subprocess
import sys
import tempfile

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from cpim_gb300.xcsp import dump_network  # noqa: E402
from tests.nary_cases import nary_arrays, to_engine  # noqa: E402

DRIVER = os.path.join(ROOT, "oracle", "_ref", "ref_driver")
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "nary_reference_cases.json")

# (name, kwargs of nary_arrays), seeds 1..5 each; one arity per network.
SHAPES = [
    ("arity2_d16", dict(n=20, d=16, n_tab=30, arities=(2,), ntup=(60, 140))),
    ("arity3_d4", dict(n=14, d=4, n_tab=8, arities=(3,), ntup=(8, 20))),
    ("arity3_d100", dict(n=12, d=100, n_tab=10, arities=(3,), ntup=(300, 800), remove=20)),
    ("arity3_d300", dict(n=10, d=300, n_tab=6, arities=(3,), ntup=(2000, 5000), remove=30)),
    ("arity5_d4", dict(n=14, d=4, n_tab=6, arities=(5,), ntup=(12, 30))),
    ("arity6_d3", dict(n=16, d=3, n_tab=6, arities=(6,), ntup=(14, 30))),
    ("arity8_d3", dict(n=20, d=3, n_tab=5, arities=(8,), ntup=(20, 40))),
    ("arity12_d2", dict(n=24, d=2, n_tab=4, arities=(12,), ntup=(10, 30), remove=2)),
]
SEEDS = (1, 2, 3, 4, 5)


def run(kw, seed, op="ac3", arg=None):
    inst = to_engine(nary_arrays(seed, **kw))
    with tempfile.NamedTemporaryFile("w", suffix=".net", delete=False) as f:
        path = f.name
    try:
        dump_network(inst, path)
        cmd = [DRIVER, "file", path, op] + ([str(arg)] if arg is not None else [])
        r = subprocess.run(cmd, capture_output=True, text=True, check=True, timeout=600)
    finally:
        os.unlink(path)
    res = json.loads(r.stdout)
    res.pop("fingerprint", None)
    res.pop("solve_ms", None)  # a timing, not a result
    return res


def main():
    if not os.path.exists(DRIVER):
        sys.exit("oracle/_ref/ref_driver is not built (make -C oracle/ref; needs the reference sources)")
    cases = []
    for name, kw in SHAPES:
        for seed in SEEDS:
            case = {"name": name, "kwargs": {k: list(v) if isinstance(v, tuple) else v for k, v in kw.items()},
                    "seed": seed, "result": run(kw, seed)}
            # SAC1 over the generic AC3 (the driver's op sac1_ac3) where its
            # tuple enumeration is affordable (domains of at most 16 values).
            if kw["d"] <= 16:
                case["sac1"] = run(kw, seed, "sac1_ac3")
                # MAC over the generic AC3 to the first solution, dom/min and
                # dom/deg (ops mac_ac3, mac_ac3_domdeg; 20 s limit).
                case["mac"] = run(kw, seed, "mac_ac3", 20000)
                case["mac_domdeg"] = run(kw, seed, "mac_ac3_domdeg", 20000)
            cases.append(case)
    with open(OUT, "w") as f:
        json.dump({"generator": "tests/nary_cases.py",
                   "driver": "oracle/ref/ref_driver.cpp (ops ac3, sac1_ac3, mac_ac3, mac_ac3_domdeg; file mode)",
                   "cases": cases}, f, indent=1)
    print("%d cases -> %s" % (len(cases), OUT))


if __name__ == "__main__":
    main()
