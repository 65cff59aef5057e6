"""Generates tests/golden/xcsp_reference_cases.json: the reference's own MAC
(dom/min variable order, min value order) and AC3bit on every XCSP instance
of its samples/bench directory, run by oracle/_ref/ref_driver on the network
this repository's reader (cpim_gb300/xcsp.py) builds, dumped in the driver's
`file` format. Stores, per instance, its path below samples/bench, the
network's fingerprint, and the reference's results (no instance content).

    make -C oracle/ref && python tests/golden/make_xcsp_golden.py
"""
import glob
import json
import os
import subprocess
import sys
import tempfile
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
DRIVER = os.path.join(ROOT, "oracle", "_ref", "ref_driver")
MAC_LIMIT_MS = 60000


def samples_dir():
    from tests.golden_cases import reference_root
    ref = reference_root()
    if not ref:
        sys.exit("reference sources absent")
    return os.path.join(ref, "samples", "bench")


def one(path, base):
    from cpim_gb300.xcsp import dump_network, read_xcsp
    m = read_xcsp(path)
    with tempfile.NamedTemporaryFile("w", suffix=".txt", delete=False) as f:
        dump = f.name
    dump_network(m.inst, dump)
    try:
        mac = json.loads(subprocess.check_output([DRIVER, "file", dump, "mac", str(MAC_LIMIT_MS)], timeout=600))
        ac = json.loads(subprocess.check_output([DRIVER, "file", dump, "ac3bit"], timeout=600))
    finally:
        os.remove(dump)
    return {"file": os.path.relpath(path, base), "n": m.inst.n, "n_bin": m.inst.n_bin, "mac": mac, "ac3bit": ac}


def main():
    base = samples_dir()
    files = sorted(glob.glob(os.path.join(base, "*.xml")) + glob.glob(os.path.join(base, "*", "*.xml")))
    from cpim_gb300.xcsp import read_xcsp
    inst_files = []
    for p in files:
        try:
            read_xcsp(p)
            inst_files.append(p)
        except ValueError:
            pass  # benchmark lists (BMPath.xml) name instances, they are none
    with ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        cases = list(ex.map(lambda p: one(p, base), inst_files))
    out = os.path.join(HERE, "xcsp_reference_cases.json")
    with open(out, "w") as f:
        json.dump({"driver": "oracle/ref/ref_driver.cpp (file mode)", "reader": "cpim_gb300/xcsp.py",
                   "mac_time_limit_ms": MAC_LIMIT_MS, "cases": cases}, f, indent=0, separators=(",", ":"))
        f.write("\n")
    print("wrote %d cases to %s" % (len(cases), out))


if __name__ == "__main__":
    main()
