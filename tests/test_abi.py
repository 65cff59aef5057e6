"""CPU tests of the C ABI: the library loads, exports every entry point that
include/*.h declares, and its host-side generator agrees with the oracle's."""
import ctypes
import glob
import os
import re

import numpy as np
import pytest

import cpim_gb300 as cp
from oracle import pyoracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"\b(cp_[a-z0-9_]+)\s*\(", text):
            names.add(m.group(1))
    return names


def test_library_builds_and_loads():
    from cpim_gb300 import build
    path = build.build()
    assert os.path.exists(path)
    L = cp.lib()
    assert L is not None


def test_exports_every_declared_symbol():
    names = _declared()
    assert len(names) >= 25
    L = ctypes.CDLL(cp.LIB_PATH)
    missing = [n for n in sorted(names) if not hasattr(L, n)]
    assert not missing, missing


@pytest.mark.parametrize("args", [(50, 16, 250, 0.3, 0.3, 0.0, 1), (40, 100, 160, 0.8, 0.8, 0.2, 2),
                                  (24, 256, 60, 0.9, 0.9, 0.3, 3), (30, 8, 120, 0.35, 0.35, 0.1, 4)])
def test_generator_matches_oracle_binary(args):
    a = cp.gen_binary(*args)
    b = O.gen_binary(*args)
    assert a.fingerprint == b.fingerprint
    assert np.array_equal(a.init, b.init)
    assert np.array_equal(a.bin_rows, b.brows)
    assert np.array_equal(a.bin_scope[0::2], b.bx) and np.array_equal(a.bin_scope[1::2], b.by)


def test_generator_matches_oracle_mixed_and_uneven():
    a = cp.gen_mixed(60, 8, 150, 0.2, 0.4, 20, 300, 0.1, 1)
    b = O.gen_mixed(60, 8, 150, 0.2, 0.4, 20, 300, 0.1, 1)
    assert a.fingerprint == b.fingerprint
    assert np.array_equal(a.tab_tuples, b.ttup)
    for s in range(3):
        assert cp.gen_uneven(1000003 + s, 20, 60, 256).fingerprint == O.gen_uneven(1000003 + s, 20, 60, 256).fingerprint


def test_generator_rejects_bad_arguments():
    with pytest.raises(cp.CPError):
        cp.gen_binary(5, 4, 100, 0.3)  # more constraints than pairs


def test_engine_fails_loudly_without_gpu():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(cp.CPError):
        cp.Engine(0)
