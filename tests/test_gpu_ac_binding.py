"""The reference-side binding (include/gpu_ac.hpp) compiled and linked
against the reference's own headers and objects (oracle/ref/Makefile builds
them from the reference sources, where present) and the engine library: the
GpuAC adapter is a complete `AC` of the reference (include/Solver.h:309-331).
Building needs the reference sources, which only the build container has;
running needs a GPU, so the binary is built and its linkage checked here."""
import glob
import os
import subprocess

import pytest

from tests.golden_cases import reference_root

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = reference_root()


def _build(out):
    from cpim_gb300 import build
    build.build()
    subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "oracle", "ref")])
    objs = [o for o in glob.glob(os.path.join(ROOT, "oracle", "_ref", "obj", "**", "*.o"), recursive=True)
            if not o.endswith("ref_driver.o")]
    lib_dir = os.path.join(ROOT, "cpim_gb300", "_build")
    cmd = ["g++", "-std=c++20", "-O2", "-w", "-include", "cstdint", "-include", "set", "-include", "cmath",
           "-include", "cstring", "-I" + os.path.join(ROOT, "oracle", "shim"), "-I" + os.path.join(REF, "include"),
           "-I/usr/local/cuda/include", "-I" + os.path.join(ROOT, "cpim_gb300", "csrc"),
           "-I" + os.path.join(ROOT, "include"), "-I" + os.path.join(ROOT, "oracle", "ref"),
           os.path.join(ROOT, "tests", "cpp", "gpu_ac_check.cpp")] + objs + \
          ["-L" + lib_dir, "-lcpgpu", "-Wl,-rpath," + lib_dir, "-o", out]
    subprocess.check_call(cmd)


@pytest.mark.skipif(REF is None, reason="reference sources absent")
def test_gpu_ac_builds_against_reference(tmp_path):
    out = str(tmp_path / "gpu_ac_check")
    _build(out)
    assert os.path.exists(out)
    syms = subprocess.run(["nm", "-D", "--undefined-only", out], capture_output=True, text=True).stdout
    for name in ("cp_engine_create", "cp_net_upload", "cp_dom_set", "cp_enforce_ac", "cp_dom_get"):
        assert name in syms, name
    ldd = subprocess.run(["ldd", out], capture_output=True, text=True).stdout
    assert "libcpgpu.so" in ldd
