"""ctypes bindings to the CPU oracle (oracle/cp_oracle.cpp).

TEST INFRASTRUCTURE ONLY: the checker for the GPU engine. Only tests/,
``__graft_entry__.smoke()`` and bench.py's CPU-baseline legs may import this
module; the product package never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
GEN_DIR = os.path.join(os.path.dirname(HERE), "cpim_gb300", "csrc")


def build(force: bool = False) -> str:
    """Compiles the oracle restatement into oracle/_build/liboracle.so."""
    src = os.path.join(HERE, "cp_oracle.cpp")
    deps = [src, os.path.join(HERE, "cp_oracle.h"), os.path.join(GEN_DIR, "cp_gen.h")]
    if not force and os.path.exists(LIB_PATH):
        if os.path.getmtime(LIB_PATH) >= max(os.path.getmtime(d) for d in deps):
            return LIB_PATH
    os.makedirs(os.path.dirname(LIB_PATH), exist_ok=True)
    tmp = LIB_PATH + ".tmp"
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-fPIC", "-shared", src, "-I" + GEN_DIR,
                           "-o", tmp, "-lpthread"])
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


class OrcNet(C.Structure):
    _fields_ = [("n", C.c_int), ("W", C.c_int), ("dom", C.POINTER(C.c_int)), ("nb", C.c_int),
                ("bx", C.POINTER(C.c_int)), ("by", C.POINTER(C.c_int)),
                ("brows", C.POINTER(C.c_uint64)), ("nt", C.c_int),
                ("tarity", C.POINTER(C.c_int)), ("tscope", C.POINTER(C.c_int)),
                ("tntup", C.POINTER(C.c_int)), ("ttup", C.POINTER(C.c_int))]


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        P64, PI, PN = C.POINTER(C.c_uint64), C.POINTER(C.c_int), C.POINTER(OrcNet)
        Pi64 = C.POINTER(C.c_int64)
        L.orc_ac3bit.argtypes = [PN, P64, Pi64]
        L.orc_gac.argtypes = [PN, P64, Pi64]
        L.orc_gac_definitional.argtypes = [PN, P64]
        L.orc_sac1.argtypes = [PN, P64, Pi64]
        L.orc_mac.argtypes = [PN, P64, C.c_int64, Pi64, Pi64, PI]
        L.orc_mac_h.argtypes = [PN, P64, C.c_int64, C.c_int, Pi64, Pi64, PI]
        L.orc_dway.argtypes = [PN, P64, C.c_int64, Pi64, Pi64, PI]
        L.orc_brute_solve.argtypes = [PN, P64, C.c_double]
        L.orc_check_solution.argtypes = [PN, PI]
        L.orc_singleton.argtypes = [PN, P64, C.c_int, C.c_int]
        L.orc_time_singletons.argtypes = [PN, P64, C.c_int64, C.c_int, Pi64, Pi64]
        L.orc_time_singletons.restype = C.c_double
        L.orc_singleton_verdicts.argtypes = [PN, P64, C.c_int, P64]
        L.orc_singleton_verdicts.restype = C.c_int64
        L.orc_sac_jacobi.argtypes = [PN, P64, C.c_int, Pi64, PI]
        L.orc_time_ac.argtypes = [PN, P64, C.c_int, Pi64]
        L.orc_time_ac.restype = C.c_double
        L.orc_gen_binary.argtypes = [C.c_int, C.c_int, C.c_int64, C.c_double, C.c_double, C.c_double, C.c_uint64]
        L.orc_gen_binary.restype = C.c_void_p
        L.orc_gen_mixed.argtypes = [C.c_int, C.c_int, C.c_int64, C.c_double, C.c_double, C.c_int, C.c_int,
                                    C.c_double, C.c_uint64]
        L.orc_gen_mixed.restype = C.c_void_p
        L.orc_gen_uneven.argtypes = [C.c_uint64, C.c_int, C.c_int, C.c_int]
        L.orc_gen_uneven.restype = C.c_void_p
        L.orc_gen_free.argtypes = [C.c_void_p]
        L.orc_gen_view.argtypes = [C.c_void_p, PN, P64, Pi64, Pi64, Pi64]
        L.orc_gen_view.restype = P64
        _lib = L
    return _lib


def _ptr(a, ct):
    return a.ctypes.data_as(C.POINTER(ct))


@dataclass
class Instance:
    """A constraint network as plain numpy arrays (the C-ABI's upload format)."""
    n: int
    W: int
    dom: np.ndarray      # int32[n]
    init: np.ndarray     # uint64[n*W]
    bx: np.ndarray       # int32[nb]
    by: np.ndarray       # int32[nb]
    brows: np.ndarray    # uint64[sum dom[bx]*W]
    tarity: np.ndarray   # int32[nt]
    tscope: np.ndarray   # int32[sum arity]
    tntup: np.ndarray    # int32[nt]
    ttup: np.ndarray     # int32[sum arity*ntup]
    fingerprint: str = ""

    @property
    def nb(self):
        return int(self.bx.shape[0])

    @property
    def nt(self):
        return int(self.tarity.shape[0])

    def view(self) -> OrcNet:
        v = OrcNet()
        v.n, v.W, v.nb, v.nt = self.n, self.W, self.nb, self.nt
        v.dom = _ptr(self.dom, C.c_int)
        v.bx, v.by = _ptr(self.bx, C.c_int), _ptr(self.by, C.c_int)
        v.brows = _ptr(self.brows, C.c_uint64)
        v.tarity, v.tscope = _ptr(self.tarity, C.c_int), _ptr(self.tscope, C.c_int)
        v.tntup, v.ttup = _ptr(self.tntup, C.c_int), _ptr(self.ttup, C.c_int)
        return v


def _from_handle(h) -> Instance:
    L = lib()
    v = OrcNet()
    fp, nbw, ntt, nts = C.c_uint64(), C.c_int64(), C.c_int64(), C.c_int64()
    init_p = L.orc_gen_view(h, C.byref(v), C.byref(fp), C.byref(nbw), C.byref(ntt), C.byref(nts))
    n, W = v.n, v.W

    def arr(p, cnt, dt):
        if cnt == 0:
            return np.zeros(0, dtype=dt)
        return np.ctypeslib.as_array(p, shape=(cnt,)).astype(dt, copy=True)

    inst = Instance(n=n, W=W, dom=arr(v.dom, n, np.int32), init=arr(init_p, n * W, np.uint64),
                    bx=arr(v.bx, v.nb, np.int32), by=arr(v.by, v.nb, np.int32),
                    brows=arr(v.brows, nbw.value, np.uint64), tarity=arr(v.tarity, v.nt, np.int32),
                    tscope=arr(v.tscope, nts.value, np.int32), tntup=arr(v.tntup, v.nt, np.int32),
                    ttup=arr(v.ttup, ntt.value, np.int32), fingerprint="%016x" % fp.value)
    L.orc_gen_free(h)
    return inst


def gen_binary(n, d, e, p_lo, p_hi=None, remove=0.0, seed=1) -> Instance:
    p_hi = p_lo if p_hi is None else p_hi
    return _from_handle(lib().orc_gen_binary(n, d, e, p_lo, p_hi, remove, seed))


def gen_mixed(n, d, e, p_lo, p_hi, k3, ntup, remove, seed) -> Instance:
    return _from_handle(lib().orc_gen_mixed(n, d, e, p_lo, p_hi, k3, ntup, remove, seed))


def gen_uneven(seed, n_lo=20, n_hi=400, d_cap=256) -> Instance:
    return _from_handle(lib().orc_gen_uneven(seed, n_lo, n_hi, d_cap))


def ac3bit(inst: Instance):
    d = inst.init.copy()
    dels = C.c_int64()
    ok = lib().orc_ac3bit(C.byref(inst.view()), _ptr(d, C.c_uint64), C.byref(dels))
    return bool(ok == 1), d, dels.value


def gac(inst: Instance, dom=None):
    d = (inst.init if dom is None else dom).copy()
    dels = C.c_int64()
    ok = lib().orc_gac(C.byref(inst.view()), _ptr(d, C.c_uint64), C.byref(dels))
    return bool(ok), d, dels.value


def gac_definitional(inst: Instance):
    d = inst.init.copy()
    ok = lib().orc_gac_definitional(C.byref(inst.view()), _ptr(d, C.c_uint64))
    return bool(ok), d


def sac1(inst: Instance, dom=None):
    d = (inst.init if dom is None else dom).copy()
    dels = C.c_int64()
    ok = lib().orc_sac1(C.byref(inst.view()), _ptr(d, C.c_uint64), C.byref(dels))
    return bool(ok), d, dels.value


def mac(inst: Instance, time_limit_ms=600000, varh=1):
    """varh: 1 = VRH_DOM_MIN, 4 = VRH_DOM_DEG_MIN, 6 = VRH_DOM_WDEG_MIN."""
    npos, nneg = C.c_int64(), C.c_int64()
    sol = np.full(inst.n, -1, dtype=np.int32)
    st = lib().orc_mac_h(C.byref(inst.view()), _ptr(inst.init, C.c_uint64), time_limit_ms, varh, C.byref(npos),
                         C.byref(nneg), _ptr(sol, C.c_int))
    if st < 0:
        raise ValueError("variable heuristic must be 1 (dom/min), 4 (dom/deg) or 6 (dom/wdeg, binary networks)")
    return {"status": st, "num_positive": npos.value, "num_negative": nneg.value,
            "solution": sol.tolist() if st == 1 else []}


def dway(inst: Instance, time_limit_ms=600000):
    """GModelSolver's d-way search to the first solution."""
    npos, nneg = C.c_int64(), C.c_int64()
    sol = np.full(inst.n, -1, dtype=np.int32)
    st = lib().orc_dway(C.byref(inst.view()), _ptr(inst.init, C.c_uint64), time_limit_ms, C.byref(npos),
                        C.byref(nneg), _ptr(sol, C.c_int))
    return {"status": st, "num_positive": npos.value, "num_negative": nneg.value,
            "solution": sol.tolist() if st == 1 else []}


def brute_solve(inst: Instance, limit=1e7):
    return lib().orc_brute_solve(C.byref(inst.view()), _ptr(inst.init, C.c_uint64), limit)


def check_solution(inst: Instance, sol) -> bool:
    s = np.asarray(sol, dtype=np.int32)
    return bool(lib().orc_check_solution(C.byref(inst.view()), _ptr(s, C.c_int)))


def singleton(inst: Instance, dom, x, a) -> bool:
    return bool(lib().orc_singleton(C.byref(inst.view()), _ptr(dom, C.c_uint64), x, a))


def time_singletons(inst: Instance, dom, count, threads):
    failed, done = C.c_int64(), C.c_int64()
    s = lib().orc_time_singletons(C.byref(inst.view()), _ptr(dom, C.c_uint64), count, threads,
                                  C.byref(failed), C.byref(done))
    return s, done.value, failed.value


def singleton_verdicts(inst: Instance, dom, threads=0):
    """(verdict words, failed tests): every live (x, a) of dom tested."""
    threads = threads or (os.cpu_count() or 1)
    d = np.ascontiguousarray(dom, dtype=np.uint64)
    out = np.zeros(inst.n * inst.W, np.uint64)
    f = lib().orc_singleton_verdicts(C.byref(inst.view()), _ptr(d, C.c_uint64), threads, _ptr(out, C.c_uint64))
    return out, int(f)


def sac_jacobi(inst: Instance, dom=None, threads=0):
    """SAC closure by Jacobi sweeps on host threads: (ok, domains, deletions, sweeps)."""
    threads = threads or (os.cpu_count() or 1)
    d = (inst.init if dom is None else dom).copy()
    dels, sw = C.c_int64(), C.c_int()
    ok = lib().orc_sac_jacobi(C.byref(inst.view()), _ptr(d, C.c_uint64), threads, C.byref(dels), C.byref(sw))
    return bool(ok), d, dels.value, sw.value


def time_ac(inst: Instance, reps=3):
    dels = C.c_int64()
    s = lib().orc_time_ac(C.byref(inst.view()), _ptr(inst.init, C.c_uint64), reps, C.byref(dels))
    return s, dels.value


def dom_hex(d: np.ndarray) -> str:
    return "".join("%016x" % int(w) for w in d)
