"""GB300-native bitset-domain constraint propagation (AC_3bit, GAC, SAC1).

Python view of the engine's C ABI (include/cpgpu.h). Every call goes to the
CUDA library cpim_gb300/_build/libcpgpu.so; there is no CPU fallback: if the
library is missing, importing the engine raises, and on a host without a GPU
creating an Engine raises.
"""
from __future__ import annotations

import ctypes as C
import enum
import os
from dataclasses import dataclass, field

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libcpgpu.so")

__all__ = ["ACAlgorithm", "VarHeuristic", "ValHeuristic", "Engine", "Net", "Batch", "Instance", "Stats",
           "SearchResult", "CPError", "gen_binary", "gen_mixed", "gen_uneven", "lib"]


class CPError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("cpgpu error %d: %s" % (code, msg))
        self.code = code


class ACAlgorithm(enum.IntEnum):
    """include/Solver.h:13-31 (only AC_3bit and, for tables, GAC run here)."""
    CA_AC1 = 0
    CA_AC2 = 1
    AC_3 = 2
    AC_4 = 3
    AC_6 = 4
    AC_7 = 5
    AC_2001 = 6
    AC_3bit = 7
    AC_3rm = 8


class VarHeuristic(enum.IntEnum):
    """Heuristic::Var, include/Solver.h:56-64."""
    VRH_LEX = 0
    VRH_DOM_MIN = 1
    VRH_DOM_DEG_MIN = 4
    VRH_DOM_WDEG_MIN = 6


class ValHeuristic(enum.IntEnum):
    """Heuristic::Val, include/Solver.h:66."""
    VLH_MIN = 0


class Stats(C.Structure):
    _fields_ = [("inconsistent", C.c_int32), ("rounds", C.c_int32), ("deletions", C.c_int64),
                ("revisions", C.c_int64), ("rows", C.c_int64), ("fixpoints", C.c_int64),
                ("branches", C.c_int64), ("sweeps", C.c_int32), ("launches", C.c_int32),
                ("device_ms", C.c_double), ("alg_bytes", C.c_double), ("kernel_ms", C.c_double),
                ("kernel_bytes", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class SearchResult(C.Structure):
    _fields_ = [("status", C.c_int32), ("pad", C.c_int32), ("num_positive", C.c_int64),
                ("num_negative", C.c_int64), ("propagations", C.c_int64), ("solve_ms", C.c_double)]


_lib = None


def lib():
    """Loads libcpgpu.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError("libcpgpu.so is not built (run: python -m cpim_gb300.build)")
    L = C.CDLL(LIB_PATH)
    vp, i, i64, d, u64 = C.c_void_p, C.c_int, C.c_int64, C.c_double, C.c_uint64
    PI, P64, PU8 = C.POINTER(C.c_int), C.POINTER(C.c_uint64), C.POINTER(C.c_uint8)
    PV = C.POINTER(C.c_void_p)
    sig = {
        "cp_last_error_string": ([], C.c_char_p),
        "cp_engine_create": ([i, PV], i),
        "cp_engine_destroy": ([vp], i),
        "cp_engine_launches": ([vp], i64),
        "cp_engine_set_tuning": ([vp, i, i, i], i),
        "cp_engine_set_sac_mode": ([vp, i], i),
        "cp_engine_set_graphs": ([vp, i], i),
        "cp_net_upload": ([vp, i, PI, i, P64, i, PI, P64, i, PI, PI, PI, PI, i, PV], i),
        "cp_net_destroy": ([vp], i),
        "cp_net_device_bytes": ([vp], i64),
        "cp_net_reload": ([vp, P64, P64], i),
        "cp_net_reload_async": ([vp, P64, P64], i),
        "cp_level_push": ([vp, i, PI], i),
        "cp_level_pop_to": ([vp, i], i),
        "cp_level_top": ([vp], i),
        "cp_dom_set_var": ([vp, i, i, P64], i),
        "cp_level_copy": ([vp, i, i], i),
        "cp_dom_get": ([vp, i, P64], i),
        "cp_dom_set": ([vp, i, P64], i),
        "cp_dom_sizes": ([vp, i, PI], i),
        "cp_reduce_to": ([vp, i, i, i], i),
        "cp_remove": ([vp, i, i, i], i),
        "cp_enforce_ac": ([vp, i, i, PI, C.POINTER(Stats)], i),
        "cp_enforce_sac1": ([vp, i, C.POINTER(Stats)], i),
        "cp_enforce_sac1_begin": ([vp, i], i),
        "cp_enforce_sac1_end": ([vp, C.POINTER(Stats)], i),
        "cp_enforce_sac1_end_domains": ([vp, C.POINTER(Stats), P64], i),
        "cp_singletons": ([vp, i, i, PI, PI, PU8, i, C.POINTER(Stats)], i),
        "cp_sac_sweep": ([vp, i, P64, C.POINTER(C.c_int64), C.POINTER(Stats)], i),
        "cp_sac_tiles": ([vp, i, i, PI, PI, PI, i, P64, C.POINTER(C.c_double)], i),
        "cp_mac_solve": ([vp, i, i, i64, C.POINTER(SearchResult), PI], i),
        "cp_gsolver_solve": ([vp, i64, C.POINTER(SearchResult), PI], i),
        "cp_gen_binary": ([i, i, i64, d, d, d, u64, PV], i),
        "cp_gen_mixed": ([i, i, i64, d, d, i, i, d, u64, PV], i),
        "cp_gen_uneven": ([u64, i, i, i, PV], i),
        "cp_gen_free": ([vp], i),
        "cp_gen_sizes": ([vp, C.POINTER(C.c_int64)], i),
        "cp_gen_export": ([vp, PI, P64, PI, P64, PI, PI, PI, PI], i),
        "cp_net_upload_instance": ([vp, vp, i, PV], i),
        "cp_gen_binary_device": ([vp, i, i, i64, d, d, d, u64, i, PV], i),
        "cp_gen_uneven_device": ([vp, u64, i, i, i, i, PV], i),
        "cp_net_rows_get": ([vp, P64], i),
        "cp_batch_create": ([vp, i, PV, i, PV], i),
        "cp_batch_destroy": ([vp], i),
        "cp_batch_ac": ([vp, C.POINTER(Stats), PU8], i),
        "cp_batch_sac1": ([vp, C.POINTER(Stats), PU8], i),
        "cp_batch_set_graphs": ([vp, i], i),
        "cp_batch_tune": ([vp], i),
        "cp_batch_info": ([vp, i, PI], i),
        "cp_batch_copy_level": ([vp, i], i),
        "cp_batch_create_levels": ([vp, i, PV, PI, PV], i),
        "cp_batch_load": ([vp, i, i, PI, PI, PI], i),
        "cp_batch_dom_get": ([vp, P64], i),
        "cp_server_create": ([vp, vp, i64, i, i, PV], i),
        "cp_server_destroy": ([vp], i),
        "cp_server_set_solve_limit": ([vp, i64], i),
        "cp_server_set_solvers": ([vp, i], i),
        "cp_engine_device": ([vp], i),
        "cp_engine_set_priority": ([vp, i], i),
        "cp_engine_set_search_mode": ([vp, i], i),
        "cp_engine_set_search_block": ([vp, i], i),
        "cp_engine_set_wait_budget": ([vp, i64], i),
        "cp_engine_inject_alloc_failure": ([vp, i64], i),
        "cp_mac_batch_start": ([vp, i, PV, PI, PI, PI, i, i, i64, PV], i),
        "cp_mac_batch_poll": ([vp, PU8, C.POINTER(SearchResult), PI], i),
        "cp_mac_batch_wait": ([vp, C.POINTER(SearchResult)], i),
        "cp_mac_batch_solution": ([vp, i, PI], i),
        "cp_mac_batch_destroy": ([vp], i),
        "cp_engine_set_cta_quota": ([vp, i], i),
        "cp_submit_instance": ([vp, i, vp, C.POINTER(C.c_int64)], i),
        "cp_wait": ([vp, i64, i64, vp], i),
        "cp_poll": ([vp, i64, vp], i),
        "cp_result_domains": ([vp, i64, P64], i),
        "cp_result_solution": ([vp, i64, PI], i),
        "cp_release": ([vp, i64], i),
        "cp_server_run_trace": ([vp, i, C.POINTER(C.c_double), vp, C.POINTER(C.c_double),
                                 C.POINTER(C.c_int32), C.POINTER(C.c_double)], i),
        "cp_server_register": ([vp, vp, i, C.POINTER(C.c_int64)], i),
        "cp_server_unregister": ([vp, i64], i),
        "cp_submit": ([vp, vp, C.POINTER(C.c_int64)], i),
        "cp_cancel": ([vp, i64], i),
    }
    for name, (args, res) in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res
    _lib = L
    return L


def _check(rc):
    if rc != 0:
        raise CPError(rc, lib().cp_last_error_string().decode())


def _p(a, ct):
    return a.ctypes.data_as(C.POINTER(ct)) if a is not None else None


@dataclass
class Instance:
    """A constraint network as the C ABI's upload arrays (numpy)."""
    n: int
    W: int
    dom: np.ndarray
    init: np.ndarray
    bin_scope: np.ndarray
    bin_rows: np.ndarray
    tab_arity: np.ndarray
    tab_scope: np.ndarray
    tab_ntup: np.ndarray
    tab_tuples: np.ndarray
    fingerprint: str = ""

    @property
    def n_bin(self):
        return int(self.bin_scope.shape[0] // 2)

    @property
    def n_tab(self):
        return int(self.tab_arity.shape[0])


def _export(h) -> Instance:
    L = lib()
    sz = (C.c_int64 * 8)()
    _check(L.cp_gen_sizes(h, sz))
    n, W, nb, nt, nrows, nsc, ntup, fp = list(sz)
    inst = Instance(n=n, W=W, dom=np.zeros(n, np.int32), init=np.zeros(n * W, np.uint64),
                    bin_scope=np.zeros(2 * nb, np.int32), bin_rows=np.zeros(nrows, np.uint64),
                    tab_arity=np.zeros(nt, np.int32), tab_scope=np.zeros(nsc, np.int32),
                    tab_ntup=np.zeros(nt, np.int32), tab_tuples=np.zeros(ntup, np.int32),
                    fingerprint="%016x" % (fp & 0xFFFFFFFFFFFFFFFF))
    _check(L.cp_gen_export(h, _p(inst.dom, C.c_int), _p(inst.init, C.c_uint64), _p(inst.bin_scope, C.c_int),
                           _p(inst.bin_rows, C.c_uint64), _p(inst.tab_arity, C.c_int), _p(inst.tab_scope, C.c_int),
                           _p(inst.tab_ntup, C.c_int), _p(inst.tab_tuples, C.c_int)))
    L.cp_gen_free(h)
    return inst


def gen_binary(n, d, e, p_lo, p_hi=None, remove=0.0, seed=1) -> Instance:
    """Model-B random binary network (cpim_gb300/csrc/cp_gen.h)."""
    h = C.c_void_p()
    _check(lib().cp_gen_binary(n, d, e, p_lo, p_lo if p_hi is None else p_hi, remove, seed, C.byref(h)))
    return _export(h)


def gen_mixed(n, d, e, p_lo, p_hi, k3, ntup, remove, seed) -> Instance:
    """Binary network plus ternary positive tables."""
    h = C.c_void_p()
    _check(lib().cp_gen_mixed(n, d, e, p_lo, p_hi, k3, ntup, remove, seed, C.byref(h)))
    return _export(h)


def gen_uneven(seed, n_lo=20, n_hi=400, d_cap=256) -> Instance:
    """One member of the uneven multi-instance batch."""
    h = C.c_void_p()
    _check(lib().cp_gen_uneven(seed, n_lo, n_hi, d_cap, C.byref(h)))
    return _export(h)


class Engine:
    """One CUDA device and stream (replaces GModel's implicit device state)."""

    def __init__(self, device: int = 0):
        self._h = C.c_void_p()
        _check(lib().cp_engine_create(device, C.byref(self._h)))

    def close(self):
        if self._h:
            lib().cp_engine_destroy(self._h)
            self._h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def launches(self) -> int:
        return lib().cp_engine_launches(self._h)

    def set_tuning(self, block=0, chunk=0, ctas_per_sm=0):
        _check(lib().cp_engine_set_tuning(self._h, block, chunk, ctas_per_sm))

    def set_priority(self, priority: int):
        """Stream priority: -1 low, 0 default, 1 high (before any upload)."""
        _check(lib().cp_engine_set_priority(self._h, int(priority)))

    def set_wait_budget(self, ns: int):
        """Longest grid-barrier wait of a CTA before the call returns a timeout."""
        _check(lib().cp_engine_set_wait_budget(self._h, int(ns)))

    def inject_alloc_failure(self, after: int):
        """Test hook: the device allocation after `after` more fails (-1: off)."""
        _check(lib().cp_engine_inject_alloc_failure(self._h, int(after)))

    def set_search_mode(self, mode: int):
        """0: MAC searches run whole on the device (one CTA); 1: host-driven."""
        _check(lib().cp_engine_set_search_mode(self._h, int(mode)))

    def set_search_block(self, block: int):
        """Threads per CTA of the device searches (0: automatic)."""
        _check(lib().cp_engine_set_search_block(self._h, int(block)))

    def set_cta_quota(self, quota: int):
        """Batch sweep CTAs retire after `quota` units (0: persistent)."""
        _check(lib().cp_engine_set_cta_quota(self._h, int(quota)))

    def set_sac_mode(self, mode: int):
        """0: tiled SAC sweep where eligible; 1: general per-branch kernel only."""
        _check(lib().cp_engine_set_sac_mode(self._h, mode))

    def set_graphs(self, on: bool):
        """SAC1 rounds of single networks as CUDA graph replays (default) or direct launches."""
        _check(lib().cp_engine_set_graphs(self._h, 1 if on else 0))

    def upload(self, inst: Instance, max_levels: int = 0) -> "Net":
        return Net(self, inst, max_levels)


class Net:
    """A device-resident network with its level stack."""

    def __init__(self, engine: Engine, inst: Instance, max_levels: int = 0):
        self.engine = engine
        self.n, self.W = inst.n, inst.W
        self.dom_sizes = inst.dom.copy()
        self._h = C.c_void_p()
        t = inst
        _check(lib().cp_net_upload(engine._h, t.n, _p(t.dom, C.c_int), t.W, _p(t.init, C.c_uint64), t.n_bin,
                                   _p(t.bin_scope, C.c_int), _p(t.bin_rows, C.c_uint64), t.n_tab,
                                   _p(t.tab_arity, C.c_int), _p(t.tab_scope, C.c_int), _p(t.tab_ntup, C.c_int),
                                   _p(t.tab_tuples, C.c_int), max_levels, C.byref(self._h)))

    def close(self):
        if self._h:
            lib().cp_net_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def device_bytes(self) -> int:
        return lib().cp_net_device_bytes(self._h)

    def reload(self, inst: Instance):
        _check(lib().cp_net_reload(self._h, _p(inst.init, C.c_uint64), _p(inst.bin_rows, C.c_uint64)))

    def reload_async(self, inst: Instance):
        """reload, queued on the engine's stream; inst's arrays must stay
        alive and unchanged until this network's next call."""
        _check(lib().cp_net_reload_async(self._h, _p(inst.init, C.c_uint64), _p(inst.bin_rows, C.c_uint64)))

    # -- level stack --
    def dom_get(self, level=0) -> np.ndarray:
        out = np.zeros(self.n * self.W, np.uint64)
        _check(lib().cp_dom_get(self._h, level, _p(out, C.c_uint64)))
        return out

    def level_push(self, src: int) -> int:
        """Network::NewLevel: level src + 1 := level src; returns src + 1."""
        out = C.c_int()
        _check(lib().cp_level_push(self._h, int(src), C.byref(out)))
        return out.value

    def level_pop_to(self, level: int):
        """Network::BackTo: level becomes the top."""
        _check(lib().cp_level_pop_to(self._h, int(level)))

    def level_top(self) -> int:
        return int(lib().cp_level_top(self._h))

    def dom_set_var(self, level, var, words):
        w = np.ascontiguousarray(words, dtype=np.uint64)
        if w.size < self.W:
            raise ValueError("need W words")
        _check(lib().cp_dom_set_var(self._h, int(level), int(var), _p(w, C.c_uint64)))

    def dom_set(self, level, words):
        w = np.ascontiguousarray(words, dtype=np.uint64)
        _check(lib().cp_dom_set(self._h, level, _p(w, C.c_uint64)))

    def sizes(self, level=0) -> np.ndarray:
        out = np.zeros(self.n, np.int32)
        _check(lib().cp_dom_sizes(self._h, level, _p(out, C.c_int)))
        return out

    def level_copy(self, src, dst):
        _check(lib().cp_level_copy(self._h, src, dst))

    def reduce_to(self, level, var, val):
        _check(lib().cp_reduce_to(self._h, level, var, val))

    def remove(self, level, var, val):
        _check(lib().cp_remove(self._h, level, var, val))

    # -- propagation --
    def enforce_ac(self, level=0, evt=None) -> Stats:
        st = Stats()
        if evt is None:
            _check(lib().cp_enforce_ac(self._h, level, 0, None, C.byref(st)))
        else:
            e = np.ascontiguousarray(evt, dtype=np.int32)
            _check(lib().cp_enforce_ac(self._h, level, len(e), _p(e, C.c_int), C.byref(st)))
        return st

    def enforce_sac1(self, level=0) -> Stats:
        st = Stats()
        _check(lib().cp_enforce_sac1(self._h, level, C.byref(st)))
        return st

    def enforce_sac1_begin(self, level=0):
        """First half of enforce_sac1: queues the first round and returns."""
        _check(lib().cp_enforce_sac1_begin(self._h, level))

    def enforce_sac1_end(self) -> Stats:
        """Second half: waits, runs the further sweeps, returns the stats."""
        st = Stats()
        _check(lib().cp_enforce_sac1_end(self._h, C.byref(st)))
        return st

    def enforce_sac1_end_domains(self):
        """Second half returning (stats, final domains of the level)."""
        st = Stats()
        out = np.zeros(self.n * self.W, np.uint64)
        _check(lib().cp_enforce_sac1_end_domains(self._h, C.byref(st), _p(out, C.c_uint64)))
        return st, out

    def singletons(self, vars_, vals, level=0, mode=0):
        v = np.ascontiguousarray(vars_, dtype=np.int32)
        a = np.ascontiguousarray(vals, dtype=np.int32)
        ok = np.zeros(len(v), np.uint8)
        st = Stats()
        _check(lib().cp_singletons(self._h, level, len(v), _p(v, C.c_int), _p(a, C.c_int), _p(ok, C.c_uint8), mode,
                                   C.byref(st)))
        return ok, st

    def sac_sweep(self, level=0):
        """One Jacobi sweep of singleton tests at `level` (after its AC):
        (verdict words, tests handed to the general kernel, Stats)."""
        out = np.zeros(self.n * self.W, np.uint64)
        deep = C.c_int64()
        st = Stats()
        _check(lib().cp_sac_sweep(self._h, level, _p(out, C.c_uint64), C.byref(deep), C.byref(st)))
        return out, deep.value, st

    def sac_tiles(self, xs, c1s, c2s, mode=0, level=0):
        """Support-count tiles (x, c1, c2): (removal words [ntiles, 128, 2],
        kernel ms). mode 0 bitwise, 1 tensor cores."""
        x = np.ascontiguousarray(xs, dtype=np.int32)
        a = np.ascontiguousarray(c1s, dtype=np.int32)
        b = np.ascontiguousarray(c2s, dtype=np.int32)
        out = np.zeros((len(x), 128, 2), np.uint64)
        ms = C.c_double()
        _check(lib().cp_sac_tiles(self._h, level, len(x), _p(x, C.c_int), _p(a, C.c_int), _p(b, C.c_int), mode,
                                  _p(out, C.c_uint64), C.byref(ms)))
        return out, ms.value

    # -- search --
    def mac_solve(self, var_h=VarHeuristic.VRH_DOM_MIN, val_h=ValHeuristic.VLH_MIN, time_limit_ms=600000):
        res = SearchResult()
        sol = np.full(self.n, -1, np.int32)
        _check(lib().cp_mac_solve(self._h, int(var_h), int(val_h), time_limit_ms, C.byref(res), _p(sol, C.c_int)))
        return {"status": res.status, "num_positive": res.num_positive, "num_negative": res.num_negative,
                "propagations": res.propagations, "solve_ms": res.solve_ms,
                "solution": sol.tolist() if res.status == 1 else []}

    def gsolver_solve(self, time_limit_ms=600000):
        res = SearchResult()
        sol = np.full(self.n, -1, np.int32)
        _check(lib().cp_gsolver_solve(self._h, time_limit_ms, C.byref(res), _p(sol, C.c_int)))
        return {"status": res.status, "num_positive": res.num_positive, "num_negative": res.num_negative,
                "propagations": res.propagations, "solve_ms": res.solve_ms,
                "solution": sol.tolist() if res.status == 1 else []}


def sac_tile_list(inst: Instance, xs, limit=None):
    """SAC support-count tiles (x, c1, c2) of a binary network: for every x in
    xs, every constraint c1 on x (joining y) and every other constraint c2 on
    y; at most `limit` tiles."""
    bx, by = inst.bin_scope[0::2], inst.bin_scope[1::2]
    inc = [[] for _ in range(inst.n)]
    for c, (a, b) in enumerate(zip(bx.tolist(), by.tolist())):
        inc[a].append(c)
        inc[b].append(c)
    tx, t1, t2 = [], [], []
    for x in xs:
        for c1 in inc[x]:
            y = int(by[c1]) if int(bx[c1]) == x else int(bx[c1])
            for c2 in inc[y]:
                if c2 == c1:
                    continue
                tx.append(x)
                t1.append(c1)
                t2.append(c2)
                if limit is not None and len(tx) >= limit:
                    return (np.array(tx, np.int32), np.array(t1, np.int32), np.array(t2, np.int32))
    return np.array(tx, np.int32), np.array(t1, np.int32), np.array(t2, np.int32)


class Batch:
    """Many independent networks propagated together (cp_batch_*)."""

    def __init__(self, engine: Engine, nets, level: int = 0, levels=None):
        """levels: per-member working levels (one network may then appear
        several times at distinct levels); default `level` for all."""
        self.engine = engine
        self.nets = list(nets)
        arr = (C.c_void_p * len(self.nets))(*[n._h.value for n in self.nets])
        self._h = C.c_void_p()
        if levels is None:
            _check(lib().cp_batch_create(engine._h, len(self.nets), arr, level, C.byref(self._h)))
        else:
            self._levels = np.ascontiguousarray(levels, dtype=np.int32)
            _check(lib().cp_batch_create_levels(engine._h, len(self.nets), arr, _p(self._levels, C.c_int),
                                                C.byref(self._h)))

    def close(self):
        if self._h:
            lib().cp_batch_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def ac(self):
        st = Stats()
        inc = np.zeros(len(self.nets), np.uint8)
        _check(lib().cp_batch_ac(self._h, C.byref(st), _p(inc, C.c_uint8)))
        return st, inc

    def sac1(self):
        st = Stats()
        inc = np.zeros(len(self.nets), np.uint8)
        _check(lib().cp_batch_sac1(self._h, C.byref(st), _p(inc, C.c_uint8)))
        return st, inc

    def set_graphs(self, on: bool):
        _check(lib().cp_batch_set_graphs(self._h, 1 if on else 0))

    def tune(self):
        _check(lib().cp_batch_tune(self._h))

    def copy_level(self, src: int):
        """Restores every member's batch level from level `src`."""
        _check(lib().cp_batch_copy_level(self._h, src))

    def load(self, src_level: int, edits=()):
        """Every member's working level := its level src_level, then each
        (member, var, val) edit reduces that variable to the value."""
        e = np.asarray(edits, dtype=np.int32).reshape(-1, 3)
        m, v, a = (np.ascontiguousarray(e[:, j]) for j in range(3))
        _check(lib().cp_batch_load(self._h, src_level, len(e), _p(m, C.c_int), _p(v, C.c_int), _p(a, C.c_int)))

    def dom_get(self):
        """Working domains of all members (list of per-member word arrays)."""
        sizes = [n.n * n.W for n in self.nets]
        out = np.zeros(sum(sizes), np.uint64)
        _check(lib().cp_batch_dom_get(self._h, _p(out, C.c_uint64)))
        return np.split(out, np.cumsum(sizes)[:-1])

    def info(self, group: int = 0):
        out = np.zeros(8, np.int32)
        _check(lib().cp_batch_info(self._h, group, _p(out, C.c_int)))
        keys = ["groups", "W", "tables", "members", "tiled", "cta_threads", "slot_cap", "cta_in_smem"]
        return dict(zip(keys, out.tolist()))


class _GeneratedNet(Net):
    """A Net whose relation rows were generated on the device."""

    def __init__(self, engine: Engine, h, n: int, W: int):
        self.engine = engine
        self.n, self.W = n, W
        self._h = h

    def rows(self, total_words: int) -> np.ndarray:
        out = np.zeros(total_words, np.uint64)
        _check(lib().cp_net_rows_get(self._h, _p(out, C.c_uint64)))
        return out


def upload_binary_device(engine: Engine, n, d, e, p_lo, p_hi=None, remove=0.0, seed=1, max_levels=0) -> Net:
    """gen_binary's network with its rows generated on the device."""
    h = C.c_void_p()
    _check(lib().cp_gen_binary_device(engine._h, n, d, e, p_lo, p_lo if p_hi is None else p_hi, remove, seed,
                                      max_levels, C.byref(h)))
    return _GeneratedNet(engine, h, n, (d + 63) // 64)


def upload_uneven_device(engine: Engine, seed, n_lo=20, n_hi=400, d_cap=256, max_levels=0):
    """gen_uneven's network with its rows generated on the device. Returns
    (net, n, d) where (n, d) is the drawn shape."""
    h = C.c_void_p()
    _check(lib().cp_gen_uneven_device(engine._h, seed, n_lo, n_hi, d_cap, max_levels, C.byref(h)))
    # The shape is not returned by the C ABI; recover it from the host shape
    # draw, which the device generator shares.
    inst_shape = _uneven_shape(seed, n_lo, n_hi, d_cap)
    return _GeneratedNet(engine, h, inst_shape[0], (inst_shape[1] + 63) // 64)


def _uneven_shape(seed, n_lo, n_hi, d_cap):
    # Same draws as cpgen::uneven_shape (cp_gen.h): splitmix-based stream.
    M = 0xFFFFFFFFFFFFFFFF

    def mix(z):
        z = (z + 0x9e3779b97f4a7c15) & M
        z = ((z ^ (z >> 30)) * 0xbf58476d1ce4e5b9) & M
        z = ((z ^ (z >> 27)) * 0x94d049bb133111eb) & M
        return z ^ (z >> 31)

    s = mix((seed ^ 0xA11CE) ^ 0x5eed5eed5eed)
    state = [s]

    def nxt():
        state[0] = (state[0] + 0x9e3779b97f4a7c15) & M
        return mix(state[0])

    def below(k):
        return (nxt() * k) >> 64

    n = n_lo + below(n_hi - n_lo + 1)
    ds = [8, 16, 32, 64, 128, 256]
    choices = sum(1 for v in ds if v <= d_cap)
    d = ds[below(max(1, choices))]
    return n, d


class Result(C.Structure):
    _fields_ = [("status", C.c_int32), ("inconsistent", C.c_int32), ("deletions", C.c_int64),
                ("num_positive", C.c_int64), ("num_negative", C.c_int64), ("mac_status", C.c_int32),
                ("type", C.c_int32), ("queue_ms", C.c_double), ("latency_ms", C.c_double)]


class MacBatch:
    """Many MAC searches in one launch (cp_mac_batch_*): jobs are (net,
    choices) pairs; one network may appear several times."""

    def __init__(self, engine: Engine, jobs, var_h=VarHeuristic.VRH_DOM_MIN, val_h=ValHeuristic.VLH_MIN,
                 time_limit_ms=600000):
        self.engine = engine
        self.nets = [n for n, _ in jobs]
        k = len(jobs)
        arr = (C.c_void_p * k)(*[n._h.value for n in self.nets])
        nch = np.array([len(c) for _, c in jobs], np.int32)
        flat = np.array([xv for _, c in jobs for xv in c], np.int32).reshape(-1, 2)
        cv, ca = np.ascontiguousarray(flat[:, 0]), np.ascontiguousarray(flat[:, 1])
        self._h = C.c_void_p()
        _check(lib().cp_mac_batch_start(engine._h, k, arr, _p(nch, C.c_int), _p(cv, C.c_int), _p(ca, C.c_int),
                                        int(var_h), int(val_h), int(time_limit_ms), C.byref(self._h)))

    def poll(self):
        k = len(self.nets)
        done = np.zeros(k, np.uint8)
        res = (SearchResult * k)()
        nd = C.c_int()
        _check(lib().cp_mac_batch_poll(self._h, _p(done, C.c_uint8), res, C.byref(nd)))
        return done, [self._dict(i, res[i]) if done[i] else None for i in range(k)]

    def wait(self):
        k = len(self.nets)
        res = (SearchResult * k)()
        _check(lib().cp_mac_batch_wait(self._h, res))
        return [self._dict(i, res[i]) for i in range(k)]

    def _dict(self, i, r):
        d = {"status": r.status, "num_positive": r.num_positive, "num_negative": r.num_negative,
             "propagations": r.propagations, "solve_ms": r.solve_ms, "solution": []}
        if r.status == 1:
            sol = np.zeros(self.nets[i].n, np.int32)
            _check(lib().cp_mac_batch_solution(self._h, i, _p(sol, C.c_int)))
            d["solution"] = sol.tolist()
        return d

    def close(self):
        if self._h:
            lib().cp_mac_batch_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Request(C.Structure):
    """cp_request: type (0 propagate, 1 SAC, 2 MAC solve), choices, and either
    a registered network id or an instance carried by the request."""
    _fields_ = [("type", C.c_int32), ("n_choice", C.c_int32), ("net_id", C.c_int64), ("inst", C.c_void_p),
                ("choice_var", C.POINTER(C.c_int)), ("choice_val", C.POINTER(C.c_int))]


def _requests(reqs):
    """(type, target, choices) tuples -> a cp_request array and the arrays it
    points into. target: registered network id (int) or InstanceHandle."""
    arr = (Request * len(reqs))()
    keep = []
    for r, (t, target, choices) in zip(arr, reqs):
        r.type = int(t)
        if isinstance(target, InstanceHandle):
            r.net_id, r.inst = 0, target._h.value
        else:
            r.net_id, r.inst = int(target), None
        ch = np.asarray(choices, dtype=np.int32).reshape(-1, 2)
        v, a = np.ascontiguousarray(ch[:, 0]), np.ascontiguousarray(ch[:, 1])
        keep += [v, a]
        r.n_choice = len(ch)
        r.choice_var = _p(v, C.c_int)
        r.choice_val = _p(a, C.c_int)
    return arr, keep


class InstanceHandle:
    """A generated instance kept in native memory (for server requests)."""

    def __init__(self, h, n, W):
        self._h, self.n, self.W = h, n, W

    @staticmethod
    def binary(n, d, e, p_lo, p_hi=None, remove=0.0, seed=1):
        h = C.c_void_p()
        _check(lib().cp_gen_binary(n, d, e, p_lo, p_lo if p_hi is None else p_hi, remove, seed, C.byref(h)))
        return InstanceHandle(h, n, (d + 63) // 64)

    @staticmethod
    def uneven(seed, n_lo=20, n_hi=400, d_cap=256):
        h = C.c_void_p()
        _check(lib().cp_gen_uneven(seed, n_lo, n_hi, d_cap, C.byref(h)))
        sz = (C.c_int64 * 8)()
        _check(lib().cp_gen_sizes(h, sz))
        return InstanceHandle(h, int(sz[0]), int(sz[1]))

    def export(self) -> Instance:
        L = lib()
        sz = (C.c_int64 * 8)()
        _check(L.cp_gen_sizes(self._h, sz))
        n, W, nb, nt, nrows, nsc, ntup, fp = list(sz)
        inst = Instance(n=n, W=W, dom=np.zeros(n, np.int32), init=np.zeros(n * W, np.uint64),
                        bin_scope=np.zeros(2 * nb, np.int32), bin_rows=np.zeros(nrows, np.uint64),
                        tab_arity=np.zeros(nt, np.int32), tab_scope=np.zeros(nsc, np.int32),
                        tab_ntup=np.zeros(nt, np.int32), tab_tuples=np.zeros(ntup, np.int32),
                        fingerprint="%016x" % (fp & 0xFFFFFFFFFFFFFFFF))
        _check(L.cp_gen_export(self._h, _p(inst.dom, C.c_int), _p(inst.init, C.c_uint64),
                               _p(inst.bin_scope, C.c_int), _p(inst.bin_rows, C.c_uint64),
                               _p(inst.tab_arity, C.c_int), _p(inst.tab_scope, C.c_int), _p(inst.tab_ntup, C.c_int),
                               _p(inst.tab_tuples, C.c_int)))
        return inst

    def __del__(self):
        try:
            if self._h:
                lib().cp_gen_free(self._h)
                self._h = None
        except Exception:
            pass


class Server:
    """Continuous-batching request server (cp_server_*). Request types:
    0 propagate, 1 SAC, 2 MAC solve."""

    def __init__(self, budget_bytes=150 * 10**9, max_batch=256, batching=True, device=0, solve_time_limit_ms=0,
                 solvers=1):
        self.eA, self.eB = Engine(device), Engine(device)
        self._h = C.c_void_p()
        _check(lib().cp_server_create(self.eA._h, self.eB._h, int(budget_bytes), max_batch, 1 if batching else 0,
                                      C.byref(self._h)))
        if solve_time_limit_ms:
            _check(lib().cp_server_set_solve_limit(self._h, int(solve_time_limit_ms)))
        if solvers > 1:
            _check(lib().cp_server_set_solvers(self._h, int(solvers)))

    def register(self, inst: InstanceHandle, slots: int = 8) -> int:
        """Makes a network resident with `slots` working levels; returns its id."""
        t = C.c_int64()
        _check(lib().cp_server_register(self._h, inst._h, int(slots), C.byref(t)))
        return t.value

    def unregister(self, net_id: int):
        _check(lib().cp_server_unregister(self._h, int(net_id)))

    def submit(self, rtype: int, target, choices=()) -> int:
        """target: an InstanceHandle (uploaded for the request) or a registered
        network id; choices: (var, val) pairs fixed before the request runs."""
        arr, keep = _requests([(rtype, target, choices)])
        t = C.c_int64()
        _check(lib().cp_submit(self._h, C.cast(arr, C.c_void_p), C.byref(t)))
        return t.value

    def cancel(self, ticket: int):
        _check(lib().cp_cancel(self._h, ticket))

    def wait(self, ticket: int, timeout_ms: int = 600000) -> Result:
        r = Result()
        _check(lib().cp_wait(self._h, ticket, timeout_ms, C.byref(r)))
        return r

    def poll(self, ticket: int):
        """The request's Result once done, else None (still queued or running)."""
        r = Result()
        rc = lib().cp_poll(self._h, ticket, C.byref(r))
        if rc == 1:
            return None
        _check(rc)
        return r

    def domains(self, ticket: int, n: int, W: int) -> np.ndarray:
        out = np.zeros(n * W, np.uint64)
        _check(lib().cp_result_domains(self._h, ticket, _p(out, C.c_uint64)))
        return out

    def solution(self, ticket: int, n: int):
        out = np.zeros(n, np.int32)
        _check(lib().cp_result_solution(self._h, ticket, _p(out, C.c_int)))
        return out.tolist()

    def release(self, ticket: int):
        _check(lib().cp_release(self._h, ticket))

    def run_trace(self, arrivals_s, reqs):
        """reqs: (type, target, choices) per request, submitted at arrivals_s
        seconds; returns latencies (ms), statuses, and [ticks, batched
        requests, wall seconds, peak admitted bytes, propagate-lane busy s,
        SAC-lane busy s, solver busy s, MAC solves that hit the limit]."""
        k = len(reqs)
        arr = np.ascontiguousarray(arrivals_s, dtype=np.float64)
        rq, keep = _requests(reqs)
        lat = np.zeros(k, np.float64)
        st = np.zeros(k, np.int32)
        stats = np.zeros(8, np.float64)
        _check(lib().cp_server_run_trace(self._h, k, _p(arr, C.c_double), C.cast(rq, C.c_void_p),
                                         _p(lat, C.c_double), _p(st, C.c_int32), _p(stats, C.c_double)))
        return lat, st, stats

    def close(self):
        if self._h:
            lib().cp_server_destroy(self._h)
            self._h = C.c_void_p()
        self.eA.close()
        self.eB.close()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()
