"""Maps a golden case's generator arguments to an instance, for either the
oracle's generator (CPU tests) or the engine's (GPU tests); both compile the
same cpim_gb300/csrc/cp_gen.h."""
import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def reference_root():
    """The reference checkout if its sources are present here ($CPIM_REFERENCE,
    else the default oracle/ref/Makefile knows), or None."""
    try:
        out = subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle", "ref"), "print-ref"],
                             capture_output=True, text=True, timeout=60).stdout.strip()
    except (OSError, subprocess.SubprocessError):
        return None
    return out or None


def make_oracle_instance(args):
    from oracle import pyoracle as O
    kind = args[0]
    if kind == "binary":
        n, d, e, plo, phi, rm, seed = args[1:]
        return O.gen_binary(n, d, e, plo, phi, rm, seed)
    if kind in ("mixed", "mixedbin"):
        n, d, e, plo, phi, k3, ntup, rm, seed = args[1:]
        inst = O.gen_mixed(n, d, e, plo, phi, k3, ntup, rm, seed)
        if kind == "mixedbin":
            import numpy as np
            inst.tarity = np.zeros(0, np.int32)
            inst.tscope = np.zeros(0, np.int32)
            inst.tntup = np.zeros(0, np.int32)
            inst.ttup = np.zeros(0, np.int32)
        return inst
    if kind == "uneven":
        seed, nlo, nhi, dcap = args[1:]
        return O.gen_uneven(seed, nlo, nhi, dcap)
    raise ValueError(kind)


def make_engine_instance(args):
    import numpy as np
    import cpim_gb300 as cp
    kind = args[0]
    if kind == "binary":
        n, d, e, plo, phi, rm, seed = args[1:]
        return cp.gen_binary(n, d, e, plo, phi, rm, seed)
    if kind in ("mixed", "mixedbin"):
        n, d, e, plo, phi, k3, ntup, rm, seed = args[1:]
        inst = cp.gen_mixed(n, d, e, plo, phi, k3, ntup, rm, seed)
        if kind == "mixedbin":
            inst.tab_arity = np.zeros(0, np.int32)
            inst.tab_scope = np.zeros(0, np.int32)
            inst.tab_ntup = np.zeros(0, np.int32)
            inst.tab_tuples = np.zeros(0, np.int32)
        return inst
    if kind == "uneven":
        seed, nlo, nhi, dcap = args[1:]
        return cp.gen_uneven(seed, nlo, nhi, dcap)
    raise ValueError(kind)


def oracle_view_of(inst):
    """Oracle Instance with the same arrays as an engine Instance."""
    import numpy as np
    from oracle import pyoracle as O
    return O.Instance(n=inst.n, W=inst.W, dom=inst.dom, init=inst.init,
                      bx=np.ascontiguousarray(inst.bin_scope[0::2]), by=np.ascontiguousarray(inst.bin_scope[1::2]),
                      brows=inst.bin_rows, tarity=inst.tab_arity, tscope=inst.tab_scope, tntup=inst.tab_ntup,
                      ttup=inst.tab_tuples, fingerprint=inst.fingerprint)


def dom_hex(words):
    return "".join("%016x" % int(w) for w in words)
