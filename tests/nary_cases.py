"""Seeded networks with positive tables of any arity (and, optionally, binary
support rows and domains wider than 256 values), as plain arrays that either
the engine's Instance or the oracle's can be made from."""
import numpy as np


def words_for(d):
    for w in (1, 2, 4, 8):
        if d <= 64 * w:
            return w
    raise ValueError("domains above 512 values")


def nary_arrays(seed, n, d, n_tab, arities, ntup, n_bin=0, p_bin=0.5, remove=3):
    """n variables of d values; n_tab tables, each of an arity drawn from
    `arities` on distinct variables with ntup (an int or a [lo, hi) range)
    distinct tuples drawn uniformly from its Cartesian product; n_bin binary
    constraints on distinct unordered pairs with each (a, b) allowed with
    probability p_bin; `remove` values cleared up front."""
    rng = np.random.default_rng(seed)
    W = words_for(d)
    ar, sc, nt, tu = [], [], [], []
    for _ in range(n_tab):
        r = int(rng.choice(arities))
        scope = rng.choice(n, size=r, replace=False)
        k = int(ntup) if np.isscalar(ntup) else int(rng.integers(*ntup))
        k = int(min(k, float(d) ** r))
        tup = np.zeros((0, r), np.int64)
        while len(tup) < k:
            more = rng.integers(0, d, size=(k - len(tup) + 8, r))
            tup = np.unique(np.concatenate([tup, more]), axis=0)
        tup = tup[np.sort(rng.choice(len(tup), size=k, replace=False))]
        ar.append(r)
        sc.extend(int(v) for v in scope)
        nt.append(k)
        tu.append(tup.reshape(-1))
    pairs = set()
    while len(pairs) < n_bin:
        x, y = (int(v) for v in rng.choice(n, size=2, replace=False))
        pairs.add((min(x, y), max(x, y)))
    bsc, rows = [], []
    for x, y in sorted(pairs):
        allowed = np.zeros((d, 64 * W), bool)
        allowed[:, :d] = rng.random((d, d)) < p_bin
        r = np.packbits(allowed, axis=1, bitorder="little").view("<u8").astype(np.uint64)
        bsc += [x, y]
        rows.append(r.reshape(-1))
    init = np.zeros(n * W, np.uint64)
    for x in range(n):
        for w in range(W):
            bits = min(64, d - 64 * w)
            init[x * W + w] = np.uint64((1 << bits) - 1) if bits > 0 else np.uint64(0)
    for _ in range(remove):
        x, a = int(rng.integers(0, n)), int(rng.integers(0, d))
        init[x * W + a // 64] &= ~(np.uint64(1) << np.uint64(a % 64))
    return dict(n=n, W=W, dom=np.full(n, d, np.int32), init=init,
                bin_scope=np.array(bsc, np.int32),
                bin_rows=np.concatenate(rows) if rows else np.zeros(0, np.uint64),
                tab_arity=np.array(ar, np.int32), tab_scope=np.array(sc, np.int32),
                tab_ntup=np.array(nt, np.int32),
                tab_tuples=np.concatenate(tu).astype(np.int32) if tu else np.zeros(0, np.int32))


def to_oracle(a):
    from oracle import pyoracle as O
    bs = a["bin_scope"]
    return O.Instance(n=a["n"], W=a["W"], dom=a["dom"], init=a["init"],
                      bx=np.ascontiguousarray(bs[0::2]), by=np.ascontiguousarray(bs[1::2]), brows=a["bin_rows"],
                      tarity=a["tab_arity"], tscope=a["tab_scope"], tntup=a["tab_ntup"], ttup=a["tab_tuples"])


def to_engine(a):
    import cpim_gb300 as cp
    return cp.Instance(**a)


# (name, kwargs) of the cases the GPU tests run and the CPU tests pin: each
# shape tight (GAC deletes values or wipes out) and loose (SAC deletes what
# GAC does not, MAC searches), over seeds 1..4.
CASES = [
    ("arity5-8_d4_tight", dict(n=14, d=4, n_tab=6, arities=(5, 6, 7, 8), ntup=(14, 60))),
    ("arity5-8_d4_loose", dict(n=14, d=4, n_tab=6, arities=(5, 6, 7, 8), ntup=(60, 200))),
    ("arity5-6_d4_bin_tight", dict(n=16, d=4, n_tab=5, arities=(5, 6), ntup=(20, 60), n_bin=10, p_bin=0.7)),
    ("arity5-6_d4_bin_loose", dict(n=16, d=4, n_tab=5, arities=(5, 6), ntup=(60, 160), n_bin=10, p_bin=0.8)),
    ("arity9-12_d3_tight", dict(n=20, d=3, n_tab=5, arities=(9, 10, 11, 12), ntup=(8, 30))),
    ("arity9-12_d3_loose", dict(n=20, d=3, n_tab=5, arities=(9, 10, 11, 12), ntup=(40, 120))),
    ("arity33-40_d2_tight", dict(n=48, d=2, n_tab=3, arities=(33, 40), ntup=(40, 80), remove=6)),
    ("arity33-40_d2_loose", dict(n=48, d=2, n_tab=3, arities=(33, 40), ntup=(100, 300), remove=1)),
    ("arity3-5_d300_tight", dict(n=10, d=300, n_tab=4, arities=(3, 5), ntup=(300, 900), n_bin=6, p_bin=0.9)),
    ("arity3-5_d300_loose", dict(n=10, d=300, n_tab=4, arities=(3, 5), ntup=(1500, 3000), n_bin=6, p_bin=0.95)),
    ("arity2-3_d512", dict(n=8, d=512, n_tab=4, arities=(2, 3), ntup=(400, 900), remove=40)),
]
SEEDS = (1, 2, 3, 4)

# More than 8192 arc + table incidences, so one propagation runs on the whole
# grid (the frontier-bitmap fixpoint), over seeds 1 and 2.
GRID_CASES = [
    ("grid_arity5-6_d8", dict(n=600, d=8, n_tab=1500, arities=(5, 6), ntup=(100, 300), n_bin=3000, p_bin=0.6)),
    ("grid_arity5-6_d8_tight", dict(n=600, d=8, n_tab=1500, arities=(5, 6), ntup=(30, 90), n_bin=3000, p_bin=0.6)),
    ("grid_arity3-4_d400", dict(n=300, d=400, n_tab=500, arities=(3, 4), ntup=(2000, 4000), n_bin=4000, p_bin=0.9)),
]
