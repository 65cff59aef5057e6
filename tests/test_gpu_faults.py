"""Failure handling without faulting the GPU: a grid-barrier wait that runs out
(budget 0) returns CP_E_TIMEOUT and leaves the engine usable; an injected
device allocation failure returns CP_E_OOM cleanly; corrupted network arrays
are rejected by host validation before any launch."""
import numpy as np
import pytest

import cpim_gb300 as cp
from oracle import pyoracle as O
from tests.golden_cases import oracle_view_of

pytestmark = pytest.mark.gpu


def test_grid_wait_runs_out_then_recovers():
    # Over 8192 arc incidences: the fixpoint runs on the whole grid with a
    # bounded barrier. A fixpoint seeded with changed variables always passes
    # the barrier after the seeding; a zero budget makes the wait of some CTA
    # there run out.
    inst = cp.gen_binary(2000, 64, 30000, 0.2, 0.5, 0.2, 3)
    ok, d, dels = O.ac3bit(oracle_view_of(inst))
    every = np.arange(inst.n, dtype=np.int32)
    with cp.Engine(0) as eng:
        net = eng.upload(inst)
        eng.set_wait_budget(0)
        codes = []
        for _ in range(3):
            net.dom_set(0, inst.init)
            try:
                net.enforce_ac(0, evt=every)
                codes.append(0)
            except cp.CPError as ex:
                codes.append(ex.code)
            if -4 in codes:
                break
        assert -4 in codes, codes  # CP_E_TIMEOUT
        eng.set_wait_budget(2 * 10**9)
        net.dom_set(0, inst.init)
        st = net.enforce_ac(0)
        assert bool(st.inconsistent) == (not ok)
        if ok:
            assert np.array_equal(net.dom_get(0), d)
            assert st.deletions == dels
        net.close()


def test_injected_allocation_failure_is_clean():
    inst = cp.gen_binary(60, 16, 300, 0.3, 0.3, 0.0, 2)
    ok, d, _ = O.ac3bit(oracle_view_of(inst))
    with cp.Engine(0) as eng:
        for after in (0, 1, 3):
            eng.inject_alloc_failure(after)
            with pytest.raises(cp.CPError) as ex:
                eng.upload(inst)
            assert ex.value.code == -2  # CP_E_OOM
        net = eng.upload(inst)  # the hook turned itself off
        st = net.enforce_ac(0)
        assert bool(st.inconsistent) == (not ok)
        if ok:
            assert np.array_equal(net.dom_get(0), d)
        net.close()


def _copy(inst, **kw):
    f = dict(n=inst.n, W=inst.W, dom=inst.dom.copy(), init=inst.init.copy(), bin_scope=inst.bin_scope.copy(),
             bin_rows=inst.bin_rows.copy(), tab_arity=inst.tab_arity.copy(), tab_scope=inst.tab_scope.copy(),
             tab_ntup=inst.tab_ntup.copy(), tab_tuples=inst.tab_tuples.copy())
    f.update(kw)
    return cp.Instance(**f)


def test_corrupted_arrays_rejected_by_host_validation():
    inst = cp.gen_mixed(30, 8, 60, 0.3, 0.5, 10, 40, 0.0, 1)
    bad_scope = inst.bin_scope.copy()
    bad_scope[5] = inst.n + 7            # a variable index past n
    self_loop = inst.bin_scope.copy()
    self_loop[1] = self_loop[0]          # x == y
    bad_tuple = inst.tab_tuples.copy()
    bad_tuple[3] = 99                    # a value past the domain
    bad_dom = inst.dom.copy()
    bad_dom[0] = 0                       # an empty domain size
    with cp.Engine(0) as eng:
        for broken in (_copy(inst, bin_scope=bad_scope), _copy(inst, bin_scope=self_loop),
                       _copy(inst, tab_tuples=bad_tuple), _copy(inst, dom=bad_dom)):
            with pytest.raises(cp.CPError) as ex:
                eng.upload(broken)
            assert ex.value.code == -1  # CP_E_ARG
        net = eng.upload(inst)          # the engine is still usable
        net.enforce_ac(0)
        net.close()
