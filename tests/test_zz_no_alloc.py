"""GPU test of the allocation-free AC entry point, cp_enforce_ac_static.

Callers that cannot allocate device memory while they run (a search or
serving loop that must not stall on cudaMalloc's device-wide synchronisation,
or a plugin inside a framework that owns the device memory) keep the network
in their own device buffers and call this entry point, whose scratch is a
static device array. This test calls it through the C ABI on buffers this
test owns (torch tensors) and checks its results against the regular entry
point, cp_enforce_ac, bit for bit, over several calls in a row on the same
static scratch, including a network at the documented limits (n = 2048
variables, 128 values, 2048 constraints); checks that a batch of calls leaves
the device's free memory unchanged (nothing allocated); and that inputs the
device-side check rejects (a constraint on one variable twice, an empty
domain size) come back as an error status without touching the domains, after
which a good call still gives the right closure. The file sorts last so that
a failure here comes after every other test has run.
"""
import ctypes as C

import numpy as np
import pytest

import cpim_gb300 as cp

pytestmark = pytest.mark.gpu


def _static_fn():
    f = cp.lib().cp_enforce_ac_static
    f.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    f.restype = C.c_int
    return f


def _device_args(inst, dom_size=None, scope=None):
    """The caller's device buffers: sizes, domains, scopes, rows, status."""
    import torch
    dev = torch.device("cuda", 0)
    ds = inst.dom if dom_size is None else dom_size
    sc = inst.bin_scope if scope is None else scope
    return [torch.from_numpy(np.asarray(ds, np.int32)).to(dev),
            torch.from_numpy(inst.init.view(np.int64).copy()).to(dev),
            torch.from_numpy(np.asarray(sc, np.int32)).to(dev),
            torch.from_numpy(inst.bin_rows.view(np.int64).copy()).to(dev),
            torch.full((4,), -7, dtype=torch.int64, device=dev)]


def _call(inst, bufs):
    import torch
    dom_size, dom, scope, rows, status = bufs
    stream = torch.cuda.current_stream(dom.device).cuda_stream
    return _static_fn()(inst.n, inst.W, dom_size.data_ptr(), dom.data_ptr(), inst.n_bin, scope.data_ptr(),
                        rows.data_ptr(), status.data_ptr(), C.c_void_p(stream))


def _run_static(inst):
    import torch
    bufs = _device_args(inst)
    rc = _call(inst, bufs)
    assert rc == 0, cp.lib().cp_last_error_string().decode()
    torch.cuda.synchronize()
    return bufs[1].cpu().numpy().view(np.uint64), bufs[4].cpu().numpy()


def _run_regular(engine, inst):
    net = engine.upload(inst)
    st = net.enforce_ac(0)
    d = net.dom_get(0)
    net.close()
    return d, st


def _instances():
    return [cp.gen_binary(50, 16, 250, 0.3, 0.3, 0.0, 1),      # consistent, d=16
            cp.gen_binary(30, 8, 120, 0.45, 0.45, 0.1, 1),     # deletions
            cp.gen_binary(40, 100, 160, 0.8, 0.8, 0.2, 2),     # W=2, ragged last word
            cp.gen_binary(30, 8, 120, 0.6, 0.6, 0.3, 4),       # wipe-out
            cp.gen_binary(2048, 128, 2048, 0.9, 0.9, 0.3, 5)]  # the documented limits, deletions


def test_static_entry_matches_enforce_ac():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    engine = cp.Engine(0)
    insts = _instances()
    # Two passes in a row over the same static scratch: results must not
    # depend on what the previous call left there.
    for _ in range(2):
        for inst in insts:
            d_ref, st_ref = _run_regular(engine, inst)
            d_st, status = _run_static(inst)
            assert status[3] == 0
            assert bool(status[0]) == bool(st_ref.inconsistent)
            if not st_ref.inconsistent:
                assert status[1] == st_ref.deletions
                assert np.array_equal(d_st, d_ref)
    engine.close()


def test_static_entry_rejects_oversized_networks():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    f = _static_fn()
    rc = f(3000, 1, None, None, 0, None, None, None, None)
    assert rc == cp.CPError(-1, "").code
    assert "limits" in cp.lib().cp_last_error_string().decode()


def test_static_entry_allocates_nothing():
    """After a first call (which looks up the static array), a batch of calls
    leaves the device's free memory exactly where it was."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    inst = cp.gen_binary(2048, 128, 2048, 0.9, 0.9, 0.3, 5)
    bufs = [_device_args(inst) for _ in range(4)]
    assert _call(inst, bufs[0]) == 0
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for b in bufs + bufs:
        assert _call(inst, b) == 0, cp.lib().cp_last_error_string().decode()
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    first = bufs[0][1].cpu().numpy()
    for b in bufs[1:]:
        assert np.array_equal(b[1].cpu().numpy(), first)


@pytest.mark.parametrize("bad", ["self_loop", "empty_domain"])
def test_static_entry_device_check_rejects_bad_input(bad):
    """The device-side check of scopes and domain sizes: status {1, 0, 0,
    CP_E_ARG}, domains untouched; the next good call on the same static
    scratch gives cp_enforce_ac's closure."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    inst = cp.gen_binary(30, 8, 120, 0.45, 0.45, 0.1, 1)
    sizes, scope = inst.dom.copy(), inst.bin_scope.copy()
    if bad == "self_loop":
        scope[2 * 7 + 1] = scope[2 * 7]
    else:
        sizes[3] = 0
    bufs = _device_args(inst, dom_size=sizes, scope=scope)
    assert _call(inst, bufs) == 0, cp.lib().cp_last_error_string().decode()
    torch.cuda.synchronize()
    status = bufs[4].cpu().numpy()
    assert status[3] == -1 and status[0] == 1, status
    assert np.array_equal(bufs[1].cpu().numpy().view(np.uint64), inst.init)
    engine = cp.Engine(0)
    d_ref, st_ref = _run_regular(engine, inst)
    engine.close()
    d_st, status = _run_static(inst)
    assert status[3] == 0 and bool(status[0]) == bool(st_ref.inconsistent)
    assert np.array_equal(d_st, d_ref)
