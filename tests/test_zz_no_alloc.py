"""GPU test of the allocation-free AC entry point, cp_enforce_ac_static.

Callers that cannot allocate device memory while they run (a search or
serving loop that must not stall on cudaMalloc's device-wide synchronisation,
or a plugin inside a framework that owns the device memory) keep the network
in their own device buffers and call this entry point, whose scratch is a
static device array. This test calls it through the C ABI on buffers this
test owns (torch tensors) and checks its results against the regular entry
point, cp_enforce_ac, bit for bit, over several calls in a row on the same
static scratch. The file sorts last so that a failure here comes after every
other test has run.
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


def _run_static(inst):
    import torch
    dev = torch.device("cuda", 0)
    dom_size = torch.from_numpy(inst.dom.astype(np.int32)).to(dev)
    dom = torch.from_numpy(inst.init.view(np.int64).copy()).to(dev)
    scope = torch.from_numpy(inst.bin_scope.astype(np.int32)).to(dev)
    rows = torch.from_numpy(inst.bin_rows.view(np.int64).copy()).to(dev)
    status = torch.full((4,), -7, dtype=torch.int64, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    rc = _static_fn()(inst.n, inst.W, dom_size.data_ptr(), dom.data_ptr(), inst.n_bin, scope.data_ptr(),
                      rows.data_ptr(), status.data_ptr(), C.c_void_p(stream))
    assert rc == 0, cp.lib().cp_last_error_string().decode()
    torch.cuda.synchronize(dev)
    return dom.cpu().numpy().view(np.uint64), status.cpu().numpy()


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
            cp.gen_binary(30, 8, 120, 0.6, 0.6, 0.3, 4)]       # wipe-out


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
