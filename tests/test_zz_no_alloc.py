"""The allocation-free filter entry point against the context filter and the
oracle.

tg_filter_noalloc exists for callers that cannot allocate device memory
(a host whose own memory pool owns the whole device, or one that must not
let a cudaMalloc synchronise the device): it filters caller-owned current
arrays using a fixed scratch array compiled into the library. This test
calls it through the C-ABI twice in a row on one context's device arrays
and checks each result against tg_filter on an identical second context,
bit for bit (the filter is exact in both paths), in 2D and 3D, for an odd
pass count (the result ends in the scratch array and is copied back) and an
even one (it ends in the caller's arrays); the first call is also checked
against the oracle's filter. A grid larger than the fixed scratch is
rejected with TG_ERR_ARG. It runs last in collection order and needs no
state from other tests.
"""
import ctypes

import numpy as np
import pytest

from tristan_gb300.config import SimConfig

pytestmark = pytest.mark.gpu


def _bind(lib):
    f = lib.tg_filter_noalloc
    f.argtypes = [ctypes.c_int32] * 6 + [ctypes.POINTER(ctypes.c_int32), ctypes.c_int32] + \
                 [ctypes.c_void_p] * 4
    f.restype = ctypes.c_int
    return f


@pytest.mark.parametrize("dims,order,ntimes", [(2, 3, 3), (2, 3, 4), (2, 1, 4), (3, 2, 3), (3, 2, 4)])
def test_filter_noalloc_matches_context_filter(dims, order, ntimes):
    import oracle
    from tristan_gb300.gpu import GpuSim, SYNC_CUR, TG_OK
    if dims == 2:
        cfg = SimConfig(dims=2, order=order, nx=96, ny=64, ntimes=ntimes, maxhlf=16)
    else:
        cfg = SimConfig(dims=3, order=order, nx=20, ny=16, nz=18, ntimes=ntimes, maxhlf=16)
    rng = np.random.default_rng(42)
    cur = {k: rng.standard_normal(cfg.ncells).astype(np.float32) for k in ("curx", "cury", "curz")}
    orc = oracle.OracleSim(cfg)
    for k, v in cur.items():
        orc.fields[k][:] = v
    orc.call("to_apply_filter1_opt")
    ref = GpuSim(cfg)
    dut = GpuSim(cfg)
    try:
        for s in (ref, dut):
            s.set_fields(**cur)
            s.sync_from_host(SYNC_CUR)
        fn = _bind(dut.lib)
        ptrs = (ctypes.c_void_p * 9)()
        assert dut.lib.tg_device_fields(dut.h, ptrs) == TG_OK
        stream = dut.lib.tg_stream(dut.h)
        periodic = (ctypes.c_int32 * 3)(1, 1, 1)
        for call in range(2):  # two calls in a row share the scratch array
            ref.apply_filter1_opt()
            rc = fn(cfg.dims, cfg.mx, cfg.my, cfg.mz, cfg.nghost, cfg.nghostz, periodic, cfg.ntimes,
                    ptrs[6], ptrs[7], ptrs[8], stream)
            assert rc == TG_OK, dut.lib.tg_last_error(None)
            ref.sync_to_host(SYNC_CUR)
            dut.sync_to_host(SYNC_CUR)
            for k in ("curx", "cury", "curz"):
                np.testing.assert_array_equal(dut.fields[k], ref.fields[k], err_msg=k)
                if call == 0:
                    np.testing.assert_array_equal(dut.fields[k], orc.fields[k], err_msg=k + " (oracle)")
    finally:
        ref.close()
        dut.close()


def test_filter_noalloc_rejects_oversized_grid():
    from tristan_gb300.gpu import TG_ERR_ARG, load_library
    lib = load_library()
    fn = _bind(lib)
    periodic = (ctypes.c_int32 * 3)(1, 1, 1)
    dummy = ctypes.c_void_p(16)  # never dereferenced: the size check comes first
    rc = fn(2, 2005, 2005, 1, 5, 5, periodic, 4, dummy, dummy, dummy, None)
    assert rc == TG_ERR_ARG
    assert b"exceeds the fixed scratch" in lib.tg_last_error(None)
