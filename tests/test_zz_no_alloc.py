"""rsh_compress_noalloc: the trim + compress entry point for callers that cannot allocate device memory
(it keeps its compress scratch in a static device array). Its outputs must equal rsh_compress's and the
CPU oracle's exactly, on two calls in a row (the second smaller than the first, so stale scratch from the
first call would show), and a call must leave the device's free memory unchanged. This file is collected
last on purpose."""
import ctypes as C

import numpy as np
import pytest

import oracle
import rsh

pytestmark = pytest.mark.gpu


def _keys(n, seed):
    rng = np.random.default_rng(seed)
    k = np.repeat(rng.integers(0, 1 << 22, n).astype(np.uint32), rng.integers(1, 12, n))[:n]
    k[rng.random(len(k)) < 0.35] = rsh.KEY_NONE
    return k


def _run(fn_noalloc, ctx, keys):
    L = rsh.lib()
    n = len(keys)
    d_keys = rsh.DeviceArray.from_numpy(keys)
    outs = []
    for use_noalloc in (False, True):
        tr = rsh.DeviceArray(n, np.uint32)
        ck = rsh.DeviceArray(n + 1, np.uint32)
        cb = rsh.DeviceArray(n + 1, np.uint32)
        cs = rsh.DeviceArray(n + 1, np.uint32)
        cnt = rsh.DeviceArray(2, np.uint32)
        if use_noalloc:
            rsh.check(fn_noalloc(d_keys.ptr, n, tr.ptr, ck.ptr, cb.ptr, cs.ptr, cnt.ptr, None), "noalloc")
        else:
            rsh.check(L.rsh_compress(ctx.handle, d_keys.ptr, n, tr.ptr, ck.ptr, cb.ptr, cs.ptr, cnt.ptr, None),
                      "compress")
        R, Cn = (int(x) for x in cnt.numpy())
        outs.append((R, Cn, tr.numpy(R), ck.numpy(Cn), cb.numpy(Cn + 1), cs.numpy(Cn)))
    return outs


def _free_bytes():
    f, t = C.c_uint64(), C.c_uint64()
    rsh.check(rsh.lib().rsh_device_memory(C.byref(f), C.byref(t)), "rsh_device_memory")
    return f.value


def test_noalloc_compress_matches_compress_twice():
    L = rsh.lib()
    ctx = rsh.Context()
    for n, seed in ((3_000_001, 1), (250_000, 2)):
        keys = _keys(n, seed)
        a, b = _run(L.rsh_compress_noalloc, ctx, keys)
        assert a[0] == b[0] and a[1] == b[1] and a[0] > 0
        for x, y in zip(a[2:], b[2:]):
            assert np.array_equal(x, y)
        tr, ck, cb, cs = oracle.compress(keys)
        assert b[0] == len(tr) and b[1] == len(ck)
        for x, y in zip(b[2:], (tr, ck, cb, cs)):
            assert np.array_equal(x, y)
    # no allocation: with inputs and outputs in place, a call of another size leaves free memory unchanged
    n = 1_000_003
    d_keys = rsh.DeviceArray.from_numpy(_keys(n, 3))
    outs = [rsh.DeviceArray(n + 1, np.uint32) for _ in range(4)] + [rsh.DeviceArray(2, np.uint32)]
    rsh.check(L.rsh_device_synchronize(), "sync")
    before = _free_bytes()
    rsh.check(L.rsh_compress_noalloc(d_keys.ptr, n, *[o.ptr for o in outs], None), "noalloc")
    rsh.check(L.rsh_device_synchronize(), "sync")
    assert _free_bytes() == before
    # the size limit is enforced before anything runs
    big = rsh.DeviceArray(1, np.uint32)
    assert L.rsh_compress_noalloc(big.ptr, (1 << 24) + 1, big.ptr, big.ptr, big.ptr, None, big.ptr, None) \
        == rsh.RSH_ERR_INVALID
    ctx.destroy()
