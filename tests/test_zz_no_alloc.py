"""rsh_compress_noalloc: the trim + compress entry point for callers that cannot allocate device memory
(it keeps its compress scratch in a static device array). Its outputs must equal rsh_compress's exactly,
on two calls in a row (the second smaller than the first, so stale scratch from the first call would
show). This file is collected last on purpose."""
import numpy as np
import pytest

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


def test_noalloc_compress_matches_compress_twice():
    L = rsh.lib()
    ctx = rsh.Context()
    for n, seed in ((3_000_001, 1), (250_000, 2)):
        a, b = _run(L.rsh_compress_noalloc, ctx, _keys(n, seed))
        assert a[0] == b[0] and a[1] == b[1] and a[0] > 0
        for x, y in zip(a[2:], b[2:]):
            assert np.array_equal(x, y)
    # the size limit is enforced before anything runs
    big = rsh.DeviceArray(1, np.uint32)
    assert L.rsh_compress_noalloc(big.ptr, (1 << 24) + 1, big.ptr, big.ptr, big.ptr, None, big.ptr, None) \
        == rsh.RSH_ERR_INVALID
    ctx.destroy()
