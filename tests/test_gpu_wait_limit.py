"""Device-side waits end by themselves: a sort pass whose predecessor tile never publishes its look-back
status must give up after its poll limit and report RSH_ERR_TIMEOUT through the device error word, without
a hang, a fault or an out-of-bounds write, and the context must keep working afterwards."""
import numpy as np
import pytest

import rsh


def test_selftest_rejects_bad_arguments():
    lib = rsh.load()
    assert lib.rsh_selftest_wait_timeout(None, 4096, None) == rsh.RSH_ERR_INVALID


@pytest.mark.gpu
def test_lookback_wait_gives_up_and_reports():
    ctx = rsh.Context()
    lib = rsh.lib()
    assert lib.rsh_selftest_wait_timeout(ctx.handle, 0, None) == rsh.RSH_ERR_INVALID
    for _ in range(2):
        assert lib.rsh_selftest_wait_timeout(ctx.handle, 4096, None) == rsh.RSH_ERR_TIMEOUT
    ctx.check_device_errors()  # the error word was cleared
    # the context still sorts correctly (stable, by the low 20 bits)
    rng = np.random.default_rng(5)
    n = 50_000
    keys = rng.integers(0, 1 << 20, n, dtype=np.uint32)
    d_k = rsh.DeviceArray.from_numpy(keys)
    d_ko, d_vo = rsh.DeviceArray(n, np.uint32), rsh.DeviceArray(n, np.uint32)
    rsh.check(lib.rsh_sort_pairs(ctx.handle, d_k.ptr, None, d_ko.ptr, d_vo.ptr, n, None, 20, None), "sort")
    ctx.check_device_errors()
    order = np.argsort(keys, kind="stable")
    assert np.array_equal(d_vo.numpy(), order.astype(np.uint32))
    assert np.array_equal(d_ko.numpy(), keys[order])
    ctx.destroy()
