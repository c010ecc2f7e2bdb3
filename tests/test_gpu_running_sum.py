"""The device FP32 running sum behind the sample graph's mean separation (thea_selftest_running_sum), bit for bit against
the sequential float32 accumulation (numpy's add.accumulate, which adds strictly in order) on sequences that cross
binades, hit ties (terms that are odd multiples of half the sum's ulp) and hold zeros, subnormals, negative and
non-finite terms."""

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def N():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from thea_gb300 import build as B
    B.build()
    from thea_gb300 import _native
    return _native


def device_sum(N, x, s0):
    import torch
    out = ctypes.c_float(0.0)
    xd = torch.from_numpy(np.ascontiguousarray(x, np.float32)).cuda()
    N.check(N.lib().thea_selftest_running_sum(ctypes.c_void_p(xd.data_ptr()), len(x), ctypes.c_float(s0),
                                              ctypes.byref(out), None))
    host = ctypes.c_float(0.0)
    xh = np.ascontiguousarray(x, np.float32)
    N.check(N.lib().thea_selftest_running_sum(xh.ctypes.data, len(x), ctypes.c_float(s0), ctypes.byref(host), None))
    assert np.float32(out.value).tobytes() == np.float32(host.value).tobytes() or (np.isnan(out.value) and
                                                                                  np.isnan(host.value))
    return np.float32(out.value)


def sequential(x, s0):
    return np.add.accumulate(np.concatenate([[np.float32(s0)], np.asarray(x, np.float32)]), dtype=np.float32)[-1]


def same(a, b):
    if np.isnan(a) or np.isnan(b):
        return np.isnan(a) and np.isnan(b)
    return np.float32(a).tobytes() == np.float32(b).tobytes()


def test_running_sum_matches_sequential(N):
    rng = np.random.default_rng(7)
    cases = []
    for n in (1, 15, 16, 17, 8191, 8192, 8193, 300000, 2000000):
        cases.append((rng.random(n, dtype=np.float32) * np.float32(0.01), 0.0))
    x = np.exp(rng.normal(size=100000) * 6).astype(np.float32)
    x[rng.integers(0, len(x), 2000)] = 0
    x[rng.integers(0, len(x), 2000)] = np.float32(1e-42)
    cases.append((x, 0.0))
    for e in (-20, 0, 7, 30):
        s0 = np.float32(np.ldexp(1.0, e) * 1.3)
        ulp = np.float32(np.ldexp(1.0, e - 23))
        k = rng.integers(0, 4, 50000)
        t = np.where(k == 0, ulp * (np.float32(0.5) + rng.integers(0, 8, 50000)),
                     np.where(k == 1, ulp * np.float32(0.5), rng.random(50000) * ulp * 64)).astype(np.float32)
        cases.append((t, float(s0)))
    below = np.nextafter(np.float32(1024.0), np.float32(0))
    cases.append((np.full(30000, np.float32(np.ldexp(1.0, 10 - 24))), float(below)))
    y = rng.random(40000).astype(np.float32)
    y[rng.integers(0, len(y), 7)] = -0.5
    cases.append((y, 0.0))
    z = y.copy()
    z[12345] = np.inf
    cases.append((z, 0.0))
    z = y.copy()
    z[33333] = np.nan
    cases.append((z, 0.0))
    cases.append((np.full(5000, np.float32(1e37)), 3e38))
    for x, s0 in cases:
        assert same(device_sum(N, x, s0), sequential(x, s0)), (len(x), s0)


def test_empty_sum_is_the_start(N):
    assert device_sum(N, np.zeros(0, np.float32), 2.5) == np.float32(2.5)
