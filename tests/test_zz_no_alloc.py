"""The allocation-free sampling entry point (thea_sample_by_area_noalloc), called through the C ABI.

Some callers cannot allocate device memory themselves or let a library do it: an application that manages a fixed
device budget through its own pool, a plugin inside such a host, or a latency-critical loop that cannot take cudaMalloc's
implicit synchronization. This entry point keeps its scratch in a fixed array inside the library, and these tests check
that it returns exactly what the ordinary entry point returns, on two calls in a row (the second call must not see
leftovers of the first), that it allocates nothing (the library's allocation counter and the device's free memory),
that it refuses out-of-range face indices without reading through them, and that it refuses what it cannot do without
allocating.

The file name makes pytest collect it last, so a run that stops at the first failure has already run every other test.
"""

import ctypes

import numpy as np
import pytest

from thea_gb300 import workloads as W

pytestmark = pytest.mark.gpu

TOL = 0.0  # the two entry points run the same FP32/FP64 arithmetic: results must be identical


@pytest.fixture(scope="module")
def lib():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from thea_gb300 import build as B
    B.build()
    from thea_gb300 import _native as N
    return N


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def _sample(N, fn, V, F, n, seed, rng):
    import torch
    pos = torch.empty((n, 3), dtype=torch.float32, device="cuda")
    nrm = torch.empty((n, 3), dtype=torch.float32, device="cuda")
    face = torch.empty((n,), dtype=torch.int32, device="cuda")
    got = ctypes.c_int64(-1)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    N.check(fn(_ptr(V), V.shape[0], _ptr(F), F.shape[0], n, ctypes.c_uint32(seed), rng, _ptr(pos), _ptr(nrm),
               _ptr(face), ctypes.byref(got), stream))
    torch.cuda.synchronize()
    return got.value, pos.cpu().numpy(), nrm.cpu().numpy(), face.cpu().numpy()


def _check_same(a, b):
    assert a[0] == b[0]
    for x, y in zip(a[1:], b[1:]):
        if x.dtype.kind == "f":
            np.testing.assert_allclose(x, y, rtol=TOL, atol=0)
        else:
            assert np.array_equal(x, y)


def test_noalloc_matches_sample_by_area_twice_in_a_row(lib):
    import torch
    N = lib
    L = N.lib()
    # first call: the 81,920-triangle config-0 mesh, 200,000 samples (four chunks of the internal word buffer)
    V0, F0, _ = W.config0()
    V0, F0 = torch.from_numpy(V0).cuda(), torch.from_numpy(F0).cuda()
    ref0 = _sample(N, L.thea_sample_by_area, V0, F0, 200000, 11, N.RNG_THEA_MT)
    new0 = _sample(N, L.thea_sample_by_area_noalloc, V0, F0, 200000, 11, N.RNG_THEA_MT)
    assert new0[0] == 200000
    _check_same(ref0, new0)
    # second call, right after: a smaller mesh and another seed, so stale table entries or generator state would show
    V1, F1 = W.noisy_icosphere(3, 12)
    V1, F1 = torch.from_numpy(V1).cuda(), torch.from_numpy(F1).cuda()
    ref1 = _sample(N, L.thea_sample_by_area, V1, F1, 70001, 12, N.RNG_THEA_MT)
    new1 = _sample(N, L.thea_sample_by_area_noalloc, V1, F1, 70001, 12, N.RNG_THEA_MT)
    _check_same(ref1, new1)
    # the counter-based stream as well
    refc = _sample(N, L.thea_sample_by_area, V1, F1, 5000, 13, N.RNG_COUNTER)
    newc = _sample(N, L.thea_sample_by_area_noalloc, V1, F1, 5000, 13, N.RNG_COUNTER)
    _check_same(refc, newc)


def test_noalloc_allocates_nothing(lib):
    """The library's allocation counter (driver and pool allocations) and the device's free memory stay unchanged across
    the call, in a fresh process or after other tests; the ordinary entry point, as a control, does allocate."""
    import torch
    N = lib
    L = N.lib()
    V, F, _ = W.config0()
    V, F = torch.from_numpy(V).cuda(), torch.from_numpy(F).cuda()
    n = 150000
    pos = torch.empty((n, 3), dtype=torch.float32, device="cuda")
    face = torch.empty((n,), dtype=torch.int32, device="cuda")
    got = ctypes.c_int64(-1)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    args = (_ptr(V), V.shape[0], _ptr(F), F.shape[0], n, ctypes.c_uint32(5), N.RNG_THEA_MT, _ptr(pos), None,
            _ptr(face), ctypes.byref(got), stream)
    N.check(L.thea_sample_by_area_noalloc(*args))  # first call on the device: looks up the fixed array's address
    torch.cuda.synchronize()
    for _ in range(2):
        count0 = L.thea_allocation_count()
        free0, _ = torch.cuda.mem_get_info()
        N.check(L.thea_sample_by_area_noalloc(*args))
        torch.cuda.synchronize()
        free1, _ = torch.cuda.mem_get_info()
        assert L.thea_allocation_count() == count0
        assert free1 == free0
        assert got.value == n
    count0 = L.thea_allocation_count()
    N.check(L.thea_sample_by_area(*args))
    torch.cuda.synchronize()
    assert L.thea_allocation_count() > count0


def test_noalloc_rejects_out_of_range_face_indices(lib):
    """A face index outside [0, num_vertices) is found on the device without being dereferenced and refused; the next
    call with a valid mesh is unaffected."""
    import torch
    N = lib
    L = N.lib()
    V, F = W.noisy_icosphere(2, 15)
    Vd = torch.from_numpy(V).cuda()
    out = torch.empty((100, 3), dtype=torch.float32, device="cuda")
    got = ctypes.c_int64(-1)
    for bad in (len(V), -1, 1 << 30):
        Fb = F.copy()
        Fb[len(F) // 2, 1] = bad
        Fd = torch.from_numpy(Fb).cuda()
        st = L.thea_sample_by_area_noalloc(_ptr(Vd), len(V), _ptr(Fd), len(F), 100, 1, N.RNG_THEA_MT, _ptr(out), None,
                                           None, ctypes.byref(got), None)
        assert st == N.THEA_ERR_INVALID_ARGUMENT and b"face index" in L.thea_last_error_message()
        assert got.value == 0
    Fd = torch.from_numpy(F).cuda()
    N.check(L.thea_sample_by_area_noalloc(_ptr(Vd), len(V), _ptr(Fd), len(F), 100, 1, N.RNG_THEA_MT, _ptr(out), None,
                                          None, ctypes.byref(got), None))
    assert got.value == 100


def test_noalloc_refuses_what_needs_an_allocation(lib):
    import torch
    N = lib
    L = N.lib()
    V, F = W.noisy_icosphere(1, 14)
    Vd, Fd = torch.from_numpy(V).cuda(), torch.from_numpy(F).cuda()
    out = torch.empty((10, 3), dtype=torch.float32, device="cuda")
    got = ctypes.c_int64(-1)
    # host arrays would need staging buffers
    st = L.thea_sample_by_area_noalloc(ctypes.c_void_p(V.ctypes.data), len(V), ctypes.c_void_p(F.ctypes.data), len(F),
                                       10, 1, N.RNG_THEA_MT, _ptr(out), None, None, ctypes.byref(got), None)
    assert st == 1 and b"device memory" in L.thea_last_error_message()
    # more triangles than the fixed table holds
    st = L.thea_sample_by_area_noalloc(_ptr(Vd), len(V), _ptr(Fd), N.NOALLOC_MAX_FACES + 1, 10, 1, N.RNG_THEA_MT,
                                       _ptr(out), None, None, ctypes.byref(got), None)
    assert st == 1 and b"THEA_NOALLOC_MAX_FACES" in L.thea_last_error_message()
    # a zero-area mesh writes nothing, as the ordinary entry point does
    Z = torch.zeros((3, 3), dtype=torch.float32, device="cuda")
    Zf = torch.tensor([[0, 1, 2]], dtype=torch.int32, device="cuda")
    st = L.thea_sample_by_area_noalloc(_ptr(Z), 3, _ptr(Zf), 1, 10, 1, N.RNG_THEA_MT, _ptr(out), None, None,
                                       ctypes.byref(got), None)
    assert st == 0 and got.value == 0
