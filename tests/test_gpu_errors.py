"""Device-side error bits reach the caller as a status, and bad inputs are refused before any kernel reads through them.

A query kernel that hits an internal limit (a traversal stack that would overflow, a tensor-core wait that gave up)
raises a bit in its handle's device error word. No input reaches those limits today (the build refuses trees too deep for
the stack), so these tests raise the bits from the host with thea_selftest_set_error_bits, a plain host-to-device copy:
nothing faults, traps or hangs on the device. Face indices outside the vertex array are refused by every entry point
that reads vertices through faces.
"""

import ctypes

import numpy as np
import pytest

from thea_gb300 import workloads as W

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


def _p(t):
    return ctypes.c_void_p(t.data_ptr())


def _closest(N, bvh, q, idx, dist):
    import torch
    return N.lib().thea_closest_element(bvh.handle, _p(q), q.shape[0], -1.0, _p(idx), _p(dist), None,
                                        ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))


def test_device_error_bits_become_a_status(N):
    import torch
    import thea_gb300 as T
    V, F = W.noisy_icosphere(3, 21)
    bvh = T.MeshBvh(torch.from_numpy(V).cuda(), torch.from_numpy(F).cuda())
    L = N.lib()
    q = torch.rand((1000, 3), device="cuda") * 2 - 1
    idx = torch.empty(1000, dtype=torch.int32, device="cuda")
    dist = torch.empty(1000, dtype=torch.float32, device="cuda")
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    assert _closest(N, bvh, q, idx, dist) == N.THEA_OK
    ref = idx.clone()
    # device arrays: the call that raised the bits returns before they are read; the next call reports them, once
    N.check(L.thea_selftest_set_error_bits(bvh.handle, 1, stream))
    assert _closest(N, bvh, q, idx, dist) == N.THEA_OK
    torch.cuda.synchronize()
    assert _closest(N, bvh, q, idx, dist) == N.THEA_ERR_INTERNAL
    assert b"stack" in L.thea_last_error_message()
    torch.cuda.synchronize()
    assert _closest(N, bvh, q, idx, dist) == N.THEA_OK
    torch.cuda.synchronize()
    assert torch.equal(idx, ref)
    assert bvh.info()["device_error_bits"] == 0
    # host arrays: the call synchronizes, so it reports the bits itself
    qh = q.cpu()
    ih = torch.empty(1000, dtype=torch.int32)
    dh = torch.empty(1000, dtype=torch.float32)
    N.check(L.thea_selftest_set_error_bits(bvh.handle, 2, stream))
    assert _closest(N, bvh, qh, ih, dh) == N.THEA_ERR_DEVICE_TIMEOUT
    assert np.array_equal(ih.numpy(), ref.cpu().numpy())  # the results are still written
    assert _closest(N, bvh, qh, ih, dh) == N.THEA_OK
    bvh.close()


def test_out_of_range_face_indices_are_refused(N):
    import torch
    import thea_gb300 as T
    V, F = W.noisy_icosphere(2, 22)
    for bad in (len(V), -1, 1 << 30):
        Fb = F.copy()
        Fb[7, 2] = bad
        for where in ("host", "device"):
            Vx, Fx = (V, Fb) if where == "host" else (torch.from_numpy(V).cuda(), torch.from_numpy(Fb).cuda())
            with pytest.raises(N.TheaError, match="face index"):
                T.MeshBvh(Vx, Fx)
            with pytest.raises(N.TheaError, match="face index"):
                T.sample_evenly_by_area(Vx, Fx, 100, 1)
    # forests check the shared vertex array too
    Fb = F.copy()
    Fb[-1, 0] = len(V)
    with pytest.raises(N.TheaError, match="face index"):
        T.MeshForest(torch.from_numpy(V).cuda(), torch.from_numpy(Fb).cuda(), np.array([0, len(F)], np.int64))
