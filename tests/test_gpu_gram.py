"""GPU tests of the tensor-core k-NN candidate path: the raw Gram tile against a PyTorch FP32 product of the same
FP16-rounded operands, and the k-NN graph with Gram-seeded search against the plain traversal (identical results)."""

import numpy as np
import pytest

from thea_gb300 import workloads as W

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def T():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from thea_gb300 import build as B
    B.build()
    import thea_gb300
    return thea_gb300


def gram_reference(a, b):
    """The tile's operands built on the host exactly as the kernel stages them, multiplied in FP32."""
    import torch
    c = a[0]
    ext = torch.max(torch.cat([(a - c).abs().reshape(-1), (b - c).abs().reshape(-1)]))
    inv = 1.0 / ext
    ar = (a - c) * inv
    br = (b - c) * inv
    A = torch.zeros((128, 16), dtype=torch.float16, device=a.device)
    B = torch.zeros((512, 16), dtype=torch.float16, device=a.device)
    A[:a.shape[0], :3] = ar.half()
    A[:a.shape[0], 3] = 1.0
    B[:b.shape[0], :3] = (-2.0 * br).half()
    x, y, z = br[:, 0], br[:, 1], br[:, 2]
    B[:b.shape[0], 3] = ((x * x + y * y) + z * z).half()
    B[b.shape[0]:, 3] = 65504.0
    return A.float() @ B.float().T


@pytest.mark.parametrize("na,nb,spread", [(128, 512, 1.0), (128, 512, 1e-3), (77, 300, 5.0), (1, 1, 1.0)])
def test_gram_tile_matches_fp32_product(T, na, nb, spread):
    import torch
    g = torch.Generator(device="cuda").manual_seed(na * 1000 + nb)
    a = 3.0 + spread * torch.randn((na, 3), generator=g, device="cuda")
    b = 3.0 + spread * torch.randn((nb, 3), generator=g, device="cuda")
    keys = T.point_gram_tile(a, b)
    ref = gram_reference(a, b)
    got = keys[:na, :nb]
    want = ref[:na, :nb]
    # the same FP16 operands, FP32 accumulation of four products: equal up to the accumulation order
    assert torch.allclose(got, want, rtol=1e-6, atol=1e-6 * float(want.abs().max()))


@pytest.mark.parametrize("k", [1, 8, 16, 32])
def test_gram_seeded_knn_graph_equals_traversal(T, oracle, k):
    import torch
    V, F, _ = W.config0()
    pos, _, _ = T.sample_evenly_by_area(torch.from_numpy(V).cuda(), torch.from_numpy(F).cuda(), 40000, 11)
    pb = T.PointBvh(pos)
    i0, d0 = pb.k_closest_self(k, device=True)
    i1, d1 = pb.k_closest_self(k, device=True, candidates="gram")
    assert torch.equal(i0, i1) and torch.equal(d0, d1)
    assert pb.info()["device_error_bits"] == 0
    if k == 8:
        # and the oracle agrees on a sample of rows
        P = pos.cpu().numpy()
        rows = np.arange(0, len(P), 997)
        bi, bd = oracle.knn_brute(P, P[rows], k + 1)
        got = i1.cpu().numpy()[rows]
        for r, row in enumerate(rows):
            ref = [j for j in bi[r] if j != row][:k]
            assert list(got[r]) == ref


def test_gram_mode_on_small_sets_falls_back(T):
    import torch
    P = torch.rand((300, 3), device="cuda")
    pb = T.PointBvh(P)
    i0, d0 = pb.k_closest_self(5, device=True)
    i1, d1 = pb.k_closest_self(5, device=True, candidates="gram")
    assert torch.equal(i0, i1) and torch.equal(d0, d1)


def test_bounded_device_wait_gives_up_and_context_survives(T):
    # failure path of the bounded mbarrier waits: a phase nothing completes; the wait reports instead of hanging
    import torch
    from thea_gb300 import _native as N
    r = N.lib().thea_selftest_bounded_wait(2000, None)
    assert r == N.THEA_ERR_DEVICE_TIMEOUT
    # the context is still usable
    P = torch.rand((1000, 3), device="cuda")
    pb = T.PointBvh(P)
    i0, d0 = pb.k_closest_self(4, device=True)
    i1, d1 = pb.k_closest_self(4, device=True, candidates="gram")
    assert torch.equal(i0, i1) and torch.equal(d0, d1)
    # invalid limits are refused on the host
    assert N.lib().thea_selftest_bounded_wait(0, None) == N.THEA_ERR_INVALID_ARGUMENT
