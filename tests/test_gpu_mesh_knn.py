"""GPU parity of the k nearest triangles of a mesh BVH (kClosestPairs on a MeshBvh) against brute force over every
(query, triangle) pair with the oracle's triangle closest point: exact FP32 squared distances, lowest index first among
ties, NaN distances (coincident vertices) never kept."""

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


def _brute(oracle, V, F, Q, k, bound=-1.0):
    tris = V[F].reshape(-1, 9)
    nq, nt = len(Q), len(F)
    _, d2 = oracle.triangle_closest_points(np.repeat(tris[None], nq, 0).reshape(-1, 9), np.repeat(Q, nt, 0))
    d2 = d2.reshape(nq, nt)
    idx = np.full((nq, k), -1, np.int32)
    out = np.full((nq, k), -1, np.float32)
    for i in range(nq):
        keep = ~np.isnan(d2[i])
        if bound >= 0:
            keep &= d2[i].astype(np.float64) < float(bound) ** 2
        cand = np.nonzero(keep)[0]
        o = cand[np.lexsort((cand, d2[i, cand]))][:k]
        idx[i, :len(o)] = o
        out[i, :len(o)] = d2[i, o]
    return idx, out


@pytest.mark.parametrize("width", [4, 8])
def test_k_nearest_triangles(T, oracle, width):
    import torch
    V, F = W.noisy_icosphere(3, 61, sigma=0.04)
    Q = W.uniform_box_points(600, [-1.4] * 3, [1.4] * 3, 62)
    Q[:50] = V[F[:50, 0]]  # queries on vertices: several triangles at distance 0
    bvh = T.MeshBvh(torch.from_numpy(V).cuda(), torch.from_numpy(F).cuda(), width=width)
    for k in (1, 4, 7, 16, 32):
        gi, gd = bvh.k_closest_pairs(torch.from_numpy(Q).cuda(), k)
        bi, bd = _brute(oracle, V, F, Q, k)
        np.testing.assert_array_equal(gi.cpu().numpy(), bi)
        np.testing.assert_array_equal(gd.cpu().numpy(), bd)
    gi, gd = bvh.k_closest_pairs(Q, 8, dist_bound=0.1)
    bi, bd = _brute(oracle, V, F, Q, 8, 0.1)
    np.testing.assert_array_equal(gi, bi)
    np.testing.assert_array_equal(gd, bd)
    bvh.close()
