"""GPU parity on the reference's sample meshes (Data/Models/{cube,sphere,teapot}.obj, read by the library's OBJ reader
into tests/golden/models.npz by tests/golden/make_model_fixtures.py): closest points, first hits, k nearest vertices and
ShapeDiameter against the oracle on real geometry, degenerate triangles included."""

import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MODELS = ("cube", "sphere", "teapot")


@pytest.fixture(scope="module")
def T():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from thea_gb300 import build as B
    B.build()
    import thea_gb300
    return thea_gb300


@pytest.fixture(scope="module")
def models(golden_dir):
    z = np.load(os.path.join(golden_dir, "models.npz"))
    return {m: (z[m + "_vertices"], z[m + "_triangles"]) for m in MODELS}


@pytest.mark.parametrize("name", MODELS)
def test_queries_on_sample_models(T, oracle, models, name):
    import torch
    V, F = models[name]
    rng = np.random.default_rng(50 + MODELS.index(name))
    lo, hi = V.min(0), V.max(0)
    c, e = (lo + hi) / 2, (hi - lo) * 0.75
    Q = (c + (rng.random((20000, 3)) * 2 - 1) * e).astype(np.float32)
    bvh = T.MeshBvh(torch.from_numpy(V).cuda(), torch.from_numpy(F).cuda())
    idx, dist, cp = bvh.closest_element(torch.from_numpy(Q).cuda())
    ri, rd2, rcp = oracle.closest_brute(V, F, Q)
    assert np.array_equal(idx.cpu().numpy(), ri)
    assert np.array_equal(dist.cpu().numpy(), np.sqrt(rd2.astype(np.float32)))
    assert np.array_equal(cp.cpu().numpy(), rcp.astype(np.float32))
    d = rng.normal(size=(20000, 3)).astype(np.float32)
    t, ti, _ = bvh.ray_structure_intersection(torch.from_numpy(Q).cuda(), torch.from_numpy(d).cuda())
    rt, rti = oracle.ray_brute(V, F, Q, d)
    assert np.array_equal(ti.cpu().numpy(), rti) and np.array_equal(t.cpu().numpy(), rt.astype(np.float32))
    # ShapeDiameter from the vertices with their closest elements' normals
    sd = bvh.shape_diameter(torch.from_numpy(V).cuda())
    np.testing.assert_array_equal(sd.cpu().numpy(), oracle.MeshIndex(V, F).shape_diameter(V))
    bvh.close()
    # k nearest vertices of each query point
    pts = T.PointBvh(torch.from_numpy(V).cuda())
    k = min(8, len(V))
    ki, kd = pts.k_closest_pairs(torch.from_numpy(Q).cuda(), k)
    bi, bd = oracle.knn_brute(V, Q, k)
    assert np.array_equal(ki.cpu().numpy(), bi) and np.array_equal(kd.cpu().numpy(), bd.astype(np.float32))
    pts.close()
