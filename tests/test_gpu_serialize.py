"""GPU tests of BVH byte images (thea_bvh_serialize / thea_bvh_deserialize): a reloaded handle answers every query
exactly as the handle it was saved from, and saving it again gives the same bytes."""

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


def same(a, b):
    for x, y in zip(a, b):
        if x is None:
            assert y is None
        else:
            np.testing.assert_array_equal(np.asarray(x), np.asarray(y))


@pytest.mark.parametrize("width", [4, 8])
def test_mesh_image_round_trip(T, width):
    V, F = W.noisy_icosphere(4, 11)
    Q = W.uniform_box_points(20000, [-1.5] * 3, [1.5] * 3, 12)
    O, D = W.random_rays(20000, [-1.5] * 3, [1.5] * 3, 13)
    a = T.MeshBvh(V, F, width=width)
    img = a.to_bytes()
    b = T.MeshBvh.from_bytes(img)
    assert b.to_bytes() == img
    ia, ib = a.info(), b.info()
    ia.pop("device_error_bits"), ib.pop("device_error_bits")
    assert ia == ib
    same(a.closest_element(Q), b.closest_element(Q))
    same(a.closest_element(Q, dist_bound=0.3), b.closest_element(Q, dist_bound=0.3))
    same(a.closest_element_ex(Q, precision="fp64"), b.closest_element_ex(Q, precision="fp64"))
    same(a.ray_structure_intersection(O, D, normals=True), b.ray_structure_intersection(O, D, normals=True))
    same(a.ray_structure_intersection_ex(O, D), b.ray_structure_intersection_ex(O, D))
    with pytest.raises(T.TheaError):
        T.PointBvh.from_bytes(img)
    # a truncated image is refused
    with pytest.raises(T.TheaError):
        T.MeshBvh.from_bytes(img[:-1])


def test_ray_only_layout_round_trip(T):
    V, F = W.noisy_icosphere(3, 21)
    O, D = W.random_rays(5000, [-1.5] * 3, [1.5] * 3, 22)
    a = T.MeshBvh(V, F, layouts=2)
    b = T.MeshBvh.from_bytes(a.to_bytes())
    same(a.ray_structure_intersection(O, D), b.ray_structure_intersection(O, D))


def test_point_image_round_trip(T):
    P = W.uniform_box_points(30000, [0] * 3, [1] * 3, 31)
    Q = W.uniform_box_points(5000, [0] * 3, [1] * 3, 32)
    a = T.PointBvh(P, width=8)
    b = T.PointBvh.from_bytes(a.to_bytes())
    assert b.n == a.n
    same(a.k_closest_pairs(Q, 8), b.k_closest_pairs(Q, 8))
    same(a.k_closest_self(6), b.k_closest_self(6))


def test_forest_image_round_trip(T):
    import torch
    Vh, Fh, foff, Qh, qoff, _ = W.config3_numpy(24, min_level=1, max_level=4, min_q=10, max_q=2000)
    a = T.MeshForest(Vh, Fh, foff)
    b = T.MeshForest.from_bytes(a.to_bytes())
    assert b.num_meshes == a.num_meshes == 24
    q = torch.from_numpy(Qh).cuda()
    qo = torch.from_numpy(qoff).cuda()
    ra = a.batch_closest_element(q, qo, closest_points=True, errors=True)
    rb = b.batch_closest_element(q, qo, closest_points=True, errors=True)
    torch.cuda.synchronize()
    same([x.cpu() for x in ra], [x.cpu() for x in rb])
