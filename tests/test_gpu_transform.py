"""GPU parity of the affine transform path (BvhN::setTransform, BvhN.hpp:903-912, 2027-2062, 2175-2184).

Closest-point and k-NN queries on a transformed handle must equal the oracle on the elements mapped into world space;
rays must equal the oracle's object-space traversal of the rays mapped by the FP32 inverse, with normals mapped back by
the inverse transpose. Bit-exact throughout (the transform arithmetic is restated in the oracle in the same order).
"""

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


def dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t):
    import torch
    torch.cuda.synchronize()
    return t.cpu().numpy() if t is not None else None


def affine(seed, scale=(1.7, 0.6, 1.2), shear=0.3, shift=(0.4, -1.1, 2.5)):
    """Rotation x anisotropic scale x shear + translation, rounded to FP32 (row-major 3x4)."""
    rng = np.random.default_rng(seed)
    q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
    S = np.diag(scale)
    H = np.eye(3)
    H[0, 1] = shear
    m = np.zeros((3, 4))
    m[:, :3] = q @ S @ H
    m[:, 3] = shift
    return m.astype(np.float32)


def bounded_contract(oracle, V, M, Q, ri, rd2, bound):
    """Closest elements under dist_bound on a BVH of V with transform M, from the unbounded lowest-index results."""
    f32 = np.float32
    lo, hi = V.min(0).astype(f32), V.max(0).astype(f32)
    c = f32(0.5) * (hi + lo)
    lo, hi = f32(1.05) * (lo - c) + c, f32(1.05) * (hi - c) + c
    corners = np.array([[(hi if k & (1 << a) else lo)[a] for a in range(3)] for k in range(8)], f32)
    w = oracle.affine_points(M, corners)
    wlo, whi = w.min(0), w.max(0)
    e = whi - wlo
    fudge = max(0.001 * float(np.sqrt(f32(e[0] * e[0] + (e[1] * e[1] + e[2] * e[2])))), float(f32(100) * f32(2.0 ** -23)))
    d = np.maximum(np.maximum(Q, wlo) - np.minimum(Q, whi), f32(0)).astype(f32)
    lb = d[:, 0] * d[:, 0] + (d[:, 1] * d[:, 1] + d[:, 2] * d[:, 2])
    keep = (lb.astype(np.float64) <= bound * bound) & (rd2.astype(np.float32).astype(np.float64) < (bound + fudge) ** 2)
    return np.where(keep, ri, -1)


def test_closest_point_on_transformed_mesh(T, oracle):
    V, F = W.noisy_icosphere(4, 51)
    M = affine(52)
    Vw = oracle.affine_points(M, V)
    lo, hi = Vw.min(0) - 0.5, Vw.max(0) + 0.5
    Q = W.uniform_box_points(30000, lo, hi, 53)
    Q = np.concatenate([Q, Vw])
    bvh = T.MeshBvh(dev(V), dev(F))
    bvh.set_transform(M)
    m, inv = bvh.transform()
    assert np.array_equal(m, M) and np.array_equal(inv, oracle.affine_inverse(M))
    idx, dist, cp = bvh.closest_element(dev(Q))
    ri, rd2, rcp = oracle.MeshIndex(Vw, F).closest_contract(Q)
    assert np.array_equal(host(idx), ri)
    assert np.array_equal(host(dist), np.sqrt(rd2.astype(np.float32)))
    assert np.array_equal(host(cp), rcp.astype(np.float32))
    # world-space bounds
    info = bvh.info()
    assert np.allclose(info["bounds_lo"], Vw.min(0)) and np.allclose(info["bounds_hi"], Vw.max(0))
    # FP64 re-check mode runs on the world-space copy too
    i64, _, _, err = bvh.closest_element_ex(dev(Q), precision="fp64")
    assert host(err).max() <= 1e-6 * max(1.0, float(np.abs(Vw).max()))
    # dist_bound applies in world space, as the reference's closestPair applies it to a transformed BVH: the root box
    # is the object-space element box grown by 1.05 and mapped by transformAndBound, a query farther than the bound
    # from it gets nothing, and the bound is loosened by 0.1 % of that box's diagonal
    bi, _, _ = bvh.closest_element(dev(Q), dist_bound=0.2)
    assert np.array_equal(host(bi), bounded_contract(oracle, V, M, Q, ri, rd2, 0.2))
    # clearing the transform restores the object-space answers
    bvh.clear_transform()
    assert bvh.transform() is None
    i0, _, _ = bvh.closest_element(dev(Q))
    assert np.array_equal(host(i0), oracle.MeshIndex(V, F).closest_contract(Q)[0])


def test_rays_on_transformed_mesh(T, oracle):
    V, F = W.noisy_icosphere(4, 61)
    M = affine(62, scale=(0.5, 2.0, 1.0), shear=-0.4)
    Vw = oracle.affine_points(M, V)
    lo, hi = Vw.min(0) - 1.0, Vw.max(0) + 1.0
    O, D = W.random_rays(30000, lo, hi, 63)
    bvh = T.MeshBvh(dev(V), dev(F))
    bvh.set_transform(M)
    t, idx, nrm = bvh.ray_structure_intersection(dev(O), dev(D), normals=True)
    t, idx, nrm = host(t), host(idx), host(nrm)
    inv = oracle.affine_inverse(M)
    Oo, Do = oracle.affine_points(inv, O), oracle.affine_vectors(inv, D)
    rt, ri = oracle.MeshIndex(V, F).ray_contract(Oo, Do)
    assert np.array_equal(idx, ri)
    assert np.array_equal(t, rt.astype(np.float32))
    hit = idx >= 0
    assert 1000 < hit.sum() < len(idx)
    tri = V[F[idx[hit]]].reshape(-1, 9)
    n_obj = oracle.triangle_props(tri)[0]
    assert np.array_equal(nrm[hit], oracle.normals_to_world(inv, n_obj))
    assert not nrm[~hit].any()
    # max_time bounds the world-space ray parameter (the same parameter in object space)
    bt, bi, _ = bvh.ray_structure_intersection(dev(O), dev(D), max_time=0.5)
    rbt, rbi = oracle.MeshIndex(V, F).ray_contract(Oo, Do, max_time=0.5)
    assert np.array_equal(host(bi), rbi) and np.array_equal(host(bt), rbt.astype(np.float32))
    # host arrays take the staged path through the same transform
    th, ih, nh = bvh.ray_structure_intersection(O, D, normals=True)
    assert np.array_equal(ih, idx) and np.array_equal(th, t) and np.array_equal(nh, nrm)


def test_ray_only_layout_takes_a_transform(T, oracle):
    V, F = W.noisy_icosphere(3, 71)
    M = affine(72)
    O, D = W.random_rays(5000, [-3] * 3, [3] * 3, 73)
    bvh = T.MeshBvh(dev(V), dev(F), layouts=2)
    bvh.set_transform(M)
    t, idx, _ = bvh.ray_structure_intersection(dev(O), dev(D))
    inv = oracle.affine_inverse(M)
    rt, ri = oracle.MeshIndex(V, F).ray_contract(oracle.affine_points(inv, O), oracle.affine_vectors(inv, D))
    assert np.array_equal(host(idx), ri)
    lo = np.array(bvh.info()["bounds_lo"])
    assert np.all(lo <= oracle.affine_points(M, V).min(0) + 1e-6)


def test_points_on_transformed_set(T, oracle):
    P = W.uniform_box_points(40000, [0] * 3, [1] * 3, 81)
    M = affine(82)
    Pw = oracle.affine_points(M, P)
    Q = W.uniform_box_points(6000, Pw.min(0), Pw.max(0), 83)
    a = T.PointBvh(dev(P))
    a.set_transform(M)
    b = T.PointBvh(dev(Pw))
    for x, y in zip(a.k_closest_pairs(dev(Q), 8), b.k_closest_pairs(dev(Q), 8)):
        assert np.array_equal(host(x), host(y))
    ri, rd2 = oracle.PointIndex(Pw).knn_contract(Q, 8)
    idx, d2 = a.k_closest_pairs(dev(Q), 8)
    assert np.array_equal(host(idx), ri) and np.array_equal(host(d2), rd2.astype(np.float32))
    for x, y in zip(a.k_closest_self(6), b.k_closest_self(6)):
        assert np.array_equal(np.asarray(x), np.asarray(y))
    ra = a.radius_neighbors(dev(Q[:500]), 0.05)
    rb = b.radius_neighbors(dev(Q[:500]), 0.05)
    for x, y in zip(ra, rb):
        assert np.array_equal(host(x), host(y))


def test_transform_survives_an_image_round_trip(T):
    V, F = W.noisy_icosphere(3, 91)
    M = affine(92)
    Q = W.uniform_box_points(5000, [-3] * 3, [3] * 3, 93)
    O, D = W.random_rays(5000, [-3] * 3, [3] * 3, 94)
    a = T.MeshBvh(dev(V), dev(F))
    a.set_transform(M)
    b = T.MeshBvh.from_bytes(a.to_bytes())
    assert np.array_equal(b.transform()[0], M)
    for x, y in zip(a.closest_element(dev(Q)), b.closest_element(dev(Q))):
        assert np.array_equal(host(x), host(y))
    for x, y in zip(a.ray_structure_intersection(dev(O), dev(D), normals=True),
                    b.ray_structure_intersection(dev(O), dev(D), normals=True)):
        assert np.array_equal(host(x), host(y))


def test_bad_transforms_are_refused(T):
    import torch
    V, F = W.noisy_icosphere(2, 101)
    bvh = T.MeshBvh(dev(V), dev(F))
    singular = np.zeros((3, 4), np.float32)
    singular[0, 0] = singular[1, 1] = 1.0
    for bad in (singular, np.full((3, 4), np.nan, np.float32)):
        with pytest.raises(T.TheaError) as e:
            bvh.set_transform(bad)
        assert e.value.status == 1
    assert bvh.transform() is None
    Vh, Fh, foff, _, _, _ = W.config3_numpy(4, min_level=1, max_level=2, min_q=1, max_q=2)
    forest = T.MeshForest(Vh, Fh, foff)
    with pytest.raises(T.TheaError):
        forest.set_transform(affine(102))
    torch.cuda.synchronize()
