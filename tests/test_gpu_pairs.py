"""GPU parity of closest pairs between two BVHs (BvhN::closestPair / kClosestPairs with a BVH query) against brute
force over every pair: exact FP32 squared distances, ties by lowest query index then lowest target index."""

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


def _pair_d2(A, B):
    """FP32 squared distances of every (a, b) pair, evaluated as dx*dx + (dy*dy + dz*dz)."""
    d = A[:, None, :] - B[None, :, :]
    return d[..., 0] * d[..., 0] + (d[..., 1] * d[..., 1] + d[..., 2] * d[..., 2])


def _sorted_pairs(d2, bound=-1.0):
    qi, ti = np.meshgrid(np.arange(d2.shape[0]), np.arange(d2.shape[1]), indexing="ij")
    qi, ti, v = qi.ravel(), ti.ravel(), d2.ravel()
    if bound >= 0:
        keep = v.astype(np.float64) < float(bound) ** 2
        qi, ti, v = qi[keep], ti[keep], v[keep]
    o = np.lexsort((ti, qi, v))
    return qi[o], ti[o], v[o]


def test_point_point_pairs(T):
    rng = np.random.default_rng(41)
    A = rng.random((1500, 3), np.float32)
    B = rng.random((2500, 3), np.float32)
    B[7] = A[11]  # an exact duplicate: distance 0
    B[9] = A[3]
    ta, tb = T.PointBvh(A), T.PointBvh(B)
    qi, ti, v = _sorted_pairs(_pair_d2(A, B))
    got = tb.closest_pair(ta)
    assert got[:3] == (int(qi[0]), int(ti[0]), float(v[0])) and (got[0], got[1]) == (3, 9)
    np.testing.assert_array_equal(got[3], A[3])
    np.testing.assert_array_equal(got[4], B[9])
    for k in (1, 5, 32):
        gq, gt, gd = tb.k_closest_pairs(ta, k)
        np.testing.assert_array_equal(gq, qi[:k])
        np.testing.assert_array_equal(gt, ti[:k])
        np.testing.assert_array_equal(gd, v[:k])
    # a bound: only pairs strictly closer; none left under a tiny bound on shifted sets
    bq, bt, bv = _sorted_pairs(_pair_d2(A, B), 0.01)
    gq, gt, gd = tb.k_closest_pairs(ta, 32, dist_bound=0.01)
    n = min(32, len(bq))
    np.testing.assert_array_equal(gq[:n], bq[:n])
    np.testing.assert_array_equal(gt[:n], bt[:n])
    assert np.all(gq[n:] == -1)
    # fewer query points than k
    tiny = T.PointBvh(A[:10])
    sq, st, sv = _sorted_pairs(_pair_d2(A[:10], B))
    gq, gt, gd = tb.k_closest_pairs(tiny, 32)
    np.testing.assert_array_equal(gq, sq[:32])
    np.testing.assert_array_equal(gt, st[:32])
    np.testing.assert_array_equal(gd, sv[:32])
    tiny.close()
    far = T.PointBvh(A + np.float32(10))
    assert tb.closest_pair(far, dist_bound=1.0) is None
    for h in (ta, tb, far):
        h.close()


def test_point_mesh_pairs_both_ways(T, oracle):
    V, F = W.noisy_icosphere(3, 42, sigma=0.05)
    rng = np.random.default_rng(43)
    P = (rng.normal(size=(3000, 3)) * 0.8).astype(np.float32)
    mesh, pts = T.MeshBvh(V, F), T.PointBvh(P)
    ri, rd2, rcp = oracle.closest_brute(V, F, P)
    d2 = rd2.astype(np.float32)
    # points query the mesh: rows are query points
    o = np.lexsort((ri, np.arange(len(P)), d2))[0]
    got = mesh.closest_pair(pts)
    assert got[:3] == (int(o), int(ri[o]), float(d2[o]))
    np.testing.assert_array_equal(got[3], P[o])
    np.testing.assert_array_equal(got[4], rcp[o].astype(np.float32))
    # the mesh queries the points: rows are target points, ties by lowest query element then lowest target point
    o2 = np.lexsort((np.arange(len(P)), ri, d2))[0]
    got2 = pts.closest_pair(mesh)
    assert got2[:3] == (int(ri[o2]), int(o2), float(d2[o2]))
    np.testing.assert_array_equal(got2[3], rcp[o2].astype(np.float32))
    np.testing.assert_array_equal(got2[4], P[o2])
    mesh.close()
    pts.close()


def _mesh_pair_check(oracle, got, want):
    """GPU (query, target, d2, query point, target point) against the oracle's, bit for bit."""
    assert want[0] >= 0 and got is not None
    assert got[:2] == (want[0], want[1])
    assert got[2] == np.float32(want[2])
    np.testing.assert_array_equal(got[3], want[3].astype(np.float32))
    np.testing.assert_array_equal(got[4], want[4].astype(np.float32))


def test_mesh_mesh_closest_pair_against_brute_force(T, oracle):
    """Closest pair between two triangle meshes: TriangleN::squaredDistance with the target triangle as "this"
    (Triangle3.hpp:314-400), lowest query then target index among ties, against every triangle pair on the CPU."""
    Vt, Ft = W.noisy_icosphere(3, 51)
    target = T.MeshBvh(Vt, Ft)
    rng = np.random.default_rng(52)
    for case in range(6):
        Vq, Fq = W.noisy_icosphere(2 + case % 2, 60 + case)
        scale = rng.uniform(0.2, 0.7)
        shift = rng.normal(size=3)
        shift *= (1.05 + scale + 0.3 * case / 5) / np.linalg.norm(shift)
        if case == 5:
            shift *= 0.5  # the spheres intersect: distance 0 at the first intersecting pair
        Vq = (Vq * scale + shift).astype(np.float32)
        query = T.MeshBvh(Vq, Fq)
        want = oracle.mesh_pair_brute(Vt, Ft, Vq, Fq)
        _mesh_pair_check(oracle, target.closest_pair(query), want)
        assert target.closest_pair(query)[:3] == tuple(oracle.MeshIndex(Vt, Ft).closest_pair_contract(Vq, Fq)[:3])
        # the other way round: roles of "this" and "other" swap
        want2 = oracle.mesh_pair_brute(Vq, Fq, Vt, Ft)
        _mesh_pair_check(oracle, query.closest_pair(target), want2)
        # a bound below the closest distance: no pair; just above it: the same pair
        d = float(np.sqrt(want[2]))
        if d > 0:
            assert target.closest_pair(query, dist_bound=d * 0.999) is None
            assert target.closest_pair(query, dist_bound=d * 1.001)[:2] == (want[0], want[1])
        query.close()
    target.close()


def test_mesh_mesh_pairs_touching_and_coplanar(T, oracle):
    """Meshes that share vertices, edges and whole faces (coplanar triangles, Moller's coplanar test) and a mesh against
    itself: every pair with a shared vertex is at distance 0, so the tie rule decides."""
    V, F = W.noisy_icosphere(2, 53)
    m = T.MeshBvh(V, F)
    got = m.closest_pair(m)
    want = oracle.mesh_pair_brute(V, F, V, F)
    _mesh_pair_check(oracle, got, want)
    assert got[:3] == (0, 0, 0.0)
    # a flat grid and a copy lifted by a little, and one with a shared strip
    Vg, Fg = W.heightfield(12, 54, amplitude=0.0)
    Vh = Vg.copy()
    Vh[:, 2] += 0.01
    g, h = T.MeshBvh(Vg, Fg), T.MeshBvh(Vh, Fg)
    _mesh_pair_check(oracle, g.closest_pair(h), oracle.mesh_pair_brute(Vg, Fg, Vh, Fg))
    Vs = Vg.copy()
    Vs[:, 0] += 0.5  # overlapping coplanar grids
    s = T.MeshBvh(Vs, Fg)
    _mesh_pair_check(oracle, g.closest_pair(s), oracle.mesh_pair_brute(Vg, Fg, Vs, Fg))
    for x in (m, g, h, s):
        x.close()


def test_mesh_mesh_pair_larger_meshes_against_the_oracle_tree(T, oracle):
    """Two 20,480-triangle noisy spheres, one stretched and shifted: the GPU pair against the oracle's kd-tree search."""
    Vt, Ft = W.noisy_icosphere(5, 55)
    Vq, Fq = W.noisy_icosphere(5, 56, scale=np.array([0.6, 1.3, 0.8]))
    Vq = (Vq + np.array([1.9, 0.4, -0.2], np.float32)).astype(np.float32)
    t, q = T.MeshBvh(Vt, Ft, width=8), T.MeshBvh(Vq, Fq)
    want = oracle.MeshIndex(Vt, Ft).closest_pair_contract(Vq, Fq)
    _mesh_pair_check(oracle, t.closest_pair(q), want)
    t.close()
    q.close()


def test_pairs_with_a_transformed_target(T, oracle):
    V, F = W.noisy_icosphere(3, 44, sigma=0.03)
    rng = np.random.default_rng(45)
    P = (rng.normal(size=(2000, 3)) * 2.0).astype(np.float32)
    xf = np.array([[0.0, 1.2, 0.0, 0.5], [-1.2, 0.0, 0.0, 0.1], [0.0, 0.0, 0.8, -0.3]], np.float32)
    mesh, pts = T.MeshBvh(V, F), T.PointBvh(P)
    mesh.set_transform(xf)
    Vw = oracle.affine_points(xf, V)
    ri, rd2, _ = oracle.closest_brute(Vw, F, P)
    d2 = rd2.astype(np.float32)
    o = np.lexsort((ri, np.arange(len(P)), d2))[0]
    assert mesh.closest_pair(pts)[:3] == (int(o), int(ri[o]), float(d2[o]))
    mesh.close()
    pts.close()
