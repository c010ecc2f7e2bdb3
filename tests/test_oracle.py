"""CPU tests of the oracle: known-answer checks, agreement between its reference and contract modes, agreement of its
tree traversals with brute force, and the committed golden fixtures."""

import os

import numpy as np
import pytest

from thea_gb300 import workloads as W


def test_random_matches_std_mt19937_where_the_variant_agrees(oracle):
    # Thea's generate() skips re-twisting word N - M = 227 (Code/Source/Random.cpp:120); everything that does not
    # depend on that word equals the standard MT19937, whose seeding and tempering Thea shares.
    for seed in (5489, 0xFFFF, 1):
        a = oracle.thea_random_bits(seed, 1248)
        b = oracle.std_mt19937_bits(seed, 1248)
        assert np.array_equal(a[:227], b[:227])
        diff = np.nonzero(a[:624] != b[:624])[0]
        assert set(diff.tolist()) <= {227, 454}
        assert 227 in diff.tolist()


def test_random_known_answer(oracle):
    # std::mt19937 with the default seed gives 3499211612 as its first output; Thea's variant shares it.
    assert oracle.thea_random_bits(5489, 1)[0] == 3499211612


def test_tree_depth_formula(oracle):
    # Math::treeDepth(n, 5, 0.5): ceil(log(n / 5) / -log(0.5f))
    assert oracle.tree_depth(81920) == 14
    assert oracle.tree_depth(5) == 0
    assert oracle.tree_depth(1) == 0
    assert oracle.tree_depth(11) == 2


@pytest.mark.parametrize("sub,seed", [(1, 1), (2, 2), (3, 3)])
def test_closest_contract_equals_brute_force(oracle, sub, seed):
    V, F = W.noisy_icosphere(sub, seed)
    Q = W.uniform_box_points(400, [-1.5] * 3, [1.5] * 3, seed + 100)
    Q = np.concatenate([Q, V[:50], (V[:50] * 1.3).astype(np.float32)])
    m = oracle.MeshIndex(V, F)
    i1, d1, c1 = m.closest_contract(Q)
    i2, d2, c2 = oracle.closest_brute(V, F, Q)
    assert np.array_equal(i1, i2) and np.array_equal(d1, d2) and np.array_equal(c1, c2)
    # reference mode picks an element at the same (bit-identical) distance
    ri, rdist, rcp = m.closest_ref(Q)
    Vt = V[F[ri]]
    cp_ref, d2_ref = oracle.triangle_closest_points(Vt.reshape(-1, 9), Q)
    assert np.array_equal(d2_ref.astype(np.float64), d1)
    assert np.array_equal(np.sqrt(d2_ref.astype(np.float64)), rdist)


def test_closest_dist_bound(oracle):
    V, F = W.noisy_icosphere(2, 5)
    Q = W.uniform_box_points(300, [-1.5] * 3, [1.5] * 3, 6)
    m = oracle.MeshIndex(V, F)
    for b in (0.05, 0.2, 0.6):
        i1, d1, _ = m.closest_contract(Q, dist_bound=b)
        i2, d2, _ = oracle.closest_brute(V, F, Q, dist_bound=b)
        assert np.array_equal(i1, i2)
        ri, _, _ = m.closest_ref(Q, dist_bound=b)
        assert np.array_equal(ri >= 0, i1 >= 0)
        # the reference loosens a given bound by 0.1 % of its root box diagonal (here about 0.0037)
        assert np.all(np.sqrt(d1[i1 >= 0]) < b + 0.004)


def test_ray_contract_equals_brute_force(oracle):
    V, F = W.heightfield(20, 7)
    o, d = W.cosine_rays_down(500, 8)
    m = oracle.MeshIndex(V, F)
    t1, i1 = m.ray_contract(o, d)
    t2, i2 = oracle.ray_brute(V, F, o, d)
    assert np.array_equal(i1, i2) and np.array_equal(t1, t2)
    rt, ri, rn = m.ray_ref(o, d)
    assert np.array_equal(rt.astype(np.float64), t1)
    for mt in (0.3, 0.55):
        t3, i3 = m.ray_contract(o, d, max_time=mt)
        t4, i4 = oracle.ray_brute(V, F, o, d, max_time=mt)
        assert np.array_equal(i3, i4) and np.array_equal(t3, t4)


def test_ray_random_directions_sphere(oracle):
    V, F = W.noisy_icosphere(2, 9)
    o, d = W.random_rays(500, [-2] * 3, [2] * 3, 10)
    m = oracle.MeshIndex(V, F)
    t1, i1 = m.ray_contract(o, d)
    t2, i2 = oracle.ray_brute(V, F, o, d)
    assert np.array_equal(i1, i2) and np.array_equal(t1, t2)


def test_knn_contract_equals_brute_force(oracle):
    P = W.uniform_box_points(3000, [0] * 3, [1] * 3, 11)
    P[100:120] = P[0]  # exact duplicates: ties at distance 0 and equal distances elsewhere
    Q = np.concatenate([P[:300], W.uniform_box_points(200, [-0.2] * 3, [1.2] * 3, 12)])
    ex = np.concatenate([np.arange(300, dtype=np.int32), -np.ones(200, np.int32)])
    pi = oracle.PointIndex(P)
    for k in (1, 3, 8, 16):
        i1, d1 = pi.knn_contract(Q, k, exclude=ex)
        i2, d2 = oracle.knn_brute(P, Q, k, exclude=ex)
        assert np.array_equal(i1, i2) and np.array_equal(d1, d2)
        ri, rd = pi.knn_ref(Q, k, exclude=ex)
        assert np.array_equal(rd, d1)  # same distances; indices may differ among ties
    i1, d1 = pi.knn_contract(Q, 8, dist_bound=0.05)
    i2, d2 = oracle.knn_brute(P, Q, 8, dist_bound=0.05)
    assert np.array_equal(i1, i2)


def test_sampler_is_deterministic_and_area_weighted(oracle):
    V, F = W.noisy_icosphere(2, 13)
    p1, n1, f1 = oracle.sample_by_area(V, F, 20000, 99)
    p2, n2, f2 = oracle.sample_by_area(V, F, 20000, 99)
    assert np.array_equal(p1, p2) and np.array_equal(f1, f2)
    _, _, _, area = oracle.triangle_props(V[F].reshape(-1, 9))
    counts = np.bincount(f1, minlength=len(F))
    expected = 20000 * area / area.sum()
    chi2 = np.sum((counts - expected) ** 2 / expected)
    assert chi2 < 2.0 * len(F)  # loose goodness of fit
    # each sample lies on its triangle's plane
    nrm, dist, _, _ = oracle.triangle_props(V[F[f1]].reshape(-1, 9))
    assert np.max(np.abs(np.sum(p1 * nrm, 1) - dist)) < 1e-5


def test_sampler_zero_area_mesh(oracle):
    V = np.zeros((3, 3), np.float32)
    F = np.array([[0, 1, 2]], np.int32)
    p, n, f = oracle.sample_by_area(V, F, 10, 1)
    assert len(p) == 0


def test_degenerate_triangles(oracle):
    # zero-area triangles: coincident vertices and collinear vertices
    V = np.array([[0, 0, 0], [1, 0, 0], [2, 0, 0], [0, 1, 0], [0, 0, 0]], np.float32)
    F = np.array([[0, 1, 2], [0, 4, 3], [0, 1, 3]], np.int32)
    Q = W.uniform_box_points(200, [-1] * 3, [2] * 3, 14)
    m = oracle.MeshIndex(V, F)
    i1, d1, _ = m.closest_contract(Q)
    i2, d2, _ = oracle.closest_brute(V, F, Q)
    assert np.array_equal(i1, i2) and np.array_equal(d1, d2)


@pytest.mark.parametrize("name", ["closest", "ray", "sample_knn", "testbvh", "random"])
def test_golden_fixtures_reproduce(oracle, golden_dir, name):
    z = np.load(os.path.join(golden_dir, name + ".npz"))
    if name == "closest":
        m = oracle.MeshIndex(z["V"], z["F"])
        i, d2, cp = m.closest_contract(z["Q"])
        assert np.array_equal(i, z["index"]) and np.array_equal(d2.astype(np.float32), z["d2"])
        assert np.array_equal(cp.astype(np.float32), z["cp"])
        ri, rd, rcp = m.closest_ref(z["Q"])
        assert np.array_equal(ri, z["ref_index"]) and np.array_equal(rd, z["ref_dist"])
        bi, bd2, _ = m.closest_contract(z["Q"], dist_bound=float(z["bound"]))
        assert np.array_equal(bi, z["bound_index"])
    elif name == "ray":
        m = oracle.MeshIndex(z["V"], z["F"])
        t, i = m.ray_contract(z["O"], z["D"])
        assert np.array_equal(i, z["index"]) and np.array_equal(t.astype(np.float32), z["time"])
        rt, ri, rn = m.ray_ref(z["O"], z["D"])
        assert np.array_equal(ri, z["ref_index"]) and np.array_equal(rn, z["ref_normal"])
    elif name == "sample_knn":
        p, n, f = oracle.sample_by_area(z["V"], z["F"], len(z["pos"]), int(z["seed"]))
        assert np.array_equal(p, z["pos"]) and np.array_equal(n, z["nrm"]) and np.array_equal(f, z["face"])
        pi = oracle.PointIndex(p)
        ki, kd = pi.knn_contract(p, 8, exclude=np.arange(len(p), dtype=np.int32))
        assert np.array_equal(ki, z["knn_index"])
    elif name == "testbvh":
        pi = oracle.PointIndex(z["points"])
        i, d = pi.knn_contract(z["query"], 3, dist_bound=0.25)
        assert np.array_equal(i, z["knn3_index"])
        tm = oracle.MeshIndex(z["tri_vertices"], z["tri_faces"])
        ti, td2, tcp = tm.closest_contract(z["query"], dist_bound=0.25)
        assert np.array_equal(ti, z["tri_index"])
        rt, ri = tm.ray_contract(np.zeros((1, 3), np.float32), z["ray_dir"][None])
        assert np.array_equal(ri, z["ray_index"])
    else:
        assert np.array_equal(oracle.thea_random_bits(5489, 2000), z["seed_5489"])
        assert np.array_equal(oracle.thea_random_bits(0xFFFF, 2000), z["seed_ffff"])


def test_range_brute_matches_numpy_restatement(oracle):
    # BallN::contains: (p - center).squaredNorm() <= radius * radius, FP32, Eigen's e0 + (e1 + e2) order
    rng = np.random.default_rng(12)
    P = rng.uniform(0, 1, (3000, 3)).astype(np.float32)
    P[100:110] = P[5]
    q = np.concatenate([P[:50], rng.uniform(-0.2, 1.2, (50, 3)).astype(np.float32)])
    ex = np.concatenate([np.arange(50, dtype=np.int32), -np.ones(50, np.int32)])
    r = np.float32(0.07)
    off, idx, d2 = oracle.range_brute(P, q, r, exclude=ex)
    for i in range(len(q)):
        diff = P - q[i]
        dd = diff[:, 0] * diff[:, 0] + (diff[:, 1] * diff[:, 1] + diff[:, 2] * diff[:, 2])
        want = np.nonzero(dd <= r * r)[0]
        want = want[want != ex[i]]
        assert np.array_equal(idx[off[i]:off[i + 1]], want)
        assert np.array_equal(d2[off[i]:off[i + 1]], dd[want])


def test_affine_restatement(oracle):
    """The transform arithmetic (AffineTransformN::inverse / operator*, normalToWorldSpace): exact on a map whose inverse
    is representable, within FP32 rounding of the FP64 inverse on a general map, identity leaves points bit-identical."""
    m = np.array([[2, 0, 0, 1], [0, 4, 0, 2], [0, 0, 8, 3]], np.float32)
    inv = oracle.affine_inverse(m)
    assert np.array_equal(inv, np.array([[0.5, 0, 0, -0.5], [0, 0.25, 0, -0.5], [0, 0, 0.125, -0.375]], np.float32))
    P = W.uniform_box_points(1000, [-5] * 3, [5] * 3, 1)
    assert np.array_equal(oracle.affine_points(np.eye(3, 4, dtype=np.float32), P), P)
    m0 = m.copy()
    m0[:, 3] = 0
    assert np.array_equal(oracle.affine_points(oracle.affine_inverse(m0), oracle.affine_points(m0, P)), P)  # exact
    rng = np.random.default_rng(2)
    for _ in range(20):
        g = rng.normal(size=(3, 4)).astype(np.float32)
        inv = oracle.affine_inverse(g)
        g64 = np.vstack([g.astype(np.float64), [0, 0, 0, 1]])
        ref = np.linalg.inv(g64)[:3]
        cond = np.linalg.cond(g64[:3, :3])
        assert np.allclose(inv, ref, rtol=0, atol=1e-5 * cond * np.abs(ref).max())
        # a point mapped there and back returns within rounding
        back = oracle.affine_points(inv, oracle.affine_points(g, P))
        assert np.allclose(back, P, atol=1e-4 * cond * 5)
    assert oracle.affine_inverse(np.array([[1, 2, 3, 0], [2, 4, 6, 0], [0, 0, 1, 0]], np.float32)) is None
    # a rotation maps unit normals like vectors
    c, s = np.float32(0.6), np.float32(0.8)
    rot = np.array([[c, -s, 0, 3], [s, c, 0, -1], [0, 0, 1, 2]], np.float32)
    n = np.array([[1, 0, 0], [0, 0, 1]], np.float32)
    w = oracle.normals_to_world(oracle.affine_inverse(rot), n)
    assert np.allclose(w, oracle.affine_vectors(rot, n), atol=1e-6)


def test_random_sphere_restatement(oracle):
    """Random::sphere (Knop's method) in the oracle equals a NumPy FP32 restatement over the same uniform stream, and
    gives unit vectors."""
    n = 3000
    words = oracle.thea_random_bits(99, 4 * n).astype(np.uint64)
    u = words.astype(np.float32) * np.float32(1.0 / 0xFFFFFFFF)
    out = []
    k = 0
    while len(out) < n:
        x = np.float32(2) * u[k] - np.float32(1)
        y = np.float32(2) * u[k + 1] - np.float32(1)
        k += 2
        m2 = np.float32(x * x) + np.float32(y * y)
        if m2 > 1 or float(m2) < 1e-10:
            continue
        z = np.float32(2) * m2 - np.float32(1)
        s = np.float32(2) * np.sqrt(np.float32(1) - m2)
        out.append([x * s, y * s, z])
    ref = np.array(out, np.float32)
    got = oracle.random_sphere(99, n)
    assert np.array_equal(got, ref)
    assert np.allclose(np.linalg.norm(got, axis=1), 1, atol=1e-6)


def test_visibility_restatement_limits(oracle):
    """Visibility of points far outside a sphere is near 1, inside it is 0, on it about one half."""
    V, F = W.noisy_icosphere(3, 5)
    m = oracle.MeshIndex(V, F)
    assert np.all(m.visibility(V[:50] * np.float32(0.5), 100, 7) == 0)
    assert np.all(m.visibility(V[:50] * np.float32(4), 100, 7) > 0.9)
    on = m.visibility(V[:200], 100, 7)
    assert 0.4 < on.mean() < 0.6


def test_shape_diameter_restatement(oracle):
    """ShapeDiameter on a sphere: every value in (0, 1); a point sampled on a face with that face's normal gives what
    the closest-element normal gives; with outward normals flipped the inward rays leave the sphere (-1)."""
    V, F = W.noisy_icosphere(3, 6, sigma=0.0)
    m = oracle.MeshIndex(V, F)
    P, Nf, _ = oracle.sample_by_area(V, F, 400, 3)
    with_normals = m.shape_diameter(P, Nf)
    assert np.all((with_normals > 0) & (with_normals < 1))
    from_closest = m.shape_diameter(P)
    assert np.mean(with_normals == from_closest) > 0.99
    assert np.all(m.shape_diameter(P * np.float32(1.01), -Nf) == -1.0)
    # a sphere's diameter relative to the padded box diagonal, with the cone's cosine weighting: a stable band
    assert 0.3 < with_normals.mean() < 0.45


def _tri_tri_distance_f64(a, b):
    """Independent FP64 triangle-triangle distance: 0 when an edge of one crosses the other, else the smallest of the
    six vertex-triangle and nine edge-edge distances (vectorised over pairs; no shared code with the oracle)."""
    def pt_tri(p, t):
        # closest point on a triangle by projection, falling back to the three edges
        v0, v1, v2 = t[:, 0], t[:, 1], t[:, 2]
        n = np.cross(v1 - v0, v2 - v0)
        n /= np.linalg.norm(n, axis=1, keepdims=True)
        proj = p - np.sum((p - v0) * n, 1, keepdims=True) * n
        inside = np.ones(len(p), bool)
        for x, y in ((v0, v1), (v1, v2), (v2, v0)):
            inside &= np.sum(np.cross(y - x, proj - x) * n, 1) >= 0
        d = np.where(inside, np.linalg.norm(p - proj, axis=1), np.inf)
        for x, y in ((v0, v1), (v1, v2), (v2, v0)):
            d = np.minimum(d, seg_seg(p, p, x, y))
        return d

    def seg_seg(p1, q1, p2, q2):
        # minimum over a fine parameter grid refined by the closed-form clamped solution
        d1, d2, r = q1 - p1, q2 - p2, p1 - p2
        a, e = np.sum(d1 * d1, 1), np.sum(d2 * d2, 1)
        b, c, f = np.sum(d1 * d2, 1), np.sum(d1 * r, 1), np.sum(d2 * r, 1)
        best = np.full(len(p1), np.inf)
        for s0 in np.linspace(0, 1, 3):
            s = np.full(len(p1), s0)
            for _ in range(60):  # alternate exact clamped minimisations (convex: converges)
                t = np.clip(np.where(e > 0, (b * s + f) / np.where(e > 0, e, 1), 0), 0, 1)
                s = np.clip(np.where(a > 0, (b * t - c) / np.where(a > 0, a, 1), 0), 0, 1)
            t = np.clip(np.where(e > 0, (b * s + f) / np.where(e > 0, e, 1), 0), 0, 1)
            best = np.minimum(best, np.linalg.norm(p1 + s[:, None] * d1 - p2 - t[:, None] * d2, axis=1))
        return best

    def crosses(t, u):
        # some edge of t passes through triangle u (Moller-Trumbore on segments)
        hit = np.zeros(len(t), bool)
        for i, j in ((0, 1), (1, 2), (2, 0)):
            o, d = t[:, i], t[:, j] - t[:, i]
            e1, e2 = u[:, 1] - u[:, 0], u[:, 2] - u[:, 0]
            pv = np.cross(d, e2)
            det = np.sum(e1 * pv, 1)
            ok = np.abs(det) > 1e-300
            inv = 1 / np.where(ok, det, 1)
            tv = o - u[:, 0]
            uu = np.sum(tv * pv, 1) * inv
            qv = np.cross(tv, e1)
            vv = np.sum(d * qv, 1) * inv
            tt = np.sum(e2 * qv, 1) * inv
            hit |= ok & (uu >= 0) & (vv >= 0) & (uu + vv <= 1) & (tt >= 0) & (tt <= 1)
        return hit

    d = np.full(len(a), np.inf)
    for k in range(3):
        d = np.minimum(d, pt_tri(a[:, k], b))
        d = np.minimum(d, pt_tri(b[:, k], a))
        for m in range(3):
            d = np.minimum(d, seg_seg(a[:, k], a[:, (k + 1) % 3], b[:, m], b[:, (m + 1) % 3]))
    return np.where(crosses(a, b) | crosses(b, a), 0.0, d)


def test_triangle_pair_distance_restatement(oracle):
    """The oracle's restatement of TriangleN::squaredDistance(triangle) (Triangle3.hpp:314-400: Moller's intersection
    test, Ericson's edge-edge and vertex-face terms) agrees with an independent FP64 computation to FP32 accuracy, on
    separated, touching, crossing and near-parallel pairs."""
    rng = np.random.default_rng(7)
    n = 4000
    a = rng.normal(size=(n, 3, 3))
    b = rng.normal(size=(n, 3, 3)) * rng.uniform(0.1, 1.5, (n, 1, 1)) + rng.normal(size=(n, 1, 3)) * rng.uniform(
        0, 3, (n, 1, 1))
    # near-parallel pairs: b is a shifted and slightly tilted copy of a
    par = slice(0, 500)
    b[par] = a[par] + rng.normal(size=(500, 1, 3)) * 0.3 + rng.normal(size=(500, 3, 3)) * 1e-3
    a32, b32 = a.astype(np.float32), b.astype(np.float32)
    d2, pa, pb = oracle.triangle_pair_distances(a32.reshape(n, 9), b32.reshape(n, 9))
    ref = _tri_tri_distance_f64(a32.astype(np.float64), b32.astype(np.float64))
    scale = np.abs(a32).max(axis=(1, 2)) + np.abs(b32).max(axis=(1, 2))
    got = np.sqrt(d2.astype(np.float64))
    assert np.all(np.abs(got - ref) <= 1e-4 * scale + 1e-5 * ref), np.max(np.abs(got - ref) / scale)
    # the reported points lie at the reported distance
    sep = np.linalg.norm(pa.astype(np.float64) - pb, axis=1)
    assert np.all(np.abs(sep - got) <= 1e-4 * scale)
    # symmetric up to FP32 rounding (the reference's result depends on which triangle is "this")
    d2r, _, _ = oracle.triangle_pair_distances(b32.reshape(n, 9), a32.reshape(n, 9))
    assert np.all(np.abs(np.sqrt(d2r.astype(np.float64)) - got) <= 1e-4 * scale)


def test_mesh_pair_oracle_tree_equals_brute_force(oracle):
    for seed in range(4):
        Vt, Ft = W.noisy_icosphere(2, 300 + seed)
        Vq, Fq = W.noisy_icosphere(2, 400 + seed)
        Vq = (Vq * 0.5 + np.array([1.6 + 0.3 * seed, 0.2, -0.1], np.float32)).astype(np.float32)
        a = oracle.MeshIndex(Vt, Ft).closest_pair_contract(Vq, Fq)
        b = oracle.mesh_pair_brute(Vt, Ft, Vq, Fq)
        assert a[:3] == b[:3]
        np.testing.assert_array_equal(a[3], b[3])
        assert b[2] > 0
        assert oracle.mesh_pair_brute(Vt, Ft, Vq, Fq, dist_bound=0.5 * np.sqrt(b[2]))[0] == -1
        assert oracle.mesh_pair_brute(Vt, Ft, Vq, Fq, dist_bound=1.01 * np.sqrt(b[2]))[:2] == b[:2]
