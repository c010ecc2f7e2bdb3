"""The oracle pinned to the reference's own code.

tests/golden/reference_outputs.npz holds outputs of the reference's BvhN, Triangle3, AxisAlignedBoxN, Random and Math
sources compiled in this build (oracle/_ref, built from the reference's files by oracle/Makefile with an Eigen subset in
place of Eigen; written by tests/golden/make_ref_golden.py). The oracle's reference mode must reproduce them bit for bit:
the kd-tree build, traversal and tie order, the FP32 triangle arithmetic and the random stream. Its lowest-index mode
(the CUDA path's contract) must give the same distances and hit times. Where the reference library itself is present,
the same comparisons run on further seeded inputs.
"""

import os
import sys

import numpy as np
import pytest

from tests.conftest import ROOT

sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
import make_ref_golden as G  # noqa: E402


@pytest.fixture(scope="module")
def ref():
    return np.load(os.path.join(ROOT, "tests", "golden", "reference_outputs.npz"))


@pytest.fixture(scope="module")
def cases():
    return G.inputs()


def test_closest_reference_mode_is_the_reference(oracle, ref, cases):
    V, F, Q = cases["closest"]
    m = oracle.MeshIndex(V, F)
    for tag, b in (("", -1.0), ("_b005", 0.05), ("_b03", 0.3)):
        i, d, cp = m.closest_ref(Q, dist_bound=b)
        assert np.array_equal(i, ref["closest_index" + tag]), tag
        assert np.array_equal(d, ref["closest_dist" + tag]), tag
        assert np.array_equal(cp, ref["closest_cp" + tag]), tag
        # lowest-index mode: the same distance for every query, an element only where the reference has one
        ci, cd2, _ = m.closest_contract(Q, dist_bound=b)
        assert np.array_equal(ci >= 0, ref["closest_index" + tag] >= 0), tag
        found = ci >= 0
        assert np.array_equal(np.sqrt(cd2[found].astype(np.float32).astype(np.float64)),
                              ref["closest_dist" + tag][found]), tag
    # the bounds are the reference's: a bound is loosened by 0.1 % of the root box diagonal, so some elements lie
    # just beyond it
    d = ref["closest_dist_b005"]
    assert np.any(d > 0.05)


def test_ray_reference_mode_is_the_reference(oracle, ref, cases):
    V, F, o, d = cases["ray"]
    m = oracle.MeshIndex(V, F)
    for tag, mt in (("", -1.0), ("_t045", 0.45)):
        t, i, n = m.ray_ref(o, d, max_time=mt)
        assert np.array_equal(t, ref["ray_time" + tag]), tag
        assert np.array_equal(i, ref["ray_index" + tag]), tag
        assert np.array_equal(n, ref["ray_normal" + tag]), tag
        ct, ci = m.ray_contract(o, d, max_time=mt)
        assert np.array_equal(ct.astype(np.float32), ref["ray_time" + tag]), tag


def test_knn_reference_mode_is_the_reference(oracle, ref, cases):
    P, Q, ex = cases["knn"]
    pi = oracle.PointIndex(P)
    for tag, b in (("", -1.0), ("_b003", 0.03)):
        i, d2 = pi.knn_ref(Q, 8, dist_bound=b, exclude=ex)
        assert np.array_equal(i, ref["knn_index" + tag]), tag
        assert np.array_equal(d2, ref["knn_mad" + tag]), tag
        ci, cd2 = pi.knn_contract(Q, 8, dist_bound=b, exclude=ex)
        assert np.array_equal(cd2.astype(np.float32).astype(np.float64), ref["knn_mad" + tag]), tag


def test_triangle_arithmetic_is_the_reference(oracle, ref, cases):
    tris, pts, other, rdir = cases["tri"]
    cp, _ = oracle.triangle_closest_points(tris, pts)
    assert np.array_equal(cp, ref["tri_closest"], equal_nan=True)
    assert np.array_equal(oracle.triangle_ray_times(tris, pts, rdir), ref["tri_ray_time"], equal_nan=True)
    d2, pa, pb = oracle.triangle_pair_distances(tris, other)
    assert np.array_equal(d2, ref["tri_pair_d2"], equal_nan=True)
    assert np.array_equal(pa, ref["tri_pair_pa"], equal_nan=True)
    assert np.array_equal(pb, ref["tri_pair_pb"], equal_nan=True)


def test_mesh_pairs_match_the_reference(oracle, ref, cases):
    """The reference's dual descent keeps the first of several pairs at the minimum distance; the lowest-index pair
    the oracle returns is at the same squared distance, and the reference's own pair is at that distance too."""
    Va, Fa, Vb, Fb = cases["pair"]
    for tag, (t, q) in (("_ab", ((Va, Fa), (Vb, Fb))), ("_ba", ((Vb, Fb), (Va, Fa)))):
        qi, ti, d2, _, _ = oracle.MeshIndex(*t).closest_pair_contract(*q)
        assert qi >= 0 and d2 == float(ref["pair_mad" + tag])
        rq, rt = ref["pair_index" + tag]
        assert qi <= rq
        rd2, _, _ = oracle.triangle_pair_distances(t[0][t[1][rt]].reshape(1, 9), q[0][q[1][rq]].reshape(1, 9))
        assert float(rd2[0]) == d2


def test_random_stream_and_tree_depth_are_the_reference(oracle, ref):
    for s in (5489, 0xFFFF, 1234):
        assert np.array_equal(oracle.thea_random_bits(s, 1248), ref["random_%d" % s])
    assert [oracle.tree_depth(int(n)) for n in ref["tree_depth_n"]] == list(ref["tree_depth"])


def test_live_reference_on_more_inputs(oracle):
    """Where the reference library was built here: more seeded meshes, queries and point sets, bit for bit."""
    from oracle import reference as R
    if not R.available():
        pytest.skip("the reference library is built only where the reference sources are present")
    from thea_gb300 import workloads as W
    for sub, seed in ((1, 1), (3, 2), (4, 3)):
        V, F = W.noisy_icosphere(sub, seed, sigma=0.03)
        Q = W.uniform_box_points(3000, [-1.5] * 3, [1.5] * 3, seed + 10)
        Q = np.concatenate([Q, V[::3], (V * np.float32(1.0 + 1e-6)).astype(np.float32)[::5]])
        m, r = oracle.MeshIndex(V, F), R.Mesh(V, F)
        for b in (-1.0, 0.02, 0.4):
            a, c = m.closest_ref(Q, dist_bound=b), r.closest(Q, dist_bound=b)
            for x, y in zip(a, c):
                assert np.array_equal(x, y), (sub, b)
        o, d = W.random_rays(3000, [-2] * 3, [2] * 3, seed + 20)
        for mt in (-1.0, 1.0):
            for x, y in zip(m.ray_ref(o, d, max_time=mt), r.ray(o, d, max_time=mt)):
                assert np.array_equal(x, y), (sub, mt)
    P = W.uniform_box_points(5000, [0] * 3, [1] * 3, 41)
    P[100:140] = P[3]
    pi, rp = oracle.PointIndex(P), R.Points(P)
    for k in (1, 5, 16, 32):
        ex = np.arange(500, dtype=np.int32)
        a, c = pi.knn_ref(P[:500], k, exclude=ex), rp.knn(P[:500], k, exclude=ex)
        assert np.array_equal(a[0], c[0]) and np.array_equal(a[1], c[1]), k


def test_best_fit_sphere_is_the_reference(oracle, ref, cases):
    """The smallest enclosing ball (BestFitSphereN, the reference's miniball): the oracle's radius rounded to float is the
    reference's radius, and the centres agree to float rounding."""
    for j, P in enumerate(cases["sphere"]):
        c, r = oracle.best_fit_sphere(P)
        rc, rr = ref["sphere_center_%d" % j], ref["sphere_radius_%d" % j]
        assert np.float32(r) == rr, j
        scale = max(1.0, float(np.abs(P).max()))
        assert np.abs(c - rc.astype(np.float64)).max() <= 4e-7 * scale, j
        # every point inside, some on the boundary
        d = np.sqrt(((P.astype(np.float64) - c) ** 2).sum(1))
        assert d.max() <= r * (1 + 1e-12) + 1e-300 and (len(P) == 1 or d.max() >= r * (1 - 1e-12)), j


def test_live_best_fit_sphere(oracle):
    """Where the reference library was built here: more seeded point sets against the reference's miniball."""
    from oracle import reference as R
    if not R.available():
        pytest.skip("the reference library is built only where the reference sources are present")
    rng = np.random.default_rng(80)
    for t in range(20):
        n = int(rng.integers(1, 3000))
        P = (rng.normal(size=(n, 3)) * rng.uniform(0.01, 10, 3) + rng.normal(size=3) * 5).astype(np.float32)
        c, r = oracle.best_fit_sphere(P)
        rc, rr = R.best_fit_sphere(P)
        assert abs(np.float32(r) - np.float32(rr)) <= np.spacing(np.float32(rr)), t
        assert np.abs(c - rc).max() <= 1e-6 * max(1.0, float(np.abs(P).max())), t
