"""GPU parity of the any-hit query (BvhN::rayIntersects) and the Visibility feature built on it
(Algorithms/SurfaceFeatures/Local/Visibility.hpp:104-126, with Random(seed) in place of Random::common()).
Bit-exact: hit flags against the oracle's first-hit verdicts, sphere directions and escaped fractions against the oracle.
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


def test_random_sphere_stream(T, oracle):
    for seed in (0, 12345):
        got = T.random_sphere(seed, 200000)
        assert np.array_equal(got, oracle.random_sphere(seed, 200000))
    d = T.random_sphere(7, 1000, device=True).cpu().numpy()
    assert np.array_equal(d, oracle.random_sphere(7, 1000))


@pytest.mark.parametrize("width", [4, 8])
def test_ray_intersects_matches_first_hit_verdicts(T, oracle, width):
    V, F = W.noisy_icosphere(4, 111)
    O, D = W.random_rays(100000, [-2] * 3, [2] * 3, 112)
    bvh = T.MeshBvh(dev(V), dev(F), width=width)
    m = oracle.MeshIndex(V, F)
    for max_time in (-1.0, 0.3, 0.0):
        hit = bvh.ray_intersects(dev(O), dev(D), max_time=max_time).cpu().numpy()
        rt, _ = m.ray_contract(O, D, max_time=max_time)
        assert np.array_equal(hit, rt >= 0), max_time
        assert 0 < hit.sum() < len(hit) or max_time == 0.0
    # host arrays (staged) give the same flags
    assert np.array_equal(bvh.ray_intersects(O, D), m.ray_contract(O, D)[0] >= 0)


def test_ray_intersects_heightfield(T, oracle):
    V, F = W.heightfield(128, 121)
    o, d = W.cosine_rays_down(80000, 122)
    bvh = T.MeshBvh(dev(V), dev(F), max_leaf_size=2)
    hit = bvh.ray_intersects(dev(o), dev(d)).cpu().numpy()
    t, _, _ = bvh.ray_structure_intersection(dev(o), dev(d))
    assert np.array_equal(hit, t.cpu().numpy() >= 0)
    rt, _ = oracle.MeshIndex(V, F).ray_contract(o, d)
    assert np.array_equal(hit, rt >= 0)


def test_visibility_matches_oracle(T, oracle):
    V, F = W.noisy_icosphere(4, 131)
    rng = np.random.default_rng(132)
    P = np.concatenate([V[:1500], (V[1500:2000] * np.float32(0.7)), (V[2000:2500] * np.float32(1.6)),
                        rng.uniform(-2, 2, size=(500, 3)).astype(np.float32)])
    bvh = T.MeshBvh(dev(V), dev(F))
    m = oracle.MeshIndex(V, F)
    got = bvh.visibility(dev(P), num_rays=100, seed=5).cpu().numpy()
    ref = m.visibility(P, 100, 5)
    assert np.array_equal(got, ref)
    assert 0.3 < got[:1500].mean() < 0.7 and np.all(got[1500:2000] == 0)
    # default ray count (num_rays <= 0 -> 100) and an odd count, host arrays
    assert np.array_equal(bvh.visibility(P[:300], num_rays=0, seed=9), m.visibility(P[:300], 100, 9))
    assert np.array_equal(bvh.visibility(P[:300], num_rays=7, seed=9), m.visibility(P[:300], 7, 9))


def test_visibility_with_a_transform(T, oracle):
    V, F = W.noisy_icosphere(3, 141)
    M = np.array([[0.0, -1.5, 0.0, 2.0], [1.5, 0.0, 0.0, -1.0], [0.0, 0.0, 0.75, 0.5]], np.float32)
    Pw = oracle.affine_points(M, V[:800])
    bvh = T.MeshBvh(dev(V), dev(F))
    bvh.set_transform(M)
    got = bvh.visibility(dev(Pw), num_rays=50, seed=3).cpu().numpy()
    assert np.array_equal(got, oracle.MeshIndex(V, F).visibility(Pw, 50, 3, transform=M))


def test_empty_and_degenerate_inputs(T, oracle):
    V, F = W.noisy_icosphere(2, 151)
    bvh = T.MeshBvh(dev(V), dev(F))
    assert len(bvh.ray_intersects(np.zeros((0, 3), np.float32), np.zeros((0, 3), np.float32))) == 0
    assert len(bvh.visibility(np.zeros((0, 3), np.float32))) == 0
    assert T.random_sphere(3, 0).shape == (0, 3)
    # zero directions and origins on vertices
    O = np.concatenate([V[:100], np.zeros((10, 3), np.float32)])
    D = np.concatenate([np.zeros((50, 3), np.float32), -V[50:100], np.ones((10, 3), np.float32)])
    hit = bvh.ray_intersects(dev(O), dev(D)).cpu().numpy()
    rt, _ = oracle.MeshIndex(V, F).ray_contract(O, D)
    assert np.array_equal(hit, rt >= 0)


def test_long_random_streams_run_in_parallel_chunks(T, oracle):
    """Streams of 1,024 twists or more run as parallel chunks from jump-ahead start states; they must equal the
    sequential stream word for word, at chunk boundaries and past them."""
    for seed in (3, 0xFFFF):
        got = T.random_sphere(seed, 1000000)
        assert np.array_equal(got, oracle.random_sphere(seed, 1000000)), seed
    V, F = W.noisy_icosphere(3, 12)
    for n in (212992, 212993, 400000):  # 3n words: exactly 1,024 twists, one word more, several chunks
        pos, nrm, face = T.sample_evenly_by_area(V, F, n, 77)
        rpos, rnrm, rface = oracle.sample_by_area(V, F, n, 77)
        assert np.array_equal(np.asarray(pos), rpos) and np.array_equal(np.asarray(face), rface), n
