"""GPU parity of the sample proximity graph (PointSet3::updateGraph without oversampling, Algorithms/PointSet3.hpp:324-391
and :586-702, with Random(seed) in place of Random::common()): neighbours, separations, degrees and both mean separations
bit-exact against the oracle's brute-force restatement, with and without normals and the reachability test."""

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


def same(got, ref):
    for g, r in zip(got[:3], ref[:3]):
        g = g.cpu().numpy() if hasattr(g, "cpu") else g
        assert np.array_equal(g, r)
    assert got[3] == ref[3]


def sphere_samples(n, seed, T):
    V, F = W.noisy_icosphere(4, seed)
    pos, nrm, _ = T.sample_evenly_by_area(V, F, n, seed + 1)
    return V, F, np.asarray(pos), np.asarray(nrm)


@pytest.mark.parametrize("max_degree", [8, 3, 12])
def test_graph_without_normals(T, oracle, max_degree):
    _, _, P, _ = sphere_samples(3000, 201, T)
    got = T.sample_graph(dev(P), max_degree=max_degree, seed=4)
    same(got, oracle.sample_graph(P, None, max_degree, 4))


def test_graph_with_normals_and_surface(T, oracle):
    V, F, P, Nm = sphere_samples(3000, 211, T)
    surf = T.MeshBvh(dev(V), dev(F))
    got = T.sample_graph(P, Nm, max_degree=8, seed=5, surface=surf)  # host arrays
    same(got, oracle.sample_graph(P, Nm, 8, 5, surface=oracle.MeshIndex(V, F)))
    same(T.sample_graph(dev(P), dev(Nm), max_degree=8, seed=5), oracle.sample_graph(P, Nm, 8, 5))


def test_reachability_blocks_edges_through_a_wall(T, oracle):
    # a floor (z = 0) split by a wall at x = 0.5, higher than any lift (5 x separation); samples on the floor with
    # upward normals
    V = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0],
                  [0.5, 0, 0], [0.5, 1, 0], [0.5, 1, 5.0], [0.5, 0, 5.0]], np.float32)
    F = np.array([[0, 1, 2], [0, 2, 3], [4, 5, 6], [4, 6, 7]], np.int32)
    rng = np.random.default_rng(221)
    P = np.concatenate([rng.uniform([0.05, 0, 0], [0.49, 1, 0], size=(700, 3)),
                        rng.uniform([0.51, 0, 0], [0.95, 1, 0], size=(700, 3))]).astype(np.float32)
    Nm = np.tile(np.array([[0, 0, 1]], np.float32), (len(P), 1))
    surf = T.MeshBvh(dev(V), dev(F))
    got = T.sample_graph(dev(P), dev(Nm), max_degree=8, seed=6, surface=surf)
    same(got, oracle.sample_graph(P, Nm, 8, 6, surface=oracle.MeshIndex(V, F)))
    nbr = got[0].cpu().numpy()
    left = P[:, 0] < 0.5
    cross = [(i, j) for i in range(len(P)) for j in nbr[i] if j >= 0 and left[i] != left[j]]
    assert not cross
    free = T.sample_graph(dev(P), dev(Nm), max_degree=8, seed=6)[0].cpu().numpy()
    assert any(left[i] != left[j] for i in range(len(P)) for j in free[i] if j >= 0)


def test_graph_file_format(T, oracle, tmp_path):
    _, _, P, _ = sphere_samples(500, 231, T)
    nbr, sep, deg, _ = T.sample_graph(P, max_degree=6, seed=7)
    path = tmp_path / "graph.txt"
    T.write_sample_graph(str(path), nbr, sep, deg, 6)
    lines = path.read_text().splitlines()
    assert lines[0] == "6" and len(lines) == 501
    rn, rs, rd, _ = oracle.sample_graph(P, None, 6, 7)
    for i in (0, 17, 499):
        k = int(rd[i])
        want = " ".join([str(k)] + [str(x) for x in rn[i, :k]] + ["%g" % x for x in rs[i, :k]])
        assert lines[i + 1] == want


def test_graph_with_duplicate_samples(T, oracle):
    """Coincident samples (separation 0, where fastSqrt gives a tiny positive value) and a small set."""
    _, _, P, _ = sphere_samples(600, 241, T)
    P = np.concatenate([P, P[:50], P[:5]]).astype(np.float32)
    got = T.sample_graph(dev(P), max_degree=8, seed=8)
    same(got, oracle.sample_graph(P, None, 8, 8))
    tiny = P[:6]
    same(T.sample_graph(tiny, max_degree=4, seed=1), oracle.sample_graph(tiny, None, 4, 1))


@pytest.mark.parametrize("max_degree", [8, 4])
def test_oversampled_graph(T, oracle, max_degree):
    """PointSet3 with a dense oversampling: the graph over samples + dense samples, then each sample's first
    max_degree samples along shortest paths (extractOriginalAdjacencies), bit-exact against the oracle's Dijkstra."""
    V, F, P, _ = sphere_samples(800, 251, T)
    D, _, _ = T.sample_evenly_by_area(V, F, 4000, 253)
    D = np.asarray(D)
    got = T.sample_graph(dev(P), max_degree=max_degree, seed=9, dense_positions=dev(D))
    same(got, oracle.sample_graph_oversampled(P, None, D, None, max_degree, 9))
    # the new separations are path lengths: never below the straight-line separation of the plain graph's metric
    nbr, sep = got[0].cpu().numpy(), got[1].cpu().numpy()
    i = np.repeat(np.arange(len(P)), max_degree).reshape(len(P), max_degree)
    ok = nbr >= 0
    straight = np.linalg.norm(P[i[ok]].astype(np.float64) - P[nbr[ok]], axis=1)
    assert np.all(sep[ok] >= straight * (1 - 5e-3))  # Math::fastSqrt is a one-step approximation


def test_oversampled_graph_with_normals_and_surface(T, oracle):
    V, F, P, Nm = sphere_samples(600, 261, T)
    D, DN, _ = T.sample_evenly_by_area(V, F, 2400, 263)
    D, DN = np.asarray(D), np.asarray(DN)
    surf = T.MeshBvh(dev(V), dev(F))
    got = T.sample_graph(P, Nm, max_degree=8, seed=10, surface=surf, dense_positions=D, dense_normals=DN)  # host
    same(got, oracle.sample_graph_oversampled(P, Nm, D, DN, 8, 10, surface=oracle.MeshIndex(V, F)))
    with pytest.raises(T.TheaError):
        T.sample_graph(P, Nm, max_degree=8, seed=10, dense_positions=D)  # dense normals are needed with normals
