"""GPU tests of forests and batched queries (one persistent launch over many meshes), CUDA-graph replay and the
autotuner, against the oracle applied mesh by mesh."""

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


@pytest.fixture(scope="module")
def batch():
    # 40 meshes, subdivision 1..4 (80 to 5,120 triangles), 100..3,000 queries each
    return W.config3_numpy(40, seed=123, min_level=1, max_level=4, min_q=100, max_q=3000)


def dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t):
    import torch
    torch.cuda.synchronize()
    return t.cpu().numpy()


def per_mesh(batch, fn):
    V, F, foff, Q, qoff, _ = batch
    outs = []
    for m in range(len(foff) - 1):
        Fm = F[foff[m]:foff[m + 1]]
        vlo = Fm.min()
        Vm = V[vlo:Fm.max() + 1]
        outs.append(fn(Vm, Fm - vlo, Q[qoff[m]:qoff[m + 1]]))
    return outs


# budget: 0 = default two-phase search, -1 = one thread per query throughout, 3 = nearly every query finishes on a warp
@pytest.mark.parametrize("width,leaf,qpw,budget", [(4, 0, 0, 0), (8, 2, 32, -1), (4, 1, 128, 3), (8, 4, 64, 3)])
def test_batch_closest_matches_per_mesh_oracle(T, oracle, batch, width, leaf, qpw, budget):
    V, F, foff, Q, qoff, _ = batch
    forest = T.MeshForest(dev(V), dev(F), foff, width=width, max_leaf_size=leaf, layouts=1)
    idx, dist, cp, _ = forest.batch_closest_element(dev(Q), dev(qoff), queries_per_warp=qpw, hard_query_budget=budget,
                                                    closest_points=True)
    idx, dist, cp = host(idx), host(dist), host(cp)
    ref = per_mesh(batch, lambda v, f, q: oracle.closest_brute(v, f, q))
    ri = np.concatenate([r[0] for r in ref])
    rd2 = np.concatenate([r[1] for r in ref])
    rcp = np.concatenate([r[2] for r in ref])
    assert np.array_equal(idx, ri)
    assert np.array_equal(dist, np.sqrt(rd2.astype(np.float32)))
    assert np.array_equal(cp, rcp.astype(np.float32))
    assert forest.info()["device_error_bits"] == 0


@pytest.mark.parametrize("budget", [0, -1, 3])
def test_batch_closest_fp64_matches_fp64_oracle(T, oracle, batch, budget):
    V, F, foff, Q, qoff, _ = batch
    forest = T.MeshForest(dev(V), dev(F), foff, layouts=1)
    idx, dist, _, err = forest.batch_closest_element(dev(Q), dev(qoff), precision="fp64", hard_query_budget=budget,
                                                     errors=True)
    idx, dist, err = host(idx), host(dist), host(err)
    ref = per_mesh(batch, lambda v, f, q: oracle.closest_brute(v, f, q, fp64=True))
    ri = np.concatenate([r[0] for r in ref])
    d64 = np.sqrt(np.concatenate([r[1] for r in ref]))
    assert np.array_equal(idx, ri)
    assert np.all(np.abs(dist - d64) <= 1e-6 * d64)
    assert np.all(err <= 1e-6 * d64)


def test_batch_ray_and_knn(T, oracle, batch):
    V, F, foff, Q, qoff, _ = batch
    forest = T.MeshForest(dev(V), dev(F), foff, layouts=2)
    rng = np.random.default_rng(5)
    d = rng.normal(size=Q.shape)
    d = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    t, idx = forest.batch_ray_intersection(dev(Q), dev(d), dev(qoff))
    t, idx = host(t), host(idx)
    ri, rt = [], []
    for m in range(len(foff) - 1):
        Fm = F[foff[m]:foff[m + 1]]
        vlo = Fm.min()
        tt, ii = oracle.ray_brute(V[vlo:Fm.max() + 1], Fm - vlo, Q[qoff[m]:qoff[m + 1]], d[qoff[m]:qoff[m + 1]])
        ri.append(ii)
        rt.append(tt)
    assert np.array_equal(idx, np.concatenate(ri))
    assert np.array_equal(t, np.concatenate(rt).astype(np.float32))
    # k nearest vertices: one point set per mesh (its vertices)
    voff = [0]
    for m in range(len(foff) - 1):
        voff.append(int(F[foff[m]:foff[m + 1]].max()) + 1)
    voff = np.array(voff, np.int64)
    pf = T.PointForest(dev(V), voff)
    ki, kd = pf.batch_k_closest(dev(Q), dev(qoff), 8)
    ki, kd = host(ki), host(kd)
    for m in range(len(foff) - 1):
        P = V[voff[m]:voff[m + 1]]
        bi, bd = oracle.knn_brute(P, Q[qoff[m]:qoff[m + 1]], 8)
        assert np.array_equal(ki[qoff[m]:qoff[m + 1]], bi)
        assert np.array_equal(kd[qoff[m]:qoff[m + 1]], bd.astype(np.float32))


def test_graph_capture_replays_batch(T, batch):
    import torch
    V, F, foff, Q, qoff, _ = batch
    forest = T.MeshForest(dev(V), dev(F), foff, layouts=1)
    Qd, qd = dev(Q), dev(qoff)
    n = len(Q)
    out = (torch.empty(n, dtype=torch.int32, device="cuda"), torch.empty(n, dtype=torch.float32, device="cuda"), None,
           None)
    ref_idx, ref_dist, _, _ = forest.batch_closest_element(Qd, qd)
    s = torch.cuda.Stream()
    torch.cuda.synchronize()
    with torch.cuda.stream(s):
        with T.Graph() as g:
            forest.batch_closest_element(Qd, qd, out=out)
        out[0].fill_(-7)
        for _ in range(3):
            g.launch()
    torch.cuda.synchronize()
    assert np.array_equal(host(out[0]), host(ref_idx)) and np.array_equal(host(out[1]), host(ref_dist))
    g.close()


def test_autotune_returns_a_valid_fast_config(T, batch):
    V, F, foff, Q, qoff, _ = batch
    tune = T.autotune_batch_closest(dev(V), dev(F), foff, dev(Q), dev(qoff))
    assert tune["candidates"] == 36
    assert tune["width"] in (4, 8) and tune["max_leaf_size"] in (1, 2, 4) and tune["queries_per_warp"] in (32, 64, 128)
    assert tune["hard_query_budget"] in (12, 32, 128, -1)
    assert 0 < tune["milliseconds"] < 1000
