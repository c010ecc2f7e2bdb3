"""Full-size parity: the benchmark configurations at their full sizes, every query checked against the oracle.

  config 0  closest point, 262,144 queries on the 81,920-triangle noisy icosphere: indices, distances and closest points
            bit-exact against the oracle's lowest-index mode; against the reference mode (the reference's kd-tree and
            traversal order), the same distance for every query; the FP64 re-check mode against the FP64 oracle
            (indices bit-exact, distances within REL_TOL).
  config 1  first hit of 4,194,304 rays on the 2,093,058-triangle heightfield: indices and hit times bit-exact, through
            device arrays and through pinned host arrays (the in-place end-to-end path).
  config 2  the k = 16 graph (self excluded) of the 1,048,576 area samples of the config-0 mesh drawn from Random(2):
            the samples bit-exact against the oracle's sampler, then every row of the graph bit-exact (indices and
            squared distances), by the traversal and by the tensor-core-seeded search.
  config 3  every 16th mesh of the 4,096-mesh batched distribution (subdivision levels 2-7, all queries of each), batched
            in one forest: FP32 bit-exact against the oracle mesh by mesh, FP64 re-check against the FP64 oracle.

These are the configurations the benchmark times; the oracle runs multi-threaded on the host.
"""

import numpy as np
import pytest

from thea_gb300 import workloads as W

pytestmark = pytest.mark.gpu

REL_TOL = 1e-6  # the stated tolerance for FP64-re-checked distances; FP32 results are compared bit for bit


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
    return t.cpu().numpy()


def test_config0_every_query(T, oracle):
    V, F, Q = W.config0()
    assert len(F) == 81920 and len(Q) == 262144
    bvh = T.MeshBvh(dev(V), dev(F), layouts=1, max_leaf_size=1)  # the benchmark's build
    idx, dist, cp = bvh.closest_element(dev(Q))
    idx, dist, cp = host(idx), host(dist), host(cp)
    m = oracle.MeshIndex(V, F)
    ri, rd2, rcp = m.closest_contract(Q)
    assert np.array_equal(idx, ri)
    assert np.array_equal(dist, np.sqrt(rd2.astype(np.float32)))
    assert np.array_equal(cp, rcp.astype(np.float32))
    # reference mode: the reference's traversal may keep another of several equidistant triangles, never a farther one
    _, fdist, _ = m.closest_ref(Q)
    assert np.array_equal(np.sqrt(rd2.astype(np.float64)), fdist)
    # FP64 re-check mode against the FP64 oracle
    i64, d64, _, _ = bvh.closest_element_ex(dev(Q), precision="fp64")
    i64, d64 = host(i64), host(d64)
    oi, od2, _ = oracle.MeshIndex(V, F, fp64=True).closest_contract(Q)
    assert np.array_equal(i64, oi)
    od = np.sqrt(od2)
    assert np.all(np.abs(d64 - od) <= REL_TOL * od)


def test_config1_every_ray(T, oracle):
    import torch
    V, F, o, d = W.config1()
    assert len(F) == 2093058 and len(o) == 4194304
    bvh = T.MeshBvh(dev(V), dev(F), layouts=2)  # the benchmark's build
    t, idx, _ = bvh.ray_structure_intersection(dev(o), dev(d))
    t, idx = host(t), host(idx)
    rt, ri = oracle.MeshIndex(V, F).ray_contract(o, d)
    assert np.array_equal(idx, ri)
    assert np.array_equal(t, rt.astype(np.float32))
    # the end-to-end path: rays and results in pinned host memory, read and written in place by the kernel
    import ctypes
    from thea_gb300 import _native as N
    ho, hd = torch.from_numpy(o).pin_memory(), torch.from_numpy(d).pin_memory()
    th = torch.empty(len(o), dtype=torch.float32).pin_memory()
    ih = torch.empty(len(o), dtype=torch.int32).pin_memory()
    p = lambda x: ctypes.c_void_p(x.data_ptr())  # noqa: E731
    N.check(N.lib().thea_ray_intersection(bvh.handle, p(ho), p(hd), len(o), -1.0, p(th), p(ih), None,
                                          ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)))
    assert np.array_equal(ih.numpy(), idx) and np.array_equal(th.numpy(), t)


def test_config2_every_row(T, oracle):
    V, F, _ = W.config0()
    pos, _, _ = T.sample_evenly_by_area(dev(V), dev(F), 1 << 20, 2)  # the benchmark's samples
    P = host(pos)
    rp, _, _ = oracle.sample_by_area(V, F, 1 << 20, 2)
    assert np.array_equal(P, rp)
    pb = T.PointBvh(pos)
    ki, kd = pb.k_closest_self(16, device=True)
    ki, kd = host(ki), host(kd)
    ri, rd = oracle.PointIndex(P).knn_contract(P, 16, exclude=np.arange(len(P), dtype=np.int32))
    assert np.array_equal(ki, ri)
    assert np.array_equal(kd, rd.astype(np.float32))
    gi, gd = pb.k_closest_self(16, device=True, candidates="gram")
    assert np.array_equal(host(gi), ki) and np.array_equal(host(gd), kd)
    assert pb.info()["device_error_bits"] == 0


def test_config3_every_16th_mesh(T, oracle):
    import torch
    from concurrent.futures import ThreadPoolExecutor
    V, F, foff, Q, qoff, levels = W.config3_torch(4096)
    qoff_h = qoff.cpu().numpy()
    meshes = np.arange(0, 4096, 16)
    assert set(levels[meshes]) == set(range(2, 8))
    sv, sf, sq, sfo, sqo, vb = [], [], [], [0], [0], 0
    for m in meshes:
        Fm = F[foff[m]:foff[m + 1]]
        lo, hi = int(Fm.min()), int(Fm.max()) + 1
        sv.append(V[lo:hi])
        sf.append(Fm - lo + vb)
        vb += hi - lo
        sq.append(Q[qoff_h[m]:qoff_h[m + 1]])
        sfo.append(sfo[-1] + Fm.shape[0])
        sqo.append(sqo[-1] + sq[-1].shape[0])
    Vs, Fs, Qs = torch.cat(sv), torch.cat(sf), torch.cat(sq)
    sfo, sqo = np.array(sfo, np.int64), np.array(sqo, np.int64)
    del V, F, Q
    forest = T.MeshForest(Vs, Fs, sfo, width=4, max_leaf_size=1, layouts=1)
    idx, dist, cp, _ = forest.batch_closest_element(Qs, dev(sqo), closest_points=True)
    i64, d64, _, _ = forest.batch_closest_element(Qs, dev(sqo), precision="fp64")
    idx, dist, cp, i64, d64 = host(idx), host(dist), host(cp), host(i64), host(d64)
    Vh, Fh, Qh = host(Vs), host(Fs), host(Qs)

    def check(j):
        Fm = Fh[sfo[j]:sfo[j + 1]]
        lo = int(Fm.min())
        Vm, Fm = Vh[lo:int(Fm.max()) + 1], Fm - lo
        Qm = Qh[sqo[j]:sqo[j + 1]]
        s = slice(sqo[j], sqo[j + 1])
        ri, rd2, rcp = oracle.MeshIndex(Vm, Fm).closest_contract(Qm, threads=2)
        oi, od2, _ = oracle.MeshIndex(Vm, Fm, fp64=True).closest_contract(Qm, threads=2)
        od = np.sqrt(od2)
        return (np.array_equal(idx[s], ri) and np.array_equal(dist[s], np.sqrt(rd2.astype(np.float32)))
                and np.array_equal(cp[s], rcp.astype(np.float32)) and np.array_equal(i64[s], oi)
                and bool(np.all(np.abs(d64[s] - od) <= REL_TOL * od)))

    with ThreadPoolExecutor(8) as ex:
        ok = list(ex.map(check, range(len(meshes))))
    bad = [int(meshes[j]) for j, g in enumerate(ok) if not g]
    assert not bad, bad
    assert forest.info()["device_error_bits"] == 0
