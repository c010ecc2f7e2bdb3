"""GPU parity: every query of the CUDA path against the CPU oracle on the same seeded inputs.

Bar: element indices bit-exact under the lowest-index tie rule; squared distances, distances, closest points and hit
times bit-exact too (the kernels evaluate the reference's FP32 expressions in the same order, without fused multiply-add),
which is stricter than the 1e-6 relative tolerance the contract states (REL_TOL below, used where a value is derived).
Against the reference-mode oracle (the reference's own kd-tree traversal, ties to the first element found), the GPU's
element must achieve the same bit-identical distance or hit time.
"""

import os

import numpy as np
import pytest

from thea_gb300 import workloads as W

pytestmark = pytest.mark.gpu

REL_TOL = 1e-6


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


def load(golden_dir, name):
    return np.load(os.path.join(golden_dir, name + ".npz"))


# ---------------------------------------------------------------------------------------------------------------------
# closest element
# ---------------------------------------------------------------------------------------------------------------------

@pytest.mark.parametrize("width,leaf", [(4, 0), (8, 0), (4, 1), (4, 16), (8, 7)])
def test_closest_golden(T, golden_dir, width, leaf):
    z = load(golden_dir, "closest")
    bvh = T.MeshBvh(dev(z["V"]), dev(z["F"]), width=width, max_leaf_size=leaf)
    idx, dist, cp = bvh.closest_element(dev(z["Q"]))
    idx, dist, cp = host(idx), host(dist), host(cp)
    assert np.array_equal(idx, z["index"])
    assert np.array_equal(dist, np.sqrt(z["d2"]))
    assert np.array_equal(cp, z["cp"])
    # reference mode: same distance (the reference returns sqrt(mad) in double; ours is the float rounding of it)
    assert np.array_equal(dist, z["ref_dist"].astype(np.float32))
    bi, bd, _ = bvh.closest_element(dev(z["Q"]), dist_bound=float(z["bound"]))
    assert np.array_equal(host(bi), z["bound_index"])
    assert bvh.info()["device_error_bits"] == 0


def test_closest_host_and_device_paths_agree(T, golden_dir):
    z = load(golden_dir, "closest")
    bvh_h = T.MeshBvh(z["V"], z["F"])  # host arrays: staged copies
    i1, d1, c1 = bvh_h.closest_element(z["Q"])
    assert np.array_equal(i1, z["index"]) and np.array_equal(c1, z["cp"])
    bvh_d = T.MeshBvh(dev(z["V"]), dev(z["F"]))
    i2, d2, c2 = bvh_d.closest_element(dev(z["Q"]))
    assert np.array_equal(i1, host(i2)) and np.array_equal(d1, host(d2))


def test_closest_reduced_config0_against_oracle(T, oracle):
    V, F = W.noisy_icosphere(4, 21)
    Q = W.uniform_box_points(30000, [-1.5] * 3, [1.5] * 3, 22)
    Q = np.concatenate([Q, V, (V * np.float32(0.999)).astype(np.float32)])
    bvh = T.MeshBvh(dev(V), dev(F))
    idx, dist, cp = bvh.closest_element(dev(Q))
    m = oracle.MeshIndex(V, F)
    ri, rd2, rcp = m.closest_contract(Q)
    assert np.array_equal(host(idx), ri)
    assert np.array_equal(host(dist), np.sqrt(rd2.astype(np.float32)))
    assert np.array_equal(host(cp), rcp.astype(np.float32))


def test_closest_full_config0_subset(T, oracle):
    V, F, Q = W.config0()
    bvh = T.MeshBvh(dev(V), dev(F))
    idx, dist, cp = bvh.closest_element(dev(Q))
    idx, dist, cp = host(idx), host(dist), host(cp)
    assert len(F) == 81920 and len(Q) == 262144
    sel = np.random.default_rng(0).choice(len(Q), 12000, replace=False)
    m = oracle.MeshIndex(V, F)
    ri, rd2, rcp = m.closest_contract(Q[sel])
    assert np.array_equal(idx[sel], ri)
    assert np.array_equal(cp[sel], rcp.astype(np.float32))
    # size-independent property over all queries: the reported closest point is at the reported distance
    d_check = np.sqrt(np.sum((cp.astype(np.float64) - Q) ** 2, 1))
    assert np.max(np.abs(d_check - dist) / np.maximum(dist, 1e-12)) < 1e-5
    assert np.all(idx >= 0)


def test_closest_dist_bounds_and_edges(T, oracle):
    V, F = W.noisy_icosphere(3, 31)
    Q = W.uniform_box_points(5000, [-2] * 3, [2] * 3, 32)
    bvh = T.MeshBvh(dev(V), dev(F))
    for b in (0.0, 0.01, 0.3, 1.0):
        idx, dist, _ = bvh.closest_element(dev(Q), dist_bound=b)
        ri, rd2, _ = oracle.closest_brute(V, F, Q, dist_bound=b)
        assert np.array_equal(host(idx), ri)
        d = host(dist)
        assert np.all(d[ri < 0] == -1.0)
    # empty query set
    i0, d0, c0 = bvh.closest_element(dev(np.zeros((0, 3), np.float32)))
    assert i0.numel() == 0


def test_closest_single_triangle_and_degenerates(T, oracle):
    Vd = np.array([[0, 0, 0], [1, 0, 0], [2, 0, 0], [0, 1, 0], [0, 0, 0], [0, 0, 1]], np.float32)
    Fd = np.array([[0, 1, 2], [0, 4, 3], [0, 1, 3], [1, 3, 5]], np.int32)
    Q = W.uniform_box_points(3000, [-1] * 3, [2] * 3, 33)
    for V, F in ((Vd[:4], Fd[2:3]), (Vd, Fd)):
        bvh = T.MeshBvh(V, F)
        idx, dist, cp = bvh.closest_element(Q)
        ri, rd2, rcp = oracle.closest_brute(V, F, Q)
        assert np.array_equal(idx, ri)
        assert np.array_equal(cp, rcp.astype(np.float32))


# ---------------------------------------------------------------------------------------------------------------------
# ray first hit
# ---------------------------------------------------------------------------------------------------------------------

@pytest.mark.parametrize("width,leaf", [(4, 0), (8, 0), (4, 1), (8, 16)])
def test_ray_golden(T, golden_dir, width, leaf):
    z = load(golden_dir, "ray")
    bvh = T.MeshBvh(dev(z["V"]), dev(z["F"]), width=width, max_leaf_size=leaf)
    t, idx, nrm = bvh.ray_structure_intersection(dev(z["O"]), dev(z["D"]), normals=True)
    t, idx, nrm = host(t), host(idx), host(nrm)
    assert np.array_equal(idx, z["index"])
    assert np.array_equal(t, z["time"])
    assert np.array_equal(t, z["ref_time"])  # reference mode: same hit time
    same = idx == z["ref_index"]
    assert np.array_equal(nrm[same], z["ref_normal"][same])
    bt, bi, _ = bvh.ray_structure_intersection(dev(z["O"]), dev(z["D"]), max_time=float(z["max_time"]))
    assert np.array_equal(host(bi), z["bound_index"]) and np.array_equal(host(bt), z["bound_time"])


def test_ray_random_sphere_rays(T, oracle):
    V, F = W.noisy_icosphere(3, 41)
    o, d = W.random_rays(20000, [-2] * 3, [2] * 3, 42)
    bvh = T.MeshBvh(dev(V), dev(F))
    t, idx, _ = bvh.ray_structure_intersection(dev(o), dev(d))
    rt, ri = oracle.ray_brute(V, F, o, d)
    assert np.array_equal(host(idx), ri)
    assert np.array_equal(host(t), rt.astype(np.float32))


@pytest.mark.parametrize("max_time", [-1.0, 1.2])
def test_ray_large_batches_equal_small_ones(T, max_time):
    # batches of 65,536 rays or more run on persistent lanes that take a new ray when theirs is done; smaller ones run
    # one thread per ray: the same traversal, the same results (times, indices, normals)
    V, F = W.noisy_icosphere(4, 43)
    o, d = W.random_rays(150000, [-2] * 3, [2] * 3, 44)
    bvh = T.MeshBvh(dev(V), dev(F))
    t, idx, nrm = bvh.ray_structure_intersection(dev(o), dev(d), max_time=max_time, normals=True)
    parts = [bvh.ray_structure_intersection(dev(o[i:i + 50000]), dev(d[i:i + 50000]), max_time=max_time, normals=True)
             for i in range(0, len(o), 50000)]
    assert np.array_equal(host(t), np.concatenate([host(p[0]) for p in parts]))
    assert np.array_equal(host(idx), np.concatenate([host(p[1]) for p in parts]))
    assert np.array_equal(host(nrm), np.concatenate([host(p[2]) for p in parts]))


def test_ray_full_config1_subset(T, oracle):
    V, F, o, d = W.config1()
    assert len(F) == 2093058 and len(o) == 4194304
    bvh = T.MeshBvh(dev(V), dev(F), layouts=2)
    t, idx, _ = bvh.ray_structure_intersection(dev(o), dev(d))
    t, idx = host(t), host(idx)
    sel = np.random.default_rng(1).choice(len(o), 40000, replace=False)
    m = oracle.MeshIndex(V, F)
    rt, ri = m.ray_contract(o[sel], d[sel])
    assert np.array_equal(idx[sel], ri)
    assert np.array_equal(t[sel], rt.astype(np.float32))
    # size-independent: every hit point lies on its triangle's plane, every miss reports -1 for both outputs
    hit = idx >= 0
    assert np.array_equal(t < 0, ~hit)
    P = o[hit].astype(np.float64) + t[hit, None].astype(np.float64) * d[hit]
    tri = V[F[idx[hit]]].astype(np.float64)
    n = np.cross(tri[:, 1] - tri[:, 0], tri[:, 2] - tri[:, 0])
    n /= np.linalg.norm(n, axis=1, keepdims=True)
    assert np.max(np.abs(np.sum((P - tri[:, 0]) * n, 1))) < 1e-5


def test_ray_host_staging_many_chunks(T, oracle):
    V, F = W.heightfield(128, 51)
    o, d = W.cosine_rays_down(600000, 52)  # several staging chunks
    bvh = T.MeshBvh(V, F)
    t, idx, _ = bvh.ray_structure_intersection(o, d)
    bvh_d = T.MeshBvh(dev(V), dev(F))
    t2, i2, _ = bvh_d.ray_structure_intersection(dev(o), dev(d))
    assert np.array_equal(idx, host(i2)) and np.array_equal(t, host(t2))
    sel = np.arange(0, len(o), 37)
    rt, ri = oracle.MeshIndex(V, F).ray_contract(o[sel], d[sel])
    assert np.array_equal(idx[sel], ri)


# ---------------------------------------------------------------------------------------------------------------------
# sampling and k nearest neighbours
# ---------------------------------------------------------------------------------------------------------------------

def test_sampler_bit_exact_with_reference_stream(T, golden_dir, oracle):
    z = load(golden_dir, "sample_knn")
    pos, nrm, face = T.sample_evenly_by_area(dev(z["V"]), dev(z["F"]), len(z["pos"]), int(z["seed"]))
    assert np.array_equal(host(pos), z["pos"])
    assert np.array_equal(host(nrm), z["nrm"])
    assert np.array_equal(host(face), z["face"])
    # longer stream (many twists) on the config-0 mesh
    V, F, _ = W.config0()
    p2, n2, f2 = T.sample_evenly_by_area(V, F, 200000, 77)
    rp, rn, rf = oracle.sample_by_area(V, F, 200000, 77)
    assert np.array_equal(p2, rp) and np.array_equal(f2, rf) and np.array_equal(n2, rn)


def test_sampler_areas_spanning_many_binades(T, oracle):
    # triangles from 1e-12 to 1e+6 in area: the cumulative FP64 sum rounds, so the parallel exact sum must hand over to
    # the sequential one; both sample streams stay bit-identical to the oracle
    rng = np.random.default_rng(8)
    tris = []
    for s in 10.0 ** rng.uniform(-6, 3, 3000):
        c = rng.uniform(-100, 100, 3)
        tris.append(c + s * rng.normal(size=(3, 3)))
    V = np.concatenate(tris).astype(np.float32)
    F = np.arange(len(V), dtype=np.int32).reshape(-1, 3)
    for rng_mode in ("thea", "counter"):
        p, n, f = T.sample_evenly_by_area(V, F, 50000, 13, rng=rng_mode)
        if rng_mode == "thea":
            rp, rn, rf = oracle.sample_by_area(V, F, 50000, 13)
            assert np.array_equal(p, rp) and np.array_equal(f, rf) and np.array_equal(n, rn)
        else:
            assert len(p) == 50000 and np.all(f >= 0)


def test_sampler_counter_mode_distribution(T, oracle):
    V, F = W.noisy_icosphere(2, 61)
    p, n, f = T.sample_evenly_by_area(V, F, 200000, 5, rng="counter")
    _, _, _, area = oracle.triangle_props(V[F].reshape(-1, 9))
    counts = np.bincount(f, minlength=len(F))
    expected = len(f) * area / area.sum()
    assert np.sum((counts - expected) ** 2 / expected) < 2.0 * len(F)
    nrm, dist, _, _ = oracle.triangle_props(V[F[f]].reshape(-1, 9))
    assert np.max(np.abs(np.sum(p * nrm, 1) - dist)) < 1e-5


def test_sampler_zero_area(T):
    V = np.zeros((3, 3), np.float32)
    F = np.array([[0, 1, 2]], np.int32)
    p, n, f = T.sample_evenly_by_area(V, F, 10, 1)
    assert len(p) == 0


def test_knn_golden_self_graph(T, golden_dir):
    z = load(golden_dir, "sample_knn")
    pb = T.PointBvh(dev(z["pos"]))
    ki, kd = pb.k_closest_self(8, device=True)
    assert np.array_equal(host(ki), z["knn_index"])
    assert np.array_equal(host(kd), z["knn_d2"])
    assert np.array_equal(host(kd).astype(np.float64), z["ref_knn_d2"])  # reference mode: same distances
    # the general query path with an explicit exclusion gives the same graph
    qi, qd = pb.k_closest_pairs(dev(z["pos"]), 8, exclude=dev(np.arange(len(z["pos"]), dtype=np.int32)))
    assert np.array_equal(host(qi), z["knn_index"])


@pytest.mark.parametrize("k", [1, 2, 3, 5, 8, 16, 17, 32])
def test_knn_against_brute_force(T, oracle, k):
    P = W.uniform_box_points(20000, [0] * 3, [1] * 3, 71)
    P[1000:1050] = P[7]  # duplicates: exact ties
    Q = np.concatenate([P[:2000], W.uniform_box_points(2000, [-0.3] * 3, [1.3] * 3, 72)])
    ex = np.concatenate([np.arange(2000, dtype=np.int32), -np.ones(2000, np.int32)])
    pb = T.PointBvh(dev(P), max_leaf_size=8 if k != 17 else 3)
    ki, kd = pb.k_closest_pairs(dev(Q), k, exclude=dev(ex))
    pi = oracle.PointIndex(P)
    ri, rd = pi.knn_contract(Q, k, exclude=ex)
    assert np.array_equal(host(ki), ri)
    assert np.array_equal(host(kd), rd.astype(np.float32))


def test_knn_bounds_and_small_sets(T, oracle):
    P = W.uniform_box_points(50, [0] * 3, [1] * 3, 81)
    Q = W.uniform_box_points(100, [0] * 3, [1] * 3, 82)
    pb = T.PointBvh(P)
    ki, kd = pb.k_closest_pairs(Q, 32, dist_bound=0.3)
    ri, rd = oracle.knn_brute(P, Q, 32, dist_bound=0.3)
    assert np.array_equal(ki, ri)
    assert np.all(kd[ri < 0] == -1.0)
    one = T.PointBvh(P[:1])
    ki, kd = one.k_closest_pairs(Q, 4)
    assert np.all(ki[:, 0] == 0) and np.all(ki[:, 1:] == -1)


def test_knn_reduced_config2(T, oracle):
    V, F, _ = W.config0()
    pos, _, _ = T.sample_evenly_by_area(dev(V), dev(F), 100000, 2024)
    pb = T.PointBvh(pos)
    ki, kd = pb.k_closest_self(16, device=True)
    ki, kd = host(ki), host(kd)
    P = host(pos)
    sel = np.random.default_rng(3).choice(len(P), 5000, replace=False)
    pi = oracle.PointIndex(P)
    ri, rd = pi.knn_contract(P[sel], 16, exclude=sel.astype(np.int32))
    assert np.array_equal(ki[sel], ri)
    assert np.array_equal(kd[sel], rd.astype(np.float32))
    # sortedness and self-exclusion hold for every row
    assert np.all(np.diff(kd, axis=1) >= 0)
    assert not np.any(ki == np.arange(len(P))[:, None])


# ---------------------------------------------------------------------------------------------------------------------
# the reference's TestBvh scenario
# ---------------------------------------------------------------------------------------------------------------------

def test_reference_testbvh_scenario(T, golden_dir):
    z = load(golden_dir, "testbvh")
    pb = T.PointBvh(z["points"])
    ki, kd = pb.k_closest_pairs(z["query"], 3, dist_bound=0.25)
    assert np.array_equal(ki, z["knn3_index"]) and np.array_equal(kd, z["knn3_d2"])
    tb = T.MeshBvh(z["tri_vertices"], z["tri_faces"])
    ti, td, tcp = tb.closest_element(z["query"], dist_bound=0.25)
    assert np.array_equal(ti, z["tri_index"]) and np.array_equal(tcp, z["tri_cp"])
    assert abs(float(td[0]) - float(z["ref_tri_dist"][0])) <= REL_TOL * float(z["ref_tri_dist"][0])
    t, i, n = tb.ray_structure_intersection(np.zeros((1, 3), np.float32), z["ray_dir"][None], normals=True)
    assert np.array_equal(i, z["ray_index"]) and np.array_equal(t, z["ray_time"])
    assert np.array_equal(n, z["ref_ray_normal"])


def test_cpp_wrapper_on_device(T):
    # the header-only C++ wrapper drives the library end to end: closest point, ray, k-NN on a tetrahedron
    import subprocess
    from tests.conftest import ROOT
    src = os.path.join(ROOT, "tests", "cpp", "wrapper_compile.cpp")
    out = os.path.join(ROOT, "tests", "cpp", "_build", "wrapper_device")
    os.makedirs(os.path.dirname(out), exist_ok=True)
    r = subprocess.run(["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"), src, "-o", out,
                        "-L", os.path.join(ROOT, "thea_gb300", "_lib"), "-lthea_gpu",
                        "-Wl,-rpath," + os.path.join(ROOT, "thea_gb300", "_lib")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([out], capture_output=True, text=True)
    assert r.returncode == 0 and "wrapper ok" in r.stdout, r.stdout + r.stderr


@pytest.mark.parametrize("radius", [0.0, 0.03, 0.12])
def test_radius_neighbors_equal_brute_force(T, oracle, radius):
    import torch
    P = W.uniform_box_points(20000, [0] * 3, [1] * 3, 81)
    P[1000:1040] = P[7]  # duplicates: zero distances
    Q = np.concatenate([P[:3000], W.uniform_box_points(2000, [-0.2] * 3, [1.2] * 3, 82)])
    ex = np.concatenate([np.arange(1500, dtype=np.int32), -np.ones(3500, np.int32)])
    pb = T.PointBvh(dev(P), max_leaf_size=4)
    off, idx, d2 = pb.radius_neighbors(dev(Q), radius, exclude=dev(ex))
    roff, ridx, rd2 = oracle.range_brute(P, Q, radius, exclude=ex)
    assert np.array_equal(host(off), roff)
    assert np.array_equal(host(idx), ridx)
    assert np.array_equal(host(d2), rd2)
    assert pb.info()["device_error_bits"] == 0
    # the same on a k-NN graph's surface samples without exclusions
    if radius == 0.03:
        V, F, _ = W.config0()
        pos, _, _ = T.sample_evenly_by_area(dev(V), dev(F), 30000, 4)
        pb2 = T.PointBvh(pos)
        off, idx, d2 = pb2.radius_neighbors(pos[:5000], 0.01)
        roff, ridx, rd2 = oracle.range_brute(host(pos), host(pos[:5000]), 0.01)
        assert np.array_equal(host(off), roff) and np.array_equal(host(idx), ridx)


@pytest.mark.parametrize("dist_bound", [-1.0, 0.05])
def test_closest_large_batches_equal_small_ones(T, dist_bound):
    # batches of 65,536 queries or more run as persistent lanes with a step budget plus one warp per query over budget;
    # smaller ones run one thread per query: the same searches, the same results
    V, F = W.noisy_icosphere(5, 45)
    Q = W.uniform_box_points(150000, [-1.5] * 3, [1.5] * 3, 46)
    bvh = T.MeshBvh(dev(V), dev(F))
    i, d, c = bvh.closest_element(dev(Q), dist_bound=dist_bound)
    parts = [bvh.closest_element(dev(Q[k:k + 50000]), dist_bound=dist_bound) for k in range(0, len(Q), 50000)]
    assert np.array_equal(host(i), np.concatenate([host(p[0]) for p in parts]))
    assert np.array_equal(host(d), np.concatenate([host(p[1]) for p in parts]))
    assert np.array_equal(host(c), np.concatenate([host(p[2]) for p in parts]))


def test_ray_pinned_host_arrays_are_read_in_place(T):
    """Rays and results in pinned host memory take the one-launch path that reads and writes them in place; results
    equal the device-resident call's, for a batch that is not a multiple of the 64-ray block, with and without the index
    output and with a time bound."""
    import ctypes
    import torch
    from thea_gb300 import _native as N
    V, F = W.heightfield(256, 301)
    o, d = W.cosine_rays_down(200003, 302)
    n = len(o)
    bvh = T.MeshBvh(dev(V), dev(F), layouts=2)
    L = N.lib()
    ho, hd = torch.from_numpy(o).pin_memory(), torch.from_numpy(d).pin_memory()
    ptr = lambda x: ctypes.c_void_p(x.data_ptr()) if x is not None else None  # noqa: E731
    for max_time, with_index in ((-1.0, True), (0.3, True), (-1.0, False)):
        t_dev, i_dev, _ = bvh.ray_structure_intersection(dev(o), dev(d), max_time=max_time)
        ht = torch.full((n,), 7.0).pin_memory()
        hi = torch.full((n,), 7, dtype=torch.int32).pin_memory() if with_index else None
        N.check(L.thea_ray_intersection(bvh.handle, ptr(ho), ptr(hd), n, max_time, ptr(ht), ptr(hi), None,
                                        ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)))
        assert torch.equal(ht, t_dev.cpu())
        if with_index:
            assert torch.equal(hi, i_dev.cpu())
    # pageable arrays take the staged path and agree too
    t_h, i_h, _ = bvh.ray_structure_intersection(o, d)
    t_dev, i_dev, _ = bvh.ray_structure_intersection(dev(o), dev(d))
    assert np.array_equal(t_h, t_dev.cpu().numpy()) and np.array_equal(i_h, i_dev.cpu().numpy())


def test_non_finite_and_huge_inputs(T, oracle):
    """NaN, infinite and huge coordinates in queries and rays end like the oracle's traversal (no element where no
    comparison can succeed), without stalling a kernel."""
    V, F = W.noisy_icosphere(3, 71)
    Q = W.uniform_box_points(2000, [-1.5] * 3, [1.5] * 3, 72)
    Q[::50] = np.nan
    Q[1::50] = np.inf
    Q[2::50, 0] = -np.inf
    Q[3::50] = 1e30
    Q[4::50, 1] = np.nan
    bvh = T.MeshBvh(dev(V), dev(F))
    idx, dist, cp = bvh.closest_element(dev(Q))
    ri, rd2, rcp = oracle.MeshIndex(V, F).closest_contract(Q)
    idx, dist = host(idx), host(dist)
    assert np.array_equal(idx, ri)
    ok = ri >= 0
    assert np.array_equal(dist[ok], np.sqrt(rd2[ok].astype(np.float32)))
    O, D = W.random_rays(2000, [-2] * 3, [2] * 3, 73)
    O[::40] = np.nan
    D[1::40] = np.nan
    D[2::40] = 0.0
    D[3::40] = np.inf
    O[4::40] = 1e30
    t, ti, _ = bvh.ray_structure_intersection(dev(O), dev(D))
    rt, rti = oracle.MeshIndex(V, F).ray_contract(O, D)
    assert np.array_equal(host(ti), rti)
    assert np.array_equal(host(t), rt.astype(np.float32))
    P = W.uniform_box_points(5000, [0] * 3, [1] * 3, 74)
    pb = T.PointBvh(dev(P))
    ki, kd = pb.k_closest_pairs(dev(Q), 4)
    rki, rkd = oracle.PointIndex(P).knn_contract(Q, 4)
    ki = host(ki)
    # a query with a NaN coordinate has no neighbours here; the reference (and the oracle) fill its list with the first
    # points their traversal admits while the list is not full, at NaN distance
    nan_rows = np.isnan(Q).any(axis=1)
    assert np.all(ki[nan_rows] == -1)
    assert np.array_equal(ki[~nan_rows], rki[~nan_rows])
    assert bvh.info()["device_error_bits"] == 0 and pb.info()["device_error_bits"] == 0


def test_closest_pinned_host_arrays_are_read_in_place(T, oracle):
    """Queries and results in pinned host memory take the in-place path (FP32, large batch); results equal the
    device-resident call's (and the oracle's on a subset), with all outputs, with the index alone and with a bound."""
    import ctypes
    import torch
    from thea_gb300 import _native as N
    V, F = W.noisy_icosphere(4, 311)
    Q = W.uniform_box_points(100003, [-1.5] * 3, [1.5] * 3, 312)
    n = len(Q)
    bvh = T.MeshBvh(dev(V), dev(F), layouts=1)
    L = N.lib()
    hq = torch.from_numpy(Q).pin_memory()
    ptr = lambda x: ctypes.c_void_p(x.data_ptr()) if x is not None else None  # noqa: E731
    for bound, all_outputs in ((-1.0, True), (0.2, True), (-1.0, False)):
        i_dev, d_dev, c_dev = bvh.closest_element(dev(Q), dist_bound=bound)
        hi = torch.full((n,), 7, dtype=torch.int32).pin_memory()
        hd = torch.full((n,), 7.0).pin_memory() if all_outputs else None
        hc = torch.full((n, 3), 7.0).pin_memory() if all_outputs else None
        N.check(L.thea_closest_element(bvh.handle, ptr(hq), n, bound, ptr(hi), ptr(hd), ptr(hc),
                                       ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)))
        assert torch.equal(hi, i_dev.cpu())
        if all_outputs:
            assert torch.equal(hd, d_dev.cpu()) and torch.equal(hc, c_dev.cpu())
    sel = np.arange(0, n, 37)
    ri, _, rcp = oracle.MeshIndex(V, F).closest_contract(Q[sel])
    assert np.array_equal(hi.numpy()[sel], ri)


def test_knn_with_pinned_host_arrays(T):
    """k-NN with pinned host arrays (query mode with exclusions, and the self graph) equals the device-resident calls."""
    import ctypes
    import torch
    from thea_gb300 import _native as N
    P = W.uniform_box_points(60000, [0] * 3, [1] * 3, 321)
    Q = W.uniform_box_points(70001, [0] * 3, [1] * 3, 322)
    ex = np.random.default_rng(323).integers(-1, len(P), size=len(Q)).astype(np.int32)
    pb = T.PointBvh(dev(P))
    L = N.lib()
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    ptr = lambda x: ctypes.c_void_p(x.data_ptr())  # noqa: E731
    ki, kd = pb.k_closest_pairs(dev(Q), 8, exclude=dev(ex))
    hq, he = torch.from_numpy(Q).pin_memory(), torch.from_numpy(ex).pin_memory()
    hi = torch.empty((len(Q), 8), dtype=torch.int32).pin_memory()
    hd = torch.empty((len(Q), 8)).pin_memory()
    N.check(L.thea_k_closest(pb.handle, ptr(hq), len(Q), 8, -1.0, ptr(he), ptr(hi), ptr(hd), st))
    assert torch.equal(hi, ki.cpu()) and torch.equal(hd, kd.cpu())
    si, sd = pb.k_closest_self(16, device=True)
    hi = torch.empty((len(P), 16), dtype=torch.int32).pin_memory()
    hd = torch.empty((len(P), 16)).pin_memory()
    N.check(L.thea_k_closest_self(pb.handle, 16, ptr(hi), ptr(hd), st))
    assert torch.equal(hi, si.cpu()) and torch.equal(hd, sd.cpu())
