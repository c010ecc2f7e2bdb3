"""Generates the committed golden fixtures under tests/golden/ from the CPU oracle (oracle/).

Inputs are small and seeded; outputs are the oracle's contract-mode results (lowest index among ties) and its
reference-mode results (the reference kd-tree and traversal order). The fixtures pin the oracle against regressions and
give the GPU tests exact expected values. Outputs of the reference itself are in reference_outputs.npz
(make_ref_golden.py), which pins the oracle's reference mode to the reference's own code.

The "testbvh" fixture restates the seeded scenario of the reference's own BVH test (Code/Source/Test/TestBvh.cpp:120-126,
143-150, 318-326, 369-378, 405-407): one Random(0xFFFF) stream feeds 10,000 points, a second set of 10,000 points, 1,000
triangles, a second set of 1,000 triangles and one ray direction, in that order, three uniform01() draws per vector.
Vector3(rand01(), rand01(), rand01()) evaluates its arguments right to left under GCC on x86-64, which this script
assumes; the query point is (0.5, 0.5, 0.5) with distance bound 0.25 and the ray starts at the origin.

Run: python tests/golden/make_golden.py
"""

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from thea_gb300 import workloads as W  # noqa: E402

NORM = np.float32(2.0 ** -32)


def uniform01(bits):
    return bits.astype(np.float32) * NORM


def vec3_gcc(u):
    """Vector3(rand01(), rand01(), rand01()) with right-to-left argument evaluation."""
    u = u.reshape(-1, 3)
    return np.ascontiguousarray(u[:, ::-1])


def testbvh_scenario():
    n_pts, n_tris = 10000, 1000
    total = 3 * n_pts * 2 + 9 * n_tris * 2 + 3
    u = uniform01(O.thea_random_bits(0xFFFF, total))
    o = 0
    pts = vec3_gcc(u[o:o + 3 * n_pts]); o += 3 * n_pts
    pts2 = vec3_gcc(u[o:o + 3 * n_pts]); o += 3 * n_pts
    tv = vec3_gcc(u[o:o + 9 * n_tris]); o += 9 * n_tris
    tv2 = vec3_gcc(u[o:o + 9 * n_tris]); o += 9 * n_tris
    rd = vec3_gcc(u[o:o + 3])[0].astype(np.float64)
    rd = (rd / np.linalg.norm(rd)).astype(np.float32)
    return pts, pts2, tv, tv2, rd


def main():
    out = {}
    # --- closest point on a small noisy icosphere (320 triangles), with queries on vertices and edges for ties
    V, F = W.noisy_icosphere(2, 101)
    Q = W.uniform_box_points(600, [-1.5] * 3, [1.5] * 3, 102)
    Q = np.concatenate([Q, V[:40] * np.float32(1.25), V[40:60]]).astype(np.float32)
    m = O.MeshIndex(V, F)
    ci, cd2, ccp = m.closest_contract(Q)
    ri, rdist, rcp = m.closest_ref(Q)
    bi, bd2, bcp = m.closest_contract(Q, dist_bound=0.3)
    np.savez_compressed(os.path.join(HERE, "closest.npz"), V=V, F=F, Q=Q, index=ci, d2=cd2.astype(np.float32),
                        cp=ccp.astype(np.float32), ref_index=ri, ref_dist=rdist, ref_cp=rcp, bound=np.float32(0.3),
                        bound_index=bi, bound_d2=bd2.astype(np.float32))

    # --- first ray hit on a small heightfield, plus rays aimed at vertices (ties on shared edges)
    HV, HF = W.heightfield(24, 103)
    o, d = W.cosine_rays_down(600, 104)
    vo = np.repeat(np.array([[0.0, 0.0, 0.5]], np.float32), 40, 0)
    vo[:, :2] = HV[::13][:40, :2]
    vd = np.tile(np.array([[0.0, 0.0, -1.0]], np.float32), (40, 1))
    o = np.concatenate([o, vo]).astype(np.float32)
    d = np.concatenate([d, vd]).astype(np.float32)
    mh = O.MeshIndex(HV, HF)
    ct, cti = mh.ray_contract(o, d)
    rt, rti, rn = mh.ray_ref(o, d)
    bt, bti = mh.ray_contract(o, d, max_time=0.45)
    np.savez_compressed(os.path.join(HERE, "ray.npz"), V=HV, F=HF, O=o, D=d, time=ct.astype(np.float32), index=cti,
                        ref_time=rt, ref_index=rti, ref_normal=rn, max_time=np.float32(0.45),
                        bound_time=bt.astype(np.float32), bound_index=bti)

    # --- area sampling with Random(seed), then the k-NN graph of the samples (k = 8, excluding self)
    pos, nrm, face = O.sample_by_area(V, F, 1500, 105)
    pidx = O.PointIndex(pos)
    ex = np.arange(len(pos), dtype=np.int32)
    ki, kd = pidx.knn_contract(pos, 8, exclude=ex)
    kri, krd = pidx.knn_ref(pos, 8, exclude=ex)
    np.savez_compressed(os.path.join(HERE, "sample_knn.npz"), V=V, F=F, seed=np.uint32(105), pos=pos, nrm=nrm, face=face,
                        knn_index=ki, knn_d2=kd.astype(np.float32), ref_knn_index=kri, ref_knn_d2=krd)

    # --- the reference's TestBvh scenario
    pts, pts2, tv, tv2, rd = testbvh_scenario()
    TF = np.arange(3 * len(tv) // 3, dtype=np.int32).reshape(-1, 3)
    q = np.array([[0.5, 0.5, 0.5]], np.float32)
    pi = O.PointIndex(pts)
    p_ref_i, p_ref_d2 = pi.knn_ref(q, 3, dist_bound=0.25)
    p_con_i, p_con_d2 = pi.knn_contract(q, 3, dist_bound=0.25)
    tm = O.MeshIndex(tv, TF)
    t_ci, t_cd2, t_ccp = tm.closest_contract(q, dist_bound=0.25)
    t_ri, t_rd, t_rcp = tm.closest_ref(q, dist_bound=0.25)
    ro = np.zeros((1, 3), np.float32)
    r_ct, r_ci = tm.ray_contract(ro, rd[None])
    r_rt, r_ri, r_rn = tm.ray_ref(ro, rd[None])
    np.savez_compressed(os.path.join(HERE, "testbvh.npz"), points=pts, points2=pts2, tri_vertices=tv, tri_faces=TF,
                        tri_vertices2=tv2, ray_dir=rd, query=q, knn3_index=p_con_i, knn3_d2=p_con_d2.astype(np.float32),
                        ref_knn3_index=p_ref_i, ref_knn3_d2=p_ref_d2, tri_index=t_ci, tri_d2=t_cd2.astype(np.float32),
                        tri_cp=t_ccp.astype(np.float32), ref_tri_index=t_ri, ref_tri_dist=t_rd, ref_tri_cp=t_rcp,
                        ray_time=r_ct.astype(np.float32), ray_index=r_ci, ref_ray_time=r_rt, ref_ray_index=r_ri,
                        ref_ray_normal=r_rn)

    # --- Thea Random stream (seed 5489 and 0xFFFF), first 2,000 words
    np.savez_compressed(os.path.join(HERE, "random.npz"), seed_5489=O.thea_random_bits(5489, 2000),
                        seed_ffff=O.thea_random_bits(0xFFFF, 2000))
    print("wrote fixtures to", HERE)


if __name__ == "__main__":
    main()
