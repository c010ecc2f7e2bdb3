"""Generates tests/golden/reference_outputs.npz from the REFERENCE's own code (oracle/_ref/libthea_ref.so).

The library compiles the reference's BvhN, Triangle3, AxisAlignedBoxN, Random and Math sources where they lie, with
oracle/ref_pin/eigen_subset.hpp standing in for Eigen (see oracle/Makefile, target `ref`). The inputs are seeded and
regenerated by the tests from thea_gb300.workloads, so the fixture holds outputs only:

  closest_*     closestElement<MetricL2> on the config-0 noisy icosphere (81,920 triangles), the first 2,048 config-0
                queries plus every 29th vertex and 400 edge midpoints (exact ties), unbounded and with bounds 0.05 / 0.3
  ray_*         rayStructureIntersection on a 128 x 128 fBm heightfield, 4,096 cosine rays, unbounded and max_time 0.45
  knn_*         kClosestPairs (k = 8) with PointSet3's self filter, 20,000 uniform points, the first 1,000 as queries
  tri_*         TriangleN<3>::closestPoint, rayIntersectionTime and squaredDistance(triangle) on random triangles,
                degenerate ones included
  pair_*        closestPair between two mesh BVHs (two noisy icospheres) in both roles
  random_*      Random(seed).bits() for three seeds; tree_depth: Math::treeDepth
  sphere_*      BestFitSphereN<3> (the reference's miniball) of seven point sets: centre and radius

Run (needs the reference sources): python tests/golden/make_ref_golden.py <the reference's Code/Source directory>
"""

import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from thea_gb300 import workloads as W  # noqa: E402


def inputs():
    """The seeded inputs of every case (shared with the tests that read the fixture)."""
    d = {}
    V, F, Q = W.config0()
    edges = np.stack([F[:, 0], F[:, 1]], 1)[::137][:400]
    d["closest"] = (V, F, np.concatenate([Q[:2048], V[::29], 0.5 * (V[edges[:, 0]] + V[edges[:, 1]])]).astype(np.float32))
    Vh, Fh = W.heightfield(128, 71)
    o, dd = W.cosine_rays_down(4096, 72)
    d["ray"] = (Vh, Fh, o, dd)
    P = W.uniform_box_points(20000, [0] * 3, [1] * 3, 73)
    P[1000:1040] = P[5]  # duplicates: exact ties
    d["knn"] = (P, P[:1000], np.arange(1000, dtype=np.int32))
    rng = np.random.default_rng(74)
    tris = rng.normal(size=(3000, 3, 3)).astype(np.float32)
    tris[:100, 2] = tris[:100, 0]  # degenerate: two equal vertices
    tris[100:200, 2] = 2 * tris[100:200, 1] - tris[100:200, 0]  # collinear
    pts = rng.normal(size=(3000, 3)).astype(np.float32) * 1.5
    pts[200:300] = tris[200:300, 1]  # on a vertex
    pts[300:400] = 0.5 * (tris[300:400, 0] + tris[300:400, 2])  # on an edge
    other = (rng.normal(size=(3000, 3, 3)) * rng.uniform(0.1, 1.5, (3000, 1, 1)) +
             rng.normal(size=(3000, 1, 3)) * rng.uniform(0, 3, (3000, 1, 1))).astype(np.float32)
    other[400:500] = tris[400:500] + np.float32(0.25) * rng.normal(size=(100, 1, 3)).astype(np.float32)
    rdir = rng.normal(size=(3000, 3)).astype(np.float32)
    d["tri"] = (tris.reshape(-1, 9), pts, other.reshape(-1, 9), rdir)
    Va, Fa = W.noisy_icosphere(3, 75)
    Vb, Fb = W.noisy_icosphere(2, 76)
    Vb = (Vb * np.float32(0.4) + np.array([1.5, 0.3, -0.2], np.float32)).astype(np.float32)
    d["pair"] = (Va, Fa, Vb, Fb)
    # point sets for the best-fit sphere: a mesh's vertices, a stretched one, a box, one and two points, points all on
    # one sphere (many equally valid supports), a planar grid (a flat support)
    Vs, _ = W.noisy_icosphere(4, 77, scale=[2.0, 0.5, 1.0], center=[0.3, -1.0, 2.0])
    Vc, _ = W.noisy_icosphere(3, 78, sigma=0.0)
    g = np.linspace(-1.0, 1.0, 21, dtype=np.float32)
    grid = np.stack(np.meshgrid(g, g, indexing="ij"), -1).reshape(-1, 2)
    plane = np.concatenate([grid, np.full((len(grid), 1), 0.3, np.float32)], 1).astype(np.float32)
    d["sphere"] = [V, Vs, W.uniform_box_points(1000, [0] * 3, [1] * 3, 79), V[:1], V[:2], Vc, plane]
    return d


def main():
    if len(sys.argv) != 2:
        raise SystemExit("usage: make_ref_golden.py <the reference's Code/Source directory>")
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref", "REF_SRC=" + sys.argv[1]], check=True)
    from oracle import reference as R
    d = inputs()
    out = {}
    V, F, Q = d["closest"]
    m = R.Mesh(V, F)
    for tag, b in (("", -1.0), ("_b005", 0.05), ("_b03", 0.3)):
        i, dist, cp = m.closest(Q, dist_bound=b)
        out["closest_index" + tag], out["closest_dist" + tag], out["closest_cp" + tag] = i, dist, cp
    Vh, Fh, o, dd = d["ray"]
    mh = R.Mesh(Vh, Fh)
    for tag, mt in (("", -1.0), ("_t045", 0.45)):
        t, i, n = mh.ray(o, dd, max_time=mt)
        out["ray_time" + tag], out["ray_index" + tag], out["ray_normal" + tag] = t, i, n
    P, Qk, ex = d["knn"]
    i, mad = R.Points(P).knn(Qk, 8, exclude=ex)
    out["knn_index"], out["knn_mad"] = i, mad
    i, mad = R.Points(P).knn(Qk, 8, dist_bound=0.03, exclude=ex)
    out["knn_index_b003"], out["knn_mad_b003"] = i, mad
    tris, pts, other, rdir = d["tri"]
    out["tri_closest"] = R.triangle_closest_points(tris, pts)
    out["tri_ray_time"] = R.triangle_ray_times(tris, pts, rdir)
    d2, pa, pb = R.triangle_pair_distances(tris, other)
    out["tri_pair_d2"], out["tri_pair_pa"], out["tri_pair_pb"] = d2, pa, pb
    Va, Fa, Vb, Fb = d["pair"]
    a, b = R.Mesh(Va, Fa), R.Mesh(Vb, Fb)
    for tag, (t, q) in (("_ab", (a, b)), ("_ba", (b, a))):
        qi, ti, mad, qp, tp = t.closest_pair(q)
        out["pair_index" + tag] = np.array([qi, ti], np.int32)
        out["pair_mad" + tag] = np.array(mad)
        out["pair_points" + tag] = np.stack([qp, tp])
    for s in (5489, 0xFFFF, 1234):
        out["random_%d" % s] = R.random_bits(s, 1248)
    for j, P in enumerate(d["sphere"]):
        out["sphere_center_%d" % j], r = R.best_fit_sphere(P)
        out["sphere_radius_%d" % j] = np.float32(r)
    ns = np.array([1, 5, 6, 11, 100, 81920, 1048576, 2093058], np.int64)
    out["tree_depth_n"] = ns
    out["tree_depth"] = np.array([R.tree_depth(int(n)) for n in ns], np.int64)
    path = os.path.join(HERE, "reference_outputs.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
