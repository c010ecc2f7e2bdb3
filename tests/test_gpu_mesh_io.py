"""GPU parity of the spatial queries on meshes read from OFF and OBJ files: the library's reader feeds MeshBvh, the
pure-Python reader restatement feeds the CPU oracle, and closest-point and first-hit results must agree bit for bit."""

import numpy as np
import pytest

from oracle import mesh_oracle as MO
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


def _polygon_obj(rng, rings=24, segments=40):
    """A closed surface of revolution written with quads, a polygonal cap (one face of `segments` vertices) and two
    groups, with a mix of reference forms."""
    lines = []
    for i in range(rings):
        phi = np.pi * (i + 1) / (rings + 1)
        r = np.sin(phi) * (1 + 0.05 * rng.normal())
        for j in range(segments):
            th = 2 * np.pi * j / segments
            lines.append("v %.8f %.8f %.8f" % (r * np.cos(th), r * np.sin(th), np.cos(phi)))
    lines.append("vn 0 0 1")
    lines.append("g body")
    for i in range(rings - 1):
        for j in range(segments):
            a = i * segments + j + 1
            b = i * segments + (j + 1) % segments + 1
            c = b + segments
            d = a + segments
            lines.append("f %d %d//1 %d %d/0/1" % (a, b, c, d))
    lines.append("g caps")
    lines.append("f " + " ".join(str(j + 1) for j in reversed(range(segments))))
    last = (rings - 1) * segments
    lines.append("f " + " ".join(str(last + j + 1) for j in range(segments)))
    return "\n".join(lines) + "\n"


def test_closest_point_and_rays_on_a_polygon_mesh_file(T, oracle, tmp_path):
    import torch
    rng = np.random.default_rng(21)
    path = tmp_path / "surface.obj"
    path.write_text(_polygon_obj(rng))
    m = T.read_mesh(str(path))
    ref = MO.read_mesh(str(path))
    assert np.array_equal(m.triangles, ref["triangles"]) and np.array_equal(m.vertices, ref["vertices"])
    V, F = ref["vertices"], ref["triangles"]
    bvh = T.MeshBvh.from_file(str(path))
    Q = W.uniform_box_points(20000, [-1.5] * 3, [1.5] * 3, 22)
    idx, dist, cp = bvh.closest_element(torch.from_numpy(Q).cuda())
    ri, rd2, rcp = oracle.closest_brute(V, F, Q)
    assert np.array_equal(idx.cpu().numpy(), ri)
    assert np.array_equal(dist.cpu().numpy(), np.sqrt(rd2.astype(np.float32)))
    assert np.array_equal(cp.cpu().numpy(), rcp.astype(np.float32))
    o = (rng.normal(size=(20000, 3)) * 0.3).astype(np.float32)
    d = rng.normal(size=(20000, 3)).astype(np.float32)
    t, ti, _ = bvh.ray_structure_intersection(torch.from_numpy(o).cuda(), torch.from_numpy(d).cuda())
    rt, rti = oracle.ray_brute(V, F, o, d)
    assert np.array_equal(ti.cpu().numpy(), rti) and np.array_equal(t.cpu().numpy(), rt.astype(np.float32))
    bvh.close()


def test_off_file_round_trip_through_the_bvh(T, oracle, tmp_path):
    import torch
    V, F = W.noisy_icosphere(3, 5)
    lines = ["OFF", "%d %d 0" % (len(V), len(F))] + ["%.9g %.9g %.9g" % tuple(v) for v in V]
    lines += ["3 %d %d %d" % tuple(f) for f in F]
    path = tmp_path / "sphere.off"
    path.write_text("\n".join(lines) + "\n")
    m = T.read_mesh(str(path))
    assert np.array_equal(m.vertices, V.astype(np.float32)) and np.array_equal(m.triangles, F)
    bvh = T.MeshBvh.from_file(str(path))
    Q = W.uniform_box_points(4096, [-1.5] * 3, [1.5] * 3, 6)
    idx, _, _ = bvh.closest_element(torch.from_numpy(Q).cuda())
    ri, _, _ = oracle.closest_brute(V, F, Q)
    assert np.array_equal(idx.cpu().numpy(), ri)
    bvh.close()
