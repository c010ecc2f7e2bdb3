"""GPU parity of ShapeDiameter (Algorithms/SurfaceFeatures/Local/ShapeDiameter.hpp:143-217) against the oracle, whose
median selection is this C++ library's own std::nth_element. The FP64 results are compared for equality: the rays, the
kept hit times and the FP64 reduction follow the same operation sequence."""

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


def _vertex_normals(V, F):
    n = np.zeros_like(V, dtype=np.float64)
    a, b, c = V[F[:, 0]], V[F[:, 1]], V[F[:, 2]]
    fn = np.cross(b - a, c - a)
    for k in range(3):
        np.add.at(n, F[:, k], fn)
    return (n / np.linalg.norm(n, axis=1, keepdims=True)).astype(np.float32)


@pytest.mark.parametrize("only_interior", [True, False])
def test_shape_diameter_with_normals(T, oracle, only_interior):
    import torch
    V, F = W.noisy_icosphere(4, 31, sigma=0.02, scale=[1.0, 0.6, 0.35])
    N = _vertex_normals(V, F)
    bvh = T.MeshBvh(torch.from_numpy(V).cuda(), torch.from_numpy(F).cuda())
    got = bvh.shape_diameter(torch.from_numpy(V).cuda(), torch.from_numpy(N).cuda(), only_interior=only_interior)
    want = oracle.MeshIndex(V, F).shape_diameter(V, N, only_interior=only_interior)
    np.testing.assert_array_equal(got.cpu().numpy(), want)
    # -1 where no ray counts (a few vertices of the noisy surface whose cone only meets back faces)
    assert np.all(((want >= 0) & (want <= 1)) | (want == -1)) and np.mean(want >= 0) > 0.99
    # host arrays and an explicit scale
    got_h = bvh.shape_diameter(V, N, scale=2.5, only_interior=only_interior)
    np.testing.assert_array_equal(got_h, oracle.MeshIndex(V, F).shape_diameter(V, N, scale=2.5,
                                                                                only_interior=only_interior))
    bvh.close()


def test_shape_diameter_from_closest_elements(T, oracle):
    import torch
    V, F = W.noisy_icosphere(3, 32, sigma=0.03)
    P, _, _ = oracle.sample_by_area(V, F, 3000, 77)
    bvh = T.MeshBvh(torch.from_numpy(V).cuda(), torch.from_numpy(F).cuda())
    got = bvh.shape_diameter(torch.from_numpy(P).cuda())
    want = oracle.MeshIndex(V, F).shape_diameter(P)
    np.testing.assert_array_equal(got.cpu().numpy(), want)
    bvh.close()


def test_shape_diameter_open_surface_and_transform(T, oracle):
    import torch
    # a heightfield with upward normals: about half the points keep a ray (hits on the undersides of nearby bumps);
    # flattened, every inward ray leaves through the open underside and nothing counts (-1)
    HV, HF = W.heightfield(32, 5)
    up = np.tile(np.array([[0, 0, 1]], np.float32), (len(HV), 1))
    for verts in (HV, np.concatenate([HV[:, :2], np.zeros((len(HV), 1), np.float32)], 1)):
        hb = T.MeshBvh(verts, HF)
        got = hb.shape_diameter(verts, up)
        want = oracle.MeshIndex(verts, HF).shape_diameter(verts, up)
        np.testing.assert_array_equal(got, want)
        hb.close()
    assert np.all(want == -1.0)
    # a transformed sphere, with the points and normals in world space
    V, F = W.noisy_icosphere(3, 33, sigma=0.02)
    N = _vertex_normals(V, F)
    xf = np.array([[0.0, -1.5, 0.0, 0.3], [1.5, 0.0, 0.0, -2.0], [0.0, 0.0, 0.75, 1.0]], np.float32)
    Pw = V @ xf[:, :3].T + xf[:, 3]
    L_inv_t = np.linalg.inv(xf[:, :3].astype(np.float64)).T
    Nw = (N @ L_inv_t.T).astype(np.float32)
    bvh = T.MeshBvh(torch.from_numpy(V).cuda(), torch.from_numpy(F).cuda())
    bvh.set_transform(xf)
    got = bvh.shape_diameter(torch.from_numpy(Pw.astype(np.float32)).cuda(), torch.from_numpy(Nw).cuda())
    want = oracle.MeshIndex(V, F).shape_diameter(Pw.astype(np.float32), Nw, transform=xf)
    np.testing.assert_array_equal(got.cpu().numpy(), want)
    bvh.close()


def test_best_fit_sphere_against_the_reference(T, oracle):
    """thea_best_fit_sphere (BestFitSphereN, the default scale of ShapeDiameter(mesh)) on the point sets whose
    reference results are recorded in tests/golden/reference_outputs.npz: the radius rounded to float equals the
    reference's (the ball is unique; both compute in double), the centre agrees to float rounding, and device and host
    inputs give the same ball."""
    import os
    import sys
    import torch
    from tests.conftest import ROOT
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    import make_ref_golden as G
    ref = np.load(os.path.join(ROOT, "tests", "golden", "reference_outputs.npz"))
    for j, P in enumerate(G.inputs()["sphere"]):
        c, r = T.best_fit_sphere(torch.from_numpy(np.ascontiguousarray(P)).cuda())
        ch, rh = T.best_fit_sphere(P)
        assert r == rh and np.array_equal(c, ch), j
        rc, rr = ref["sphere_center_%d" % j], ref["sphere_radius_%d" % j]
        assert np.float32(r) == rr, (j, r, rr)
        scale = max(1.0, float(np.abs(P).max()))
        assert np.abs(c - rc.astype(np.float64)).max() <= 4e-7 * scale, j
        oc, orad = oracle.best_fit_sphere(P)
        assert abs(r - orad) <= 1e-12 * max(orad, 1.0), j
    # the constructor's default scale, passed explicitly
    V, F, _ = W.config0()
    assert T.shape_diameter_scale(V) == float(np.float32(2) * ref["sphere_radius_0"])


def test_best_fit_sphere_edge_cases(T, oracle):
    c, r = T.best_fit_sphere(np.zeros((0, 3), np.float32))
    assert r == 0.0 and not c.any()
    P = W.uniform_box_points(5000, [-2] * 3, [3] * 3, 81)
    P[::7] = np.nan  # non-finite points are skipped
    P[3] = [np.inf, 0, 0]
    c, r = T.best_fit_sphere(P)
    oc, orad = oracle.best_fit_sphere(P)
    assert abs(r - orad) <= 1e-12 * orad and np.abs(c - oc).max() <= 1e-9
    Q = np.repeat(P[1:2], 100, 0)  # one point, repeated
    c, r = T.best_fit_sphere(Q)
    assert r == 0.0 and np.array_equal(c, Q[0].astype(np.float64))
