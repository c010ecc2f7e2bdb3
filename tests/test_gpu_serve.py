"""GPU tests of the serving loop: every request's results equal those of the single-BVH calls on the same mesh
(bit-identical), alone and in a mix of concurrent requests of all kinds and sizes, from host and device arrays."""

import numpy as np
import pytest

from thea_gb300 import _native as N
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
def meshes():
    out = []
    for i, (level, sc) in enumerate(((2, (1.0, 0.6, 1.7)), (3, (0.5, 1.2, 1.0)), (4, (2.0, 1.0, 0.7)))):
        out.append(W.noisy_icosphere(level, 40 + i, scale=np.array(sc)))
    return out


def queries(n, seed, scale=1.5):
    return np.random.default_rng(seed).uniform(-scale * 2, scale * 2, (n, 3)).astype(np.float32)


def directions(n, seed):
    d = np.random.default_rng(seed).normal(size=(n, 3))
    return (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)


class Reference:
    """The single-BVH calls on each mesh: what every server request must reproduce."""

    def __init__(self, T, meshes, precision):
        self.mesh = [T.MeshBvh(V, F) for V, F in meshes]
        self.pts = [T.PointBvh(V) for V, _ in meshes]
        self.precision = precision

    def __call__(self, kind, m, q, d=None, bound=-1.0, k=8):
        if kind == "closest":
            i, v, p, _ = self.mesh[m].closest_element_ex(q, dist_bound=bound, precision=self.precision, errors=False)
            return i, v, p
        if kind == "ray":
            t, i, _ = self.mesh[m].ray_structure_intersection(q, d, max_time=bound)
            return i, t, None
        i, d2 = self.pts[m].k_closest_pairs(q, k, dist_bound=bound)
        return i, d2, None


def host(a):
    return a if isinstance(a, np.ndarray) else a.cpu().numpy()


def check(ticket, ref):
    assert ticket.wait(timeout_us=60_000_000) and ticket.status == N.THEA_OK
    i, v, p = ref
    assert np.array_equal(host(ticket.index), i)
    assert np.array_equal(host(ticket.value), v)
    if p is not None and ticket.point is not None:
        assert np.array_equal(host(ticket.point), p)


REQUESTS = [("closest", 0, 1, -1.0), ("closest", 1, 777, -1.0), ("closest", 2, 5000, 0.3), ("ray", 0, 3, -1.0),
            ("ray", 2, 4096, 2.5), ("knn", 1, 100, -1.0), ("knn", 2, 3000, 0.2), ("closest", 2, 70000, -1.0),
            ("ray", 1, 65537, -1.0), ("knn", 0, 20000, -1.0)]


# hard_query_budget: 0 = one thread per query throughout (default), 256 = two-phase, 3 = nearly every closest-point
# query finishes on a warp of its own
@pytest.mark.parametrize("precision,budget", [("fp32", 0), ("fp64", 0), ("fp32", 3), ("fp64", 3), ("fp32", 256)])
def test_requests_alone_and_in_a_mix_equal_the_single_bvh_calls(T, meshes, precision, budget):
    ref = Reference(T, meshes, precision)
    with T.Server(precision=precision, max_piece_queries=4096, max_batch_queries=16384, slots=3,
                  hard_query_budget=budget) as s:
        ids = [s.add_mesh(V, F) for V, F in meshes]
        cases = []
        for j, (kind, m, n, bound) in enumerate(REQUESTS):
            q = queries(n, j)
            d = directions(n, 100 + j) if kind == "ray" else None
            cases.append((kind, m, q, d, bound, ref(kind, m, q, d, bound)))
        # alone: one request at a time
        for kind, m, q, d, bound, r in cases:
            check(s.submit(kind, ids[m], q, directions=d, bound=bound, k=8, closest_points=True), r)
        # in a mix: everything at once, twice over, host arrays and device tensors
        import torch
        tickets = []
        for rep in range(2):
            for kind, m, q, d, bound, r in cases:
                if rep:
                    qd = torch.from_numpy(q).cuda()
                    dd = torch.from_numpy(d).cuda() if d is not None else None
                    t = s.submit(kind, ids[m], qd, directions=dd, bound=bound, k=8, closest_points=True)
                else:
                    t = s.submit(kind, ids[m], q, directions=d, bound=bound, k=8, closest_points=True)
                tickets.append((t, r))
        for t, r in tickets:
            check(t, r)
        st = s.stats()
        assert st["completed"] == 3 * len(cases) and st["failed"] == 0
        assert st["p99_ms"] >= st["p50_ms"] > 0 and st["batches"] > len(cases)
    for b in ref.mesh + ref.pts:
        assert b.info()["device_error_bits"] == 0


def test_k_up_to_32_and_pinned_host_arrays(T, meshes):
    import torch
    ref = Reference(T, meshes, "fp32")
    with T.Server() as s:
        m = s.add_mesh(*meshes[1])
        for k in (1, 13, 32):
            q = torch.from_numpy(queries(2000, k)).pin_memory()
            out = (torch.empty((2000, k), dtype=torch.int32).pin_memory(),
                   torch.empty((2000, k), dtype=torch.float32).pin_memory())
            t = s.submit("knn", m, q, k=k, out=out)
            i, d2, _ = ref("knn", 1, q.numpy(), k=k)
            assert t.wait() and t.status == N.THEA_OK
            assert np.array_equal(out[0].numpy(), i) and np.array_equal(out[1].numpy(), d2)


@pytest.mark.timeout(300)
def test_removing_meshes_while_other_requests_run(T, meshes):
    """A mesh removed while its own and other meshes' requests are in flight stays usable by the requests already
    submitted, is released when the last of them ends (its BVHs destroyed outside the server's lock, while other slots'
    completions keep arriving), and every request's results still equal the single-BVH calls."""
    ref = Reference(T, meshes, "fp32")
    with T.Server(slots=3, max_batch_queries=16384, max_piece_queries=4096) as s:
        ids = [s.add_mesh(V, F) for V, F in meshes]
        for rep in range(3):
            spare = s.add_mesh(*meshes[rep % 3])
            tickets = []
            for r in range(24):
                kind = ("closest", "ray", "knn")[r % 3]
                m = r % 3
                q = queries(3000 + 500 * r, 900 + 31 * rep + r)
                d = directions(len(q), 7 + r) if kind == "ray" else None
                on_spare = r % 4 == 0 and r <= 12
                mesh_id = spare if on_spare else ids[m]
                src = rep % 3 if on_spare else m
                tickets.append((s.submit(kind, mesh_id, q, directions=d, k=8), ref(kind, src, q, d)))
                if r == 12:
                    s.remove_mesh(spare)  # requests on it are in flight; later ones may not use it
            for t, want in tickets:
                check(t, want)
        assert s.stats()["resident_bytes"] > 0
