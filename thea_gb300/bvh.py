"""Python host mirror of the reference's spatial-query interface, over the C ABI.

Names follow Thea's ``BvhN`` / ``MeshBvh`` / ``MeshSampler`` (Code/Source/Algorithms/BvhN.hpp, MeshBvh.hpp,
MeshSampler.hpp), in batched form: every query method takes arrays of queries and returns arrays of results with the
reference's sentinels (index -1, time -1, distance -1 for "none").

Arrays may be NumPy arrays (host memory; results come back as NumPy arrays, the library stages the copies) or CUDA
torch tensors (device memory; results are CUDA tensors produced asynchronously on torch's current stream).
"""

import ctypes

import numpy as np

from . import _native as N


def _is_torch(x):
    return type(x).__module__.startswith("torch")


def _cuda_ready():
    import torch
    return torch.cuda.is_available() and torch.cuda.is_initialized()


def _stream_of(on_device):
    if not on_device:
        return None
    import torch
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


class _Arrays:
    """Normalises inputs to contiguous float32/int32 arrays on one side (host or device) and allocates outputs there."""

    def __init__(self, like):
        self.device = _is_torch(like) and like.is_cuda
        self.keep = []

    def input(self, a, dtype, cols=None):
        if a is None:
            return None, 0
        if self.device:
            import torch
            tdt = torch.float32 if dtype == np.float32 else torch.int32
            t = a.to(dtype=tdt).contiguous()
            if cols:
                t = t.reshape(-1, cols)
            self.keep.append(t)
            return ctypes.c_void_p(t.data_ptr()), t.shape[0]
        if _is_torch(a):
            a = a.detach().cpu().numpy()
        arr = np.ascontiguousarray(a, dtype=dtype)
        if cols:
            arr = arr.reshape(-1, cols)
        self.keep.append(arr)
        return ctypes.c_void_p(arr.ctypes.data), arr.shape[0]

    def output(self, shape, dtype):
        if self.device:
            import torch
            tdt = torch.float32 if dtype == np.float32 else torch.int32
            t = torch.empty(shape, dtype=tdt, device="cuda")
            return t, ctypes.c_void_p(t.data_ptr() if t.numel() else 0)
        arr = np.empty(shape, dtype=dtype)
        return arr, ctypes.c_void_p(arr.ctypes.data if arr.size else 0)


def _config(width, max_leaf_size, layouts, query_order=0):
    cfg = N.BuildConfig()
    cfg.width = int(width)
    cfg.max_leaf_size = int(max_leaf_size)
    cfg.layouts = int(layouts)
    cfg.query_order = int(query_order)
    return cfg


class _Bvh:
    def __init__(self):
        self._h = ctypes.c_void_p()

    def info(self):
        inf = N.BvhInfo()
        N.check(N.lib().thea_bvh_get_info(self._h, ctypes.byref(inf)))
        return {"num_elements": inf.num_elements, "num_nodes": inf.num_nodes, "width": inf.width,
                "max_leaf_size": inf.max_leaf_size, "is_mesh": bool(inf.is_mesh), "depth": inf.depth,
                "device_bytes": inf.device_bytes, "bounds_lo": list(inf.bounds_lo), "bounds_hi": list(inf.bounds_hi),
                "device_error_bits": inf.device_error_bits, "num_segments": inf.num_segments}

    def set_transform(self, affine):
        """BvhN::setTransform: queries then act on the elements mapped by ``affine`` (3x4 [L | t], or 4x4 with last row
        0 0 0 1). Rays go into object space with the FP32 inverse, closest-point / k-NN / radius queries run on a
        world-space copy of the records built on the device."""
        m = np.asarray(affine, np.float32)
        if m.shape == (4, 4):
            m = m[:3]
        if m.shape != (3, 4):
            raise ValueError("affine must be 3x4 or 4x4")
        m = np.ascontiguousarray(m)
        N.check(N.lib().thea_bvh_set_transform(self._h, m.ctypes.data, _stream_of(_cuda_ready())))

    def clear_transform(self):
        N.check(N.lib().thea_bvh_clear_transform(self._h))

    def transform(self):
        """(affine 3x4, its FP32 inverse 3x4), or None without a transform."""
        has = ctypes.c_int32()
        m = np.empty((3, 4), np.float32)
        inv = np.empty((3, 4), np.float32)
        N.check(N.lib().thea_bvh_get_transform(self._h, ctypes.byref(has), m.ctypes.data, inv.ctypes.data))
        return (m, inv) if has.value else None

    def to_bytes(self):
        """Byte image of the built BVH (thea_bvh_serialize); ``type(self).from_bytes`` reloads it without a rebuild."""
        size = ctypes.c_int64()
        N.check(N.lib().thea_bvh_serialize(self._h, None, 0, ctypes.byref(size), None))
        buf = ctypes.create_string_buffer(size.value)
        N.check(N.lib().thea_bvh_serialize(self._h, buf, size.value, ctypes.byref(size), None))
        return buf.raw[:size.value]

    @classmethod
    def from_bytes(cls, image):
        """A handle on the current device from a byte image (thea_bvh_deserialize); the image's kind (mesh or points)
        must match the class."""
        image = bytes(image)
        buf = (ctypes.c_char * max(len(image), 1)).from_buffer_copy(image or b"\0")
        obj = cls.__new__(cls)
        _Bvh.__init__(obj)
        N.check(N.lib().thea_bvh_deserialize(buf, len(image), None, ctypes.byref(obj._h)))
        inf = obj.info()
        if inf["is_mesh"] != issubclass(cls, (MeshBvh, MeshForest)):
            obj.close()
            raise N.TheaError(N.THEA_ERR_INVALID_ARGUMENT, "bvh_deserialize: the image holds a %s BVH, not a %s" %
                              ("mesh" if inf["is_mesh"] else "point", cls.__name__))
        obj._restored(inf)
        return obj

    def _restored(self, inf):
        pass

    def closest_pair(self, query, dist_bound=-1.0):
        """BvhN::closestPair with another BVH (``query``) as the query: (query index, target index, squared distance,
        query point, target point), or None when no pair qualifies. Points and meshes on either side; between two
        meshes the distance is TriangleN::squaredDistance with the target triangle as "this"."""
        qi, ti, d2 = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_float()
        qp, tp = np.zeros(3, np.float32), np.zeros(3, np.float32)
        N.check(N.lib().thea_bvh_closest_pair(self._h, query.handle, float(dist_bound), ctypes.byref(qi),
                                              ctypes.byref(ti), ctypes.byref(d2), qp.ctypes.data, tp.ctypes.data,
                                              _stream_of(_cuda_ready())))
        if qi.value < 0:
            return None
        return qi.value, ti.value, d2.value, qp, tp

    def k_closest_pairs(self, queries, k, dist_bound=-1.0, exclude=None):
        """BvhN::kClosestPairs: the k nearest elements of each query point (points of a PointBvh, triangles of a
        MeshBvh): (indices [n, k], squared distances [n, k]); unused slots -1. With another BVH as the query: the k
        closest pairs between the two (see k_closest_pairs_bvh)."""
        if isinstance(queries, _Bvh):
            return self.k_closest_pairs_bvh(queries, k, dist_bound)
        io = _Arrays(queries)
        pq, n = io.input(queries, np.float32, 3)
        pe, _ = io.input(exclude, np.int32) if exclude is not None else (None, 0)
        idx, pidx = io.output((n, k), np.int32)
        d2, pd2 = io.output((n, k), np.float32)
        N.check(N.lib().thea_k_closest(self._h, pq, n, int(k), float(dist_bound), pe, pidx, pd2,
                                       _stream_of(io.device)))
        return idx, d2

    def k_closest_pairs_bvh(self, query, k, dist_bound=-1.0):
        """BvhN::kClosestPairs between two point BVHs: (query indices, target indices, squared distances) of the k
        closest pairs, ascending, -1 past the number found. PointBvh.k_closest_pairs forwards here for a BVH query."""
        qi, ti = np.empty(k, np.int32), np.empty(k, np.int32)
        d2 = np.empty(k, np.float32)
        cnt = ctypes.c_int32()
        N.check(N.lib().thea_bvh_k_closest_pairs(self._h, query.handle, int(k), float(dist_bound), qi.ctypes.data,
                                                 ti.ctypes.data, d2.ctypes.data, ctypes.byref(cnt),
                                                 _stream_of(_cuda_ready())))
        return qi, ti, d2

    def close(self):
        if self._h:
            N.check(N.lib().thea_bvh_destroy(self._h))
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h


class MeshBvh(_Bvh):
    """BVH over the triangles of a mesh (MeshBvh::add + MeshBvh::init). Element index = face index."""

    def __init__(self, vertices, faces, width=4, max_leaf_size=0, layouts=0, query_order=0):
        super().__init__()
        io = _Arrays(vertices)
        pv, nv = io.input(vertices, np.float32, 3)
        pf, nf = io.input(faces, np.int32, 3)
        cfg = _config(width, max_leaf_size, layouts, query_order)
        N.check(N.lib().thea_mesh_bvh_build(pv, nv, pf, nf, ctypes.byref(cfg), _stream_of(io.device),
                                            ctypes.byref(self._h)))

    @classmethod
    def from_file(cls, path, **kwargs):
        """BVH over the triangles of an OFF, OBJ or PLY file, in the order MeshGroup::load + MeshBvh::add give them."""
        m = read_mesh(path)
        return cls(m.vertices, m.triangles, **kwargs)

    def closest_element(self, queries, dist_bound=-1.0, closest_points=True):
        """BvhN::closestElement<MetricL2>: (index, distance, closest point or None) per query."""
        io = _Arrays(queries)
        pq, n = io.input(queries, np.float32, 3)
        idx, pidx = io.output((n,), np.int32)
        dist, pdist = io.output((n,), np.float32)
        cp, pcp = io.output((n, 3), np.float32) if closest_points else (None, None)
        N.check(N.lib().thea_closest_element(self._h, pq, n, float(dist_bound), pidx, pdist, pcp,
                                             _stream_of(io.device)))
        return idx, dist, cp

    def ray_structure_intersection(self, origins, directions, max_time=-1.0, normals=False):
        """BvhN::rayStructureIntersection: (time, element index, unit normal or None) per ray; -1 on a miss."""
        io = _Arrays(origins)
        po, n = io.input(origins, np.float32, 3)
        pd, nd = io.input(directions, np.float32, 3)
        if nd != n:
            raise ValueError("origins and directions differ in length")
        t, pt = io.output((n,), np.float32)
        idx, pidx = io.output((n,), np.int32)
        nrm, pn = io.output((n, 3), np.float32) if normals else (None, None)
        N.check(N.lib().thea_ray_intersection(self._h, po, pd, n, float(max_time), pt, pidx, pn,
                                              _stream_of(io.device)))
        return t, idx, nrm

    def ray_intersection_time(self, origins, directions, max_time=-1.0):
        """BvhN::rayIntersectionTime: hit time per ray, -1 on a miss."""
        return self.ray_structure_intersection(origins, directions, max_time)[0]

    def ray_intersects(self, origins, directions, max_time=-1.0):
        """BvhN::rayIntersects: per ray, whether some element is hit at a time in [0, max_time] (any-hit search)."""
        io = _Arrays(origins)
        po, n = io.input(origins, np.float32, 3)
        pd, nd = io.input(directions, np.float32, 3)
        if nd != n:
            raise ValueError("origins and directions differ in length")
        if io.device:
            import torch
            hit = torch.empty(n, dtype=torch.uint8, device="cuda")
            ph = ctypes.c_void_p(hit.data_ptr() if n else 0)
        else:
            hit = np.empty(n, np.uint8)
            ph = ctypes.c_void_p(hit.ctypes.data if n else 0)
        N.check(N.lib().thea_ray_intersects(self._h, po, pd, n, float(max_time), ph, _stream_of(io.device)))
        return hit.bool() if io.device else hit.astype(bool)

    def visibility(self, positions, num_rays=100, seed=0):
        """Visibility::compute for each position (fraction of num_rays rays that escape), with Random(seed) in place of
        the reference's Random::common(); float64 per point (CUDA tensor for CUDA input)."""
        io = _Arrays(positions)
        pp, n = io.input(positions, np.float32, 3)
        if io.device:
            import torch
            out = torch.empty(n, dtype=torch.float64, device="cuda")
            po = ctypes.c_void_p(out.data_ptr() if n else 0)
        else:
            out = np.empty(n, np.float64)
            po = ctypes.c_void_p(out.ctypes.data if n else 0)
        N.check(N.lib().thea_visibility(self._h, pp, n, int(num_rays), int(seed) & 0xffffffff, po,
                                        _stream_of(io.device)))
        return out

    def shape_diameter(self, positions, normals=None, scale=-1.0, only_interior=True):
        """ShapeDiameter(bvh, scale)::compute for each position (normals: outward normals, or None for each point's
        closest element's normal); float64 per point in [0, 1], -1 where no ray counts (CUDA tensor for CUDA input)."""
        io = _Arrays(positions)
        pp, n = io.input(positions, np.float32, 3)
        pn, _ = io.input(normals, np.float32, 3) if normals is not None else (None, 0)
        if io.device:
            import torch
            out = torch.empty(n, dtype=torch.float64, device="cuda")
            po = ctypes.c_void_p(out.data_ptr() if n else 0)
        else:
            out = np.empty(n, np.float64)
            po = ctypes.c_void_p(out.ctypes.data if n else 0)
        N.check(N.lib().thea_shape_diameter(self._h, pp, pn, n, float(scale), 1 if only_interior else 0, po,
                                            _stream_of(io.device)))
        return out

    def closest_element_ex(self, queries, dist_bound=-1.0, precision="fp32", closest_points=True, errors=True):
        """closest_element with a precision mode ("fp32": the reference's arithmetic; "fp64": FP64 re-check band) and
        per-query |returned distance - FP64 distance of the returned element|: (index, distance, cp, error)."""
        io = _Arrays(queries)
        pq, n = io.input(queries, np.float32, 3)
        idx, pidx = io.output((n,), np.int32)
        dist, pdist = io.output((n,), np.float32)
        cp, pcp = io.output((n, 3), np.float32) if closest_points else (None, None)
        err, perr = io.output((n,), np.float32) if errors else (None, None)
        N.check(N.lib().thea_closest_element_ex(self._h, pq, n, float(dist_bound), _precision(precision), pidx, pdist,
                                                pcp, perr, _stream_of(io.device)))
        return idx, dist, cp, err

    def ray_structure_intersection_ex(self, origins, directions, max_time=-1.0, precision="fp64"):
        """Ray first hit with the FP64 watertight verdict beside the reference's FP32 one:
        (time, index, time_fp64, index_fp64, flags)."""
        io = _Arrays(origins)
        po, n = io.input(origins, np.float32, 3)
        pd, _ = io.input(directions, np.float32, 3)
        t, pt = io.output((n,), np.float32)
        idx, pidx = io.output((n,), np.int32)
        t64, pt64 = io.output((n,), np.float32)
        i64, pi64 = io.output((n,), np.int32)
        fl, pfl = io.output((n,), np.int32)
        N.check(N.lib().thea_ray_intersection_ex(self._h, po, pd, n, float(max_time), _precision(precision), pt, pidx,
                                                 None, pt64, pi64, pfl, _stream_of(io.device)))
        return t, idx, t64, i64, fl


def _precision(p):
    return {"fp32": N.PRECISION_FP32_REFERENCE, "fp64": N.PRECISION_FP64_RECHECK}[p]


def _offsets_ptr(off):
    off = np.ascontiguousarray(off, dtype=np.int64)
    return off, off.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))


class MeshForest(_Bvh):
    """One BVH per mesh, built in one pass (thea_mesh_forest_build). `faces` index the shared vertex array; mesh m owns
    faces [face_offsets[m], face_offsets[m+1]). Queries are CUDA tensors grouped by mesh (query_offsets, int64 CUDA)."""

    def __init__(self, vertices, faces, face_offsets, width=4, max_leaf_size=0, layouts=0):
        super().__init__()
        io = _Arrays(vertices)
        pv, nv = io.input(vertices, np.float32, 3)
        pf, _ = io.input(faces, np.int32, 3)
        self._off, poff = _offsets_ptr(face_offsets)
        self.num_meshes = len(self._off) - 1
        cfg = _config(width, max_leaf_size, layouts)
        N.check(N.lib().thea_mesh_forest_build(pv, nv, pf, poff, self.num_meshes, ctypes.byref(cfg),
                                               _stream_of(io.device), ctypes.byref(self._h)))

    def _restored(self, inf):
        self.num_meshes = inf["num_segments"]

    def batch_closest_element(self, queries, query_offsets, dist_bound=-1.0, precision="fp32", queries_per_warp=0,
                              hard_query_budget=0, closest_points=False, errors=False, out=None):
        import torch
        n = queries.shape[0]
        if out is None:
            out = (torch.empty(n, dtype=torch.int32, device="cuda"), torch.empty(n, dtype=torch.float32, device="cuda"),
                   torch.empty((n, 3), dtype=torch.float32, device="cuda") if closest_points else None,
                   torch.empty(n, dtype=torch.float32, device="cuda") if errors else None)
        idx, dist, cp, err = out
        ptr = lambda t: ctypes.c_void_p(t.data_ptr()) if t is not None else None  # noqa: E731
        N.check(N.lib().thea_batch_closest_element(self._h, ptr(queries), ptr(query_offsets), n, float(dist_bound),
                                                   _precision(precision), int(queries_per_warp),
                                                   int(hard_query_budget), ptr(idx), ptr(dist), ptr(cp), ptr(err),
                                                   _stream_of(True)))
        return out

    def batch_ray_intersection(self, origins, directions, query_offsets, max_time=-1.0, queries_per_warp=0):
        import torch
        n = origins.shape[0]
        t = torch.empty(n, dtype=torch.float32, device="cuda")
        idx = torch.empty(n, dtype=torch.int32, device="cuda")
        ptr = lambda x: ctypes.c_void_p(x.data_ptr())  # noqa: E731
        N.check(N.lib().thea_batch_ray_intersection(self._h, ptr(origins), ptr(directions), ptr(query_offsets), n,
                                                    float(max_time), int(queries_per_warp), ptr(t), ptr(idx),
                                                    _stream_of(True)))
        return t, idx


class PointForest(_Bvh):
    """One point BVH per point set (thea_point_forest_build); set m owns points [set_offsets[m], set_offsets[m+1])."""

    def __init__(self, points, set_offsets, width=4, max_leaf_size=0):
        super().__init__()
        io = _Arrays(points)
        pp, _ = io.input(points, np.float32, 3)
        self._off, poff = _offsets_ptr(set_offsets)
        cfg = _config(width, max_leaf_size, 0)
        N.check(N.lib().thea_point_forest_build(pp, poff, len(self._off) - 1, ctypes.byref(cfg), _stream_of(io.device),
                                                ctypes.byref(self._h)))

    def batch_k_closest(self, queries, query_offsets, k, dist_bound=-1.0, queries_per_warp=0):
        import torch
        n = queries.shape[0]
        idx = torch.empty((n, k), dtype=torch.int32, device="cuda")
        d2 = torch.empty((n, k), dtype=torch.float32, device="cuda")
        ptr = lambda x: ctypes.c_void_p(x.data_ptr())  # noqa: E731
        N.check(N.lib().thea_batch_k_closest(self._h, ptr(queries), ptr(query_offsets), n, int(k), float(dist_bound),
                                             int(queries_per_warp), ptr(idx), ptr(d2), _stream_of(True)))
        return idx, d2


class Graph:
    """A CUDA graph captured from library calls issued on torch's current (non-default) stream:

        with Graph() as g:
            forest.batch_closest_element(...)
        g.launch()
    """

    def __init__(self):
        self._g = ctypes.c_void_p()

    def __enter__(self):
        import torch
        self._stream = torch.cuda.current_stream()
        N.check(N.lib().thea_graph_capture_begin(ctypes.c_void_p(self._stream.cuda_stream)))
        return self

    def __exit__(self, exc_type, exc, tb):
        st = N.lib().thea_graph_capture_end(ctypes.c_void_p(self._stream.cuda_stream), ctypes.byref(self._g))
        if exc_type is None:
            N.check(st)

    def launch(self):
        import torch
        N.check(N.lib().thea_graph_launch(self._g, ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)))

    def close(self):
        if self._g:
            N.check(N.lib().thea_graph_destroy(self._g))
            self._g = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def autotune_batch_closest(vertices, faces, face_offsets, queries, query_offsets, precision="fp32"):
    """Times width x leaf size x queries-per-warp on a sample workload; returns the fastest as a dict."""
    io = _Arrays(vertices)
    pv, nv = io.input(vertices, np.float32, 3)
    pf, _ = io.input(faces, np.int32, 3)
    off, poff = _offsets_ptr(face_offsets)
    t = N.Tuning()
    N.check(N.lib().thea_autotune_batch_closest(pv, nv, pf, poff, len(off) - 1, ctypes.c_void_p(queries.data_ptr()),
                                                ctypes.c_void_p(query_offsets.data_ptr()), queries.shape[0],
                                                _precision(precision), _stream_of(True), ctypes.byref(t)))
    return {"width": t.width, "max_leaf_size": t.max_leaf_size, "queries_per_warp": t.queries_per_warp,
            "hard_query_budget": t.hard_query_budget, "milliseconds": t.milliseconds, "candidates": t.candidates}


class PointBvh(_Bvh):
    """BVH over points (BvhN<Vector3, 3>). Element index = point index."""

    def __init__(self, points, width=4, max_leaf_size=0, query_order=0):
        super().__init__()
        io = _Arrays(points)
        pp, n = io.input(points, np.float32, 3)
        cfg = _config(width, max_leaf_size, 0, query_order)
        N.check(N.lib().thea_point_bvh_build(pp, n, ctypes.byref(cfg), _stream_of(io.device), ctypes.byref(self._h)))
        self.n = n

    def _restored(self, inf):
        self.n = inf["num_elements"]

    def radius_neighbors(self, queries, radius, exclude=None):
        """BvhN::rangeQueryIndices with a Ball3: every point within `radius` (inclusive) of each CUDA-tensor query, as
        CSR (offsets [n + 1] int64, indices [total] int32 in ascending order per query, squared distances [total])."""
        import torch
        q = queries.to(torch.float32).contiguous()
        n = q.shape[0]
        ex = exclude.to(torch.int32).contiguous() if exclude is not None else None
        off = torch.empty(n + 1, dtype=torch.int64, device=q.device)
        pex = ctypes.c_void_p(ex.data_ptr()) if ex is not None else None
        st = _stream_of(True)
        N.check(N.lib().thea_radius_neighbors(self._h, ctypes.c_void_p(q.data_ptr()), n, float(radius), pex,
                                              ctypes.c_void_p(off.data_ptr()), None, None, st))
        total = int(off[-1].item()) if n else 0
        idx = torch.empty(total, dtype=torch.int32, device=q.device)
        d2 = torch.empty(total, dtype=torch.float32, device=q.device)
        if total:
            N.check(N.lib().thea_radius_neighbors(self._h, ctypes.c_void_p(q.data_ptr()), n, float(radius), pex,
                                                  ctypes.c_void_p(off.data_ptr()), ctypes.c_void_p(idx.data_ptr()),
                                                  ctypes.c_void_p(d2.data_ptr()), st))
        return off, idx, d2

    def k_closest_self(self, k, device=False, candidates="traversal"):
        """k-nearest-neighbour graph of the indexed points, each excluding itself; rows in point order.
        candidates="gram": tensor-core Gram tiles seed the search with an exact bound (same results)."""
        if device:
            import torch
            io = _Arrays(torch.empty(0, device="cuda"))
        else:
            io = _Arrays(np.empty(0))
        idx, pidx = io.output((self.n, k), np.int32)
        d2, pd2 = io.output((self.n, k), np.float32)
        mode = {"traversal": N.KNN_CANDIDATES_TRAVERSAL, "gram": N.KNN_CANDIDATES_GRAM}[candidates]
        N.check(N.lib().thea_k_closest_self_ex(self._h, int(k), mode, pidx, pd2, _stream_of(io.device)))
        return idx, d2


def point_gram_tile(a, b):
    """Tensor-core Gram tile of two CUDA point sets (a: <= 128 points, b: <= 512): keys [128, 512] with
    keys[r, j] = |b_j|^2 - 2 a_r . b_j in the tile's normalised FP16 frame (thea_point_gram_tile)."""
    import torch
    a = a.to(torch.float32).contiguous()
    b = b.to(torch.float32).contiguous()
    keys = torch.empty((128, 512), dtype=torch.float32, device=a.device)
    N.check(N.lib().thea_point_gram_tile(ctypes.c_void_p(a.data_ptr()), a.shape[0], ctypes.c_void_p(b.data_ptr()),
                                         b.shape[0], ctypes.c_void_p(keys.data_ptr()), _stream_of(True)))
    return keys


def sample_graph(positions, normals=None, max_degree=8, seed=0, surface=None, dense_positions=None,
                 dense_normals=None):
    """PointSet3::updateGraph with Random(seed) for the separation estimate. Returns (neighbours [n, max_degree] int32
    with -1 past the degree, separations [n, max_degree], degrees [n], (estimate, final mean separation)). surface: a
    MeshBvh for the reachability test (used with normals, as in the reference). dense_positions (and dense_normals,
    needed with normals): an oversampling (PointSet3::addOversampling); neighbours are then the nearest samples along
    shortest paths through the graph of all points (extractOriginalAdjacencies)."""
    io = _Arrays(positions)
    pp, n = io.input(positions, np.float32, 3)
    pn, _ = io.input(normals, np.float32, 3) if normals is not None else (None, 0)
    nbr, pnb = io.output((n, max_degree), np.int32)
    sep, psp = io.output((n, max_degree), np.float32)
    deg, pdg = io.output((n,), np.int32)
    avg = np.zeros(2, np.float32)
    sh = surface.handle if surface is not None else None
    if dense_positions is None:
        N.check(N.lib().thea_sample_graph(pp, pn, n, int(max_degree), int(seed) & 0xffffffff, sh, pnb, psp, pdg,
                                          avg.ctypes.data, _stream_of(io.device)))
    else:
        pd, nd = io.input(dense_positions, np.float32, 3)
        pdn, _ = io.input(dense_normals, np.float32, 3) if dense_normals is not None else (None, 0)
        N.check(N.lib().thea_sample_graph_oversampled(pp, pn, n, pd, pdn, nd, int(max_degree), int(seed) & 0xffffffff,
                                                      sh, pnb, psp, pdg, avg.ctypes.data, _stream_of(io.device)))
    return nbr, sep, deg, (float(avg[0]), float(avg[1]))


def write_sample_graph(path, neighbors, separations, degrees, max_degree, write_distances=True):
    """PointSet3::save's graph file (PointSet3.cpp:321-348): the maximum degree, then one line per sample: its degree,
    its neighbours' indices and (optionally) their separations, formatted as C++ streams print floats (%g)."""
    nb = np.asarray(neighbors)
    sp = np.asarray(separations)
    dg = np.asarray(degrees)
    with open(path, "w", newline="\n") as f:
        f.write("%d\n" % max_degree)
        for i in range(len(dg)):
            k = int(dg[i])
            parts = [str(k)] + [str(int(x)) for x in nb[i, :k]]
            if write_distances:
                parts += ["%g" % float(x) for x in sp[i, :k]]
            f.write(" ".join(parts) + "\n")


def best_fit_sphere(points):
    """BestFitSphereN<3>: the smallest ball enclosing the points (float32 [n, 3], host array or CUDA tensor), as
    (centre: float64 [3], radius: float)."""
    io = _Arrays(points)
    pp, n = io.input(points, np.float32, 3)
    c = np.zeros(3, np.float64)
    r = ctypes.c_double(0.0)
    N.check(N.lib().thea_best_fit_sphere(pp, n, ctypes.c_void_p(c.ctypes.data), ctypes.byref(r),
                                         _stream_of(io.device)))
    return c, r.value


def shape_diameter_scale(vertices):
    """The default scale of ShapeDiameter(mesh) (ShapeDiameter.hpp:60-70): the diameter of the mesh vertices' best-fit
    sphere, in float32 as the reference's Real. Pass it as MeshBvh.shape_diameter(..., scale=...)."""
    _, r = best_fit_sphere(vertices)
    return float(np.float32(2.0) * np.float32(r))


def random_sphere(seed, count, device=False):
    """`count` directions of Random(seed).sphere() in stream order (float32 [count, 3])."""
    if device:
        import torch
        out = torch.empty((count, 3), dtype=torch.float32, device="cuda")
        N.check(N.lib().thea_random_sphere(int(seed) & 0xffffffff, int(count), ctypes.c_void_p(out.data_ptr()),
                                           _stream_of(True)))
        return out
    out = np.empty((count, 3), np.float32)
    N.check(N.lib().thea_random_sphere(int(seed) & 0xffffffff, int(count), ctypes.c_void_p(out.ctypes.data), None))
    return out


class MeshData:
    """A mesh file read as MeshGroup<DisplayMesh>::load reads it (OFF, OBJ or PLY, by extension), flattened: vertices
    [nv, 3] float32, vertex_source [nv] (file vertex index), triangles [nt, 3] int32, triangle_face [nt] (source face
    index), submesh_vertex_offsets and submesh_triangle_offsets [submeshes + 1] int64, num_faces (faces that produced
    triangles). Pass (vertices, triangles) to MeshBvh for the reference's element order."""

    def __init__(self, vertices, vertex_source, triangles, triangle_face, submesh_vertex_offsets,
                 submesh_triangle_offsets, num_faces):
        self.vertices = vertices
        self.vertex_source = vertex_source
        self.triangles = triangles
        self.triangle_face = triangle_face
        self.submesh_vertex_offsets = submesh_vertex_offsets
        self.submesh_triangle_offsets = submesh_triangle_offsets
        self.num_faces = num_faces


def read_mesh(path, codec=None):
    """Reads a 3DS, OFF, OBJ or PLY file into host arrays (MeshData). ``path`` may also be the file's bytes, with
    ``codec`` ("3ds", "obj", "off" or "ply") naming the format."""
    lib = N.lib()
    h = ctypes.c_void_p()
    if isinstance(path, (bytes, bytearray, memoryview)):
        if codec is None:
            raise ValueError("read_mesh: a byte buffer needs codec='3ds', 'obj', 'off' or 'ply'")
        buf = bytes(path)
        N.check(lib.thea_mesh_read_buffer(buf, len(buf), str(codec).encode(), ctypes.byref(h)))
    else:
        N.check(lib.thea_mesh_read(str(path).encode(), ctypes.byref(h)))
    try:
        inf = N.MeshInfo()
        N.check(lib.thea_mesh_get_info(h, ctypes.byref(inf)))
        nv, nt, ns = inf.num_vertices, inf.num_triangles, inf.num_submeshes
        v = np.empty((nv, 3), np.float32)
        vs = np.empty(nv, np.int32)
        t = np.empty((nt, 3), np.int32)
        tf = np.empty(nt, np.int32)
        svo = np.empty(ns + 1, np.int64)
        sto = np.empty(ns + 1, np.int64)
        N.check(lib.thea_mesh_copy(h, v.ctypes.data, vs.ctypes.data, t.ctypes.data, tf.ctypes.data, svo.ctypes.data,
                                   sto.ctypes.data))
        return MeshData(v, vs, t, tf, svo, sto, int(inf.num_faces))
    finally:
        lib.thea_mesh_destroy(h)


def triangulate_face(positions):
    """Triangles of one polygon (positions [n, 3]) as DisplayMesh::addFace makes them: int32 [t, 3] local indices."""
    p = np.ascontiguousarray(positions, np.float32).reshape(-1, 3)
    n = len(p)
    out = np.empty((max(n - 2, 0), 3), np.int32)
    cnt = ctypes.c_int32(0)
    N.check(N.lib().thea_triangulate_face(p.ctypes.data, n, out.ctypes.data if n >= 3 else None, ctypes.byref(cnt)))
    return out[:cnt.value]


def sample_evenly_by_area(vertices, faces, num_samples, seed, rng="thea"):
    """MeshSampler::sampleEvenlyByArea (EXACT count mode) drawing from Random(seed) (rng="thea") or a counter-based
    stream (rng="counter"). Returns (positions [n, 3], face normals [n, 3], face indices [n])."""
    io = _Arrays(vertices)
    pv, nv = io.input(vertices, np.float32, 3)
    pf, nf = io.input(faces, np.int32, 3)
    pos, ppos = io.output((num_samples, 3), np.float32)
    nrm, pnrm = io.output((num_samples, 3), np.float32)
    fc, pfc = io.output((num_samples,), np.int32)
    got = ctypes.c_int64(0)
    mode = {"thea": N.RNG_THEA_MT, "counter": N.RNG_COUNTER}[rng]
    N.check(N.lib().thea_sample_by_area(pv, nv, pf, nf, int(num_samples), ctypes.c_uint32(seed), mode, ppos, pnrm, pfc,
                                        ctypes.byref(got), _stream_of(io.device)))
    g = got.value
    return pos[:g], nrm[:g], fc[:g]


def launch_count():
    return N.lib().thea_launch_count()


def profiling(enable):
    N.check(N.lib().thea_profiling_enable(1 if enable else 0))


def profiling_reset():
    N.check(N.lib().thea_profiling_reset())


def profiling_read(kernel_substring):
    ms = ctypes.c_double(0)
    cnt = ctypes.c_int64(0)
    N.check(N.lib().thea_profiling_read(kernel_substring.encode(), ctypes.byref(ms), ctypes.byref(cnt)))
    return ms.value, cnt.value
