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


def _config(width, max_leaf_size, layouts):
    cfg = N.BuildConfig()
    cfg.width = int(width)
    cfg.max_leaf_size = int(max_leaf_size)
    cfg.layouts = int(layouts)
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
                "device_error_bits": inf.device_error_bits}

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

    def __init__(self, vertices, faces, width=4, max_leaf_size=0, layouts=0):
        super().__init__()
        io = _Arrays(vertices)
        pv, nv = io.input(vertices, np.float32, 3)
        pf, nf = io.input(faces, np.int32, 3)
        cfg = _config(width, max_leaf_size, layouts)
        N.check(N.lib().thea_mesh_bvh_build(pv, nv, pf, nf, ctypes.byref(cfg), _stream_of(io.device),
                                            ctypes.byref(self._h)))

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


class PointBvh(_Bvh):
    """BVH over points (BvhN<Vector3, 3>). Element index = point index."""

    def __init__(self, points, width=4, max_leaf_size=0):
        super().__init__()
        io = _Arrays(points)
        pp, n = io.input(points, np.float32, 3)
        cfg = _config(width, max_leaf_size, 0)
        N.check(N.lib().thea_point_bvh_build(pp, n, ctypes.byref(cfg), _stream_of(io.device), ctypes.byref(self._h)))
        self.n = n

    def k_closest_pairs(self, queries, k, dist_bound=-1.0, exclude=None):
        """BvhN::kClosestPairs: (indices [n, k], squared distances [n, k]); unused slots -1."""
        io = _Arrays(queries)
        pq, n = io.input(queries, np.float32, 3)
        pe, _ = io.input(exclude, np.int32) if exclude is not None else (None, 0)
        idx, pidx = io.output((n, k), np.int32)
        d2, pd2 = io.output((n, k), np.float32)
        N.check(N.lib().thea_k_closest(self._h, pq, n, int(k), float(dist_bound), pe, pidx, pd2,
                                       _stream_of(io.device)))
        return idx, d2

    def k_closest_self(self, k, device=False):
        """k-nearest-neighbour graph of the indexed points, each excluding itself; rows in point order."""
        if device:
            import torch
            io = _Arrays(torch.empty(0, device="cuda"))
        else:
            io = _Arrays(np.empty(0))
        idx, pidx = io.output((self.n, k), np.int32)
        d2, pd2 = io.output((self.n, k), np.float32)
        N.check(N.lib().thea_k_closest_self(self._h, int(k), pidx, pd2, _stream_of(io.device)))
        return idx, d2


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
