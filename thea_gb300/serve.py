"""Serving loop over resident meshes (thea_server_* in ``include/thea_gpu.h``).

A :class:`Server` keeps built BVHs of its meshes in device memory, admits requests by a memory budget and batches
pending closest-point / ray / k-NN requests as they arrive (continuous batching on a few streams). Request arrays are
NumPy arrays (host memory, pinned or not) or CUDA tensors; the server holds a reference to them until the request has
been waited for.
"""

import ctypes

import numpy as np

from . import _native as N

KINDS = {"closest": N.REQUEST_CLOSEST, "ray": N.REQUEST_RAY, "knn": N.REQUEST_KNN}


def _ptr(a):
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        return a.ctypes.data
    return a.data_ptr()


class Ticket:
    """One submitted request: its id and the arrays it reads and writes."""

    def __init__(self, server, tid, kind, arrays):
        self.server, self.id, self.kind, self.arrays = server, tid, kind, arrays
        self.status = None
        self.latency_ms = None

    @property
    def index(self):
        return self.arrays["out_index"]

    @property
    def value(self):
        return self.arrays["out_value"]

    @property
    def point(self):
        return self.arrays.get("out_point")

    def wait(self, timeout_us=-1):
        """Blocks until the request ends (or the timeout passes: returns False). Returns True when it ended; its
        outcome is then in ``status`` (a THEA status code) and ``latency_ms``."""
        if self.status is not None:
            return True
        st = ctypes.c_int(0)
        lat = ctypes.c_double(0.0)
        r = N.lib().thea_server_wait(self.server._h, self.id, int(timeout_us), ctypes.byref(st), ctypes.byref(lat))
        if r == N.THEA_ERR_WAIT_TIMEOUT:
            return False
        N.check(r)
        self.status, self.latency_ms = st.value, lat.value
        return True

    def cancel(self):
        N.check(N.lib().thea_server_cancel(self.server._h, self.id))


class Server:
    def __init__(self, memory_budget_bytes=0, slots=0, max_batch_queries=0, max_piece_queries=0, precision="fp32",
                 width=4, max_leaf_size=0, small_request_queries=0, max_wait_ms=0, test_executor=False,
                 test_ns_per_query=0, hard_query_budget=0):
        cfg = N.ServerConfig()
        cfg.memory_budget_bytes = int(memory_budget_bytes)
        cfg.slots = int(slots)
        cfg.max_batch_queries = int(max_batch_queries)
        cfg.max_piece_queries = int(max_piece_queries)
        cfg.precision = {"fp32": N.PRECISION_FP32_REFERENCE, "fp64": N.PRECISION_FP64_RECHECK}[precision]
        cfg.width = int(width)
        cfg.max_leaf_size = int(max_leaf_size)
        cfg.small_request_queries = int(small_request_queries)
        cfg.max_wait_ms = int(max_wait_ms)
        cfg.test_executor = 1 if test_executor else 0
        cfg.test_ns_per_query = int(test_ns_per_query)
        cfg.hard_query_budget = int(hard_query_budget)
        self._h = ctypes.c_void_p()
        N.check(N.lib().thea_server_create(ctypes.byref(cfg), ctypes.byref(self._h)))

    def close(self):
        if self._h:
            N.check(N.lib().thea_server_destroy(self._h))
            self._h = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add_mesh(self, vertices, faces):
        """Builds and keeps resident one mesh (arrays on the host or CUDA tensors); returns its id."""
        if isinstance(vertices, np.ndarray):
            vertices = np.ascontiguousarray(vertices, dtype=np.float32)
            faces = np.ascontiguousarray(faces, dtype=np.int32)
        else:
            import torch
            vertices = vertices.to(torch.float32).contiguous()
            faces = faces.to(torch.int32).contiguous()
        mid = ctypes.c_int32(-1)
        N.check(N.lib().thea_server_add_mesh(self._h, ctypes.c_void_p(_ptr(vertices)), vertices.shape[0],
                                             ctypes.c_void_p(_ptr(faces)), faces.shape[0], ctypes.byref(mid)))
        return mid.value

    def remove_mesh(self, mesh):
        N.check(N.lib().thea_server_remove_mesh(self._h, int(mesh)))

    def submit(self, kind, mesh, queries, directions=None, bound=-1.0, k=1, closest_points=False, out=None):
        """Queues a request and returns its :class:`Ticket`. Outputs are allocated beside the queries (host or device)
        unless ``out`` gives (index, value[, point])."""
        n = queries.shape[0]
        rows = k if kind == "knn" else 1
        host = isinstance(queries, np.ndarray)
        arrays = {"queries": queries, "directions": directions}
        if out is not None:
            arrays["out_index"], arrays["out_value"] = out[0], out[1]
            if len(out) > 2:
                arrays["out_point"] = out[2]
        elif host:
            arrays["out_index"] = np.empty((n, rows) if kind == "knn" else n, np.int32)
            arrays["out_value"] = np.empty((n, rows) if kind == "knn" else n, np.float32)
            if kind == "closest" and closest_points:
                arrays["out_point"] = np.empty((n, 3), np.float32)
        else:
            import torch
            shape = (n, rows) if kind == "knn" else (n,)
            arrays["out_index"] = torch.empty(shape, dtype=torch.int32, device=queries.device)
            arrays["out_value"] = torch.empty(shape, dtype=torch.float32, device=queries.device)
            if kind == "closest" and closest_points:
                arrays["out_point"] = torch.empty((n, 3), dtype=torch.float32, device=queries.device)
        r = N.Request()
        r.type = KINDS[kind]
        r.mesh = int(mesh)
        r.num_queries = n
        r.queries = _ptr(queries)
        r.directions = _ptr(directions)
        r.bound = float(bound)
        r.k = int(k)
        r.out_index = _ptr(arrays["out_index"])
        r.out_value = _ptr(arrays["out_value"])
        r.out_point = _ptr(arrays.get("out_point"))
        tid = ctypes.c_uint64(0)
        N.check(N.lib().thea_server_submit(self._h, ctypes.byref(r), ctypes.byref(tid)))
        return Ticket(self, tid.value, kind, arrays)

    def stats(self):
        s = N.ServerStats()
        N.check(N.lib().thea_server_get_stats(self._h, ctypes.byref(s)))
        return {name: getattr(s, name) for name, _ in N.ServerStats._fields_}

    def reset_stats(self):
        N.check(N.lib().thea_server_reset_stats(self._h))
