"""TEST INFRASTRUCTURE ONLY -- ctypes binding of the reference's own spatial-query code (``oracle/_ref/libthea_ref.so``).

The library is compiled by ``oracle/Makefile`` (target ``ref``) from the reference's sources where they lie (BvhN,
Triangle3, AxisAlignedBoxN, Random, Math, ... under Code/Source) with ``oracle/ref_pin/eigen_subset.hpp`` standing in for
Eigen, which is absent here. It pins the oracle: ``tests/golden/make_ref_golden.py`` records its outputs as fixtures and
the CPU tests compare the oracle's reference mode with them (and with the library itself where it was built). It exists
only where the reference sources do; nothing on the GPU path or in the timed benchmark uses it.
"""

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_ref", "libthea_ref.so")
_lib = None

_f32p = ctypes.POINTER(ctypes.c_float)
_f64p = ctypes.POINTER(ctypes.c_double)
_i32p = ctypes.POINTER(ctypes.c_int32)
_u32p = ctypes.POINTER(ctypes.c_uint32)
_vp = ctypes.c_void_p
_i64 = ctypes.c_int64


def build():
    """Compile the reference library (needs the reference sources; see oracle/Makefile)."""
    subprocess.run(["make", "-s", "-C", _HERE, "ref"], check=True)


def available():
    return os.path.exists(LIB_PATH)


def lib():
    global _lib
    if _lib is None:
        L = ctypes.CDLL(LIB_PATH)
        L.ref_mesh_create.restype = _vp
        L.ref_mesh_create.argtypes = [_f32p, _i64, _i32p, _i64]
        L.ref_mesh_destroy.argtypes = [_vp]
        L.ref_closest.argtypes = [_vp, _f32p, _i64, ctypes.c_double, _i32p, _f64p, _f32p]
        L.ref_ray.argtypes = [_vp, _f32p, _f32p, _i64, ctypes.c_float, _f32p, _i32p, _f32p]
        L.ref_mesh_pair.restype = ctypes.c_int32
        L.ref_mesh_pair.argtypes = [_vp, _vp, ctypes.c_double, _i32p, _i32p, _f64p, _f32p, _f32p]
        L.ref_points_create.restype = _vp
        L.ref_points_create.argtypes = [_f32p, _i64]
        L.ref_points_destroy.argtypes = [_vp]
        L.ref_knn.argtypes = [_vp, _f32p, _i64, ctypes.c_int, ctypes.c_double, _i32p, _i32p, _f64p]
        L.ref_triangle_closest_points.argtypes = [_f32p, _f32p, _i64, _f32p]
        L.ref_triangle_pair_distances.argtypes = [_f32p, _f32p, _i64, _f32p, _f32p, _f32p]
        L.ref_triangle_ray_times.argtypes = [_f32p, _f32p, _f32p, _i64, ctypes.c_float, _f32p]
        L.ref_random_bits.argtypes = [ctypes.c_uint32, _i64, _u32p]
        L.ref_tree_depth.restype = _i64
        L.ref_tree_depth.argtypes = [_i64, ctypes.c_int]
        L.ref_best_fit_sphere.argtypes = [_f32p, _i64, _f32p, _f32p]
        _lib = L
    return _lib


def _p(a, t):
    return None if a is None else a.ctypes.data_as(t)


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


class Mesh:
    """The reference's BvhN<Triangle3, 3> over the triangles of a mesh (element i = triangle i)."""

    def __init__(self, V, F):
        self.V, self.F = _f32(V).reshape(-1, 3), _i32(F).reshape(-1, 3)
        self.h = lib().ref_mesh_create(_p(self.V, _f32p), len(self.V), _p(self.F, _i32p), len(self.F))

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.ref_mesh_destroy(self.h)
            self.h = None

    def closest(self, q, dist_bound=-1.0):
        """closestElement<MetricL2>: (index, distance (double), closest point (float32))."""
        q = _f32(q).reshape(-1, 3)
        n = len(q)
        idx, dist, cp = np.empty(n, np.int32), np.empty(n, np.float64), np.empty((n, 3), np.float32)
        lib().ref_closest(self.h, _p(q, _f32p), n, float(dist_bound), _p(idx, _i32p), _p(dist, _f64p), _p(cp, _f32p))
        return idx, dist, cp

    def ray(self, o, d, max_time=-1.0):
        """rayStructureIntersection<RayIntersectionTester>: (time, index, normal); -1 on a miss."""
        o, d = _f32(o).reshape(-1, 3), _f32(d).reshape(-1, 3)
        n = len(o)
        t, idx, nrm = np.empty(n, np.float32), np.empty(n, np.int32), np.empty((n, 3), np.float32)
        lib().ref_ray(self.h, _p(o, _f32p), _p(d, _f32p), n, float(max_time), _p(t, _f32p), _p(idx, _i32p),
                      _p(nrm, _f32p))
        return t, idx, nrm

    def closest_pair(self, query, dist_bound=-1.0):
        """closestPair<MetricL2> with another Mesh as the query: (query index, target index, squared distance,
        query point, target point), indices -1 when no pair."""
        qi, ti, mad = ctypes.c_int32(-1), ctypes.c_int32(-1), ctypes.c_double(-1)
        qp, tp = np.zeros(3, np.float32), np.zeros(3, np.float32)
        lib().ref_mesh_pair(self.h, query.h, float(dist_bound), ctypes.byref(qi), ctypes.byref(ti), ctypes.byref(mad),
                            _p(qp, _f32p), _p(tp, _f32p))
        return qi.value, ti.value, mad.value, qp, tp


class Points:
    """The reference's BvhN over pointers to points (as PointSet3 builds it)."""

    def __init__(self, P):
        self.P = _f32(P).reshape(-1, 3)
        self.h = lib().ref_points_create(_p(self.P, _f32p), len(self.P))

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.ref_points_destroy(self.h)
            self.h = None

    def knn(self, q, k, dist_bound=-1.0, exclude=None):
        """kClosestPairs<MetricL2> with PointSet3's self filter: (indices [n, k], squared distances [n, k]), -1 past
        the neighbours found."""
        q = _f32(q).reshape(-1, 3)
        n = len(q)
        idx, mad = np.empty((n, k), np.int32), np.empty((n, k), np.float64)
        ex = None if exclude is None else _i32(exclude)
        lib().ref_knn(self.h, _p(q, _f32p), n, int(k), float(dist_bound), _p(ex, _i32p), _p(idx, _i32p),
                      _p(mad, _f64p))
        return idx, mad


def triangle_closest_points(tris, p):
    tris, p = _f32(tris).reshape(-1, 9), _f32(p).reshape(-1, 3)
    cp = np.empty((len(p), 3), np.float32)
    lib().ref_triangle_closest_points(_p(tris, _f32p), _p(p, _f32p), len(p), _p(cp, _f32p))
    return cp


def triangle_pair_distances(a, b):
    a, b = _f32(a).reshape(-1, 9), _f32(b).reshape(-1, 9)
    n = len(a)
    d2, pa, pb = np.empty(n, np.float32), np.empty((n, 3), np.float32), np.empty((n, 3), np.float32)
    lib().ref_triangle_pair_distances(_p(a, _f32p), _p(b, _f32p), n, _p(d2, _f32p), _p(pa, _f32p), _p(pb, _f32p))
    return d2, pa, pb


def triangle_ray_times(tris, o, d, max_time=-1.0):
    tris, o, d = _f32(tris).reshape(-1, 9), _f32(o).reshape(-1, 3), _f32(d).reshape(-1, 3)
    t = np.empty(len(o), np.float32)
    lib().ref_triangle_ray_times(_p(tris, _f32p), _p(o, _f32p), _p(d, _f32p), len(o), float(max_time), _p(t, _f32p))
    return t


def random_bits(seed, n):
    out = np.empty(n, np.uint32)
    lib().ref_random_bits(int(seed), int(n), _p(out, _u32p))
    return out


def tree_depth(n, max_leaf=5):
    return lib().ref_tree_depth(int(n), int(max_leaf))


def best_fit_sphere(P):
    """BestFitSphereN<3> of the points: (centre float32 [3], radius float32), the reference's Real."""
    P = _f32(P)
    c = np.zeros(3, np.float32)
    r = np.zeros(1, np.float32)
    lib().ref_best_fit_sphere(_p(P, _f32p), len(P), _p(c, _f32p), _p(r, _f32p))
    return c, float(r[0])
