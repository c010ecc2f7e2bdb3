"""TEST INFRASTRUCTURE ONLY -- ctypes binding of the CPU oracle (``oracle/_build/liboracle.so``).

Only the tests, ``__graft_entry__.smoke()`` and the CPU-baseline legs of ``bench.py`` may import this module. It restates
Thea's CPU spatial-query path (reference mode: the reference's kd-tree and traversal order; contract mode: lowest index
among ties) and is never used by the product path. Parity status: pinned to the reference's own code, compiled here with
an Eigen subset (oracle/reference.py; tests/test_oracle_pinned.py).
"""

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
# the same sources compiled with the reference's own release flags and nothing else (multiply-adds may fuse on hosts
# that have them): the library the CPU-baseline timings use; results are not compared bit for bit
_TIMED_PATH = os.path.join(_HERE, "_build", "liboracle_timed.so")
_lib = None
_timed = None

_f32p = ctypes.POINTER(ctypes.c_float)
_f64p = ctypes.POINTER(ctypes.c_double)
_i32p = ctypes.POINTER(ctypes.c_int32)
_u32p = ctypes.POINTER(ctypes.c_uint32)
_vp = ctypes.c_void_p
_i64 = ctypes.c_int64


def build():
    """Compile the oracle with its Makefile (idempotent)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)


def lib(timed=False):
    """The parity build of the oracle, or with timed=True the build with the reference's release flags."""
    global _lib, _timed
    if timed:
        if _timed is None:
            if not os.path.exists(_TIMED_PATH):
                build()
            _timed = _declare(ctypes.CDLL(_TIMED_PATH))
        return _timed
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        _lib = _declare(ctypes.CDLL(_LIB_PATH))
    return _lib


def _declare(L):
    """Declares the C signatures of one build of the oracle."""
    L.oracle_mesh_create.restype = _vp
    L.oracle_mesh_create.argtypes = [_f32p, _i64, _i32p, _i64, _i64, ctypes.c_int]
    L.oracle_mesh_destroy.argtypes = [_vp]
    L.oracle_mesh_num_nodes.restype = _i64
    L.oracle_mesh_num_nodes.argtypes = [_vp]
    L.oracle_mesh_max_depth.restype = _i64
    L.oracle_mesh_max_depth.argtypes = [_vp]
    L.oracle_closest_ref.argtypes = [_vp, _f32p, _i64, ctypes.c_double, _i32p, _f64p, _f32p, ctypes.c_int]
    L.oracle_closest_contract.argtypes = [_vp, _f32p, _i64, ctypes.c_double, _i32p, _f64p, _f64p, ctypes.c_int]
    L.oracle_closest_brute.argtypes = [_f32p, _i64, _i32p, _i64, _f32p, _i64, ctypes.c_double, _i32p, _f64p, _f64p,
                                       ctypes.c_int, ctypes.c_int]
    L.oracle_ray_ref.argtypes = [_vp, _f32p, _f32p, _i64, ctypes.c_float, _f32p, _i32p, _f32p, ctypes.c_int]
    L.oracle_ray_contract.argtypes = [_vp, _f32p, _f32p, _i64, ctypes.c_double, _f64p, _i32p, ctypes.c_int]
    L.oracle_ray_brute.argtypes = [_f32p, _i64, _i32p, _i64, _f32p, _f32p, _i64, ctypes.c_double, _f64p, _i32p,
                                   ctypes.c_int, ctypes.c_int]
    L.oracle_points_create.restype = _vp
    L.oracle_points_create.argtypes = [_f32p, _i64, _i64, ctypes.c_int]
    L.oracle_points_destroy.argtypes = [_vp]
    for name in ("oracle_knn_ref", "oracle_knn_contract"):
        getattr(L, name).argtypes = [_vp, _f32p, _i64, ctypes.c_int, ctypes.c_double, _i32p, _i32p, _f64p,
                                     ctypes.c_int]
    L.oracle_range_brute.argtypes = [_f32p, _i64, _f32p, _i64, ctypes.c_float, _i32p,
                                     ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64), _i32p, _f32p,
                                     ctypes.c_int]
    L.oracle_range_brute.restype = None
    L.oracle_knn_brute.argtypes = [_f32p, _i64, _f32p, _i64, ctypes.c_int, ctypes.c_double, _i32p, _i32p, _f64p,
                                   ctypes.c_int, ctypes.c_int]
    L.oracle_sample_by_area.restype = _i64
    L.oracle_sample_by_area.argtypes = [_f32p, _i64, _i32p, _i64, _i64, ctypes.c_uint32, _f32p, _f32p, _i32p]
    L.oracle_thea_random_bits.argtypes = [ctypes.c_uint32, _i64, _u32p]
    L.oracle_std_mt19937_bits.argtypes = [ctypes.c_uint32, _i64, _u32p]
    L.oracle_triangle_closest_points.argtypes = [_f32p, _f32p, _i64, _f32p, _f32p]
    L.oracle_triangle_ray_times.argtypes = [_f32p, _f32p, _f32p, _i64, ctypes.c_float, _f32p]
    L.oracle_triangle_props.argtypes = [_f32p, _i64, _f32p, _f32p, _i32p, _f32p]
    L.oracle_box_ray_time.restype = ctypes.c_float
    L.oracle_box_ray_time.argtypes = [_f32p, _f32p, _f32p, _f32p, ctypes.c_float]
    L.oracle_tree_depth.restype = _i64
    L.oracle_tree_depth.argtypes = [_i64, ctypes.c_int]
    L.oracle_random_sphere.argtypes = [ctypes.c_uint32, _i64, _f32p]
    L.oracle_sample_graph.argtypes = [_f32p, _f32p, _i64, ctypes.c_int, ctypes.c_uint32, _vp, _i32p, _f32p, _i32p,
                                      _f32p, ctypes.c_int]
    L.oracle_visibility.argtypes = [_vp, _f32p, _i64, _i64, ctypes.c_uint32, _f32p, _f64p, ctypes.c_int]
    L.oracle_shape_diameter.argtypes = [_vp, _f32p, _f32p, _i64, ctypes.c_float, ctypes.c_int, _f32p, _f64p,
                                         ctypes.c_int]
    L.oracle_affine_inverse.restype = ctypes.c_int
    L.oracle_affine_inverse.argtypes = [_f32p, _f32p]
    for name in ("oracle_affine_points", "oracle_affine_vectors", "oracle_normals_to_world"):
        getattr(L, name).argtypes = [_f32p, _f32p, _i64, _f32p]
    L.oracle_mesh_pair_contract.argtypes = [_vp, _f32p, _i32p, _i64, ctypes.c_double, _i32p, _i32p, _f64p, _f64p,
                                            _f64p, ctypes.c_int]
    L.oracle_mesh_pair_brute.argtypes = [_f32p, _i32p, _i64, _f32p, _i32p, _i64, ctypes.c_double, _i32p, _i32p, _f64p,
                                         _f64p, _f64p, ctypes.c_int, ctypes.c_int]
    L.oracle_triangle_pair_distances.argtypes = [_f32p, _f32p, _i64, _f32p, _f32p, _f32p]
    return L


def _p(a, t):
    if a is None:
        return None
    return a.ctypes.data_as(t)


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def default_threads():
    return os.cpu_count() or 1


class MeshIndex:
    """Reference kd-tree over mesh triangles (BvhN::init with Method::KDTREE, leaf size 5 by default)."""

    def __init__(self, V, F, max_leaf=-1, fp64=False, timed=False):
        self.V = _f32(V).reshape(-1, 3)
        self.F = _i32(F).reshape(-1, 3)
        self.fp64 = bool(fp64)
        self._L = lib(timed)
        self.h = self._L.oracle_mesh_create(_p(self.V, _f32p), len(self.V), _p(self.F, _i32p), len(self.F), max_leaf,
                                          int(fp64))

    def __del__(self):
        if getattr(self, "h", None) and getattr(self, "_L", None) is not None:
            self._L.oracle_mesh_destroy(self.h)
            self.h = None

    @property
    def num_nodes(self):
        return self._L.oracle_mesh_num_nodes(self.h)

    @property
    def max_depth(self):
        return self._L.oracle_mesh_max_depth(self.h)

    def closest_ref(self, q, dist_bound=-1.0, threads=None):
        """Reference mode: returns (index, distance (double, sqrt of mad), closest point (float32))."""
        q = _f32(q).reshape(-1, 3)
        n = len(q)
        idx = np.empty(n, np.int32)
        dist = np.empty(n, np.float64)
        cp = np.empty((n, 3), np.float32)
        self._L.oracle_closest_ref(self.h, _p(q, _f32p), n, float(dist_bound), _p(idx, _i32p), _p(dist, _f64p),
                                 _p(cp, _f32p), threads or default_threads())
        return idx, dist, cp

    def closest_contract(self, q, dist_bound=-1.0, threads=None):
        """Contract mode: returns (index, squared distance, closest point), lowest index among ties."""
        q = _f32(q).reshape(-1, 3)
        n = len(q)
        idx = np.empty(n, np.int32)
        d2 = np.empty(n, np.float64)
        cp = np.empty((n, 3), np.float64)
        self._L.oracle_closest_contract(self.h, _p(q, _f32p), n, float(dist_bound), _p(idx, _i32p), _p(d2, _f64p),
                                      _p(cp, _f64p), threads or default_threads())
        return idx, d2, cp

    def ray_ref(self, o, d, max_time=-1.0, threads=None):
        """Reference mode rayStructureIntersection: returns (time, index, normal); time -1 on a miss."""
        o = _f32(o).reshape(-1, 3)
        d = _f32(d).reshape(-1, 3)
        n = len(o)
        t = np.empty(n, np.float32)
        idx = np.empty(n, np.int32)
        nrm = np.empty((n, 3), np.float32)
        self._L.oracle_ray_ref(self.h, _p(o, _f32p), _p(d, _f32p), n, float(max_time), _p(t, _f32p), _p(idx, _i32p),
                             _p(nrm, _f32p), threads or default_threads())
        return t, idx, nrm

    def visibility(self, positions, num_rays, seed, transform=None, threads=None):
        """Visibility::compute per position with Random(seed) in place of Random::common() (FP32 handle only);
        transform: an affine map (3x4) set on the BVH."""
        p = _f32(positions).reshape(-1, 3)
        out = np.empty(len(p), np.float64)
        xf = _affine(transform) if transform is not None else None
        self._L.oracle_visibility(self.h, _p(p, _f32p), len(p), int(num_rays), int(seed),
                                _p(xf, _f32p) if xf is not None else None, _p(out, _f64p), threads or default_threads())
        return out

    def shape_diameter(self, positions, normals=None, scale=-1.0, only_interior=True, transform=None, threads=None):
        """ShapeDiameter::compute per position (FP32 handle; normals None: the closest element's normal, which needs
        no transform); transform: an affine map (3x4) set on the BVH."""
        p = _f32(positions).reshape(-1, 3)
        nr = _f32(normals).reshape(-1, 3) if normals is not None else None
        out = np.empty(len(p), np.float64)
        xf = _affine(transform) if transform is not None else None
        self._L.oracle_shape_diameter(self.h, _p(p, _f32p), _p(nr, _f32p) if nr is not None else None, len(p),
                                    float(scale), 1 if only_interior else 0,
                                    _p(xf, _f32p) if xf is not None else None, _p(out, _f64p),
                                    threads or default_threads())
        return out

    def closest_pair_contract(self, Vq, Fq, dist_bound=-1.0, threads=None):
        """Closest pair between this mesh (target) and a query mesh, contract mode: (query index, target index, squared
        distance, query point, target point); indices -1 when no pair."""
        Vq = _f32(Vq).reshape(-1, 3)
        Fq = _i32(Fq).reshape(-1, 3)
        qi, ti = ctypes.c_int32(-1), ctypes.c_int32(-1)
        d2 = ctypes.c_double(-1.0)
        qp, tp = np.zeros(3), np.zeros(3)
        self._L.oracle_mesh_pair_contract(self.h, _p(Vq, _f32p), _p(Fq, _i32p), len(Fq), float(dist_bound),
                                          ctypes.byref(qi), ctypes.byref(ti), ctypes.byref(d2), _p(qp, _f64p),
                                          _p(tp, _f64p), threads or default_threads())
        return qi.value, ti.value, d2.value, qp, tp

    def ray_contract(self, o, d, max_time=-1.0, threads=None):
        o = _f32(o).reshape(-1, 3)
        d = _f32(d).reshape(-1, 3)
        n = len(o)
        t = np.empty(n, np.float64)
        idx = np.empty(n, np.int32)
        self._L.oracle_ray_contract(self.h, _p(o, _f32p), _p(d, _f32p), n, float(max_time), _p(t, _f64p),
                                  _p(idx, _i32p), threads or default_threads())
        return t, idx


def closest_brute(V, F, q, dist_bound=-1.0, fp64=False, threads=None):
    V = _f32(V).reshape(-1, 3)
    F = _i32(F).reshape(-1, 3)
    q = _f32(q).reshape(-1, 3)
    n = len(q)
    idx = np.empty(n, np.int32)
    d2 = np.empty(n, np.float64)
    cp = np.empty((n, 3), np.float64)
    lib().oracle_closest_brute(_p(V, _f32p), len(V), _p(F, _i32p), len(F), _p(q, _f32p), n, float(dist_bound),
                               _p(idx, _i32p), _p(d2, _f64p), _p(cp, _f64p), int(fp64), threads or default_threads())
    return idx, d2, cp


def mesh_pair_brute(Vt, Ft, Vq, Fq, dist_bound=-1.0, fp64=False, threads=None):
    """Closest pair between two meshes by testing every triangle pair (contract mode): as closest_pair_contract."""
    Vt, Vq = _f32(Vt).reshape(-1, 3), _f32(Vq).reshape(-1, 3)
    Ft, Fq = _i32(Ft).reshape(-1, 3), _i32(Fq).reshape(-1, 3)
    qi, ti = ctypes.c_int32(-1), ctypes.c_int32(-1)
    d2 = ctypes.c_double(-1.0)
    qp, tp = np.zeros(3), np.zeros(3)
    lib().oracle_mesh_pair_brute(_p(Vt, _f32p), _p(Ft, _i32p), len(Ft), _p(Vq, _f32p), _p(Fq, _i32p), len(Fq),
                                 float(dist_bound), ctypes.byref(qi), ctypes.byref(ti), ctypes.byref(d2), _p(qp, _f64p),
                                 _p(tp, _f64p), int(fp64), threads or default_threads())
    return qi.value, ti.value, d2.value, qp, tp


def triangle_pair_distances(a, b):
    """Squared distance and closest points of triangle pairs (TriangleN::squaredDistance, a as "this"), FP32."""
    a = _f32(a).reshape(-1, 9)
    b = _f32(b).reshape(-1, 9)
    n = len(a)
    d2 = np.empty(n, np.float32)
    pa, pb = np.empty((n, 3), np.float32), np.empty((n, 3), np.float32)
    lib().oracle_triangle_pair_distances(_p(a, _f32p), _p(b, _f32p), n, _p(d2, _f32p), _p(pa, _f32p), _p(pb, _f32p))
    return d2, pa, pb


def ray_brute(V, F, o, d, max_time=-1.0, fp64=False, threads=None):
    V = _f32(V).reshape(-1, 3)
    F = _i32(F).reshape(-1, 3)
    o = _f32(o).reshape(-1, 3)
    d = _f32(d).reshape(-1, 3)
    n = len(o)
    t = np.empty(n, np.float64)
    idx = np.empty(n, np.int32)
    lib().oracle_ray_brute(_p(V, _f32p), len(V), _p(F, _i32p), len(F), _p(o, _f32p), _p(d, _f32p), n,
                           float(max_time), _p(t, _f64p), _p(idx, _i32p), int(fp64), threads or default_threads())
    return t, idx


class PointIndex:
    """Reference kd-tree over points (BvhN<Vector3, 3>)."""

    def __init__(self, P, max_leaf=-1, fp64=False, timed=False):
        self.P = _f32(P).reshape(-1, 3)
        self._L = lib(timed)
        self.h = self._L.oracle_points_create(_p(self.P, _f32p), len(self.P), max_leaf, int(fp64))

    def __del__(self):
        if getattr(self, "h", None) and getattr(self, "_L", None) is not None:
            self._L.oracle_points_destroy(self.h)
            self.h = None

    def _knn(self, fn, q, k, dist_bound, exclude, threads):
        q = _f32(q).reshape(-1, 3)
        n = len(q)
        idx = np.empty((n, k), np.int32)
        d2 = np.empty((n, k), np.float64)
        ex = None if exclude is None else _i32(exclude)
        fn(self.h, _p(q, _f32p), n, int(k), float(dist_bound), _p(ex, _i32p), _p(idx, _i32p), _p(d2, _f64p),
           threads or default_threads())
        return idx, d2

    def knn_ref(self, q, k, dist_bound=-1.0, exclude=None, threads=None):
        return self._knn(self._L.oracle_knn_ref, q, k, dist_bound, exclude, threads)

    def knn_contract(self, q, k, dist_bound=-1.0, exclude=None, threads=None):
        return self._knn(self._L.oracle_knn_contract, q, k, dist_bound, exclude, threads)


def knn_brute(P, q, k, dist_bound=-1.0, exclude=None, fp64=False, threads=None):
    P = _f32(P).reshape(-1, 3)
    q = _f32(q).reshape(-1, 3)
    n = len(q)
    idx = np.empty((n, k), np.int32)
    d2 = np.empty((n, k), np.float64)
    ex = None if exclude is None else _i32(exclude)
    lib().oracle_knn_brute(_p(P, _f32p), len(P), _p(q, _f32p), n, int(k), float(dist_bound), _p(ex, _i32p),
                           _p(idx, _i32p), _p(d2, _f64p), int(fp64), threads or default_threads())
    return idx, d2


def range_brute(P, q, radius, exclude=None, threads=None):
    """Every point within `radius` (inclusive, FP32) of each query, by brute force: CSR (offsets, indices, d2)."""
    P = _f32(P).reshape(-1, 3)
    q = _f32(q).reshape(-1, 3)
    n = len(q)
    ex = None if exclude is None else _i32(exclude)
    i64p = ctypes.POINTER(ctypes.c_int64)
    counts = np.zeros(n, np.int64)
    lib().oracle_range_brute(_p(P, _f32p), len(P), _p(q, _f32p), n, float(radius), _p(ex, _i32p), _p(counts, i64p),
                             None, None, None, threads or default_threads())
    off = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
    idx = np.empty(int(off[-1]), np.int32)
    d2 = np.empty(int(off[-1]), np.float32)
    if len(idx):
        lib().oracle_range_brute(_p(P, _f32p), len(P), _p(q, _f32p), n, float(radius), _p(ex, _i32p), None,
                                 _p(off, i64p), _p(idx, _i32p), _p(d2, _f32p), threads or default_threads())
    return off, idx, d2


def sample_by_area(V, F, n, seed):
    """MeshSampler::sampleEvenlyByArea (EXACT) with Random(seed): returns (positions, face normals, face indices)."""
    V = _f32(V).reshape(-1, 3)
    F = _i32(F).reshape(-1, 3)
    pos = np.empty((n, 3), np.float32)
    nrm = np.empty((n, 3), np.float32)
    face = np.empty(n, np.int32)
    got = lib().oracle_sample_by_area(_p(V, _f32p), len(V), _p(F, _i32p), len(F), int(n), ctypes.c_uint32(seed),
                                      _p(pos, _f32p), _p(nrm, _f32p), _p(face, _i32p))
    return pos[:got], nrm[:got], face[:got]


def thea_random_bits(seed, n):
    out = np.empty(n, np.uint32)
    lib().oracle_thea_random_bits(ctypes.c_uint32(seed), n, _p(out, _u32p))
    return out


def std_mt19937_bits(seed, n):
    out = np.empty(n, np.uint32)
    lib().oracle_std_mt19937_bits(ctypes.c_uint32(seed), n, _p(out, _u32p))
    return out


def triangle_closest_points(tris, p):
    tris = _f32(tris).reshape(-1, 9)
    p = _f32(p).reshape(-1, 3)
    n = len(p)
    cp = np.empty((n, 3), np.float32)
    d2 = np.empty(n, np.float32)
    lib().oracle_triangle_closest_points(_p(tris, _f32p), _p(p, _f32p), n, _p(cp, _f32p), _p(d2, _f32p))
    return cp, d2


def triangle_ray_times(tris, o, d, max_time=-1.0):
    tris = _f32(tris).reshape(-1, 9)
    o = _f32(o).reshape(-1, 3)
    d = _f32(d).reshape(-1, 3)
    n = len(o)
    t = np.empty(n, np.float32)
    lib().oracle_triangle_ray_times(_p(tris, _f32p), _p(o, _f32p), _p(d, _f32p), n, float(max_time), _p(t, _f32p))
    return t


def triangle_props(tris):
    tris = _f32(tris).reshape(-1, 9)
    n = len(tris)
    nrm = np.empty((n, 3), np.float32)
    dist = np.empty(n, np.float32)
    axis = np.empty(n, np.int32)
    area = np.empty(n, np.float32)
    lib().oracle_triangle_props(_p(tris, _f32p), n, _p(nrm, _f32p), _p(dist, _f32p), _p(axis, _i32p), _p(area, _f32p))
    return nrm, dist, axis, area


def tree_depth(n, max_leaf=5):
    return lib().oracle_tree_depth(int(n), int(max_leaf))


# ---------------------------------------------------------------------------------------------------------------------
# Affine transforms (BvhN::setTransform semantics): row-major 3x4 [L | t] in FP32
# ---------------------------------------------------------------------------------------------------------------------

def _affine(m):
    m = _f32(m)
    if m.shape == (4, 4):
        m = np.ascontiguousarray(m[:3])
    return m.reshape(3, 4)


def affine_inverse(m):
    """AffineTransformN::inverse in FP32 (Eigen's 3x3 cofactor inverse); None if the linear part is singular."""
    m = _affine(m)
    inv = np.empty((3, 4), np.float32)
    return inv if lib().oracle_affine_inverse(_p(m, _f32p), _p(inv, _f32p)) else None


def _apply(name, m, v):
    m = _affine(m)
    v = _f32(v).reshape(-1, 3)
    out = np.empty_like(v)
    getattr(lib(), name)(_p(m, _f32p), _p(v, _f32p), len(v), _p(out, _f32p))
    return out


def affine_points(m, p):
    """L p + t per point (AffineTransformN::operator*)."""
    return _apply("oracle_affine_points", m, p)


def affine_vectors(m, v):
    """L v per vector (the linear part, as for ray directions)."""
    return _apply("oracle_affine_vectors", m, v)


def normals_to_world(inv, n):
    """normalToWorldSpace: (L^-1)^T n normalised, with inv the inverse transform."""
    return _apply("oracle_normals_to_world", inv, n)


def random_sphere(seed, n):
    """Random(seed).sphere() directions in stream order (Knop's method)."""
    out = np.empty((int(n), 3), np.float32)
    lib().oracle_random_sphere(int(seed), int(n), _p(out, _f32p))
    return out


def sample_graph(P, N=None, max_degree=8, seed=0, surface=None, threads=None):
    """PointSet3::updateGraph (no oversampling) with Random(seed): (neighbours, separations, degrees, (estimate, final
    mean separation)); surface: a MeshIndex for the reachability test (used with normals)."""
    P = _f32(P).reshape(-1, 3)
    n = len(P)
    Nn = _f32(N).reshape(-1, 3) if N is not None else None
    nbr = np.empty((n, max_degree), np.int32)
    sep = np.empty((n, max_degree), np.float32)
    deg = np.empty(n, np.int32)
    avg = np.empty(2, np.float32)
    lib().oracle_sample_graph(_p(P, _f32p), _p(Nn, _f32p), n, int(max_degree), int(seed),
                              surface.h if surface is not None else None, _p(nbr, _i32p), _p(sep, _f32p),
                              _p(deg, _i32p), _p(avg, _f32p), threads or default_threads())
    return nbr, sep, deg, (float(avg[0]), float(avg[1]))


def sample_graph_oversampled(P, N, D, DN, max_degree=8, seed=0, surface=None, threads=None):
    """PointSet3::updateGraph with a dense oversampling D (normals DN, used when N is given): the graph of sample_graph
    over P followed by D, then extractOriginalAdjacencies (PointSet3.cpp:157-176): per sample, Dijkstra over that graph
    (edge lengths the separations, summed in double; ties settle the lowest index) until max_degree other samples of P
    are settled; separations the path lengths as float, neighbours in (separation, index) order. Returns the outputs of
    sample_graph for P (the estimate over P and D, the final mean over P's new neighbours)."""
    import heapq
    P = _f32(P).reshape(-1, 3)
    D = _f32(D).reshape(-1, 3)
    n, m = len(P), int(max_degree)
    agg = np.concatenate([P, D])
    aggn = np.concatenate([_f32(N).reshape(-1, 3), _f32(DN).reshape(-1, 3)]) if N is not None else None
    nbr, sep, deg, (est, _) = sample_graph(agg, aggn, m, seed, surface, threads)
    out_n = np.full((n, m), -1, np.int32)
    out_s = np.zeros((n, m), np.float32)
    out_d = np.zeros(n, np.int32)
    for src in range(n):
        dist = {src: 0.0}
        done = set()
        heap = [(0.0, src)]
        found = []
        while heap:
            d, v = heapq.heappop(heap)
            if v in done or d > dist[v]:
                continue
            done.add(v)
            if v != src and v < n:
                found.append((np.float32(d), v))
                if len(found) >= m:
                    break
            for k in range(int(deg[v])):
                u = int(nbr[v, k])
                nd = d + float(sep[v, k])
                if u not in done and nd < dist.get(u, np.inf):
                    dist[u] = nd
                    heapq.heappush(heap, (nd, u))
        found.sort()
        out_d[src] = len(found)
        for k, (sp, v) in enumerate(found):
            out_n[src, k] = v
            out_s[src, k] = sp
    # updateAverageSeparation (PointSet3.hpp:688-702): a float sum in sample order
    avg = np.float32(0)
    edges = 0
    for i in range(n):
        for k in range(int(out_d[i])):
            avg = np.float32(avg + out_s[i, k])
        edges += int(out_d[i])
    if edges:
        avg = np.float32(avg / np.float32(edges))
    return out_n, out_s, out_d, (est, float(avg))


def best_fit_sphere(P):
    """BestFitSphereN<3> (Algorithms/BestFitSphereN.hpp:62-91): the smallest ball enclosing the points, computed in
    double from the float coordinates as the reference's miniball is. This restatement uses Welzl's move-to-front
    recursion (Gaertner's form: the support set grows by the point found outside, the loop restarts over the points
    before it), not the reference's pivoting code; the ball is unique, so both give it up to rounding. Non-finite
    points are skipped; no points give the zero ball at the origin. Returns (centre float64 [3], radius float)."""
    pts = [tuple(float(x) for x in p) for p in np.asarray(P, np.float32).reshape(-1, 3) if np.all(np.isfinite(p))]
    if not pts:
        return np.zeros(3), 0.0

    def ball_of(sup):
        # the ball through the support points with its centre in their affine hull
        p0 = np.array(sup[0])
        if len(sup) == 1:
            return p0, 0.0
        v = np.array(sup[1:]) - p0
        A = 2.0 * v @ v.T
        b = (v * v).sum(1)
        lam = np.linalg.solve(A, b)
        c = p0 + lam @ v
        return c, max(float(((np.array(s) - c) ** 2).sum()) for s in sup)

    def outside(p, c, r2):
        d = (p[0] - c[0]) ** 2 + (p[1] - c[1]) ** 2 + (p[2] - c[2]) ** 2
        return d > r2 * (1.0 + 1e-12) + 1e-300

    def mtf(end, sup):
        c, r2 = ball_of(sup) if sup else (np.zeros(3), -1.0)
        if len(sup) == 4:
            return c, r2
        i = 0
        while i < end:
            p = pts[i]
            if outside(p, c, r2):
                c, r2 = mtf(i, sup + [p])
                pts.insert(0, pts.pop(i))  # move to front
            i += 1
        return c, r2

    c, r2 = mtf(len(pts), [])
    return np.asarray(c, np.float64), float(np.sqrt(max(r2, 0.0)))
