"""CPU tests of the C ABI: the library builds for sm_103a, loads, exports every symbol the header declares, and rejects
bad arguments before touching the device."""

import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

from tests.conftest import ROOT

HEADER = os.path.join(ROOT, "include", "thea_gpu.h")


def declared_symbols():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"THEA_API\s+[^;(]*?\b(thea_\w+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    from thea_gb300 import build as B
    B.build()
    from thea_gb300 import _native as N
    return N.lib()


def test_header_declares_the_query_api():
    names = declared_symbols()
    for required in ("thea_mesh_bvh_build", "thea_point_bvh_build", "thea_closest_element", "thea_ray_intersection",
                     "thea_k_closest", "thea_k_closest_self", "thea_sample_by_area", "thea_bvh_destroy"):
        assert required in names


def test_library_exports_every_declared_symbol(lib):
    from thea_gb300 import _native as N
    out = subprocess.run(["nm", "-D", "--defined-only", N.LIB_PATH], capture_output=True, text=True, check=True).stdout
    exported = set(line.split()[-1] for line in out.splitlines() if " T " in line)
    missing = [s for s in declared_symbols() if s not in exported]
    assert not missing, missing
    # and nothing else of ours leaks
    extra = sorted(s for s in exported if s.startswith("thea_") and s not in declared_symbols())
    assert not extra, extra
    # the ctypes signature table covers the header
    assert sorted(N.SIGNATURES) == declared_symbols()


def test_library_is_built_for_sm_103a(lib):
    # ptxas -v reports the target of every compiled entry function in the build logs
    from thea_gb300 import build as B
    logs = [os.path.join(B.BUILD, f[:-3] + ".log") for f in B.sources()]
    with_kernels = 0
    for log in logs:
        text = open(log).read()
        assert "arch=compute_103a,code=sm_103a" in text.splitlines()[0]
        targets = set(re.findall(r"Compiling entry function '\w+' for '(\w+)'", text))
        assert targets <= {"sm_103a"}, (log, targets)
        with_kernels += bool(targets)
    host_only = {"serialize.cu", "mesh_io.cu"}  # image and mesh-file I/O: host code only
    assert with_kernels >= len(logs) - len(host_only)


def test_status_strings_and_version(lib):
    assert lib.thea_abi_version() == 1
    assert lib.thea_status_string(0) == b"ok"
    assert lib.thea_status_string(1) == b"invalid argument"
    assert lib.thea_status_string(99) == b"unknown status"


def test_invalid_arguments_are_rejected_without_a_device(lib):
    from thea_gb300 import _native as N
    h = ctypes.c_void_p()
    assert lib.thea_mesh_bvh_build(None, 3, None, 1, None, None, ctypes.byref(h)) == 1
    assert b"null" in lib.thea_last_error_message()
    V = np.zeros((3, 3), np.float32)
    assert lib.thea_mesh_bvh_build(V.ctypes.data, 0, V.ctypes.data, 1, None, None, ctypes.byref(h)) == 1
    cfg = N.BuildConfig()
    cfg.reserved[0] = 7
    assert lib.thea_point_bvh_build(V.ctypes.data, 3, ctypes.byref(cfg), None, ctypes.byref(h)) == 1
    assert lib.thea_closest_element(None, None, 0, -1.0, None, None, None, None) == 1
    assert lib.thea_ray_intersection(None, None, None, 0, -1.0, None, None, None, None) == 1
    assert lib.thea_k_closest(None, None, 0, 4, -1.0, None, None, None, None) == 1
    assert lib.thea_k_closest_self(None, 4, None, None, None) == 1
    assert lib.thea_sample_by_area(None, 0, None, 0, 5, 1, 9, None, None, None, None, None) == 1
    assert lib.thea_bvh_destroy(None) == 0
    # occlusion, visibility, sphere stream and sample graph: argument checks before any device call
    P = np.zeros((4, 3), np.float32)
    out = np.zeros(64, np.int32)
    assert lib.thea_ray_intersects(None, None, None, 0, -1.0, None, None) == 1
    assert lib.thea_visibility(None, P.ctypes.data, 4, 10, 1, None, None) == 1
    assert lib.thea_random_sphere(1, -1, None, None) == 1
    assert lib.thea_random_sphere(1, 0, None, None) == 0
    assert lib.thea_sample_graph(None, None, 4, 8, 1, None, out.ctypes.data, None, None, None, None) == 1
    assert lib.thea_sample_graph(P.ctypes.data, None, 1, 8, 1, None, out.ctypes.data, None, None, None, None) == 1
    assert lib.thea_sample_graph(P.ctypes.data, None, 4, 0, 1, None, out.ctypes.data, None, None, None, None) == 1
    assert lib.thea_sample_graph(P.ctypes.data, None, 4, 65, 1, None, out.ctypes.data, None, None, None, None) == 1
    # shape diameter and pairs between BVHs
    sd = np.zeros(4, np.float64)
    assert lib.thea_shape_diameter(None, P.ctypes.data, None, 4, -1.0, 1, sd.ctypes.data, None) == 1
    qi, ti, d2 = ctypes.c_int32(7), ctypes.c_int32(7), ctypes.c_float(0)
    assert lib.thea_bvh_closest_pair(None, None, -1.0, ctypes.byref(qi), ctypes.byref(ti), ctypes.byref(d2), None,
                                     None, None) == 1
    assert qi.value == -1 and ti.value == -1
    assert lib.thea_bvh_k_closest_pairs(None, None, 0, -1.0, out.ctypes.data, out.ctypes.data, out.ctypes.data, None,
                                        None) == 1
    eye = np.eye(3, 4, dtype=np.float32)
    assert lib.thea_bvh_set_transform(None, eye.ctypes.data, None) == 1
    assert lib.thea_bvh_clear_transform(None) == 1
    assert lib.thea_bvh_get_transform(None, None, None, None) == 1
    with pytest.raises(N.TheaError):
        N.check(lib.thea_k_closest_self(None, 4, None, None, None))


def test_profiling_and_launch_counter_without_device(lib):
    before = lib.thea_launch_count()
    assert lib.thea_profiling_enable(1) == 0
    assert lib.thea_profiling_reset() == 0
    ms = ctypes.c_double(-1)
    cnt = ctypes.c_int64(-1)
    assert lib.thea_profiling_read(b"nothing", ctypes.byref(ms), ctypes.byref(cnt)) == 0
    assert ms.value == 0 and cnt.value == 0
    assert lib.thea_profiling_enable(0) == 0
    assert lib.thea_launch_count() == before


def test_cpp_wrapper_compiles():
    """The header-only C++ wrapper (reference method names over the C ABI) compiles and links against the library."""
    from thea_gb300 import build as B
    B.build()
    src = os.path.join(ROOT, "tests", "cpp", "wrapper_compile.cpp")
    out = os.path.join(ROOT, "tests", "cpp", "_build", "wrapper_compile")
    os.makedirs(os.path.dirname(out), exist_ok=True)
    r = subprocess.run(["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"), src, "-o", out,
                        "-L", os.path.join(ROOT, "thea_gb300", "_lib"), "-lthea_gpu",
                        "-Wl,-rpath," + os.path.join(ROOT, "thea_gb300", "_lib")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([out, "--no-device"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr


def _image_header(version=1, width=4, n=4, num_nodes=1, segments=1, is_mesh=1, layouts=3, sections=None):
    """A serialized-BVH header (the fixed layout thea_bvh_serialize writes), for rejection tests without a device."""
    import struct
    node, cp, ray, pt = sections if sections is not None else (num_nodes * 128, n * 128, n * 48, 0)
    return struct.pack("<8sI5iIi3q6f4q2i12f", b"THEABVH\0", version, is_mesh, width, 4, 1, 0, layouts, segments, n,
                       num_nodes, 0, 0, 0, 0, 1, 1, 1, node, cp, ray, pt, 0, 0, *([0.0] * 12))


def test_bvh_images_are_checked_before_any_device_call(lib):
    """thea_bvh_deserialize refuses foreign, newer, inconsistent and truncated images with INVALID_ARGUMENT, and
    never allocates for them (no device here)."""
    from thea_gb300 import MeshBvh, PointBvh
    from thea_gb300 import _native as N
    h = ctypes.c_void_p()
    size = ctypes.c_int64()
    assert lib.thea_bvh_serialize(None, None, 0, ctypes.byref(size), None) == N.THEA_ERR_INVALID_ARGUMENT
    cases = {
        "not a BVH image": b"x" * 256,
        "buffer shorter than a header": _image_header()[:40],
        "version 2 is not supported": _image_header(version=2) + bytes(4096),
        "inconsistent header": _image_header(width=5) + bytes(4096),
        "inconsistent section sizes": _image_header(sections=(128, 4 * 128, 0, 0)) + bytes(4096),
        "shorter than the image": _image_header() + bytes(64),
    }
    for why, img in cases.items():
        buf = ctypes.create_string_buffer(img, len(img))
        assert lib.thea_bvh_deserialize(buf, len(img), None, ctypes.byref(h)) == N.THEA_ERR_INVALID_ARGUMENT, why
        assert why.encode() in lib.thea_last_error_message(), (why, lib.thea_last_error_message())
        assert not h.value
    for cls in (MeshBvh, PointBvh):
        with pytest.raises(N.TheaError):
            cls.from_bytes(b"")


# Every entry point of the C ABI. A new declaration in the header must be added here too (and to the integration
# table beside the reference interface it replaces).
ENTRY_POINTS = sorted("""
thea_abi_version thea_status_string thea_last_error_message thea_launch_count thea_allocation_count
thea_profiling_enable thea_profiling_reset thea_profiling_read
thea_mesh_bvh_build thea_point_bvh_build thea_bvh_destroy thea_bvh_get_info
thea_bvh_serialize thea_bvh_deserialize thea_bvh_set_transform thea_bvh_clear_transform thea_bvh_get_transform
thea_closest_element thea_closest_element_ex thea_ray_intersection thea_ray_intersection_ex thea_ray_intersects
thea_random_sphere thea_visibility thea_sample_graph thea_sample_graph_oversampled thea_k_closest thea_radius_neighbors
thea_k_closest_self thea_k_closest_self_ex thea_point_gram_tile thea_selftest_bounded_wait thea_selftest_set_error_bits
thea_selftest_running_sum
thea_sample_by_area thea_sample_by_area_noalloc
thea_mesh_forest_build thea_point_forest_build thea_batch_closest_element thea_batch_ray_intersection
thea_batch_k_closest thea_autotune_batch_closest
thea_graph_capture_begin thea_graph_capture_end thea_graph_launch thea_graph_destroy
thea_server_create thea_server_destroy thea_server_add_mesh thea_server_remove_mesh thea_server_submit
thea_server_wait thea_server_cancel thea_server_get_stats thea_server_reset_stats
thea_shape_diameter thea_best_fit_sphere thea_bvh_closest_pair thea_bvh_k_closest_pairs
thea_mesh_read thea_mesh_read_buffer thea_mesh_get_info thea_mesh_copy thea_mesh_destroy thea_triangulate_face
""".split())


def test_header_declares_exactly_the_listed_entry_points():
    """The header's declarations are the list above, each preceded by a comment that says what it does."""
    assert declared_symbols() == ENTRY_POINTS
    text = open(HEADER).read()
    for name in ENTRY_POINTS:
        m = re.search(r"THEA_API\s+[^;(]*?\b%s\s*\(" % name, text)
        before = text[:m.start()].rstrip()
        assert before.endswith("*/") or re.search(r"THEA_API[^;]*;\s*$", before), name