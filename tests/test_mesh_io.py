"""CPU tests of the mesh-file readers and face triangulation (host code of the library) against the pure-Python
restatement in oracle/mesh_oracle.py, plus hand-derived answers for small cases."""

import struct

import numpy as np
import pytest

from oracle import mesh_oracle as MO


@pytest.fixture(scope="module")
def T():
    from thea_gb300 import build as B
    B.build()
    import thea_gb300
    return thea_gb300


def _lib_tris(T, pts):
    return [tuple(int(x) for x in t) for t in T.triangulate_face(np.asarray(pts, np.float32))]


def _same_mesh(got, want):
    np.testing.assert_array_equal(got.vertices, want["vertices"])
    np.testing.assert_array_equal(got.vertex_source, want["vertex_source"])
    np.testing.assert_array_equal(got.triangles, want["triangles"])
    np.testing.assert_array_equal(got.triangle_face, want["triangle_face"])
    np.testing.assert_array_equal(got.submesh_vertex_offsets, want["submesh_vertex_offsets"])
    np.testing.assert_array_equal(got.submesh_triangle_offsets, want["submesh_triangle_offsets"])
    assert got.num_faces == want["num_faces"]


# ---- triangulation ---------------------------------------------------------------------------------------------------

def test_known_triangulations(T):
    sq = [(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0)]
    assert _lib_tris(T, sq) == MO.triangulate_face(sq) == [(0, 1, 2), (2, 3, 0)]
    # a dart whose diagonal 0-2 lies outside: the quad splits along 1-3
    dart = [(0, 0, 0), (2, 1, 0), (0, 2, 0), (1, 1, 0)]
    assert _lib_tris(T, dart) == MO.triangulate_face(dart) == [(1, 2, 3), (3, 0, 1)]
    # collinear quad: no triangle; half-degenerate quad: one
    line = [(0, 0, 0), (1, 0, 0), (2, 0, 0), (3, 0, 0)]
    assert _lib_tris(T, line) == MO.triangulate_face(line) == []
    half = [(0, 0, 0), (1, 0, 0), (2, 0, 0), (1, 1, 0)]
    assert _lib_tris(T, half) == MO.triangulate_face(half) == [(2, 3, 0)]
    # convex counter-clockwise pentagon: ears (4, 0, 1), (1, 2, 3), (3, 4, 1)
    pent = [(np.cos(a), np.sin(a), 0.0) for a in np.arange(5) * 2 * np.pi / 5]
    assert _lib_tris(T, pent) == MO.triangulate_face(pent) == [(4, 0, 1), (1, 2, 3), (3, 4, 1)]
    # the same pentagon clockwise: the polygon is walked reversed and each triangle emitted reversed
    cw = pent[::-1]
    assert _lib_tris(T, cw) == MO.triangulate_face(cw)
    assert len(_lib_tris(T, cw)) == 3
    # fewer than three vertices and a plain triangle
    assert _lib_tris(T, pent[:2]) == [] and _lib_tris(T, pent[:3]) == [(0, 1, 2)]


def _random_polygon(rng, n, concave):
    ang = np.sort(rng.uniform(0, 2 * np.pi, n))
    rad = rng.uniform(0.3, 1.0, n) if concave else np.ones(n)
    xy = np.stack([rad * np.cos(ang), rad * np.sin(ang), np.zeros(n)], 1)
    if rng.random() < 0.5:
        xy = xy[::-1]
    q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
    return (xy @ q.T * rng.uniform(0.01, 100) + rng.normal(size=3) * 10).astype(np.float32)


@pytest.mark.parametrize("concave", [False, True])
def test_random_polygons_match_the_restatement(T, concave):
    rng = np.random.default_rng(11 + concave)
    for _ in range(400):
        n = int(rng.integers(3, 13))
        p = _random_polygon(rng, n, concave)
        got, want = _lib_tris(T, p), MO.triangulate_face(p)
        assert got == want, (p.tolist(), got, want)
        if not concave:
            assert len(got) == n - 2


def test_degenerate_polygons_match_the_restatement(T):
    rng = np.random.default_rng(5)
    for _ in range(200):
        n = int(rng.integers(4, 9))
        p = _random_polygon(rng, n, True)
        k = int(rng.integers(0, n))
        p[(k + 1) % n] = p[k]                      # a repeated vertex
        if rng.random() < 0.3:
            p[:, 2] = p[0, 2]; p[:, 1] = p[0, 1]   # all collinear
        assert _lib_tris(T, p) == MO.triangulate_face(p)


# ---- OFF -------------------------------------------------------------------------------------------------------------

OFF_TEXT = """OFF
# a comment, then a blank line

7 8 0
0 0 0
1 0 0
1 1 0
0 1 0
2 0.5 0.25
# another comment
1.5 2 1e-3
-1 -1 -1
4 0 1 2 3
3 1 4 2
5 0 1 4 5 3
3 0 1 9
3 0 1 1
2 0 1
0
6 0 1 4 2 5 6 7 8
"""


def test_off_ascii(T, tmp_path):
    path = tmp_path / "m.off"
    path.write_bytes(OFF_TEXT.replace("\n", "\r\n").encode())
    m = T.read_mesh(str(path))
    _same_mesh(m, MO.read_mesh(str(path)))
    assert m.vertices.shape == (7, 3) and m.vertex_source.tolist() == list(range(7))
    # faces 0 (quad), 1 (triangle), 2 (pentagon) and 7 (hexagon; extra indices on the line are ignored) produce
    # triangles; 3 (index out of range), 4 (repeated vertex), 5 (two vertices) and 6 (empty) do not
    assert sorted(set(m.triangle_face.tolist())) == [0, 1, 2, 7]
    assert m.triangles[:2].tolist() == [[0, 1, 2], [2, 3, 0]] and m.triangles[2].tolist() == [1, 4, 2]
    assert m.num_faces == 4 and m.submesh_triangle_offsets.tolist() == [0, len(m.triangle_face)]


def _binary_off(nv_list, faces, trailing=b""):
    b = b"OFF BINARY\n" + struct.pack(">iii", len(nv_list), len(faces), 0)
    for v in nv_list:
        b += struct.pack(">fff", *v)
    for f in faces:
        b += f
    return b + trailing


def test_off_binary(T, tmp_path):
    V = [(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0), (0.5, 2, 0.5)]
    faces = [
        struct.pack(">iiiii", 4, 0, 1, 2, 3) + struct.pack(">i", 0),            # quad, no colour
        struct.pack(">iiii", 3, 1, 4, 2) + struct.pack(">ifff", 3, 1, 0, 0),    # triangle with an RGB colour
        struct.pack(">iiii", 3, 0, 0, 2) + struct.pack(">i", 0),                # repeated vertex: skipped
        # an out-of-range index ends the face's indices; the next word (index 1) is taken as the colour count and
        # skips the real colour count, so the stream stays aligned
        struct.pack(">iiii", 3, 0, 99, 1) + struct.pack(">i", 0),
        struct.pack(">iiii", 3, 2, 3, 4) + struct.pack(">i", 0),
    ]
    path = tmp_path / "m.off"
    path.write_bytes(_binary_off(V, faces))
    m = T.read_mesh(str(path))
    _same_mesh(m, MO.read_mesh(str(path)))
    assert m.triangle_face.tolist() == [0, 0, 1, 4]
    assert m.triangles.tolist() == [[0, 1, 2], [2, 3, 0], [1, 4, 2], [2, 3, 4]]


def test_off_errors(T, tmp_path):
    from thea_gb300 import TheaError
    bad = tmp_path / "bad.off"
    bad.write_text("COFF\n1 0 0\n0 0 0\n")
    with pytest.raises(TheaError, match="does not start with 'OFF'"):
        T.read_mesh(str(bad))
    short = tmp_path / "short.off"
    short.write_text("OFF\n3 1 0\n0 0 0\n1 0 0\n")
    with pytest.raises(TheaError, match="end of input"):
        T.read_mesh(str(short))
    empty = tmp_path / "empty.off"
    empty.write_text("OFF\n0 0 0\n")
    m = T.read_mesh(str(empty))
    assert m.vertices.shape == (0, 3) and m.submesh_triangle_offsets.tolist() == [0]
    for name in ("m.ply", "m.3ds", "m.stl"):
        (tmp_path / name).write_text("x")
        with pytest.raises(TheaError):
            T.read_mesh(str(tmp_path / name))
    with pytest.raises(TheaError, match="cannot open"):
        T.read_mesh(str(tmp_path / "missing.obj"))


# ---- OBJ -------------------------------------------------------------------------------------------------------------

OBJ_TEXT = """# header comment
mtllib ignored.mtl
v 0 0 0
v 1 0 0
v 1 1 0
v 0 1 0
v 2 0.5 0.5
vt 0 0
vt 1 0
vt 1 1
vn 0 0 1
vn 0 0 -1
f 1/1/1 2/2/1 3/3/1 4/1/1
f 2//2 5//2 3//2
usemtl whatever
g second
f -1 -4 -3
f 1/2 2/3 5/1 3/2 4/3
p 1
f 1 0 2
f 1 2 7
o third
f 1 2 2
f 1 2 3 4/9/9
g
s off
f 4 3 2
"""


def test_obj_groups_and_references(T, tmp_path):
    path = tmp_path / "m.obj"
    path.write_text(OBJ_TEXT)
    m = T.read_mesh(str(path))
    want = MO.read_mesh(str(path))
    _same_mesh(m, want)
    # the first submesh's vertices are its distinct (v, t, n) references in ascending order: (1,1,1) (2,0,2) (2,2,1)
    # (3,0,2) (3,3,1) (4,1,1) (5,0,2)
    s0 = slice(m.submesh_vertex_offsets[0], m.submesh_vertex_offsets[1])
    assert m.vertex_source[s0].tolist() == [0, 1, 1, 2, 2, 3, 4]
    # four submeshes: the anonymous one, 'second', 'third' and the bare 'g'. Faces are numbered over the whole file;
    # the bad faces (index 0, index 7) are not numbered, the point 'p 1' (face 4) is but makes no triangle, and the
    # degenerate 'f 1 2 2' (face 5) is kept as a triangle
    assert m.submesh_triangle_offsets.tolist()[0] == 0 and len(m.submesh_triangle_offsets) == 5
    assert sorted(set(m.triangle_face.tolist())) == [0, 1, 2, 3, 5, 6, 7]


def test_obj_drops_groups_without_triangles(T, tmp_path):
    path = tmp_path / "m.obj"
    path.write_text("v 0 0 0\nv 1 0 0\nv 2 0 0\nv 0 1 0\ng a\nf 1 2 3 1/1\np 4\ng b\nf 1 2 4\n")
    m = T.read_mesh(str(path))
    _same_mesh(m, MO.read_mesh(str(path)))
    # group a: a quad whose references 1 and 1/1 are the same vertex (no texture coordinates exist, so /1 is dropped)
    # is collinear, and a point: no triangle, so the group is dropped; group b's face is the file's third
    assert m.submesh_vertex_offsets.tolist() == [0, 3] and m.triangle_face.tolist() == [2]


def _random_obj(rng, n_vertices, n_faces):
    V = rng.normal(size=(n_vertices, 3)).astype(np.float32)
    lines = ["v %.9g %.9g %.9g" % tuple(v) for v in V] + ["vt 0.5 0.5", "vn 0 0 1"]
    for f in range(n_faces):
        if rng.random() < 0.05:
            lines.append("g grp%d" % f)
        k = int(rng.integers(1, 9))
        ids = rng.choice(n_vertices, size=k, replace=False) + 1
        forms = ["%d", "%d/1", "%d//1", "%d/1/1"]
        fields = []
        for i in ids:
            i = int(i) if rng.random() < 0.8 else int(i) - n_vertices - 1   # some negative references
            fields.append(forms[int(rng.integers(0, 4))] % i)
        lines.append(("p " if k == 1 else "f ") + " ".join(fields))
    return "\n".join(lines) + "\n"


def test_random_obj_matches_the_restatement(T, tmp_path):
    rng = np.random.default_rng(3)
    for trial in range(6):
        path = tmp_path / ("r%d.obj" % trial)
        path.write_text(_random_obj(rng, 60, 300))
        _same_mesh(T.read_mesh(str(path)), MO.read_mesh(str(path)))


def test_random_off_matches_the_restatement(T, tmp_path):
    rng = np.random.default_rng(4)
    for trial in range(4):
        V = rng.normal(size=(50, 3)).astype(np.float32)
        lines = ["OFF", "50 200 0"] + ["%.9g %.9g %.9g" % tuple(v) for v in V]
        for _ in range(200):
            k = int(rng.integers(1, 8))
            ids = rng.integers(0, 52, size=k)   # some out of range, some repeated
            lines.append(" ".join(str(int(x)) for x in [k, *ids]))
        path = tmp_path / ("r%d.off" % trial)
        path.write_text("\n".join(lines) + "\n")
        _same_mesh(T.read_mesh(str(path)), MO.read_mesh(str(path)))


# ---- PLY -------------------------------------------------------------------------------------------------------------

PLY_ASCII = """ply
format ascii 1.0
comment made by hand
element vertex 6
property float x
property float y
property float z
property uchar red
element edge 1
property int vertex1
property int vertex2
element face 6
property list uchar int vertex_indices
property float quality
end_header
0 0 0 255
1 0 0 0
comment inside the data
1 1 0 7

0 1 0 1
2 0.5 0.25 3
1.5 2 1e-3 9
0 1
4 0 1 2 3 0.5
3 1 4 2
5 0 1 4 5 3 0.25
3 0 1 9
3 0 0 1
2 0 1
"""


def test_ply_ascii(T, tmp_path):
    path = tmp_path / "m.ply"
    path.write_text(PLY_ASCII)
    m = T.read_mesh(str(path))
    _same_mesh(m, MO.read_mesh(str(path)))
    # the out-of-range and repeated faces are not handed to the mesh, so they take no face number; the two-vertex face
    # does (number 3) but makes no triangle
    assert m.vertex_source.tolist() == list(range(6))
    assert m.triangle_face.tolist() == [0, 0, 1, 2, 2, 2] and m.num_faces == 3
    assert m.triangles[:3].tolist() == [[0, 1, 2], [2, 3, 0], [1, 4, 2]]


def _ply_binary(order, verts, faces, extra_vertex_props=True, edges=True):
    e = "binary_little_endian" if order == "<" else "binary_big_endian"
    head = ["ply", "format %s 1.0" % e, "element vertex %d" % len(verts), "property double x", "property double y",
            "property double z"]
    if extra_vertex_props:
        head += ["property float nx", "property list uchar float extra", "property uchar red"]
    if edges:
        head += ["element edge 1", "property int a", "property int b"]
    head += ["element face %d" % len(faces), "property list uchar uint vertex_indices", "property short flags",
             "end_header"]
    b = ("\n".join(head) + "\n").encode()
    for i, v in enumerate(verts):
        b += struct.pack(order + "ddd", *v)
        if extra_vertex_props:
            n = i % 3
            b += struct.pack(order + "fB" + "f" * n + "B", 1.0, n, *([2.0] * n), 200)
    if edges:
        b += struct.pack(order + "ii", 0, 1)
    for f in faces:
        b += struct.pack(order + "B" + "I" * len(f) + "h", len(f), *f, -3)
    return b


@pytest.mark.parametrize("order", ["<", ">"])
@pytest.mark.parametrize("extras", [False, True])
def test_ply_binary(T, tmp_path, order, extras):
    rng = np.random.default_rng(9)
    V = [tuple(x) for x in rng.normal(size=(12, 3))]
    F = [[0, 1, 2], [2, 3, 4, 5], [5, 6, 7, 8, 9], [0, 99, 1], [1, 1, 2], [], [3, 4], [9, 10, 11, 0, 1, 2]]
    path = tmp_path / "m.ply"
    path.write_bytes(_ply_binary(order, V, F, extras, extras))
    m = T.read_mesh(str(path))
    _same_mesh(m, MO.read_mesh(str(path)))
    np.testing.assert_array_equal(m.vertices, np.asarray(V, np.float64).astype(np.float32))
    # faces handed to the mesh: 0, 1, 2, the two-vertex face (3) and the hexagon (4)
    assert sorted(set(m.triangle_face.tolist())) == [0, 1, 2, 4]


def test_ply_errors(T, tmp_path):
    from thea_gb300 import TheaError
    cases = {
        "ply\nformat ascii 1.0\nelement vertex 1\nproperty float x\n": "end_header",
        "ply\nformat text 1.0\nend_header\n": "format specifier",
        "ply\nformat ascii 1.0\nelement vertex 1\nproperty float x\nproperty float y\nend_header\n0 0\n": "three",
        "ply\nformat ascii 1.0\nelement face 1\nproperty float q\nend_header\n1\n": "list of integer",
        "ply\nformat ascii 1.0\nelement vertex 1\nproperty half x\nend_header\n": "unknown property type",
        "ply\nformat ascii 1.0\nelement vertex 2\nproperty float x\nproperty float y\nproperty float z\n"
        "end_header\n0 0 0\n": "end of input",
        "plx\n": "does not start with 'ply'",
    }
    for i, (text, msg) in enumerate(cases.items()):
        path = tmp_path / ("e%d.ply" % i)
        path.write_text(text)
        with pytest.raises(TheaError, match=msg):
            T.read_mesh(str(path))


def test_off_bin_extension(T, tmp_path):
    V = [(0, 0, 0), (1, 0, 0), (0, 1, 0)]
    path = tmp_path / "m.off.bin"
    path.write_bytes(_binary_off(V, [struct.pack(">iiiii", 3, 0, 1, 2, 0)]))
    m = T.read_mesh(str(path))
    assert m.triangles.tolist() == [[0, 1, 2]]


def test_sample_model_fixture(golden_dir):
    """The fixture of the reference's sample meshes (tests/golden/make_model_fixtures.py) is self-consistent."""
    import os
    z = np.load(os.path.join(golden_dir, "models.npz"))
    for name, nv, nt in (("cube", 8, 12), ("sphere", 946, 1888), ("teapot", 3644, 6320)):
        V, F = z[name + "_vertices"], z[name + "_triangles"]
        assert V.shape == (nv, 3) and F.shape == (nt, 3)
        assert F.min() >= 0 and F.max() < nv
        assert z[name + "_submesh_triangle_offsets"][-1] == nt and len(z[name + "_sha256"]) == 32


def test_ply_binary_list_longer_than_the_file(T, tmp_path):
    from thea_gb300 import TheaError
    head = b"ply\nformat binary_little_endian 1.0\nelement vertex 3\nproperty float x\nproperty float y\n" \
           b"property float z\nelement face 1\nproperty list uint int vertex_indices\nend_header\n"
    body = struct.pack("<9f", 0, 0, 0, 1, 0, 0, 0, 1, 0) + struct.pack("<I", 4000000000) + struct.pack("<3i", 0, 1, 2)
    path = tmp_path / "long.ply"
    path.write_bytes(head + body)
    with pytest.raises(TheaError, match="end of input"):
        T.read_mesh(str(path))


def test_number_syntax_follows_stream_extraction(T, tmp_path):
    """Coordinates parse as successive std::istream >> double reads do: a leading '+', an underflow to zero and junk
    after the last number are accepted; "inf", "nan", a lone exponent, "+-", an overflow and junk before the next
    number are errors, as they are for the reference's reader."""
    from thea_gb300 import TheaError
    ok = tmp_path / "ok.obj"
    ok.write_text("v +2.5 1e-400 -0\nv 1 2 3x\nv .5 5. 1E+2\nf 1 2 3\n")
    m = T.read_mesh(str(ok))
    np.testing.assert_array_equal(m.vertices, np.array([[2.5, 0, -0.0], [1, 2, 3], [0.5, 5, 100]], np.float32))
    assert np.signbit(m.vertices[0, 2])
    for i, bad in enumerate(("v inf 0 0", "v nan 0 0", "v 1e 0 0", "v 1e+ 0 0", "v +-1 0 0", "v 1e400 0 0",
                             "v 1.5e3x 2 3")):
        path = tmp_path / ("bad%d.obj" % i)
        path.write_text(bad + "\n")
        with pytest.raises(TheaError, match="vertex position"):
            T.read_mesh(str(path))
    # OFF counts and indices as std::istream >> long long: '+' accepted, overflow rejected
    off = tmp_path / "plus.off"
    off.write_text("OFF\n+3 +1 0\n0 0 0\n1 0 0\n0 1 0\n3 +0 1 2\n")
    assert T.read_mesh(str(off)).triangles.tolist() == [[0, 1, 2]]
    big = tmp_path / "big.off"
    big.write_text("OFF\n99999999999999999999 1 0\n")
    with pytest.raises(TheaError, match="statistics"):
        T.read_mesh(str(big))


def test_read_from_memory(T, tmp_path):
    path = tmp_path / "m.obj"
    path.write_text(OBJ_TEXT)
    a = T.read_mesh(str(path))
    b = T.read_mesh(OBJ_TEXT.encode(), codec="obj")
    np.testing.assert_array_equal(a.triangles, b.triangles)
    np.testing.assert_array_equal(a.vertices, b.vertices)
    c = T.read_mesh(PLY_ASCII.encode(), codec="PLY")
    assert len(c.triangles) == 6
    from thea_gb300 import TheaError
    with pytest.raises(TheaError, match="unknown codec"):
        T.read_mesh(b"x", codec="stl")
    with pytest.raises(ValueError):
        T.read_mesh(b"x")


# ---- 3DS -------------------------------------------------------------------------------------------------------------

def _chunk(cid, payload):
    return struct.pack("<HI", cid, 6 + len(payload)) + payload


def _tri_object(points, faces, extra=b"", texels=None):
    body = _chunk(0x4110, struct.pack("<H", len(points)) + b"".join(struct.pack("<3f", *p) for p in points))
    if texels is not None:
        body += _chunk(0x4140, struct.pack("<H", len(texels)) + b"".join(struct.pack("<2f", *t) for t in texels))
    smoothing = _chunk(0x4150, b"\0" * 4 * len(faces))
    body += _chunk(0x4120, struct.pack("<H", len(faces)) + b"".join(struct.pack("<4H", *f, 7) for f in faces) + smoothing)
    body += _chunk(0x4160, struct.pack("<12f", *range(12)))   # mesh matrix: not applied
    return _chunk(0x4100, body + extra)


def _named(name, *subchunks):
    return _chunk(0x4000, name + b"\0" + b"".join(subchunks))


def _file_3ds(*objects, top=0x4D4D, keyframer=True):
    editor = _chunk(0x3D3E, struct.pack("<I", 3)) + _chunk(0xAFFF, _chunk(0xA000, b"mat\0")) + b"".join(objects)
    body = _chunk(0x0002, struct.pack("<I", 3)) + _chunk(0x3D3D, editor)
    if keyframer:
        body += _chunk(0xB000, _chunk(0xB00A, b"\0" * 10))
    return _chunk(top, body)


def test_3ds_meshes_sorted_by_name_and_numbered_over_the_file(T, tmp_path):
    sq = [(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0)]
    data = _file_3ds(
        _named(b"zeta", _tri_object(sq, [(0, 1, 2), (0, 2, 3)])),
        _named(b"Light01", _chunk(0x4600, struct.pack("<3f", 1, 2, 3))),           # a light: no mesh
        _named(b"alpha", _tri_object(sq[:3], [(0, 1, 5), (0, 0, 1), (2, 1, 0)], texels=[(0, 0)] * 3)),
        _named(b"empty", _tri_object([], [])),                                     # no points: skipped
        _named(b"points", _tri_object([(5, 5, 5)], [])),                           # points only: kept
        _named(b"alpha", _tri_object([(0, 0, 2), (1, 0, 2), (0, 1, 2)], [(0, 1, 2)])))
    path = tmp_path / "m.3ds"
    path.write_bytes(data)
    m = T.read_mesh(str(path))
    _same_mesh(m, MO.read_mesh(str(path)))
    # lib3ds order: alpha (first in the file), alpha (second), points, zeta
    assert m.submesh_vertex_offsets.tolist() == [0, 3, 6, 7, 11]
    assert m.submesh_triangle_offsets.tolist() == [0, 1, 2, 2, 4]
    # alpha's faces 0 (index 5) and 1 (repeated index) are skipped but numbered; zeta's faces are numbers 4 and 5
    assert m.triangle_face.tolist() == [2, 3, 4, 5]
    assert m.triangles.tolist() == [[2, 1, 0], [3, 4, 5], [7, 8, 9], [7, 9, 10]]
    assert m.vertex_source.tolist() == list(range(11)) and m.num_faces == 4
    np.testing.assert_array_equal(m.vertices[6], [5, 5, 5])
    # the same bytes through the buffer entry point, and a file that is only the editor chunk
    _same_mesh(T.read_mesh(data, codec="3ds"), MO.read_mesh(str(path)))
    bare = data[6 + 10:]                       # skip the file header and the version chunk
    bare = bare[:struct.unpack_from("<I", bare, 2)[0]]
    _same_mesh(T.read_mesh(bare, codec="3DS"), MO.read_mesh(str(path)))


def test_random_3ds_matches_the_restatement(T, tmp_path):
    rng = np.random.default_rng(5)
    for trial in range(6):
        objects = []
        for o in range(int(rng.integers(1, 7))):
            nv = int(rng.integers(0, 40))
            pts = [tuple(float(x) for x in rng.normal(size=3).astype(np.float32)) for _ in range(nv)]
            faces = [tuple(int(x) for x in rng.integers(0, nv + 3, size=3)) for _ in range(int(rng.integers(0, 60)))]
            name = bytes(rng.choice(list(b"abAB_\xe9"), size=int(rng.integers(0, 4))).tolist())
            objects.append(_named(name, _tri_object(pts, faces)))
        path = tmp_path / ("r%d.3ds" % trial)
        path.write_bytes(_file_3ds(*objects, top=[0x4D4D, 0xC23D][trial % 2], keyframer=trial % 3 != 0))
        _same_mesh(T.read_mesh(str(path)), MO.read_mesh(str(path)))


def test_3ds_errors(T, tmp_path):
    good = _file_3ds(_named(b"a", _tri_object([(0, 0, 0), (1, 0, 0), (0, 1, 0)], [(0, 1, 2)])))
    cases = {
        "unknown top chunk": _chunk(0x1234, b""),
        "truncated": good[:-5],
        "chunk past parent": good[:2] + struct.pack("<I", len(good) + 10) + good[6:],
        "long name": _file_3ds(_named(b"n" * 64, _tri_object([(0, 0, 0)], []))),
        "short point array": _file_3ds(_named(b"a", _chunk(0x4100, _chunk(0x4110, struct.pack("<H", 3) + b"\0" * 24)))),
    }
    for why, data in cases.items():
        path = tmp_path / "bad.3ds"
        path.write_bytes(data)
        with pytest.raises(Exception):
            T.read_mesh(str(path))
        with pytest.raises(ValueError):
            MO.read_mesh(str(path))
    path = tmp_path / "ok63.3ds"
    path.write_bytes(_file_3ds(_named(b"n" * 63, _tri_object([(0, 0, 0), (1, 0, 0), (0, 1, 0)], [(0, 1, 2)]))))
    assert T.read_mesh(str(path)).triangles.tolist() == [[0, 1, 2]]
