"""TEST INFRASTRUCTURE ONLY -- pure-Python restatement of Thea's mesh-file readers and face triangulation.

Only the tests may import this module; the product reads mesh files in C++ (thea_gb300/csrc/mesh_io.cu). It restates,
in FP32 with one rounding per operation (numpy float32 scalars) and Eigen's 3-term reduction order e0 + (e1 + e2):

- DisplayMesh::addFace (Graphics/DisplayMesh.cpp:249-320): < 3 vertices skipped, triangles kept, quads by
  Polygon3::triangulateQuad (Polygon3.hpp:245-285), larger faces by Polygon3::triangulate (Polygon3.cpp:179-288) with
  Polygon3::computeNormal (Polygon3.hpp:180-208) and Math::orthonormalBasis (MatrixUtil.hpp:225-249);
- the non-strict OFF reader (Graphics/MeshCodecOff.hpp:154-330, ASCII and big-endian binary);
- the OBJ reader with texcoords and normals read (Graphics/MeshCodecObj.hpp:210-545): a submesh per g/o group whose
  vertices are the distinct (v, t, n) references of its faces in ascending order;
- the PLY reader (Graphics/MeshCodecPly.hpp:229-700), ASCII and binary; binary properties and elements beyond the
  vertex coordinates and the face index list are skipped as the header describes them.
- the 3DS reader (Graphics/MeshCodec3ds.hpp:160-395) over lib3ds 1.3.0, a third-party library that is not part of
  the reference: lib3ds keeps the file's triangle meshes in a list sorted by object name (a new mesh goes after every
  mesh whose name is not greater, as strcmp orders them), each mesh being the N_TRI_OBJECT chunk (0x4100) of a named
  object (0x4000) of the editor chunk (0x3D3D), with its points in POINT_ARRAY (0x4110) and faces in FACE_ARRAY
  (0x4120); the codec, with its default options, skips meshes without points, applies no transforms, and skips (but
  numbers) faces with an out-of-range or repeated index, numbering vertices and faces over the whole file.

Small inputs only (pure-Python loops). Parity status: unpinned (the reference's readers cannot be built here).
"""

import struct

import numpy as np

f32 = np.float32
EPS = f32(1.1920928955078125e-07)


def _v(p):
    return (f32(p[0]), f32(p[1]), f32(p[2]))


def _sub(a, b):
    return (a[0] - b[0], a[1] - b[1], a[2] - b[2])


def _cross(a, b):
    return (a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0])


def _dot(a, b):
    return a[0] * b[0] + (a[1] * b[1] + a[2] * b[2])


def _normalized(a):
    z = _dot(a, a)
    if z > 0:
        r = np.sqrt(z)
        return (a[0] / r, a[1] / r, a[2] / r)
    return a


def _max_abs_axis(a):
    m, best = 0, abs(a[0])
    if abs(a[1]) > best:
        m, best = 1, abs(a[1])
    if abs(a[2]) > best:
        m = 2
    return m


def triangulate_quad(p0, p1, p2, p3):
    """Polygon3::triangulateQuad: list of local index triples (0, 1 or 2 of them)."""
    p0, p1, p2, p3 = _v(p0), _v(p1), _v(p2), _v(p3)
    n0 = _cross(_sub(p1, p0), _sub(p2, p0))
    n1 = _cross(_sub(p2, p0), _sub(p3, p0))
    if _dot(n0, n1) < 0:
        n0 = _cross(_sub(p2, p1), _sub(p3, p1))
        n1 = _cross(_sub(p3, p1), _sub(p0, p1))
        t0, t1 = (1, 2, 3), (3, 0, 1)
    else:
        t0, t1 = (0, 1, 2), (2, 3, 0)
    e2 = EPS * EPS
    d0, d1 = _dot(n0, n0) < e2, _dot(n1, n1) < e2
    if d0:
        return [] if d1 else [t1]
    return [t0] if d1 else [t0, t1]


def _poly_normal(p):
    n = len(p)
    p0, p1 = p[0], p[1]
    i2 = 2 % n
    for _ in range(n):
        p2 = p[i2]
        nrm = _cross(_sub(p2, p1), _sub(p0, p1))
        if _dot(nrm, nrm) >= f32(1e-10):
            return _normalized(nrm)
        p0, p1 = p1, p2
        i2 = (i2 + 1) % n
    return (f32(0), f32(0), f32(0))


def _inside(A, B, C, P):
    ax, ay = C[0] - B[0], C[1] - B[1]
    bx, by = A[0] - C[0], A[1] - C[1]
    cx, cy = B[0] - A[0], B[1] - A[1]
    apx, apy = P[0] - A[0], P[1] - A[1]
    bpx, bpy = P[0] - B[0], P[1] - B[1]
    cpx, cpy = P[0] - C[0], P[1] - C[1]
    return ax * bpy - ay * bpx >= 0 and bx * cpy - by * cpx >= 0 and cx * apy - cy * apx >= 0


def triangulate_polygon(points):
    """Polygon3::triangulate (ear clipping in the polygon's plane): list of local index triples."""
    p = [_v(x) for x in points]
    n = len(p)
    normal = _poly_normal(p)
    w = _normalized(normal)
    if _max_abs_axis(normal) == 0:
        u = _normalized((normal[1], -normal[0], f32(0)))
    else:
        u = _normalized((f32(0), normal[2], -normal[1]))
    v = _cross(w, u)
    q = []
    for x in p:
        d = _sub(x, p[0])
        q.append((_dot(d, u), _dot(d, v)))
    area = f32(0)
    a = n - 1
    for b in range(n):
        area = area + (q[a][0] * q[b][1] - q[b][0] * q[a][1])
        a = b
    area = f32(0.5) * area
    flipped = not (area > 0)
    idx = list(range(n - 1, -1, -1)) if flipped else list(range(n))
    out = []
    nv = n
    count = 2 * nv
    cur = nv - 1
    while nv > 2:
        if count == 0:
            break
        count -= 1
        a = cur if cur < nv else 0
        cur = a + 1 if a + 1 < nv else 0
        c = cur + 1 if cur + 1 < nv else 0
        A, B, C = q[idx[a]], q[idx[cur]], q[idx[c]]
        ear = not (EPS > ((B[0] - A[0]) * (C[1] - A[1]) - (B[1] - A[1]) * (C[0] - A[0])))
        if ear:
            for k in range(nv):
                if k not in (a, cur, c) and _inside(A, B, C, q[idx[k]]):
                    ear = False
                    break
        if ear:
            t = (idx[a], idx[cur], idx[c])
            out.append(t[::-1] if flipped else t)
            del idx[cur]
            nv -= 1
            count = 2 * nv
    return out


def triangulate_face(points):
    """DisplayMesh::addFace's triangles of one face: list of local index triples."""
    n = len(points)
    if n < 3:
        return []
    if n == 3:
        return [(0, 1, 2)]
    if n == 4:
        return triangulate_quad(*points)
    return triangulate_polygon(points)


class _Mesh:
    def __init__(self):
        self.vertices, self.vertex_source, self.triangles, self.triangle_face = [], [], [], []
        self.sv, self.st = [0], [0]
        self.num_faces = 0

    def arrays(self):
        return {"vertices": np.array(self.vertices, np.float32).reshape(-1, 3),
                "vertex_source": np.array(self.vertex_source, np.int32),
                "triangles": np.array(self.triangles, np.int32).reshape(-1, 3),
                "triangle_face": np.array(self.triangle_face, np.int32),
                "submesh_vertex_offsets": np.array(self.sv, np.int64),
                "submesh_triangle_offsets": np.array(self.st, np.int64), "num_faces": self.num_faces}


def _add_submesh(m, verts, sources, faces, keep_empty=False):
    """One display mesh: its vertices, then each (local indices, source face) in order."""
    base = len(m.vertex_source)
    tris, tface, nfaces = [], [], 0
    for local, src in faces:
        tt = triangulate_face([verts[i] for i in local])
        for t in tt:
            tris.append(tuple(base + local[k] for k in t))
            tface.append(src)
        nfaces += 1 if tt else 0
    if nfaces == 0 and not keep_empty:
        return
    for x, s in zip(verts, sources):
        m.vertices.extend(x)
        m.vertex_source.append(s)
    m.triangles.extend(tris)
    m.triangle_face.extend(tface)
    m.num_faces += nfaces
    m.sv.append(len(m.vertex_source))
    m.st.append(len(m.triangle_face))


def _int_prefix(s, i):
    """std::istream >> long long on s[i:] without leading whitespace: (value, next position) or (None, i)."""
    j = i
    if j < len(s) and s[j] in "+-":
        j += 1
    k = j
    while k < len(s) and s[k].isdigit():
        k += 1
    if k == j:
        return None, i
    return int(s[i:k]), k


def read_off(data):
    """The non-strict OFF reader on the bytes of a file: dict of arrays as thea_mesh_copy returns them."""
    m = _Mesh()
    nl = data.find(b"\n")
    header = (data if nl < 0 else data[:nl]).decode("latin-1").strip()
    if header != "OFF" and not header.startswith("OFF "):
        raise ValueError("not an OFF file")
    rest = b"" if nl < 0 else data[nl + 1:]
    if header == "OFF BINARY" or header.startswith("OFF BINARY "):
        return _read_off_binary(m, rest)
    lines = iter(rest.decode("latin-1").split("\n"))

    def data_line():
        for ln in lines:
            ln = ln.strip()
            if ln and ln[0] != "#":
                return ln
        raise ValueError("unexpected end of input")

    nv, nf, _ = (int(x) for x in data_line().split()[:3])
    if nv <= 0:
        return m.arrays()
    verts = []
    for _ in range(nv):
        x = data_line().split()
        verts.append(tuple(f32(float(t)) for t in x[:3]))
    faces = []
    for f in range(nf):
        tok = data_line().split()
        k = int(tok[0])
        if k <= 0:
            continue
        face, skip = [], False
        for j in range(k):
            if j + 1 >= len(tok):
                skip = True
                break
            idx = int(tok[j + 1])
            if idx < 0 or idx >= nv or idx in face:
                skip = True
                break
            face.append(idx)
        if not skip:
            faces.append((face, f))
    _add_submesh(m, verts, list(range(nv)), faces, keep_empty=True)
    return m.arrays()


def _read_off_binary(m, b):
    pos = 0

    def word(fmt):
        nonlocal pos
        if pos + 4 > len(b):
            raise ValueError("unexpected end of input")
        v = struct.unpack(">" + fmt, b[pos:pos + 4])[0]
        pos += 4
        return v

    nv, nf, _ = word("i"), word("i"), word("i")
    if nv <= 0:
        return m.arrays()
    verts = [tuple(f32(word("f")) for _ in range(3)) for _ in range(nv)]
    faces = []
    for f in range(nf):
        k = word("i")
        if k <= 0:
            continue
        face, skip = [], False
        for _ in range(k):
            if skip:
                word("i")
                continue
            idx = word("i")
            if idx < 0 or idx >= nv:
                skip = True
                break
            skip = idx in face
            face.append(idx)
        ncol = word("i")
        if ncol > 0:
            pos += 4 * ncol
        if not skip:
            faces.append((face, f))
    _add_submesh(m, verts, list(range(nv)), faces, keep_empty=True)
    return m.arrays()


def _vtn(field, nv, nt, nn):
    """One OBJ vertex reference v[/[t][/n]] resolved as the reader does, or None for a bad reference."""
    r = [0, 0, 0]
    v, i = _int_prefix(field, 0)
    if v is None:
        return None
    r[0] = v
    if i < len(field) and field[i] == "/":
        i += 1
        if i < len(field) and field[i] == "/":
            n, i = _int_prefix(field, i + 1)
            if n is None:
                return None
            r[2] = n
        else:
            t, i = _int_prefix(field, i)
            if t is None:
                return None
            r[1] = t
            if i < len(field) and field[i] == "/":
                n, i = _int_prefix(field, i + 1)
                if n is None:
                    return None
                r[2] = n
    if abs(r[0]) < 1 or abs(r[0]) > nv:
        return None
    if abs(r[1]) > nt:
        r[1] = 0
    if abs(r[2]) > nn:
        r[2] = 0
    for j, size in enumerate((nv, nt, nn)):
        if r[j] < 0:
            r[j] = size + 1 + r[j]
    return tuple(r)


def read_obj(data):
    """The OBJ reader on the bytes of a file: dict of arrays as thea_mesh_copy returns them."""
    m = _Mesh()
    pos, nt, nn = [], 0, 0
    faces = []          # (list of VTN) of the current group
    counter = [0]

    def flush():
        if not faces:
            return
        keys = sorted(set(r for f in faces for r in f))
        local = {k: i for i, k in enumerate(keys)}
        verts = [pos[k[0] - 1] for k in keys]
        srcs = [k[0] - 1 for k in keys]
        fl = []
        for f in faces:
            fl.append(([local[r] for r in f], counter[0]))
            counter[0] += 1
        _add_submesh(m, verts, srcs, fl)
        faces.clear()

    for raw in data.decode("latin-1").split("\n"):
        ln = raw.strip()
        if not ln:
            continue
        c0 = ln[0]
        if c0 == "v" and len(ln) >= 2:
            if ln[1] == "t":
                nt += 1
            elif ln[1] == "n":
                nn += 1
            elif ln[1] in " \t":
                x = ln[1:].split()
                pos.append(tuple(f32(float(t)) for t in x[:3]))
        elif c0 in "fp" and len(ln) >= 2 and ln[1] in " \t":
            refs = []
            for field in ln.lstrip("fp \t").split():
                r = _vtn(field, len(pos), nt, nn)
                if r is None:
                    refs = None
                    break
                refs.append(r)
            if refs is not None:
                faces.append(refs)
        elif c0 in "go" and (len(ln) < 2 or ln[1] in " \t"):
            flush()
    flush()
    return m.arrays()


_PLY_TYPES = {"int8": "b", "char": "b", "int16": "h", "short": "h", "int32": "i", "int": "i", "uint8": "B",
              "uchar": "B", "uint16": "H", "ushort": "H", "uint32": "I", "uint": "I", "float32": "f", "float": "f",
              "float64": "d", "double": "d"}


def read_ply(data):
    """The PLY reader on the bytes of a file: dict of arrays as thea_mesh_copy returns them."""
    pos = 0

    def line():
        nonlocal pos
        e = data.find(b"\n", pos)
        e = len(data) if e < 0 else e
        s = data[pos:e].decode("latin-1")
        pos = min(e + 1, len(data))
        return s

    if line().strip() != "ply":
        raise ValueError("not a PLY file")
    binary, order, blocks = False, "<", []
    while True:
        if pos >= len(data):
            raise ValueError("header not closed")
        ln = line().strip()
        if not ln:
            continue
        if ln == "end_header":
            break
        w = ln.split()
        if w[0] == "format":
            binary = w[1] != "ascii"
            order = ">" if w[1] == "binary_big_endian" else "<"
        elif w[0] == "element":
            blocks.append((w[1], int(w[2]), []))
        elif w[0] == "property":
            blocks[-1][2].append(("list", _PLY_TYPES[w[2]], _PLY_TYPES[w[3]]) if w[1] == "list"
                                 else (_PLY_TYPES[w[1]],))

    def num(code):
        nonlocal pos
        size = struct.calcsize(code)
        if pos + size > len(data):
            raise ValueError("unexpected end of input")
        v = struct.unpack(order + code, data[pos:pos + size])[0]
        pos += size
        return v

    def skip(prop):
        if prop[0] == "list":
            for _ in range(num(prop[1])):
                num(prop[2])
        else:
            num(prop[0])

    verts, faces = [], []
    for kind, count, props in blocks:
        for _ in range(count):
            if not binary:
                while True:
                    if pos >= len(data):
                        raise ValueError("unexpected end of input")
                    ln = line().strip()
                    if ln and not ln.startswith("comment"):
                        break
                tok = ln.split()
                if kind == "vertex":
                    verts.append(tuple(f32(float(t)) for t in tok[:3]))
                elif kind == "face":
                    k = int(tok[0])
                    if k > 0:
                        idx = [int(t) for t in tok[1:k + 1]]
                        if len(idx) == k:
                            faces.append(idx)
                continue
            if kind == "vertex":
                verts.append(tuple(f32(num(props[j][0])) for j in range(3)))
                for p in props[3:]:
                    skip(p)
            elif kind == "face":
                idx = [num(props[0][2]) for _ in range(num(props[0][1]))]
                for p in props[1:]:
                    skip(p)
                if idx:
                    faces.append(idx)
            else:
                for p in props:
                    skip(p)
    m = _Mesh()
    nv = len(verts)
    kept = []
    for idx in faces:
        if all(0 <= v < nv for v in idx) and len(set(idx)) == len(idx):
            kept.append((idx, len(kept)))
    _add_submesh(m, verts, list(range(nv)), kept, keep_empty=nv > 0)
    return m.arrays()


def _chunks_3ds(b, start, end):
    """(id, payload start, chunk end) of the little-endian chunks in b[start:end]."""
    pos = start
    while pos < end:
        if end - pos < 6:
            raise ValueError("truncated 3DS chunk header")
        cid, length = struct.unpack_from("<HI", b, pos)
        if length < 6 or length > end - pos:
            raise ValueError("3DS chunk runs past its parent")
        yield cid, pos + 6, pos + length
        pos += length


def read_3ds(data):
    b = bytes(data)
    meshes = []   # (name, points, faces)

    def tri_object(name, p, e):
        pts, faces = [], []
        for cid, q, ce in _chunks_3ds(b, p, e):
            if cid == 0x4110:
                (n,) = struct.unpack_from("<H", b, q)
                if ce - q - 2 < 12 * n:
                    raise ValueError("truncated 3DS array")
                v = struct.unpack_from("<%df" % (3 * n), b, q + 2)
                pts = [tuple(np.float32(x) for x in v[3 * i:3 * i + 3]) for i in range(n)]
            elif cid == 0x4120:
                (n,) = struct.unpack_from("<H", b, q)
                if ce - q - 2 < 8 * n:
                    raise ValueError("truncated 3DS array")
                w = struct.unpack_from("<%dH" % (4 * n), b, q + 2)
                faces = [w[4 * i:4 * i + 3] for i in range(n)]
        meshes.append((name, pts, faces))

    def named_object(p, e):
        z = b.index(b"\0", p, e)
        if z - p > 63:
            raise ValueError("3DS object name longer than 63 bytes")
        name = b[p:z]
        for cid, q, ce in _chunks_3ds(b, z + 1, e):
            if cid == 0x4100:
                tri_object(name, q, ce)

    def editor(p, e):
        for cid, q, ce in _chunks_3ds(b, p, e):
            if cid == 0x4000:
                named_object(q, ce)

    if len(b) < 6:
        raise ValueError("truncated 3DS chunk header")
    top, e = struct.unpack_from("<HI", b, 0)
    if e < 6 or e > len(b):
        raise ValueError("3DS chunk runs past its parent")
    p = 6
    if top in (0x4D4D, 0x3DAA, 0xC23D):
        for cid, q, ce in _chunks_3ds(b, p, e):
            if cid == 0x3D3D:
                editor(q, ce)
    elif top == 0x3D3D:
        editor(p, e)
    else:
        raise ValueError("not a 3DS file")
    ordered = []
    for mesh in meshes:   # lib3ds's sorted insertion
        k = len(ordered)
        for i, other in enumerate(ordered):
            if mesh[0] < other[0]:
                k = i
                break
        ordered.insert(k, mesh)
    m = _Mesh()
    nv_total = nf_total = 0
    for name, pts, faces in ordered:
        nv = len(pts)
        if nv <= 0:
            continue
        kept = []
        for i, f in enumerate(faces):
            if max(f) < nv and len(set(f)) == 3:
                kept.append((list(f), nf_total + i))
        nf_total += len(faces)
        _add_submesh(m, pts, list(range(nv_total, nv_total + nv)), kept, keep_empty=True)
        nv_total += nv
    return m.arrays()


def read_mesh(path):
    with open(path, "rb") as f:
        data = f.read()
    p = str(path).lower()
    if p.endswith(".obj"):
        return read_obj(data)
    if p.endswith(".ply"):
        return read_ply(data)
    if p.endswith(".3ds"):
        return read_3ds(data)
    return read_off(data)
