// Mesh file readers and face triangulation (host code).
//
// Restates, as far as geometry goes, the reference's non-strict OFF reader (Graphics/MeshCodecOff.hpp:154-330: ASCII and
// big-endian binary), its PLY reader (Graphics/MeshCodecPly.hpp:229-700: ASCII and either byte order), its OBJ reader (Graphics/MeshCodecObj.hpp:210-545: one submesh per g/o group, each submesh's
// vertices being the distinct (vertex, texcoord, normal) references of its faces in sorted order) and the triangulation
// of DisplayMesh::addFace (Graphics/DisplayMesh.cpp:249-320): quads by Polygon3::triangulateQuad (Polygon3.hpp:245-285),
// larger polygons by Polygon3::triangulate (Polygon3.cpp:109-288: ear clipping after projecting onto the plane of
// Polygon3::computeNormal, Polygon3.hpp:180-208, in the basis of Math::orthonormalBasis, MatrixUtil.hpp:225-249).
// The 3DS reader (Graphics/MeshCodec3ds.hpp) restates the part of lib3ds 1.x it relies on (below).
// FP32 arithmetic in the reference's operation order; this file is compiled without floating-point contraction.
#include "mesh_io.hpp"

#include <algorithm>
#include <charconv>
#include <cstdlib>
#include <array>
#include <cctype>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <fstream>
#include <sstream>

namespace thea {
namespace {

float const FLT_EPS = 1.1920928955078125e-07f;  // Math::eps<float>()

struct V2 {
  float x, y;
};

// Polygon3::triangulateQuad: the diagonal p0-p2 unless its two triangles face opposite ways, then the degeneracy test
// against eps^2
int triangulate_quad(V3 p0, V3 p1, V3 p2, V3 p3, int (&t)[6]) {
  V3 n0 = cross(p1 - p0, p2 - p0);
  V3 n1 = cross(p2 - p0, p3 - p0);
  static int const diag02[6] = {0, 1, 2, 2, 3, 0};
  static int const diag13[6] = {1, 2, 3, 3, 0, 1};
  if (dot(n0, n1) < 0.f) {
    n0 = cross(p2 - p1, p3 - p1);
    n1 = cross(p3 - p1, p0 - p1);
    std::copy(diag13, diag13 + 6, t);
  } else {
    std::copy(diag02, diag02 + 6, t);
  }
  float e2 = FLT_EPS * FLT_EPS;
  if (squared_norm(n0) < e2) {
    if (squared_norm(n1) < e2) return 0;
    std::copy(t + 3, t + 6, t);  // the second triangle is the only non-degenerate one
    return 1;
  }
  return squared_norm(n1) < e2 ? 1 : 2;
}

// Polygon3::computeNormal: the first (p2 - p1) x (p0 - p1) over consecutive vertex triples (n tries, wrapping around)
// with squared norm >= 1e-10, normalised; zero if there is none
V3 polygon_normal(std::vector<V3> const & p) {
  size_t n = p.size();
  V3 p0 = p[0], p1 = p[1];
  size_t i2 = 2 % n;
  for (size_t k = 0; k < n; ++k) {
    V3 p2 = p[i2];
    V3 nrm = cross(p2 - p1, p0 - p1);
    if (squared_norm(nrm) >= 1e-10f) return normalized(nrm);
    p0 = p1;
    p1 = p2;
    i2 = (i2 + 1) % n;
  }
  return V3{0.f, 0.f, 0.f};
}

// P inside or on the triangle ABC (counter-clockwise), by the signs of three edge cross products
bool inside_triangle2(V2 A, V2 B, V2 C, V2 P) {
  float ax = C.x - B.x, ay = C.y - B.y;
  float bx = A.x - C.x, by = A.y - C.y;
  float cx = B.x - A.x, cy = B.y - A.y;
  float apx = P.x - A.x, apy = P.y - A.y;
  float bpx = P.x - B.x, bpy = P.y - B.y;
  float cpx = P.x - C.x, cpy = P.y - C.y;
  float a_bp = ax * bpy - ay * bpx;
  float c_ap = cx * apy - cy * apx;
  float b_cp = bx * cpy - by * cpx;
  return a_bp >= 0.f && b_cp >= 0.f && c_ap >= 0.f;
}

// An ear (u, v, w) of the remaining polygon: convex by more than eps and containing none of its other vertices
bool is_ear(std::vector<V2> const & q, size_t u, size_t v, size_t w, size_t n, std::vector<size_t> const & idx) {
  V2 A = q[idx[u]], B = q[idx[v]], C = q[idx[w]];
  if (FLT_EPS > (((B.x - A.x) * (C.y - A.y)) - ((B.y - A.y) * (C.x - A.x)))) return false;
  for (size_t p = 0; p < n; ++p) {
    if (p == u || p == v || p == w) continue;
    if (inside_triangle2(A, B, C, q[idx[p]])) return false;
  }
  return true;
}

// Polygon3::triangulate with the default epsilon
int triangulate_polygon(std::vector<V3> const & p, std::vector<int32_t> & tris) {
  size_t n = p.size();
  size_t before = tris.size();
  // Math::orthonormalBasis(normal): u = orthogonalDirection(normal), v = normalized(normal) x u
  V3 normal = polygon_normal(p);
  V3 w = normalized(normal);
  V3 u = max_abs_axis(normal) == 0 ? normalized(V3{normal.y, -normal.x, 0.f}) : normalized(V3{0.f, normal.z, -normal.y});
  V3 v = cross(w, u);
  std::vector<V2> q(n);
  for (size_t i = 0; i < n; ++i) {
    V3 d = p[i] - p[0];
    q[i] = V2{dot(d, u), dot(d, v)};
  }
  // signed area of the projected polygon (Polygon3::projArea)
  float area = 0.f;
  for (size_t a = n - 1, b = 0; b < n; a = b++) area += q[a].x * q[b].y - q[b].x * q[a].y;
  area = 0.5f * area;
  bool flipped = !(area > 0.f);
  std::vector<size_t> idx(n);
  for (size_t i = 0; i < n; ++i) idx[i] = flipped ? (n - 1) - i : i;
  // clip ears walking around the polygon; give up after two fruitless laps
  size_t nv = n;
  size_t tries = 2 * nv;
  for (size_t cur = nv - 1; nv > 2;) {
    if (tries-- == 0) break;
    size_t a = cur < nv ? cur : 0;
    cur = a + 1 < nv ? a + 1 : 0;
    size_t c = cur + 1 < nv ? cur + 1 : 0;
    if (is_ear(q, a, cur, c, nv, idx)) {
      int32_t ia = (int32_t)idx[a], ib = (int32_t)idx[cur], ic = (int32_t)idx[c];
      if (flipped) std::swap(ia, ic);
      tris.push_back(ia);
      tris.push_back(ib);
      tris.push_back(ic);
      idx.erase(idx.begin() + (std::ptrdiff_t)cur);
      --nv;
      tries = 2 * nv;
    }
  }
  return (int)((tris.size() - before) / 3);
}

std::string trim(std::string const & s) {
  size_t b = s.find_first_not_of(" \t\r\n\f\v");
  if (b == std::string::npos) return std::string();
  size_t e = s.find_last_not_of(" \t\r\n\f\v");
  return s.substr(b, e - b + 1);
}

[[noreturn]] void fail(std::string const & path, std::string const & why) {
  throw Error(THEA_ERR_INVALID_ARGUMENT, "mesh_read: " + path + ": " + why);
}

// The whole file with a read cursor: lines for the text formats, big-endian words for binary OFF
struct Input {
  std::string data;
  size_t pos = 0;
  std::string path;

  bool has_more() const { return pos < data.size(); }
  std::string line() {
    size_t e = data.find('\n', pos);
    std::string s = data.substr(pos, e == std::string::npos ? std::string::npos : e - pos);
    pos = e == std::string::npos ? data.size() : e + 1;
    return s;
  }
  // an unsigned word of `bytes` bytes (1, 2, 4 or 8) in the given byte order
  uint64_t word(int bytes, bool big_endian) {
    if (data.size() - pos < (size_t)bytes) fail(path, "unexpected end of input");
    uint64_t w = 0;
    for (int i = 0; i < bytes; ++i) {
      int k = big_endian ? i : bytes - 1 - i;
      w = (w << 8) | (uint64_t)(unsigned char)data[pos + (size_t)k];
    }
    pos += (size_t)bytes;
    return w;
  }
  uint32_t be32() { return (uint32_t)word(4, true); }
  int32_t int32() { return (int32_t)be32(); }
  float float32() {
    uint32_t w = be32();
    float f;
    std::memcpy(&f, &w, 4);
    return f;
  }
  void skip(int64_t bytes) {
    if (bytes < 0 || (uint64_t)bytes > data.size() - pos) fail(path, "unexpected end of input");
    pos += (size_t)bytes;
  }
};

bool is_space(char c) { return c == ' ' || c == '\t' || c == '\r' || c == '\n' || c == '\f' || c == '\v'; }

// A line of the file as [b, e) with surrounding white space removed (no copy)
struct Span {
  char const * b;
  char const * e;
  bool empty() const { return b == e; }
  size_t size() const { return (size_t)(e - b); }
  char operator[](size_t i) const { return b[i]; }
  std::string str() const { return std::string(b, e); }
};

Span next_line(Input & in) {
  char const * base = in.data.data();
  size_t stop = in.data.find('\n', in.pos);
  char const * b = base + in.pos;
  char const * e = base + (stop == std::string::npos ? in.data.size() : stop);
  in.pos = stop == std::string::npos ? in.data.size() : stop + 1;
  while (b < e && is_space(*b)) ++b;
  while (e > b && is_space(e[-1])) --e;
  return Span{b, e};
}

// Successive reads from a line with the semantics of std::istream extraction (operator>> of long long and double,
// get, peek) for the inputs a mesh file holds: numbers skip leading white space and take the longest valid prefix;
// a read that fails leaves the scan failed. Doubles are correctly rounded (std::from_chars, as strtod); a lone or
// incomplete exponent, "inf" and "nan" fail as they do for a stream, and an underflow gives the rounded value.
struct Scan {
  char const * p;
  char const * e;
  bool good = true;
  Scan(char const * b, char const * end) : p(b), e(end) {}
  explicit Scan(Span s) : p(s.b), e(s.e) {}

  void skip_ws() {
    while (p < e && is_space(*p)) ++p;
  }
  int get() { return p < e ? (unsigned char)*p++ : -1; }
  int peek() const { return p < e ? (unsigned char)*p : -1; }

  bool read(long long & v) {
    if (!good) return false;
    skip_ws();
    char const * b = p;
    if (b < e && *b == '+') {
      ++b;
      if (b == e || *b < '0' || *b > '9') return good = false;
    }
    auto r = std::from_chars(b, e, v);
    if (r.ec != std::errc()) return good = false;
    p = r.ptr;
    return true;
  }

  bool read(double & v) {
    if (!good) return false;
    skip_ws();
    char const * b = p;
    if (b < e && *b == '+') {
      ++b;
      if (b < e && (*b == '+' || *b == '-')) return good = false;
    }
    char const * m = b < e && *b == '-' ? b + 1 : b;
    if (m < e && ((*m | 0x20) == 'i' || (*m | 0x20) == 'n')) return good = false;  // no inf / nan
    auto r = std::from_chars(b, e, v);
    if (r.ec == std::errc::invalid_argument) return good = false;
    bool has_exp = false;
    for (char const * c = b; c < r.ptr; ++c) has_exp |= (*c | 0x20) == 'e';
    if (!has_exp && r.ptr < e && (*r.ptr | 0x20) == 'e') return good = false;  // "1e", "1e+": an incomplete exponent
    if (r.ec == std::errc::result_out_of_range) {
      std::string tok(b, r.ptr);
      double w = std::strtod(tok.c_str(), nullptr);
      if (w == HUGE_VAL || w == -HUGE_VAL) return good = false;  // overflow fails; underflow gives the rounded value
      v = w;
    }
    p = r.ptr;
    return true;
  }
};

// The next line that is neither blank nor a comment (the OFF reader's loop)
Span off_data_line(Input & in) {
  Span line = next_line(in);
  while (line.empty() || line[0] == '#') {
    if (!in.has_more()) fail(in.path, "unexpected end of input");
    line = next_line(in);
  }
  return line;
}

// Builds the display mesh of one submesh: vertices appended, faces added in order with running source indices
struct SubmeshBuilder {
  MeshData & m;
  int64_t first_vertex, first_triangle, faces_before;
  std::vector<float> pos;      // scratch: the positions of the face being triangulated
  std::vector<int32_t> local;  // scratch: its triangles in local indices

  explicit SubmeshBuilder(MeshData & m_)
      : m(m_), first_vertex((int64_t)m_.vertices.size() / 3), first_triangle((int64_t)m_.triangle_face.size()),
        faces_before(m_.num_faces) {}

  void add_vertex(float x, float y, float z, int32_t source) {
    m.vertices.push_back(x);
    m.vertices.push_back(y);
    m.vertices.push_back(z);
    m.vertex_source.push_back(source);
  }

  // DisplayMesh::addFace with local vertex indices
  void add_face(std::vector<int32_t> const & face, int32_t src_face) {
    int n = (int)face.size();
    if (n < 3) return;
    if (n == 3) {  // DisplayMesh::addTriangle
      for (int k = 0; k < 3; ++k) m.triangles.push_back((int32_t)first_vertex + face[(size_t)k]);
      m.triangle_face.push_back(src_face);
      ++m.num_faces;
      return;
    }
    pos.resize((size_t)3 * n);
    for (int i = 0; i < n; ++i)
      for (int c = 0; c < 3; ++c) pos[(size_t)3 * i + c] = m.vertices[(size_t)(3 * (first_vertex + face[(size_t)i]) + c)];
    local.clear();
    int nt = triangulate_face(pos.data(), n, local);
    if (nt <= 0) return;
    for (int t = 0; t < nt; ++t) {
      for (int k = 0; k < 3; ++k) m.triangles.push_back((int32_t)first_vertex + face[(size_t)local[(size_t)3 * t + k]]);
      m.triangle_face.push_back(src_face);
    }
    ++m.num_faces;
  }

  // Ends the submesh; the mesh group keeps it only if it has faces (skip_empty_meshes)
  void end() {
    if (m.num_faces == faces_before) {
      m.vertices.resize((size_t)(3 * first_vertex));
      m.vertex_source.resize((size_t)first_vertex);
      m.triangles.resize((size_t)(3 * first_triangle));
      m.triangle_face.resize((size_t)first_triangle);
      return;
    }
    m.submesh_vertex_offsets.push_back((int64_t)m.vertex_source.size());
    m.submesh_triangle_offsets.push_back((int64_t)m.triangle_face.size());
  }
};

MeshData read_off_ascii(Input & in) {
  MeshData m;
  Scan counts(off_data_line(in));
  long long nv = 0, nf = 0, ne = 0;
  if (!(counts.read(nv) && counts.read(nf) && counts.read(ne))) fail(in.path, "could not read the mesh statistics");
  if (nv <= 0) return m;
  SubmeshBuilder b(m);
  m.vertices.reserve((size_t)std::min<long long>(nv, 1 << 26) * 3);
  for (long long v = 0; v < nv; ++v) {
    Scan vs(off_data_line(in));
    double x, y, z;
    if (!(vs.read(x) && vs.read(y) && vs.read(z))) fail(in.path, "could not read a vertex");
    b.add_vertex((float)x, (float)y, (float)z, (int32_t)v);
  }
  std::vector<int32_t> face;
  for (long long f = 0; f < nf; ++f) {
    Scan fs(off_data_line(in));
    long long k = 0;
    if (!fs.read(k)) fail(in.path, "could not read the number of vertices of a face");
    if (k <= 0) continue;
    face.clear();
    bool skip = false;
    for (long long v = 0; v < k && !skip; ++v) {
      long long index;
      if (!fs.read(index) || index < 0 || index >= nv) {
        skip = true;  // unreadable or out of range: the face is skipped
        break;
      }
      skip = std::find(face.begin(), face.end(), (int32_t)index) != face.end();  // repeated vertex
      face.push_back((int32_t)index);
    }
    if (!skip) b.add_face(face, (int32_t)f);
  }
  m.submesh_vertex_offsets.push_back((int64_t)m.vertex_source.size());  // the OFF mesh is kept even without faces
  m.submesh_triangle_offsets.push_back((int64_t)m.triangle_face.size());
  return m;
}

MeshData read_off_binary(Input & in) {
  MeshData m;
  int64_t nv = in.int32(), nf = in.int32();
  in.int32();  // number of edges
  if (nv <= 0) return m;
  SubmeshBuilder b(m);
  for (int64_t v = 0; v < nv; ++v) {
    float x = in.float32(), y = in.float32(), z = in.float32();
    b.add_vertex(x, y, z, (int32_t)v);
  }
  std::vector<int32_t> face;
  for (int64_t f = 0; f < nf; ++f) {
    int32_t k = in.int32();
    if (k <= 0) continue;
    face.clear();
    bool skip = false;
    for (int32_t v = 0; v < k; ++v) {
      if (skip) {
        in.skip(4);  // the rest of a face with a repeated vertex
        continue;
      }
      int32_t index = in.int32();
      if (index < 0 || index >= nv) {
        // The reference stops reading this face's indices here and takes the next word as the colour count; the same
        // words are consumed here so that files read identically.
        skip = true;
        break;
      }
      skip = std::find(face.begin(), face.end(), index) != face.end();
      face.push_back(index);
    }
    int32_t colours = in.int32();
    if (colours > 0) in.skip(4 * (int64_t)colours);
    if (!skip) b.add_face(face, (int32_t)f);
  }
  m.submesh_vertex_offsets.push_back((int64_t)m.vertex_source.size());
  m.submesh_triangle_offsets.push_back((int64_t)m.triangle_face.size());
  return m;
}

MeshData read_off(Input & in) {
  std::string header = trim(in.line());
  if (header != "OFF" && header.rfind("OFF ", 0) != 0) fail(in.path, "invalid OFF stream (does not start with 'OFF')");
  bool binary = header == "OFF BINARY" || header.rfind("OFF BINARY ", 0) == 0;
  return binary ? read_off_binary(in) : read_off_ascii(in);
}

using VTN = std::array<long long, 3>;  // 1-based vertex, texcoord, normal (0: none), compared lexicographically

// Adds one OBJ submesh: its vertices are the distinct VTN references of its faces in ascending order (the reference
// collects them in a sorted map). `mark` is scratch of one entry per file vertex, all -1 between calls.
void construct_obj_submesh(MeshData & m, std::vector<float> const & positions, std::vector<VTN> const & refs,
                           std::vector<size_t> const & face_starts, int64_t & num_faces, std::vector<int32_t> & mark) {
  SubmeshBuilder b(m);
  std::vector<int32_t> local(refs.size());
  bool plain = std::all_of(refs.begin(), refs.end(), [](VTN const & r) { return r[1] == 0 && r[2] == 0; });
  if (plain) {
    // references by vertex only: the distinct vertices in ascending order, then a lookup through `mark`
    std::vector<int32_t> used;
    for (VTN const & r : refs) {
      int32_t v = (int32_t)(r[0] - 1);
      if (mark[(size_t)v] < 0) {
        mark[(size_t)v] = 0;
        used.push_back(v);
      }
    }
    std::sort(used.begin(), used.end());
    for (size_t i = 0; i < used.size(); ++i) {
      size_t q = (size_t)used[i];
      mark[q] = (int32_t)i;
      b.add_vertex(positions[3 * q], positions[3 * q + 1], positions[3 * q + 2], (int32_t)q);
    }
    for (size_t j = 0; j < refs.size(); ++j) local[j] = mark[(size_t)(refs[j][0] - 1)];
    for (int32_t v : used) mark[(size_t)v] = -1;
  } else {
    std::vector<VTN> keys(refs);
    std::sort(keys.begin(), keys.end());
    keys.erase(std::unique(keys.begin(), keys.end()), keys.end());
    for (VTN const & k : keys) {
      size_t q = (size_t)(k[0] - 1);
      b.add_vertex(positions[3 * q], positions[3 * q + 1], positions[3 * q + 2], (int32_t)q);
    }
    for (size_t j = 0; j < refs.size(); ++j)
      local[j] = (int32_t)(std::lower_bound(keys.begin(), keys.end(), refs[j]) - keys.begin());
  }
  std::vector<int32_t> face;
  for (size_t i = 0; i < face_starts.size(); ++i) {
    size_t e = i + 1 < face_starts.size() ? face_starts[i + 1] : refs.size();
    face.assign(local.begin() + (std::ptrdiff_t)face_starts[i], local.begin() + (std::ptrdiff_t)e);
    b.add_face(face, (int32_t)num_faces);
    ++num_faces;  // every face is numbered, including those the triangulation drops
  }
  b.end();
}

MeshData read_obj(Input & in) {
  MeshData m;
  std::vector<float> positions;
  long long num_tex = 0, num_nrm = 0;
  std::vector<VTN> refs;          // references of the current submesh's faces, concatenated
  std::vector<size_t> face_starts;
  std::vector<int32_t> mark;
  int64_t num_faces = 0;
  auto flush = [&]() {
    if (face_starts.empty()) return;
    mark.resize(positions.size() / 3, -1);
    construct_obj_submesh(m, positions, refs, face_starts, num_faces, mark);
  };
  while (in.has_more()) {
    Span line = next_line(in);
    if (line.empty()) continue;
    char c0 = line[0];
    if (c0 == 'v' && line.size() >= 2) {
      if (line[1] == 't') {
        Scan vs(line.b + 2, line.e);
        double x, y;
        if (!(vs.read(x) && vs.read(y)))
          fail(in.path, "could not read a texture coordinate on line '" + line.str() + "'");
        ++num_tex;
      } else if (line[1] == 'n') {
        Scan vs(line.b + 2, line.e);
        double x, y, z;
        if (!(vs.read(x) && vs.read(y) && vs.read(z))) fail(in.path, "could not read a normal on line '" + line.str() + "'");
        ++num_nrm;
      } else if (line[1] == ' ' || line[1] == '\t') {
        Scan vs(line.b + 1, line.e);
        double x, y, z;
        if (!(vs.read(x) && vs.read(y) && vs.read(z)))
          fail(in.path, "could not read a vertex position on line '" + line.str() + "'");
        positions.push_back((float)x);
        positions.push_back((float)y);
        positions.push_back((float)z);
      }
    } else if ((c0 == 'f' || c0 == 'p') && line.size() >= 2 && (line[1] == ' ' || line[1] == '\t')) {
      size_t start = refs.size();
      long long nvtx = (long long)(positions.size() / 3);
      // fields start after the leading run of 'f', 'p', spaces and tabs, and are separated by spaces and tabs
      char const * fb = line.b;
      while (fb < line.e && (*fb == 'f' || *fb == 'p' || *fb == ' ' || *fb == '\t')) ++fb;
      if (fb == line.e) fail(in.path, "malformed face '" + line.str() + "'");
      bool bad_face = false;
      while (fb < line.e) {
        char const * fe = fb;
        while (fe < line.e && *fe != ' ' && *fe != '\t') ++fe;
        Scan fs(fb, fe);
        VTN r{0, 0, 0};
        bool bad = !fs.read(r[0]);
        if (!bad && fs.get() == '/') {
          if (fs.peek() == '/') {
            fs.get();
            bad = !fs.read(r[2]);
          } else {
            bad = !fs.read(r[1]);
            if (!bad && fs.get() == '/') bad = !fs.read(r[2]);
          }
        }
        if (bad || std::llabs(r[0]) < 1 || std::llabs(r[0]) > nvtx) {
          bad_face = true;
          break;
        }
        if (std::llabs(r[1]) > num_tex) r[1] = 0;
        if (std::llabs(r[2]) > num_nrm) r[2] = 0;
        if (r[0] < 0) r[0] = nvtx + 1 + r[0];
        if (r[1] < 0) r[1] = num_tex + 1 + r[1];
        if (r[2] < 0) r[2] = num_nrm + 1 + r[2];
        refs.push_back(r);
        fb = fe;
        while (fb < line.e && (*fb == ' ' || *fb == '\t')) ++fb;
      }
      if (bad_face)
        refs.resize(start);  // the non-strict reader drops the face
      else
        face_starts.push_back(start);
    } else if ((c0 == 'g' || c0 == 'o') && (line.size() < 2 || line[1] == ' ' || line[1] == '\t')) {
      flush();
      refs.clear();
      face_starts.clear();
    }
  }
  flush();
  return m;
}

// ---- PLY (Graphics/MeshCodecPly.hpp:229-700) -------------------------------------------------------------------------

enum class PlyType { INVALID, LIST, INT8, INT16, INT32, UINT8, UINT16, UINT32, FLOAT32, FLOAT64 };

PlyType ply_type(std::string const & name) {
  static std::pair<char const *, PlyType> const names[] = {
      {"list", PlyType::LIST},     {"int8", PlyType::INT8},       {"int16", PlyType::INT16},
      {"int32", PlyType::INT32},   {"uint8", PlyType::UINT8},     {"uint16", PlyType::UINT16},
      {"uint32", PlyType::UINT32}, {"float32", PlyType::FLOAT32}, {"float64", PlyType::FLOAT64},
      {"char", PlyType::INT8},     {"short", PlyType::INT16},     {"int", PlyType::INT32},
      {"uchar", PlyType::UINT8},   {"ushort", PlyType::UINT16},   {"uint", PlyType::UINT32},
      {"float", PlyType::FLOAT32}, {"double", PlyType::FLOAT64}};
  for (auto const & n : names)
    if (name == n.first) return n.second;
  return PlyType::INVALID;
}

int ply_bytes(PlyType t) {
  switch (t) {
    case PlyType::INT8: case PlyType::UINT8: return 1;
    case PlyType::INT16: case PlyType::UINT16: return 2;
    case PlyType::INT32: case PlyType::UINT32: case PlyType::FLOAT32: return 4;
    case PlyType::FLOAT64: return 8;
    default: return 0;
  }
}

bool ply_integer(PlyType t) { return t != PlyType::FLOAT32 && t != PlyType::FLOAT64 && ply_bytes(t) > 0; }

struct PlyProperty {
  PlyType type = PlyType::INVALID, count_type = PlyType::INVALID, item_type = PlyType::INVALID;
};

enum class PlyElement { VERTEX, FACE, OTHER };

struct PlyBlock {
  PlyElement kind = PlyElement::OTHER;
  long long count = 0;
  std::vector<PlyProperty> props;
};

struct PlyHeader {
  bool binary = false, big_endian = false;
  std::vector<PlyBlock> blocks;
};

PlyHeader read_ply_header(Input & in) {
  if (trim(in.line()) != "ply") fail(in.path, "invalid PLY stream (does not start with 'ply')");
  PlyHeader h;
  bool have_format = false;
  while (in.has_more()) {
    std::string line = trim(in.line());
    if (line.empty()) continue;
    if (line == "end_header") return h;
    std::istringstream ls(line);
    std::string field;
    ls >> field;
    if (field == "format") {
      if (have_format) fail(in.path, "format specifier must be first line after magic string");
      if (!(ls >> field)) fail(in.path, "could not read ascii/binary specifier");
      if (field == "ascii") {
        h.binary = false;
      } else if (field == "binary_little_endian" || field == "binary_big_endian") {
        h.binary = true;
        h.big_endian = field == "binary_big_endian";
      } else {
        fail(in.path, "invalid format specifier");
      }
      have_format = true;
    } else if (field == "element") {
      PlyBlock b;
      if (!(ls >> field)) fail(in.path, "could not read element type");
      if (!(ls >> b.count)) fail(in.path, "could not read number of elements of type '" + field + "'");
      b.kind = field == "vertex" ? PlyElement::VERTEX : field == "face" ? PlyElement::FACE : PlyElement::OTHER;
      h.blocks.push_back(b);
    } else if (field == "property") {
      if (h.blocks.empty()) fail(in.path, "property specification outside an element block");
      PlyProperty p;
      if (!(ls >> field)) fail(in.path, "could not read property type");
      p.type = ply_type(field);
      if (p.type == PlyType::INVALID) fail(in.path, "unknown property type '" + field + "'");
      if (p.type == PlyType::LIST) {
        std::string c, t;
        if (!(ls >> c >> t)) fail(in.path, "could not read list item and count types");
        p.count_type = ply_type(c);
        p.item_type = ply_type(t);
        if (ply_bytes(p.count_type) == 0) fail(in.path, "unknown list count type '" + c + "'");
        if (ply_bytes(p.item_type) == 0) fail(in.path, "unknown list item type '" + t + "'");
      }
      h.blocks.back().props.push_back(p);
    }
    // comment, obj_info and other header lines are ignored
  }
  fail(in.path, "no end_header token, header not closed");
}

void check_ply_block(PlyBlock const & b, std::string const & path) {
  if (b.kind == PlyElement::VERTEX) {
    if (b.props.size() < 3 || b.props[0].type == PlyType::LIST || b.props[1].type == PlyType::LIST ||
        b.props[2].type == PlyType::LIST)
      fail(path, "vertex element must start with three numerical coordinates");
  } else if (b.kind == PlyElement::FACE) {
    if (b.props.empty() || b.props[0].type != PlyType::LIST || !ply_integer(b.props[0].count_type) ||
        !ply_integer(b.props[0].item_type))
      fail(path, "face element must start with a list of integer indices");
  }
}

// One binary number of type t, as a double (integers of up to 32 bits and floats convert exactly)
double ply_number(Input & in, PlyType t, bool big) {
  uint64_t w = in.word(ply_bytes(t), big);
  switch (t) {
    case PlyType::INT8: return (double)(int8_t)(uint8_t)w;
    case PlyType::INT16: return (double)(int16_t)(uint16_t)w;
    case PlyType::INT32: return (double)(int32_t)(uint32_t)w;
    case PlyType::UINT8: case PlyType::UINT16: case PlyType::UINT32: return (double)w;
    case PlyType::FLOAT32: {
      uint32_t u = (uint32_t)w;
      float f;
      std::memcpy(&f, &u, 4);
      return (double)f;
    }
    case PlyType::FLOAT64: {
      double d;
      std::memcpy(&d, &w, 8);
      return d;
    }
    default: fail(in.path, "unknown property type");
  }
}

void skip_ply_property(Input & in, PlyProperty const & p, bool big) {
  if (p.type == PlyType::LIST) {
    double n = ply_number(in, p.count_type, big);
    if (n > 0) in.skip((int64_t)n * ply_bytes(p.item_type));
  } else {
    in.skip(ply_bytes(p.type));
  }
}

// Adds a face of file vertex indices unless an index is out of range or repeated (the non-strict reader's rule);
// returns whether it was added
bool add_checked_face(SubmeshBuilder & b, std::vector<long long> const & idx, long long nv, int64_t src_face) {
  std::vector<int32_t> face;
  for (long long v : idx) {
    if (v < 0 || v >= nv) return false;
    if (std::find(face.begin(), face.end(), (int32_t)v) != face.end()) return false;
    face.push_back((int32_t)v);
  }
  b.add_face(face, (int32_t)src_face);
  return true;
}

MeshData read_ply(Input & in) {
  PlyHeader h = read_ply_header(in);
  MeshData m;
  SubmeshBuilder b(m);
  long long nv = 0;
  int64_t nf = 0;  // faces handed to the mesh: the source index of the next one
  std::vector<long long> idx;
  for (PlyBlock const & blk : h.blocks) {
    check_ply_block(blk, in.path);
    for (long long e = 0; e < blk.count; ++e) {
      if (!h.binary) {
        Span line;
        do {
          if (!in.has_more()) fail(in.path, "unexpected end of input");
          line = next_line(in);
        } while (line.empty() || (line.size() >= 7 && std::memcmp(line.b, "comment", 7) == 0));
        Scan ls(line);
        if (blk.kind == PlyElement::VERTEX) {
          double x, y, z;
          if (!(ls.read(x) && ls.read(y) && ls.read(z)))
            fail(in.path, "could not read vertex on line '" + line.str() + "'");
          b.add_vertex((float)x, (float)y, (float)z, (int32_t)nv++);
        } else if (blk.kind == PlyElement::FACE) {
          long long k;
          if (!ls.read(k)) fail(in.path, "could not read number of vertices in face on line '" + line.str() + "'");
          if (k <= 0) continue;
          idx.clear();
          long long v;
          bool readable = true;
          for (long long j = 0; j < k && readable; ++j) {
            readable = ls.read(v);
            idx.push_back(v);
          }
          if (readable && add_checked_face(b, idx, nv, nf)) ++nf;
        }
        continue;
      }
      // Binary. Properties after a vertex's coordinates or a face's index list, and elements of other kinds, are
      // skipped as the header describes them (the reference's loop over extra vertex properties does not advance, and
      // it skips neither extra face properties nor other elements, so it cannot read such files).
      if (blk.kind == PlyElement::VERTEX) {
        float c[3];
        for (int k = 0; k < 3; ++k) c[k] = (float)ply_number(in, blk.props[(size_t)k].type, h.big_endian);
        for (size_t k = 3; k < blk.props.size(); ++k) skip_ply_property(in, blk.props[k], h.big_endian);
        b.add_vertex(c[0], c[1], c[2], (int32_t)nv++);
      } else if (blk.kind == PlyElement::FACE) {
        PlyProperty const & p = blk.props[0];
        double n = ply_number(in, p.count_type, h.big_endian);
        if (n < 0) fail(in.path, "list has negative size");
        if (n * ply_bytes(p.item_type) > (double)(in.data.size() - in.pos)) fail(in.path, "unexpected end of input");
        idx.resize((size_t)n);
        for (auto & v : idx) v = (long long)ply_number(in, p.item_type, h.big_endian);
        for (size_t k = 1; k < blk.props.size(); ++k) skip_ply_property(in, blk.props[k], h.big_endian);
        if (!idx.empty() && add_checked_face(b, idx, nv, nf)) ++nf;
      } else {
        for (PlyProperty const & p : blk.props) skip_ply_property(in, p, h.big_endian);
      }
    }
  }
  if (nv > 0 || m.num_faces > 0) {  // the mesh is kept if it has vertices or faces
    m.submesh_vertex_offsets.push_back((int64_t)m.vertex_source.size());
    m.submesh_triangle_offsets.push_back((int64_t)m.triangle_face.size());
  }
  return m;
}

}  // namespace

// ---- 3DS (Graphics/MeshCodec3ds.hpp:160-395 over lib3ds 1.3.0) ---------------------------------------------------------
// The reference hands the file to lib3ds 1.x (the codec reads lib3ds 1.x's mesh fields points / pointL / faceL) and
// converts its mesh list with the default options: no node transforms, one display mesh per lib3ds mesh, meshes without
// vertices skipped, faces with an index out of range or a repeated index skipped but counted, vertex and face indices
// running over the whole file. lib3ds keeps its mesh list sorted by name (insertion after every mesh whose name is not
// greater), and the node tree the codec then walks attaches no further meshes. Restated here from the published chunk
// layout: a chunk is a little-endian u16 id and u32 length (header included); the meshes are the N_TRI_OBJECT chunks
// (0x4100) of the named objects (0x4000: a zero-terminated name of at most 63 bytes, then sub-chunks) of the editor
// chunk (0x3D3D) under the file chunk (0x4D4D, or a material or project file's 0x3DAA / 0xC23D), with points in
// POINT_ARRAY (0x4110: u16 count, three f32 each) and faces in FACE_ARRAY (0x4120: u16 count, three u16 indices and a
// u16 flag word each). A later point or face array of the same mesh replaces the earlier one, as lib3ds does. Every
// other chunk is skipped whole. A chunk that runs past its parent or a truncated array is an error.

struct Mesh3ds {
  std::string name;
  std::vector<float> points;     // xyz
  std::vector<uint16_t> faces;   // three vertex indices per face
};

struct Chunk3ds {
  uint16_t id;
  size_t end;  // one past the chunk's last byte
};

Chunk3ds chunk_3ds(Input & in, size_t limit) {
  if (limit < in.pos || limit - in.pos < 6) fail(in.path, "truncated 3DS chunk header");
  size_t start = in.pos;
  uint16_t id = (uint16_t)in.word(2, false);
  uint32_t len = (uint32_t)in.word(4, false);
  if (len < 6 || (size_t)len > limit - start) fail(in.path, "3DS chunk runs past its parent");
  return {id, start + (size_t)len};
}

void need_3ds(Input & in, size_t end, size_t bytes) {
  if (end < in.pos || end - in.pos < bytes) fail(in.path, "truncated 3DS array");
}

float f32_le(Input & in) {
  uint32_t w = (uint32_t)in.word(4, false);
  float f;
  std::memcpy(&f, &w, 4);
  return f;
}

void read_tri_object_3ds(Input & in, size_t end, Mesh3ds & mesh) {
  while (in.pos < end) {
    Chunk3ds c = chunk_3ds(in, end);
    if (c.id == 0x4110) {  // POINT_ARRAY
      need_3ds(in, c.end, 2);
      size_t n = (size_t)in.word(2, false);
      need_3ds(in, c.end, 12 * n);
      mesh.points.resize(3 * n);
      for (size_t i = 0; i < 3 * n; ++i) mesh.points[i] = f32_le(in);
    } else if (c.id == 0x4120) {  // FACE_ARRAY (its material and smoothing sub-chunks are skipped)
      need_3ds(in, c.end, 2);
      size_t n = (size_t)in.word(2, false);
      need_3ds(in, c.end, 8 * n);
      mesh.faces.resize(3 * n);
      for (size_t f = 0; f < n; ++f) {
        for (int k = 0; k < 3; ++k) mesh.faces[3 * f + (size_t)k] = (uint16_t)in.word(2, false);
        in.word(2, false);  // edge visibility flags
      }
    }
    in.pos = c.end;
  }
}

void read_named_object_3ds(Input & in, size_t end, std::vector<Mesh3ds> & meshes) {
  std::string name;
  for (;;) {
    if (in.pos >= end) fail(in.path, "unterminated 3DS object name");
    char ch = in.data[in.pos++];
    if (ch == '\0') break;
    if (name.size() == 63) fail(in.path, "3DS object name longer than 63 bytes");
    name.push_back(ch);
  }
  while (in.pos < end) {
    Chunk3ds c = chunk_3ds(in, end);
    if (c.id == 0x4100) {  // N_TRI_OBJECT
      Mesh3ds mesh;
      mesh.name = name;
      read_tri_object_3ds(in, c.end, mesh);
      meshes.push_back(std::move(mesh));
    }
    in.pos = c.end;
  }
}

// lib3ds's name order: byte-wise, as strcmp compares (unsigned)
bool name_less_3ds(std::string const & a, std::string const & b) {
  size_t n = std::min(a.size(), b.size());
  for (size_t i = 0; i < n; ++i) {
    unsigned char x = (unsigned char)a[i], y = (unsigned char)b[i];
    if (x != y) return x < y;
  }
  return a.size() < b.size();
}

MeshData read_3ds(Input & in) {
  size_t size = in.data.size();
  Chunk3ds top = chunk_3ds(in, size);
  std::vector<Mesh3ds> meshes;
  auto editor = [&](size_t end) {
    while (in.pos < end) {
      Chunk3ds c = chunk_3ds(in, end);
      if (c.id == 0x4000) read_named_object_3ds(in, c.end, meshes);
      in.pos = c.end;
    }
  };
  if (top.id == 0x4D4D || top.id == 0x3DAA || top.id == 0xC23D) {
    while (in.pos < top.end) {
      Chunk3ds c = chunk_3ds(in, top.end);
      if (c.id == 0x3D3D) editor(c.end);
      in.pos = c.end;
    }
  } else if (top.id == 0x3D3D) {
    editor(top.end);
  } else {
    fail(in.path, "not a 3DS file (unknown top-level chunk)");
  }
  std::stable_sort(meshes.begin(), meshes.end(),
                   [](Mesh3ds const & a, Mesh3ds const & b) { return name_less_3ds(a.name, b.name); });

  MeshData m;
  int64_t vertex_count = 0, face_count = 0;
  std::vector<int32_t> face(3);
  for (Mesh3ds const & mesh : meshes) {
    int64_t nv = (int64_t)(mesh.points.size() / 3);
    if (nv <= 0) continue;  // skip_empty_meshes
    SubmeshBuilder b(m);
    for (int64_t v = 0; v < nv; ++v)
      b.add_vertex(mesh.points[(size_t)(3 * v)], mesh.points[(size_t)(3 * v + 1)], mesh.points[(size_t)(3 * v + 2)],
                   (int32_t)vertex_count++);
    for (size_t f = 0; f < mesh.faces.size() / 3; ++f, ++face_count) {
      int64_t a = mesh.faces[3 * f], c1 = mesh.faces[3 * f + 1], c2 = mesh.faces[3 * f + 2];
      if (a >= nv || c1 >= nv || c2 >= nv) continue;      // out of range: skipped, still counted
      if (a == c1 || c1 == c2 || c2 == a) continue;       // repeated vertex: skipped, still counted
      face[0] = (int32_t)a;
      face[1] = (int32_t)c1;
      face[2] = (int32_t)c2;
      b.add_face(face, (int32_t)face_count);
    }
    m.submesh_vertex_offsets.push_back((int64_t)m.vertex_source.size());  // kept even without faces
    m.submesh_triangle_offsets.push_back((int64_t)m.triangle_face.size());
  }
  return m;
}

int triangulate_face(float const * pos, int n, std::vector<int32_t> & tris) {
  if (n < 3) return 0;
  auto P = [&](int i) { return V3{pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]}; };
  if (n == 3) {
    tris.insert(tris.end(), {0, 1, 2});
    return 1;
  }
  if (n == 4) {
    int t[6];
    int nt = triangulate_quad(P(0), P(1), P(2), P(3), t);
    tris.insert(tris.end(), t, t + 3 * nt);
    return nt;
  }
  std::vector<V3> p((size_t)n);
  for (int i = 0; i < n; ++i) p[(size_t)i] = P(i);
  return triangulate_polygon(p, tris);
}

MeshData read_mesh_file(std::string const & path) {
  std::string lower = path;
  for (char & ch : lower) ch = (char)std::tolower((unsigned char)ch);
  auto ends_with = [&](char const * ext) {
    size_t n = std::strlen(ext);
    return lower.size() >= n && lower.compare(lower.size() - n, n, ext) == 0;
  };
  // codecs in the reference's order of detection: 3DS, OBJ, OFF (.off, .off.bin), PLY
  bool tds = ends_with(".3ds");
  bool obj = ends_with(".obj"), off = ends_with(".off") || ends_with(".off.bin"), ply = ends_with(".ply");
  if (!tds && !obj && !off && !ply) fail(path, "could not detect the codec from the file extension");
  std::ifstream f(path, std::ios::binary);
  if (!f) fail(path, "cannot open the file");
  Input in;
  in.path = path;
  f.seekg(0, std::ios::end);
  std::streamoff size = f.tellg();
  f.seekg(0, std::ios::beg);
  if (size < 0) fail(path, "cannot read the file");
  in.data.resize((size_t)size);
  if (size > 0 && !f.read(&in.data[0], size)) fail(path, "cannot read the file");
  return tds ? read_3ds(in) : obj ? read_obj(in) : off ? read_off(in) : read_ply(in);
}

MeshData read_mesh_buffer(void const * data, int64_t bytes, std::string const & codec) {
  std::string c = codec;
  for (char & ch : c) ch = (char)std::tolower((unsigned char)ch);
  if (c != "3ds" && c != "obj" && c != "off" && c != "ply")
    fail("<buffer>", "unknown codec '" + codec + "' (3ds, obj, off or ply)");
  Input in;
  in.path = "<buffer>";
  if (bytes > 0) in.data.assign(static_cast<char const *>(data), (size_t)bytes);
  return c == "3ds" ? read_3ds(in) : c == "obj" ? read_obj(in) : c == "off" ? read_off(in) : read_ply(in);
}

}  // namespace thea
