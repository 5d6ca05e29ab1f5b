// ingest_parse.cpp -- host parsers of mesh ingest (see ingest_parse.h).
//
// OBJ, XYZ and PTS follow the line rules of the reference's own readers
// (io.cpp:292-480, 590-640, 659-685): fgets-sized pieces of at most 255
// (PTS: 1023) bytes, the same sscanf patterns tried in the same order, the
// same colour packing and index correction. PLY, OFF and STL follow their
// published format descriptions (the reference reads them through jtk,
// which it does not ship).
#include "ingest_parse.h"

#include <ctype.h>
#include <stdarg.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <thread>

namespace j3dg {
namespace ingest {

int type_size(int t) {
  switch (t) {
    case T_I8: case T_U8: return 1;
    case T_I16: case T_U16: return 2;
    case T_I32: case T_U32: case T_F32: return 4;
    case T_F64: return 8;
    default: return 0;
  }
}

bool PlyElement::has_list() const {
  for (const auto& p : props)
    if (p.list) return true;
  return false;
}

uint32_t PlyElement::fixed_size() const {
  uint32_t s = 0;
  for (const auto& p : props) {
    if (p.list) return 0;
    s += (uint32_t)type_size(p.type);
  }
  return s;
}

int PlyElement::find(const char* n) const {
  for (size_t i = 0; i < props.size(); ++i)
    if (props[i].name == n) return (int)i;
  return -1;
}

namespace {

int8_t type_of(const std::string& s) {
  if (s == "char" || s == "int8") return T_I8;
  if (s == "uchar" || s == "uint8") return T_U8;
  if (s == "short" || s == "int16") return T_I16;
  if (s == "ushort" || s == "uint16") return T_U16;
  if (s == "int" || s == "int32") return T_I32;
  if (s == "uint" || s == "uint32") return T_U32;
  if (s == "float" || s == "float32") return T_F32;
  if (s == "double" || s == "float64") return T_F64;
  return T_NONE;
}

std::vector<std::string> words(const std::string& line) {
  std::vector<std::string> w;
  size_t i = 0;
  while (i < line.size()) {
    while (i < line.size() && isspace((unsigned char)line[i])) ++i;
    size_t j = i;
    while (j < line.size() && !isspace((unsigned char)line[j])) ++j;
    if (j > i) w.push_back(line.substr(i, j - i));
    i = j;
  }
  return w;
}

uint64_t read_uint_le_be(const uint8_t* p, int size, bool be) {
  uint64_t v = 0;
  for (int i = 0; i < size; ++i) v |= (uint64_t)p[be ? size - 1 - i : i] << (8 * i);
  return v;
}

// A list count as a signed value (negative counts are malformed).
bool read_count(const uint8_t* p, int t, bool be, int64_t* out) {
  const int s = type_size(t);
  uint64_t v = read_uint_le_be(p, s, be);
  switch (t) {
    case T_I8: *out = (int8_t)v; break;
    case T_U8: *out = (uint8_t)v; break;
    case T_I16: *out = (int16_t)v; break;
    case T_U16: *out = (uint16_t)v; break;
    case T_I32: *out = (int32_t)v; break;
    case T_U32: *out = (uint32_t)v; break;
    default: return false;  // float counts are not valid PLY
  }
  return *out >= 0;
}

}  // namespace

bool parse_ply_header(const char* p, size_t n, PlyHeader& h, std::string& err) {
  h = PlyHeader();
  err.clear();
  size_t at = 0;
  bool first = true, have_format = false;
  while (true) {
    const char* nl = (const char*)memchr(p + at, '\n', n - at);
    if (!nl) return false;  // incomplete
    std::string line(p + at, nl - (p + at));
    at = (nl - p) + 1;
    if (!line.empty() && line.back() == '\r') line.pop_back();
    std::vector<std::string> w = words(line);
    if (first) {
      first = false;
      if (w.size() != 1 || w[0] != "ply") {
        err = "ply: missing magic";
        return false;
      }
      continue;
    }
    if (w.empty() || w[0] == "comment" || w[0] == "obj_info") continue;
    if (w[0] == "format") {
      if (w.size() < 2) { err = "ply: bad format line"; return false; }
      if (w[1] == "ascii") h.encoding = 0;
      else if (w[1] == "binary_little_endian") h.encoding = 1;
      else if (w[1] == "binary_big_endian") h.encoding = 2;
      else { err = "ply: unknown format " + w[1]; return false; }
      have_format = true;
    } else if (w[0] == "element") {
      if (w.size() != 3) { err = "ply: bad element line"; return false; }
      PlyElement e;
      e.name = w[1];
      char* end = nullptr;
      e.count = strtoull(w[2].c_str(), &end, 10);
      if (*end || w[2][0] == '-') { err = "ply: bad element count"; return false; }
      h.elements.push_back(e);
    } else if (w[0] == "property") {
      if (h.elements.empty()) { err = "ply: property before element"; return false; }
      PlyProp pr;
      if (w.size() == 5 && w[1] == "list") {
        pr.list = true;
        pr.count_type = type_of(w[2]);
        pr.item_type = type_of(w[3]);
        pr.name = w[4];
        if (!pr.count_type || !pr.item_type || pr.count_type == T_F32 || pr.count_type == T_F64) {
          err = "ply: bad list property";
          return false;
        }
      } else if (w.size() == 3) {
        pr.type = type_of(w[1]);
        pr.name = w[2];
        if (!pr.type) { err = "ply: unknown property type " + w[1]; return false; }
      } else {
        err = "ply: bad property line";
        return false;
      }
      h.elements.back().props.push_back(pr);
    } else if (w[0] == "end_header") {
      if (!have_format) { err = "ply: no format line"; return false; }
      h.header_bytes = at;
      return true;
    } else {
      err = "ply: unknown header line '" + w[0] + "'";
      return false;
    }
  }
}

bool skip_binary_element(const uint8_t* body, size_t n, size_t at, const PlyElement& e, bool be, size_t* end) {
  const uint32_t fs = e.fixed_size();
  if (fs) {
    if (e.count > (n - std::min(n, at)) / fs) return false;
    *end = at + (size_t)e.count * fs;
    return true;
  }
  for (uint64_t r = 0; r < e.count; ++r) {
    for (const auto& p : e.props) {
      if (!p.list) {
        at += type_size(p.type);
        continue;
      }
      const int cs = type_size(p.count_type);
      if (at + cs > n) return false;
      int64_t c;
      if (!read_count(body + at, p.count_type, be, &c)) return false;
      at += cs + (size_t)c * type_size(p.item_type);
    }
    if (at > n) return false;
  }
  *end = at;
  return true;
}

bool walk_binary_faces(const uint8_t* body, size_t n, size_t at, const PlyElement& e, bool be, int index_prop,
                       int tc_prop, std::vector<uint64_t>& list_off, std::vector<uint64_t>& tc_off,
                       std::vector<uint32_t>& tri_base, uint64_t* n_tris, size_t* end, std::string& err) {
  list_off.resize(e.count);
  tri_base.resize(e.count);
  if (tc_prop >= 0) tc_off.resize(e.count);
  uint64_t tris = 0;
  for (uint64_t r = 0; r < e.count; ++r) {
    for (int k = 0; k < (int)e.props.size(); ++k) {
      const PlyProp& p = e.props[k];
      if (!p.list) {
        at += type_size(p.type);
        continue;
      }
      const int cs = type_size(p.count_type);
      if (at + cs > n) { err = "ply: truncated face element"; return false; }
      int64_t c;
      if (!read_count(body + at, p.count_type, be, &c)) { err = "ply: bad list count"; return false; }
      if (k == index_prop) {
        list_off[r] = at;
        tri_base[r] = (uint32_t)tris;
        if (c >= 3) tris += (uint64_t)(c - 2);
        if (tris >= 0xffffffffull) { err = "ply: more than 2^32 triangles"; return false; }
      } else if (k == tc_prop) {
        tc_off[r] = at;
      }
      at += cs + (size_t)c * type_size(p.item_type);
    }
    if (at > n) { err = "ply: truncated face element"; return false; }
  }
  *n_tris = tris;
  *end = at;
  return true;
}

// ------------------------------------------------------------------ scan

int scan(const char* s, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  int n = 0;
  const char* f = fmt;
  while (*f) {
    if (isspace((unsigned char)*f)) {
      while (isspace((unsigned char)*f)) ++f;
      while (isspace((unsigned char)*s)) ++s;
      continue;
    }
    if (*f == '%') {
      const char conv = f[1];
      f += 2;
      while (isspace((unsigned char)*s)) ++s;
      if (!*s) {
        va_end(ap);
        return n ? n : -1;
      }
      char* e = nullptr;
      if (conv == 'f') {
        const float v = strtof(s, &e);
        if (e == s) break;
        *va_arg(ap, float*) = v;
      } else if (conv == 'd') {
        const long v = strtol(s, &e, 10);
        if (e == s) break;
        *va_arg(ap, int*) = (int)v;
      } else if (conv == 's') {
        char* out = va_arg(ap, char*);
        int k = 0;
        e = const_cast<char*>(s);
        while (*e && !isspace((unsigned char)*e)) {
          if (k < 255) out[k++] = *e;
          ++e;
        }
        out[k] = 0;
      } else {
        break;
      }
      s = e;
      ++n;
      continue;
    }
    if (!*s) {
      va_end(ap);
      return n ? n : -1;
    }
    if (*s != *f) break;
    ++s;
    ++f;
  }
  va_end(ap);
  return n;
}

namespace {

// fgets(buffer, cap + 1, f) pieces: at most cap bytes, ending after '\n'.
// The piece is copied NUL-terminated with zeroed bytes after it, so the
// fixed-index tests of the readers see no stale characters.
template <class F>
bool for_each_piece(const char* p, const char* end, size_t cap, F&& f) {
  std::vector<char> buf(cap + 16);
  while (p < end) {
    size_t len = 0;
    while (len < cap && p + len < end)
      if (p[len++] == '\n') break;
    memcpy(buf.data(), p, len);
    memset(buf.data() + len, 0, 16);
    if (!f(buf.data())) return false;
    p += len;
  }
  return true;
}

// (uint8_t)(x * 255.f) as the reference's x86 build evaluates it: a
// truncating conversion to int32 (out of range: INT32_MIN), then the low byte.
uint32_t byte_of(float x) {
  const float y = x * 255.f;
  int32_t i = INT32_MIN;
  if (y > -2147483648.f && y < 2147483648.f) i = (int32_t)y;
  return (uint32_t)(uint8_t)i;
}

struct ObjPart {
  std::vector<float> v, vn, vt;
  std::vector<uint32_t> clr, tri, tuv;
  std::string mtl, err;
};

// io.cpp:313-422, one piece
bool obj_piece(const char* b, ObjPart& o) {
  int ws = 0;
  while (ws < 250 && (b[ws] == ' ' || b[ws] == '\t')) ++ws;
  const char* q = b + ws;
  if (q[0] == 'm' && q[1] == 't' && q[2] == 'l' && q[3] == 'l' && q[4] == 'i' && q[5] == 'b') {
    char name[256];
    if (scan(q, "mtllib %s\n", name) == 1) o.mtl = name;
  }
  if (q[0] == 'v' && q[1] == ' ') {
    float x, y, z, r, g, bl;
    const int e = scan(q, "v %f %f %f %f %f %f\n", &x, &y, &z, &r, &g, &bl);
    if (e != 3 && e != 6) {
      o.err = "obj: bad vertex line";
      return false;
    }
    o.v.insert(o.v.end(), {x, y, z});
    if (e == 6) o.clr.push_back(0xff000000u | (byte_of(bl) << 16) | (byte_of(g) << 8) | byte_of(r));
  } else if (q[0] == 'v' && q[1] == 'n' && b[2] == ' ') {
    float x, y, z;
    if (scan(q, "vn %f %f %f\n", &x, &y, &z) != 3) {
      o.err = "obj: bad normal line";
      return false;
    }
    o.vn.insert(o.vn.end(), {x, y, z});
  } else if (q[0] == 'v' && q[1] == 't' && b[2] == ' ') {
    float x, y;
    if (scan(q, "vt %f %f\n", &x, &y) != 2) {
      o.err = "obj: bad texture coordinate line";
      return false;
    }
    o.vt.insert(o.vt.end(), {x, y});
  } else if (q[0] == 'f' && q[1] == ' ') {
    int t0, t1, t2, t3, v0, v1, v2, v3;
    auto tri = [&](int a, int b_, int c) { o.tri.insert(o.tri.end(), {(uint32_t)a - 1u, (uint32_t)b_ - 1u, (uint32_t)c - 1u}); };
    auto tuv = [&](int a, int b_, int c) { o.tuv.insert(o.tuv.end(), {(uint32_t)a - 1u, (uint32_t)b_ - 1u, (uint32_t)c - 1u}); };
    int e = scan(q, "f %d/%d %d/%d %d/%d %d/%d\n", &t0, &v0, &t1, &v1, &t2, &v2, &t3, &v3);
    if (e != 6 && e != 8) e = scan(q, "f %d/%d/ %d/%d/ %d/%d/ %d/%d/\n", &t0, &v0, &t1, &v1, &t2, &v2, &t3, &v3);
    if (e == 6 || e == 8) {
      tuv(v0, v1, v2);
      tri(t0, t1, t2);
      if (e == 8) {
        tuv(v0, v2, v3);
        tri(t0, t2, t3);
      }
      return true;
    }
    e = scan(q, "f %d %d %d %d\n", &t0, &t1, &t2, &t3);
    if (e == 3 || e == 4) {
      tri(t0, t1, t2);
      if (e == 4) tri(t0, t2, t3);
      return true;
    }
    int x0, x1, x2, x3;
    e = scan(q, "f %d/%d/%d %d/%d/%d %d/%d/%d %d/%d/%d\n", &t0, &v0, &x0, &t1, &v1, &x1, &t2, &v2, &x2, &t3, &v3, &x3);
    if (e == 9 || e == 12) {
      tuv(v0, v1, v2);
      tri(t0, t1, t2);
      if (e == 12) {
        tuv(v0, v2, v3);
        tri(t0, t2, t3);
      }
      return true;
    }
    o.err = "obj: unsupported face line";
    return false;
  }
  return true;
}

// Line-aligned chunks for the worker threads.
std::vector<std::pair<const char*, const char*>> chunks(const char* p, size_t n, int parts) {
  std::vector<std::pair<const char*, const char*>> out;
  const char* end = p + n;
  const char* at = p;
  for (int k = 1; k <= parts && at < end; ++k) {
    const char* c = (k == parts) ? end : p + (n * (size_t)k) / (size_t)parts;
    if (c < at) c = at;
    if (c < end) {
      const char* nl = (const char*)memchr(c, '\n', end - c);
      c = nl ? nl + 1 : end;
    }
    out.emplace_back(at, c);
    at = c;
  }
  return out;
}

template <class T>
void append(std::vector<T>& dst, const std::vector<T>& src) {
  dst.insert(dst.end(), src.begin(), src.end());
}

}  // namespace

bool parse_obj(const char* p, size_t n, int threads, HostGeometry& g, std::string& err) {
  g = HostGeometry();
  const int parts = std::max(1, std::min(threads, (int)(n / (1 << 20)) + 1));
  auto ranges = chunks(p, n, parts);
  std::vector<ObjPart> res(ranges.size());
  std::vector<std::thread> pool;
  std::vector<char> ok(ranges.size(), 1);
  for (size_t k = 0; k < ranges.size(); ++k) {
    auto work = [&, k] {
      ok[k] = for_each_piece(ranges[k].first, ranges[k].second, 255, [&](const char* b) { return obj_piece(b, res[k]); });
    };
    if (k + 1 == ranges.size()) work();
    else pool.emplace_back(work);
  }
  for (auto& t : pool) t.join();
  ObjPart all;
  for (size_t k = 0; k < res.size(); ++k) {
    if (!ok[k]) {
      err = res[k].err;
      return false;
    }
    append(all.v, res[k].v);
    append(all.vn, res[k].vn);
    append(all.vt, res[k].vt);
    append(all.clr, res[k].clr);
    append(all.tri, res[k].tri);
    append(all.tuv, res[k].tuv);
  }
  // io.cpp:437-452
  if (!all.tuv.empty() && all.tri.size() != all.tuv.size()) {
    err = "obj: faces with and without texture coordinates";
    return false;
  }
  const size_t nv = all.v.size() / 3;
  if (!all.tri.empty()) {  // correct_vertices_and_triangles (io.cpp:232-262)
    uint32_t lo = all.tri[0], hi = lo;
    for (uint32_t t : all.tri) {
      lo = std::min(lo, t);
      hi = std::max(hi, t);
    }
    if (hi >= nv && lo > 0) {
      for (auto& t : all.tri) t -= lo;
      for (auto& t : all.tuv) t -= lo;
    }
  }
  if (!all.tuv.empty()) {
    const size_t nt = all.vt.size() / 2;
    g.uv.resize(all.tuv.size() * 2);
    for (size_t i = 0; i < all.tuv.size(); ++i) {
      const uint32_t t = all.tuv[i];
      if (t >= nt) {
        err = "obj: texture coordinate index out of range";
        return false;
      }
      g.uv[2 * i] = all.vt[2 * t];
      g.uv[2 * i + 1] = 1.f - all.vt[2 * t + 1];
    }
  }
  g.vertices.swap(all.v);
  g.triangles.swap(all.tri);
  if (all.clr.size() == nv) g.colors.swap(all.clr);
  if (all.vn.size() == 3 * nv) g.normals.swap(all.vn);
  return true;
}

bool parse_pts(const char* p, size_t n, HostGeometry& g, std::string& err) {
  g = HostGeometry();
  std::vector<uint32_t> clr;
  uint32_t count = 0;
  bool have_count = false;
  bool ok = for_each_piece(p, p + n, 1023, [&](const char* b) {  // io.cpp:598-638
    int ws = 0;
    while (ws < 250 && (b[ws] == ' ' || b[ws] == '\t')) ++ws;
    const char* q = b + ws;
    float x, y, z;
    int in, r, gg, bb;
    int e = scan(q, "%f %f %f %d %d %d %d\n", &x, &y, &z, &in, &r, &gg, &bb);
    if (e == 7) {
      g.vertices.insert(g.vertices.end(), {x, y, z});
      clr.push_back(0xff000000u | ((uint32_t)bb << 16) | ((uint32_t)gg << 8) | (uint32_t)r);
      return true;
    }
    if (scan(q, "%f %f %f\n", &x, &y, &z) == 3) {
      g.vertices.insert(g.vertices.end(), {x, y, z});
      return true;
    }
    int c;
    if (scan(q, "%d\n", &c) != 1) {
      err = "pts: invalid line";
      return false;
    }
    count = (uint32_t)c;
    have_count = true;
    return true;
  });
  if (!ok) return false;
  if (have_count && count && g.vertices.size() / 3 != count) {
    err = "pts: point count does not match the header";
    return false;
  }
  if (clr.size() == g.vertices.size() / 3) g.colors.swap(clr);
  return true;
}

bool parse_xyz(const char* p, size_t n, HostGeometry& g, std::string& err) {
  g = HostGeometry();
  const char* end = p + n;
  while (p < end) {
    const char* nl = (const char*)memchr(p, '\n', end - p);
    const char* le = nl ? nl : end;
    std::string line(p, le);
    p = nl ? nl + 1 : end;
    bool blank = true;
    for (char ch : line)
      if (!isspace((unsigned char)ch)) blank = false;
    if (blank) continue;
    float v[3] = {0.f, 0.f, 0.f};
    const char* s = line.c_str();
    for (int k = 0; k < 3; ++k) {
      char* e = nullptr;
      const float x = strtof(s, &e);
      if (e == s) break;
      v[k] = x;
      s = e;
    }
    g.vertices.insert(g.vertices.end(), v, v + 3);
  }
  return true;
}

// ---------------------------------------------------------- token reader

namespace {

struct Tokens {
  const char* p;
  const char* end;
  bool next(const char** s, size_t* len) {
    while (p < end && isspace((unsigned char)*p)) ++p;
    if (p >= end) return false;
    *s = p;
    while (p < end && !isspace((unsigned char)*p)) ++p;
    *len = p - *s;
    return true;
  }
  bool number(double* out, bool as_float, float* fout) {
    const char* s;
    size_t len;
    if (!next(&s, &len) || len > 63) return false;
    char buf[64];
    memcpy(buf, s, len);
    buf[len] = 0;
    char* e = nullptr;
    if (as_float) {
      *fout = strtof(buf, &e);
      *out = *fout;
    } else {
      *out = strtod(buf, &e);
    }
    return e == buf + len;
  }
  bool integer(int64_t* out) {
    const char* s;
    size_t len;
    if (!next(&s, &len) || len > 63) return false;
    char buf[64];
    memcpy(buf, s, len);
    buf[len] = 0;
    char* e = nullptr;
    *out = strtoll(buf, &e, 10);
    return e == buf + len;
  }
};

// A value of a PLY property in its own type, widened.
struct Val {
  double d = 0;
  float f = 0;
  int64_t i = 0;
};

bool read_val(Tokens& t, int type, Val* v) {
  if (type == T_F32) {
    if (!t.number(&v->d, true, &v->f)) return false;
    return true;
  }
  if (type == T_F64) {
    if (!t.number(&v->d, false, &v->f)) return false;
    v->f = (float)v->d;
    return true;
  }
  if (!t.integer(&v->i)) return false;
  v->f = (float)v->i;
  return true;
}

// A colour channel: bytes as they are, other integers clamped to 0..255,
// floats scaled by 255, clamped and truncated.
uint32_t channel(int type, const Val& v) {
  if (type == T_F32 || type == T_F64) {
    float x = v.f * 255.f;
    x = x < 0.f ? 0.f : (x > 255.f ? 255.f : x);
    return x == x ? (uint32_t)x : 0u;
  }
  return (uint32_t)std::min<int64_t>(255, std::max<int64_t>(0, v.i));
}

}  // namespace

bool parse_ply_ascii(const char* p, size_t n, const PlyHeader& h, HostGeometry& g, std::string& err) {
  g = HostGeometry();
  Tokens t{p, p + n};
  bool uv_ok = true;
  for (const auto& e : h.elements) {
    const bool is_v = e.name == "vertex", is_f = e.name == "face";
    int ix = -1, iy = -1, iz = -1, inx = -1, iny = -1, inz = -1, ir = -1, ig = -1, ib = -1, il = -1, itc = -1;
    if (is_v) {
      ix = e.find("x"), iy = e.find("y"), iz = e.find("z");
      inx = e.find("nx"), iny = e.find("ny"), inz = e.find("nz");
      ir = e.find("red"), ig = e.find("green"), ib = e.find("blue");
      if (ix < 0 || iy < 0 || iz < 0) {
        err = "ply: vertex element without x, y, z";
        return false;
      }
      g.vertices.reserve(3 * e.count);
    }
    if (is_f) {
      il = e.find("vertex_indices");
      if (il < 0) il = e.find("vertex_index");
      itc = e.find("texcoord");
      if (itc < 0) itc = e.find("texcoords");
      if (il < 0 || !e.props[il].list) {
        err = "ply: face element without a vertex_indices list";
        return false;
      }
      if (itc >= 0 && !e.props[itc].list) itc = -1;
    }
    const bool normals = is_v && inx >= 0 && iny >= 0 && inz >= 0;
    const bool colors = is_v && ir >= 0 && ig >= 0 && ib >= 0;
    std::vector<Val> vals(e.props.size());
    std::vector<uint32_t> idx;
    std::vector<float> tc;
    for (uint64_t r = 0; r < e.count; ++r) {
      idx.clear();
      tc.clear();
      for (int k = 0; k < (int)e.props.size(); ++k) {
        const PlyProp& pr = e.props[k];
        if (!pr.list) {
          if (!read_val(t, pr.type, &vals[k])) {
            err = "ply: bad or missing value in element " + e.name;
            return false;
          }
          continue;
        }
        int64_t c;
        if (!t.integer(&c) || c < 0) {
          err = "ply: bad list count in element " + e.name;
          return false;
        }
        for (int64_t j = 0; j < c; ++j) {
          Val v;
          if (!read_val(t, pr.item_type, &v)) {
            err = "ply: bad or missing list item in element " + e.name;
            return false;
          }
          if (k == il) idx.push_back((uint32_t)v.i);
          if (k == itc) tc.push_back(v.f);
        }
      }
      if (is_v) {
        g.vertices.insert(g.vertices.end(), {vals[ix].f, vals[iy].f, vals[iz].f});
        if (normals) g.normals.insert(g.normals.end(), {vals[inx].f, vals[iny].f, vals[inz].f});
        if (colors)
          g.colors.push_back(0xff000000u | (channel(e.props[ib].type, vals[ib]) << 16) |
                             (channel(e.props[ig].type, vals[ig]) << 8) | channel(e.props[ir].type, vals[ir]));
      }
      if (is_f) {
        const size_t c = idx.size();
        const bool tc_here = itc >= 0 && tc.size() == 2 * c;
        if (itc >= 0 && !tc_here && c >= 3) uv_ok = false;
        for (size_t k = 0; c >= 3 && k + 2 < c; ++k) {
          g.triangles.insert(g.triangles.end(), {idx[0], idx[k + 1], idx[k + 2]});
          if (tc_here)
            g.uv.insert(g.uv.end(), {tc[0], tc[1], tc[2 * (k + 1)], tc[2 * (k + 1) + 1], tc[2 * (k + 2)], tc[2 * (k + 2) + 1]});
        }
      }
    }
  }
  if (!uv_ok || g.uv.size() != 2 * g.triangles.size()) g.uv.clear();
  return true;
}

// OFF: "OFF" (or "COFF"), counts "nv nf ne", nv vertex lines "x y z [r g b [a]]",
// nf face lines "n i0 .. i(n-1) [colour]"; '#' starts a comment.
bool parse_off(const char* p, size_t n, HostGeometry& g, std::string& err) {
  g = HostGeometry();
  const char* end = p + n;
  std::vector<std::string> lines;
  auto next_line = [&](std::vector<std::string>& w) -> bool {
    while (p < end) {
      const char* nl = (const char*)memchr(p, '\n', end - p);
      const char* le = nl ? nl : end;
      std::string line(p, le);
      p = nl ? nl + 1 : end;
      const size_t hash = line.find('#');
      if (hash != std::string::npos) line.resize(hash);
      w = words(line);
      if (!w.empty()) return true;
    }
    return false;
  };
  std::vector<std::string> w;
  if (!next_line(w) || (w[0] != "OFF" && w[0] != "COFF")) {
    err = "off: missing OFF magic";
    return false;
  }
  w.erase(w.begin());
  if (w.empty() && !next_line(w)) {
    err = "off: missing counts";
    return false;
  }
  if (w.size() < 2) {
    err = "off: bad counts line";
    return false;
  }
  char* e1 = nullptr;
  char* e2 = nullptr;
  const long long nv = strtoll(w[0].c_str(), &e1, 10), nf = strtoll(w[1].c_str(), &e2, 10);
  if (*e1 || *e2 || nv < 0 || nf < 0) {
    err = "off: bad counts line";
    return false;
  }
  std::vector<uint32_t> clr;
  for (long long i = 0; i < nv; ++i) {
    if (!next_line(w) || w.size() < 3) {
      err = "off: missing vertex line";
      return false;
    }
    float v[3];
    for (int k = 0; k < 3; ++k) {
      char* e = nullptr;
      v[k] = strtof(w[k].c_str(), &e);
      if (*e) {
        err = "off: bad vertex value";
        return false;
      }
    }
    g.vertices.insert(g.vertices.end(), v, v + 3);
    if (w.size() >= 6) {
      uint32_t ch[3];
      for (int k = 0; k < 3; ++k) {
        const std::string& s = w[3 + k];
        Val val;
        const bool is_float = s.find_first_of(".eE") != std::string::npos;
        if (is_float) val.f = strtof(s.c_str(), nullptr);
        else val.i = strtoll(s.c_str(), nullptr, 10);
        ch[k] = channel(is_float ? T_F32 : T_I32, val);
      }
      clr.push_back(0xff000000u | (ch[2] << 16) | (ch[1] << 8) | ch[0]);
    }
  }
  for (long long i = 0; i < nf; ++i) {
    if (!next_line(w)) {
      err = "off: missing face line";
      return false;
    }
    char* e = nullptr;
    const long long c = strtoll(w[0].c_str(), &e, 10);
    if (*e || c < 0 || (long long)w.size() < c + 1) {
      err = "off: bad face line";
      return false;
    }
    std::vector<uint32_t> idx(c);
    for (long long k = 0; k < c; ++k) idx[k] = (uint32_t)strtoll(w[1 + k].c_str(), nullptr, 10);
    for (long long k = 0; k + 2 < c; ++k) g.triangles.insert(g.triangles.end(), {idx[0], idx[k + 1], idx[k + 2]});
  }
  if (clr.size() == g.vertices.size() / 3) g.colors.swap(clr);
  return true;
}

// ASCII STL: every "vertex x y z" in order; three make a triangle (no
// welding: V = 3 T, triangle i = (3i, 3i+1, 3i+2)).
bool parse_stl_ascii(const char* p, size_t n, HostGeometry& g, std::string& err) {
  g = HostGeometry();
  Tokens t{p, p + n};
  const char* s;
  size_t len;
  if (!t.next(&s, &len) || len != 5 || memcmp(s, "solid", 5) != 0) {
    err = "stl: not an ASCII STL file";
    return false;
  }
  while (t.next(&s, &len)) {
    if (len == 6 && memcmp(s, "vertex", 6) == 0) {
      for (int k = 0; k < 3; ++k) {
        double d;
        float f;
        if (!t.number(&d, true, &f)) {
          err = "stl: bad vertex";
          return false;
        }
        g.vertices.push_back(f);
      }
    }
  }
  if (g.vertices.size() % 9) {
    err = "stl: vertex count is not a multiple of 3";
    return false;
  }
  const uint32_t nt = (uint32_t)(g.vertices.size() / 9);
  g.triangles.resize(3 * (size_t)nt);
  for (uint32_t i = 0; i < 3 * nt; ++i) g.triangles[i] = i;
  return true;
}

std::vector<uint32_t> dummy_texture(int w, int h, int block) {
  std::vector<uint32_t> im((size_t)w * h);
  for (int y = 0; y < h; ++y) {
    const bool y_odd = ((y / block) & 1) == 1;
    for (int x = 0; x < w; ++x) {
      const bool x_odd = ((x / block) & 1) == 1;
      const bool black = (x_odd && y_odd) || (!x_odd && !y_odd);
      im[(size_t)y * w + x] = black ? 0xff000000u : 0xffffffffu;
    }
  }
  return im;
}

}  // namespace ingest
}  // namespace j3dg
