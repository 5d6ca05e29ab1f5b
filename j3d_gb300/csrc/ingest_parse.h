// ingest_parse.h -- host side of mesh ingest: the PLY header and the text
// formats (ASCII PLY, OBJ, OFF, ASCII STL, XYZ, PTS). Binary bodies (PLY,
// STL) are not touched here: their record layouts (PlyHeader) go to the
// device decoders in ingest.cu.
#pragma once
#include <stddef.h>
#include <stdint.h>

#include <string>
#include <vector>

namespace j3dg {
namespace ingest {

// PLY scalar types (char/int8 ... double/float64)
enum ScalarType : int8_t { T_NONE = 0, T_I8, T_U8, T_I16, T_U16, T_I32, T_U32, T_F32, T_F64 };
int type_size(int t);

struct PlyProp {
  std::string name;
  int8_t type = T_NONE;        // scalar property type
  bool list = false;
  int8_t count_type = T_NONE;  // list: type of the count
  int8_t item_type = T_NONE;   // list: type of the items
};

struct PlyElement {
  std::string name;
  uint64_t count = 0;
  std::vector<PlyProp> props;
  bool has_list() const;
  uint32_t fixed_size() const;  // record bytes when there is no list, else 0
  int find(const char* name) const;
};

struct PlyHeader {
  int encoding = 0;  // 0 ascii, 1 binary little endian, 2 binary big endian
  std::vector<PlyElement> elements;
  size_t header_bytes = 0;  // offset of the body
};

// Decoded arrays of a text format (uploaded as they are).
struct HostGeometry {
  std::vector<float> vertices;      // 3 V
  std::vector<uint32_t> triangles;  // 3 T
  std::vector<uint32_t> colors;     // V, or empty
  std::vector<float> normals;       // 3 V, or empty
  std::vector<float> uv;            // 6 T, or empty
};

// Parses the header from p[0..n). Returns false with `err` when the header
// is malformed, or when it is incomplete in n bytes (err empty then).
bool parse_ply_header(const char* p, size_t n, PlyHeader& h, std::string& err);

// Walks the binary records of one element from `at` and returns the offset
// after them (for elements with list properties), or false when the body
// ends early.
bool skip_binary_element(const uint8_t* body, size_t n, size_t at, const PlyElement& e, bool big_endian,
                         size_t* end);

// Record offsets of a binary face element whose lists vary in length: for
// each record the offset of its index-list count, of its texcoord-list
// count (or UINT64_MAX), and the first output triangle (fan triangulation,
// max(count - 2, 0) triangles per record).
bool walk_binary_faces(const uint8_t* body, size_t n, size_t at, const PlyElement& e, bool big_endian,
                       int index_prop, int tc_prop, std::vector<uint64_t>& list_off, std::vector<uint64_t>& tc_off,
                       std::vector<uint32_t>& tri_base, uint64_t* n_tris, size_t* end, std::string& err);

bool parse_ply_ascii(const char* p, size_t n, const PlyHeader& h, HostGeometry& g, std::string& err);
bool parse_obj(const char* p, size_t n, int threads, HostGeometry& g, std::string& err);
bool parse_off(const char* p, size_t n, HostGeometry& g, std::string& err);
bool parse_stl_ascii(const char* p, size_t n, HostGeometry& g, std::string& err);
bool parse_xyz(const char* p, size_t n, HostGeometry& g, std::string& err);
bool parse_pts(const char* p, size_t n, HostGeometry& g, std::string& err);

// mesh.cpp:21-36 make_dummy_texture(w, h, block_size)
std::vector<uint32_t> dummy_texture(int w, int h, int block);

// The sscanf subset io.cpp's readers use (%f, %d, %s, whitespace, literal
// characters), on a NUL-terminated string. Exposed for tests.
int scan(const char* s, const char* fmt, ...);

}  // namespace ingest
}  // namespace j3dg
