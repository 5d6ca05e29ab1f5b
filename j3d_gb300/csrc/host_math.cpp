// host_math.cpp -- host-side j3d math of libj3dgpu.so (no GPU needed).
//
// Camera, scene and matcap functions restate the reference's own host code
// (file:line on each function) in the fp32 operation order the device kernels
// use. The synthetic-workload generators stand in for j3d's mesh readers
// (not on the hot path): they use their own PRNG (splitmix64 -> PCG32) and
// their own sine so that x86 and Arm hosts produce the same bytes.
//
// Built with -ffp-contract=off and without -ffast-math.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <limits>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/j3dg.h"
#include "internal.h"

namespace {

// float4x4 (column-major) times float4: r_i = ((m[i]x + m[4+i]y) + m[8+i]z) + m[12+i]w
void mat_vec(const float* m, const float* v, float* r) {
  float out[4];
  for (int i = 0; i < 4; ++i) {
    float s = m[i] * v[0];
    s = s + m[4 + i] * v[1];
    s = s + m[8 + i] * v[2];
    s = s + m[12 + i] * v[3];
    out[i] = s;
  }
  std::memcpy(r, out, sizeof(out));
}

void frustum(float left, float right, float bottom, float top, float n, float f, float* out) {
  // camera.cpp:18-24
  const float m[16] = {2.f * n / (right - left), 0.f, 0.f, 0.f,
                       0.f, -2.f * n / (top - bottom), 0.f, 0.f,
                       (right + left) / (right - left), -(top + bottom) / (top - bottom), -(f + n) / (f - n), -1.f,
                       0.f, 0.f, -(2.f * f * n) / (f - n), 0.f};
  std::memcpy(out, m, sizeof(m));
}

// ---------------------------------------------------------- determinism ----

uint64_t splitmix64(uint64_t& s) {
  uint64_t z = (s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// PCG32 (O'Neill 2014, XSH RR) seeded from splitmix64(seed).
struct Pcg32 {
  uint64_t state = 0, inc = 1;
  explicit Pcg32(uint64_t seed) {
    uint64_t s = seed;
    uint64_t init_state = splitmix64(s);
    uint64_t init_seq = splitmix64(s);
    inc = (init_seq << 1u) | 1u;
    next();
    state += init_state;
    next();
  }
  uint32_t next() {
    uint64_t old = state;
    state = old * 6364136223846793005ull + inc;
    uint32_t xs = (uint32_t)(((old >> 18u) ^ old) >> 27u);
    uint32_t rot = (uint32_t)(old >> 59u);
    return (xs >> rot) | (xs << ((32u - rot) & 31u));
  }
  // 24-bit uniform in [0, 1)
  double u01() { return (double)(next() >> 8) * (1.0 / 16777216.0); }
  double uniform(double a, double b) { return a + (b - a) * u01(); }
  // uniform direction by rejection from the cube (no transcendental calls)
  void unit3(double* v) {
    for (;;) {
      double x = uniform(-1.0, 1.0), y = uniform(-1.0, 1.0), z = uniform(-1.0, 1.0);
      double n2 = x * x + y * y + z * z;
      if (n2 > 1e-6 && n2 <= 1.0) {
        double n = std::sqrt(n2);
        v[0] = x / n;
        v[1] = y / n;
        v[2] = z / n;
        return;
      }
    }
  }
};

const double kPi = 3.141592653589793116;         // nearest double to pi
const double kPiLo = 1.2246467991473532e-16;     // pi - kPi
const double kTwoPi = 6.283185307179586232;
const double kTwoPiLo = 2.4492935982947064e-16;

// sin on doubles: Cody-Waite reduction by 2*pi, fold to [-pi/2, pi/2], odd
// Taylor polynomial to x^23 (error < 1e-17 there). IEEE +,-,*,/ and floor only.
double det_sin(double x) {
  double k = std::floor(x / kTwoPi + 0.5);
  double r = (x - k * kTwoPi) - k * kTwoPiLo;  // ~[-pi, pi]
  if (r > 0.5 * kPi)
    r = (kPi - r) + kPiLo;
  else if (r < -0.5 * kPi)
    r = (-kPi - r) - kPiLo;
  // sin r = r * sum_j (-1)^j r^(2j) / (2j+1)!, j = 0..11, Horner in r^2
  static const double C[12] = {1.0,
                               -1.0 / 6.0,
                               1.0 / 120.0,
                               -1.0 / 5040.0,
                               1.0 / 362880.0,
                               -1.0 / 39916800.0,
                               1.0 / 6227020800.0,
                               -1.0 / 1307674368000.0,
                               1.0 / 355687428096000.0,
                               -1.0 / 121645100408832000.0,
                               1.0 / 51090942171709440000.0,
                               -1.0 / 25852016738884976640000.0};
  double r2 = r * r;
  double p = C[11];
  for (int j = 10; j >= 0; --j) p = p * r2 + C[j];
  return r * p;
}

}  // namespace

// --------------------------------------------------------------- camera ----

extern "C" void j3dg_make_default_camera(j3dg_camera* c) {
  // camera.cpp:5-16
  c->focal_length = 35.f;
  c->film_aperture_width_inch = 1.024f;
  c->film_aperture_height_inch = 0.768f;
  c->near_clipping_plane = 0.1f;
  c->far_clipping_plane = std::numeric_limits<float>::max();
  c->fit_film = 1;
  c->zoom = 1.f;
}

extern "C" void j3dg_make_projection_matrix(const j3dg_camera* c, int screen_w, int screen_h, float* out) {
  // camera.cpp:32-73
  const float inchToMm = 25.4f;
  float top = ((c->film_aperture_height_inch * inchToMm / 2.f) / c->focal_length) * c->near_clipping_plane;
  float right = ((c->film_aperture_width_inch * inchToMm / 2.f) / c->focal_length) * c->near_clipping_plane;
  float xscale = c->zoom, yscale = c->zoom;
  float device_aspect = screen_w / (float)screen_h;
  float film_aspect = c->film_aperture_width_inch / c->film_aperture_height_inch;
  if (c->fit_film == 1) {  // Overscan
    if (film_aspect > device_aspect)
      yscale *= film_aspect / device_aspect;
    else
      xscale *= device_aspect / film_aspect;
  } else {  // Fill
    if (film_aspect > device_aspect)
      xscale *= device_aspect / film_aspect;
    else
      yscale *= film_aspect / device_aspect;
  }
  right *= xscale;
  top *= yscale;
  frustum(-right, right, -top, top, c->near_clipping_plane, c->far_clipping_plane, out);
}

extern "C" void j3dg_invert_projection_matrix(const float* in, float* out) {
  // camera.cpp:26-30
  const float m[16] = {1.f / in[0], 0.f, 0.f, 0.f, 0.f, 1.f / in[5], 0.f, 0.f, 0.f, 0.f, 0.f, 1.f / in[14],
                       in[8] / in[0], in[9] / in[5], -1.f, in[10] / in[14]};
  std::memcpy(out, m, sizeof(m));
}

extern "C" void j3dg_invert_orthonormal(const float* m, float* o) {
  // transpose of the rotation, translation -(R^T t) with fixed dot order
  float r[16] = {m[0], m[4], m[8], 0.f, m[1], m[5], m[9], 0.f, m[2], m[6], m[10], 0.f, 0.f, 0.f, 0.f, 1.f};
  for (int i = 0; i < 3; ++i) {
    float s = m[4 * i + 0] * m[12];
    s = s + m[4 * i + 1] * m[13];
    s = s + m[4 * i + 2] * m[14];
    r[12 + i] = -s;
  }
  std::memcpy(o, r, sizeof(r));
}

// ---------------------------------------------------------------- scene ----

extern "C" int j3dg_prepare_scene(const j3dg_instance* objects, uint32_t n, float* mn, float* mx, float* diagonal) {
  // scene.cpp:50-89 over mesh objects: bbox of each object taken through its cs
  if (!mn || !mx || !diagonal || (n && !objects)) return J3DG_ERR_INVALID_ARGUMENT;
  auto tp = [](const float* cs, const float* p, float* o) {
    float v[4] = {p[0], p[1], p[2], 1.f}, r[4];
    mat_vec(cs, v, r);
    o[0] = r[0];
    o[1] = r[1];
    o[2] = r[2];
  };
  for (uint32_t i = 0; i < n; ++i)
    if (!objects[i].mesh) return J3DG_ERR_INVALID_ARGUMENT;
  if (n == 0) {
    for (int k = 0; k < 3; ++k) mn[k] = mx[k] = 0.f;
  } else {
    float a[3], b[3];
    tp(objects[0].cs, objects[0].mesh->min_bb, a);
    tp(objects[0].cs, objects[0].mesh->max_bb, b);
    for (int k = 0; k < 3; ++k) {
      mn[k] = std::min(a[k], b[k]);
      mx[k] = std::max(a[k], b[k]);
    }
  }
  for (uint32_t i = 0; i < n; ++i) {
    float a[3], b[3];
    tp(objects[i].cs, objects[i].mesh->min_bb, a);
    tp(objects[i].cs, objects[i].mesh->max_bb, b);
    for (int k = 0; k < 3; ++k) {
      mn[k] = std::min(mn[k], std::min(a[k], b[k]));
      mx[k] = std::max(mx[k], std::max(a[k], b[k]));
    }
  }
  float d = mx[0] - mn[0];
  d = std::max<float>(d, mx[1] - mn[1]);
  d = std::max<float>(d, mx[2] - mn[2]);
  *diagonal = d;
  return J3DG_OK;
}

extern "C" int j3dg_prepare_scene_pointclouds(const j3dg_instance* objects, uint32_t n, const j3dg_pointcloud_instance* pcs,
                                              uint32_t n_pcs, float* mn, float* mx, float* diagonal) {
  // scene.cpp:50-89: the first mesh object's box (else the first cloud's)
  // widened by every object's and every cloud's box, each through its cs
  if (!mn || !mx || !diagonal || (n && !objects) || (n_pcs && !pcs)) return J3DG_ERR_INVALID_ARGUMENT;
  if (int rc = j3dg_prepare_scene(objects, n, mn, mx, diagonal)) return rc;
  for (uint32_t i = 0; i < n_pcs; ++i) {
    if (!pcs[i].pointcloud) return J3DG_ERR_INVALID_ARGUMENT;
    float a[3], b[3], v[4], r[4];
    for (int k = 0; k < 3; ++k) v[k] = pcs[i].pointcloud->min_bb[k];
    v[3] = 1.f;
    mat_vec(pcs[i].cs, v, r);
    for (int k = 0; k < 3; ++k) a[k] = r[k];
    for (int k = 0; k < 3; ++k) v[k] = pcs[i].pointcloud->max_bb[k];
    mat_vec(pcs[i].cs, v, r);
    for (int k = 0; k < 3; ++k) b[k] = r[k];
    for (int k = 0; k < 3; ++k) {
      const float lo = std::min(a[k], b[k]), hi = std::max(a[k], b[k]);
      mn[k] = (n == 0 && i == 0) ? lo : std::min(mn[k], lo);
      mx[k] = (n == 0 && i == 0) ? hi : std::max(mx[k], hi);
    }
  }
  float d = mx[0] - mn[0];
  d = std::max<float>(d, mx[1] - mn[1]);
  d = std::max<float>(d, mx[2] - mn[2]);
  *diagonal = d;
  return J3DG_OK;
}

extern "C" void j3dg_unzoom(const float* mn, const float* mx, float diagonal, float* cs, float* cs_inv, float* pivot) {
  // scene.cpp:91-110, y axis up
  for (int i = 0; i < 16; ++i) cs[i] = (i % 5 == 0) ? 1.f : 0.f;
  for (int j = 0; j < 3; ++j) pivot[j] = (mn[j] + mx[j]) * 0.5f;
  cs[12] = pivot[0];
  cs[13] = pivot[1];
  cs[14] = pivot[2] + diagonal * 2.f;
  j3dg_invert_orthonormal(cs, cs_inv);
}

// -------------------------------------------------------------- picking ----

extern "C" uint32_t j3dg_get_closest_vertex(const j3dg_pixel* p, const float* V, const uint32_t* T) {
  // pixel.cpp:6-25
  const uint32_t* t = T + 3 * (size_t)p->object_id;
  const float* A = V + 3 * (size_t)t[0];
  const float* B = V + 3 * (size_t)t[1];
  const float* C = V + 3 * (size_t)t[2];
  const float wgt = 1.f - p->barycentric_u - p->barycentric_v;
  float pos[3], d[3] = {0.f, 0.f, 0.f};
  for (int k = 0; k < 3; ++k) pos[k] = A[k] * wgt + p->barycentric_u * B[k] + p->barycentric_v * C[k];
  const float* P[3] = {A, B, C};
  for (int j = 0; j < 3; ++j) {
    float e0 = pos[0] - P[j][0], e1 = pos[1] - P[j][1], e2 = pos[2] - P[j][2];
    float s = e0 * e0;
    s = s + e1 * e1;
    d[j] = s + e2 * e2;
  }
  return (d[0] < d[1]) ? ((d[0] < d[2]) ? t[0] : t[2]) : ((d[1] < d[2]) ? t[1] : t[2]);
}

extern "C" void j3dg_get_world_position(const j3dg_pixel* p, const float* V, const uint32_t* T, const float* cs,
                                        float* out) {
  // view.cpp:439-459, mesh branch: barycentric point, then cs x point
  const uint32_t* t = T + 3 * (size_t)p->object_id;
  const float* A = V + 3 * (size_t)t[0];
  const float* B = V + 3 * (size_t)t[1];
  const float* C = V + 3 * (size_t)t[2];
  const float wgt = 1.f - p->barycentric_u - p->barycentric_v;
  float pos[4];
  for (int k = 0; k < 3; ++k) pos[k] = A[k] * wgt + p->barycentric_u * B[k] + p->barycentric_v * C[k];
  pos[3] = 1.f * wgt + p->barycentric_u * 1.f + p->barycentric_v * 1.f;
  float w[4];
  mat_vec(cs, pos, w);
  out[0] = w[0];
  out[1] = w[1];
  out[2] = w[2];
}

// --------------------------------------------------------------- canvas ----

extern "C" void j3dg_fill_background(uint32_t* bg, uint32_t w, uint32_t h, uint32_t top, uint32_t bottom) {
  // canvas.cpp:55-78
  uint32_t tr = top & 0xff, tg = (top >> 8) & 0xff, tb = (top >> 16) & 0xff;
  uint32_t br = bottom & 0xff, bgr = (bottom >> 8) & 0xff, bb = (bottom >> 16) & 0xff;
  for (uint32_t y = 0; y < h; ++y) {
    float scale = (float)y / (float)h;
    uint32_t r = (uint32_t)(scale * (float)br + (1.f - scale) * (float)tr);
    uint32_t g = (uint32_t)(scale * (float)bgr + (1.f - scale) * (float)tg);
    uint32_t b = (uint32_t)(scale * (float)bb + (1.f - scale) * (float)tb);
    uint32_t clr = 0xff000000u | ((uint32_t)(unsigned char)b << 16) | ((uint32_t)(unsigned char)g << 8) |
                   (uint32_t)(unsigned char)r;
    for (uint32_t x = 0; x < w; ++x) bg[(size_t)y * w + x] = clr;
  }
}

extern "C" int j3dg_make_matcap(int type, uint32_t* px, uint32_t* pw, uint32_t* ph, uint32_t* cavity) {
  // matcap.cpp:9-268 (procedural matcaps; PNG matcaps arrive as pixels)
  if (!px || type < 0 || type > 3) return J3DG_ERR_INVALID_ARGUMENT;
  const uint32_t w = 512, h = 512;
  if (pw) *pw = w;
  if (ph) *ph = h;
  uint32_t cav;
  if (type == 3) {  // sketch, matcap.cpp:241-268
    cav = 0xFF505050u;
    const float thres = 0.4f;
    for (uint32_t y = 0; y < h; ++y) {
      uint32_t* row = px + (size_t)(h - y - 1) * w;
      for (uint32_t x = 0; x < w; ++x) {
        float u = (float)x / (float)(w - 1) * 2.f - 1.f;
        float v = (float)y / (float)(h - 1) * 2.f - 1.f;
        float val = std::fabs(1.f - u * u - v * v);
        if (val < thres) {
          uint32_t s = (uint32_t)((val / thres) * (float)0xe1);
          row[x] = 0xff000000u | (s << 16) | (s << 8) | s;
        } else {
          row[x] = 0xffe1e1e1u;
        }
      }
    }
    if (cavity) *cavity = cav;
    return J3DG_OK;
  }
  // per-type weights of the four lobes and the channel offsets
  float k1[3], k2[3], off[3];
  const float k3[3] = {50.f, 50.f, 50.f}, k4[3] = {30.f, 30.f, 30.f};
  if (type == 0) {  // red wax, matcap.cpp:164-239
    cav = 0xFF7D7DFFu;
    const float a[3] = {200.f / 1.5f, 200.f / 4.f, 150.f / 4.f}, b[3] = {30.f, 25.f, 20.f}, o[3] = {32.f, 0.f, 0.f};
    std::memcpy(k1, a, sizeof a);
    std::memcpy(k2, b, sizeof b);
    std::memcpy(off, o, sizeof o);
  } else if (type == 1) {  // gray, matcap.cpp:9-84
    cav = 0xff505050u;
    const float a[3] = {200.f / 4.f, 200.f / 4.f, 200.f / 4.f}, b[3] = {50.f, 50.f, 50.f}, o[3] = {32.f, 32.f, 32.f};
    std::memcpy(k1, a, sizeof a);
    std::memcpy(k2, b, sizeof b);
    std::memcpy(off, o, sizeof o);
  } else {  // brown, matcap.cpp:87-162
    cav = 0xff405060u;
    const float a[3] = {200.f / 4.f, 180.f / 4.f, 160.f / 4.f}, b[3] = {50.f, 40.f, 30.f}, o[3] = {32.f, 20.f, 10.f};
    std::memcpy(k1, a, sizeof a);
    std::memcpy(k2, b, sizeof b);
    std::memcpy(off, o, sizeof o);
  }
  auto nrm = [](float x, float y, float z, float* o) {
    float len = std::sqrt((x * x + y * y) + z * z);
    o[0] = x / len;
    o[1] = y / len;
    o[2] = z / len;
  };
  float n1[3], n2[3], n3[3];
  nrm(0.f, 0.8f, 1.f, n1);
  nrm(0.f, 0.4f, 1.f, n2);
  nrm(0.f, 0.f, 1.f, n3);
  auto dot = [](const float* a, const float* b) {
    float s = a[0] * b[0];
    s = s + a[1] * b[1];
    return s + a[2] * b[2];
  };
  for (uint32_t y = 0; y < h; ++y) {
    uint32_t* row = px + (size_t)(h - y - 1) * w;
    for (uint32_t x = 0; x < w; ++x) {
      float u = (float)x / (float)(w - 1) * 2.f - 1.f;
      float v = (float)y / (float)(h - 1) * 2.f - 1.f;
      if (u * u + v * v <= 1.01f) {
        float sp[3] = {u, v, std::sqrt(1.01f - u * u - v * v)};
        float c1 = dot(sp, n1);
        float c2 = std::pow(dot(sp, n2), 3.f);
        float c3 = std::pow(dot(sp, n3), 5.f);
        float c4 = std::pow(dot(sp, n3), 50.f);
        unsigned char ch[3];
        for (int k = 0; k < 3; ++k) {
          float s = k1[k] * c1 + k2[k] * c2 + k3[k] * c3 + k4[k] * c4;
          float val = off[k] + s / 1.f;
          if (val > 255.f) val = 255.f;
          if (val < 0.f) val = 0.f;
          ch[k] = (unsigned char)val;
        }
        row[x] = 0xff000000u | ((uint32_t)ch[2] << 16) | ((uint32_t)ch[1] << 8) | (uint32_t)ch[0];
      } else {
        row[x] = 0xff000000u;
      }
    }
  }
  if (cavity) *cavity = cav;
  return J3DG_OK;
}

// ------------------------------------------------------------ workloads ----

extern "C" float j3dg_focal_for_vfov(float vfov_deg, float film_h_inch) {
  double half = 0.5 * (double)vfov_deg * (kPi / 180.0);
  double t = det_sin(half) / det_sin(half + 0.5 * kPi);
  return (float)(((double)film_h_inch * 25.4 * 0.5) / t);
}

extern "C" int j3dg_synth_icosphere(uint32_t level, uint64_t seed, float amp, float* V, uint32_t* T) {
  if (!V || !T || level > 11) return J3DG_ERR_INVALID_ARGUMENT;
  const double p = (1.0 + std::sqrt(5.0)) * 0.5;
  std::vector<double> P = {-1, p, 0, 1, p, 0, -1, -p, 0, 1, -p, 0, 0, -1, p, 0, 1, p,
                           0, -1, -p, 0, 1, -p, p, 0, -1, p, 0, 1, -p, 0, -1, -p, 0, 1};
  std::vector<uint32_t> F = {0, 11, 5, 0, 5,  1,  0,  1,  7,  0,  7,  10, 0,  10, 11, 1, 5, 9, 5, 11,
                             4, 11, 10, 2, 10, 7, 6, 7, 1, 8, 3, 9, 4, 3, 4, 2, 3, 2, 6, 3,
                             6, 8, 3, 8, 9, 4, 9, 5, 2, 4, 11, 6, 2, 10, 8, 6, 7, 9, 8, 1};
  auto norm = [](double* v) {
    double n = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    v[0] /= n;
    v[1] /= n;
    v[2] /= n;
  };
  for (size_t i = 0; i < P.size(); i += 3) norm(&P[i]);
  for (uint32_t l = 0; l < level; ++l) {
    std::unordered_map<uint64_t, uint32_t> mid;
    mid.reserve(F.size());
    std::vector<uint32_t> G;
    G.reserve(F.size() * 4);
    auto midpoint = [&](uint32_t a, uint32_t b) {
      uint64_t key = a < b ? ((uint64_t)a << 32 | b) : ((uint64_t)b << 32 | a);
      auto it = mid.find(key);
      if (it != mid.end()) return it->second;
      double m[3] = {P[3 * a] + P[3 * b], P[3 * a + 1] + P[3 * b + 1], P[3 * a + 2] + P[3 * b + 2]};
      norm(m);
      uint32_t id = (uint32_t)(P.size() / 3);
      P.insert(P.end(), m, m + 3);
      mid.emplace(key, id);
      return id;
    };
    for (size_t f = 0; f < F.size(); f += 3) {
      uint32_t a = F[f], b = F[f + 1], c = F[f + 2];
      uint32_t ab = midpoint(a, b), bc = midpoint(b, c), ca = midpoint(c, a);
      const uint32_t t[12] = {a, ab, ca, b, bc, ab, c, ca, bc, ab, bc, ca};
      G.insert(G.end(), t, t + 12);
    }
    F.swap(G);
  }
  // radial displacement, draws in this order per term: a, f, u (rejection), phi
  Pcg32 rng(seed);
  double a[8], f[8], u[8][3], ph[8];
  for (int k = 0; k < 8; ++k) {
    a[k] = rng.u01();
    f[k] = rng.uniform(2.0, 12.0);
    rng.unit3(u[k]);
    ph[k] = rng.uniform(0.0, kTwoPi);
  }
  const size_t nv = P.size() / 3;
  for (size_t i = 0; i < nv; ++i) {
    const double* d = &P[3 * i];
    double s = 0.0;
    for (int k = 0; k < 8; ++k) s += a[k] * det_sin(f[k] * (d[0] * u[k][0] + d[1] * u[k][1] + d[2] * u[k][2]) + ph[k]);
    double rad = 1.0 + (double)amp * s;
    for (int c = 0; c < 3; ++c) V[3 * i + c] = (float)(rad * d[c]);
  }
  std::memcpy(T, F.data(), F.size() * sizeof(uint32_t));
  return J3DG_OK;
}

extern "C" int j3dg_synth_torus(uint32_t nu, uint32_t nv, float R, float r, uint64_t seed, float amp, float* V,
                                uint32_t* T) {
  if (!V || !T || nu < 3 || nv < 3) return J3DG_ERR_INVALID_ARGUMENT;
  const int K = 16;
  // draws per term: amplitude a ~ U(0,1), integer frequencies m in [1,24] and
  // n in [1,12] (periodic in both grid directions), phase ~ U(0, 2 pi)
  Pcg32 rng(seed);
  double a[K], ps[K];
  int m[K], n[K];
  for (int k = 0; k < K; ++k) {
    a[k] = rng.u01();
    m[k] = 1 + (int)(rng.next() % 24u);
    n[k] = 1 + (int)(rng.next() % 12u);
    ps[k] = rng.uniform(0.0, kTwoPi);
  }
  // sin(m theta + n phi + psi) = sinA cosB + cosA sinB with per-grid-line tables
  std::vector<double> sA((size_t)K * nu), cA((size_t)K * nu), sB((size_t)K * nv), cB((size_t)K * nv);
  std::vector<double> cth(nu), sth(nu), cph(nv), sph(nv);
  for (uint32_t i = 0; i < nu; ++i) {
    double th = kTwoPi * (double)i / (double)nu;
    sth[i] = det_sin(th);
    cth[i] = det_sin(th + 0.5 * kPi);
    for (int k = 0; k < K; ++k) {
      double A = (double)m[k] * th;
      sA[(size_t)k * nu + i] = det_sin(A);
      cA[(size_t)k * nu + i] = det_sin(A + 0.5 * kPi);
    }
  }
  for (uint32_t j = 0; j < nv; ++j) {
    double ph = kTwoPi * (double)j / (double)nv;
    sph[j] = det_sin(ph);
    cph[j] = det_sin(ph + 0.5 * kPi);
    for (int k = 0; k < K; ++k) {
      double B = (double)n[k] * ph + ps[k];
      sB[(size_t)k * nv + j] = det_sin(B);
      cB[(size_t)k * nv + j] = det_sin(B + 0.5 * kPi);
    }
  }
  unsigned nth = std::max(1u, std::min(64u, std::thread::hardware_concurrency()));
  std::vector<std::thread> th;
  for (unsigned t = 0; t < nth; ++t)
    th.emplace_back([&, t] {
      for (uint32_t i = t; i < nu; i += nth) {
        for (uint32_t j = 0; j < nv; ++j) {
          double s = 0.0;
          for (int k = 0; k < K; ++k)
            s += a[k] * (sA[(size_t)k * nu + i] * cB[(size_t)k * nv + j] + cA[(size_t)k * nu + i] * sB[(size_t)k * nv + j]);
          double rr = (double)r + (double)amp * s;
          double ring = (double)R + rr * cph[j];
          size_t vi = (size_t)i * nv + j;
          V[3 * vi + 0] = (float)(ring * cth[i]);
          V[3 * vi + 1] = (float)(rr * sph[j]);
          V[3 * vi + 2] = (float)(ring * sth[i]);
          uint32_t i1 = (i + 1 == nu) ? 0 : i + 1, j1 = (j + 1 == nv) ? 0 : j + 1;
          uint32_t q0 = i * nv + j, q1 = i1 * nv + j, q2 = i1 * nv + j1, q3 = i * nv + j1;
          uint32_t* t6 = T + 6 * vi;
          t6[0] = q0;
          t6[1] = q1;
          t6[2] = q2;
          t6[3] = q0;
          t6[4] = q2;
          t6[5] = q3;
        }
      }
    });
  for (auto& x : th) x.join();
  return J3DG_OK;
}

extern "C" int j3dg_synth_cameras(uint32_t n, uint64_t seed, float r0, float r1, const float* target, float* cs) {
  if (!cs || !target) return J3DG_ERR_INVALID_ARGUMENT;
  // draws per camera: direction (rejection), radius ~ U(r0, r1)
  Pcg32 rng(seed);
  for (uint32_t c = 0; c < n; ++c) {
    double d[3];
    rng.unit3(d);
    double rad = rng.uniform((double)r0, (double)r1);
    double up0[3] = {0.0, 1.0, 0.0};
    if (std::fabs(d[1]) > 0.99) {
      up0[1] = 0.0;
      up0[2] = 1.0;
    }
    // right = normalize(up0 x back), up = back x right, back = d
    double rt[3] = {up0[1] * d[2] - up0[2] * d[1], up0[2] * d[0] - up0[0] * d[2], up0[0] * d[1] - up0[1] * d[0]};
    double rn = std::sqrt(rt[0] * rt[0] + rt[1] * rt[1] + rt[2] * rt[2]);
    for (double& x : rt) x /= rn;
    double up[3] = {d[1] * rt[2] - d[2] * rt[1], d[2] * rt[0] - d[0] * rt[2], d[0] * rt[1] - d[1] * rt[0]};
    float* M = cs + 16 * (size_t)c;
    for (int k = 0; k < 3; ++k) {
      M[k] = (float)rt[k];
      M[4 + k] = (float)up[k];
      M[8 + k] = (float)d[k];
      M[12 + k] = (float)((double)target[k] + rad * d[k]);
    }
    M[3] = M[7] = M[11] = 0.f;
    M[15] = 1.f;
  }
  return J3DG_OK;
}
