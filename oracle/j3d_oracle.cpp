/*
 * j3d_oracle.cpp -- CPU oracle for j3d's ray-cast hot path.
 *
 * TEST INFRASTRUCTURE ONLY. Imported by tests/, __graft_entry__.smoke() and
 * bench.py's CPU-baseline leg, always as the checker. Never linked by the
 * product library.
 *
 * Parity: "parity unpinned". The reference's BVH and ray/triangle code
 * (jtk/qbvh.h, jtk/geometry.h, jtk/vec.h) is an absent, un-pinned git
 * submodule (reference .gitmodules:1-3), and the reference has no tests. The
 * parts of the hot path that the reference tree holds are restated here line
 * by line with file:line citations; the jtk parts follow named published
 * methods with their fp32 operation order fixed here:
 *
 *   mat x vec       r_i = ((m[i]*x + m[4+i]*y) + m[8+i]*z) + m[12+i]*w
 *                   (float4x4 column-major, translation in [12..14] as in
 *                   scene.cpp:105-108)
 *   dot3            (a.x*b.x + a.y*b.y) + a.z*b.z ; dot4 adds + a.w*b.w last
 *   cross           (a.y*b.z - a.z*b.y, a.z*b.x - a.x*b.z, a.x*b.y - a.y*b.x)
 *   normalize       v / sqrt(dot3(v, v)) per component (zero vector kept)
 *   triangle test   Moller-Trumbore 1997, double sided, accept iff
 *                   det != 0, u >= 0, v >= 0, u + v <= 1, t > t_near and the
 *                   bounds gate below; closest hit = smallest (t, instance,
 *                   triangle id), strictly t < t_far.
 *   bounds gate     the hit t must lie inside the ray's slab interval of the
 *                   triangle's own AABB (same slab formula as the BVH nodes).
 *                   Node boxes contain their triangles' boxes exactly and the
 *                   slab formula is monotone in the box planes, so no BVH
 *                   whatever its shape can cull an accepted triangle: results
 *                   are independent of the BVH topology, which is what lets
 *                   the GPU build a different tree and still match bit for bit.
 *   slab            per ray: d' = d with |d_i| < 1e-12 replaced by
 *                   copysign(1e-12, d_i); inv_i = 1/d'_i;
 *                   pad = (max|o_i| + mesh_scale) * 2^-19;
 *                   near/far origin o_i -/+ pad chosen by sign(inv_i);
 *                   t_plane = fmaf(plane, inv_i, -(o_shifted_i) * inv_i);
 *                   t_enter = max over axes, t_exit = min over axes (fmaxf/fminf).
 *   BVH             4-wide binned SAH (Wald 2007 binning, Dammertz et al. 2008
 *                   QBVH layout), leaf <= leaf_max triangles.
 *
 * Compile with -ffp-contract=off and without -ffast-math: the restatement
 * relies on every fp32 operation being rounded where it is written.
 */
#include "j3d_oracle.h"

#include <algorithm>
#include <atomic>
#include <cfloat>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <limits>
#include <mutex>
#include <thread>
#include <vector>

namespace {

// ---------------------------------------------------------------- math ----

struct f3 {
  float x, y, z;
};

inline f3 sub3(f3 a, f3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline float dot3(f3 a, f3 b) {
  float s = a.x * b.x;
  s = s + a.y * b.y;
  s = s + a.z * b.z;
  return s;
}
inline f3 cross3(f3 a, f3 b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
inline f3 load3(const float* p) { return {p[0], p[1], p[2]}; }

// jtk matrix_vector_multiply (column-major), fixed order.
inline void mat_vec(const float* m, const float* v, float* r) {
  float out[4];
  for (int i = 0; i < 4; ++i) {
    float s = m[i] * v[0];
    s = s + m[4 + i] * v[1];
    s = s + m[8 + i] * v[2];
    s = s + m[12 + i] * v[3];
    out[i] = s;
  }
  r[0] = out[0];
  r[1] = out[1];
  r[2] = out[2];
  r[3] = out[3];
}

inline float dot4(const float* a, const float* b) {
  float s = a[0] * b[0];
  s = s + a[1] * b[1];
  s = s + a[2] * b[2];
  s = s + a[3] * b[3];
  return s;
}

// ------------------------------------------------------ ray preparation ----

struct RayPre {
  f3 o, d;
  float inv[3];
  float nn[3], nf[3];
  int neg[3];
  float t_near;
};

inline RayPre prep_ray(f3 o, f3 d, float t_near, float mesh_scale) {
  RayPre r;
  r.o = o;
  r.d = d;
  r.t_near = t_near;
  float mo = std::max(std::max(std::fabs(o.x), std::fabs(o.y)), std::fabs(o.z));
  float pad = (mo + mesh_scale) * 0x1p-19f;
  const float oc[3] = {o.x, o.y, o.z};
  const float dc[3] = {d.x, d.y, d.z};
  for (int i = 0; i < 3; ++i) {
    float di = dc[i];
    if (std::fabs(di) < 1e-12f) di = std::copysign(1e-12f, di);
    float inv = 1.f / di;
    r.inv[i] = inv;
    r.neg[i] = inv < 0.f;
    float on = r.neg[i] ? oc[i] - pad : oc[i] + pad;
    float of = r.neg[i] ? oc[i] + pad : oc[i] - pad;
    r.nn[i] = (-on) * inv;
    r.nf[i] = (-of) * inv;
  }
  return r;
}

// Slab interval of the box [lo, hi] for the prepared ray.
inline void slab(const RayPre& r, const float lo[3], const float hi[3], float& tn, float& tf) {
  float a[3], b[3];
  for (int i = 0; i < 3; ++i) {
    float pn = r.neg[i] ? hi[i] : lo[i];
    float pf = r.neg[i] ? lo[i] : hi[i];
    a[i] = std::fmaf(pn, r.inv[i], r.nn[i]);
    b[i] = std::fmaf(pf, r.inv[i], r.nf[i]);
  }
  tn = std::fmax(std::fmax(a[0], a[1]), a[2]);
  tf = std::fmin(std::fmin(b[0], b[1]), b[2]);
}

// Moller-Trumbore + bounds gate. Returns true iff the triangle is accepted.
inline bool tri_test(const RayPre& r, f3 v0, f3 v1, f3 v2, float& t, float& u, float& v) {
  f3 e1 = sub3(v1, v0);
  f3 e2 = sub3(v2, v0);
  f3 p = cross3(r.d, e2);
  float det = dot3(e1, p);
  if (det == 0.f) return false;
  float inv = 1.f / det;
  f3 s = sub3(r.o, v0);
  u = dot3(s, p) * inv;
  f3 q = cross3(s, e1);
  v = dot3(r.d, q) * inv;
  t = dot3(e2, q) * inv;
  if (!(u >= 0.f && v >= 0.f && u + v <= 1.f)) return false;
  if (!(t > r.t_near)) return false;
  float lo[3] = {std::fmin(std::fmin(v0.x, v1.x), v2.x), std::fmin(std::fmin(v0.y, v1.y), v2.y),
                 std::fmin(std::fmin(v0.z, v1.z), v2.z)};
  float hi[3] = {std::fmax(std::fmax(v0.x, v1.x), v2.x), std::fmax(std::fmax(v0.y, v1.y), v2.y),
                 std::fmax(std::fmax(v0.z, v1.z), v2.z)};
  float tn, tf;
  slab(r, lo, hi, tn, tf);
  return tn <= t && t <= tf;
}

// ------------------------------------------------------------------ BVH ----

struct Node4 {
  float lo[3][4];
  float hi[3][4];
  int32_t child[4];   // >= 0 node index (count == 0) or first prim (count > 0); -1 empty
  uint32_t count[4];  // leaf triangle count, 0 for an inner child
};

struct Box {
  float lo[3], hi[3];
  void empty() {
    for (int i = 0; i < 3; ++i) {
      lo[i] = FLT_MAX;
      hi[i] = -FLT_MAX;
    }
  }
  void grow(const Box& b) {
    for (int i = 0; i < 3; ++i) {
      lo[i] = std::fmin(lo[i], b.lo[i]);
      hi[i] = std::fmax(hi[i], b.hi[i]);
    }
  }
  void grow(const float* p) {
    for (int i = 0; i < 3; ++i) {
      lo[i] = std::fmin(lo[i], p[i]);
      hi[i] = std::fmax(hi[i], p[i]);
    }
  }
  float area() const {
    float dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
    if (dx < 0.f) return 0.f;
    return dx * dy + dy * dz + dz * dx;
  }
};

}  // namespace

struct orc_mesh {
  const float* vertices = nullptr;
  const uint32_t* tris = nullptr;
  uint32_t nv = 0, nt = 0;
  std::vector<float> normals;
  float min_bb[3] = {0, 0, 0}, max_bb[3] = {0, 0, 0};
  float scale = 0.f;
  std::vector<Node4> nodes;
  std::vector<uint32_t> prims;
  uint32_t max_depth = 0;
  bool has_root_leaf = false;  // tiny mesh: the root is a single leaf
  const float* colors = nullptr;
  const float* uv = nullptr;
  const uint32_t* tex = nullptr;
  uint32_t tex_w = 0, tex_h = 0;
};

namespace {

struct Builder {
  const std::vector<Box>* boxes;
  const std::vector<float>* cent;  // 3 per prim
  std::vector<uint32_t>* prims;
  Node4* nodes;
  std::atomic<uint32_t> n_nodes{0};
  std::atomic<uint32_t> max_depth{0};
  std::atomic<int> free_threads{0};
  uint32_t leaf_max = 4;

  // Splits [b, e) into two by binned SAH on centroids; returns the split point.
  uint32_t split(uint32_t b, uint32_t e) {
    uint32_t* P = prims->data();
    const float* C = cent->data();
    float cmin[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, cmax[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    for (uint32_t i = b; i < e; ++i) {
      const float* c = C + 3 * (size_t)P[i];
      for (int k = 0; k < 3; ++k) {
        cmin[k] = std::fmin(cmin[k], c[k]);
        cmax[k] = std::fmax(cmax[k], c[k]);
      }
    }
    int axis = 0;
    float ext[3] = {cmax[0] - cmin[0], cmax[1] - cmin[1], cmax[2] - cmin[2]};
    if (ext[1] > ext[axis]) axis = 1;
    if (ext[2] > ext[axis]) axis = 2;
    uint32_t mid = b + (e - b) / 2;
    if (!(ext[axis] > 0.f)) return mid;
    const int NB = 16;
    Box bb[NB];
    uint32_t cnt[NB] = {0};
    for (int k = 0; k < NB; ++k) bb[k].empty();
    const float kscale = (float)NB / ext[axis];
    for (uint32_t i = b; i < e; ++i) {
      float c = C[3 * (size_t)P[i] + axis];
      int bin = (int)((c - cmin[axis]) * kscale);
      if (bin < 0) bin = 0;
      if (bin > NB - 1) bin = NB - 1;
      cnt[bin]++;
      bb[bin].grow((*boxes)[P[i]]);
    }
    float right_area[NB];
    uint32_t right_cnt[NB];
    Box acc;
    acc.empty();
    uint32_t c = 0;
    for (int k = NB - 1; k > 0; --k) {
      acc.grow(bb[k]);
      c += cnt[k];
      right_area[k] = acc.area();
      right_cnt[k] = c;
    }
    acc.empty();
    c = 0;
    float best = FLT_MAX;
    int best_k = -1;
    for (int k = 1; k < NB; ++k) {
      acc.grow(bb[k - 1]);
      c += cnt[k - 1];
      if (c == 0 || right_cnt[k] == 0) continue;
      float cost = acc.area() * (float)c + right_area[k] * (float)right_cnt[k];
      if (cost < best) {
        best = cost;
        best_k = k;
      }
    }
    if (best_k < 0) return mid;
    uint32_t* it = std::partition(P + b, P + e, [&](uint32_t p) {
      int bin = (int)((C[3 * (size_t)p + axis] - cmin[axis]) * kscale);
      if (bin < 0) bin = 0;
      if (bin > NB - 1) bin = NB - 1;
      return bin < best_k;
    });
    uint32_t m = (uint32_t)(it - P);
    if (m == b || m == e) return mid;
    return m;
  }

  Box range_box(uint32_t b, uint32_t e) {
    Box r;
    r.empty();
    const uint32_t* P = prims->data();
    for (uint32_t i = b; i < e; ++i) r.grow((*boxes)[P[i]]);
    return r;
  }

  void build_node(uint32_t node, uint32_t b, uint32_t e, uint32_t depth) {
    uint32_t d = max_depth.load();
    while (depth > d && !max_depth.compare_exchange_weak(d, depth)) {
    }
    // Up to four ranges: split once, then split each half again.
    uint32_t rb[4], re[4];
    int n = 0;
    uint32_t m = split(b, e);
    uint32_t halves[2][2] = {{b, m}, {m, e}};
    for (int h = 0; h < 2; ++h) {
      uint32_t hb = halves[h][0], he = halves[h][1];
      if (he - hb > leaf_max) {
        uint32_t mm = split(hb, he);
        rb[n] = hb;
        re[n] = mm;
        ++n;
        rb[n] = mm;
        re[n] = he;
        ++n;
      } else {
        rb[n] = hb;
        re[n] = he;
        ++n;
      }
    }
    Node4& N = nodes[node];
    std::thread workers[4];
    bool spawned[4] = {false, false, false, false};
    for (int k = 0; k < 4; ++k) {
      if (k >= n) {
        for (int a = 0; a < 3; ++a) {
          N.lo[a][k] = FLT_MAX;
          N.hi[a][k] = -FLT_MAX;
        }
        N.child[k] = -1;
        N.count[k] = 0;
        continue;
      }
      Box bx = range_box(rb[k], re[k]);
      for (int a = 0; a < 3; ++a) {
        N.lo[a][k] = bx.lo[a];
        N.hi[a][k] = bx.hi[a];
      }
      uint32_t cnt = re[k] - rb[k];
      if (cnt <= leaf_max) {
        N.child[k] = (int32_t)rb[k];
        N.count[k] = cnt;
      } else {
        uint32_t c = n_nodes.fetch_add(1);
        N.child[k] = (int32_t)c;
        N.count[k] = 0;
        uint32_t cb = rb[k], ce = re[k];
        if (cnt > 50000 && free_threads.fetch_sub(1) > 0) {
          spawned[k] = true;
          workers[k] = std::thread([this, c, cb, ce, depth] {
            build_node(c, cb, ce, depth + 1);
            free_threads.fetch_add(1);
          });
        } else {
          if (cnt > 50000) free_threads.fetch_add(1);
          build_node(c, cb, ce, depth + 1);
        }
      }
    }
    for (int k = 0; k < 4; ++k)
      if (spawned[k]) workers[k].join();
  }
};

// Closest-hit / any-hit state shared across the instances of one ray.
struct HitState {
  float t_best;
  uint64_t key_best;  // (instance << 32) | triangle, 0 = none yet
  bool found;
  float u, v;
  uint32_t tri, inst;
};

inline bool better(float t, uint64_t key, const HitState& h) {
  return t < h.t_best || (t == h.t_best && key < h.key_best);
}

inline void leaf_test(const orc_mesh& m, const RayPre& r, uint32_t first, uint32_t count,
                      uint32_t inst, HitState& hs, bool any_hit, uint64_t& tri_tests) {
  for (uint32_t k = 0; k < count; ++k) {
    uint32_t id = m.prims[first + k];
    const uint32_t* T = m.tris + 3 * (size_t)id;
    f3 v0 = load3(m.vertices + 3 * (size_t)T[0]);
    f3 v1 = load3(m.vertices + 3 * (size_t)T[1]);
    f3 v2 = load3(m.vertices + 3 * (size_t)T[2]);
    float t, u, v;
    ++tri_tests;
    if (!tri_test(r, v0, v1, v2, t, u, v)) continue;
    uint64_t key = ((uint64_t)inst << 32) | id;
    if (better(t, key, hs)) {
      hs.t_best = t;
      hs.key_best = key;
      hs.found = true;
      hs.u = u;
      hs.v = v;
      hs.tri = id;
      hs.inst = inst;
      if (any_hit) return;
    }
  }
}

// BVH traversal of one instance with an object-space ray.
void traverse(const orc_mesh& m, const RayPre& r, uint32_t inst, HitState& hs, bool any_hit,
              uint64_t& node_visits, uint64_t& tri_tests) {
  if (m.nt == 0) return;
  if (m.has_root_leaf) {
    leaf_test(m, r, 0, m.nt, inst, hs, any_hit, tri_tests);
    return;
  }
  struct Entry {
    uint32_t node;
    float t;
  };
  Entry stack[256];
  int sp = 0;
  stack[sp++] = {0u, -FLT_MAX};
  while (sp > 0) {
    Entry e = stack[--sp];
    if (e.t > hs.t_best) continue;
    const Node4& N = m.nodes[e.node];
    ++node_visits;
    float tin[4];
    int order[4];
    int ninner = 0;
    for (int k = 0; k < 4; ++k) {
      if (N.child[k] < 0) continue;
      float lo[3] = {N.lo[0][k], N.lo[1][k], N.lo[2][k]};
      float hi[3] = {N.hi[0][k], N.hi[1][k], N.hi[2][k]};
      float tn, tf;
      slab(r, lo, hi, tn, tf);
      float a = std::fmax(tn, r.t_near);
      float b = std::fmin(tf, hs.t_best);
      if (!(a <= b)) continue;
      if (N.count[k] > 0) {
        leaf_test(m, r, (uint32_t)N.child[k], N.count[k], inst, hs, any_hit, tri_tests);
        if (any_hit && hs.found) return;
      } else {
        tin[ninner] = a;
        order[ninner] = k;
        ++ninner;
      }
    }
    // push far-to-near so that the nearest child is popped first
    for (int i = 0; i < ninner; ++i)
      for (int j = i + 1; j < ninner; ++j)
        if (tin[j] > tin[i]) {
          std::swap(tin[i], tin[j]);
          std::swap(order[i], order[j]);
        }
    if (sp + ninner > 256) std::abort();  // binned-SAH trees stay far below this depth
    for (int i = 0; i < ninner; ++i) stack[sp++] = {(uint32_t)N.child[order[i]], tin[i]};
  }
}

void brute(const orc_mesh& m, const RayPre& r, uint32_t inst, HitState& hs, bool any_hit,
           uint64_t& tri_tests) {
  for (uint32_t id = 0; id < m.nt; ++id) {
    const uint32_t* T = m.tris + 3 * (size_t)id;
    f3 v0 = load3(m.vertices + 3 * (size_t)T[0]);
    f3 v1 = load3(m.vertices + 3 * (size_t)T[1]);
    f3 v2 = load3(m.vertices + 3 * (size_t)T[2]);
    float t, u, v;
    ++tri_tests;
    if (!tri_test(r, v0, v1, v2, t, u, v)) continue;
    uint64_t key = ((uint64_t)inst << 32) | id;
    if (better(t, key, hs)) {
      hs.t_best = t;
      hs.key_best = key;
      hs.found = true;
      hs.u = u;
      hs.v = v;
      hs.tri = id;
      hs.inst = inst;
      if (any_hit) return;
    }
  }
}

struct Scene2 {
  const orc_instance* inst;
  uint32_t n;
  std::vector<float> inv;  // 16 per instance: invert_orthonormal(obj.cs), canvas.cpp:734
};

void invert_orthonormal(const float* m, float* o) {
  o[0] = m[0];
  o[1] = m[4];
  o[2] = m[8];
  o[3] = 0.f;
  o[4] = m[1];
  o[5] = m[5];
  o[6] = m[9];
  o[7] = 0.f;
  o[8] = m[2];
  o[9] = m[6];
  o[10] = m[10];
  o[11] = 0.f;
  float t0 = m[0] * m[12];
  t0 = t0 + m[1] * m[13];
  t0 = t0 + m[2] * m[14];
  float t1 = m[4] * m[12];
  t1 = t1 + m[5] * m[13];
  t1 = t1 + m[6] * m[14];
  float t2 = m[8] * m[12];
  t2 = t2 + m[9] * m[13];
  t2 = t2 + m[10] * m[14];
  o[12] = -t0;
  o[13] = -t1;
  o[14] = -t2;
  o[15] = 1.f;
}

Scene2 make_scene(const orc_instance* inst, uint32_t n) {
  Scene2 s;
  s.inst = inst;
  s.n = n;
  s.inv.resize(16 * (size_t)n);
  for (uint32_t i = 0; i < n; ++i) invert_orthonormal(inst[i].cs, &s.inv[16 * (size_t)i]);
  return s;
}

// qbvh_two_level_with_transformations::find_closest_triangle restated: the
// world ray is taken to each object's space (origin as a point, direction as
// a vector) and the closest accepted (t, instance, triangle) wins.
HitState find_closest(const Scene2& s, const float* orig, const float* dir, float t_near, float t_far,
                      bool any_hit, int mode, uint64_t& nv, uint64_t& nt) {
  HitState hs;
  hs.t_best = t_far;
  hs.key_best = 0;
  hs.found = false;
  hs.u = hs.v = 0.f;
  hs.tri = hs.inst = 0;
  for (uint32_t i = 0; i < s.n; ++i) {
    const orc_mesh& m = *s.inst[i].mesh;
    const float* M = &s.inv[16 * (size_t)i];
    float o4[4] = {orig[0], orig[1], orig[2], 1.f};
    float d4[4] = {dir[0], dir[1], dir[2], 0.f};
    float oo[4], dd[4];
    mat_vec(M, o4, oo);
    mat_vec(M, d4, dd);
    RayPre r = prep_ray({oo[0], oo[1], oo[2]}, {dd[0], dd[1], dd[2]}, t_near, m.scale);
    if (mode == 1)
      brute(m, r, i, hs, any_hit, nt);
    else
      traverse(m, r, i, hs, any_hit, nv, nt);
    if (any_hit && hs.found) break;
  }
  return hs;
}

// Row pool in the manner of pooled_parallel_for over jtk's thread_pool
// (canvas.cpp:765, canvas.h:100): the workers start once, on first use, and
// sleep between jobs; a job hands out items [y0, y1) one at a time through an
// atomic counter, and the calling thread works on it too (slot 0). No thread
// is created per call, so a frame's timing holds only the work.
class RowPool {
 public:
  static RowPool& get() {
    static RowPool* p = new RowPool();  // never destroyed: workers sleep until exit
    return *p;
  }
  int capacity() const { return (int)workers_.size() + 1; }

  void run(uint32_t y0, uint32_t y1, int n_threads, const std::function<void(uint32_t, int)>& f) {
    std::lock_guard<std::mutex> job(job_mu_);
    const int helpers = std::min(n_threads, capacity()) - 1;
    {
      std::lock_guard<std::mutex> lk(mu_);
      fn_ = &f;
      next_.store(y0);
      end_ = y1;
      want_ = helpers;
      pending_ = helpers;
      ++generation_;
    }
    cv_.notify_all();
    drain(0);
    std::unique_lock<std::mutex> lk(mu_);
    done_cv_.wait(lk, [&] { return pending_ == 0; });
    fn_ = nullptr;
  }

 private:
  RowPool() {
    unsigned n = std::max(1u, std::thread::hardware_concurrency());
    for (unsigned k = 1; k < n; ++k) workers_.emplace_back([this, k] { loop((int)k); });
    for (auto& t : workers_) t.detach();
  }
  void drain(int slot) {
    for (;;) {
      uint32_t y = next_.fetch_add(1);
      if (y >= end_) break;
      (*fn_)(y, slot);
    }
  }
  void loop(int slot) {
    uint64_t seen = 0;
    for (;;) {
      {
        std::unique_lock<std::mutex> lk(mu_);
        cv_.wait(lk, [&] { return generation_ != seen; });
        seen = generation_;
        if (slot > want_) continue;  // not part of this job
      }
      drain(slot);
      std::lock_guard<std::mutex> lk(mu_);
      if (--pending_ == 0) done_cv_.notify_all();
    }
  }
  std::vector<std::thread> workers_;
  std::mutex job_mu_, mu_;
  std::condition_variable cv_, done_cv_;
  const std::function<void(uint32_t, int)>* fn_ = nullptr;
  std::atomic<uint32_t> next_{0};
  uint32_t end_ = 0;
  int want_ = 0, pending_ = 0;
  uint64_t generation_ = 0;
};

template <class F>
void parallel_rows(uint32_t y0, uint32_t y1, int n_threads, F&& f) {
  if (n_threads <= 1 || y1 - y0 < 2) {
    for (uint32_t y = y0; y < y1; ++y) f(y, 0);
    return;
  }
  const std::function<void(uint32_t, int)> fn = [&](uint32_t y, int t) { f(y, t); };
  RowPool::get().run(y0, y1, n_threads, fn);
}

inline uint32_t make_color(uint32_t r, uint32_t g, uint32_t b) {
  return 0xff000000u | (b << 16) | (g << 8) | r;
}

// canvas.cpp:320-328 with out-of-range indices clamped to the texture.
inline uint32_t tex_index(float f, uint32_t size) {
  if (!(f >= 0.f)) f = 0.f;
  float mx = (float)(size - 1);
  if (f > mx) f = mx;
  return (uint32_t)f;
}
inline uint32_t get_U(float u, uint32_t W) {
  return tex_index(std::floor(0.5f + (u + 1.f) * (float)(W - 1) * 0.5f), W);
}
inline uint32_t get_V(float v, uint32_t H) {
  return tex_index(std::floor(0.5f + (-v + 1.f) * (float)(H - 1) * 0.5f), H);
}

// canvas.cpp:330-344
inline uint32_t get_color(const uint32_t* mc, uint32_t mw, uint32_t U, uint32_t V, uint32_t shadow) {
  uint32_t clr = mc[(size_t)V * mw + U];
  if (shadow) {
    uint32_t r = clr & 0xffu, g = (clr >> 8) & 0xffu, b = (clr >> 16) & 0xffu;
    clr = 0xff000000u | ((b >> 2) << 16) | ((g >> 2) << 8) | (r >> 2);
  }
  return clr;
}

// canvas.cpp:346-389
inline uint32_t get_angle_color(float angle, const uint32_t* mc, uint32_t mw, uint32_t mh, uint32_t cavity,
                                float u, float v, uint32_t mark) {
  uint32_t U = get_U(u, mw), V = get_V(v, mh);
  uint32_t clr = get_color(mc, mw, U, V, mark);
  if (std::fabs(angle) <= 1.f) {
    uint32_t r = clr & 0xffu, g = (clr >> 8) & 0xffu, b = (clr >> 16) & 0xffu;
    const float hp = 1.57079632679489f;
    float scale = (hp - std::fabs(std::acos(angle) - hp)) / hp;
    scale = std::sqrt(1.f - scale);
    uint32_t r2 = cavity & 0xffu, g2 = (cavity >> 8) & 0xffu, b2 = (cavity >> 16) & 0xffu;
    float f = angle > 0.f ? 1.2f : 0.5f;
    r = (uint32_t)((float)r * (1.f - scale) + (float)r2 * scale * f);
    g = (uint32_t)((float)g * (1.f - scale) + (float)g2 * scale * f);
    b = (uint32_t)((float)b * (1.f - scale) + (float)b2 * scale * f);
    if (r > 255) r = 255;
    if (g > 255) g = 255;
    if (b > 255) b = 255;
    clr = make_color(r, g, b);
  }
  return clr;
}

// canvas.cpp:402-441 (_get_color)
inline uint32_t get_pixel_color(const orc_pixel* p, const orc_settings& st, const uint32_t* mc, uint32_t mw,
                                uint32_t mh, float u, float v) {
  if (p->mark & 2) {
    if (st.shading) {
      float nz = std::sqrt(1.f - u * u - v * v);
      float nor[4] = {u, v, nz, 0.f};
      float lig[4] = {0.f, 0.f, 1.f, 0.f};
      float occ = (p->mark & 1) ? 0.3f : 1.f;
      float d = dot4(nor, lig);
      d = d < 0.f ? 0.f : (d > 1.f ? 1.f : d);
      float dif = d * occ;
      return 0xff000000u | ((uint32_t)((float)p->b * dif) << 16) | ((uint32_t)((float)p->g * dif) << 8) |
             (uint32_t)((float)p->r * dif);
    }
    if (p->mark & 1)
      return 0xff000000u | ((uint32_t)(p->b >> 2) << 16) | ((uint32_t)(p->g >> 2) << 8) | (uint32_t)(p->r >> 2);
    return 0xff000000u | ((uint32_t)p->b << 16) | ((uint32_t)p->g << 8) | (uint32_t)p->r;
  }
  return get_color(mc, mw, get_U(u, mw), get_V(v, mh), p->mark);
}

// canvas.cpp:287-315
float convex_cos_angle(const orc_view& view, uint32_t W, uint32_t H, float x1, float y1, float u1, float v1,
                       float depth1, float x2, float y2, float u2, float v2, float depth2) {
  float s1[4] = {2.f * ((x1 + 0.5f) / (float)W) - 1.f, 2.f * ((y1 + 0.5f) / (float)H) - 1.f,
                 view.near_clipping_plane, 1.f};
  float d1[4];
  mat_vec(view.projection_inv, s1, d1);
  d1[3] = 0.f;
  float p1[4] = {depth1 * d1[0], depth1 * d1[1], depth1 * d1[2], depth1 * d1[3]};
  float s2[4] = {2.f * ((x2 + 0.5f) / (float)W) - 1.f, 2.f * ((y2 + 0.5f) / (float)H) - 1.f,
                 view.near_clipping_plane, 1.f};
  float d2[4];
  mat_vec(view.projection_inv, s2, d2);
  d2[3] = 0.f;
  float p2[4] = {depth2 * d2[0], depth2 * d2[1], depth2 * d2[2], depth2 * d2[3]};
  float n1[4] = {u1, v1, std::sqrt(1.f - u1 * u1 - v1 * v1), 0.f};
  float n2[4] = {u2, v2, std::sqrt(1.f - u2 * u2 - v2 * v2), 0.f};
  float angle;
  if ((double)std::fabs(dot4(n1, n2) - 1.f) > 0.0001) {
    float pt[4] = {p2[0] - p1[0], p2[1] - p1[1], p2[2] - p1[2], p2[3] - p1[3]};
    float len = std::sqrt(dot4(pt, pt));
    for (int i = 0; i < 4; ++i) pt[i] = pt[i] / len;
    angle = dot4(pt, n1);
  } else {
    angle = 0.f;
  }
  return angle;
}

inline bool differs(const orc_pixel* a, const orc_pixel* b) {
  const float threshold = 0.001f;
  return b->object_id != 0xffffffffu && (std::fabs(a->u - b->u) > threshold || std::fabs(a->v - b->v) > threshold);
}

}  // namespace

extern "C" {

// camera.cpp:5-16
void orc_make_default_camera(orc_camera* c) {
  c->focal_length = 35.f;
  c->film_aperture_width_inch = 1.024f;
  c->film_aperture_height_inch = 0.768f;
  c->near_clipping_plane = 0.1f;
  c->far_clipping_plane = std::numeric_limits<float>::max();
  c->fit_film = 1;
  c->zoom = 1.f;
}

// camera.cpp:18-24
void orc_frustum(float left, float right, float bottom, float top, float n, float f, float* out) {
  float m[16] = {2.f * n / (right - left),
                 0.f,
                 0.f,
                 0.f,
                 0.f,
                 -2.f * n / (top - bottom),
                 0.f,
                 0.f,
                 (right + left) / (right - left),
                 -(top + bottom) / (top - bottom),
                 -(f + n) / (f - n),
                 -1.f,
                 0.f,
                 0.f,
                 -(2.f * f * n) / (f - n),
                 0.f};
  std::memcpy(out, m, sizeof(m));
}

// camera.cpp:26-30
void orc_invert_projection_matrix(const float* in, float* out) {
  float m[16] = {1.f / in[0], 0.f, 0.f, 0.f, 0.f, 1.f / in[5], 0.f, 0.f, 0.f, 0.f, 0.f, 1.f / in[14],
                 in[8] / in[0], in[9] / in[5], -1.f, in[10] / in[14]};
  std::memcpy(out, m, sizeof(m));
}

// camera.cpp:32-73
void orc_make_projection_matrix(const orc_camera* c, int screen_w, int screen_h, float* out) {
  const float inchToMm = 25.4f;
  float top = ((c->film_aperture_height_inch * inchToMm / 2.f) / c->focal_length) * c->near_clipping_plane;
  float right = ((c->film_aperture_width_inch * inchToMm / 2.f) / c->focal_length) * c->near_clipping_plane;
  float xscale = c->zoom;
  float yscale = c->zoom;
  float deviceAspectRatio = screen_w / (float)screen_h;
  float filmAspectRatio = c->film_aperture_width_inch / c->film_aperture_height_inch;
  if (c->fit_film == 1) {
    if (filmAspectRatio > deviceAspectRatio)
      yscale *= filmAspectRatio / deviceAspectRatio;
    else
      xscale *= deviceAspectRatio / filmAspectRatio;
  } else {
    if (filmAspectRatio > deviceAspectRatio)
      xscale *= deviceAspectRatio / filmAspectRatio;
    else
      yscale *= filmAspectRatio / deviceAspectRatio;
  }
  right *= xscale;
  top *= yscale;
  float bottom = -top;
  float left = -right;
  orc_frustum(left, right, bottom, top, c->near_clipping_plane, c->far_clipping_plane, out);
}

void orc_invert_orthonormal(const float* in, float* out) { invert_orthonormal(in, out); }

void orc_matrix_vector_multiply(const float* m, const float* v, float* out) { mat_vec(m, v, out); }

// mesh.cpp:39-58
void orc_compute_bb(const float* V, uint32_t nv, float* mn, float* mx) {
  if (nv == 0) return;
  for (int k = 0; k < 3; ++k) mn[k] = mx[k] = V[k];
  for (uint32_t i = 1; i < nv; ++i)
    for (int k = 0; k < 3; ++k) {
      mn[k] = std::min<float>(mn[k], V[3 * (size_t)i + k]);
      mx[k] = std::max<float>(mx[k], V[3 * (size_t)i + k]);
    }
}

// jtk transform(float4x4, vec3): the point (p, 1) through mat x vec.
static void transform_point(const float* m, const float* p, float* out) {
  float v[4] = {p[0], p[1], p[2], 1.f}, r[4];
  mat_vec(m, v, r);
  out[0] = r[0];
  out[1] = r[1];
  out[2] = r[2];
}

// scene.cpp:50-89 (mesh objects only; point clouds are not on this path)
void orc_prepare_scene(const float* omin, const float* omax, const float* ocs, uint32_t n, float* mn, float* mx,
                       float* diagonal) {
  if (n == 0) {
    for (int k = 0; k < 3; ++k) mn[k] = mx[k] = 0.f;
  } else {
    float a[3], b[3];
    transform_point(ocs, omin, a);
    transform_point(ocs, omax, b);
    for (int k = 0; k < 3; ++k) {
      mn[k] = std::min(a[k], b[k]);
      mx[k] = std::max(a[k], b[k]);
    }
  }
  for (uint32_t i = 0; i < n; ++i) {
    float a[3], b[3];
    transform_point(ocs + 16 * (size_t)i, omin + 3 * (size_t)i, a);
    transform_point(ocs + 16 * (size_t)i, omax + 3 * (size_t)i, b);
    for (int k = 0; k < 3; ++k) {
      mn[k] = std::min(mn[k], std::min(a[k], b[k]));
      mx[k] = std::max(mx[k], std::max(a[k], b[k]));
    }
  }
  float d = mx[0] - mn[0];
  d = std::max<float>(d, mx[1] - mn[1]);
  d = std::max<float>(d, mx[2] - mn[2]);
  *diagonal = d;
}

// scene.cpp:91-110 (the y-axis-up branch)
void orc_unzoom(const float* mn, const float* mx, float diagonal, float* cs, float* cs_inv, float* pivot) {
  for (int i = 0; i < 16; ++i) cs[i] = (i % 5 == 0) ? 1.f : 0.f;
  for (int j = 0; j < 3; ++j) pivot[j] = (mn[j] + mx[j]) * 0.5f;
  cs[12] = pivot[0];
  cs[13] = pivot[1];
  cs[14] = pivot[2] + diagonal * 2.f;
  invert_orthonormal(cs, cs_inv);
}

// jtk compute_triangle_normals (called at scene.cpp:20): normalize(cross(V1-V0, V2-V0))
void orc_compute_triangle_normals(const float* V, const uint32_t* T, uint32_t nt, float* N) {
  for (uint32_t i = 0; i < nt; ++i) {
    f3 v0 = load3(V + 3 * (size_t)T[3 * (size_t)i + 0]);
    f3 v1 = load3(V + 3 * (size_t)T[3 * (size_t)i + 1]);
    f3 v2 = load3(V + 3 * (size_t)T[3 * (size_t)i + 2]);
    f3 n = cross3(sub3(v1, v0), sub3(v2, v0));
    float len = std::sqrt(dot3(n, n));
    if (len > 0.f) n = {n.x / len, n.y / len, n.z / len};
    N[3 * (size_t)i + 0] = n.x;
    N[3 * (size_t)i + 1] = n.y;
    N[3 * (size_t)i + 2] = n.z;
  }
}

// scene.cpp:8-38 (add_object): normals, bbox, new qbvh(triangles, vertices)
orc_mesh* orc_mesh_build(const float* V, uint32_t nv, const uint32_t* T, uint32_t nt, uint32_t leaf_max,
                         int n_threads, double* build_seconds) {
  auto t0 = std::chrono::steady_clock::now();
  orc_mesh* m = new orc_mesh;
  m->vertices = V;
  m->tris = T;
  m->nv = nv;
  m->nt = nt;
  if (leaf_max < 1) leaf_max = 1;
  if (leaf_max > 16) leaf_max = 16;
  m->normals.resize(3 * (size_t)nt);
  if (n_threads < 1) n_threads = 1;
  // normals in parallel chunks
  {
    std::vector<std::thread> th;
    uint32_t chunk = (nt + n_threads - 1) / (uint32_t)n_threads;
    for (int t = 0; t < n_threads; ++t) {
      uint32_t b = (uint32_t)t * chunk, e = std::min(nt, b + chunk);
      if (b >= e) break;
      th.emplace_back([=] { orc_compute_triangle_normals(V, T + 3 * (size_t)b, e - b, m->normals.data() + 3 * (size_t)b); });
    }
    for (auto& x : th) x.join();
  }
  orc_compute_bb(V, nv, m->min_bb, m->max_bb);
  float sc = 0.f;
  for (int k = 0; k < 3; ++k) sc = std::fmax(sc, std::fmax(std::fabs(m->min_bb[k]), std::fabs(m->max_bb[k])));
  m->scale = sc;
  m->prims.resize(nt);
  for (uint32_t i = 0; i < nt; ++i) m->prims[i] = i;
  if (nt <= leaf_max) {
    m->has_root_leaf = true;
  } else {
    std::vector<Box> boxes(nt);
    std::vector<float> cent(3 * (size_t)nt);
    {
      std::vector<std::thread> th;
      uint32_t chunk = (nt + n_threads - 1) / (uint32_t)n_threads;
      for (int t = 0; t < n_threads; ++t) {
        uint32_t b = (uint32_t)t * chunk, e = std::min(nt, b + chunk);
        if (b >= e) break;
        th.emplace_back([&, b, e] {
          for (uint32_t i = b; i < e; ++i) {
            Box bx;
            bx.empty();
            for (int k = 0; k < 3; ++k) bx.grow(V + 3 * (size_t)T[3 * (size_t)i + k]);
            boxes[i] = bx;
            for (int a = 0; a < 3; ++a) cent[3 * (size_t)i + a] = (bx.lo[a] + bx.hi[a]) * 0.5f;
          }
        });
      }
      for (auto& x : th) x.join();
    }
    size_t cap = (size_t)nt + 1;
    Node4* nodes = (Node4*)std::malloc(cap * sizeof(Node4));
    Builder B;
    B.boxes = &boxes;
    B.cent = &cent;
    B.prims = &m->prims;
    B.nodes = nodes;
    B.leaf_max = leaf_max;
    B.n_nodes = 1;
    B.free_threads = n_threads - 1;
    B.build_node(0, 0, nt, 1);
    m->nodes.assign(nodes, nodes + B.n_nodes.load());
    std::free(nodes);
    m->max_depth = B.max_depth.load();
  }
  auto t1 = std::chrono::steady_clock::now();
  if (build_seconds) *build_seconds = std::chrono::duration<double>(t1 - t0).count();
  return m;
}

void orc_mesh_free(orc_mesh* m) { delete m; }
uint32_t orc_mesh_node_count(const orc_mesh* m) { return (uint32_t)m->nodes.size(); }
uint32_t orc_mesh_max_depth(const orc_mesh* m) { return m->max_depth; }
const float* orc_mesh_normals(const orc_mesh* m) { return m->normals.data(); }
void orc_mesh_set_vertex_colors(orc_mesh* m, const float* c) { m->colors = c; }
void orc_mesh_set_uv(orc_mesh* m, const float* uv) { m->uv = uv; }
void orc_mesh_set_texture(orc_mesh* m, const uint32_t* tex, uint32_t w, uint32_t h) {
  m->tex = tex;
  m->tex_w = w;
  m->tex_h = h;
}

void orc_find_closest(const orc_instance* inst, uint32_t n_inst, const orc_ray* rays, uint32_t n, orc_hit* hits,
                      int mode, int any_hit, int n_threads, orc_stats* stats) {
  Scene2 s = make_scene(inst, n_inst);
  const uint32_t chunk = 256;
  uint32_t nchunks = (n + chunk - 1) / chunk;
  int nt = std::max(1, n_threads);
  std::vector<uint64_t> nvis(nt, 0), ntri(nt, 0);
  parallel_rows(0, nchunks, nt, [&](uint32_t c, int t) {
    for (uint32_t i = c * chunk; i < std::min(n, (c + 1) * chunk); ++i) {
      const orc_ray& r = rays[i];
      HitState hs = find_closest(s, r.orig, r.dir, r.t_near, r.t_far, any_hit != 0, mode, nvis[t], ntri[t]);
      hits[i].found = hs.found ? 1u : 0u;
      hits[i].distance = hs.found ? hs.t_best : r.t_far;
      hits[i].u = hs.u;
      hits[i].v = hs.v;
      hits[i].object_id = hs.found ? hs.tri : 0xffffffffu;
      hits[i].two_level_index = hs.found ? hs.inst : 0xffffffffu;
    }
  });
  if (stats) {
    stats->rays += n;
    for (int t = 0; t < nt; ++t) {
      stats->node_visits += nvis[t];
      stats->tri_tests += ntri[t];
    }
  }
}

// All accepted triangles along the ray (t < t_far), through the BVH (any
// node whose slab interval meets [t_near, t_far]) or by brute force.
static void all_hits(const orc_mesh& m, const RayPre& r, float t_far, bool brute, std::vector<orc_hit>& out) {
  auto test = [&](uint32_t id) {
    const uint32_t* T = m.tris + 3 * (size_t)id;
    float t, u, v;
    if (!tri_test(r, load3(m.vertices + 3 * (size_t)T[0]), load3(m.vertices + 3 * (size_t)T[1]),
                  load3(m.vertices + 3 * (size_t)T[2]), t, u, v))
      return;
    if (!(t < t_far)) return;
    out.push_back({1u, t, u, v, id, 0u});
  };
  if (brute || m.has_root_leaf) {
    for (uint32_t id = 0; id < m.nt; ++id) test(id);
  } else {
    std::vector<uint32_t> stack{0u};
    while (!stack.empty()) {
      const Node4& N = m.nodes[stack.back()];
      stack.pop_back();
      for (int k = 0; k < 4; ++k) {
        if (N.child[k] < 0) continue;
        float lo[3] = {N.lo[0][k], N.lo[1][k], N.lo[2][k]};
        float hi[3] = {N.hi[0][k], N.hi[1][k], N.hi[2][k]};
        float tn, tf;
        slab(r, lo, hi, tn, tf);
        if (!(std::fmax(tn, r.t_near) <= std::fmin(tf, t_far))) continue;
        if (N.count[k] > 0) {
          for (uint32_t j = 0; j < N.count[k]; ++j) test(m.prims[(uint32_t)N.child[k] + j]);
        } else {
          stack.push_back((uint32_t)N.child[k]);
        }
      }
    }
  }
  std::sort(out.begin(), out.end(), [](const orc_hit& a, const orc_hit& b) {
    return a.distance < b.distance || (a.distance == b.distance && a.object_id < b.object_id);
  });
}

static uint32_t find_all_impl(const orc_mesh* m, const orc_ray* ray, orc_hit* hits, uint32_t cap, bool brute) {
  RayPre r = prep_ray({ray->orig[0], ray->orig[1], ray->orig[2]}, {ray->dir[0], ray->dir[1], ray->dir[2]},
                      ray->t_near, m->scale);
  std::vector<orc_hit> all;
  all_hits(*m, r, ray->t_far, brute, all);
  for (uint32_t i = 0; i < (uint32_t)all.size() && i < cap; ++i) hits[i] = all[i];
  return (uint32_t)all.size();
}

uint32_t orc_find_all(const orc_mesh* m, const orc_ray* ray, orc_hit* hits, uint32_t cap) {
  return find_all_impl(m, ray, hits, cap, false);
}

uint32_t orc_find_all_brute(const orc_mesh* m, const orc_ray* ray, orc_hit* hits, uint32_t cap) {
  return find_all_impl(m, ray, hits, cap, true);
}

// canvas.cpp:55-78
void orc_fill_background(uint32_t* bg, uint32_t w, uint32_t h, uint32_t clr_top, uint32_t clr_bottom) {
  uint32_t top_red = clr_top & 0xff, top_green = (clr_top >> 8) & 0xff, top_blue = (clr_top >> 16) & 0xff;
  uint32_t bottom_red = clr_bottom & 0xff, bottom_green = (clr_bottom >> 8) & 0xff,
           bottom_blue = (clr_bottom >> 16) & 0xff;
  for (uint32_t y = 0; y < h; ++y) {
    float scale = (float)y / (float)h;
    uint32_t red = (uint32_t)(scale * (float)bottom_red + (1.f - scale) * (float)top_red);
    uint32_t green = (uint32_t)(scale * (float)bottom_green + (1.f - scale) * (float)top_green);
    uint32_t blue = (uint32_t)(scale * (float)bottom_blue + (1.f - scale) * (float)top_blue);
    uint32_t clr = make_color((unsigned char)red, (unsigned char)green, (unsigned char)blue);
    for (uint32_t x = 0; x < w; ++x) bg[(size_t)y * w + x] = clr;
  }
}

// canvas.cpp:677-874 (update_canvas)
void orc_update_canvas(orc_pixel* out, uint32_t w, uint32_t h, int x0, int y0, int x1, int y1,
                       const orc_instance* inst, uint32_t n_inst, const orc_view* view, const orc_settings* st,
                       int n_threads, orc_stats* stats) {
  if (w == 0 || h == 0) return;
  if (x0 < 0) x0 = 0;
  if (y0 < 0) y0 = 0;
  if (x1 < 0) x1 = 0;
  if (y1 < 0) y1 = 0;
  if (x0 >= (int)w) x0 = w - 1;
  if (y0 >= (int)h) y0 = h - 1;
  if (x1 >= (int)w) x1 = w - 1;
  if (y1 >= (int)h) y1 = h - 1;
  const float* cs = view->coordinate_system;
  float o4[4] = {0.f, 0.f, 0.f, 1.f};
  float origin[4];
  mat_vec(cs, o4, origin);
  float l4[4] = {view->pivot[0] + view->diagonal * 3.f, view->pivot[1] + view->diagonal * 3.f,
                 view->pivot[2] + view->diagonal * 3.f, 1.f};
  float light[4];
  mat_vec(cs, l4, light);
  if (n_inst == 0) {
    for (int y = y0; y <= y1; ++y)
      for (int x = x0; x <= x1; ++x) {
        orc_pixel* p = out + (size_t)y * w + x;
        p->db_id = 0;
        p->object_id = 0xffffffffu;
        p->u = 0.f;
        p->v = 0.f;
        p->depth = std::numeric_limits<float>::max();
      }
    return;
  }
  Scene2 s = make_scene(inst, n_inst);
  int nt = std::max(1, n_threads);
  std::vector<uint64_t> nvis(nt, 0), ntri(nt, 0), nrays(nt, 0);
  parallel_rows((uint32_t)y0, (uint32_t)y1 + 1, nt, [&](uint32_t y, int t) {
    orc_pixel* p = out + (size_t)y * w + x0;
    for (int x = x0; x <= x1; ++x, ++p) {
      float sp[4] = {2.f * (((float)x + 0.5f) / (float)w) - 1.f, 2.f * (((float)y + 0.5f) / (float)h) - 1.f,
                     view->near_clipping_plane, 1.f};
      float dir[4];
      mat_vec(view->projection_inv, sp, dir);
      dir[3] = 0.f;
      mat_vec(cs, dir, dir);
      float t_near = view->diagonal / 100.f;
      ++nrays[t];
      HitState hs = find_closest(s, origin, dir, t_near, std::numeric_limits<float>::max(), false, 0, nvis[t], ntri[t]);
      if (hs.found) {
        const orc_mesh& m = *inst[hs.inst].mesh;
        const float* objcs = inst[hs.inst].cs;
        float n[4] = {m.normals[3 * (size_t)hs.tri], m.normals[3 * (size_t)hs.tri + 1],
                      m.normals[3 * (size_t)hs.tri + 2], 0.f};
        mat_vec(view->coordinate_system_inv, n, n);
        mat_vec(objcs, n, n);
        p->u = n[0];
        p->v = n[1];
        p->depth = hs.t_best;
        p->object_id = hs.tri;
        p->barycentric_u = hs.u;
        p->barycentric_v = hs.v;
        p->db_id = inst[hs.inst].db_id;
        p->mark = 0;
        const uint32_t* T = m.tris + 3 * (size_t)hs.tri;
        if (st->textured && m.uv != nullptr && m.tex != nullptr) {
          const float* uv = m.uv + 6 * (size_t)hs.tri;
          float wgt = 1.f - hs.u - hs.v;
          float c0 = wgt * uv[0] + hs.u * uv[2] + hs.v * uv[4];
          float c1 = wgt * uv[1] + hs.u * uv[3] + hs.v * uv[5];
          c0 = std::max(std::min(c0, 1.f), 0.f);
          c1 = std::max(std::min(c1, 1.f), 0.f);
          const int tw = (int)m.tex_w, th = (int)m.tex_h;
          int tx = (int)(c0 * (float)tw);
          int ty = (int)(c1 * (float)th);
          tx = tx < 0 ? 0 : tx >= tw ? tw - 1 : tx;
          ty = ty < 0 ? 0 : ty >= th ? th - 1 : ty;
          uint32_t color = m.tex[(size_t)ty * m.tex_w + tx];
          p->r = color & 0xff;
          p->g = (color >> 8) & 0xff;
          p->b = (color >> 16) & 0xff;
          p->mark |= 2;
        } else if (st->vertexcolors && m.colors != nullptr) {
          const float* c0 = m.colors + 3 * (size_t)T[0];
          const float* c1 = m.colors + 3 * (size_t)T[1];
          const float* c2 = m.colors + 3 * (size_t)T[2];
          float wgt = 1.f - hs.u - hs.v;
          float c[3];
          for (int k = 0; k < 3; ++k) c[k] = c0[k] * wgt + hs.u * c1[k] + hs.v * c2[k];
          p->r = (uint8_t)(c[0] * 255.f);
          p->g = (uint8_t)(c[1] * 255.f);
          p->b = (uint8_t)(c[2] * 255.f);
          p->mark |= 2;
        }
        if (st->shadow) {
          float V0[4] = {m.vertices[3 * (size_t)T[0]], m.vertices[3 * (size_t)T[0] + 1], m.vertices[3 * (size_t)T[0] + 2], 1.f};
          float V1[4] = {m.vertices[3 * (size_t)T[1]], m.vertices[3 * (size_t)T[1] + 1], m.vertices[3 * (size_t)T[1] + 2], 1.f};
          float V2[4] = {m.vertices[3 * (size_t)T[2]], m.vertices[3 * (size_t)T[2] + 1], m.vertices[3 * (size_t)T[2] + 2], 1.f};
          mat_vec(objcs, V0, V0);
          mat_vec(objcs, V1, V1);
          mat_vec(objcs, V2, V2);
          float wgt = 1.f - hs.u - hs.v;
          float pos[4], ld[4];
          for (int k = 0; k < 4; ++k) {
            pos[k] = V0[k] * wgt + hs.u * V1[k] + hs.v * V2[k];
            ld[k] = light[k] - pos[k];
          }
          ++nrays[t];
          HitState h2 = find_closest(s, pos, ld, 1e-3f, std::numeric_limits<float>::max(), true, 0, nvis[t], ntri[t]);
          if (h2.found) p->mark |= 1;
        }
      } else {
        p->db_id = 0;
        p->object_id = 0xffffffffu;
        p->u = 0.f;
        p->v = 0.f;
        p->depth = std::numeric_limits<float>::max();
      }
    }
  });
  if (stats)
    for (int t = 0; t < nt; ++t) {
      stats->rays += nrays[t];
      stats->node_visits += nvis[t];
      stats->tri_tests += ntri[t];
    }
}

// canvas.cpp:449-670 (canvas_to_image with its one-bit, wireframe, edges and plain modes)
void orc_canvas_to_image(const orc_pixel* pix, uint32_t w, uint32_t h, const orc_view* view, const orc_settings* st,
                         const uint32_t* mc, uint32_t mw, uint32_t mh, uint32_t cavity, uint32_t* im) {
  if (w == 0 || h == 0) return;
  const uint32_t NONE = 0xffffffffu;
  if (st->one_bit) {
    const uint32_t black = 0xff000000u, white = 0xffffffffu;
    for (uint32_t y = 0; y < h; ++y) {
      const orc_pixel* row = pix + (size_t)y * w;
      const orc_pixel* up = pix + (size_t)(y == 0 ? 0 : y - 1) * w;
      uint32_t* o = im + (size_t)y * w;
      for (uint32_t x = 0; x + 1 < w; ++x) {
        const orc_pixel* p = row + x;
        if (p->object_id == NONE) continue;
        float angle = 1.f;
        const orc_pixel* q = nullptr;
        if (differs(p, row + x + 1))
          q = row + x + 1;
        else if (differs(p, up + x))
          q = up + x;
        if (q) {
          float w1 = std::sqrt(1.f - p->u * p->u - p->v * p->v);
          float w2 = std::sqrt(1.f - q->u * q->u - q->v * q->v);
          angle = p->u * q->u + p->v * q->v + w1 * w2;
        }
        uint32_t clr = get_color(mc, mw, get_U(p->u, mw), get_V(p->v, mh), p->mark);
        int res = (int)((((clr & 0xff0000u) >> 16) + ((clr & 0xff00u) >> 8) + (clr & 0xffu)) >> 7);
        ++res;
        bool clr_black = ((x % (uint32_t)res == 0) && (y % (uint32_t)res == 0));
        if (std::fabs(angle) < 0.95f) clr_black = (res == 1) ? !clr_black : true;
        o[x] = clr_black ? black : white;
      }
      const orc_pixel* p = row + (w - 1);
      if (p->object_id != NONE) {
        uint32_t clr = get_color(mc, mw, get_U(p->u, mw), get_V(p->v, mh), p->mark);
        int res = (int)((((clr & 0xff0000u) >> 16) + ((clr & 0xff00u) >> 8) + (clr & 0xffu)) >> 7);
        ++res;
        o[w - 1] = (((w - 1) % (uint32_t)res == 0) && (y % (uint32_t)res == 0)) ? black : white;
      }
    }
    return;
  }
  if (st->wireframe) {
    for (uint32_t y = 0; y < h; ++y) {
      const orc_pixel* row = pix + (size_t)y * w;
      const orc_pixel* up = pix + (size_t)(y == 0 ? 0 : y - 1) * w;
      uint32_t* o = im + (size_t)y * w;
      for (uint32_t x = 0; x + 1 < w; ++x) {
        const orc_pixel* p = row + x;
        if (p->object_id == NONE) continue;
        const orc_pixel* r = row + x + 1;
        const orc_pixel* u = up + x;
        if ((r->object_id != NONE && r->object_id != p->object_id) ||
            (u->object_id != NONE && u->object_id != p->object_id)) {
          const float scale = (p->u * p->u + p->v * p->v) * 0.5f;
          uint32_t c = (unsigned char)(255.f * scale);
          o[x] = make_color(c, c, c);
        } else {
          o[x] = get_pixel_color(p, *st, mc, mw, mh, p->u, p->v);
        }
      }
      const orc_pixel* p = row + (w - 1);
      if (p->object_id != NONE) o[w - 1] = get_pixel_color(p, *st, mc, mw, mh, p->u, p->v);
    }
    return;
  }
  if (st->edges) {
    for (uint32_t y = 0; y < h; ++y) {
      const orc_pixel* row = pix + (size_t)y * w;
      const orc_pixel* up = pix + (size_t)(y == 0 ? 0 : y - 1) * w;
      uint32_t* o = im + (size_t)y * w;
      for (uint32_t x = 0; x + 1 < w; ++x) {
        const orc_pixel* p = row + x;
        if (p->object_id == NONE) continue;
        const orc_pixel* r = row + x + 1;
        const orc_pixel* u = up + x;
        if (differs(p, r)) {
          float angle = convex_cos_angle(*view, w, h, (float)x, (float)y, p->u, p->v, p->depth, (float)x + 1.f,
                                         (float)y, r->u, r->v, r->depth);
          o[x] = get_angle_color(angle, mc, mw, mh, cavity, p->u, p->v, p->mark);
        } else if (differs(p, u)) {
          float angle = convex_cos_angle(*view, w, h, (float)x, (float)y, p->u, p->v, p->depth, (float)x,
                                         (float)y - 1.f, u->u, u->v, u->depth);
          o[x] = get_angle_color(angle, mc, mw, mh, cavity, p->u, p->v, p->mark);
        } else {
          o[x] = get_pixel_color(p, *st, mc, mw, mh, p->u, p->v);
        }
      }
      const orc_pixel* p = row + (w - 1);
      if (p->object_id != NONE) o[w - 1] = get_pixel_color(p, *st, mc, mw, mh, p->u, p->v);
    }
    return;
  }
  for (uint32_t y = 0; y < h; ++y)
    for (uint32_t x = 0; x < w; ++x) {
      const orc_pixel* p = pix + (size_t)y * w + x;
      if (p->object_id != NONE) im[(size_t)y * w + x] = get_pixel_color(p, *st, mc, mw, mh, p->u, p->v);
    }
}

void orc_render_frame(orc_pixel* pix, uint32_t* im, const uint32_t* background, uint32_t w, uint32_t h,
                      const orc_instance* inst, uint32_t n_inst, const orc_view* view, const orc_settings* st,
                      const uint32_t* mc, uint32_t mw, uint32_t mh, uint32_t cavity, int n_threads,
                      double seconds[2], orc_stats* stats) {
  auto t0 = std::chrono::steady_clock::now();
  if (background)
    std::memcpy(im, background, sizeof(uint32_t) * (size_t)w * h);
  orc_update_canvas(pix, w, h, 0, 0, (int)w - 1, (int)h - 1, inst, n_inst, view, st, n_threads, stats);
  auto t1 = std::chrono::steady_clock::now();
  orc_canvas_to_image(pix, w, h, view, st, mc, mw, mh, cavity, im);
  auto t2 = std::chrono::steady_clock::now();
  if (seconds) {
    seconds[0] = std::chrono::duration<double>(t1 - t0).count();
    seconds[1] = std::chrono::duration<double>(t2 - t1).count();
  }
}

// matcap.cpp:9-268 (the four procedural matcaps, 512 x 512)
void orc_make_matcap(int type, uint32_t* px, uint32_t* cavity) {
  const uint32_t w = 512, h = 512;
  if (type == 3) {  // sketch, matcap.cpp:241-268
    *cavity = 0xFF505050u;
    const float thres = 0.4f;
    for (uint32_t y = 0; y < h; ++y) {
      uint32_t* row = px + (size_t)(h - y - 1) * w;
      for (uint32_t x = 0; x < w; ++x) {
        float u = (float)x / (float)(w - 1) * 2.f - 1.f;
        float v = (float)y / (float)(h - 1) * 2.f - 1.f;
        float val = std::fabs(1.f - u * u - v * v);
        if (val < thres) {
          float scale = val / thres;
          uint32_t s = (uint32_t)(scale * (float)0xe1);
          row[x] = 0xff000000u | (s << 16) | (s << 8) | s;
        } else {
          row[x] = 0xffe1e1e1u;
        }
      }
    }
    return;
  }
  float c1[3], c2[3], c3[3] = {50.f, 50.f, 50.f}, c4[3] = {30.f, 30.f, 30.f}, off[3];
  if (type == 1) {  // gray, matcap.cpp:9-84
    *cavity = 0xff505050u;
    float a[3] = {200.f / 4.f, 200.f / 4.f, 200.f / 4.f}, b[3] = {50.f, 50.f, 50.f}, o[3] = {32.f, 32.f, 32.f};
    std::memcpy(c1, a, sizeof a);
    std::memcpy(c2, b, sizeof b);
    std::memcpy(off, o, sizeof o);
  } else if (type == 2) {  // brown, matcap.cpp:87-162
    *cavity = 0xff405060u;
    float a[3] = {200.f / 4.f, 180.f / 4.f, 160.f / 4.f}, b[3] = {50.f, 40.f, 30.f}, o[3] = {32.f, 20.f, 10.f};
    std::memcpy(c1, a, sizeof a);
    std::memcpy(c2, b, sizeof b);
    std::memcpy(off, o, sizeof o);
  } else {  // red wax, matcap.cpp:164-239
    *cavity = 0xFF7D7DFFu;
    float a[3] = {200.f / 1.5f, 200.f / 4.f, 150.f / 4.f}, b[3] = {30.f, 25.f, 20.f}, o[3] = {32.f, 0.f, 0.f};
    std::memcpy(c1, a, sizeof a);
    std::memcpy(c2, b, sizeof b);
    std::memcpy(off, o, sizeof o);
  }
  auto normalize = [](f3 v) {
    float len = std::sqrt(dot3(v, v));
    return f3{v.x / len, v.y / len, v.z / len};
  };
  f3 n1 = normalize({0.f, 0.8f, 1.f}), n2 = normalize({0.f, 0.4f, 1.f}), n3 = normalize({0.f, 0.f, 1.f});
  for (uint32_t y = 0; y < h; ++y) {
    uint32_t* row = px + (size_t)(h - y - 1) * w;
    for (uint32_t x = 0; x < w; ++x) {
      float u = (float)x / (float)(w - 1) * 2.f - 1.f;
      float v = (float)y / (float)(h - 1) * 2.f - 1.f;
      if (u * u + v * v <= 1.01f) {
        float lw = std::sqrt(1.01f - u * u - v * v);
        f3 sp = {u, v, lw};
        float a1 = dot3(sp, n1);
        float a2 = std::pow(dot3(sp, n2), 3.f);
        float a3 = std::pow(dot3(sp, n3), 5.f);
        float a4 = std::pow(dot3(sp, n3), 50.f);
        float ch[3];
        for (int k = 0; k < 3; ++k) {
          float s = c1[k] * a1 + c2[k] * a2 + c3[k] * a3 + c4[k] * a4;
          float val = off[k] + s / 1.f;
          if (val > 255.f) val = 255.f;
          if (val < 0.f) val = 0.f;
          ch[k] = val;
        }
        row[x] = make_color((unsigned char)ch[0], (unsigned char)ch[1], (unsigned char)ch[2]);
      } else {
        row[x] = 0xff000000u;
      }
    }
  }
}

// pixel.cpp:6-25
uint32_t orc_get_closest_vertex(const orc_pixel* p, const float* V, const uint32_t* T) {
  const uint32_t* t = T + 3 * (size_t)p->object_id;
  f3 V0 = load3(V + 3 * (size_t)t[0]), V1 = load3(V + 3 * (size_t)t[1]), V2 = load3(V + 3 * (size_t)t[2]);
  float wgt = 1.f - p->barycentric_u - p->barycentric_v;
  f3 pos = {V0.x * wgt + p->barycentric_u * V1.x + p->barycentric_v * V2.x,
            V0.y * wgt + p->barycentric_u * V1.y + p->barycentric_v * V2.y,
            V0.z * wgt + p->barycentric_u * V1.z + p->barycentric_v * V2.z};
  f3 A = sub3(pos, V0), B = sub3(pos, V1), C = sub3(pos, V2);
  float dA = dot3(A, A), dB = dot3(B, B), dC = dot3(C, C);
  return (dA < dB) ? ((dA < dC) ? t[0] : t[2]) : ((dB < dC) ? t[1] : t[2]);
}

// view.cpp:439-459, mesh branch
void orc_get_world_position(const orc_pixel* p, const float* V, const uint32_t* T, const float* cs, float* out) {
  const uint32_t* t = T + 3 * (size_t)p->object_id;
  const float* A = V + 3 * (size_t)t[0];
  const float* B = V + 3 * (size_t)t[1];
  const float* C = V + 3 * (size_t)t[2];
  float wgt = 1.f - p->barycentric_u - p->barycentric_v;
  float pos[4];
  for (int k = 0; k < 3; ++k) pos[k] = A[k] * wgt + p->barycentric_u * B[k] + p->barycentric_v * C[k];
  pos[3] = 1.f * wgt + p->barycentric_u * 1.f + p->barycentric_v * 1.f;
  float w[4];
  mat_vec(cs, pos, w);
  out[0] = w[0];
  out[1] = w[1];
  out[2] = w[2];
}

// vox.cpp:154-173
static uint8_t color_to_index(uint8_t r, uint8_t g, uint8_t b) {
  r = r < 16 ? 0 : (uint8_t)(r - 16);
  g = g < 16 ? 0 : (uint8_t)(g - 16);
  b = b < 32 ? 0 : (uint8_t)(b - 32);
  uint8_t ret = (uint8_t)(((r >> 5) << 5) | ((g >> 5) << 2) | (b >> 6));
  return ret == 0 ? 1 : ret;
}

static uint32_t vox_cell(float p, float lo, float hi, uint32_t dim) {
  float x = (p - lo) / (hi - lo);
  float f = x * (float)dim;
  uint32_t X = f > 0.f ? (uint32_t)f : 0u;
  if (X >= dim) X = dim - 1;
  return X;
}

// vox.cpp:284-380
uint64_t orc_voxelize(const orc_mesh* m, uint32_t max_dim, uint32_t* dims, uint8_t* out, uint64_t cap) {
  const float* mn = m->min_bb;
  const float* mx = m->max_bb;
  int L = 0;
  if ((mx[1] - mn[1]) > (mx[L] - mn[L])) L = 1;
  if ((mx[2] - mn[2]) > (mx[L] - mn[L])) L = 2;
  uint32_t dim[3];
  for (int j = 0; j < 3; ++j) {
    dim[j] = (uint32_t)((float)max_dim * (mx[j] - mn[j]) / (mx[L] - mn[L]));
    if (dim[j] == 0) dim[j] = 1;
    dims[j] = dim[j];
  }
  uint64_t total = (uint64_t)dim[0] * dim[1] * dim[2];
  if (!out || cap < total) return total;
  std::memset(out, 0, total);
  const bool use_texture = m->uv != nullptr && m->tex != nullptr && m->tex_w > 0 && m->tex_h > 0;
  const bool use_colors = !use_texture && m->colors != nullptr;
  std::vector<orc_hit> hits(1u << 16);
  for (int dd = 0; dd < 3; ++dd) {
    float dir[3] = {0.f, 0.f, 0.f};
    dir[dd] = dd == 2 ? 2.f : 1.f;  // vox.cpp:311-315
    const int d1i = (dd + 1) % 3, d2i = (dd + 2) % 3;
    for (uint32_t d1 = 0; d1 < dim[d1i]; ++d1)
      for (uint32_t d2 = 0; d2 < dim[d2i]; ++d2) {
        float st[3];
        st[dd] = mn[dd];
        st[d1i] = (((float)d1 + 0.5f) / (float)dim[d1i]) * (mx[d1i] - mn[d1i]) + mn[d1i];
        st[d2i] = (((float)d2 + 0.5f) / (float)dim[d2i]) * (mx[d2i] - mn[d2i]) + mn[d2i];
        orc_ray r;
        r.orig[0] = st[0];
        r.orig[1] = st[1];
        r.orig[2] = st[2];
        r.orig[3] = 1.f;
        r.dir[0] = dir[0];
        r.dir[1] = dir[1];
        r.dir[2] = dir[2];
        r.dir[3] = 0.f;
        r.t_near = 0.f;
        r.t_far = std::numeric_limits<float>::max();
        uint32_t n = orc_find_all(m, &r, hits.data(), (uint32_t)hits.size());
        for (uint32_t i = 0; i < n && i < hits.size(); ++i) {
          const orc_hit& h = hits[i];
          const uint32_t* t = m->tris + 3 * (size_t)h.object_id;
          const float* A = m->vertices + 3 * (size_t)t[0];
          const float* B = m->vertices + 3 * (size_t)t[1];
          const float* C = m->vertices + 3 * (size_t)t[2];
          float wgt = 1.f - h.u - h.v;
          float pos[3];
          for (int k = 0; k < 3; ++k) pos[k] = A[k] * wgt + h.u * B[k] + h.v * C[k];
          float clr[3] = {1.f, 1.f, 1.f};
          if (use_texture) {
            const float* uv = m->uv + 6 * (size_t)h.object_id;
            float c0 = wgt * uv[0] + h.u * uv[2] + h.v * uv[4];
            float c1 = wgt * uv[1] + h.u * uv[3] + h.v * uv[5];
            c0 = std::max(std::min(c0, 1.f), 0.f);
            c1 = std::max(std::min(c1, 1.f), 0.f);
            int x = (int)(c0 * (float)(m->tex_w - 1));
            int y = (int)(c1 * (float)(m->tex_h - 1));
            uint32_t color = m->tex[(size_t)y * m->tex_w + x];
            clr[0] = (float)(color & 255) / 255.f;
            clr[1] = (float)((color >> 8) & 255) / 255.f;
            clr[2] = (float)((color >> 16) & 255) / 255.f;
          } else if (use_colors) {
            const float* c0 = m->colors + 3 * (size_t)t[0];
            const float* c1 = m->colors + 3 * (size_t)t[1];
            const float* c2 = m->colors + 3 * (size_t)t[2];
            for (int k = 0; k < 3; ++k) clr[k] = c0[k] * wgt + h.u * c1[k] + h.v * c2[k];
          }
          uint32_t X = vox_cell(pos[0], mn[0], mx[0], dim[0]);
          uint32_t Y = vox_cell(pos[1], mn[1], mx[1], dim[1]);
          uint32_t Z = vox_cell(pos[2], mn[2], mx[2], dim[2]);
          uint8_t ci = color_to_index((uint8_t)(clr[0] * 255.f), (uint8_t)(clr[1] * 255.f), (uint8_t)(clr[2] * 255.f));
          out[X + ((size_t)Y + (size_t)Z * dim[1]) * dim[0]] = ci;  // vox.cpp:123-127
        }
      }
  }
  return total;
}

}  // extern "C"

// canvas.cpp:952-1030 render_pointclouds_on_image (sequential restatement)
void orc_render_pointclouds(orc_pixel* pix, uint32_t* im, uint32_t w, uint32_t h, const float* P,
                            const float* cs_inv, float near_plane, uint32_t n_clouds, const float* const* vertices,
                            const uint64_t* counts, const uint32_t* const* colors, const float* cs,
                            const uint32_t* db_ids, int one_bit) {
  const size_t npix = (size_t)w * h;
  std::vector<float> z(npix);
  for (size_t i = 0; i < npix; ++i) z[i] = pix[i].db_id != 0 ? 1.f / pix[i].depth : 0.f;  // canvas.cpp:966
  const float half_w = 0.5f * (float)w, half_h = 0.5f * (float)h;
  for (uint32_t k = 0; k < n_clouds; ++k) {
    const float* V = vertices[k];
    const float* M = cs + 16 * (size_t)k;
    for (uint64_t i = 0; i < counts[k]; ++i) {
      float v[4] = {V[3 * i], V[3 * i + 1], V[3 * i + 2], 1.f}, wv[4], cv[4];
      mat_vec(M, v, wv);
      mat_vec(cs_inv, wv, cv);
      const float d = -cv[2];
      if (!(d > near_plane)) continue;
      const float inv_d = 1.f / d;
      float sx = P[0] * cv[0];
      sx = sx * inv_d;
      sx = sx + P[8];
      float sy = P[5] * cv[1];
      sy = sy * inv_d;
      sy = sy + P[9];
      const float fx = (sx + 1.f) * half_w;
      const float fy = (sy + 1.f) * half_h;
      if (!(fx >= 0.f && fx < (float)w && fy >= 0.f && fy < (float)h)) continue;
      const uint32_t col = std::min((uint32_t)fx, w - 1), row = std::min((uint32_t)fy, h - 1);
      const size_t idx = (size_t)row * w + col;
      if (inv_d > z[idx]) {
        z[idx] = inv_d;
        pix[idx].object_id = (uint32_t)i;
        pix[idx].depth = 1.f / z[idx];
        pix[idx].db_id = db_ids[k];
        im[idx] = (colors[k] && !one_bit) ? colors[k][i] : 0xffffffffu;
      }
    }
  }
}

