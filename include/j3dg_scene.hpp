// j3dg_scene.hpp -- header-only C++ shim with j3d's own scene / canvas / matcap
// signatures over the C-ABI of j3dg.h, so that j3d's view code keeps its call
// sites:
//
//   add_object(id, scene, db)            scene.cpp:8-38   -> add_object(ctx, id, scene, vertices, ...)
//   remove_object / prepare_scene / unzoom scene.cpp:40-110
//   canvas(w, h), resize, update_settings, set_background_color,
//   update_canvas(x0, y0, x1, y1, scene), render_scene(const scene*),
//   canvas_to_image(matcap), canvas_to_image(pixels, matcap),
//   get_pixels(), get_image()          canvas.h:27-101
//   make_matcap_*                        matcap.cpp:9-347
//
// The jtk types of the reference (vec3, float4x4, image<T>) become plain
// arrays and std::vector; float4x4 stays column-major with the translation in
// [12..14]. Errors from the C-ABI are thrown as j3dgpu::error (the reference
// has no error channel on these calls; its blit_onto throws std::runtime_error).
#pragma once

#include <cstdint>
#include <cstring>
#include <list>
#include <stdexcept>
#include <string>
#include <vector>

#include "j3dg.h"

namespace j3dgpu {

struct error : std::runtime_error {
  int status;
  error(int s, const std::string& what) : std::runtime_error(what), status(s) {}
};

inline void check(int status, const j3dg_ctx* ctx, const char* where) {
  if (status != J3DG_OK) {
    std::string msg = std::string(where) + ": " + j3dg_status_string(status);
    if (ctx) msg += std::string(" (") + j3dg_last_error(ctx) + ")";
    throw error(status, msg);
  }
}

using pixel = j3dg_pixel;  // pixel.h:11-27, byte-identical

class context {
 public:
  explicit context(int device = 0) { check(j3dg_ctx_create(device, &ctx_), nullptr, "j3dg_ctx_create"); }
  ~context() {
    if (ctx_) j3dg_ctx_destroy(ctx_);
  }
  context(const context&) = delete;
  context& operator=(const context&) = delete;
  j3dg_ctx* get() const { return ctx_; }
  void synchronize() { check(j3dg_ctx_synchronize(ctx_), ctx_, "synchronize"); }

 private:
  j3dg_ctx* ctx_ = nullptr;
};

inline void identity(float m[16]) {
  for (int i = 0; i < 16; ++i) m[i] = (i % 5 == 0) ? 1.f : 0.f;
}

// scene_object (scene.h:10-25): the BVH lives on the device.
struct scene_object {
  uint32_t db_id = 0;
  j3dg_mesh* bvh = nullptr;
  float cs[16];
  float min_bb[3], max_bb[3];
};

// scene_pointcloud (scene.h:27-38): the points live on the device.
struct scene_pointcloud {
  uint32_t db_id = 0;
  j3dg_pointcloud* points = nullptr;
  float cs[16];
  float min_bb[3], max_bb[3];
};

// scene (scene.h:40-51)
struct scene {
  float coordinate_system[16], coordinate_system_inv[16];
  float pivot[3] = {0, 0, 0};
  float min_bb[3] = {0, 0, 0}, max_bb[3] = {0, 0, 0};
  float diagonal = 0.f;
  std::list<scene_object> objects;
  std::list<scene_pointcloud> pointclouds;
  scene() {
    identity(coordinate_system);
    identity(coordinate_system_inv);
  }
  ~scene() {
    for (auto& o : objects) j3dg_mesh_destroy(o.bvh);
    for (auto& o : pointclouds) j3dg_pointcloud_destroy(o.points);
  }
  scene(const scene&) = delete;
  scene& operator=(const scene&) = delete;
};

// add_object (scene.cpp:8-38): normals, bbox and the BVH, built on the GPU.
inline void add_object(context& ctx, uint32_t id, scene& s, const float* vertices, uint32_t n_vertices,
                       const uint32_t* triangles, uint32_t n_triangles, const float* cs = nullptr,
                       uint32_t leaf_size = 2) {
  scene_object o;
  o.db_id = id;
  if (cs)
    std::memcpy(o.cs, cs, sizeof(o.cs));
  else
    identity(o.cs);
  j3dg_build_opts opts{leaf_size, 0};
  check(j3dg_mesh_build(ctx.get(), vertices, n_vertices, triangles, n_triangles, &opts, &o.bvh), ctx.get(),
        "add_object");
  j3dg_mesh_info info;
  check(j3dg_mesh_get_info(o.bvh, &info), ctx.get(), "add_object");
  std::memcpy(o.min_bb, info.min_bb, sizeof(o.min_bb));
  std::memcpy(o.max_bb, info.max_bb, sizeof(o.max_bb));
  s.objects.push_back(o);
}

// add_object's point-cloud branch (scene.cpp:27-36): n points (n x 3
// floats), optional packed RGBA8 colours.
inline void add_pointcloud(context& ctx, uint32_t id, scene& s, const float* vertices, uint64_t n,
                           const uint32_t* colors = nullptr, const float* cs = nullptr) {
  scene_pointcloud o;
  o.db_id = id;
  if (cs)
    std::memcpy(o.cs, cs, sizeof(o.cs));
  else
    identity(o.cs);
  check(j3dg_pointcloud_create(ctx.get(), vertices, n, colors, &o.points), ctx.get(), "add_pointcloud");
  check(j3dg_pointcloud_get_bounds(o.points, o.min_bb, o.max_bb), ctx.get(), "add_pointcloud");
  s.pointclouds.push_back(o);
}

// read_from_file (mesh.cpp:76-176 / pc.cpp:32-110) + add_object: the file is
// decoded on the device; a file with triangles becomes a mesh object with its
// BVH, one without becomes a point cloud. Returns true for a mesh.
inline bool add_object_from_file(context& ctx, uint32_t id, scene& s, const char* path, const float* cs = nullptr,
                                 uint32_t leaf_size = 2) {
  j3dg_geometry* g = nullptr;
  check(j3dg_geometry_read_file(ctx.get(), path, J3DG_FORMAT_AUTO, &g), ctx.get(), "read_from_file");
  j3dg_geometry_info info;
  j3dg_geometry_get_info(g, &info);
  const bool is_mesh = info.n_triangles > 0;
  int rc = J3DG_OK;
  if (is_mesh) {
    scene_object o;
    o.db_id = id;
    if (cs)
      std::memcpy(o.cs, cs, sizeof(o.cs));
    else
      identity(o.cs);
    j3dg_build_opts opts{leaf_size, 0};
    rc = j3dg_mesh_build_geometry(ctx.get(), g, &opts, &o.bvh);
    if (rc == J3DG_OK) {
      j3dg_mesh_info mi;
      j3dg_mesh_get_info(o.bvh, &mi);
      std::memcpy(o.min_bb, mi.min_bb, sizeof(o.min_bb));
      std::memcpy(o.max_bb, mi.max_bb, sizeof(o.max_bb));
      s.objects.push_back(o);
    }
  } else {
    scene_pointcloud o;
    o.db_id = id;
    if (cs)
      std::memcpy(o.cs, cs, sizeof(o.cs));
    else
      identity(o.cs);
    rc = j3dg_pointcloud_from_geometry(ctx.get(), g, &o.points);
    if (rc == J3DG_OK) {
      j3dg_pointcloud_get_bounds(o.points, o.min_bb, o.max_bb);
      s.pointclouds.push_back(o);
    }
  }
  j3dg_geometry_destroy(g);
  check(rc, ctx.get(), "read_from_file");
  return is_mesh;
}

// remove_object (scene.cpp:40-48)
inline void remove_object(uint32_t id, scene& s) {
  for (auto it = s.objects.begin(); it != s.objects.end(); ++it)
    if (it->db_id == id) {
      j3dg_mesh_destroy(it->bvh);
      s.objects.erase(it);
      break;
    }
  for (auto it = s.pointclouds.begin(); it != s.pointclouds.end(); ++it)
    if (it->db_id == id) {
      j3dg_pointcloud_destroy(it->points);
      s.pointclouds.erase(it);
      break;
    }
}

inline std::vector<j3dg_pointcloud_instance> pointcloud_instances(const scene& s) {
  std::vector<j3dg_pointcloud_instance> v;
  v.reserve(s.pointclouds.size());
  for (const auto& o : s.pointclouds) {
    j3dg_pointcloud_instance i;
    i.pointcloud = o.points;
    std::memcpy(i.cs, o.cs, sizeof(i.cs));
    i.db_id = o.db_id;
    i.reserved = 0;
    v.push_back(i);
  }
  return v;
}

inline std::vector<j3dg_instance> instances(const scene& s) {
  std::vector<j3dg_instance> v;
  v.reserve(s.objects.size());
  for (const auto& o : s.objects) {
    j3dg_instance i;
    i.mesh = o.bvh;
    std::memcpy(i.cs, o.cs, sizeof(i.cs));
    i.db_id = o.db_id;
    i.reserved = 0;
    v.push_back(i);
  }
  return v;
}

// prepare_scene (scene.cpp:50-89)
inline void prepare_scene(scene& s) {
  auto inst = instances(s);
  auto pcs = pointcloud_instances(s);
  check(j3dg_prepare_scene_pointclouds(inst.data(), (uint32_t)inst.size(), pcs.data(), (uint32_t)pcs.size(),
                                       s.min_bb, s.max_bb, &s.diagonal),
        nullptr, "prepare_scene");
}

// unzoom (scene.cpp:91-110)
inline void unzoom(scene& s) { j3dg_unzoom(s.min_bb, s.max_bb, s.diagonal, s.coordinate_system, s.coordinate_system_inv, s.pivot); }

inline j3dg_scene to_c(const scene& s, std::vector<j3dg_instance>& keep) {
  keep = instances(s);
  j3dg_scene c;
  c.objects = keep.data();
  c.n_objects = (uint32_t)keep.size();
  c.reserved = 0;
  std::memcpy(c.coordinate_system, s.coordinate_system, sizeof(c.coordinate_system));
  std::memcpy(c.coordinate_system_inv, s.coordinate_system_inv, sizeof(c.coordinate_system_inv));
  std::memcpy(c.pivot, s.pivot, sizeof(c.pivot));
  c.diagonal = s.diagonal;
  return c;
}

enum class matcap_type { MATCAP_TYPE_INTERNAL_REDWAX, MATCAP_TYPE_INTERNAL_GRAY, MATCAP_TYPE_INTERNAL_BROWN,
                         MATCAP_TYPE_INTERNAL_SKETCH, MATCAP_TYPE_EXTERNAL_FILE };

// matcap (matcap.h:18-24), uploaded to the device once.
class matcap {
 public:
  matcap(context& ctx, matcap_type t) : ctx_(ctx) {
    int kind = t == matcap_type::MATCAP_TYPE_INTERNAL_GRAY ? 1
               : t == matcap_type::MATCAP_TYPE_INTERNAL_BROWN ? 2
               : t == matcap_type::MATCAP_TYPE_INTERNAL_SKETCH ? 3 : 0;
    im.resize(512 * 512);
    check(j3dg_make_matcap(kind, im.data(), &w, &h, &cavity_clr), nullptr, "make_matcap");
    upload();
  }
  // a PNG matcap decoded by the caller (make_matcap_from_file, matcap.cpp:270-308)
  matcap(context& ctx, const uint32_t* pixels, uint32_t w_, uint32_t h_, uint32_t cavity) : ctx_(ctx) {
    im.assign(pixels, pixels + (size_t)w_ * h_);
    w = w_;
    h = h_;
    cavity_clr = cavity;
    upload();
  }
  ~matcap() {
    if (dev_) j3dg_matcap_destroy(dev_);
  }
  matcap(const matcap&) = delete;
  matcap& operator=(const matcap&) = delete;
  const j3dg_matcap* get() const { return dev_; }
  std::vector<uint32_t> im;
  uint32_t w = 0, h = 0, cavity_clr = 0;

 private:
  void upload() { check(j3dg_matcap_create(ctx_.get(), im.data(), w, h, cavity_clr, &dev_), ctx_.get(), "matcap"); }
  context& ctx_;
  j3dg_matcap* dev_ = nullptr;
};

// canvas (canvas.h:27-101)
class canvas {
 public:
  using canvas_settings = j3dg_canvas_settings;

  canvas(context& ctx, uint32_t w, uint32_t h) : ctx_(ctx) {
    check(j3dg_canvas_create(ctx.get(), w, h, &cv_), ctx.get(), "canvas");
    w_ = w;
    h_ = h;
  }
  ~canvas() {
    if (cv_) j3dg_canvas_destroy(cv_);
  }
  canvas(const canvas&) = delete;
  canvas& operator=(const canvas&) = delete;

  void resize(uint32_t w, uint32_t h) {
    check(j3dg_canvas_resize(cv_, w, h), ctx_.get(), "resize");
    w_ = w;
    h_ = h;
  }
  void set_camera(const j3dg_camera& c) { check(j3dg_canvas_set_camera(cv_, &c), ctx_.get(), "set_camera"); }
  void update_settings(const canvas_settings& s) { check(j3dg_canvas_update_settings(cv_, &s), ctx_.get(), "update_settings"); }
  void set_background_color(uint32_t clr_top = 0xff000000, uint32_t clr_bottom = 0xff404040) {
    check(j3dg_canvas_set_background_color(cv_, clr_top, clr_bottom), ctx_.get(), "set_background_color");
  }
  void update_canvas(int x0, int y0, int x1, int y1, const scene& s) {
    std::vector<j3dg_instance> keep;
    j3dg_scene c = to_c(s, keep);
    check(j3dg_canvas_update_canvas(cv_, x0, y0, x1, y1, &c), ctx_.get(), "update_canvas");
  }
  void render_scene(const scene* s) {
    if (!s) {
      check(j3dg_canvas_render_scene(cv_, nullptr), ctx_.get(), "render_scene");
      return;
    }
    std::vector<j3dg_instance> keep;
    j3dg_scene c = to_c(*s, keep);
    check(j3dg_canvas_render_scene(cv_, &c), ctx_.get(), "render_scene");
  }
  void canvas_to_image(const matcap& m) { check(j3dg_canvas_to_image(cv_, m.get()), ctx_.get(), "canvas_to_image"); }
  void canvas_to_image(const std::vector<pixel>& pixels, const matcap& m) {
    check(j3dg_canvas_to_image_from(cv_, pixels.data(), m.get()), ctx_.get(), "canvas_to_image");
  }
  // view::render_scene (view.cpp:421-430) in one call
  void render_frame(const scene* s, const matcap& m) {
    std::vector<j3dg_instance> keep;
    j3dg_scene c;
    if (s) c = to_c(*s, keep);
    check(j3dg_canvas_render_frame(cv_, s ? &c : nullptr, m.get()), ctx_.get(), "render_frame");
  }
  // canvas::render_pointclouds_on_image (canvas.cpp:952-1030), after a frame
  void render_pointclouds_on_image(const scene* s) {
    if (!s || s->pointclouds.empty()) return;
    std::vector<j3dg_instance> keep;
    j3dg_scene c = to_c(*s, keep);
    auto pcs = pointcloud_instances(*s);
    check(j3dg_canvas_render_pointclouds(cv_, &c, pcs.data(), (uint32_t)pcs.size()), ctx_.get(),
          "render_pointclouds_on_image");
  }
  std::vector<pixel> get_pixels() const {
    std::vector<pixel> out((size_t)w_ * h_);
    check(j3dg_canvas_get_pixels(cv_, out.data()), ctx_.get(), "get_pixels");
    return out;
  }
  std::vector<uint32_t> get_image() const {
    std::vector<uint32_t> out((size_t)w_ * h_);
    check(j3dg_canvas_get_image(cv_, out.data()), ctx_.get(), "get_image");
    return out;
  }
  uint32_t width() const { return w_; }
  uint32_t height() const { return h_; }
  j3dg_canvas* get() const { return cv_; }

 private:
  context& ctx_;
  j3dg_canvas* cv_ = nullptr;
  uint32_t w_ = 0, h_ = 0;
};

}  // namespace j3dgpu
