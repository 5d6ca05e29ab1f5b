/*
 * j3d_oracle.h -- C-ABI of the CPU oracle (test infrastructure only).
 *
 * The oracle is a portable C++ restatement of j3d's ray-cast hot path, used
 * ONLY by the test suite, by __graft_entry__.smoke() and by bench.py's CPU
 * baseline leg, always as the checker and never as the thing measured or
 * shipped. The product (libj3dgpu.so) never links or loads it.
 *
 * Parity status: "parity unpinned" for the BVH and the ray/triangle test.
 * Those live in jtk/qbvh.h, an un-vendored submodule (github.com/janm31415/jtk,
 * no pinned commit) that is absent from the reference tree, and the reference
 * has no tests or golden vectors. Everything that the reference tree does hold
 * (camera, scene, canvas, matcap) is restated here line by line, each function
 * citing the reference file:line it follows.
 */
#pragma once
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* pixel.h:11-27 -- 32-byte G-buffer record */
typedef struct orc_pixel {
  uint8_t mark, r, g, b;
  float u, v, depth;
  uint32_t object_id;
  float barycentric_u, barycentric_v;
  uint32_t db_id;
} orc_pixel;

/* jtk::ray as used by canvas.cpp:778-782 */
typedef struct orc_ray {
  float orig[4];
  float dir[4];
  float t_near, t_far;
} orc_ray;

/* jtk::hit {found, distance, u, v} + find_closest_triangle's out-params */
typedef struct orc_hit {
  uint32_t found;
  float distance, u, v;
  uint32_t object_id;
  uint32_t two_level_index;
} orc_hit;

/* camera.h:5-16 */
typedef struct orc_camera {
  float focal_length;
  float film_aperture_width_inch;
  float film_aperture_height_inch;
  float near_clipping_plane;
  float far_clipping_plane;
  float zoom;
  int32_t fit_film; /* 0 = Fill, 1 = Overscan */
} orc_camera;

/* canvas.h:16-25 */
typedef struct orc_settings {
  uint8_t one_bit, shadow, edges, wireframe, shading, textured, vertexcolors, reserved;
} orc_settings;

typedef struct orc_mesh orc_mesh; /* vertices, triangles, normals, qbvh */

/* One scene_object as gathered by canvas.cpp:729-742 */
typedef struct orc_instance {
  const orc_mesh* mesh;
  float cs[16];
  uint32_t db_id;
  uint32_t reserved;
} orc_instance;

/* scene.h:40-51 (the parts update_canvas reads) + the canvas projection */
typedef struct orc_view {
  float coordinate_system[16];
  float coordinate_system_inv[16];
  float pivot[3];
  float diagonal;
  float projection_inv[16];
  float near_clipping_plane;
} orc_view;

typedef struct orc_stats {
  uint64_t rays, node_visits, tri_tests;
} orc_stats;

/* ---- camera.cpp ---- */
void orc_make_default_camera(orc_camera* c);
void orc_frustum(float l, float r, float b, float t, float n, float f, float out[16]);
void orc_invert_projection_matrix(const float in[16], float out[16]);
void orc_make_projection_matrix(const orc_camera* c, int w, int h, float out[16]);
/* jtk invert_orthonormal */
void orc_invert_orthonormal(const float in[16], float out[16]);
void orc_matrix_vector_multiply(const float m[16], const float v[4], float out[4]);

/* ---- mesh.cpp / geometry.h / scene.cpp ---- */
void orc_compute_bb(const float* vertices, uint32_t nv, float min_bb[3], float max_bb[3]);
void orc_compute_triangle_normals(const float* vertices, const uint32_t* tris, uint32_t nt, float* normals);

/* scene.cpp:50-89 prepare_scene over mesh objects (bbox of each object
   transformed by its cs) -> scene bbox and diagonal. */
void orc_prepare_scene(const float* obj_min_bb, const float* obj_max_bb, const float* obj_cs, uint32_t n,
                       float min_bb[3], float max_bb[3], float* diagonal);
/* scene.cpp:91-110 unzoom (y axis up) -> coordinate_system, its inverse, pivot */
void orc_unzoom(const float min_bb[3], const float max_bb[3], float diagonal, float cs[16], float cs_inv[16],
                float pivot[3]);

/* ---- qbvh restatement ---- */
/* Builds normals, bbox and a 4-wide binned-SAH BVH (leaf <= leaf_max) with
   n_threads worker threads. The mesh keeps pointers to the caller's arrays. */
orc_mesh* orc_mesh_build(const float* vertices, uint32_t nv, const uint32_t* tris, uint32_t nt,
                         uint32_t leaf_max, int n_threads, double* build_seconds);
void orc_mesh_free(orc_mesh* m);
uint32_t orc_mesh_node_count(const orc_mesh* m);
uint32_t orc_mesh_max_depth(const orc_mesh* m);
const float* orc_mesh_normals(const orc_mesh* m);
void orc_mesh_set_vertex_colors(orc_mesh* m, const float* colors);
void orc_mesh_set_uv(orc_mesh* m, const float* uv /* nt*6 */);
void orc_mesh_set_texture(orc_mesh* m, const uint32_t* tex, uint32_t w, uint32_t h);

/* find_closest_triangle over a two-level scene; mode 0 = BVH, 1 = brute force.
   any_hit != 0 stops at the first accepted triangle (only found is exact). */
void orc_find_closest(const orc_instance* inst, uint32_t n_inst, const orc_ray* rays, uint32_t n,
                      orc_hit* hits, int mode, int any_hit, int n_threads, orc_stats* stats);

/* find_all_triangles (vox.cpp:333): every accepted triangle along the ray
   (t < t_far), sorted by (t, id); through the BVH or by brute force.
   Returns the count; writes up to cap hits. */
uint32_t orc_find_all(const orc_mesh* m, const orc_ray* ray, orc_hit* hits, uint32_t cap);
uint32_t orc_find_all_brute(const orc_mesh* m, const orc_ray* ray, orc_hit* hits, uint32_t cap);

/* ---- canvas.cpp ---- */
/* canvas::render_pointclouds_on_image (canvas.cpp:952-1030), restated
   sequentially: z-buffer of 1/depth from the G-buffer (0 where db_id is
   0); for each cloud in order and each point in id order, the point in
   camera space (cloud cs, then cs_inv), d = -z; drawn only for d > near;
   pixel (floor((P0 x/d + P8 + 1) w/2), floor((P5 y/d + P9 + 1) h/2)); kept
   when 1/d > z-buffer; sets object_id = point id, depth = 1/(1/d), db_id and
   the image colour (the point colour, white without colours or one_bit).
   colors[k] may be NULL. */
void orc_render_pointclouds(orc_pixel* pix, uint32_t* im, uint32_t w, uint32_t h, const float projection[16],
                            const float cs_inv[16], float near_plane, uint32_t n_clouds, const float* const* vertices,
                            const uint64_t* counts, const uint32_t* const* colors, const float* cs,
                            const uint32_t* db_ids, int one_bit);

void orc_fill_background(uint32_t* bg, uint32_t w, uint32_t h, uint32_t clr_top, uint32_t clr_bottom);
void orc_update_canvas(orc_pixel* out, uint32_t w, uint32_t h, int x0, int y0, int x1, int y1,
                       const orc_instance* inst, uint32_t n_inst, const orc_view* view,
                       const orc_settings* settings, int n_threads, orc_stats* stats);
void orc_canvas_to_image(const orc_pixel* pix, uint32_t w, uint32_t h, const orc_view* view,
                         const orc_settings* settings, const uint32_t* matcap, uint32_t mw,
                         uint32_t mh, uint32_t cavity_clr, uint32_t* im);
/* view::render_scene (view.cpp:421-430): background copy, update_canvas over
   the whole canvas, canvas_to_image. Returns seconds for (render, shade). */
void orc_render_frame(orc_pixel* pix, uint32_t* im, const uint32_t* background, uint32_t w, uint32_t h,
                      const orc_instance* inst, uint32_t n_inst, const orc_view* view,
                      const orc_settings* settings, const uint32_t* matcap, uint32_t mw, uint32_t mh,
                      uint32_t cavity_clr, int n_threads, double seconds[2], orc_stats* stats);

/* ---- matcap.cpp ---- 0 red wax, 1 gray, 2 brown, 3 sketch; 512x512 */
void orc_make_matcap(int type, uint32_t* pixels, uint32_t* cavity_clr);

/* view.cpp:439-480 picking helpers */
uint32_t orc_get_closest_vertex(const orc_pixel* p, const float* vertices, const uint32_t* tris);
/* view.cpp:439-459 (mesh branch): world position of the pixel's hit point */
void orc_get_world_position(const orc_pixel* p, const float* vertices, const uint32_t* tris, const float cs[16],
                            float out[3]);

/* vox.cpp:284-380 (the voxel grid of write_vox): grid dims from max_dim and
   the mesh bbox, three axis-aligned ray sweeps with find_all_triangles, each
   hit's voxel set to its colour index; writes in sweep order, hits in (t, id)
   order, the last write of a voxel wins. Colours: uv + texture if set, else
   vertex colours if set, else white. Returns the voxel count (dims product);
   fills dims and, if out != NULL and cap is large enough, the voxels. */
uint64_t orc_voxelize(const orc_mesh* m, uint32_t max_dim, uint32_t dims[3], uint8_t* out, uint64_t cap);

#ifdef __cplusplus
}
#endif
