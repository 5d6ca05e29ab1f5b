/*
 * j3dg.h -- C-ABI of libj3dgpu.so, the GB300 (sm_103a) implementation of
 * j3d's ray-cast rendering hot path.
 *
 * The reference has no FFI for this path: its boundary is the in-process C++
 * API of jtk::qbvh (built at scene.cpp:23, queried at canvas.cpp:762,786,854
 * and vox.cpp:307,333) and, above it, class canvas (canvas.h:27-101) driven by
 * view::render_scene (view.cpp:421-430). Every entry point below names the
 * reference call it replaces. All entry points:
 *   - are extern "C", take plain pointers and sizes, never throw;
 *   - return j3dg_status (J3DG_OK == 0); j3dg_last_error() gives the text;
 *   - accept host or device pointers for bulk arrays (detected per call) --
 *     device pointers must live on the context's device;
 *   - run on the context's single CUDA stream. A context, and everything made
 *     from it, must not be used from two threads at once (j3d serialises the
 *     same calls behind view::_mut, view.cpp:1262).
 * There is no CPU fallback: without a usable GPU, j3dg_ctx_create fails.
 */
#ifndef J3DG_H
#define J3DG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define J3DG_ABI_VERSION 1

typedef enum j3dg_status {
  J3DG_OK = 0,
  J3DG_ERR_INVALID_ARGUMENT = 1,
  J3DG_ERR_CUDA = 2,
  J3DG_ERR_OUT_OF_MEMORY = 3,
  J3DG_ERR_NO_DEVICE = 4,
  J3DG_ERR_DEVICE_STATUS = 5, /* a kernel raised its status word (see j3dg_ctx_device_status) */
  J3DG_ERR_UNSUPPORTED = 6
} j3dg_status;

/* Device status word bits raised by kernels instead of trapping. */
#define J3DG_DEV_STACK_OVERFLOW 0x1u
#define J3DG_DEV_VISIT_CAP 0x2u
#define J3DG_DEV_BAD_INDEX 0x4u
#define J3DG_DEV_HIT_OVERFLOW 0x8u /* more than 64 hits on one voxelization ray */
#define J3DG_DEV_WAIT_TIMEOUT 0x10u /* a frame waited too long for its canvas's previous frame */

typedef struct j3dg_ctx j3dg_ctx;
typedef struct j3dg_mesh j3dg_mesh;
typedef struct j3dg_canvas j3dg_canvas;
typedef struct j3dg_matcap j3dg_matcap;

/* pixel.h:11-27 -- byte-identical 32-byte G-buffer record.
   mark bit 0: in shadow; bit 1: r,g,b hold texture / vertex colour. */
typedef struct j3dg_pixel {
  uint8_t mark, r, g, b;
  float u;
  float v;
  float depth;
  uint32_t object_id;
  float barycentric_u;
  float barycentric_v;
  uint32_t db_id;
} j3dg_pixel;

/* jtk::ray {float4 orig, dir; float t_near, t_far} (canvas.cpp:778-782) */
typedef struct j3dg_ray {
  float orig[4];
  float dir[4];
  float t_near;
  float t_far;
} j3dg_ray;

/* jtk::hit {found, distance, u, v} plus the two out-parameters of
   find_closest_triangle (object_id = triangle, two_level_index = object). */
typedef struct j3dg_hit {
  uint32_t found;
  float distance;
  float u;
  float v;
  uint32_t object_id;
  uint32_t two_level_index;
} j3dg_hit;

/* One scene_object as canvas.cpp:729-742 gathers it: the mesh (with its BVH),
   the object's coordinate system and its db id. */
typedef struct j3dg_instance {
  const j3dg_mesh* mesh;
  float cs[16];
  uint32_t db_id;
  uint32_t reserved;
} j3dg_instance;

/* scene.h:40-51, the fields update_canvas reads (canvas.cpp:700-742). */
typedef struct j3dg_scene {
  const j3dg_instance* objects;
  uint32_t n_objects;
  uint32_t reserved;
  float coordinate_system[16];
  float coordinate_system_inv[16];
  float pivot[3];
  float diagonal;
} j3dg_scene;

/* camera.h:5-16 (fit_film: 0 = Fill, 1 = Overscan) */
typedef struct j3dg_camera {
  float focal_length;
  float film_aperture_width_inch;
  float film_aperture_height_inch;
  float near_clipping_plane;
  float far_clipping_plane;
  float zoom;
  int32_t fit_film;
} j3dg_camera;

/* canvas.h:16-25 */
typedef struct j3dg_canvas_settings {
  uint8_t one_bit;
  uint8_t shadow;
  uint8_t edges;
  uint8_t wireframe;
  uint8_t shading;
  uint8_t textured;
  uint8_t vertexcolors;
  uint8_t reserved;
} j3dg_canvas_settings;

/* BVH build options (NULL = defaults). */
typedef struct j3dg_build_opts {
  uint32_t leaf_size;  /* max triangles per leaf, 1..8 (default 2: fastest on the torus frames) */
  uint32_t flags;      /* 0: the default builder; J3DG_BUILD_LBVH: see below */
} j3dg_build_opts;
/* The default binary tree has binned-SAH top levels down to ranges of 64
   triangles and parallel locally-ordered clustering (Meister and Bittner
   2018) within them, collapsed by a cost-optimal programme: the fewest node
   visits per ray. J3DG_BUILD_LBVH splits at Morton prefixes instead (4-wide
   only): about 40 % of the build time (12.0 vs 30.6 ms for 28M triangles),
   about 19 % more node visits per ray. Either build is one CUDA
   graph with device-driven level loops. The traversal results are the same
   for either tree. */
#define J3DG_BUILD_LBVH 0x1u
/* BVH width (children per node) of the default builder: 4 unless one of
   these is set. The cost-optimal collapse of the binary tree is run for the
   chosen width; results do not depend on it. Nodes are 64 B (2 children),
   128 B (4) or 256 B (8). Meshes of one frame, batch or ray query must share
   a width; all-hits queries, voxel grids and learned networks need width 4. */
#define J3DG_BUILD_WIDTH2 0x2u
#define J3DG_BUILD_WIDTH8 0x4u
/* A mesh that a batch can rebuild inside its graph (j3dg_batch_create2 with
   J3DG_BATCH_REBUILD): it keeps a device copy of its vertices and its node
   array at the size bound (nt - 1 nodes), so the rebuild writes in place.
   Either builder. No reference counterpart. */
#define J3DG_BUILD_REBUILDABLE 0x8u

typedef struct j3dg_mesh_info {
  uint32_t n_vertices;
  uint32_t n_triangles;
  float min_bb[3];
  float max_bb[3];
  uint32_t n_nodes;
  uint32_t max_depth;
  uint64_t device_bytes;
  float build_ms; /* device time of the last build, CUDA events */
  uint32_t width; /* children per BVH node: 2, 4 or 8 */
} j3dg_mesh_info;

/* ---------------------------------------------------------------- context */

/* No reference counterpart (j3d owns no device). One stream per context. */
int j3dg_ctx_create(int device, j3dg_ctx** out);
/* Returns J3DG_ERR_INVALID_ARGUMENT, and keeps the context, while meshes,
   geometries, point clouds, matcaps, canvases, batches or learned predictors
   made from it are not destroyed. */
int j3dg_ctx_destroy(j3dg_ctx* ctx);
/* Waits for the stream; returns J3DG_ERR_DEVICE_STATUS if a kernel raised
   the status word since the last check (the word is then cleared). */
int j3dg_ctx_synchronize(j3dg_ctx* ctx);
int j3dg_ctx_device_status(j3dg_ctx* ctx, uint32_t* status);
/* The context's cudaStream_t, for callers that order their own work. */
void* j3dg_ctx_stream(j3dg_ctx* ctx);
const char* j3dg_last_error(const j3dg_ctx* ctx);
/* Instrumentation (no reference counterpart): when enabled, frame kernels
   add their BVH node visits and triangle tests to two device counters. */
int j3dg_ctx_set_counting(j3dg_ctx* ctx, int enable);
int j3dg_ctx_read_counters(j3dg_ctx* ctx, uint64_t out[2], int reset);
/* Scenes of two or more objects are walked through a per-frame top level,
   a BVH4 over the objects' world boxes (the two-level structure of
   qbvh_two_level_with_transformations, canvas.cpp:762, 786, 854). With
   enable = 0 the kernels walk the objects one after the other instead (the
   same results; for measurement). Default 1. */
int j3dg_ctx_set_top_level(j3dg_ctx* ctx, int enable);
/* Overlapped frames (no reference counterpart): a traced frame of a canvas
   (j3dg_canvas_render_frame) is launched so that it may start while the
   canvas's previous frame finishes its last pixels; each pixel carries the
   number of the frame that last wrote it, and a frame writes a pixel only
   once the previous frame's number is there, so results are those of
   frames run one after the other. Frames after other writes to the canvas
   (rectangles, rasterised or learned frames, batches, shading) do not
   overlap. enable = 0 runs every frame after the previous one has ended
   (for measurement). Default 1. */
int j3dg_ctx_set_frame_overlap(j3dg_ctx* ctx, int enable);
/* Diagnostics: the canvas's next traced frame waits for every pixel to carry
   frame number seq. A number no frame wrote makes the waits run out (half a
   second): the frame raises J3DG_DEV_WAIT_TIMEOUT (J3DG_ERR_DEVICE_STATUS at
   the next synchronising call) and the context stays usable. */
int j3dg_canvas_expect_frame(j3dg_canvas* cv, uint32_t seq);
/* Device memory as the context sees it (no reference counterpart; the
   reference has no device memory): out[0..1] free and total bytes of the
   device (cudaMemGetInfo), out[2..3] bytes reserved and in use by the
   context's canvas pool, out[4..5] the same for the device's default
   stream-ordered pool (BVH build scratch). */
int j3dg_ctx_memory(j3dg_ctx* ctx, uint64_t out[6]);
/* How canvas frames (render_frame, update_canvas, render_scene) find the
   primary hits (no reference counterpart; the result is the same either
   way). TRACE walks the BVH per pixel. RASTER projects every triangle's box
   to the screen and runs the traversal's own ray / triangle test on the
   pixels inside, keeping each pixel's minimum of (t, object, triangle id),
   which is the traversal's closest hit; it needs every object's box in
   front of the camera and reads every triangle once per frame (frames
   that do not allow it are traced). AUTO (the default) traces. Shadow rays
   are always traced. */
#define J3DG_PRIMARY_AUTO 0
#define J3DG_PRIMARY_TRACE 1
#define J3DG_PRIMARY_RASTER 2
int j3dg_ctx_set_primary_mode(j3dg_ctx* ctx, int mode);
const char* j3dg_status_string(int status);
int j3dg_abi_version(void);

/* ----------------------------------------------------------------- meshes */

/* Replaces scene.cpp:20-23 in add_object: compute_triangle_normals,
   compute_bb (mesh.cpp:39-58) and `new jtk::qbvh(triangles, vertices)`.
   vertices: n_vertices x 3 float; triangles: n_triangles x 3 uint32 (host or
   device). The arrays are copied; the caller keeps them. */
int j3dg_mesh_build(j3dg_ctx* ctx, const float* vertices, uint32_t n_vertices, const uint32_t* triangles,
                    uint32_t n_triangles, const j3dg_build_opts* opts, j3dg_mesh** out);
/* No reference counterpart (add_object builds one mesh at a time): many
   meshes built at once, up to max_concurrent (0: 8) at a time, each on its
   own stream from its own host thread, so that one build's host round
   trips overlap the others' device work. opts: one per mesh, or NULL for
   the defaults. On failure every mesh of the call is destroyed and out[]
   holds NULLs. The context stream's earlier work completes first. */
typedef struct j3dg_mesh_source {
  const float* vertices; /* n_vertices x 3, host or device */
  uint32_t n_vertices;
  uint32_t n_triangles;
  const uint32_t* triangles; /* n_triangles x 3, host or device */
} j3dg_mesh_source;
int j3dg_mesh_build_many(j3dg_ctx* ctx, uint32_t n, const j3dg_mesh_source* sources, const j3dg_build_opts* opts,
                         uint32_t max_concurrent, j3dg_mesh** out);
int j3dg_mesh_destroy(j3dg_mesh* mesh);
int j3dg_mesh_get_info(const j3dg_mesh* mesh, j3dg_mesh_info* info);
/* Copies the first `bytes` of the mesh's BVH node array (n_nodes nodes of
   16, 32 or 64 floats by the width: planes [6][W], refs [W], padding) to
   host memory; for tools that export or check a tree. No reference
   counterpart. */
int j3dg_mesh_get_nodes(const j3dg_mesh* mesh, void* dst, uint64_t bytes);
/* scene_object::triangle_normals (scene.h:14): n_triangles x 3 floats out. */
int j3dg_mesh_get_triangle_normals(const j3dg_mesh* mesh, float* normals);
/* Optional per-mesh data for the textured / vertex-colour branches of
   canvas.cpp:803-834 (mesh.h:28-30). colors: n_vertices x 3 float in [0,1];
   uv: n_triangles x 3 x 2 float; texture: w x h RGBA8. */
int j3dg_mesh_set_vertex_colors(j3dg_mesh* mesh, const float* colors);
int j3dg_mesh_set_uv(j3dg_mesh* mesh, const float* uv);
int j3dg_mesh_set_texture(j3dg_mesh* mesh, const uint32_t* texture, uint32_t w, uint32_t h);

/* ------------------------------------------------------------ ray queries */

/* qbvh_two_level_with_transformations(bvhs, object_cs, n) +
   find_closest_triangle (canvas.cpp:762,786) over a batch of rays. */
int j3dg_find_closest(j3dg_ctx* ctx, const j3dg_instance* objects, uint32_t n_objects, const j3dg_ray* rays,
                      uint32_t n_rays, j3dg_hit* hits);
/* Occlusion form of the same query (canvas.cpp:854-856 only reads found). */
int j3dg_find_any(j3dg_ctx* ctx, const j3dg_instance* objects, uint32_t n_objects, const j3dg_ray* rays,
                  uint32_t n_rays, j3dg_hit* hits);

/* jtk find_all_triangles (vox.cpp:333) on one mesh: for each ray, every
   accepted triangle with t < t_far, sorted by (t, triangle id); the first
   `cap` go to hits[ray * cap ...], the full count to counts[ray]. */
int j3dg_find_all(j3dg_ctx* ctx, const j3dg_mesh* mesh, const j3dg_ray* rays, uint32_t n_rays, uint32_t cap,
                  j3dg_hit* hits, uint32_t* counts);

/* The voxel grid of write_vox (vox.cpp:284-380): dims from max_dim and the
   mesh bbox (vox.cpp:292-299), three axis-aligned sweeps of all-hits rays,
   each hit's voxel (index x + (y + z dim1) dim0) set to its colour index
   (vox.cpp:154-173; texture if uv and texture are set, else vertex colours,
   else white). Sweep, ray and hit order are fixed and the last write wins.
   With voxels == NULL only dims are returned; otherwise capacity must hold
   dims[0] * dims[1] * dims[2] bytes. max_dim <= 1024. */
int j3dg_voxelize(j3dg_ctx* ctx, const j3dg_mesh* mesh, uint32_t max_dim, uint32_t dims[3], uint8_t* voxels,
                  uint64_t capacity);

/* No counterpart in the reference. The same voxel grid as j3dg_voxelize,
   for callers that must not allocate device memory while they run: a
   viewer or service that reserved its memory budget up front (for instance
   a render server sized to its HBM cap, or a host whose device memory is
   owned by another allocator), or a caller that cannot afford the device
   synchronisation an allocation may cause in the middle of its work. The
   call allocates nothing: its scratch (a 4-byte key and 1 staging byte per
   voxel) is a fixed array inside the library, J3DG_NOALLOC_MAX_VOXELS voxels
   (2,097,152, e.g. 128 x 128 x 128) on every GPU that loads the library,
   kept until the process exits. Grids larger than that are rejected with
   J3DG_ERR_INVALID_ARGUMENT and a message naming both sizes. The caller
   passes the mesh and the output (device or host memory, capacity >= the
   dims product). j3dg_ctx_create looks the scratch's device address up
   (cudaGetSymbolAddress, with the context's device current), which also
   loads the array, so this function never allocates it; under CUDA's lazy
   loading the driver may still load the kernels' code at their first
   launch (CUDA_MODULE_LOADING=EAGER loads it at start). All calls
   share the one scratch array, which keeps the last call's contents (the
   call clears what must start at zero): calls that overlap on the GPU,
   from two contexts or two threads, race on it. */
#define J3DG_NOALLOC_MAX_VOXELS (1u << 21)
int j3dg_voxelize_noalloc(j3dg_ctx* ctx, const j3dg_mesh* mesh, uint32_t max_dim, uint32_t dims[3],
                          uint8_t* voxels, uint64_t capacity);

/* ----------------------------------------------------------- mesh ingest --
   mesh.cpp:76-176 read_from_file and pc.cpp:32-110 pick a reader from the
   file extension (io.h:8-43; PLY/STL/OFF through jtk, OBJ/XYZ/PTS in
   io.cpp:292-713) and hand host vectors to add_object. Here the file goes
   to the device in pinned chunks and binary bodies (PLY, STL) are decoded
   there; text formats are parsed on host threads and uploaded. The decoded
   arrays stay on the device and feed j3dg_mesh_build_geometry (which
   computes the bbox and normals on the device, scene.cpp:20) without a host
   round trip. TRC (trico) is not supported: its format has no
   specification in the reference. */

typedef struct j3dg_geometry j3dg_geometry;

typedef enum j3dg_file_format {
  J3DG_FORMAT_AUTO = 0, /* from the extension (read_file) or the content (read_memory) */
  J3DG_FORMAT_PLY = 1,
  J3DG_FORMAT_STL = 2,
  J3DG_FORMAT_OBJ = 3,
  J3DG_FORMAT_OFF = 4,
  J3DG_FORMAT_XYZ = 5,
  J3DG_FORMAT_PTS = 6
} j3dg_file_format;

typedef struct j3dg_geometry_info {
  uint64_t n_vertices;
  uint64_t n_triangles;
  uint32_t format;      /* j3dg_file_format that was read */
  uint32_t encoding;    /* 0 text, 1 binary little endian, 2 binary big endian */
  uint32_t has_colors;  /* per-vertex 0xff000000 | b << 16 | g << 8 | r */
  uint32_t has_normals; /* per-vertex normals (3 floats) */
  uint32_t has_uv;      /* per-triangle texture coordinates (6 floats) */
  uint32_t device_decoded; /* 1 when the body was decoded by device kernels */
  uint64_t file_bytes;
  float read_ms;        /* file -> host (pinned chunks) */
  float decode_ms;      /* host parse + upload + device decode after the read */
  float total_ms;       /* wall time of the whole call */
  float reserved;
} j3dg_geometry_info;

/* read_from_file's reader dispatch (mesh.cpp:76-176, pc.cpp:32-110) into
   device arrays. format = J3DG_FORMAT_AUTO picks the reader from the
   extension as mesh.cpp:88-92 does. */
int j3dg_geometry_read_file(j3dg_ctx* ctx, const char* path, int format, j3dg_geometry** out);
/* The same readers over bytes already in memory (format AUTO: PLY/OFF by
   their magic, "solid" or the binary size rule for STL, else an error). */
int j3dg_geometry_read_memory(j3dg_ctx* ctx, const void* bytes, uint64_t n_bytes, int format,
                              j3dg_geometry** out);
int j3dg_geometry_get_info(const j3dg_geometry* g, j3dg_geometry_info* info);
/* Copies the arrays out (host or device pointers; NULL skips an array):
   vertices V x 3, triangles T x 3, colors V, normals V x 3, uv T x 6. */
int j3dg_geometry_get_arrays(const j3dg_geometry* g, float* vertices, uint32_t* triangles, uint32_t* colors,
                             float* normals, float* uv);
int j3dg_geometry_destroy(j3dg_geometry* g);
/* add_object's mesh (scene.cpp:17-26) from decoded geometry: the BVH build
   of j3dg_mesh_build on the device arrays, vertex colours converted as
   mesh.cpp:216-228 does, uv kept, and mesh.cpp:172-173's 512 x 512 dummy
   checker texture when there are uv but no texture. */
int j3dg_mesh_build_geometry(j3dg_ctx* ctx, const j3dg_geometry* g, const j3dg_build_opts* opts, j3dg_mesh** out);

/* ------------------------------------------------------------ point clouds --
   pc.h:23-31 / scene_pointcloud (scene.h:27-38): vertices (+ packed RGBA8
   colours) resident on the device, drawn after the mesh frame by
   canvas::render_pointclouds_on_image (canvas.cpp:952-1030). */

typedef struct j3dg_pointcloud j3dg_pointcloud;

typedef struct j3dg_pointcloud_instance {
  const j3dg_pointcloud* pointcloud;
  float cs[16];     /* pc::cs, column-major */
  uint32_t db_id;
  uint32_t reserved;
} j3dg_pointcloud_instance;

/* Uploads n points (vertices n x 3, colors n or NULL; host or device
   pointers) and computes their bbox (compute_bb, mesh.cpp:39-58). */
int j3dg_pointcloud_create(j3dg_ctx* ctx, const float* vertices, uint64_t n, const uint32_t* colors,
                           j3dg_pointcloud** out);
/* The vertices (and colours) of decoded geometry as a point cloud, on the
   device (pc.cpp:32-110 reads point clouds with the mesh readers). */
int j3dg_pointcloud_from_geometry(j3dg_ctx* ctx, const j3dg_geometry* g, j3dg_pointcloud** out);
int j3dg_pointcloud_destroy(j3dg_pointcloud* pc);
int j3dg_pointcloud_get_bounds(const j3dg_pointcloud* pc, float min_bb[3], float max_bb[3]);
/* scene.cpp:50-89 prepare_scene over mesh objects and point clouds. */
int j3dg_prepare_scene_pointclouds(const j3dg_instance* objects, uint32_t n, const j3dg_pointcloud_instance* pcs,
                                   uint32_t n_pcs, float min_bb[3], float max_bb[3], float* diagonal);
/* canvas::render_pointclouds_on_image (canvas.cpp:952-1030) after a frame:
   a depth buffer of 1/depth from the G-buffer (0 where db_id is 0), then
   each cloud in order: every point projected through its cs, the scene's
   coordinate_system_inv and the canvas projection onto the pixel whose
   primary ray passes nearest to it, kept where its 1/depth is strictly
   greater (equal depths: the smaller vertex id); the pixel's object_id,
   depth (1 / (1/depth)) and db_id are set and its image colour becomes the
   point's colour (white without colours or in one_bit mode). Points at or
   before the near clipping plane are not drawn. The shading of points by
   their normals is not done (jtk/render.h, which does it, is absent). */
int j3dg_canvas_render_pointclouds(j3dg_canvas* c, const j3dg_scene* s, const j3dg_pointcloud_instance* pcs,
                                   uint32_t n_pcs);

/* ---------------------------------------------------------------- matcaps */

/* matcap.h:18-24: a w x h RGBA8 texture plus its cavity colour, uploaded once. */
int j3dg_matcap_create(j3dg_ctx* ctx, const uint32_t* pixels, uint32_t w, uint32_t h, uint32_t cavity_clr,
                       j3dg_matcap** out);
int j3dg_matcap_destroy(j3dg_matcap* m);

/* ----------------------------------------------------------------- canvas */

/* canvas::canvas(w, h) + resize (canvas.cpp:102-134): device G-buffer, image
   and background; default camera (camera.cpp:5-16) and its projection.
   The buffers come from a stream-ordered pool of the context: create,
   resize and destroy are ordered on the context stream (after a pending
   download) and do not wait for the device. */
int j3dg_canvas_create(j3dg_ctx* ctx, uint32_t w, uint32_t h, j3dg_canvas** out);
int j3dg_canvas_destroy(j3dg_canvas* c);
int j3dg_canvas_resize(j3dg_canvas* c, uint32_t w, uint32_t h);
/* j3d keeps canvas::_camera at make_default_camera(); this lets a caller set
   another film-gate camera (e.g. a 60 degree vertical field of view). */
int j3dg_canvas_set_camera(j3dg_canvas* c, const j3dg_camera* cam);
int j3dg_canvas_get_projection(const j3dg_canvas* c, float projection[16], float projection_inv[16]);
/* canvas::set_background_color (canvas.cpp:136-139 -> fill_background 55-78) */
int j3dg_canvas_set_background_color(j3dg_canvas* c, uint32_t clr_top, uint32_t clr_bottom);
/* canvas::update_settings (canvas.h:56-59) */
int j3dg_canvas_update_settings(j3dg_canvas* c, const j3dg_canvas_settings* s);
/* canvas::update_canvas(x0, y0, x1, y1, scene) (canvas.cpp:672-874):
   G-buffer only, for the clamped rectangle. */
int j3dg_canvas_update_canvas(j3dg_canvas* c, int x0, int y0, int x1, int y1, const j3dg_scene* s);
/* canvas::render_scene(const scene*) (canvas.cpp:893-898): image <- background,
   then update_canvas over the whole canvas (s == NULL clears the G-buffer ids). */
int j3dg_canvas_render_scene(j3dg_canvas* c, const j3dg_scene* s);
/* canvas::canvas_to_image(matcap) (canvas.cpp:396-399, 582-670): shades the
   canvas's G-buffer into its image; background pixels are left as they are. */
int j3dg_canvas_to_image(j3dg_canvas* c, const j3dg_matcap* m);
/* canvas_to_image(const image<pixel>&, matcap) (canvas.cpp:582): shades a
   caller G-buffer (w x h records, host or device) into the canvas image. */
int j3dg_canvas_to_image_from(j3dg_canvas* c, const j3dg_pixel* pixels, const j3dg_matcap* m);
/* view::render_scene (view.cpp:421-430) fused: background, update_canvas,
   canvas_to_image in one pass (one kernel for plain shading, two for the
   neighbour-reading modes). Asynchronous on the context stream. */
int j3dg_canvas_render_frame(j3dg_canvas* c, const j3dg_scene* s, const j3dg_matcap* m);
/* canvas::get_pixels / get_image (canvas.h:81-87): copy out (host or device
   destination, w x h elements). Synchronous; reports device status. */
int j3dg_canvas_get_pixels(j3dg_canvas* c, j3dg_pixel* dst);
int j3dg_canvas_get_image(j3dg_canvas* c, uint32_t* dst);
/* No reference counterpart. Starts copying the G-buffer and/or the image
   (either may be NULL; host memory should be pinned for the copy to run
   asynchronously) on the context's copy stream, after the work already
   queued on the canvas, and returns at once; the context stream keeps
   rendering (another canvas, typically) while the copy runs. Calls that
   write this canvas later wait on the device for the copy. */
int j3dg_canvas_download_async(j3dg_canvas* c, j3dg_pixel* pixels, uint32_t* image);
/* Blocks the host until the canvas's last download_async has completed
   (device status is reported by j3dg_ctx_synchronize). */
int j3dg_canvas_download_wait(j3dg_canvas* c);
/* Upload a caller G-buffer into the canvas (w x h records). */
int j3dg_canvas_set_pixels(j3dg_canvas* c, const j3dg_pixel* src);
/* Counts the canvas's G-buffer records with a hit and with the shadow bit
   (no reference counterpart; for ray accounting without a copy-out). */
int j3dg_canvas_count_hits(j3dg_canvas* c, uint64_t* hits, uint64_t* shadowed);
/* The primary-hit method of the canvas's last frame: J3DG_PRIMARY_TRACE or
   J3DG_PRIMARY_RASTER (a rasterised frame whose list of large triangles
   overflowed is traced on the device and still reports RASTER). */
int j3dg_canvas_last_primary(const j3dg_canvas* c);
/* Device pointers of the canvas buffers (valid until resize/destroy). */
int j3dg_canvas_device_buffers(j3dg_canvas* c, j3dg_pixel** pixels, uint32_t** image, uint32_t** background);

/* ---------------------------------------------------------------- batches
   No reference counterpart (j3d renders one canvas per call): many frames,
   each its own canvas (any resolution), scene and matcap, rendered by one
   persistent launch over all their pixels, so uneven frames share the GPU
   with a single tail. Shading modes other than plain add one shading pass
   per such frame. Canvases of one batch must be distinct. */
typedef struct j3dg_frame {
  j3dg_canvas* canvas;
  const j3dg_scene* scene;
  const j3dg_matcap* matcap;
} j3dg_frame;

typedef struct j3dg_batch j3dg_batch;

/* One-shot: packs the frames' parameters, one upload, one launch. Async. */
int j3dg_render_batch(j3dg_ctx* ctx, const j3dg_frame* frames, uint32_t n);
/* Block shape of batched launches (64, 128 or 256 threads; default 128),
   for an autotuner. Applies to batches created or rendered afterwards. */
int j3dg_ctx_set_batch_block(j3dg_ctx* ctx, int threads);
/* A fixed set of frames captured once as a CUDA graph (parameter upload,
   counter reset, the persistent launch, shading passes); replayed by
   j3dg_batch_launch. */
int j3dg_batch_create(j3dg_ctx* ctx, const j3dg_frame* frames, uint32_t n, j3dg_batch** out);
/* Replaces frame i's scene (camera pose, objects) for the next launches; the
   number of objects must not exceed the one given at creation. Waits for
   the previous launch of this batch. */
/* As j3dg_batch_create, with flags. J3DG_BATCH_REBUILD: every launch first
   rebuilds the BVH of every mesh of the batch's scenes from the mesh's kept
   vertices and triangles (all built with J3DG_BUILD_REBUILDABLE, by the
   builder each was built with), then renders the frames: builds and frames are one graph launch
   (builds of up to 8 meshes at a time on forked capture streams, each
   build's level loops device-driven). A rebuild gives the mesh the same tree
   as its first build. Other work must not use these meshes while a launch
   runs. No reference counterpart (the reference builds on the host, one
   mesh at a time). */
#define J3DG_BATCH_REBUILD 0x1u
int j3dg_batch_create2(j3dg_ctx* ctx, const j3dg_frame* frames, uint32_t n, uint32_t flags, j3dg_batch** out);
int j3dg_batch_set_scene(j3dg_batch* b, uint32_t i, const j3dg_scene* scene);
int j3dg_batch_launch(j3dg_batch* b);
int j3dg_batch_destroy(j3dg_batch* b);

/* ----------------------------------------------------------- learned tmax
   No reference counterpart. A network predicts, from a ray, which of the
   mesh's clusters (the BVH subtrees at cluster_depth: at most 4096, Morton-
   ordered ranges of triangles) holds its closest hit: 16-band Fourier
   features of origin and direction, four 128-wide GELU layers, 4096 logits;
   bf16 weights, fp32 accumulation on the tensor cores; trained on the GPU
   (softmax cross-entropy, Adam) on rays traced by the plain method. A
   learned query traverses its two predicted clusters first and seeds the
   exact traversal with their best hit: results equal j3dg_find_closest's. */
typedef struct j3dg_learned j3dg_learned;
typedef struct j3dg_learned_opts {
  uint32_t cluster_depth; /* BVH depth of the clusters, 1..6 (default 6) */
  uint32_t batch;         /* training batch, a multiple of 128 (default 16384) */
  float lr;               /* Adam learning rate (default 2e-3) */
  uint32_t reserved;
  uint64_t seed;          /* weights and training rays */
} j3dg_learned_opts;

int j3dg_learned_create(j3dg_ctx* ctx, const j3dg_mesh* mesh, const j3dg_learned_opts* opts, j3dg_learned** out);
int j3dg_learned_destroy(j3dg_learned* l);
int j3dg_learned_info(const j3dg_learned* l, uint32_t* n_clusters, uint64_t* n_params);
/* Trains on n_rays rays from cameras at radius r0..r1 around the mesh
   (generated and traced on the GPU); reports the last batch's loss and
   top-1 accuracy over its hit rays, and the wall time. */
int j3dg_learned_train(j3dg_learned* l, uint64_t n_rays, float r0, float r1, float* final_loss, float* accuracy,
                       float* seconds);
/* The two most likely clusters of each ray (n x 2, host or device), by the
   fused inference kernel (tcgen05, activations and logits kept on chip). */
int j3dg_learned_predict(j3dg_learned* l, const j3dg_ray* rays, uint32_t n, uint32_t* top2);
/* The same with a choice of implementation: 1 the fused tcgen05 kernel, 0 the
   layer-by-layer tcgen05 GEMMs of training (fused epilogues) plus a top-2
   pass over the logits. Both round activations to bf16 at the same points;
   the fp32 accumulation order differs, so near-ties may rank differently. */
int j3dg_learned_predict_impl(j3dg_learned* l, const j3dg_ray* rays, uint32_t n, uint32_t* top2, int impl);
/* Closest hits through the learned tmax (host or device arrays). */
int j3dg_learned_find_closest(j3dg_learned* l, const j3dg_ray* rays, uint32_t n, j3dg_hit* hits);
/* The same, reporting what each phase cost: stats = {node visits and
   triangle tests of the two predicted clusters, node visits and triangle
   tests of the exact traversal seeded with their best hit}. The exact
   phase never visits more nodes than the plain traversal of the same rays
   (its best-so-far is never larger at any step); the difference is what
   the network's prediction saves it. */
int j3dg_learned_find_closest_stats(j3dg_learned* l, const j3dg_ray* rays, uint32_t n, j3dg_hit* hits,
                                    uint64_t stats[4]);
/* Parameters (fp32 master copy, layout W1 b1 ... W5 b5, W row-major [in][out]). */
int j3dg_learned_get_params(j3dg_learned* l, float* out);
int j3dg_learned_set_params(j3dg_learned* l, const float* in);
/* Mean loss and gradients of a batch of features (B x 256 fp32, B a
   multiple of 128) and labels (-1 = no hit), for gradient checks. */
int j3dg_learned_loss_grad(j3dg_learned* l, const float* features, const int32_t* labels, uint32_t B, float* loss,
                           float* grads);
/* A whole canvas frame (canvas::render_scene's update_canvas + canvas_to_image,
   canvas.cpp:677-874, 582-670) whose primary hits come from the learned
   path: the frame's primary rays go through the network and the exact
   traversal it seeds, then the hit records, shadow rays and shading are the
   plain path's. The G-buffer and image equal j3dg_canvas_render_frame's. The
   scene must hold the network's mesh as its only object, with the identity
   transform (the network works in the mesh's space). */
int j3dg_learned_render_frame(j3dg_learned* l, j3dg_canvas* canvas, const j3dg_scene* scene,
                              const j3dg_matcap* matcap);
/* Checkpoint (header + fp32 parameters). */
int j3dg_learned_save(j3dg_learned* l, const char* path);
int j3dg_learned_load(j3dg_learned* l, const char* path);

/* Diagnostics (no reference counterpart): the network's bf16 tensor-core
   GEMM (tcgen05, accumulator in tensor memory; M, N % 128, K % 64),
   C[M x N] fp32 = A[M x K] . Bt[N x K]^T on device arrays (A, Bt bf16
   row-major). impl 1: one CTA per output tile; impl 0: split-K, CTAs over
   K ranges adding into C with atomics (the weight gradients' form); impl 2:
   the kernel with its MMAs withheld, so that its bounded mbarrier wait runs
   out (~0.25 s): the call must return J3DG_ERR_DEVICE_STATUS with
   J3DG_DEV_VISIT_CAP raised, and the context stays usable. Synchronous. */
int j3dg_gemm_bf16(j3dg_ctx* ctx, const void* A, const void* Bt, float* C, uint32_t M, uint32_t N, uint32_t K,
                   int impl);

/* ---------------------------------------------------- host-side j3d math --
   Plain C++ (no GPU), the same fp32 operation order as the device code. */

/* camera.cpp:5-16 */
void j3dg_make_default_camera(j3dg_camera* c);
/* camera.cpp:32-73 */
void j3dg_make_projection_matrix(const j3dg_camera* c, int w, int h, float out[16]);
/* camera.cpp:26-30 */
void j3dg_invert_projection_matrix(const float in[16], float out[16]);
/* jtk invert_orthonormal (canvas.cpp:734, scene.cpp:109) */
void j3dg_invert_orthonormal(const float in[16], float out[16]);
/* scene.cpp:50-89 prepare_scene over the mesh objects */
int j3dg_prepare_scene(const j3dg_instance* objects, uint32_t n, float min_bb[3], float max_bb[3],
                       float* diagonal);
/* scene.cpp:91-110 unzoom */
void j3dg_unzoom(const float min_bb[3], const float max_bb[3], float diagonal, float cs[16], float cs_inv[16],
                 float pivot[3]);
/* pixel.cpp:6-25 get_closest_vertex: the vertex of the pixel's triangle
   nearest to its hit point (vertices: V x 3 float, triangles: T x 3). */
uint32_t j3dg_get_closest_vertex(const j3dg_pixel* p, const float* vertices, const uint32_t* triangles);
/* view.cpp:439-459 get_world_position (mesh branch): the hit point of the
   pixel in world space through the object's cs. */
void j3dg_get_world_position(const j3dg_pixel* p, const float* vertices, const uint32_t* triangles,
                             const float cs[16], float out[3]);
/* matcap.cpp:9-268: type 0 red wax, 1 gray, 2 brown, 3 sketch; pixels must
   hold 512 x 512. */
int j3dg_make_matcap(int type, uint32_t* pixels, uint32_t* w, uint32_t* h, uint32_t* cavity_clr);
/* canvas.cpp:55-78 */
void j3dg_fill_background(uint32_t* bg, uint32_t w, uint32_t h, uint32_t clr_top, uint32_t clr_bottom);

/* ------------------------------------------------- synthetic workloads ----
   No reference counterpart: seeded stand-ins for the meshes j3d loads from
   files (the mesh readers are not on this path). Deterministic on every
   host: own PRNG and own sine, no libm transcendental calls. */

/* Icosphere subdivided `level` times; radius 1 + amp * sum_k a_k sin(f_k (d.u_k) + phi_k)
   with 8 seeded terms. V = 10*4^level + 2, T = 20*4^level. */
int j3dg_synth_icosphere(uint32_t level, uint64_t seed, float amp, float* vertices, uint32_t* triangles);
/* Torus R, r on an nu x nv periodic grid (V = nu*nv, T = 2*nu*nv); radial
   displacement amp * sum of 16 seeded periodic sinusoids. */
int j3dg_synth_torus(uint32_t nu, uint32_t nv, float R, float r, uint64_t seed, float amp, float* vertices,
                     uint32_t* triangles);
/* Camera-to-world look-at poses: n directions uniform on the sphere, radius
   uniform in [r0, r1], looking at target. cs: n x 16 floats. */
int j3dg_synth_cameras(uint32_t n, uint64_t seed, float r0, float r1, const float target[3], float* cs);
/* Camera focal length (mm) giving a vertical field of view (degrees) for the
   default film gate (camera.cpp:9-10). */
float j3dg_focal_for_vfov(float vfov_deg, float film_aperture_height_inch);

#ifdef __cplusplus
}
#endif

#endif /* J3DG_H */
