// Drives the C++ shim the way j3d loads files and draws a frame: each file
// through read_from_file + add_object (a mesh, or a point cloud when the file
// has no triangles), prepare_scene, unzoom, then view::render_scene
// (view.cpp:421-430): update_settings, render_scene, get_pixels,
// canvas_to_image, render_pointclouds_on_image. Writes G-buffer and image.
//   shim_files <w> <h> <pixels.bin> <image.bin> <file>...
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "j3dg_scene.hpp"

int main(int argc, char** argv) {
  if (argc < 6) {
    std::fprintf(stderr, "usage: shim_files w h pixels.bin image.bin file...\n");
    return 2;
  }
  const uint32_t w = (uint32_t)std::atoi(argv[1]), h = (uint32_t)std::atoi(argv[2]);
  try {
    j3dgpu::context ctx(0);
    j3dgpu::scene s;
    for (int k = 5; k < argc; ++k) j3dgpu::add_object_from_file(ctx, (uint32_t)(k - 4), s, argv[k]);
    j3dgpu::prepare_scene(s);
    j3dgpu::unzoom(s);
    j3dgpu::canvas cv(ctx, w, h);
    cv.set_background_color();
    j3dgpu::matcap mc(ctx, j3dgpu::matcap_type::MATCAP_TYPE_INTERNAL_REDWAX);
    j3dg_canvas_settings st{};
    st.shadow = 1;
    st.shading = 1;
    st.vertexcolors = 1;
    cv.update_settings(st);
    cv.render_scene(&s);
    std::vector<j3dgpu::pixel> pixels = cv.get_pixels();
    cv.canvas_to_image(pixels, mc);
    cv.render_pointclouds_on_image(&s);
    pixels = cv.get_pixels();
    std::vector<uint32_t> im = cv.get_image();
    FILE* f = std::fopen(argv[3], "wb");
    std::fwrite(pixels.data(), sizeof(j3dgpu::pixel), pixels.size(), f);
    std::fclose(f);
    f = std::fopen(argv[4], "wb");
    std::fwrite(im.data(), 4, im.size(), f);
    std::fclose(f);
  } catch (const j3dgpu::error& e) {
    std::fprintf(stderr, "j3dgpu error %d: %s\n", e.status, e.what());
    return 1;
  }
  return 0;
}
