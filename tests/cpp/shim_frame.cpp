// Drives the C++ shim (include/j3dg_scene.hpp) the way j3d's view does:
// add_object, prepare_scene, unzoom, then view::render_scene's sequence
// (view.cpp:421-430): update_settings, render_scene, get_pixels,
// canvas_to_image(pixels, matcap). Writes the G-buffer and image to files.
//   shim_frame <level> <w> <h> <pose_z> <edges 0|1> <pixels.bin> <image.bin>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "j3dg_scene.hpp"

int main(int argc, char** argv) {
  if (argc != 8) {
    std::fprintf(stderr, "usage: shim_frame level w h pose_z edges pixels.bin image.bin\n");
    return 2;
  }
  const uint32_t level = (uint32_t)std::atoi(argv[1]);
  const uint32_t w = (uint32_t)std::atoi(argv[2]), h = (uint32_t)std::atoi(argv[3]);
  const float pose_z = (float)std::atof(argv[4]);
  const bool edges = std::atoi(argv[5]) != 0;
  try {
    const uint32_t nv = 10u * (1u << (2 * level)) + 2u, nt = 20u * (1u << (2 * level));
    std::vector<float> V(3 * (size_t)nv);
    std::vector<uint32_t> T(3 * (size_t)nt);
    j3dgpu::check(j3dg_synth_icosphere(level, 0x6A3D0000ull, 0.05f, V.data(), T.data()), nullptr, "synth");

    j3dgpu::context ctx(0);
    j3dgpu::scene s;
    j3dgpu::add_object(ctx, 1, s, V.data(), nv, T.data(), nt);
    j3dgpu::prepare_scene(s);
    j3dgpu::unzoom(s);
    // camera on +z at pose_z looking at the origin
    j3dgpu::identity(s.coordinate_system);
    s.coordinate_system[14] = pose_z;
    j3dg_invert_orthonormal(s.coordinate_system, s.coordinate_system_inv);

    j3dgpu::canvas cv(ctx, w, h);
    j3dg_camera cam;
    j3dg_make_default_camera(&cam);
    cam.focal_length = j3dg_focal_for_vfov(60.f, cam.film_aperture_height_inch);
    cv.set_camera(cam);
    cv.set_background_color();
    j3dgpu::matcap mc(ctx, j3dgpu::matcap_type::MATCAP_TYPE_INTERNAL_REDWAX);
    j3dg_canvas_settings st{};
    st.shadow = 1;
    st.edges = edges ? 1 : 0;
    st.shading = 1;
    cv.update_settings(st);
    cv.render_scene(&s);
    std::vector<j3dgpu::pixel> pixels = cv.get_pixels();
    cv.canvas_to_image(pixels, mc);
    std::vector<uint32_t> im = cv.get_image();
    FILE* f = std::fopen(argv[6], "wb");
    std::fwrite(pixels.data(), sizeof(j3dgpu::pixel), pixels.size(), f);
    std::fclose(f);
    f = std::fopen(argv[7], "wb");
    std::fwrite(im.data(), 4, im.size(), f);
    std::fclose(f);
  } catch (const j3dgpu::error& e) {
    std::fprintf(stderr, "j3dgpu error %d: %s\n", e.status, e.what());
    return 1;
  }
  return 0;
}
