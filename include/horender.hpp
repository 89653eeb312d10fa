// C++ facade over the C ABI in horender.h, shaped like the reference's Scene
// (FEM-AABB/raytracer.h:53-344): load -> build_bvh -> render. Header-only;
// every failure throws horender::Error with the library's status code and
// message. The C ABI itself never throws.
#pragma once

#include <cstdint>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "horender.h"

namespace horender {

class Error : public std::runtime_error {
 public:
  Error(int code, const std::string& what) : std::runtime_error(what), code_(code) {}
  int code() const { return code_; }

 private:
  int code_;
};

// Pinhole camera (FEM-AABB/raytracer.h:31-48, aperture 0).
inline ho_camera make_camera(const float lookfrom[3], const float lookat[3], float vfov_deg,
                             const float vup[3] = nullptr) {
  ho_camera c{};
  for (int a = 0; a < 3; ++a) {
    c.lookfrom[a] = lookfrom[a];
    c.lookat[a] = lookat[a];
    c.vup[a] = vup ? vup[a] : (a == 1 ? 1.0f : 0.0f);
  }
  c.vfov_deg = vfov_deg;
  c.focus_dist = 0.0f;
  return c;
}

class Scene {
 public:
  explicit Scene(int device = 0) {
    const int rc = ho_create(device, &h_);
    if (rc != HO_OK) throw Error(rc, "ho_create failed (device " + std::to_string(device) + ")");
  }
  ~Scene() { ho_destroy(h_); }
  Scene(const Scene&) = delete;
  Scene& operator=(const Scene&) = delete;
  Scene(Scene&& o) noexcept : h_(std::exchange(o.h_, nullptr)) {}
  Scene& operator=(Scene&& o) noexcept {
    if (this != &o) {
      ho_destroy(h_);
      h_ = std::exchange(o.h_, nullptr);
    }
    return *this;
  }

  ho_context* handle() const { return h_; }

  // load_xml_fld(xml, fld, scene) (FEM-AABB/xml_fld_loader.h:14-16)
  void load_xml_fld(const std::string& xml, const std::string& fld) {
    check(ho_load_xml_fld(h_, xml.c_str(), fld.c_str()), "load_xml_fld");
  }
  // load_vtu_file(path, scene) (FEM-AABB/vtu_loader.h:9)
  void load_vtu(const std::string& path) { check(ho_load_vtu(h_, path.c_str()), "load_vtu"); }
  // Scene::build_bvh() (FEM-AABB/raytracer.h:338-344)
  void build_bvh() { check(ho_build_bvh(h_), "build_bvh"); }

  void set_mode(int mode) { check(ho_set_mode(h_, mode), "set_mode"); }
  void set_option(int option, int64_t value) { check(ho_set_option(h_, option, value), "set_option"); }

  ho_scene_info info() const {
    ho_scene_info s{};
    check(ho_scene_info_get(h_, &s), "scene_info");
    return s;
  }
  ho_stats stats() const {
    ho_stats s{};
    check(ho_get_stats(h_, &s), "get_stats");
    return s;
  }

  // Box over every element and primitive after build_bvh (lo xyz, hi xyz);
  // false when the scene is empty.
  bool bounds(float lo[3], float hi[3]) const {
    const ho_scene_info s = info();
    bool any = false;
    auto grow = [&](const float* b) {
      for (int a = 0; a < 3; ++a) {
        lo[a] = any ? (b[a] < lo[a] ? b[a] : lo[a]) : b[a];
        hi[a] = any ? (b[3 + a] > hi[a] ? b[3 + a] : hi[a]) : b[3 + a];
      }
      any = true;
    };
    if (s.n_elem > 0) grow(s.bounds);
    const int64_t np = s.n_prisms + s.n_quads + s.n_tris;
    if (np > 0) {
      std::vector<float> boxes(static_cast<size_t>(np) * 6);
      check(ho_get_prim_boxes(h_, boxes.data()), "get_prim_boxes");
      for (int64_t i = 0; i < np; ++i) grow(boxes.data() + 6 * i);
    }
    return any;
  }

  // One primary ray per pixel centre, Lambert-shaded (8-bit RGB, rows as
  // the reference writes them); n_iso images back to back.
  std::vector<uint8_t> render(const ho_camera& cam, const std::vector<float>& iso, int width, int height,
                              bool iso_zero_disables = true) {
    std::vector<uint8_t> rgb(iso.size() * static_cast<size_t>(width) * height * 3);
    check(ho_render(h_, &cam, iso.data(), static_cast<int>(iso.size()), width, height, iso_zero_disables ? 1 : 0,
                    rgb.data(), nullptr),
          "render");
    return rgb;
  }

  // render_kernel at spp samples and max_depth bounces (FEM-AABB/raytracer.cu:410-476).
  std::vector<uint8_t> path_trace(const ho_camera& cam, const std::vector<float>& iso, int width, int height, int spp,
                                  int max_depth, uint64_t seed, bool iso_zero_disables = true,
                                  int64_t* rays_traced = nullptr) {
    std::vector<uint8_t> rgb(iso.size() * static_cast<size_t>(width) * height * 3);
    check(ho_path_trace(h_, &cam, iso.data(), static_cast<int>(iso.size()), width, height, spp, max_depth, seed,
                        iso_zero_disables ? 1 : 0, rgb.data(), rays_traced),
          "path_trace");
    return rgb;
  }

  // save_image_ppm (FEM-AABB/raytracer.cu:480-494), and the same as PNG.
  static void save_ppm(const std::vector<uint8_t>& rgb, int width, int height, const std::string& path,
                       size_t image = 0) {
    const int rc = ho_save_ppm(rgb.data() + image * static_cast<size_t>(width) * height * 3, width, height,
                               path.c_str());
    if (rc != HO_OK) throw Error(rc, "cannot write " + path);
  }
  static void save_png(const std::vector<uint8_t>& rgb, int width, int height, const std::string& path,
                       size_t image = 0) {
    const int rc = ho_save_png(rgb.data() + image * static_cast<size_t>(width) * height * 3, width, height,
                               path.c_str());
    if (rc != HO_OK) throw Error(rc, "cannot write " + path);
  }

 private:
  void check(int rc, const char* what) const {
    if (rc != HO_OK) throw Error(rc, std::string(what) + ": " + ho_last_error(h_));
  }
  ho_context* h_ = nullptr;
};

}  // namespace horender
