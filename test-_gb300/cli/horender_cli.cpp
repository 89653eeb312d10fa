// Command-line renderer mirroring the reference's main program
// (FEM-AABB/main.cu:23-598): load a scene file (.xml with its .fld, or .vtu),
// frame the camera on the scene's box, path-trace 640x360 at 10 samples and
// depth 5, write output.ppm and, from the opposite side, output_back.ppm.
//
// Differences from the reference: the sample seed is an argument (the
// reference seeds with the time, so its images are not reproducible); the
// camera is framed on the box over the elements' and primitives' sampled
// boxes (the reference takes the hexahedra's loader boxes and the other
// primitives' vertices); sizes, samples, depth, isovalue and output names
// can be changed by flags; a missing input file is an error rather than a
// silent exit.
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "horender.hpp"

namespace {

struct Args {
  std::string scene, fld, out = "output";
  int width = 640, height = 360, spp = 10, depth = 5, device = 0, mode = HO_MODE_BATCHED;
  float iso = 0.0f;  // the reference's Scene::iso_value default: isosurface off
  uint64_t seed = 1;
  bool png = false, back = true;
};

void usage(FILE* f) {
  std::fprintf(f,
               "usage: horender_cli [scene.xml [scene.fld] | scene.vtu] [options]\n"
               "  --width W --height H   image size (640 x 360)\n"
               "  --spp N                samples per pixel (10)\n"
               "  --depth N              maximum path depth (5)\n"
               "  --iso V                isovalue; 0 turns the isosurface off (0)\n"
               "  --seed S               sample seed (1)\n"
               "  --mode plain|batched   intersection engine (batched)\n"
               "  --out PREFIX           output PREFIX.ppm and PREFIX_back.ppm (output)\n"
               "  --png                  also write PREFIX.png and PREFIX_back.png\n"
               "  --no-back              skip the view from the opposite side\n"
               "  --device N             CUDA device (0)\n"
               "Without a scene argument, Hex_CurvedFace.xml in the working directory is loaded.\n");
}

bool file_exists(const std::string& p) {
  FILE* f = std::fopen(p.c_str(), "rb");
  if (!f) return false;
  std::fclose(f);
  return true;
}

std::string lower_ext(const std::string& p) {
  const auto dot = p.find_last_of('.');
  if (dot == std::string::npos) return "";
  std::string e = p.substr(dot);
  for (char& c : e) c = static_cast<char>(std::tolower(static_cast<unsigned char>(c)));
  return e;
}

// Returns 0 to go on, 1 for --help, 2 on a bad argument.
int parse(int argc, char** argv, Args& a) {
  std::vector<std::string> pos;
  for (int i = 1; i < argc; ++i) {
    const std::string s = argv[i];
    auto need = [&](const char* name) -> const char* {
      if (i + 1 >= argc) {
        std::fprintf(stderr, "%s needs a value\n", name);
        return nullptr;
      }
      return argv[++i];
    };
    auto as_int = [&](const char* v, int& out) {
      char* end = nullptr;
      const long x = v ? std::strtol(v, &end, 10) : 0;
      if (!v || *end || x <= 0 || x > (1 << 20)) return false;
      out = static_cast<int>(x);
      return true;
    };
    if (s == "--help" || s == "-h") return 1;
    if (s == "--width" || s == "--height" || s == "--spp" || s == "--depth") {
      int* dst = s == "--width" ? &a.width : s == "--height" ? &a.height : s == "--spp" ? &a.spp : &a.depth;
      if (!as_int(need(s.c_str()), *dst)) {
        std::fprintf(stderr, "%s: expected a positive integer\n", s.c_str());
        return 2;
      }
    } else if (s == "--device") {
      const char* v = need("--device");
      if (!v) return 2;
      a.device = std::atoi(v);
    } else if (s == "--iso") {
      const char* v = need("--iso");
      if (!v) return 2;
      a.iso = std::strtof(v, nullptr);
    } else if (s == "--seed") {
      const char* v = need("--seed");
      if (!v) return 2;
      a.seed = std::strtoull(v, nullptr, 10);
    } else if (s == "--mode") {
      const char* v = need("--mode");
      if (!v) return 2;
      const std::string m = v;
      if (m == "plain") a.mode = HO_MODE_PLAIN;
      else if (m == "batched") a.mode = HO_MODE_BATCHED;
      else {
        std::fprintf(stderr, "--mode: plain or batched\n");
        return 2;
      }
    } else if (s == "--out") {
      const char* v = need("--out");
      if (!v) return 2;
      a.out = v;
    } else if (s == "--png") {
      a.png = true;
    } else if (s == "--no-back") {
      a.back = false;
    } else if (!s.empty() && s[0] == '-') {
      std::fprintf(stderr, "unknown option %s\n", s.c_str());
      return 2;
    } else {
      pos.push_back(s);
    }
  }
  if (pos.size() > 2) {
    std::fprintf(stderr, "too many scene arguments\n");
    return 2;
  }
  a.scene = pos.empty() ? "Hex_CurvedFace.xml" : pos[0];
  if (pos.size() == 2) a.fld = pos[1];
  return 0;
}

void write(const std::vector<uint8_t>& rgb, const Args& a, const std::string& name) {
  horender::Scene::save_ppm(rgb, a.width, a.height, name + ".ppm");
  std::printf("Image saved as %s.ppm\n", name.c_str());
  if (a.png) {
    horender::Scene::save_png(rgb, a.width, a.height, name + ".png");
    std::printf("Image saved as %s.png\n", name.c_str());
  }
}

}  // namespace

int main(int argc, char** argv) {
  Args a;
  const int pr = parse(argc, argv, a);
  if (pr == 1) {
    usage(stdout);
    return 0;
  }
  if (pr == 2) {
    usage(stderr);
    return 2;
  }
  const std::string ext = lower_ext(a.scene);
  std::string xml = a.scene, fld = a.fld;
  if (ext == ".xml" || ext == ".fld") {
    // the pair: an explicit second argument, else the sibling with the same stem
    const std::string stem = a.scene.substr(0, a.scene.size() - ext.size());
    if (ext == ".fld") {
      xml = stem + ".xml";
      if (fld.empty()) fld = a.scene;
    } else if (fld.empty()) {
      fld = stem + ".fld";
    }
  } else if (ext != ".vtu") {
    std::fprintf(stderr, "unsupported scene file %s (expected .xml, .fld or .vtu)\n", a.scene.c_str());
    return 2;
  }
  if (!file_exists(xml)) {
    std::fprintf(stderr, "cannot read %s\n", xml.c_str());
    return 1;
  }
  try {
    horender::Scene scene(a.device);
    std::printf("Loading scene from file: %s\n", a.scene.c_str());
    if (ext == ".vtu") scene.load_vtu(xml);
    else scene.load_xml_fld(xml, file_exists(fld) ? fld : std::string());
    scene.build_bvh();
    scene.set_mode(a.mode);
    float lo[3], hi[3];
    if (!scene.bounds(lo, hi)) {
      std::fprintf(stderr, "[Error] No geometry loaded.\n");
      return 1;
    }
    // camera framing of main.cu:255-278: look at the box centre from
    // centre + (2.5, -2.5, -2.0) * largest extent, vfov 20 degrees
    float c[3], ext3 = 0.0f;
    for (int k = 0; k < 3; ++k) {
      c[k] = 0.5f * (lo[k] + hi[k]);
      ext3 = std::fmax(ext3, hi[k] - lo[k]);
    }
    if (ext3 <= 0.0f) ext3 = 1.0f;
    std::printf("Model Bounds: Min(%g,%g,%g) Max(%g,%g,%g)\n", lo[0], lo[1], lo[2], hi[0], hi[1], hi[2]);
    const float from[3] = {c[0] + 2.5f * ext3, c[1] - 2.5f * ext3, c[2] - 2.0f * ext3};
    const ho_camera cam = horender::make_camera(from, c, 20.0f);
    std::printf("Camera: lookfrom %.9g %.9g %.9g lookat %.9g %.9g %.9g\n", from[0], from[1], from[2], c[0], c[1],
                c[2]);
    std::printf("Rendering...\n");
    int64_t rays = 0;
    const std::vector<float> iso = {a.iso};
    write(scene.path_trace(cam, iso, a.width, a.height, a.spp, a.depth, a.seed, true, &rays), a, a.out);
    if (a.back) {
      // main.cu:549-576: the view from the opposite side of the centre
      const float back[3] = {2.0f * c[0] - from[0], 2.0f * c[1] - from[1], 2.0f * c[2] - from[2]};
      const ho_camera cam2 = horender::make_camera(back, c, 20.0f);
      write(scene.path_trace(cam2, iso, a.width, a.height, a.spp, a.depth, a.seed, true), a, a.out + "_back");
    }
    std::printf("Render complete: %lld ray queries in the first view.\n", static_cast<long long>(rays));
  } catch (const horender::Error& e) {
    std::fprintf(stderr, "error %d: %s\n", e.code(), e.what());
    return 1;
  }
  return 0;
}
