// bin/render.rs on the GPU through geon.hpp: the same arguments and defaults
// (bin/render.rs:22-67), the same observers per metric (:94-129), the same
// printed lines (:85-88, :136-140), and a PNG of write_png's bytes
// (render.rs:169-183), tonemapped on the device. The PNG is written with stored
// (uncompressed) deflate blocks, so no compression library is needed.
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <sys/stat.h>
#include <vector>

#include "geon.hpp"
#include "rust_fmt.hpp"

using namespace rustfmt;

namespace {

uint32_t crc_table[256];
void crc_init() {
  for (uint32_t n = 0; n < 256; ++n) {
    uint32_t c = n;
    for (int k = 0; k < 8; ++k) c = (c & 1) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
    crc_table[n] = c;
  }
}
uint32_t crc(const uint8_t* p, size_t n, uint32_t c = 0xFFFFFFFFu) {
  for (size_t i = 0; i < n; ++i) c = crc_table[(c ^ p[i]) & 0xFF] ^ (c >> 8);
  return c;
}
void be32(std::vector<uint8_t>& v, uint32_t x) {
  for (int s = 24; s >= 0; s -= 8) v.push_back((uint8_t)(x >> s));
}
void chunk(std::vector<uint8_t>& out, const char* tag, const std::vector<uint8_t>& data) {
  be32(out, (uint32_t)data.size());
  std::vector<uint8_t> td(tag, tag + 4);
  td.insert(td.end(), data.begin(), data.end());
  out.insert(out.end(), td.begin(), td.end());
  be32(out, crc(td.data(), td.size()) ^ 0xFFFFFFFFu);
}

// 8-bit RGB PNG: filter byte 0 per row, zlib stream of stored blocks.
bool write_png(const std::string& path, const std::vector<uint8_t>& rgb, size_t w, size_t h) {
  crc_init();
  std::vector<uint8_t> raw;
  raw.reserve(h * (3 * w + 1));
  for (size_t j = 0; j < h; ++j) {
    raw.push_back(0);
    raw.insert(raw.end(), rgb.begin() + j * 3 * w, rgb.begin() + (j + 1) * 3 * w);
  }
  std::vector<uint8_t> z = {0x78, 0x01};
  uint32_t a = 1, b = 0;  // Adler-32
  for (uint8_t c : raw) {
    a = (a + c) % 65521u;
    b = (b + a) % 65521u;
  }
  for (size_t off = 0; off < raw.size() || off == 0; off += 65535) {
    const size_t n = raw.size() - off < 65535 ? raw.size() - off : 65535;
    z.push_back(off + n >= raw.size() ? 1 : 0);
    z.push_back((uint8_t)(n & 0xFF));
    z.push_back((uint8_t)(n >> 8));
    z.push_back((uint8_t)(~n & 0xFF));
    z.push_back((uint8_t)((~n >> 8) & 0xFF));
    z.insert(z.end(), raw.begin() + off, raw.begin() + off + n);
    if (raw.empty()) break;
  }
  be32(z, (b << 16) | a);
  std::vector<uint8_t> png = {0x89, 'P', 'N', 'G', 0x0D, 0x0A, 0x1A, 0x0A};
  std::vector<uint8_t> ihdr;
  be32(ihdr, (uint32_t)w);
  be32(ihdr, (uint32_t)h);
  ihdr.insert(ihdr.end(), {8, 2, 0, 0, 0});
  chunk(png, "IHDR", ihdr);
  chunk(png, "IDAT", z);
  chunk(png, "IEND", {});
  FILE* f = std::fopen(path.c_str(), "wb");
  if (!f) return false;
  const bool ok = std::fwrite(png.data(), 1, png.size(), f) == png.size();
  return std::fclose(f) == 0 && ok;
}

void mkdirs(const std::string& path) {
  for (size_t i = 1; i < path.size(); ++i)
    if (path[i] == '/') mkdir(path.substr(0, i).c_str(), 0755);
}

}  // namespace

int main(int argc, char** argv) {
  std::string metric = "schwarzschild", out = "outputs/render.png";
  size_t width = 1024, height = 1024, max_steps = 20000, samples = 1;
  double fov = 60.0, r_obs = 20.0, step = 0.05, bubble_v = 0.5;
  bool no_stars = false;
  for (int i = 1; i < argc; ++i) {
    const std::string a = argv[i];
    auto val = [&]() -> std::string {
      if (i + 1 >= argc) {
        std::fprintf(stderr, "error: %s needs a value\n", a.c_str());
        std::exit(2);
      }
      return argv[++i];
    };
    if (a == "--metric") metric = val();
    else if (a == "--width") width = std::strtoull(val().c_str(), nullptr, 10);
    else if (a == "--height") height = std::strtoull(val().c_str(), nullptr, 10);
    else if (a == "--fov") fov = std::atof(val().c_str());
    else if (a == "--r-obs") r_obs = std::atof(val().c_str());
    else if (a == "--step") step = std::atof(val().c_str());
    else if (a == "--max-steps") max_steps = std::strtoull(val().c_str(), nullptr, 10);
    else if (a == "--samples") samples = std::strtoull(val().c_str(), nullptr, 10);
    else if (a == "--no-stars") no_stars = true;
    else if (a == "--out") out = val();
    else if (a == "--bubble-v") bubble_v = std::atof(val().c_str());
    else {
      std::fprintf(stderr, "error: unexpected argument '%s'\n", a.c_str());
      return 2;
    }
  }
  const char* debug_name = metric == "minkowski" ? "Minkowski"
                           : metric == "schwarzschild" ? "Schwarzschild"
                           : metric == "alcubierre" ? "Alcubierre"
                           : metric == "morris-thorne" ? "MorrisThorne" : nullptr;
  if (!debug_name) {
    std::fprintf(stderr, "error: invalid value '%s' for '--metric'\n", metric.c_str());
    return 2;
  }
  try {
    geon::set_show_stars(!no_stars);
    geon::RenderConfig cfg = geon::RenderConfig::default_();
    cfg.step = step;
    cfg.max_steps = max_steps;
    cfg.samples_per_axis = samples;
    mkdirs(out);
    std::printf("rendering %s @ %zux%zu, fov %s°, r_obs %s, step %s\n", debug_name, width, height,
                display(fov).c_str(), display(r_obs).c_str(), display(step).c_str());
    const double half_pi = 1.5707963267948966;
    geon::Metric m = metric == "minkowski"       ? geon::Minkowski()
                     : metric == "schwarzschild" ? geon::Schwarzschild(1.0)
                     : metric == "alcubierre"    ? geon::Alcubierre(2.0, 0.5, bubble_v, 0.0)
                                                 : geon::MorrisThorne();
    const bool polar = metric == "schwarzschild" || metric == "morris-thorne";
    const geon::Camera cam = geon::Camera::new_({0.0, r_obs, polar ? half_pi : 0.0, 0.0}, fov, width, height);
    const auto [px, stats] = geon::render_u8(m, cam, cfg);
    if (!write_png(out, px, width, height)) {
      std::fprintf(stderr, "error: cannot write %s\n", out.c_str());
      return 1;
    }
    std::printf("done. captured=%zu, escaped=%zu, diverged=%zu, avg_steps=%s, max_null_residual=%s\n", stats.captured,
                stats.escaped, stats.diverged, fixed(stats.avg_steps, 1).c_str(),
                exp(stats.max_null_residual, 3).c_str());
    std::printf("wrote %s\n", out.c_str());
    return 0;
  } catch (const geon::Panic& e) {
    std::fprintf(stderr, "%s\n", e.what());
    return 101;
  }
}
