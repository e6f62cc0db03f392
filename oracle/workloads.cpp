// Test infrastructure (oracle) — NOT part of the product.
//
// The seeded synthetic workloads of the closest-hit measurement, restated
// from their specification (include/rtgb/rt_scenes.h and rtCameraLookAt in
// include/rtgb/rt_api.h) so that the timed reference arm and the CPU
// checks can make their inputs without loading the product library. A CPU
// test pins every output here byte for byte against the library's own
// generators.
//
//   * Random stream: SplitMix64 (Steele, Lea and Flood, OOPSLA 2014), one
//     64-bit state advanced by the golden-ratio increment; a uniform double
//     is the top 53 bits times 2^-53.
//   * Normal deviates: Marsaglia's polar method, one value per accepted pair
//     (the partner is dropped). The logarithm is the atanh series
//     ln m = 2 (s + s^3/3 + ...), s = (m - 1)/(m + 1), on the frexp mantissa
//     folded into [sqrt(1/2), sqrt(2)), 16 terms — so only IEEE +, -, *, /
//     and sqrt are used and every host gives the same bits.
//   * Icosphere: the 12 icosahedron vertices ((+-1, +-p, 0) cyclic, p the
//     golden ratio) and 20 faces, subdivided by edge midpoints (a midpoint is
//     numbered when first met, faces in order, edges ab, bc, ca), every new
//     point projected to the unit sphere; then vertex i is scaled by
//     radius * (1 + sigma * N_i), N_i the i-th normal deviate.
//   * Camera rays: d = normalize(ll + (x/W) hor + (y/H) ver - origin) in
//     fp32; random rays: origin U[lo,hi]^3 (double, rounded once), direction
//     a normalized triple of normal deviates (redrawn below length 1e-12).
//
// Compiled with -ffp-contract=off (oracle/Makefile).
#include <cmath>
#include <cstdint>
#include <cstring>
#include <map>
#include <vector>

namespace {

struct Stream {
  uint64_t state;
  uint64_t bits() {
    state += 0x9E3779B97F4A7C15ull;
    uint64_t z = state;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  double unit() { return (double)(bits() >> 11) / 9007199254740992.0; }
};

double ln_series(double x) {
  int e;
  double m = std::frexp(x, &e);
  if (m < 0.70710678118654752440) {
    m = m * 2.0;
    e = e - 1;
  }
  const double s = (m - 1.0) / (m + 1.0), s2 = s * s;
  double acc = 0.0, pw = s;
  for (int k = 0; k < 16; k++) {
    acc += pw / (double)(2 * k + 1);
    pw *= s2;
  }
  return (double)e * 0.69314718055994530942 + 2.0 * acc;
}

double gauss(Stream &g) {
  for (;;) {
    const double a = 2.0 * g.unit() - 1.0;
    const double b = 2.0 * g.unit() - 1.0;
    const double q = a * a + b * b;
    if (q > 0.0 && q < 1.0) return a * std::sqrt(-2.0 * ln_series(q) / q);
  }
}

struct Sphere {
  std::vector<double> xyz;
  std::vector<uint32_t> tri;
  uint32_t add_unit(double x, double y, double z) {
    const double len = std::sqrt(x * x + y * y + z * z);
    xyz.insert(xyz.end(), {x / len, y / len, z / len});
    return (uint32_t)(xyz.size() / 3 - 1);
  }
};

Sphere subdivided_icosahedron(uint32_t level) {
  Sphere s;
  const double p = (1.0 + std::sqrt(5.0)) / 2.0;
  const double v[12][3] = {{-1, p, 0}, {1, p, 0}, {-1, -p, 0}, {1, -p, 0}, {0, -1, p}, {0, 1, p},
                           {0, -1, -p}, {0, 1, -p}, {p, 0, -1}, {p, 0, 1}, {-p, 0, -1}, {-p, 0, 1}};
  const uint32_t f[60] = {0, 11, 5, 0, 5, 1, 0, 1, 7, 0, 7, 10, 0, 10, 11, 1, 5, 9, 5, 11, 4, 11, 10, 2,
                          10, 7, 6, 7, 1, 8, 3, 9, 4, 3, 4, 2, 3, 2, 6, 3, 6, 8, 3, 8, 9, 4, 9, 5,
                          2, 4, 11, 6, 2, 10, 8, 6, 7, 9, 8, 1};
  for (int i = 0; i < 12; i++) s.add_unit(v[i][0], v[i][1], v[i][2]);
  s.tri.assign(f, f + 60);
  for (uint32_t l = 0; l < level; l++) {
    std::map<std::pair<uint32_t, uint32_t>, uint32_t> edge_mid;
    auto mid = [&](uint32_t a, uint32_t b) -> uint32_t {
      const std::pair<uint32_t, uint32_t> key = a < b ? std::make_pair(a, b) : std::make_pair(b, a);
      const auto found = edge_mid.find(key);
      if (found != edge_mid.end()) return found->second;
      const uint32_t id = s.add_unit((s.xyz[3 * a] + s.xyz[3 * b]) * 0.5, (s.xyz[3 * a + 1] + s.xyz[3 * b + 1]) * 0.5,
                                     (s.xyz[3 * a + 2] + s.xyz[3 * b + 2]) * 0.5);
      edge_mid[key] = id;
      return id;
    };
    std::vector<uint32_t> out;
    out.reserve(4 * s.tri.size());
    for (size_t i = 0; i + 2 < s.tri.size(); i += 3) {
      const uint32_t a = s.tri[i], b = s.tri[i + 1], c = s.tri[i + 2];
      const uint32_t ab = mid(a, b), bc = mid(b, c), ca = mid(c, a);
      out.insert(out.end(), {a, ab, ca, b, bc, ab, c, ca, bc, ab, bc, ca});
    }
    s.tri.swap(out);
  }
  return s;
}

// One 48-byte triangle record: v0, v1, v2 in 16-byte slots, material at 44.
void put_triangle(float *rec, const double *a, const double *b, const double *c, uint32_t material) {
  std::memset(rec, 0, 48);
  for (int k = 0; k < 3; k++) {
    rec[k] = (float)a[k];
    rec[4 + k] = (float)b[k];
    rec[8 + k] = (float)c[k];
  }
  std::memcpy(rec + 11, &material, 4);
}

}  // namespace

extern "C" {

// Displaced icosphere, 20 * 4^level triangles of 12 floats.
uint32_t oracle_gen_icosphere(uint64_t seed, uint32_t level, float radius, float sigma, uint32_t material,
                              float *out) {
  const uint32_t count = (uint32_t)(20ull << (2 * level));
  if (!out || level > 10) return count;
  Sphere s = subdivided_icosahedron(level);
  Stream g{seed};
  const size_t nv = s.xyz.size() / 3;
  std::vector<double> pos(3 * nv);
  for (size_t i = 0; i < nv; i++) {
    const double scale = (double)radius * (1.0 + (double)sigma * gauss(g));
    for (int k = 0; k < 3; k++) pos[3 * i + k] = s.xyz[3 * i + k] * scale;
  }
  for (size_t t = 0; t < s.tri.size() / 3; t++)
    put_triangle(out + 12 * t, &pos[3 * s.tri[3 * t]], &pos[3 * s.tri[3 * t + 1]], &pos[3 * s.tri[3 * t + 2]],
                 material);
  return count;
}

// Pinhole camera as 12 floats: origin, lower-left, horizontal, vertical.
// Computed in double and rounded once per stored value. Returns 0 on a
// degenerate frame.
int oracle_camera_look_at(const float *eye, const float *target, const float *up, float vfov_deg, uint32_t W,
                          uint32_t H, float *cam) {
  double fw[3], rt[3], uu[3];
  for (int k = 0; k < 3; k++) fw[k] = (double)target[k] - (double)eye[k];
  const double fl = std::sqrt(fw[0] * fw[0] + fw[1] * fw[1] + fw[2] * fw[2]);
  if (!(fl > 0.0)) return 0;
  for (double &x : fw) x /= fl;
  rt[0] = fw[1] * up[2] - fw[2] * up[1];
  rt[1] = fw[2] * up[0] - fw[0] * up[2];
  rt[2] = fw[0] * up[1] - fw[1] * up[0];
  const double rl = std::sqrt(rt[0] * rt[0] + rt[1] * rt[1] + rt[2] * rt[2]);
  if (!(rl > 0.0)) return 0;
  for (double &x : rt) x /= rl;
  uu[0] = rt[1] * fw[2] - rt[2] * fw[1];
  uu[1] = rt[2] * fw[0] - rt[0] * fw[2];
  uu[2] = rt[0] * fw[1] - rt[1] * fw[0];
  const double vh = 2.0 * std::tan((double)vfov_deg * 3.14159265358979323846 / 360.0);
  const double vw = vh * (double)W / (double)H;
  for (int k = 0; k < 3; k++) {
    const double hor = vw * rt[k], ver = -vh * uu[k];
    cam[k] = eye[k];
    cam[6 + k] = (float)hor;
    cam[9 + k] = (float)ver;
    cam[3 + k] = (float)((double)eye[k] + fw[k] - 0.5 * hor - 0.5 * ver);
  }
  return 1;
}

// One ray per pixel, row-major: 8 floats (o, tmin, d, tmax).
void oracle_gen_camera_rays(const float *cam, uint32_t W, uint32_t H, float tmin, float tmax, float *rays) {
  for (uint32_t y = 0; y < H; y++) {
    const float fy = (float)y / (float)H;
    for (uint32_t x = 0; x < W; x++) {
      const float fx = (float)x / (float)W;
      float d[3];
      for (int k = 0; k < 3; k++) d[k] = cam[3 + k] + fx * cam[6 + k] + fy * cam[9 + k] - cam[k];
      const float len = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
      float *r = rays + 8ull * ((size_t)y * W + x);
      for (int k = 0; k < 3; k++) {
        r[k] = cam[k];
        r[4 + k] = d[k] / len;
      }
      r[3] = tmin;
      r[7] = tmax;
    }
  }
}

void oracle_gen_random_rays(uint64_t seed, uint64_t n, float lo, float hi, float tmin, float tmax, float *rays) {
  Stream g{seed};
  const double span = (double)hi - (double)lo;
  for (uint64_t i = 0; i < n; i++) {
    float *r = rays + 8 * i;
    for (int k = 0; k < 3; k++) r[k] = (float)((double)lo + span * g.unit());
    double d[3], len;
    do {
      for (int k = 0; k < 3; k++) d[k] = gauss(g);
      len = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    } while (len < 1e-12);
    for (int k = 0; k < 3; k++) r[4 + k] = (float)(d[k] / len);
    r[3] = tmin;
    r[7] = tmax;
  }
}

}  // extern "C"
