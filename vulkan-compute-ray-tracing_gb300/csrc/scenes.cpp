// Deterministic synthetic workloads (see include/rtgb/rt_scenes.h).
//
// Built with -ffp-contract=off: the only floating-point operations are IEEE
// +, -, *, / and sqrt, so results are identical on every host.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <unordered_map>
#include <vector>

#include "rtgb/rt_scenes.h"

namespace {

// SplitMix64 (Steele, Lea, Flood: "Fast splittable pseudorandom number
// generators", 2014), counter-based so any draw can be addressed.
struct SplitMix {
  uint64_t s;
  uint64_t next() {
    s += 0x9E3779B97F4A7C15ull;
    uint64_t z = s;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
  // Natural logarithm from frexp and the atanh series
  // ln(m) = 2 * (s + s^3/3 + s^5/5 + ...), s = (m - 1) / (m + 1),
  // with m in [sqrt(1/2), sqrt(2)) so |s| < 0.172 and 16 terms reach 1e-25.
  static double series_log(double x) {
    int e = 0;
    double m = std::frexp(x, &e);
    if (m < 0.70710678118654752440) {
      m *= 2.0;
      e -= 1;
    }
    double s = (m - 1.0) / (m + 1.0);
    double s2 = s * s, term = s, sum = 0.0;
    for (int k = 0; k < 16; k++) {
      sum += term / (double)(2 * k + 1);
      term *= s2;
    }
    return (double)e * 0.69314718055994530942 + 2.0 * sum;
  }
  // Standard normal by Marsaglia's polar method (one value per call; the
  // partner value is discarded so that every call consumes whole pairs).
  double normal() {
    for (;;) {
      double u = 2.0 * uniform() - 1.0, v = 2.0 * uniform() - 1.0;
      double s = u * u + v * v;
      if (s > 0.0 && s < 1.0) return u * std::sqrt(-2.0 * series_log(s) / s);
    }
  }
};

inline void set3(float *d, double x, double y, double z) {
  d[0] = (float)x;
  d[1] = (float)y;
  d[2] = (float)z;
}

inline rt_triangle tri(const double *a, const double *b, const double *c, uint32_t m) {
  rt_triangle t;
  std::memset(&t, 0, sizeof(t));
  set3(t.v0, a[0], a[1], a[2]);
  set3(t.v1, b[0], b[1], b[2]);
  set3(t.v2, c[0], c[1], c[2]);
  t.material_index = m;
  return t;
}

// Two triangles for the quad p0 p1 p2 p3 (counter-clockwise).
inline void quad(rt_triangle *out, const double p[4][3], uint32_t m) {
  out[0] = tri(p[0], p[1], p[2], m);
  out[1] = tri(p[0], p[2], p[3], m);
}

void cornell_box(rt_triangle *t, double s) {
  const double L = -5.0 * s, H = 5.0 * s;
  const double floor_[4][3] = {{L, L, L}, {H, L, L}, {H, L, H}, {L, L, H}};
  const double ceil_[4][3] = {{L, H, L}, {L, H, H}, {H, H, H}, {H, H, L}};
  const double back[4][3] = {{L, L, H}, {H, L, H}, {H, H, H}, {L, H, H}};
  const double left[4][3] = {{L, L, L}, {L, L, H}, {L, H, H}, {L, H, L}};
  const double right[4][3] = {{H, L, L}, {H, H, L}, {H, H, H}, {H, L, H}};
  const double ly = 4.99 * s, lq = 1.5 * s;
  const double light[4][3] = {{-lq, ly, -lq}, {-lq, ly, lq}, {lq, ly, lq}, {lq, ly, -lq}};
  quad(t + 0, floor_, 0);
  quad(t + 2, ceil_, 0);
  quad(t + 4, back, 0);
  quad(t + 6, left, 1);
  quad(t + 8, right, 2);
  quad(t + 10, light, 7);
}

void materials8(SplitMix &g, float light_radiance, rt_material *m) {
  std::memset(m, 0, 8 * sizeof(rt_material));
  for (int i = 0; i < 4; i++) {
    m[i].type = RT_MATERIAL_LAMBERTIAN;
    for (int a = 0; a < 3; a++) m[i].albedo[a] = (float)g.uniform();
  }
  for (int i = 4; i < 6; i++) {
    m[i].type = RT_MATERIAL_METAL;
    for (int a = 0; a < 3; a++) m[i].albedo[a] = (float)(0.5 + 0.5 * g.uniform());
    m[i].fuzz = (float)(0.5 * g.uniform());
  }
  m[6].type = RT_MATERIAL_GLASS;
  m[6].ior = 1.5f;
  for (int a = 0; a < 3; a++) m[6].albedo[a] = 1.0f;
  m[7].type = RT_MATERIAL_LIGHT;
  for (int a = 0; a < 3; a++) m[7].albedo[a] = light_radiance;
}

struct Mesh {
  std::vector<double> v;  // xyz triples
  std::vector<uint32_t> f;
};

Mesh icosphere(uint32_t level) {
  const double p = (1.0 + std::sqrt(5.0)) / 2.0;
  const double base[12][3] = {{-1, p, 0}, {1, p, 0}, {-1, -p, 0}, {1, -p, 0}, {0, -1, p}, {0, 1, p},
                              {0, -1, -p}, {0, 1, -p}, {p, 0, -1}, {p, 0, 1}, {-p, 0, -1}, {-p, 0, 1}};
  const uint32_t faces[20][3] = {{0, 11, 5}, {0, 5, 1},  {0, 1, 7},   {0, 7, 10}, {0, 10, 11},
                                 {1, 5, 9},  {5, 11, 4}, {11, 10, 2}, {10, 7, 6}, {7, 1, 8},
                                 {3, 9, 4},  {3, 4, 2},  {3, 2, 6},   {3, 6, 8},  {3, 8, 9},
                                 {4, 9, 5},  {2, 4, 11}, {6, 2, 10},  {8, 6, 7},  {9, 8, 1}};
  Mesh m;
  auto push_unit = [&](double x, double y, double z) {
    double r = std::sqrt(x * x + y * y + z * z);
    m.v.push_back(x / r);
    m.v.push_back(y / r);
    m.v.push_back(z / r);
    return (uint32_t)(m.v.size() / 3 - 1);
  };
  for (auto &b : base) push_unit(b[0], b[1], b[2]);
  for (auto &f : faces) m.f.insert(m.f.end(), f, f + 3);
  for (uint32_t l = 0; l < level; l++) {
    std::unordered_map<uint64_t, uint32_t> mid;
    mid.reserve(m.f.size() * 2);
    auto midpoint = [&](uint32_t a, uint32_t b) {
      uint64_t key = a < b ? ((uint64_t)a << 32) | b : ((uint64_t)b << 32) | a;
      auto it = mid.find(key);
      if (it != mid.end()) return it->second;
      double x = (m.v[3 * a] + m.v[3 * b]) * 0.5, y = (m.v[3 * a + 1] + m.v[3 * b + 1]) * 0.5,
             z = (m.v[3 * a + 2] + m.v[3 * b + 2]) * 0.5;
      uint32_t id = push_unit(x, y, z);
      mid.emplace(key, id);
      return id;
    };
    std::vector<uint32_t> nf;
    nf.reserve(m.f.size() * 4);
    for (size_t i = 0; i < m.f.size(); i += 3) {
      uint32_t a = m.f[i], b = m.f[i + 1], c = m.f[i + 2];
      uint32_t ab = midpoint(a, b), bc = midpoint(b, c), ca = midpoint(c, a);
      const uint32_t add[12] = {a, ab, ca, b, bc, ab, c, ca, bc, ab, bc, ca};
      nf.insert(nf.end(), add, add + 12);
    }
    m.f.swap(nf);
  }
  return m;
}

}  // namespace

extern "C" {

double rtgbUniform(uint64_t seed, uint64_t index) {
  SplitMix g{seed * 0x2545F4914F6CDD1Dull + index * 0x9E3779B97F4A7C15ull};
  return g.uniform();
}

uint32_t rtgbGenCornell(uint64_t seed, uint32_t n_soup, uint32_t n_spheres, float r_lo, float r_hi,
                        float light_radiance, rt_triangle *tris, rt_material *mats, rt_sphere *spheres) {
  SplitMix g{seed};
  materials8(g, light_radiance, mats);
  cornell_box(tris, 1.0);
  for (uint32_t i = 0; i < n_soup; i++) {
    double c[3], v[3][3];
    for (int a = 0; a < 3; a++) c[a] = -4.0 + 8.0 * g.uniform();
    for (int k = 0; k < 3; k++)
      for (int a = 0; a < 3; a++) v[k][a] = c[a] + 0.25 * g.normal();
    uint32_t m = (uint32_t)(7.0 * g.uniform());
    if (m > 6) m = 6;
    tris[12 + i] = tri(v[0], v[1], v[2], m);
  }
  for (uint32_t j = 0; j < n_spheres; j++) {
    rt_sphere s;
    std::memset(&s, 0, sizeof(s));
    for (int a = 0; a < 3; a++) s.s[a] = (float)(-3.5 + 7.0 * g.uniform());
    s.s[3] = (float)((double)r_lo + ((double)r_hi - (double)r_lo) * g.uniform());
    uint32_t m = (uint32_t)(7.0 * g.uniform());
    s.material_index = m > 6 ? 6 : m;
    spheres[j] = s;
  }
  return 12 + n_soup;
}

uint32_t rtgbGenIcosphere(uint64_t seed, uint32_t level, float radius, float sigma, uint32_t material,
                          rt_triangle *tris) {
  uint64_t count = 20ull << (2 * level);
  if (!tris || level > 10) return (uint32_t)count;
  Mesh m = icosphere(level);
  SplitMix g{seed};
  size_t nv = m.v.size() / 3;
  std::vector<double> pos(m.v.size());
  for (size_t i = 0; i < nv; i++) {
    double s = (double)radius * (1.0 + (double)sigma * g.normal());
    for (int a = 0; a < 3; a++) pos[3 * i + a] = m.v[3 * i + a] * s;
  }
  for (size_t f = 0; f < m.f.size() / 3; f++)
    tris[f] = tri(&pos[3 * m.f[3 * f]], &pos[3 * m.f[3 * f + 1]], &pos[3 * m.f[3 * f + 2]], material);
  return (uint32_t)count;
}

void rtgbGenCameraRays(const rt_camera *cam, uint32_t W, uint32_t H, float tmin, float tmax, rt_ray *rays) {
  for (uint32_t y = 0; y < H; y++) {
    for (uint32_t x = 0; x < W; x++) {
      float u = (float)x / (float)W, v = (float)y / (float)H;
      float d[3];
      for (int a = 0; a < 3; a++)
        d[a] = cam->lower_left[a] + u * cam->horizontal[a] + v * cam->vertical[a] - cam->origin[a];
      float len = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
      rt_ray &r = rays[(size_t)y * W + x];
      for (int a = 0; a < 3; a++) {
        r.o[a] = cam->origin[a];
        r.d[a] = d[a] / len;
      }
      r.tmin = tmin;
      r.tmax = tmax;
    }
  }
}

void rtgbGenRandomRays(uint64_t seed, uint64_t n, float lo, float hi, float tmin, float tmax, rt_ray *rays) {
  SplitMix g{seed};
  for (uint64_t i = 0; i < n; i++) {
    rt_ray &r = rays[i];
    for (int a = 0; a < 3; a++) r.o[a] = (float)((double)lo + ((double)hi - (double)lo) * g.uniform());
    double d[3], len;
    do {
      for (int a = 0; a < 3; a++) d[a] = g.normal();
      len = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    } while (len < 1e-12);
    for (int a = 0; a < 3; a++) r.d[a] = (float)(d[a] / len);
    r.tmin = tmin;
    r.tmax = tmax;
  }
}

uint32_t rtgbGenGrid(uint64_t seed, uint32_t gx, uint32_t gz, uint32_t level, float flatten, float sigma,
                     uint32_t keep_per_sphere, float box_scale, rt_triangle *tris, rt_material *mats) {
  uint32_t per = (uint32_t)(20ull << (2 * level));
  if (keep_per_sphere > per) keep_per_sphere = per;
  uint32_t total = 12 + gx * gz * keep_per_sphere;
  if (!tris) return total;
  SplitMix g{seed};
  materials8(g, 4.0f, mats);
  cornell_box(tris, (double)box_scale);
  Mesh m = icosphere(level);
  size_t nv = m.v.size() / 3;
  std::vector<double> pos(m.v.size());
  uint32_t out = 12;
  const double span = 10.0 * (double)box_scale * 0.8;
  const double cell_x = span / (double)gx, cell_z = span / (double)gz;
  const double rad = 0.42 * (cell_x < cell_z ? cell_x : cell_z);
  for (uint32_t iz = 0; iz < gz; iz++) {
    for (uint32_t ix = 0; ix < gx; ix++) {
      double cx = -0.5 * span + (ix + 0.5) * cell_x, cz = -0.5 * span + (iz + 0.5) * cell_z;
      double cy = -5.0 * (double)box_scale + rad * (double)flatten;
      double pick = g.uniform();
      // 40% glass (6), 30% metal (4/5), 30% lambertian (0-3).
      uint32_t mat = pick < 0.4 ? 6u : (pick < 0.7 ? 4u + (uint32_t)(2.0 * g.uniform()) : (uint32_t)(4.0 * g.uniform()));
      if (mat > 6) mat = 6;
      for (size_t i = 0; i < nv; i++) {
        double s = rad * (1.0 + (double)sigma * g.normal());
        pos[3 * i + 0] = cx + m.v[3 * i + 0] * s;
        pos[3 * i + 1] = cy + m.v[3 * i + 1] * s * (double)flatten;
        pos[3 * i + 2] = cz + m.v[3 * i + 2] * s;
      }
      for (uint32_t f = 0; f < keep_per_sphere; f++)
        tris[out++] = tri(&pos[3 * m.f[3 * f]], &pos[3 * m.f[3 * f + 1]], &pos[3 * m.f[3 * f + 2]], mat);
    }
  }
  return out;
}
}
