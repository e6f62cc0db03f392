// Wavefront OBJ triangles and the reference's demo scene (rt_obj.h).
//
// The reference reads its OBJ files with tinyobjloader (an un-vendored
// submodule, external/obj-loader, version not pinned) in
// src/scene/mesh.cpp:96-139 and turns each face into a GpuModel::Triangle of
// vertex positions in RtScene.h:13-31. Only positions and face order matter
// for the path, so this is a small position-only parser of its own:
//   * coordinates: sign, integer digits accumulated as m = 10 m + d, fraction
//     digit k adding d * 10^-k, exponent applied as ldexp(m * 5^e, e), all in
//     double, then one rounding to float (the scheme tinyobjloader publishes
//     for its parser); unparsable fields read as 0 as there;
//   * faces: the vertex part of each index, 1-based or negative-relative,
//     fanned from the first vertex when a face has more than three.
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "rtgb/rt_obj.h"

namespace {

thread_local std::string g_obj_error;

rt_status obj_fail(rt_status s, const std::string &msg) {
  g_obj_error = msg;
  return s;
}

inline bool is_space(char c) { return c == ' ' || c == '\t'; }
inline bool is_digit(char c) { return c >= '0' && c <= '9'; }

// Negative powers of ten as the nearest doubles (decimal literals round
// correctly); beyond the table std::pow is used.
constexpr double kNegPow10[] = {1.0,   1e-1,  1e-2,  1e-3,  1e-4,  1e-5,  1e-6,  1e-7,  1e-8,  1e-9,  1e-10,
                                1e-11, 1e-12, 1e-13, 1e-14, 1e-15, 1e-16, 1e-17, 1e-18, 1e-19, 1e-20};

// Parses one real starting at p (no leading whitespace); advances p past the
// token. Returns false (value 0) when the token is not a number.
bool parse_real(const char *&p, const char *end, double &out) {
  const char *s = p;
  while (p < end && !is_space(*p)) p++;  // the token is [s, p)
  out = 0.0;
  const char *c = s;
  double sign = 1.0;
  if (c < p && (*c == '+' || *c == '-')) {
    if (*c == '-') sign = -1.0;
    c++;
  }
  double m = 0.0;
  int digits = 0;
  while (c < p && is_digit(*c)) {
    m = m * 10.0 + (double)(*c - '0');
    c++;
    digits++;
  }
  if (c < p && *c == '.') {
    c++;
    int k = 1;
    while (c < p && is_digit(*c)) {
      const double scale = k < (int)(sizeof(kNegPow10) / sizeof(kNegPow10[0])) ? kNegPow10[k] : std::pow(10.0, -k);
      m += (double)(*c - '0') * scale;
      c++;
      k++;
      digits++;
    }
  }
  if (digits == 0) return false;
  int e = 0;
  if (c < p && (*c == 'e' || *c == 'E')) {
    c++;
    int esign = 1;
    if (c < p && (*c == '+' || *c == '-')) {
      if (*c == '-') esign = -1;
      c++;
    }
    int ed = 0;
    while (c < p && is_digit(*c)) {
      if (e < 100000) e = e * 10 + (*c - '0');
      c++;
      ed++;
    }
    if (ed == 0) return false;
    e *= esign;
  }
  if (c != p) return false;  // trailing garbage
  out = sign * (e != 0 ? std::ldexp(m * std::pow(5.0, (double)e), e) : m);
  return true;
}

// Vertex index of a face token `v`, `v/vt`, `v//vn` or `v/vt/vn`.
bool parse_face_index(const char *&p, const char *end, long &idx) {
  const char *s = p;
  while (p < end && !is_space(*p)) p++;
  const char *c = s;
  bool neg = false;
  if (c < p && (*c == '+' || *c == '-')) {
    neg = *c == '-';
    c++;
  }
  long v = 0;
  int nd = 0;
  while (c < p && is_digit(*c)) {
    if (v < (1L << 40)) v = v * 10 + (*c - '0');
    c++;
    nd++;
  }
  if (nd == 0 || (c < p && *c != '/')) return false;
  idx = neg ? -v : v;
  return true;
}

rt_status parse_obj(const std::string &path, uint32_t material, std::vector<rt_triangle> &tris) {
  FILE *f = std::fopen(path.c_str(), "rb");
  if (!f) return obj_fail(RT_ERR_NOT_FOUND, "rtLoadObj: cannot open " + path + ": " + std::strerror(errno));
  std::string text;
  char buf[1 << 16];
  size_t got;
  while ((got = std::fread(buf, 1, sizeof(buf), f)) > 0) text.append(buf, got);
  const bool bad = std::ferror(f) != 0;
  std::fclose(f);
  if (bad) return obj_fail(RT_ERR_NOT_FOUND, "rtLoadObj: read error on " + path);

  std::vector<float> verts;  // xyz per vertex
  std::vector<long> face;
  const char *p = text.data(), *end = p + text.size();
  uint64_t line_no = 0;
  while (p < end) {
    const char *eol = p;
    while (eol < end && *eol != '\n' && *eol != '\r') eol++;
    line_no++;
    const char *q = p;
    while (q < eol && is_space(*q)) q++;
    if (eol - q >= 2 && q[0] == 'v' && is_space(q[1])) {
      q += 2;
      double xyz[3] = {0.0, 0.0, 0.0};
      for (int k = 0; k < 3; k++) {
        while (q < eol && is_space(*q)) q++;
        if (q >= eol) break;
        parse_real(q, eol, xyz[k]);
      }
      for (int k = 0; k < 3; k++) verts.push_back((float)xyz[k]);
    } else if (eol - q >= 2 && q[0] == 'f' && is_space(q[1])) {
      q += 2;
      face.clear();
      const long nv = (long)(verts.size() / 3);
      for (;;) {
        while (q < eol && is_space(*q)) q++;
        if (q >= eol) break;
        long idx = 0;
        if (!parse_face_index(q, eol, idx) || idx == 0)
          return obj_fail(RT_ERR_INVALID_SCENE, path + ":" + std::to_string(line_no) + ": bad face index");
        long v = idx > 0 ? idx - 1 : nv + idx;
        if (v < 0 || v >= nv)
          return obj_fail(RT_ERR_INVALID_SCENE,
                          path + ":" + std::to_string(line_no) + ": face index " + std::to_string(idx) +
                              " outside the " + std::to_string(nv) + " vertices read so far");
        face.push_back(v);
      }
      for (size_t k = 1; k + 1 < face.size(); k++) {
        rt_triangle t;
        std::memset(&t, 0, sizeof(t));
        const long ids[3] = {face[0], face[k], face[k + 1]};
        float *dst[3] = {t.v0, t.v1, t.v2};
        for (int j = 0; j < 3; j++)
          for (int a = 0; a < 3; a++) dst[j][a] = verts[3 * ids[j] + a];
        t.material_index = material;
        tris.push_back(t);
        if (tris.size() > 0xffffffffull) return obj_fail(RT_ERR_INVALID_SCENE, path + ": too many triangles");
      }
    }
    // Line end: \n, \r\n or a lone \r.
    p = eol;
    if (p < end && *p == '\r') p++;
    if (p < end && *p == '\n') p++;
  }
  return RT_SUCCESS;
}

rt_material make_material(uint32_t type, float r, float g, float b) {
  rt_material m;
  std::memset(&m, 0, sizeof(m));
  m.type = type;
  m.albedo[0] = r;
  m.albedo[1] = g;
  m.albedo[2] = b;
  return m;
}

}  // namespace

extern "C" {

const char *rtObjLastError(void) { return g_obj_error.c_str(); }

rt_status rtLoadObj(const char *path, uint32_t material_index, rt_triangle *out, uint32_t capacity,
                    uint32_t *count) {
  if (!path || !count) return obj_fail(RT_ERR_INVALID_ARGUMENT, "rtLoadObj: null argument");
  std::vector<rt_triangle> tris;
  rt_status s = parse_obj(path, material_index, tris);
  if (s != RT_SUCCESS) return s;
  *count = (uint32_t)tris.size();
  if (!out) return RT_SUCCESS;
  if (capacity < tris.size())
    return obj_fail(RT_ERR_INVALID_ARGUMENT, "rtLoadObj: capacity " + std::to_string(capacity) + " below " +
                                                 std::to_string(tris.size()) + " triangles");
  if (!tris.empty()) std::memcpy(out, tris.data(), tris.size() * sizeof(rt_triangle));
  return RT_SUCCESS;
}

rt_status rtLoadReferenceScene(const char *model_dir, rt_triangle *tris, uint32_t capacity, uint32_t *n_tris,
                               rt_material *mats, rt_sphere *spheres) {
  if (!model_dir || !n_tris) return obj_fail(RT_ERR_INVALID_ARGUMENT, "rtLoadReferenceScene: null argument");
  // Files and materials of RtScene.h:64-76, in the order RtScene.h:78-85
  // inserts them: doge, cheems, right, left, back, ceil, floor, light.
  static const struct {
    const char *file;
    uint32_t material;
  } kObjects[] = {{"buff-doge.obj", 0}, {"cheems.obj", 0}, {"right.obj", 1}, {"left.obj", 2},
                  {"back.obj", 0},      {"ceil.obj", 0},   {"floor.obj", 0}, {"light.obj", 3}};
  std::vector<rt_triangle> all;
  for (const auto &o : kObjects) {
    std::string path = std::string(model_dir) + "/" + o.file;
    rt_status s = parse_obj(path, o.material, all);
    if (s != RT_SUCCESS) return s;
  }
  *n_tris = (uint32_t)all.size();
  if (tris) {
    if (capacity < all.size())
      return obj_fail(RT_ERR_INVALID_ARGUMENT, "rtLoadReferenceScene: capacity " + std::to_string(capacity) +
                                                   " below " + std::to_string(all.size()) + " triangles");
    std::memcpy(tris, all.data(), all.size() * sizeof(rt_triangle));
  }
  if (mats) {
    // RtScene.h:48-60: gray, red, green, white light, metal, glass.
    mats[0] = make_material(RT_MATERIAL_LAMBERTIAN, 0.3f, 0.3f, 0.3f);
    mats[1] = make_material(RT_MATERIAL_LAMBERTIAN, 0.9f, 0.1f, 0.1f);
    mats[2] = make_material(RT_MATERIAL_LAMBERTIAN, 0.1f, 0.9f, 0.1f);
    mats[3] = make_material(RT_MATERIAL_LIGHT, 2.0f, 2.0f, 2.0f);
    mats[4] = make_material(RT_MATERIAL_METAL, 1.0f, 1.0f, 1.0f);
    mats[5] = make_material(RT_MATERIAL_GLASS, 1.0f, 1.0f, 1.0f);
  }
  if (spheres) {
    // RtScene.h:98: glm::vec4(0.6, 1, -1, 0.6) with material 5 (glass).
    std::memset(spheres, 0, sizeof(rt_sphere));
    spheres[0].s[0] = 0.6f;
    spheres[0].s[1] = 1.0f;
    spheres[0].s[2] = -1.0f;
    spheres[0].s[3] = 0.6f;
    spheres[0].material_index = 5;
  }
  return RT_SUCCESS;
}

}  // extern "C"
