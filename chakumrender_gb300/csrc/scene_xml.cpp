// scene_xml.cpp — the reference's scene XML API, on the host: SceneParser
// (src/sceneParser.cpp) and prepareScreenCamera / prepareObjects /
// prepareLightSources (src/prepareScene.cpp), producing a ckr_scene_desc and a
// ckr_camera.
//
// The XML reader is written for this schema only: elements with text content,
// comments, several top-level elements; no attributes are used by the schema.
// Semantics kept from the reference:
//   - vectors/doubles are read as "%lf %lf %lf" / "%lf", sizes as "%u";
//   - COLOR or TEMPERATURE (tempToColor, src/mathPrimitives.cpp:32-60);
//   - material tags ALPHA, SPECCOEF, REFLECTANCE, BRDF required, INTIOR/EXTIOR
//     optional, defaults of SP_Base (headers/sceneParser.h:22-29); an
//     unrecognised BRDF name (e.g. DIFFUSE) becomes BRDF_NONE, which shades 0;
//   - CLASSIC_PHONG takes ALPHA as its exponent (MaterialType(alpha, spec));
//   - meshes: v' = R_seq . S . v + T (src/prepareScene.cpp:62-77, 194-205),
//     rotations by quaternion (src/transformations.cpp:26-42);
//   - objects first (mesh objects, sphere objects, then the reference's dummy
//     sphere and degenerate dummy triangle, src/prepareScene.cpp:238-241),
//     then lights, whose emitters are also visible primitives
//     (headers/lightSources.h:178-203).
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/ckr.h"

namespace {

constexpr double kPI = 3.14159265359;  // headers/mathPrimitives.h:4

struct Node {
  std::string name, text;
  std::vector<std::unique_ptr<Node>> kids;
  const Node *child(const char *n) const {
    for (auto &k : kids)
      if (k->name == n) return k.get();
    return nullptr;
  }
  std::vector<const Node *> all(const char *n) const {
    std::vector<const Node *> r;
    for (auto &k : kids)
      if (k->name == n) r.push_back(k.get());
    return r;
  }
};

class XmlReader {
 public:
  explicit XmlReader(const std::string &s) : s_(s) {}
  bool parse(Node &root) {
    while (true) {
      skip_ws();
      if (i_ >= s_.size()) return true;
      if (!element_or_misc(root)) return false;
    }
  }

 private:
  const std::string &s_;
  size_t i_ = 0;
  void skip_ws() {
    while (i_ < s_.size() && std::isspace((unsigned char)s_[i_])) ++i_;
  }
  bool starts(const char *p) const { return s_.compare(i_, std::strlen(p), p) == 0; }
  bool skip_until(const char *end) {
    size_t j = s_.find(end, i_);
    if (j == std::string::npos) return false;
    i_ = j + std::strlen(end);
    return true;
  }
  // Parses one item at the current position into `parent`: an element, a
  // comment, a declaration, or text.
  bool element_or_misc(Node &parent) {
    if (starts("<!--")) return skip_until("-->");
    if (starts("<?")) return skip_until("?>");
    if (starts("<!")) return skip_until(">");
    if (s_[i_] != '<') {
      size_t j = s_.find('<', i_);
      parent.text += s_.substr(i_, j == std::string::npos ? std::string::npos : j - i_);
      i_ = j == std::string::npos ? s_.size() : j;
      return true;
    }
    ++i_;
    size_t j = i_;
    while (j < s_.size() && !std::isspace((unsigned char)s_[j]) && s_[j] != '>' && s_[j] != '/') ++j;
    auto node = std::make_unique<Node>();
    node->name = s_.substr(i_, j - i_);
    if (node->name.empty()) return false;
    size_t close = s_.find('>', j);
    if (close == std::string::npos) return false;
    bool self = s_[close - 1] == '/';
    i_ = close + 1;
    if (!self) {
      std::string end = "</" + node->name;
      while (true) {
        if (i_ >= s_.size()) return false;
        if (starts(end.c_str())) {
          if (!skip_until(">")) return false;
          break;
        }
        if (!element_or_misc(*node)) return false;
      }
    }
    parent.kids.push_back(std::move(node));
    return true;
  }
};

struct V {
  double x = 0, y = 0, z = 0;
};
V vadd(V a, V b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
V vmul(V a, double s) { return {a.x * s, a.y * s, a.z * s}; }
V cross(V a, V b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
double len(V a) { return std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }
V norm(V a) { return vmul(a, 1.0 / len(a)); }
V maxnorm(V a) {
  double m = a.x;
  if (m < a.y) m = a.y;
  if (m < a.z) m = a.z;
  return {a.x / m, a.y / m, a.z / m};
}

// Row-major 3x3 matrix (the reference's mat3 after its constructors' transposes).
struct M {
  double a[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
  V mul(V v) const {
    return {a[0] * v.x + a[1] * v.y + a[2] * v.z, a[3] * v.x + a[4] * v.y + a[5] * v.z,
            a[6] * v.x + a[7] * v.y + a[8] * v.z};
  }
  M mul(const M &m) const {
    M r;
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) r.a[3 * i + j] = a[3 * i] * m.a[j] + a[3 * i + 1] * m.a[3 + j] + a[3 * i + 2] * m.a[6 + j];
    return r;
  }
};

// rotate(axis, theta) (src/transformations.cpp:26-42): quaternion to matrix.
M rotate(V axis, double theta) {
  V q = norm(axis);
  theta /= 2.0;
  double q0 = std::cos(theta);
  q = vmul(q, std::sin(theta));
  M m;
  m.a[0] = 1.0 - 2.0 * q.y * q.y - 2.0 * q.z * q.z;
  m.a[3] = 2.0 * q.x * q.y + 2.0 * q.z * q0;
  m.a[6] = 2.0 * q.x * q.z - 2.0 * q.y * q0;
  m.a[1] = 2.0 * q.x * q.y - 2.0 * q.z * q0;
  m.a[4] = 1.0 - 2.0 * q.x * q.x - 2.0 * q.z * q.z;
  m.a[7] = 2.0 * q.y * q.z + 2.0 * q.x * q0;
  m.a[2] = 2.0 * q.x * q.z + 2.0 * q.y * q0;
  m.a[5] = 2.0 * q.y * q.z - 2.0 * q.x * q0;
  m.a[8] = 1.0 - 2.0 * q.x * q.x - 2.0 * q.y * q.y;
  return m;
}

// tempToColor (src/mathPrimitives.cpp:32-60): blackbody temperature to RGB.
V temp_to_color(double temperature) {
  temperature = temperature < 1000.0 ? 1000.0 : (temperature > 40000.0 ? 40000.0 : temperature);
  temperature = temperature / 100.0;
  double red, green, blue;
  if (temperature <= 66) {
    red = 255;
    green = 99.4708025861 * std::log(temperature) - 161.1195681661;
    blue = temperature <= 19 ? 0 : 138.5177312231 * std::log(temperature - 10.0) - 305.0447927307;
  } else {
    red = 329.698727446 * std::pow(temperature - 60.0, -0.1332047592);
    green = 288.1221695283 * std::pow(temperature - 60, -0.0755148492);
    blue = 255;
  }
  auto c = [](double v) { return (v < 0.0 ? 0.0 : (v > 255.0 ? 255.0 : v)) / 255.0; };
  return {c(red), c(green), c(blue)};
}

bool text_of(const Node *p, const char *tag, const char **out) {
  const Node *c = p ? p->child(tag) : nullptr;
  if (!c || c->text.find_first_not_of(" \t\r\n") == std::string::npos) return false;
  *out = c->text.c_str();
  return true;
}
bool get_vec(const Node *p, const char *tag, V &v) {
  const char *t;
  return text_of(p, tag, &t) && std::sscanf(t, "%lf %lf %lf", &v.x, &v.y, &v.z) == 3;
}
bool get_double(const Node *p, const char *tag, double &x) {
  const char *t;
  return text_of(p, tag, &t) && std::sscanf(t, "%lf", &x) == 1;
}
bool get_uint(const Node *p, const char *tag, uint32_t &x) {
  const char *t;
  return text_of(p, tag, &t) && std::sscanf(t, "%u", &x) == 1;
}
bool get_string(const Node *p, const char *tag, std::string &s) {
  const Node *c = p ? p->child(tag) : nullptr;
  if (!c || c->kids.size() > 0 || c->text.empty()) return false;
  s = c->text;  // parseString keeps the text node as is
  return true;
}
bool get_color(const Node *p, V &col) {
  if (get_vec(p, "COLOR", col)) return true;
  double T;
  if (!get_double(p, "TEMPERATURE", T)) return false;
  col = temp_to_color(T);
  return true;
}

struct Mat {
  double alpha = 1.0, int_ior = 10000.0, ext_ior = 1, spec = 0, refl = 1.0;
  std::string brdf = "DIFFUSE";
};
bool get_material(const Node *p, Mat &m) {
  if (!get_double(p, "ALPHA", m.alpha) || !get_double(p, "SPECCOEF", m.spec) ||
      !get_double(p, "REFLECTANCE", m.refl) || !get_string(p, "BRDF", m.brdf))
    return false;
  if (p->child("INTIOR") && !get_double(p, "INTIOR", m.int_ior)) return false;
  if (p->child("EXTIOR") && !get_double(p, "EXTIOR", m.ext_ior)) return false;
  return true;
}

int32_t brdf_of(const std::string &s) {
  if (s == "GGX") return 2;
  if (s == "BECKMANN") return 3;
  if (s == "PHONG") return 4;
  if (s == "GGXAPPROX") return 5;
  if (s == "CLASSIC_PHONG") return 1;
  return 0;
}

// MaterialType constructors (headers/materialTypes.h:41-97) + colour/reflectance.
ckr_material surface_material(const Mat &m, V col) {
  ckr_material r;
  std::memset(&r, 0, sizeof(r));
  r.brdf = brdf_of(m.brdf);
  double sc = m.spec * (m.spec < 0 ? -1.0 : 1.0);
  r.spec = (float)(sc <= 1 ? sc : 1);
  if (r.brdf == 1) {
    r.phong_exp = (float)(m.alpha >= 0 ? m.alpha : -m.alpha);
  } else {
    r.alpha = (float)m.alpha;
    r.int_ior = (float)m.int_ior;
    r.ext_ior = (float)m.ext_ior;
  }
  r.reflectance = (float)m.refl;
  r.color[0] = (float)col.x;
  r.color[1] = (float)col.y;
  r.color[2] = (float)col.z;
  return r;
}

ckr_material emitter_material(int32_t light_type, V radiance) {
  ckr_material r;
  std::memset(&r, 0, sizeof(r));
  r.light_type = light_type;
  r.radiance[0] = (float)radiance.x;
  r.radiance[1] = (float)radiance.y;
  r.radiance[2] = (float)radiance.z;
  return r;
}

struct Tri {
  V v1, v2, v3, col;
  double radiance = 0;
  Mat m;
};

bool parse_mesh(const Node *p, bool material, std::vector<Tri> &tris, V &trans, V &scale, M &rot) {
  auto trs = p->all("TR");
  if (trs.empty()) return false;
  for (const Node *t : trs) {
    Tri tr;
    if (!get_vec(t, "V1", tr.v1) || !get_vec(t, "V2", tr.v2) || !get_vec(t, "V3", tr.v3) || !get_color(t, tr.col))
      return false;
    if (material && !get_material(t, tr.m)) return false;
    if (t->child("RADIANCE") && !get_double(t, "RADIANCE", tr.radiance)) return false;
    tris.push_back(tr);
  }
  trans = V();
  if (p->child("TRANSLATE") && !get_vec(p, "TRANSLATE", trans)) return false;
  scale = {1, 1, 1};
  if (p->child("SCALE") && !get_vec(p, "SCALE", scale)) return false;
  rot = M();
  if (const Node *rs = p->child("ROTSEQ")) {
    auto rr = rs->all("R");
    if (rr.empty()) return false;
    for (const Node *r : rr) {
      V axis;
      double deg;
      if (!get_vec(r, "AXIS", axis) || !get_double(r, "ROT", deg)) return false;
      rot = rot.mul(rotate(axis, deg * kPI / 180.0));
    }
  }
  return true;
}

}  // namespace

struct ckr_xml_scene {
  std::vector<float> tri9, sph4;
  std::vector<uint32_t> tri_mat, sph_mat;
  std::vector<ckr_material> mats;
  std::vector<ckr_light> lights;
  ckr_camera cam;
  void add_tri(V a, V b, V c, const ckr_material &m) {
    V p[3] = {a, b, c};
    for (auto &v : p) {
      tri9.push_back((float)v.x);
      tri9.push_back((float)v.y);
      tri9.push_back((float)v.z);
    }
    tri_mat.push_back((uint32_t)mats.size());
    mats.push_back(m);
  }
  void add_sphere(V c, double r, const ckr_material &m) {
    sph4.push_back((float)c.x);
    sph4.push_back((float)c.y);
    sph4.push_back((float)c.z);
    sph4.push_back((float)r);
    sph_mat.push_back((uint32_t)mats.size());
    mats.push_back(m);
  }
};

extern "C" int ckr_xml_load(const char *path, ckr_xml_scene **out) {
  if (!path || !out) return CKR_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  std::ifstream f(path, std::ios::binary);
  if (!f) return CKR_ERR_IO;
  std::stringstream ss;
  ss << f.rdbuf();
  std::string text = ss.str();
  Node doc;
  if (!XmlReader(text).parse(doc)) return CKR_ERR_PARSE;
  auto S = std::make_unique<ckr_xml_scene>();
  // prepareScreenCamera (src/prepareScene.cpp:12-36).
  const Node *screen = doc.child("SCREEN"), *camera = doc.child("CAMERA");
  uint32_t w, h;
  V pos, dir, up;
  double fovx, fovy;
  if (!screen || !get_uint(screen, "WIDTH", w) || !get_uint(screen, "HEIGHT", h) || !camera ||
      !get_vec(camera, "POSITION", pos) || !get_vec(camera, "LOOKAT", dir) || !get_vec(camera, "UP", up) ||
      !get_double(camera, "FOVX", fovx) || !get_double(camera, "FOVY", fovy) || w == 0 || h == 0)
    return CKR_ERR_PARSE;
  V cd = norm(dir);
  V cx = cross(cd, up);
  if (len(cx) < 1e-20) return CKR_ERR_PARSE;
  cx = vmul(norm(cx), ((double)w / h) * std::tan(fovx * kPI / 360.0));
  V cy = vmul(norm(cross(cx, cd)), std::tan(fovy * kPI / 360.0));
  ckr_camera &c = S->cam;
  float *dst[4] = {c.pos, c.dir, c.cx, c.cy};
  V src[4] = {pos, cd, cx, cy};
  for (int k = 0; k < 4; ++k) {
    dst[k][0] = (float)src[k].x;
    dst[k][1] = (float)src[k].y;
    dst[k][2] = (float)src[k].z;
  }
  c.width = w;
  c.height = h;
  // prepareObjects (src/prepareScene.cpp:180-280).
  for (const Node *mo : doc.all("MESHOBJECT")) {
    std::vector<Tri> tris;
    V trans, scale;
    M rot;
    if (!parse_mesh(mo, true, tris, trans, scale, rot)) return CKR_ERR_PARSE;
    M sm;
    sm.a[0] = scale.x;
    sm.a[4] = scale.y;
    sm.a[8] = scale.z;
    M m = rot.mul(sm);
    for (const Tri &t : tris)
      S->add_tri(vadd(m.mul(t.v1), trans), vadd(m.mul(t.v2), trans), vadd(m.mul(t.v3), trans),
                 surface_material(t.m, t.col));
  }
  for (const Node *so : doc.all("SPHEREOBJECT")) {
    auto sps = so->all("SP");
    if (sps.empty()) return CKR_ERR_PARSE;
    V trans;
    if (so->child("TRANSLATE") && !get_vec(so, "TRANSLATE", trans)) return CKR_ERR_PARSE;
    for (const Node *sp : sps) {
      double r;
      V p, col;
      Mat m;
      if (!get_double(sp, "RADIUS", r) || !get_vec(sp, "POSITION", p) || !get_color(sp, col) || !get_material(sp, m))
        return CKR_ERR_PARSE;
      S->add_sphere(vadd(p, trans), r, surface_material(m, col));
    }
  }
  {
    // The reference's dummies: a sphere far above the scene and a degenerate
    // triangle (three vertices equal to Vec(1e6, 0, 0)).
    Mat dm;
    dm.alpha = 200.2;
    dm.spec = 1;
    dm.brdf = "CLASSIC_PHONG";
    S->add_sphere({27, 1e5, 47}, 1, surface_material(dm, {.999, .999, .999}));
    Mat tm;
    tm.alpha = 1.0;
    tm.spec = 0.5;
    tm.refl = 0.9;
    tm.brdf = "CLASSIC_PHONG";
    S->add_tri({1e6, 0, 0}, {1e6, 0, 0}, {1e6, 0, 0}, surface_material(tm, {0.0, 0, 0.9}));
  }
  // prepareLightSources (src/prepareScene.cpp:54-157).
  for (const Node *ms : doc.all("MESHSOURCE")) {
    std::vector<Tri> tris;
    V trans, scale;
    M rot;
    if (!parse_mesh(ms, false, tris, trans, scale, rot)) return CKR_ERR_PARSE;
    M sm;
    sm.a[0] = scale.x;
    sm.a[4] = scale.y;
    sm.a[8] = scale.z;
    M m = rot.mul(sm);
    ckr_light L;
    std::memset(&L, 0, sizeof(L));
    L.type = CKR_LIGHT_MESH;
    L.first = (uint32_t)S->tri_mat.size();
    for (const Tri &t : tris) {
      V rad = vmul(maxnorm(t.col), t.radiance);  // BaseSource(col, intensity)
      S->add_tri(vadd(m.mul(t.v1), trans), vadd(m.mul(t.v2), trans), vadd(m.mul(t.v3), trans),
                 emitter_material(3 /* PLANAR */, rad));
    }
    L.count = (uint32_t)tris.size();
    S->lights.push_back(L);
  }
  for (const Node *ts : doc.all("TRISOURCE")) {
    std::vector<Tri> tris;
    V trans, scale;
    M rot;
    if (!parse_mesh(ts, false, tris, trans, scale, rot)) return CKR_ERR_PARSE;
    M sm;
    sm.a[0] = scale.x;
    sm.a[4] = scale.y;
    sm.a[8] = scale.z;
    M m = rot.mul(sm);
    const Tri &t = tris[0];
    ckr_light L;
    std::memset(&L, 0, sizeof(L));
    L.type = CKR_LIGHT_TRI;
    L.first = (uint32_t)S->tri_mat.size();
    L.count = 1;
    S->add_tri(vadd(m.mul(t.v1), trans), vadd(m.mul(t.v2), trans), vadd(m.mul(t.v3), trans),
               emitter_material(3, vmul(maxnorm(t.col), t.radiance)));
    S->lights.push_back(L);
  }
  for (const Node *ps : doc.all("POINTSOURCE")) {
    V p, col;
    double power;
    if (!get_vec(ps, "POSITION", p) || !get_color(ps, col) || !get_double(ps, "POWER", power)) return CKR_ERR_PARSE;
    ckr_light L;
    std::memset(&L, 0, sizeof(L));
    L.type = CKR_LIGHT_POINT;
    L.pos[0] = (float)p.x; L.pos[1] = (float)p.y; L.pos[2] = (float)p.z;
    V pw = vmul(maxnorm(col), power);
    L.power[0] = (float)pw.x; L.power[1] = (float)pw.y; L.power[2] = (float)pw.z;
    S->lights.push_back(L);
  }
  for (const Node *ss : doc.all("SPHERESOURCE")) {
    double r, radiance;
    V p, col;
    if (!get_double(ss, "RADIUS", r) || !get_vec(ss, "POSITION", p) || !get_color(ss, col)) return CKR_ERR_PARSE;
    if (!get_double(ss, "RADIANCE", radiance)) {
      double power;
      if (!get_double(ss, "POWER", power)) return CKR_ERR_PARSE;
      radiance = power / (4.0 * 3.1415927 * 3.1415927 * r * r);
    }
    ckr_light L;
    std::memset(&L, 0, sizeof(L));
    L.type = CKR_LIGHT_SPHERE;
    L.first = (uint32_t)S->sph_mat.size();
    S->add_sphere(p, r, emitter_material(2 /* VOLUME */, vmul(maxnorm(col), radiance)));
    S->lights.push_back(L);
  }
  *out = S.release();
  return CKR_OK;
}

extern "C" int ckr_xml_get(const ckr_xml_scene *s, ckr_scene_desc *desc, ckr_camera *cam) {
  if (!s) return CKR_ERR_INVALID_ARGUMENT;
  if (desc) {
    std::memset(desc, 0, sizeof(*desc));
    desc->tri9 = s->tri9.data();
    desc->tri_material = s->tri_mat.data();
    desc->ntri = (uint32_t)s->tri_mat.size();
    desc->sph4 = s->sph4.data();
    desc->sph_material = s->sph_mat.data();
    desc->nsph = (uint32_t)s->sph_mat.size();
    desc->materials = s->mats.data();
    desc->nmaterials = (uint32_t)s->mats.size();
    desc->lights = s->lights.data();
    desc->nlights = (uint32_t)s->lights.size();
  }
  if (cam) *cam = s->cam;
  return CKR_OK;
}

extern "C" int ckr_xml_free(ckr_xml_scene *s) {
  if (!s) return CKR_ERR_INVALID_ARGUMENT;
  delete s;
  return CKR_OK;
}

// P3 PPM of src/main.cpp:98-117.
extern "C" int ckr_write_ppm(const char *path, const float *rgb, uint32_t width, uint32_t height) {
  if (!path || !rgb || !width || !height) return CKR_ERR_INVALID_ARGUMENT;
  FILE *f = std::fopen(path, "w");
  if (!f) return CKR_ERR_IO;
  std::fprintf(f, "P3\n%d %d\n%d\n", width, height, 255);
  auto disp = [](double x) {
    x = x < 0.0 ? 0.0 : (x > 1.0 ? 1.0 : x);
    return (int)(std::pow(x, 1.0 / 2.2) * 255 + .5);
  };
  for (size_t p = 0; p < (size_t)width * height; ++p)
    std::fprintf(f, "%d %d %d ", disp(rgb[3 * p]), disp(rgb[3 * p + 1]), disp(rgb[3 * p + 2]));
  return std::fclose(f) == 0 ? CKR_OK : CKR_ERR_IO;
}
