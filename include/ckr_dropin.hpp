/*
 * ckr_dropin.hpp — the reference's same-named C++ host API, over the C ABI of
 * libckr.so (ckr.h).  Header only (C++17); link the program with -lckr.
 *
 * The reference (Sayantan2048/ChakumRender) keeps its hot path behind process
 * globals and free functions that main() calls in this order:
 *
 *   initSceneParser(file)                       headers/prepareScene.h:7
 *   prepareScreenCamera(w, h, pos, dir, cx, cy) headers/prepareScene.h:8
 *   prepareObjects(), prepareLightSources()     headers/prepareScene.h:9-10
 *   loadAccels()                                headers/objects.h:17
 *   loadLightSampler()                          headers/mis.h:40
 *   shade(Ray, depth) per pixel                 headers/shader.h:4
 *   shadow(Ray, dist)                           headers/shader.h:6
 *   bvhAccelT->intersectT, bvhAccelS->intersectS headers/bvhAccel.h:73-74
 *
 * This header provides the same names with the same argument meaning, so a
 * caller written against the reference compiles against it.  Underneath, the
 * scene lives on the GPU (ckr_scene) and every query is a batch: the per-ray
 * forms are batches of one, and batched overloads take arrays.
 *
 * Differences a caller sees, all deliberate:
 *  - Ids from intersectT / intersectS are the INPUT index of the primitive; the
 *    reference reorders its primitive list into BVH order in place
 *    (src/bvhAccel.cpp:95-124) and returns that order.
 *  - shade() is the reference's shipped shader (shadeDirectOnly with
 *    getLightFromMeshSource_Analytic_MISCV, src/shader.cpp:339-378) unless
 *    ckr_dropin::shade_config() selects another.  The reference draws its
 *    random numbers from a clock()-seeded generator (src/domainSampler.cpp:55),
 *    so no fixed stream reproduces it; here the per-ray shade(r, depth) draws
 *    from a stream keyed by the ray's bits (deterministic and re-entrant), and
 *    the batched shade(rays, n, out) gives ray i the stream of pixel i, so a
 *    batch of camera rays in output-pixel order reproduces ckr_render's image.
 *  - Errors: the reference prints to std::cerr and returns false or exits; here
 *    the same functions return false (or a miss / black) and
 *    ckr_dropin::last_status() holds the library's status code.
 *
 * Types: Vec, Ray, Sphere and Triangle carry the reference's member names
 * (headers/mathPrimitives.h:13-44, headers/geometryPrimitives.h:37-117) with
 * the geometry fields, the primitive colour and a material index into the
 * parsed scene; materials and lights are the library's (ckr_material,
 * ckr_light), read from the scene file.  A reference main() includes this
 * header in place of the reference's own headers.
 *
 * Threading: the per-ray functions may be called from several host threads
 * (the reference calls shade() from an OpenMP loop); scene set-up is not
 * thread-safe, as in the reference.
 */
#ifndef CKR_DROPIN_HPP
#define CKR_DROPIN_HPP

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <iostream>
#include <mutex>
#include <vector>

#include "ckr.h"

/* headers/mathPrimitives.h:13-37: FP64 vector, `%` is the cross product. */
struct Vec {
  double x, y, z;
  Vec(double x_ = 0, double y_ = 0, double z_ = 0) : x(x_), y(y_), z(z_) {}
  Vec operator+(const Vec &b) const { return Vec(x + b.x, y + b.y, z + b.z); }
  Vec operator-(const Vec &b) const { return Vec(x - b.x, y - b.y, z - b.z); }
  Vec operator*(double b) const { return Vec(x * b, y * b, z * b); }
  Vec operator/(double b) const { return Vec(x / b, y / b, z / b); }
  Vec operator%(const Vec &b) const { return Vec(y * b.z - z * b.y, z * b.x - x * b.z, x * b.y - y * b.x); }
  double dot(const Vec &b) const { return x * b.x + y * b.y + z * b.z; }
  Vec mult(const Vec &b) const { return Vec(x * b.x, y * b.y, z * b.z); }
  double length() const { return std::sqrt(dot(*this)); }
  Vec &norm() { return *this = *this * (1.0 / length()); }
};

/* headers/mathPrimitives.h:39-44: origin and (normalised) direction. */
struct Ray {
  Vec o, d;
  Ray(Vec o_, Vec d_) : o(o_), d(d_) {}
};

/* Geometry of headers/geometryPrimitives.h:37-61 (Sphere) and :63-117
 * (Triangle), plus the index of the primitive's material in the parsed scene
 * and its colour (BasePrimitive::c). */
struct Sphere {
  double r;
  Vec p, c;
  uint32_t material;
  Sphere(double r_ = 1.0, Vec p_ = Vec(), Vec c_ = Vec(), uint32_t material_ = 0)
      : r(r_), p(p_), c(c_), material(material_) {}
};

struct Triangle {
  Vec A, B, C, n, c;
  double area;
  uint32_t material;
  Triangle(Vec A_ = Vec(1, 1, 1), Vec B_ = Vec(1, 1, 1), Vec C_ = Vec(1, 1, 1), Vec c_ = Vec(1, 1, 1),
           uint32_t material_ = 0)
      : A(A_), B(B_), C(C_), c(c_), material(material_) {
    n = (C - A) % (B - A);  // as the reference: (C - A) x (B - A), normalised
    area = 0.5 * n.length();
    if (area > 0) n.norm();
  }
};

namespace ckr_dropin {

/* Process state behind the reference's globals. */
struct State {
  ckr_xml_scene *xml = nullptr;
  ckr_scene_desc desc{};
  ckr_camera cam{};
  std::vector<ckr_material> materials;
  std::vector<ckr_light> lights;
  std::vector<float> tri9, sph4;
  std::vector<uint32_t> tri_mat, sph_mat;
  ckr_scene *scene = nullptr;  // geometry + materials + lights (shade, shadow)
  ckr_render_cfg shade_cfg{CKR_SHADER_DIRECT_MISCV, 1, 1, 10, 60, 0.3f, 1, 0, 0};  // headers/mis.h:8-12
  int status = CKR_OK;
  std::mutex mu;  // guards `status`
};

inline State &state() {
  static State s;
  return s;
}

/* The status of the last failing library call (CKR_OK if none failed). */
inline int last_status() {
  std::lock_guard<std::mutex> lock(state().mu);
  return state().status;
}

inline bool ok(int st, const char *what) {
  if (st == CKR_OK) return true;
  char buf[128];
  ckr_status_string(st, buf, sizeof buf);
  std::cerr << "ckr_dropin: " << what << ": " << buf << "\n";
  std::lock_guard<std::mutex> lock(state().mu);
  state().status = st;
  return false;
}

/* The shader, sample counts and seed shade() uses (default: the reference's
 * shipped shadeDirectOnly + MISCV, 10 light and 60 BRDF samples). */
inline ckr_render_cfg &shade_config() { return state().shade_cfg; }

/* The device scene behind shade() and shadow() (NULL before loadAccels()). */
inline ckr_scene *device_scene() { return state().scene; }

inline ckr_ray to_ray(const Ray &r, float tmin = 0.f, float tmax = 1e30f) {
  ckr_ray q;
  q.ox = (float)r.o.x, q.oy = (float)r.o.y, q.oz = (float)r.o.z, q.tmin = tmin;
  q.dx = (float)r.d.x, q.dy = (float)r.d.y, q.dz = (float)r.d.z, q.tmax = tmax;
  return q;
}

/* splitmix64 over the ray's float bits: the per-ray shade() stream. */
inline uint64_t ray_stream(const ckr_ray &q) {
  uint32_t w[8];
  std::memcpy(w, &q, sizeof w);
  uint64_t h = 0x243F6A8885A308D3ull;
  for (uint32_t v : w) {
    h += v + 0x9E3779B97F4A7C15ull;
    h = (h ^ (h >> 30)) * 0xBF58476D1CE4E5B9ull;
    h = (h ^ (h >> 27)) * 0x94D049BB133111EBull;
    h ^= h >> 31;
  }
  return h;
}

}  // namespace ckr_dropin

/* headers/bvhAccel.h:62-76: an accelerator over a primitive list.  The list is
 * the reference's (uint8_t *)list with element size sizeof(Triangle) or
 * sizeof(Sphere); initAccel() builds the device BVH (ckr_scene_create). */
class BvhAccel {
  const uint8_t *list_;
  uint32_t n_;
  std::size_t size_;
  ckr_scene *scene_ = nullptr;
  bool spheres_;

 public:
  BvhAccel(uint8_t *list, uint32_t nP, std::size_t sz)
      : list_(list), n_(nP), size_(sz), spheres_(sz == sizeof(Sphere) && sz != sizeof(Triangle)) {}
  ~BvhAccel() {
    if (scene_) ckr_scene_destroy(scene_);
  }
  BvhAccel(const BvhAccel &) = delete;
  BvhAccel &operator=(const BvhAccel &) = delete;

  /* BvhAccel::initAccel (src/bvhAccel.cpp:13-22). */
  void initAccel() {
    if (scene_) ckr_scene_destroy(scene_), scene_ = nullptr;
    if (n_ == 0) return;
    std::vector<float> g;
    if (spheres_) {
      g.resize(4 * (size_t)n_);
      for (uint32_t i = 0; i < n_; ++i) {
        const Sphere &s = *reinterpret_cast<const Sphere *>(list_ + i * size_);
        g[4 * i] = (float)s.p.x, g[4 * i + 1] = (float)s.p.y, g[4 * i + 2] = (float)s.p.z, g[4 * i + 3] = (float)s.r;
      }
      ckr_dropin::ok(ckr_scene_create(nullptr, 0, g.data(), n_, nullptr, &scene_), "BvhAccel::initAccel");
    } else {
      g.resize(9 * (size_t)n_);
      for (uint32_t i = 0; i < n_; ++i) {
        const Triangle &t = *reinterpret_cast<const Triangle *>(list_ + i * size_);
        const Vec *v[3] = {&t.A, &t.B, &t.C};
        for (int k = 0; k < 3; ++k)
          g[9 * i + 3 * k] = (float)v[k]->x, g[9 * i + 3 * k + 1] = (float)v[k]->y, g[9 * i + 3 * k + 2] = (float)v[k]->z;
      }
      ckr_dropin::ok(ckr_scene_create(g.data(), n_, nullptr, 0, nullptr, &scene_), "BvhAccel::initAccel");
    }
  }

  /* Batched closest hit: t[i] (1e20 on a miss, headers/mathPrimitives.h:5) and
   * id[i] (0xFFFFFFFF on a miss, else the input index). */
  bool intersect(const Ray *rays, uint32_t n, double *t, int *id) const {
    std::vector<ckr_ray> q(n);
    for (uint32_t i = 0; i < n; ++i) q[i] = ckr_dropin::to_ray(rays[i]);
    std::vector<uint32_t> hid(n, CKR_MISS);
    std::vector<float> ht(n, 0.f);
    bool good = !scene_ || ckr_dropin::ok(ckr_trace_closest_host(scene_, q.data(), n, hid.data(), ht.data(), nullptr),
                                          "BvhAccel::intersect");
    for (uint32_t i = 0; i < n; ++i) {
      const bool hit = scene_ && good && hid[i] != CKR_MISS;
      id[i] = hit ? (int)(hid[i] & ~CKR_SPHERE_BIT) : (int)0xFFFFFFFF;
      t[i] = hit ? (double)ht[i] : 1e20;
    }
    return good;
  }

  /* BvhAccel::intersectT (src/bvhAccel.cpp:200-249): closest triangle, its
   * unit normal turned towards the ray origin (Triangle::intersect,
   * src/geometryPrimitives.cpp:29-71). */
  bool intersectT(const Ray &r, double &t, Vec &N, int &id) const {
    intersect(&r, 1, &t, &id);
    if (id == (int)0xFFFFFFFF || spheres_) return false;
    const Triangle &tri = *reinterpret_cast<const Triangle *>(list_ + (size_t)id * size_);
    N = tri.n;
    if (r.d.dot(N) > 0) N = N * -1.0;
    return true;
  }

  /* BvhAccel::intersectS (src/bvhAccel.cpp:151-198): closest sphere. */
  bool intersectS(const Ray &r, double &t, int &id) const {
    intersect(&r, 1, &t, &id);
    return id != (int)0xFFFFFFFF && spheres_;
  }
};

/* The reference's globals (headers/objects.h:7-14, headers/bvhAccel.h:78). */
inline std::vector<Sphere> vSphereList;
inline std::vector<Triangle> vTriangleList;
inline uint32_t nSpheres = 0, nTriangles = 0;
inline Sphere *sphereList = nullptr;
inline Triangle *triangleList = nullptr;
inline BvhAccel *bvhAccelT = nullptr, *bvhAccelS = nullptr;

/* initSceneParser (src/prepareScene.cpp via SceneParser): loads the XML scene. */
inline bool initSceneParser(const char *fileName) {
  ckr_dropin::State &S = ckr_dropin::state();
  if (S.xml) ckr_xml_free(S.xml), S.xml = nullptr;
  if (!ckr_dropin::ok(ckr_xml_load(fileName, &S.xml), "initSceneParser")) return false;
  return ckr_dropin::ok(ckr_xml_get(S.xml, &S.desc, &S.cam), "initSceneParser");
}

/* prepareScreenCamera (src/prepareScene.cpp:12-36). */
inline bool prepareScreenCamera(uint32_t &width, uint32_t &height, Vec &camPos, Vec &camDir, Vec &cx, Vec &cy,
                                bool verbose) {
  const ckr_camera &c = ckr_dropin::state().cam;
  if (!ckr_dropin::state().xml) return false;
  width = c.width, height = c.height;
  camPos = Vec(c.pos[0], c.pos[1], c.pos[2]);
  camDir = Vec(c.dir[0], c.dir[1], c.dir[2]);
  cx = Vec(c.cx[0], c.cx[1], c.cx[2]);
  cy = Vec(c.cy[0], c.cy[1], c.cy[2]);
  if (verbose) std::cerr << "screen " << width << " x " << height << "\n";
  return true;
}

/* prepareObjects (src/prepareScene.cpp:54-236): the scene's triangles and
 * spheres into vTriangleList / vSphereList, materials kept for loadAccels(). */
inline bool prepareObjects(bool verbose) {
  ckr_dropin::State &S = ckr_dropin::state();
  if (!S.xml) return false;
  const ckr_scene_desc &d = S.desc;
  S.materials.assign(d.materials, d.materials + d.nmaterials);
  vTriangleList.clear();
  vSphereList.clear();
  for (uint32_t i = 0; i < d.ntri; ++i) {
    const float *v = d.tri9 + 9 * (size_t)i;
    const uint32_t m = d.tri_material ? d.tri_material[i] : 0;
    const float *c = S.materials[m].color;
    vTriangleList.push_back(Triangle(Vec(v[0], v[1], v[2]), Vec(v[3], v[4], v[5]), Vec(v[6], v[7], v[8]),
                                     Vec(c[0], c[1], c[2]), m));
  }
  for (uint32_t i = 0; i < d.nsph; ++i) {
    const float *s = d.sph4 + 4 * (size_t)i;
    const uint32_t m = d.sph_material ? d.sph_material[i] : 0;
    const float *c = S.materials[m].color;
    vSphereList.push_back(Sphere(s[3], Vec(s[0], s[1], s[2]), Vec(c[0], c[1], c[2]), m));
  }
  if (verbose) std::cerr << vTriangleList.size() << " triangles, " << vSphereList.size() << " spheres\n";
  return true;
}

/* prepareLightSources (src/prepareScene.cpp:238-280). */
inline bool prepareLightSources(bool verbose) {
  ckr_dropin::State &S = ckr_dropin::state();
  if (!S.xml) return false;
  S.lights.assign(S.desc.lights, S.desc.lights + S.desc.nlights);
  if (verbose) std::cerr << S.lights.size() << " light sources\n";
  return true;
}

/* loadAccels (src/objects.cpp:38-56): copies the lists into triangleList /
 * sphereList, builds bvhAccelT / bvhAccelS over them and the device scene that
 * shade() and shadow() use (geometry + the parsed materials and lights). */
inline void loadAccels() {
  ckr_dropin::State &S = ckr_dropin::state();
  nTriangles = (uint32_t)vTriangleList.size();
  nSpheres = (uint32_t)vSphereList.size();
  triangleList = vTriangleList.data();
  sphereList = vSphereList.data();
  delete bvhAccelT;
  delete bvhAccelS;
  bvhAccelT = new BvhAccel(reinterpret_cast<uint8_t *>(triangleList), nTriangles, sizeof(Triangle));
  bvhAccelT->initAccel();
  bvhAccelS = new BvhAccel(reinterpret_cast<uint8_t *>(sphereList), nSpheres, sizeof(Sphere));
  bvhAccelS->initAccel();
  S.tri9.resize(9 * (size_t)nTriangles);
  S.tri_mat.resize(nTriangles);
  for (uint32_t i = 0; i < nTriangles; ++i) {
    const Triangle &t = triangleList[i];
    const Vec *v[3] = {&t.A, &t.B, &t.C};
    for (int k = 0; k < 3; ++k)
      S.tri9[9 * i + 3 * k] = (float)v[k]->x, S.tri9[9 * i + 3 * k + 1] = (float)v[k]->y,
                        S.tri9[9 * i + 3 * k + 2] = (float)v[k]->z;
    S.tri_mat[i] = t.material;
  }
  S.sph4.resize(4 * (size_t)nSpheres);
  S.sph_mat.resize(nSpheres);
  for (uint32_t i = 0; i < nSpheres; ++i) {
    const Sphere &s = sphereList[i];
    S.sph4[4 * i] = (float)s.p.x, S.sph4[4 * i + 1] = (float)s.p.y, S.sph4[4 * i + 2] = (float)s.p.z;
    S.sph4[4 * i + 3] = (float)s.r;
    S.sph_mat[i] = s.material;
  }
  if (S.scene) ckr_scene_destroy(S.scene), S.scene = nullptr;
  if (S.materials.empty()) S.materials.push_back(ckr_material{});  // geometry-only scenes
  ckr_scene_desc d{};
  d.tri9 = S.tri9.data(), d.tri_material = S.tri_mat.data(), d.ntri = nTriangles;
  d.sph4 = S.sph4.data(), d.sph_material = S.sph_mat.data(), d.nsph = nSpheres;
  d.materials = S.materials.data(), d.nmaterials = (uint32_t)S.materials.size();
  d.lights = S.lights.data(), d.nlights = (uint32_t)S.lights.size();
  d.env = S.xml ? S.desc.env : nullptr;
  ckr_dropin::ok(ckr_scene_create_ex(&d, &S.scene), "loadAccels");
}

/* loadLightSampler (src/mis.cpp:225-233): the light sampler (per-light CDFs,
 * MIS counts) is part of the device scene loadAccels() built; nothing to do. */
inline void loadLightSampler() {}

/* Batched shade(): out[i] = radiance along rays[i], drawn from the stream of
 * pixel i (seed = shade_config().seed).  Rays are expected normalised, as
 * shade() requires (src/shader.cpp:362). */
inline bool shade(const Ray *rays, uint32_t n, Vec *out) {
  ckr_dropin::State &S = ckr_dropin::state();
  std::vector<ckr_ray> q(n);
  for (uint32_t i = 0; i < n; ++i) q[i] = ckr_dropin::to_ray(rays[i], 0.f, 3.0e38f);
  std::vector<float> rgb(3 * (size_t)n, 0.f);
  bool good = S.scene && n &&
              ckr_dropin::ok(ckr_shade_rays_host(S.scene, q.data(), n, &S.shade_cfg, rgb.data(), nullptr), "shade");
  for (uint32_t i = 0; i < n; ++i) out[i] = good ? Vec(rgb[3 * i], rgb[3 * i + 1], rgb[3 * i + 2]) : Vec();
  return good;
}

/* shade() (headers/shader.h:4, src/shader.cpp:363-378): radiance along r.
 * `depth` is accepted and unused, as by the shipped shadeDirectOnly. */
inline Vec shade(const Ray &r, int &depth) {
  (void)depth;
  ckr_dropin::State &S = ckr_dropin::state();
  if (!S.scene) return Vec();
  ckr_ray q = ckr_dropin::to_ray(r, 0.f, 3.0e38f);
  ckr_render_cfg cfg = S.shade_cfg;
  cfg.seed ^= ckr_dropin::ray_stream(q);
  float rgb[3] = {0.f, 0.f, 0.f};
  if (!ckr_dropin::ok(ckr_shade_rays_host(S.scene, &q, 1, &cfg, rgb, nullptr), "shade")) return Vec();
  return Vec(rgb[0], rgb[1], rgb[2]);
}

/* Batched shadow(): out[i] = 0 when something lies within distance[i] - 1e-5 of
 * rays[i].o along rays[i].d, else 1. */
inline bool shadow(const Ray *rays, const double *distance, uint32_t n, double *out) {
  ckr_dropin::State &S = ckr_dropin::state();
  std::vector<ckr_ray> q(n);
  for (uint32_t i = 0; i < n; ++i) q[i] = ckr_dropin::to_ray(rays[i], 0.f, (float)(distance[i] - 1e-5));
  std::vector<uint8_t> occ(n, 0);
  bool good = !S.scene || ckr_dropin::ok(ckr_trace_any_host(S.scene, q.data(), n, occ.data(), nullptr), "shadow");
  for (uint32_t i = 0; i < n; ++i) out[i] = occ[i] ? 0.0 : 1.0;
  return good;
}

/* shadow() (headers/shader.h:6, src/shader.cpp:76-97): 0 if shadowed, else 1.
 * The reference returns 0 when the closest sphere or triangle hit t satisfies
 * t + 1e-5 < distanceLightSource; an any-hit query up to that distance is the
 * same test. */
inline double shadow(const Ray &shadowRay, double distanceLightSource) {
  double v = 1.0;
  shadow(&shadowRay, &distanceLightSource, 1, &v);
  return v;
}

#endif
