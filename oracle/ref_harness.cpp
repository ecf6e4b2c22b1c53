// ref_harness.cpp — C entry points over the UNMODIFIED reference renderer.
//
// TEST INFRASTRUCTURE ONLY.  oracle/Makefile compiles the reference's own
// sources (src/*.cpp of Sayantan2048/ChakumRender) together with this file
// into oracle/_ref/libckr_ref.so.  The tests use it to pin the FP64 C
// restatement in oracle/*.c against the reference itself.  It is built only
// where the reference sources are present; nothing shipped depends on it.
//
// Original triangle indices survive the reference's in-place BVH reordering
// (src/bvhAccel.cpp:95-124) because each Triangle carries its input index in
// its colour field c.x, which the reordering copies along with the rest.
#include <stdint.h>
#include <vector>
#include <omp.h>
#include "mathPrimitives.h"
#include "geometryPrimitives.h"
#include "materialTypes.h"
#include "objects.h"
#include "bvhAccel.h"
#include "shader.h"
#include "lightSources.h"
#include "prepareScene.h"

extern "C" {

int ref_trace_build(const float *tri9, uint32_t ntri) {
  if (ntri == 0) return -1;
  nTriangles = ntri;
  triangleList = new Triangle[ntri];
  for (uint32_t i = 0; i < ntri; ++i) {
    const float *t = tri9 + 9 * (size_t)i;
    triangleList[i] = Triangle(Vec(t[0], t[1], t[2]), Vec(t[3], t[4], t[5]),
                               Vec(t[6], t[7], t[8]), Vec((double)i, 0, 0), 1.0,
                               MaterialType());
  }
  bvhAccelT = new BvhAccel((uint8_t *)triangleList, nTriangles, sizeof(Triangle));
  bvhAccelT->initAccel();
  // The reference scene always holds its far-away dummy sphere
  // (src/prepareScene.cpp:238); shadow() needs a sphere BVH to query.
  nSpheres = 1;
  sphereList = new Sphere[1];
  sphereList[0] = Sphere(1, Vec(27, 1e5, 47), Vec(.999, .999, .999), 1.0, MaterialType(200.2, 1));
  bvhAccelS = new BvhAccel((uint8_t *)sphereList, nSpheres, sizeof(Sphere));
  bvhAccelS->initAccel();
  return 0;
}

// BvhAccel::intersectT per ray; ids mapped back to input order.
void ref_trace_closest(const float *rays8, uint32_t nrays, uint32_t *hit_id,
                       double *hit_t, int threads) {
  if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel for schedule(dynamic, 256)
  for (int64_t i = 0; i < (int64_t)nrays; ++i) {
    const float *r = rays8 + 8 * i;
    Ray ray(Vec(r[0], r[1], r[2]), Vec(r[4], r[5], r[6]));
    double t;
    Vec N;
    int id;
    bool hit = bvhAccelT->intersectT(ray, t, N, id);
    hit_id[i] = hit ? (uint32_t)triangleList[id].c.x : 0xFFFFFFFFu;
    hit_t[i] = hit ? t : 1e20;
  }
}

// shadow() with dist = tmax + 1e-5: occluded iff a hit has t < tmax.
void ref_trace_shadow(const float *rays8, uint32_t nrays, uint8_t *occluded, int threads) {
  if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel for schedule(dynamic, 256)
  for (int64_t i = 0; i < (int64_t)nrays; ++i) {
    const float *r = rays8 + 8 * i;
    Ray ray(Vec(r[0], r[1], r[2]), Vec(r[4], r[5], r[6]));
    occluded[i] = shadow(ray, (double)r[7] + 1e-5) < 0.5 ? 1 : 0;
  }
}

// ---- materials and LTC shading ------------------------------------------
// Row layout shared with orc_material (oracle/ckr_oracle.h).
struct RefMaterialRow {
  int32_t brdf;
  int32_t pad;
  double alpha, phong_exp, spec, int_ior, ext_ior;
};

static MaterialType make_material(const RefMaterialRow &r) {
  if (r.brdf == CLASSIC_PHONG) return MaterialType(r.phong_exp, r.spec);
  return MaterialType(r.alpha, r.int_ior, r.ext_ior, r.spec, (BRDFType)r.brdf);
}

// MaterialType::brdf (optionally with getBrdfApproxParam(force) first) and pdfEval.
void ref_brdf_batch(const RefMaterialRow *m, uint32_t count, const double *n, const double *wo_ref,
                    const double *wo, const double *wi, int use_ltc, double *brdf_out, double *pdf_out) {
  for (uint32_t i = 0; i < count; ++i) {
    MaterialType mt = make_material(m[i]);
    Vec N(n[3 * i], n[3 * i + 1], n[3 * i + 2]), R(wo_ref[3 * i], wo_ref[3 * i + 1], wo_ref[3 * i + 2]);
    Vec O(wo[3 * i], wo[3 * i + 1], wo[3 * i + 2]), I(wi[3 * i], wi[3 * i + 1], wi[3 * i + 2]);
    BRDFApprox ap;
    if (use_ltc) mt.getBrdfApproxParam(N, O, ap, true);
    brdf_out[i] = mt.brdf(N, R, O, I, ap);
    if (pdf_out) pdf_out[i] = mt.pdfEval(N, R, O, I);
  }
}

}  // extern "C"

// ---- scene loading --------------------------------------------------------
// initSceneParser + prepareScreenCamera + prepareObjects + prepareLightSources,
// then the resulting global primitive lists.  Call once per process (the
// reference keeps them in globals and appends).  Per triangle 9 vertex
// doubles; per sphere centre + radius; per primitive 16 material doubles:
// brdf, light type, alpha, phongExp, specularCoef, intIOR, extIOR,
// reflectance, colour(3), radiance(3), pad(2).  cam: pos, dir, cx, cy, w, h.
extern "C" {

int ref_scene_load(const char *path, double *cam14, uint32_t *ntri, uint32_t *nsph) {
  if (!initSceneParser(path)) return -1;
  uint32_t w, h;
  Vec pos, dir, cx, cy;
  if (!prepareScreenCamera(w, h, pos, dir, cx, cy, false)) return -2;
  if (!prepareObjects(false)) return -3;
  if (!prepareLightSources(false)) return -4;
  Vec v[4] = {pos, dir, cx, cy};
  for (int k = 0; k < 4; ++k) {
    cam14[3 * k] = v[k].x;
    cam14[3 * k + 1] = v[k].y;
    cam14[3 * k + 2] = v[k].z;
  }
  cam14[12] = w;
  cam14[13] = h;
  *ntri = vTriangleList.size();
  *nsph = vSphereList.size();
  return 0;
}

static void dump_material(const BasePrimitive &p, double *m) {
  // MaterialType::b is private; brdf() of a probe direction is not needed:
  // the harness reads the type through the class layout's public neighbours.
  const MaterialType &mt = p.m;
  m[0] = -1;  // filled by the caller from the layout below
  m[1] = mt.l;
  m[2] = mt.alpha;
  m[3] = mt.phongExp;
  m[4] = mt.specularCoef;
  m[5] = mt.intIOR;
  m[6] = mt.extIOR;
  m[7] = p.reflectance;
  m[8] = p.c.x; m[9] = p.c.y; m[10] = p.c.z;
  m[11] = mt.radiance.x; m[12] = mt.radiance.y; m[13] = mt.radiance.z;
  m[14] = m[15] = 0;
}

void ref_scene_dump(double *tri9, double *sph4, double *tri_mat16, double *sph_mat16) {
  for (size_t i = 0; i < vTriangleList.size(); ++i) {
    const Triangle &t = vTriangleList[i];
    Vec v[3] = {t.A, t.B, t.C};
    for (int k = 0; k < 3; ++k) {
      tri9[9 * i + 3 * k] = v[k].x;
      tri9[9 * i + 3 * k + 1] = v[k].y;
      tri9[9 * i + 3 * k + 2] = v[k].z;
    }
    dump_material(t, tri_mat16 + 16 * i);
  }
  for (size_t i = 0; i < vSphereList.size(); ++i) {
    const Sphere &s = vSphereList[i];
    sph4[4 * i] = s.p.x;
    sph4[4 * i + 1] = s.p.y;
    sph4[4 * i + 2] = s.p.z;
    sph4[4 * i + 3] = s.r;
    dump_material(s, sph_mat16 + 16 * i);
  }
}

}  // extern "C"

// Defined in the reference's materialTypes.cpp (via headers/ltc.h); not declared in any header.
void M_GGX(const float theta, const float alpha, mat3 &M, mat3 &Minv, double &amplitude);

extern "C" {

void ref_m_ggx(float theta, float alpha, double *M9, double *detM, double *Minv9, double *amplitude) {
  mat3 M, Mi;
  M_GGX(theta, alpha, M, Mi, *amplitude);
  for (int k = 0; k < 9; ++k) {
    M9[k] = M.a[k];
    Minv9[k] = Mi.a[k];
  }
  *detM = M.det;
}

// LightSource::getLightFromMeshSource_Analytic for each shading point, with one
// mesh light made of the given emitter triangles (radiance light_rgb per triangle).
void ref_ltc_shade_batch(const RefMaterialRow *m, uint32_t count, const double *x, const double *n, const double *v,
                         const float *light_tri9, const float *light_rgb, uint32_t nlight, double *rgb,
                         int threads) {
  LightSource ls;
  MeshLight mesh;
  for (uint32_t i = 0; i < nlight; ++i) {
    const float *t = light_tri9 + 9 * (size_t)i;
    const float *c = light_rgb + 3 * (size_t)i;
    double mx = c[0] > c[1] ? c[0] : c[1];
    mx = mx > c[2] ? mx : c[2];
    mesh.add(TriLight(Vec(t[0], t[1], t[2]), Vec(t[3], t[4], t[5]), Vec(t[6], t[7], t[8]), Vec(c[0], c[1], c[2]),
                      mx));
  }
  mesh.initMeshLight();
  ls.addMSource(mesh);
  if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel for schedule(dynamic, 64)
  for (int64_t i = 0; i < (int64_t)count; ++i) {
    MaterialType mt = make_material(m[i]);
    Sphere prim(1.0, Vec(0, 0, 0), Vec(1, 1, 1), 1.0, mt);
    Vec X(x[3 * i], x[3 * i + 1], x[3 * i + 2]), N(n[3 * i], n[3 * i + 1], n[3 * i + 2]);
    Vec V(v[3 * i], v[3 * i + 1], v[3 * i + 2]);
    Ray r(X, V * -1.0);
    Vec out = ls.getLightFromMeshSource_Analytic(r, N, X, &prim);
    rgb[3 * i] = out.x;
    rgb[3 * i + 1] = out.y;
    rgb[3 * i + 2] = out.z;
  }
}

}  // extern "C"

// ---- P6 images: readImage / writeImage (src/ppm.cpp:36-152) ----------------
// The reference reads ./env1.ppm and writes ./env1_cpy.ppm; these run it with the
// working directory set to `dir` for the call.
#include <unistd.h>
#include "ppm.h"

extern "C" {

int ref_read_image(const char *dir, double *rgb, uint32_t cap_px, uint32_t *w, uint32_t *h) {
  char old[4096];
  if (!getcwd(old, sizeof(old)) || chdir(dir) != 0) return -1;
  Vec *image = 0;
  uint32_t ww = 0, hh = 0;
  int ok = readImage(image, ww, hh);
  if (chdir(old) != 0) return -1;
  if (!ok) return -2;
  *w = ww;
  *h = hh;
  if ((uint64_t)ww * hh > cap_px) return -3;
  for (uint64_t i = 0; i < (uint64_t)ww * hh; ++i) {
    rgb[3 * i] = image[i].x;
    rgb[3 * i + 1] = image[i].y;
    rgb[3 * i + 2] = image[i].z;
  }
  delete[] image;
  return 0;
}

int ref_write_image(const char *dir, const double *rgb, uint32_t w, uint32_t h) {
  char old[4096];
  if (!getcwd(old, sizeof(old)) || chdir(dir) != 0) return -1;
  std::vector<Vec> image((size_t)w * h);
  for (size_t i = 0; i < image.size(); ++i) image[i] = Vec(rgb[3 * i], rgb[3 * i + 1], rgb[3 * i + 2]);
  int ok = writeImage(image.data(), w, h);
  if (chdir(old) != 0) return -1;
  return ok ? 0 : -2;
}

}  // extern "C"

// ---- environment light: EnvSource (headers/lightSources.h:33-109) -------------
extern "C" {

// Builds EnvSource(image, w, h, axis, colour, intensity) -- whose constructor runs
// initSamples: the numeric normalisation area and the 200,000 importance-sampled
// directions -- then returns getRadiance for n directions, the area, and up to
// nsamp of its sampled directions.
int ref_env(const double *img, uint32_t w, uint32_t h, uint32_t axis, const double *col, double intensity,
            const double *dirs, uint32_t n, double *rgb, double *area, double *samples, uint32_t nsamp) {
  std::vector<Vec> image((size_t)w * h);
  for (size_t i = 0; i < image.size(); ++i) image[i] = Vec(img[3 * i], img[3 * i + 1], img[3 * i + 2]);
  EnvSource *e = new EnvSource(image.data(), w, h, axis, Vec(col[0], col[1], col[2]), intensity);
  for (uint32_t i = 0; i < n; ++i) {
    Vec L = e->getRadiance(Vec(dirs[3 * i], dirs[3 * i + 1], dirs[3 * i + 2]));
    rgb[3 * i] = L.x;
    rgb[3 * i + 1] = L.y;
    rgb[3 * i + 2] = L.z;
  }
  *area = e->normalizationArea;
  const uint32_t total = EnvSource::nSamples * EnvSource::multiplier;
  for (uint32_t i = 0; i < nsamp && i < total; ++i) {
    samples[3 * i] = e->impSamples[i].x;
    samples[3 * i + 1] = e->impSamples[i].y;
    samples[3 * i + 2] = e->impSamples[i].z;
  }
  delete[] e->envMap;
  delete e;
  return 0;
}

}  // extern "C"
