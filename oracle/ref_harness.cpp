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

}  // extern "C"
