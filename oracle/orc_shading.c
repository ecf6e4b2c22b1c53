/*
 * orc_shading.c — FP64 restatement of the reference's materials, direction
 * samplers and LTC polygon-light shading.  TEST INFRASTRUCTURE ONLY.
 *
 * Follows, in the same evaluation order:
 *   MaterialType::brdf / pdfEval / fresnel / ggxDist / ggxG1 / beckmannDist /
 *     beckmannG1 / phongG1 / approxLTC_BRDF / getBrdfApproxParam
 *                                    src/materialTypes.cpp:9-258
 *   mat3 (row-major, 9-arg and 3-column constructors store the transpose,
 *     cached det)                   headers/mathPrimitives.h:46-170
 *   M_GGX (64x64 table, lerp in theta only, det not refreshed)
 *                                    headers/ltc.h:18-61
 *   LightSource::integrateEdge, clipTriangle (both variants, including the
 *     x-only test on edge CA), getLightAnalyticDiffuse, getLightAnalytic,
 *     getLightFromMeshSource_Analytic
 *                                    src/lightSources_CV.cpp:8-333
 *   SphericalSampler direction samplers, with the table lookups replaced by
 *     the uniforms passed in       src/domainSampler.cpp:14-369
 * PI is the reference's 3.14159265359 (headers/mathPrimitives.h:4).
 */
#include "ckr_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define RPI 3.14159265359

typedef struct { double x, y, z; } V3;
static inline V3 v3(double x, double y, double z) { V3 r = {x, y, z}; return r; }
static inline V3 vsub(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline V3 vadd(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline V3 vmul(V3 a, double s) { return v3(a.x * s, a.y * s, a.z * s); }
static inline V3 vdiv(V3 a, double s) { return v3(a.x / s, a.y / s, a.z / s); }
static inline double vdot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline V3 vcross(V3 a, V3 b) { return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
static inline V3 vnorm(V3 a) { return vmul(a, 1.0 / sqrt(a.x * a.x + a.y * a.y + a.z * a.z)); }
static inline double vlen(V3 a) { return sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }
static inline V3 vld(const double *p) { return v3(p[0], p[1], p[2]); }
static inline V3 vldf(const float *p) { return v3(p[0], p[1], p[2]); }

/* ---- mat3 ------------------------------------------------------------- */
typedef struct { double a[9]; double det; } M3;

static void m3_calc_det(M3 *m) {
  const double *a = m->a;
  m->det = a[0] * (a[4] * a[8] - a[5] * a[7]) - a[1] * (a[3] * a[8] - a[5] * a[6]) + a[2] * (a[3] * a[7] - a[4] * a[6]);
}
/* mat3(a0..a8): stores the transpose (headers/mathPrimitives.h:151-165). */
static M3 m3_from9(const double *m) {
  M3 r;
  r.a[0] = m[0]; r.a[3] = m[1]; r.a[6] = m[2];
  r.a[1] = m[3]; r.a[4] = m[4]; r.a[7] = m[5];
  r.a[2] = m[6]; r.a[5] = m[7]; r.a[8] = m[8];
  m3_calc_det(&r);
  return r;
}
/* mat3(col0, col1, col2) (headers/mathPrimitives.h:137-149). */
static M3 m3_cols(V3 c0, V3 c1, V3 c2) {
  M3 r;
  r.a[0] = c0.x; r.a[3] = c0.y; r.a[6] = c0.z;
  r.a[1] = c1.x; r.a[4] = c1.y; r.a[7] = c1.z;
  r.a[2] = c2.x; r.a[5] = c2.y; r.a[8] = c2.z;
  m3_calc_det(&r);
  return r;
}
static M3 m3_transpose(M3 m) {
  M3 r;
  r.a[0] = m.a[0]; r.a[1] = m.a[3]; r.a[2] = m.a[6];
  r.a[3] = m.a[1]; r.a[4] = m.a[4]; r.a[5] = m.a[7];
  r.a[6] = m.a[2]; r.a[7] = m.a[5]; r.a[8] = m.a[8];
  r.det = m.det;
  return r;
}
static M3 m3_mul(M3 p, M3 m) {
  M3 r;
  const double *a = p.a;
  r.a[0] = a[0] * m.a[0] + a[1] * m.a[3] + a[2] * m.a[6];
  r.a[1] = a[0] * m.a[1] + a[1] * m.a[4] + a[2] * m.a[7];
  r.a[2] = a[0] * m.a[2] + a[1] * m.a[5] + a[2] * m.a[8];
  r.a[3] = a[3] * m.a[0] + a[4] * m.a[3] + a[5] * m.a[6];
  r.a[4] = a[3] * m.a[1] + a[4] * m.a[4] + a[5] * m.a[7];
  r.a[5] = a[3] * m.a[2] + a[4] * m.a[5] + a[5] * m.a[8];
  r.a[6] = a[6] * m.a[0] + a[7] * m.a[3] + a[8] * m.a[6];
  r.a[7] = a[6] * m.a[1] + a[7] * m.a[4] + a[8] * m.a[7];
  r.a[8] = a[6] * m.a[2] + a[7] * m.a[5] + a[8] * m.a[8];
  r.det = p.det * m.det;
  return r;
}
static V3 m3_mulv(const M3 *m, V3 v) {
  const double *a = m->a;
  return v3(a[0] * v.x + a[1] * v.y + a[2] * v.z, a[3] * v.x + a[4] * v.y + a[5] * v.z,
            a[6] * v.x + a[7] * v.y + a[8] * v.z);
}

/* ---- LTC table (headers/ltc.h, headers/ltc.inc) ------------------------ */
static int g_size = 0;
static double *g_tabM = NULL, *g_tabMinv = NULL;
static float *g_tabAmp = NULL;

int orc_ltc_load(const char *path) {
  FILE *f = fopen(path, "rb");
  if (!f) return -1;
  char magic[8];
  int hdr[2];
  if (fread(magic, 1, 8, f) != 8 || memcmp(magic, "CKRLTC1", 7) != 0 || fread(hdr, 4, 2, f) != 2) {
    fclose(f);
    return -2;
  }
  int n = hdr[0] * hdr[0];
  free(g_tabM); free(g_tabMinv); free(g_tabAmp);
  g_tabM = (double *)malloc(sizeof(double) * 9 * n);
  g_tabMinv = (double *)malloc(sizeof(double) * 9 * n);
  g_tabAmp = (float *)malloc(sizeof(float) * n);
  if (fread(g_tabM, 8, 9 * (size_t)n, f) != 9 * (size_t)n || fread(g_tabMinv, 8, 9 * (size_t)n, f) != 9 * (size_t)n ||
      fread(g_tabAmp, 4, (size_t)n, f) != (size_t)n) {
    fclose(f);
    return -3;
  }
  fclose(f);
  g_size = hdr[0];
  return 0;
}

typedef struct { M3 M, Minv; double amplitude; int is_set; } Approx; /* BRDFApprox */

/* headers/ltc.h:18-61 (theta and alpha are float parameters there too). */
static void m_ggx(float theta, float alpha, M3 *M, M3 *Minv, double *amplitude) {
  int size = g_size;
  int t = (int)floor(theta / (0.5 * RPI) * size);
  t = t < size - 1 ? t : size - 1;
  t = t > 0 ? t : 0;
  int a = (int)floor(sqrt(alpha) * size);
  a = a < size - 1 ? a : size - 1;
  a = a > 0 ? a : 0;
  int t1 = (size - 1) < (t + 1) ? (size - 1) : (t + 1);
  *M = m3_from9(g_tabM + 9 * (size_t)(a + t * size));
  *Minv = m3_from9(g_tabMinv + 9 * (size_t)(a + t * size));
  *amplitude = (double)g_tabAmp[a + t * size];
  if (t == t1) return;
  float mult = theta / (0.5 * RPI) * size - (float)t;
  M3 Mn = m3_from9(g_tabM + 9 * (size_t)(a + t1 * size));
  M3 Mi = m3_from9(g_tabMinv + 9 * (size_t)(a + t1 * size));
  double ampn = (double)g_tabAmp[a + t1 * size];
  for (int k = 0; k < 9; ++k) M->a[k] = M->a[k] + (Mn.a[k] - M->a[k]) * mult;
  for (int k = 0; k < 9; ++k) Minv->a[k] = Minv->a[k] + (Mi.a[k] - Minv->a[k]) * mult;
  *amplitude = *amplitude + (ampn - *amplitude) * mult;
}

void orc_m_ggx(float theta, float alpha, double *M9, double *detM, double *Minv9, double *amplitude) {
  M3 M, Mi;
  m_ggx(theta, alpha, &M, &Mi, amplitude);
  memcpy(M9, M.a, sizeof(M.a));
  memcpy(Minv9, Mi.a, sizeof(Mi.a));
  *detM = M.det;
}

/* ---- materials (src/materialTypes.cpp) --------------------------------- */
enum { B_NONE = 0, B_CLASSIC_PHONG, B_GGX, B_BECKMANN, B_PHONG, B_GGXAPPROX };

static double fresnel(const orc_material *m, double c) {
  double g = m->int_ior / m->ext_ior;
  g *= g;
  g += c * c - 1.0;
  g = sqrt(g);
  double t1 = g - c, t2 = g + c;
  double temp = c * t2 - 1.0;
  double F = temp * temp;
  temp = c * t1 + 1.0;
  F /= (temp * temp);
  F += 1.0;
  temp = t1 / t2;
  temp *= temp;
  F *= 0.5 * temp;
  return F;
}
static double ggx_dist(const orc_material *m, V3 h, V3 n) {
  double cs = vdot(h, n);
  cs *= cs;
  double ts = 1.0 / cs - 1.0;
  double as = m->alpha * m->alpha;
  ts += as;
  ts *= ts;
  return as / (RPI * cs * cs * ts);
}
static double ggx_g1(const orc_material *m, V3 v, V3 h, V3 n) {
  double cs = vdot(v, n);
  cs *= cs;
  double ts = 1.0 / cs - 1.0;
  if (ts <= 1e-15) return 1.0;
  else if (vdot(h, v) <= 1e-15) return 0;
  double as = m->alpha * m->alpha;
  ts *= as;
  ts += 1.0;
  ts = 1.0 + sqrt(ts);
  return 2.0 / ts;
}
static double beckmann_dist(const orc_material *m, V3 h, V3 n) {
  double cs = vdot(h, n);
  cs *= cs;
  double ts = 1.0 / cs - 1.0;
  double as = m->alpha * m->alpha;
  ts /= as;
  ts *= -1.0;
  return exp(ts) / (RPI * cs * cs * as);
}
static double rational_g1(double a) { return (3.535 * a + 2.181 * a * a) / (1.0 + 2.276 * a + 2.577 * a * a); }
static double beckmann_g1(const orc_material *m, V3 v, V3 h, V3 n) {
  double cs = vdot(v, n);
  cs *= cs;
  double a = 1.0 / (m->alpha * sqrt(1.0 / cs - 1.0));
  if (cs >= 0.999999) return 1.0;
  else if (vdot(h, v) <= 1e-15) return 0;
  if (a < 1.6) return rational_g1(a);
  return 1;
}
static double phong_g1(const orc_material *m, V3 v, V3 h, V3 n) {
  double cs = vdot(v, n);
  cs *= cs;
  double a = 0.5 * m->alpha + 1;
  a /= (1.0 / cs - 1.0);
  a = sqrt(a);
  if (cs >= 0.999999) return 1.0;
  else if (vdot(h, v) <= 1e-15) return 0;
  if (a < 1.6) return rational_g1(a);
  return 1;
}
static double approx_ltc_brdf(V3 wi, const Approx *ap) {
  V3 Lo = m3_mulv(&ap->Minv, wi);
  Lo = vnorm(Lo);
  V3 L_ = m3_mulv(&ap->M, Lo);
  double l = vlen(L_);
  double jac = ap->M.det / (l * l * l);
  double D = 1.0 / RPI * (0 > Lo.z ? 0 : Lo.z);
  return ap->amplitude * D / jac;
}
static double brdf_eval(const orc_material *m, V3 n, V3 wo_ref, V3 wo, V3 wi, const Approx *ap) {
  double spec = m->spec;
  if (ap && ap->is_set)
    return spec * approx_ltc_brdf(wi, ap) / vdot(wi, n) + (1 - spec) / RPI;
  if (m->brdf == B_CLASSIC_PHONG) {
    double c = vdot(wo_ref, wi);
    return (spec * (m->phong_exp + 1) * pow(c > 0 ? c : 0, m->phong_exp) / (2 * RPI)) + (1 - spec) / RPI;
  }
  if (m->brdf == B_GGX || m->brdf == B_BECKMANN || m->brdf == B_PHONG) {
    V3 h = vnorm(vadd(wo, wi));
    double F = fresnel(m, vdot(h, wi));
    double D, G;
    if (m->brdf == B_GGX) {
      D = ggx_dist(m, h, n);
      G = ggx_g1(m, wo, h, n) * ggx_g1(m, wi, h, n);
    } else if (m->brdf == B_BECKMANN) {
      D = beckmann_dist(m, h, n);
      G = beckmann_g1(m, wo, h, n) * beckmann_g1(m, wi, h, n);
    } else {
      D = (m->alpha + 2) * pow(vdot(h, n), m->alpha) / (2 * RPI);
      G = phong_g1(m, wo, h, n) * phong_g1(m, wi, h, n);
    }
    return (spec * F * D * G) / (4.0 * vdot(wi, n) * vdot(wo, n)) + (1 - spec) / RPI;
  }
  return 0.0; /* BRDF_NONE / GGXAPPROX without parameters: "Undefined BRDF" */
}
static double pdf_eval(const orc_material *m, V3 n, V3 wo_ref, V3 wo, V3 wi) {
  double diffuse = (1.0 - m->spec) * vdot(wi, n) / RPI;
  double spec = m->spec;
  if (m->brdf == B_CLASSIC_PHONG) {
    double c = vdot(wi, wo_ref);
    spec *= ((m->phong_exp + 1) * pow(c > 0 ? c : 0, m->phong_exp)) / (2 * RPI);
  } else if (m->brdf == B_GGX || m->brdf == B_BECKMANN || m->brdf == B_PHONG) {
    V3 h = vnorm(vadd(wo, wi));
    double D = 0;
    if (m->brdf == B_GGX) D = ggx_dist(m, h, n);
    else if (m->brdf == B_BECKMANN) D = beckmann_dist(m, h, n);
    else D = (m->alpha + 2) * pow(vdot(h, n), m->alpha) / (2 * RPI);
    spec *= D * vdot(h, n) / (4.0 * vdot(h, wo));
  }
  return spec + diffuse;
}
static void ref_frame(V3 n, V3 *X, V3 *Y);

/* src/materialTypes.cpp:52-74 */
static void brdf_approx_param(const orc_material *m, V3 n, V3 wo, int force, Approx *ap) {
  if (m->brdf == B_GGXAPPROX || (m->brdf == B_GGX && force)) {
    m_ggx((float)acos(vdot(n, wo)), (float)m->alpha, &ap->M, &ap->Minv, &ap->amplitude);
    V3 T1 = vsub(wo, vmul(n, vdot(n, wo)));
    if (vdot(T1, T1) == 0.0) {
      /* Exact normal incidence: the reference normalises a zero vector (NaN);
       * the fit is isotropic there, so take the sampling frame's X axis. */
      V3 Y;
      ref_frame(n, &T1, &Y);
    } else {
      T1 = vnorm(T1);
    }
    V3 T2 = vnorm(vcross(n, T1));
    M3 rot_inv = m3_transpose(m3_cols(T1, T2, n));
    ap->Minv = m3_mul(ap->Minv, rot_inv);
    ap->is_set = 1;
  } else {
    ap->is_set = 0;
  }
}

static V3 vrow(const double *p, size_t i) { return vld(p + 3 * i); }

void orc_brdf_batch(const orc_material *m, uint32_t count, const double *n, const double *wo_ref, const double *wo,
                    const double *wi, int use_ltc, double *brdf_out, double *pdf_out) {
  for (uint32_t i = 0; i < count; ++i) {
    const orc_material *mi = m + i;
    V3 N = vrow(n, i), R = vrow(wo_ref, i), O = vrow(wo, i), I = vrow(wi, i);
    Approx ap;
    memset(&ap, 0, sizeof(ap));
    if (use_ltc) brdf_approx_param(mi, N, O, 1, &ap);
    brdf_out[i] = brdf_eval(mi, N, R, O, I, use_ltc ? &ap : NULL);
    if (pdf_out) pdf_out[i] = pdf_eval(mi, N, R, O, I);
  }
}

/* ---- LTC polygon integration (src/lightSources_CV.cpp) ----------------- */
static double integrate_edge_n(V3 v1, V3 v2, V3 n) {
  double c = vdot(v1, v2);
  double th = acos(c);
  double d = vdot(vcross(v1, v2), n);
  return d * ((th > 0.001) ? th / sin(th) : 1.0);
}
static double integrate_edge_z(V3 v1, V3 v2) {
  double c = vdot(v1, v2);
  double th = acos(c);
  double d = vcross(v1, v2).z;
  return d * ((th > 0.001) ? th / sin(th) : 1.0);
}

/* General variant: plane through P with normal n (src/lightSources_CV.cpp:28-130). */
static int clip_triangle_n(V3 A, V3 B, V3 C, V3 n, V3 P, double nA, double nB, double nC, V3 *clip) {
  const double eps = 1e-15;
  int iab = 0, ibc = 0, ica = 0, idx = 0;
  V3 dAB = vsub(A, B), dBC = vsub(B, C), dCA = vsub(C, A);
  double nAB = vdot(n, dAB), nBC = vdot(n, dBC), nCA = vdot(n, dCA);
  double pA = vdot(n, vsub(P, A)), pB = vdot(n, vsub(P, B)), pC = vdot(n, vsub(P, C));
  double d;
  if (nAB * nAB > eps) {
    d = pA / nAB;
    V3 i = vadd(vmul(dAB, d), A);
    if (vdot(vsub(i, A), vsub(B, i)) > 0) {
      iab = 1;
      if (nA < 0) { clip[idx++] = i; clip[idx++] = B; }
      else { clip[idx++] = A; clip[idx++] = i; }
    }
  } else if (pA * pA < eps) return 0;
  if (nBC * nBC > eps) {
    d = pB / nBC;
    V3 i = vadd(vmul(dBC, d), B);
    if (vdot(vsub(i, B), vsub(C, i)) > 0) {
      ibc = 1;
      if (nB < 0) { clip[idx++] = i; clip[idx++] = C; }
      else { clip[idx++] = B; clip[idx++] = i; }
    }
  } else if (pB * pB < eps) return 0;
  if (nCA * nCA > eps) {
    d = pC / nCA;
    V3 i = vadd(vmul(dCA, d), C);
    /* The reference builds Vec(x, 0, 0) here (src/lightSources_CV.cpp:101-102). */
    double k1 = i.x - C.x, k2 = A.x - i.x;
    if (k1 * k2 > 0) {
      ica = 1;
      if (nC < 0) { clip[idx++] = i; clip[idx++] = A; }
      else { clip[idx++] = C; clip[idx++] = i; }
    }
  } else if (pC * pC < eps) return 0;
  return (iab + ibc + ica) > 1;
}

/* Simplified variant: plane z = 0 (src/lightSources_CV.cpp:133-219). */
static int clip_triangle_z(V3 A, V3 B, V3 C, double nA, double nB, double nC, V3 *clip) {
  const double eps = 1e-15;
  int iab = 0, ibc = 0, ica = 0, idx = 0;
  V3 dAB = vsub(A, B), dBC = vsub(B, C), dCA = vsub(C, A);
  double d;
  if (dAB.z * dAB.z > eps) {
    d = -A.z / dAB.z;
    V3 i = vadd(vmul(dAB, d), A);
    if (vdot(vsub(i, A), vsub(B, i)) > 0) {
      iab = 1;
      if (nA < 0) { clip[idx++] = i; clip[idx++] = B; }
      else { clip[idx++] = A; clip[idx++] = i; }
    }
  } else if (A.z * A.z < eps) return 0;
  if (dBC.z * dBC.z > eps) {
    d = -B.z / dBC.z;
    V3 i = vadd(vmul(dBC, d), B);
    if (vdot(vsub(i, B), vsub(C, i)) > 0) {
      ibc = 1;
      if (nB < 0) { clip[idx++] = i; clip[idx++] = C; }
      else { clip[idx++] = B; clip[idx++] = i; }
    }
  } else if (B.z * B.z < eps) return 0;
  if (dCA.z * dCA.z > eps) {
    d = -C.z / dCA.z;
    V3 i = vadd(vmul(dCA, d), C);
    double k1 = i.x - C.x, k2 = A.x - i.x;
    if (k1 * k2 > 0) {
      ica = 1;
      if (nC < 0) { clip[idx++] = i; clip[idx++] = A; }
      else { clip[idx++] = C; clip[idx++] = i; }
    }
  } else if (C.z * C.z < eps) return 0;
  return (iab + ibc + ica) > 1;
}

/* getLightAnalyticDiffuse (src/lightSources_CV.cpp:221-269) for one emitter
 * triangle: |sum of edge integrals| (before the 1/2pi and the radiance). */
static double ltc_diffuse_tri(V3 A, V3 B, V3 C, V3 n, V3 x) {
  V3 e1 = vnorm(vsub(A, x)), e2 = vnorm(vsub(B, x)), e3 = vnorm(vsub(C, x));
  double nA = vdot(e1, n), nB = vdot(e2, n), nC = vdot(e3, n);
  double sum = 0;
  if (nA > 0 && nB > 0 && nC > 0) {
    sum = integrate_edge_n(e1, e2, n);
    sum += integrate_edge_n(e2, e3, n);
    sum += integrate_edge_n(e3, e1, n);
  } else if (nA < 0 && nB < 0 && nC < 0) {
    return 0.0;
  } else {
    V3 clip[4];
    memset(clip, 0, sizeof(clip));
    if (!clip_triangle_n(A, B, C, n, x, nA, nB, nC, clip)) return 0.0;
    e1 = vnorm(vsub(clip[0], x));
    e2 = vnorm(vsub(clip[1], x));
    e3 = vnorm(vsub(clip[2], x));
    V3 e4 = vnorm(vsub(clip[3], x));
    sum = integrate_edge_n(e1, e2, n);
    sum += integrate_edge_n(e2, e3, n);
    sum += integrate_edge_n(e3, e4, n);
    sum += integrate_edge_n(e4, e1, n);
  }
  return sum > 0 ? sum : -sum;
}

/* getLightAnalytic (src/lightSources_CV.cpp:271-321) for one emitter triangle. */
static double ltc_spec_tri(V3 A, V3 B, V3 C, V3 x, const M3 *Minv) {
  V3 e1 = m3_mulv(Minv, vsub(A, x)), e2 = m3_mulv(Minv, vsub(B, x)), e3 = m3_mulv(Minv, vsub(C, x));
  double sum = 0;
  if (e1.z > 0 && e2.z > 0 && e3.z > 0) {
    e1 = vnorm(e1); e2 = vnorm(e2); e3 = vnorm(e3);
    sum = integrate_edge_z(e1, e2);
    sum += integrate_edge_z(e2, e3);
    sum += integrate_edge_z(e3, e1);
  } else if (e1.z < 0 && e2.z < 0 && e3.z < 0) {
    return 0.0;
  } else {
    V3 clip[4];
    memset(clip, 0, sizeof(clip));
    if (!clip_triangle_z(e1, e2, e3, e1.z / vlen(e1), e2.z / vlen(e2), e3.z / vlen(e3), clip)) return 0.0;
    e1 = vnorm(clip[0]); e2 = vnorm(clip[1]); e3 = vnorm(clip[2]);
    V3 e4 = vnorm(clip[3]);
    sum = integrate_edge_z(e1, e2);
    sum += integrate_edge_z(e2, e3);
    sum += integrate_edge_z(e3, e4);
    sum += integrate_edge_z(e4, e1);
  }
  return sum > 0 ? sum : -sum;
}

/* getLightFromMeshSource_Analytic (src/lightSources_CV.cpp:323-333) with the
 * view direction v = -r.d.  light_tri9/light_rgb: emitter triangles and their
 * radiance.  Writes the RGB result (without the primitive colour). */
void orc_ltc_shade(const orc_material *m, const double *x3, const double *n3, const double *v3_,
                   const float *light_tri9, const float *light_rgb, uint32_t nlight, double *rgb) {
  V3 x = vld(x3), n = vld(n3), wo = vld(v3_);
  Approx ap;
  memset(&ap, 0, sizeof(ap));
  brdf_approx_param(m, n, wo, 1, &ap);
  double spec[3] = {0, 0, 0}, diff[3] = {0, 0, 0};
  for (uint32_t i = 0; i < nlight; ++i) {
    const float *t = light_tri9 + 9 * (size_t)i;
    V3 A = vldf(t), B = vldf(t + 3), C = vldf(t + 6);
    double s = ap.is_set ? ltc_spec_tri(A, B, C, x, &ap.Minv) : 0.0;
    double d = ltc_diffuse_tri(A, B, C, n, x);
    for (int k = 0; k < 3; ++k) {
      spec[k] = spec[k] + light_rgb[3 * i + k] * s;
      diff[k] = diff[k] + light_rgb[3 * i + k] * d;
    }
  }
  for (int k = 0; k < 3; ++k) {
    double G = spec[k] / (2.0 * RPI) * ap.amplitude * m->spec;
    rgb[k] = G + diff[k] / (2.0 * RPI) * (1 - m->spec);
  }
}

void orc_ltc_shade_batch(const orc_material *m, uint32_t count, const double *x, const double *n, const double *v,
                         const float *light_tri9, const float *light_rgb, uint32_t nlight, double *rgb, int threads) {
  (void)threads;
#pragma omp parallel for schedule(dynamic, 64) num_threads(threads > 0 ? threads : 1)
  for (int64_t i = 0; i < (int64_t)count; ++i)
    orc_ltc_shade(m + i, x + 3 * i, n + 3 * i, v + 3 * i, light_tri9, light_rgb, nlight, rgb + 3 * i);
}

/* ---- direction samplers (src/domainSampler.cpp), one sample from uniforms */
/* Tangent frame of the reference (src/domainSampler.cpp:163-176). */
static void ref_frame(V3 n, V3 *X, V3 *Y) {
  V3 nx;
  if (n.x != 0) nx = v3((-n.y - n.z) / n.x, 1.0, 1.0);
  else if (n.y != 0) nx = v3(1.0, -n.z / n.y, 1.0);
  else nx = v3(1.0, 1.0, 0);
  *X = vnorm(nx);
  *Y = vnorm(vcross(n, *X));
}
static V3 to_world(V3 X, V3 Y, V3 Z, double x, double y, double z) {
  return v3(x * X.x + y * Y.x + z * Z.x, x * X.y + y * Y.y + z * Z.y, x * X.z + y * Y.z + z * Z.z);
}

/* kind: 0 cosine (getCosineDirectionSamples with the table's construction,
 * :29-40 and :154-189); 1..3 half-vector GGX/BECKMANN/PHONG
 * (getBrdfDirectionSamples :193-260, brdf = kind + 1); 4 classic Phong lobe
 * about w (:264-314); 5 cone of half-angle param about w
 * (getSolidDirectionSamples :320-369). */
void orc_sample_dir(int kind, const double *n3, const double *w3, double param, double e1, double e2, double *out3) {
  V3 n = vld(n3), w = w3 ? vld(w3) : n, X, Y, r;
  if (kind == 0) {
    ref_frame(n, &X, &Y);
    double th = asin(sqrt(e1)), ph = 2 * RPI * e2;
    r = to_world(X, Y, n, sin(th) * cos(ph), sin(th) * sin(ph), cos(th));
  } else if (kind >= 1 && kind <= 3) {
    ref_frame(n, &X, &Y);
    double ct = 0, st = 0;
    if (kind == 1) {
      double tt = param * sqrt(e1) / sqrt(1 - e1 + 1e-10);
      ct = 1.0 / sqrt(1 + tt * tt);
      st = tt * ct;
    } else if (kind == 2) {
      double tt = sqrt(param * param * log(1 - e1 + 1e-20) * -1.0);
      ct = 1.0 / sqrt(1 + tt * tt);
      st = tt * ct;
    } else {
      ct = pow(e1, 1.0 / (param + 2.0));
      st = sqrt(1.0 - ct * ct);
    }
    double ph = 2 * RPI * e2;
    V3 h = to_world(X, Y, n, st * cos(ph), st * sin(ph), ct);
    r = vnorm(vsub(vmul(h, 2.0 * vdot(h, w)), w));
  } else if (kind == 4) {
    ref_frame(w, &X, &Y);
    double ct = pow((1.0 - e1), 1.0 / (param + 1)), th = acos(ct), ph = 2 * RPI * e2;
    r = to_world(X, Y, w, sin(th) * cos(ph), sin(th) * sin(ph), ct);
  } else {
    ref_frame(w, &X, &Y);
    double A = 2.0 * RPI * (1 - cos(param));
    double ct = 1.0 - (A * e1) / (2.0 * RPI), th = acos(ct), ph = 2 * RPI * e2;
    r = to_world(X, Y, w, sin(th) * cos(ph), sin(th) * sin(ph), ct);
  }
  out3[0] = r.x; out3[1] = r.y; out3[2] = r.z;
}

#include "orc_render.inc"
