/*
 * orc_traverse.c — FP64 restatement of the reference's BVH build and
 * closest-hit / shadow traversal.  TEST INFRASTRUCTURE ONLY (see ckr_oracle.h).
 *
 * Follows, operation for operation and in the same evaluation order:
 *   Triangle ctor            headers/geometryPrimitives.h:61-79
 *   Triangle::intersect      src/geometryPrimitives.cpp:29-71
 *   Sphere::intersect        src/geometryPrimitives.cpp:12-27
 *   AABBox ctor/uNion/intersect/maximumExtent
 *                            src/geometryPrimitives.cpp:73-149
 *   PrimitiveInfo            headers/bvhAccel.h:5-12
 *   BvhAccel::recursiveBuild src/bvhAccel.cpp:24-93 (std::partition semantics
 *                            of libstdc++ for bidirectional iterators)
 *   BvhAccel::build/flatten  src/bvhAccel.cpp:95-149
 *   BvhAccel::intersectT     src/bvhAccel.cpp:200-248
 *   shadow()                 src/shader.cpp:76-97
 */
#include "ckr_oracle.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct { double x, y, z; } V3;

static inline V3 v3(double x, double y, double z) { V3 r = {x, y, z}; return r; }
static inline V3 vsub(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline V3 vadd(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline V3 vmul(V3 a, double s) { return v3(a.x * s, a.y * s, a.z * s); }
static inline double vdot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline V3 vcross(V3 a, V3 b) {
  return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
static inline V3 vnorm(V3 a) { return vmul(a, 1.0 / sqrt(a.x * a.x + a.y * a.y + a.z * a.z)); }
static inline double vget(V3 a, int k) { return k == 0 ? a.x : (k == 1 ? a.y : a.z); }
#define MIN_(a, b) ((a) < (b) ? (a) : (b))
#define MAX_(a, b) ((a) > (b) ? (a) : (b))

typedef struct { V3 lo, hi; } Box;

typedef struct {
  V3 A, B, C, n; /* n = normalize((C-A) x (B-A)) */
} Tri;

static Tri make_tri(const float *t9) {
  Tri t;
  t.A = v3(t9[0], t9[1], t9[2]);
  t.B = v3(t9[3], t9[4], t9[5]);
  t.C = v3(t9[6], t9[7], t9[8]);
  V3 n = vsub(t.B, t.A);
  V3 c = vsub(t.C, t.A);
  n = vcross(c, n);
  t.n = vnorm(n);
  return t;
}

/* src/geometryPrimitives.cpp:29-71 */
static double tri_intersect(const Tri *tr, V3 o, V3 d, double *margin, double *ddn) {
  double raydotn = vdot(d, tr->n);
  V3 N = tr->n;
  if (ddn) *ddn = fabs(raydotn);
  if (margin) *margin = -1.0;
  if (raydotn > 0) {
    N = vmul(tr->n, -1.0);
    raydotn = -raydotn;
  }
  if (raydotn * raydotn <= 1e-10) return ORC_INF;
  double t = vdot(vsub(tr->A, o), N) / raydotn;
  if (t < 0) return ORC_INF;
  V3 P = vadd(o, vmul(d, t));
  V3 v0 = vsub(P, tr->A);
  V3 v1 = vsub(tr->B, tr->A);
  V3 v2 = vsub(tr->C, tr->A);
  double k0 = vdot(v0, v1);
  double k1 = vdot(v0, v2);
  double b0 = vdot(v1, v1);
  double b1 = vdot(v1, v2);
  double c0 = vdot(v2, v1);
  double c1 = vdot(v2, v2);
  double gamma = (k0 * b1 - k1 * b0) / (c0 * b1 - c1 * b0);
  double beta = (k0 - gamma * c0) / b0;
  if (margin) {
    double m = MIN_(beta, gamma);
    m = MIN_(m, 1.0 - beta - gamma);
    *margin = m;
  }
  if (gamma + beta > 1) return ORC_INF;
  else if (0 > gamma || gamma > 1) return ORC_INF;
  else if (0 > beta || beta > 1) return ORC_INF;
  return t;
}

double orc_tri_intersect(const float *tri9, const float *ray8, double *margin, double *ddotn) {
  Tri t = make_tri(tri9);
  return tri_intersect(&t, v3(ray8[0], ray8[1], ray8[2]), v3(ray8[4], ray8[5], ray8[6]), margin, ddotn);
}

/* src/geometryPrimitives.cpp:12-27 */
double orc_sphere_intersect(const double *c3, double r, const double *o3, const double *d3) {
  V3 op = v3(c3[0] - o3[0], c3[1] - o3[1], c3[2] - o3[2]);
  V3 d = v3(d3[0], d3[1], d3[2]);
  double t;
  double b = vdot(op, d);
  double det = b * b - vdot(op, op) + r * r;
  if (det < 0) return ORC_INF;
  det = sqrt(det);
  return (t = b - det) > 1e-4 ? t : ((t = b + det) > 1e-4 ? t : ORC_INF);
}

/* src/geometryPrimitives.cpp:107-139: slab test returning t0 (may be < 0). */
static double box_intersect(const Box *b, V3 o, V3 d) {
  double t0 = -ORC_INF, t1 = ORC_INF, tmp;
  double inv, tn, tf;
#define SLAB(c)                                              \
  inv = 1. / d.c;                                            \
  tn = (b->lo.c - o.c) * inv;                                \
  tf = (b->hi.c - o.c) * inv;                                \
  if (tn > tf) { tmp = tn; tn = tf; tf = tmp; }              \
  t0 = tn > t0 ? tn : t0;                                    \
  t1 = tf < t1 ? tf : t1;                                    \
  if (t0 > t1) return ORC_INF;
  SLAB(x) SLAB(y) SLAB(z)
#undef SLAB
  return t0;
}

static Box box_pts(V3 p1, V3 p2) {
  Box b;
  b.lo = v3(MIN_(p1.x, p2.x), MIN_(p1.y, p2.y), MIN_(p1.z, p2.z));
  b.hi = v3(MAX_(p1.x, p2.x), MAX_(p1.y, p2.y), MAX_(p1.z, p2.z));
  return b;
}
static Box box_union_pt(Box b, V3 p) {
  Box r = b;
  r.lo.x = MIN_(b.lo.x, p.x); r.lo.y = MIN_(b.lo.y, p.y); r.lo.z = MIN_(b.lo.z, p.z);
  r.hi.x = MAX_(b.hi.x, p.x); r.hi.y = MAX_(b.hi.y, p.y); r.hi.z = MAX_(b.hi.z, p.z);
  return r;
}
static Box box_union(Box a, Box b) {
  Box r = b;
  r.lo.x = MIN_(a.lo.x, b.lo.x); r.lo.y = MIN_(a.lo.y, b.lo.y); r.lo.z = MIN_(a.lo.z, b.lo.z);
  r.hi.x = MAX_(a.hi.x, b.hi.x); r.hi.y = MAX_(a.hi.y, b.hi.y); r.hi.z = MAX_(a.hi.z, b.hi.z);
  return r;
}
static int max_extent(Box b) {
  V3 d = vsub(b.hi, b.lo);
  if (d.x > d.y && d.x > d.z) return 0;
  else if (d.y > d.z) return 1;
  return 2;
}

typedef struct { Box box; uint32_t idx; V3 centroid; } PInfo;

typedef struct BNode {
  Box bounds;
  struct BNode *child[2];
  uint32_t axis, first, nprims;
} BNode;

typedef struct {
  Box bounds;
  uint32_t offset; /* leaf: first primitive; interior: second child */
  uint32_t nprims; /* 0 = interior */
  uint32_t axis;
} LNode;

struct orc_bvh {
  Tri *tris;          /* in BVH (reordered) order */
  uint32_t *order;    /* BVH position -> original triangle index */
  uint32_t ntri;
  LNode *nodes;
  uint32_t nnodes;
};

typedef struct {
  PInfo *info;
  uint32_t *order;
  uint32_t norder;
  uint32_t total;
  BNode *pool;
  uint32_t npool;
} BuildCtx;

static void make_leaf(BuildCtx *c, BNode *node, uint32_t start, uint32_t end, Box bbox) {
  node->first = c->norder;
  for (uint32_t i = start; i < end; ++i) c->order[c->norder++] = c->info[i].idx;
  node->nprims = end - start;
  node->bounds = bbox;
}

/* src/bvhAccel.cpp:24-93 */
static BNode *recursive_build(BuildCtx *c, uint32_t start, uint32_t end) {
  BNode *node = &c->pool[c->npool++];
  memset(node, 0, sizeof(*node));
  c->total++;
  Box bbox = c->info[start].box;
  for (uint32_t i = start + 1; i < end; ++i) bbox = box_union(bbox, c->info[i].box);
  uint32_t n = end - start;
  if (n == 1) {
    make_leaf(c, node, start, end, bbox);
    return node;
  }
  Box cb;
  cb.lo = cb.hi = c->info[start].centroid;
  for (uint32_t i = start + 1; i < end; ++i) cb = box_union_pt(cb, c->info[i].centroid);
  int dim = max_extent(cb);
  if ((cb.hi.x == cb.lo.x && dim == 0) || (cb.hi.y == cb.lo.y && dim == 1) ||
      (cb.hi.z == cb.lo.z && dim == 2)) {
    make_leaf(c, node, start, end, bbox);
    return node;
  }
  V3 pmid = vmul(vadd(cb.lo, cb.hi), 0.5);
  double m = vget(pmid, dim);
  /* libstdc++ std::partition on bidirectional iterators: scan from the front
   * for an element failing the predicate, from the back for one passing it,
   * swap, repeat. */
  PInfo *first = c->info + start, *last = c->info + end;
  for (;;) {
    for (;;) {
      if (first == last) goto done;
      if (vget(first->centroid, dim) < m) ++first; else break;
    }
    --last;
    for (;;) {
      if (first == last) goto done;
      if (!(vget(last->centroid, dim) < m)) --last; else break;
    }
    PInfo tmp = *first; *first = *last; *last = tmp;
    ++first;
  }
done:;
  uint32_t mid = (uint32_t)(first - c->info);
  if (mid == end || mid == start) {
    make_leaf(c, node, start, end, bbox);
    return node;
  }
  node->child[0] = recursive_build(c, start, mid);
  node->child[1] = recursive_build(c, mid, end);
  node->bounds = box_union(node->child[0]->bounds, node->child[1]->bounds);
  node->axis = (uint32_t)dim;
  node->nprims = 0;
  return node;
}

/* src/bvhAccel.cpp:126-143 */
static uint32_t flatten(orc_bvh *b, BNode *node, uint32_t *offset) {
  LNode *ln = &b->nodes[*offset];
  ln->bounds = node->bounds;
  uint32_t my = (*offset)++;
  if (node->nprims > 0) {
    ln->offset = node->first;
    ln->nprims = node->nprims;
  } else {
    ln->axis = node->axis;
    ln->nprims = 0;
    flatten(b, node->child[0], offset);
    ln->offset = flatten(b, node->child[1], offset);
  }
  return my;
}

orc_bvh *orc_bvh_build(const float *tri9, uint32_t ntri) {
  if (ntri == 0) return NULL;
  orc_bvh *b = (orc_bvh *)calloc(1, sizeof(orc_bvh));
  BuildCtx c;
  memset(&c, 0, sizeof(c));
  c.info = (PInfo *)malloc(sizeof(PInfo) * ntri);
  c.order = (uint32_t *)malloc(sizeof(uint32_t) * ntri);
  c.pool = (BNode *)malloc(sizeof(BNode) * (2 * (size_t)ntri));
  Tri *orig = (Tri *)malloc(sizeof(Tri) * ntri);
  if (!b || !c.info || !c.order || !c.pool || !orig) return NULL;
  for (uint32_t i = 0; i < ntri; ++i) {
    orig[i] = make_tri(tri9 + 9 * (size_t)i);
    Box bx = box_union_pt(box_pts(orig[i].A, orig[i].B), orig[i].C);
    c.info[i].box = bx;
    c.info[i].idx = i;
    c.info[i].centroid = vadd(vmul(bx.lo, 0.5), vmul(bx.hi, 0.5));
  }
  BNode *root = recursive_build(&c, 0, ntri);
  b->ntri = ntri;
  b->order = c.order;
  b->tris = (Tri *)malloc(sizeof(Tri) * ntri);
  for (uint32_t i = 0; i < ntri; ++i) b->tris[i] = orig[c.order[i]];
  b->nnodes = c.total;
  b->nodes = (LNode *)calloc(c.total, sizeof(LNode));
  uint32_t off = 0;
  flatten(b, root, &off);
  free(orig);
  free(c.info);
  free(c.pool);
  return b;
}

void orc_bvh_free(orc_bvh *b) {
  if (!b) return;
  free(b->tris);
  free(b->order);
  free(b->nodes);
  free(b);
}

uint32_t orc_bvh_node_count(const orc_bvh *b) { return b ? b->nnodes : 0; }

/* src/bvhAccel.cpp:200-248 (with a deeper stack than the reference's 64 and
 * an overflow stop, since a midpoint tree is not depth-bounded). */
static uint32_t intersect_t(const orc_bvh *b, V3 o, V3 d, double *t_out,
                            uint32_t *nvis, uint32_t *ntest) {
  V3 inv = v3(1.0 / d.x, 1.0 / d.y, 1.0 / d.z);
  int neg[3] = {inv.x < 0, inv.y < 0, inv.z < 0};
  uint32_t todo[256];
  uint32_t top = 0, cur = 0, id = ORC_MISS;
  uint32_t visits = 0, tests = 0;
  double t = ORC_INF, dd;
  for (;;) {
    const LNode *node = &b->nodes[cur];
    visits++;
    if (box_intersect(&node->bounds, o, d) < ORC_INF) {
      if (node->nprims > 0) {
        for (uint32_t i = 0; i < node->nprims; ++i) {
          tests++;
          if ((dd = tri_intersect(&b->tris[node->offset + i], o, d, NULL, NULL)) != 0.0 && dd < t) {
            t = dd;
            id = node->offset + i;
          }
        }
        if (top == 0) break;
        cur = todo[--top];
      } else {
        if (top >= 255) break;
        if (neg[node->axis]) {
          todo[top++] = cur + 1;
          cur = node->offset;
        } else {
          todo[top++] = node->offset;
          cur = cur + 1;
        }
      }
    } else {
      if (top == 0) break;
      cur = todo[--top];
    }
  }
  *t_out = t;
  if (nvis) *nvis = visits;
  if (ntest) *ntest = tests;
  return id == ORC_MISS ? ORC_MISS : b->order[id];
}

/* One ray, FP64 origin/direction: BvhAccel::intersectT.  Returns the input
 * triangle index or ORC_MISS; *t = distance (ORC_INF on a miss). */
uint32_t orc_bvh_closest1(const orc_bvh *b, const double *o3, const double *d3, double *t) {
  if (!b) {
    *t = ORC_INF;
    return ORC_MISS;
  }
  return intersect_t(b, v3(o3[0], o3[1], o3[2]), v3(d3[0], d3[1], d3[2]), t, NULL, NULL);
}

static int nthreads(int threads) {
#ifdef _OPENMP
  return threads > 0 ? threads : omp_get_max_threads();
#else
  (void)threads;
  return 1;
#endif
}

void orc_trace_closest(const orc_bvh *b, const float *rays8, uint32_t nrays,
                       uint32_t *hit_id, double *hit_t,
                       uint32_t *nodes, uint32_t *tris, int threads) {
  int nt = nthreads(threads);
  (void)nt;
#pragma omp parallel for schedule(dynamic, 256) num_threads(nt)
  for (int64_t i = 0; i < (int64_t)nrays; ++i) {
    const float *r = rays8 + 8 * i;
    double t;
    uint32_t nv = 0, nx = 0;
    uint32_t id = intersect_t(b, v3(r[0], r[1], r[2]), v3(r[4], r[5], r[6]), &t, &nv, &nx);
    hit_id[i] = id;
    hit_t[i] = t;
    if (nodes) nodes[i] = nv;
    if (tris) tris[i] = nx;
  }
}

void orc_trace_shadow(const orc_bvh *b, const float *rays8, uint32_t nrays,
                      uint8_t *occluded, int threads) {
  int nt = nthreads(threads);
  (void)nt;
#pragma omp parallel for schedule(dynamic, 256) num_threads(nt)
  for (int64_t i = 0; i < (int64_t)nrays; ++i) {
    const float *r = rays8 + 8 * i;
    double t;
    double dist = (double)r[7] + 1e-5;
    uint32_t id = intersect_t(b, v3(r[0], r[1], r[2]), v3(r[4], r[5], r[6]), &t, NULL, NULL);
    occluded[i] = (id != ORC_MISS && t + 1e-5 < dist) ? 1 : 0;
  }
}

/* The sphere half of shade()'s closest hit (src/shader.cpp:16-51 over
 * BvhAccel::intersectS, src/bvhAccel.cpp:151-198): the nearest sphere by
 * Sphere::intersect.  A linear scan returns the same sphere as the
 * reference's sphere BVH except at exact ties. */
void orc_spheres_closest(const float *sph4, uint32_t nsph, const float *rays8, uint32_t nrays,
                         uint32_t *hit_id, double *hit_t) {
  for (uint32_t i = 0; i < nrays; ++i) {
    const float *r = rays8 + 8 * (size_t)i;
    double o[3] = {r[0], r[1], r[2]}, d[3] = {r[4], r[5], r[6]};
    double best = ORC_INF;
    uint32_t id = ORC_MISS;
    for (uint32_t k = 0; k < nsph; ++k) {
      double c[3] = {sph4[4 * k], sph4[4 * k + 1], sph4[4 * k + 2]};
      double t = orc_sphere_intersect(c, sph4[4 * k + 3], o, d);
      if (t != 0.0 && t < best) {
        best = t;
        id = k;
      }
    }
    hit_id[i] = id;
    hit_t[i] = best;
  }
}

/* Signed distance, in scene units, from the point where the ray meets the
 * triangle's plane to the triangle's boundary: negative inside (minus the
 * distance to the nearest edge), positive outside.  Used by the parity
 * checker to recognise rays that graze an edge or vertex, where FP32 and FP64
 * tests may legitimately disagree.  Returns 1e300 for rays parallel to the
 * plane. */
static double seg_dist(V3 p, V3 a, V3 b) {
  V3 ab = vsub(b, a), ap = vsub(p, a);
  double L = vdot(ab, ab);
  double s = L > 0 ? vdot(ap, ab) / L : 0.0;
  s = s < 0 ? 0 : (s > 1 ? 1 : s);
  V3 q = vsub(p, vadd(a, vmul(ab, s)));
  return sqrt(vdot(q, q));
}

double orc_tri_edge_distance(const float *tri9, const float *ray8, double *t_plane) {
  Tri tr = make_tri(tri9);
  V3 o = v3(ray8[0], ray8[1], ray8[2]), d = v3(ray8[4], ray8[5], ray8[6]);
  V3 e1 = vsub(tr.B, tr.A), e2 = vsub(tr.C, tr.A);
  V3 n = vcross(e1, e2);
  double dn = vdot(d, n);
  if (dn == 0.0 || vdot(n, n) == 0.0) return 1e300;
  double t = vdot(vsub(tr.A, o), n) / dn;
  if (t_plane) *t_plane = t;
  V3 p = vadd(o, vmul(d, t));
  double dist = seg_dist(p, tr.A, tr.B);
  double d2 = seg_dist(p, tr.B, tr.C), d3 = seg_dist(p, tr.C, tr.A);
  dist = d2 < dist ? d2 : dist;
  dist = d3 < dist ? d3 : dist;
  /* inside test by edge-function signs relative to n */
  double s0 = vdot(vcross(vsub(tr.B, tr.A), vsub(p, tr.A)), n);
  double s1 = vdot(vcross(vsub(tr.C, tr.B), vsub(p, tr.B)), n);
  double s2 = vdot(vcross(vsub(tr.A, tr.C), vsub(p, tr.C)), n);
  int inside = (s0 >= 0 && s1 >= 0 && s2 >= 0) || (s0 <= 0 && s1 <= 0 && s2 <= 0);
  return inside ? -dist : dist;
}
