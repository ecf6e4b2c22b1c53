// Exercises the per-ray forms of include/ckr_dropin.hpp the way the reference
// calls them (one ray at a time, from several OpenMP threads) and writes the
// answers for tests/test_dropin_gpu.py to check against the C ABI and the
// oracle.
//
//   dropin_queries <scene.xml> <rays.bin> <out.bin>
//
// rays.bin: uint32 n, then n x (o.xyz, d.xyz, dist) as float64.
// out.bin:  per ray: int32 idT, float64 tT, float64 N.xyz, int32 idS, float64 tS,
//           float64 shadow, float64 shade.xyz (per-ray shade, called twice: both
//           must agree), then n x int32 idT of the batched BvhAccel::intersect.
#include <cstdio>
#include <vector>

#include "ckr_dropin.hpp"

int main(int argc, char **argv) {
  if (argc != 4) return 2;
  if (!initSceneParser(argv[1])) return 3;
  uint32_t w, h;
  Vec pos, dir, cx, cy;
  if (!prepareScreenCamera(w, h, pos, dir, cx, cy, false) || !prepareObjects(false) || !prepareLightSources(false))
    return 3;
  loadAccels();
  loadLightSampler();
  FILE *f = std::fopen(argv[2], "rb");
  if (!f) return 4;
  uint32_t n = 0;
  if (std::fread(&n, 4, 1, f) != 1) return 4;
  std::vector<double> in(7 * (size_t)n);
  if (std::fread(in.data(), sizeof(double), in.size(), f) != in.size()) return 4;
  std::fclose(f);
  std::vector<Ray> rays;
  for (uint32_t i = 0; i < n; ++i)
    rays.push_back(Ray(Vec(in[7 * i], in[7 * i + 1], in[7 * i + 2]), Vec(in[7 * i + 3], in[7 * i + 4], in[7 * i + 5])));
  struct Out {
    int idT;
    double tT, N[3];
    int idS;
    double tS, shadow, shade[3];
  };
  std::vector<Out> out(n);
  int mismatched_shade = 0;
#pragma omp parallel for schedule(dynamic, 8) reduction(+ : mismatched_shade)
  for (int i = 0; i < (int)n; ++i) {
    Out &o = out[i];
    Vec N;
    double t;
    int id;
    o.idT = bvhAccelT->intersectT(rays[i], t, N, id) ? id : -1;
    o.tT = t;
    o.N[0] = N.x, o.N[1] = N.y, o.N[2] = N.z;
    o.idS = bvhAccelS->intersectS(rays[i], t, id) ? id : -1;
    o.tS = t;
    o.shadow = shadow(rays[i], in[7 * i + 6]);
    int depth = 2;
    Vec c1 = shade(rays[i], depth), c2 = shade(rays[i], depth);
    mismatched_shade += !(c1.x == c2.x && c1.y == c2.y && c1.z == c2.z);
    o.shade[0] = c1.x, o.shade[1] = c1.y, o.shade[2] = c1.z;
  }
  std::vector<double> tb(n);
  std::vector<int> idb(n);
  bvhAccelT->intersect(rays.data(), n, tb.data(), idb.data());
  f = std::fopen(argv[3], "wb");
  if (!f) return 5;
  for (const Out &o : out) {
    std::fwrite(&o.idT, 4, 1, f), std::fwrite(&o.tT, 8, 1, f), std::fwrite(o.N, 8, 3, f);
    std::fwrite(&o.idS, 4, 1, f), std::fwrite(&o.tS, 8, 1, f), std::fwrite(&o.shadow, 8, 1, f);
    std::fwrite(o.shade, 8, 3, f);
  }
  std::fwrite(idb.data(), 4, n, f);
  std::fclose(f);
  std::printf("rays %u, per-ray shade repeat mismatches %d, status %d\n", n, mismatched_shade,
              ckr_dropin::last_status());
  return mismatched_shade == 0 && ckr_dropin::last_status() == CKR_OK ? 0 : 6;
}
