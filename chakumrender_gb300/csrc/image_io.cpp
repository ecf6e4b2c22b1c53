// image_io.cpp — scene and image files around the hot path: Wavefront OBJ geometry,
// binary P6 PPM images (read and write) and FP32 PFM images.
//
// OBJ follows the public format description (Wavefront "Object Files (.obj)"):
// `v x y z [w]` vertices, `f` polygons whose corners are `v`, `v/vt`, `v//vn` or
// `v/vt/vn` with 1-based or negative (relative) vertex indices; polygons are
// triangulated as fans around their first corner.  Other statements (vt, vn, g, o,
// s, usemtl, mtllib, l, p, ...) are skipped.  The reference carries an unused
// third-party loader (externLib/objectLoader) and no OBJ asset; this one is written
// from the format.
//
// P6 mirrors the reference's readImage / writeImage (src/ppm.cpp:36-152): "P6",
// optional comment lines, width, height, maxval 255 (others rejected), the rest of
// that line, then width x height x 3 bytes; reading maps byte b to b / 255,
// writing clamps to [0, 1] and truncates x * 255 (negative values, which the
// reference passes to an unsigned-char conversion, are clamped to 0 here).
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/ckr.h"

namespace {

bool read_file(const char *path, std::string &out) {
  FILE *f = std::fopen(path, "rb");
  if (!f) return false;
  char buf[1 << 16];
  size_t n;
  while ((n = std::fread(buf, 1, sizeof(buf), f)) > 0) out.append(buf, n);
  bool ok = !std::ferror(f);
  std::fclose(f);
  return ok;
}

// One pass over an OBJ text: calls emit(a, b, c) with vertex indices (0-based) of
// every fan triangle.  Returns CKR_OK or CKR_ERR_PARSE.
template <class Emit>
int parse_obj(const std::string &text, std::vector<float> &verts, Emit emit) {
  verts.clear();
  std::vector<long> poly;
  size_t pos = 0;
  const size_t end = text.size();
  while (pos < end) {
    size_t eol = text.find('\n', pos);
    if (eol == std::string::npos) eol = end;
    // Line continuation ("\" at the end) is not part of common OBJ output; a line is one statement.
    std::string line = text.substr(pos, eol - pos);
    pos = eol + 1;
    if (!line.empty() && line.back() == '\r') line.pop_back();
    const char *s = line.c_str();
    while (*s == ' ' || *s == '\t') ++s;
    if (s[0] == 'v' && (s[1] == ' ' || s[1] == '\t')) {
      char *p = const_cast<char *>(s + 2);
      for (int k = 0; k < 3; ++k) {
        char *q;
        double x = std::strtod(p, &q);
        if (q == p) return CKR_ERR_PARSE;
        verts.push_back((float)x);
        p = q;
      }
    } else if (s[0] == 'f' && (s[1] == ' ' || s[1] == '\t')) {
      poly.clear();
      const char *p = s + 2;
      for (;;) {
        while (*p == ' ' || *p == '\t') ++p;
        if (*p == 0 || *p == '#') break;
        char *q;
        long v = std::strtol(p, &q, 10);
        if (q == p || v == 0) return CKR_ERR_PARSE;
        const long nv = (long)(verts.size() / 3);
        long idx = v > 0 ? v - 1 : nv + v;  // negative: relative to the vertices read so far
        if (idx < 0 || idx >= nv) return CKR_ERR_PARSE;
        poly.push_back(idx);
        p = q;
        // Skip the /vt/vn part of the corner.
        while (*p && *p != ' ' && *p != '\t') {
          if (*p != '/' && *p != '-' && !std::isdigit((unsigned char)*p)) return CKR_ERR_PARSE;
          ++p;
        }
      }
      if (poly.size() < 3) return CKR_ERR_PARSE;
      for (size_t k = 1; k + 1 < poly.size(); ++k) emit(poly[0], poly[k], poly[k + 1]);
    }
  }
  return CKR_OK;
}

}  // namespace

extern "C" int ckr_obj_load(const char *path, float *tri9, uint32_t capacity, uint32_t *ntri) {
  if (!path || !ntri) return CKR_ERR_INVALID_ARGUMENT;
  std::string text;
  if (!read_file(path, text)) return CKR_ERR_IO;
  std::vector<float> verts;
  uint64_t count = 0;
  bool overflow = false;
  int st = parse_obj(text, verts, [&](long a, long b, long c) {
    if (tri9 && count < capacity) {
      float *t = tri9 + 9 * count;
      std::memcpy(t, &verts[3 * a], 12);
      std::memcpy(t + 3, &verts[3 * b], 12);
      std::memcpy(t + 6, &verts[3 * c], 12);
    } else if (tri9) {
      overflow = true;
    }
    ++count;
  });
  if (st != CKR_OK) return st;
  if (count > 0xFFFFFFFFull) return CKR_ERR_TOO_LARGE;
  *ntri = (uint32_t)count;
  return overflow ? CKR_ERR_TOO_LARGE : CKR_OK;
}

extern "C" int ckr_read_ppm_p6(const char *path, float *rgb, uint32_t capacity_px, uint32_t *width,
                               uint32_t *height) {
  if (!path || !width || !height) return CKR_ERR_INVALID_ARGUMENT;
  std::string d;
  if (!read_file(path, d)) return CKR_ERR_IO;
  size_t p = 0;
  auto skip_ws_comments = [&]() {
    for (;;) {
      while (p < d.size() && std::isspace((unsigned char)d[p])) ++p;
      if (p < d.size() && d[p] == '#') {
        while (p < d.size() && d[p] != '\n') ++p;
        continue;
      }
      return;
    }
  };
  auto number = [&](long &v) {
    skip_ws_comments();
    size_t q = p;
    while (q < d.size() && std::isdigit((unsigned char)d[q])) ++q;
    if (q == p || q - p > 9) return false;
    v = std::strtol(d.substr(p, q - p).c_str(), nullptr, 10);
    p = q;
    return true;
  };
  if (d.size() < 2 || d[0] != 'P' || d[1] != '6') return CKR_ERR_PARSE;
  p = 2;
  long w, h, maxval;
  if (!number(w) || !number(h) || !number(maxval)) return CKR_ERR_PARSE;
  if (w <= 0 || h <= 0 || maxval != 255) return CKR_ERR_PARSE;
  // As the reference (src/ppm.cpp:92): the rest of the maxval line, newline included.
  while (p < d.size() && d[p] != '\n') ++p;
  if (p >= d.size()) return CKR_ERR_PARSE;
  ++p;
  const uint64_t npx = (uint64_t)w * (uint64_t)h;
  if (npx > 0xFFFFFFFFull || d.size() - p < 3 * npx) return CKR_ERR_PARSE;
  *width = (uint32_t)w;
  *height = (uint32_t)h;
  if (!rgb) return CKR_OK;  // size query
  if (capacity_px < npx) return CKR_ERR_TOO_LARGE;
  const unsigned char *px = reinterpret_cast<const unsigned char *>(d.data() + p);
  for (uint64_t i = 0; i < 3 * npx; ++i) rgb[i] = (float)((double)px[i] / 255.0);
  return CKR_OK;
}

extern "C" int ckr_write_ppm_p6(const char *path, const float *rgb, uint32_t width, uint32_t height) {
  if (!path || !rgb || !width || !height) return CKR_ERR_INVALID_ARGUMENT;
  FILE *f = std::fopen(path, "wb");
  if (!f) return CKR_ERR_IO;
  std::fprintf(f, "P6\n%u %u\n255\n", width, height);
  std::vector<unsigned char> raw((size_t)width * height * 3);
  for (size_t i = 0; i < raw.size(); ++i) {
    double x = rgb[i];
    x = x > 1.0 ? 1.0 : (x > 0.0 ? x : 0.0);
    raw[i] = (unsigned char)(x * 255);
  }
  bool ok = std::fwrite(raw.data(), 1, raw.size(), f) == raw.size();
  return (std::fclose(f) == 0 && ok) ? CKR_OK : CKR_ERR_IO;
}

extern "C" int ckr_write_pfm(const char *path, const float *rgb, uint32_t width, uint32_t height) {
  if (!path || !rgb || !width || !height) return CKR_ERR_INVALID_ARGUMENT;
  FILE *f = std::fopen(path, "wb");
  if (!f) return CKR_ERR_IO;
  // PFM: "PF", size, scale (negative = little endian); rows stored bottom to top.
  uint16_t probe = 1;
  const bool little = *reinterpret_cast<const unsigned char *>(&probe) == 1;
  std::fprintf(f, "PF\n%u %u\n%s\n", width, height, little ? "-1.0" : "1.0");
  bool ok = true;
  for (uint32_t y = height; y-- > 0 && ok;)
    ok = std::fwrite(rgb + (size_t)y * width * 3, sizeof(float), (size_t)width * 3, f) == (size_t)width * 3;
  return (std::fclose(f) == 0 && ok) ? CKR_OK : CKR_ERR_IO;
}
