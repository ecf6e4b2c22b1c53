/*
 * orc_mlp.c — FP64 restatement of the learned light-selection network of the
 * CUDA renderer (chakumrender_gb300/csrc/mlp.cu).  TEST INFRASTRUCTURE ONLY.
 *
 * The network has no counterpart in the reference (which samples every light,
 * src/mis.cpp:100-146); this file is written from the mathematics:
 *
 *   features f (96): for each coordinate c of the normalised position
 *     p = (x - centre) * scale and each frequency k < 12: sin(2^k pi p_c),
 *     cos(2^k pi p_c) at 24c + 2k, 24c + 2k + 1; then the normal (72..74), the
 *     outgoing direction (75..77), the GGX roughness (78), the constant 1 (79,
 *     the first layer's bias), zeros (80..95);
 *   h1 = relu(W1 f), h2 = relu(W2 h1 + b2), h3 = relu(W3 h2 + b3),
 *   z = W4 h3 + b4, p = softmax of z over the first C entries (the clusters);
 *   loss over R records (f_r, cluster k_r, weight w_r >= 0):
 *     L = -(1/R) sum_r (w_r / mean(w)) log p_r[k_r],
 *   the Monte Carlo estimate of the cross-entropy between the distribution of the
 *   clusters' direct-light contributions and p; Adam (Kingma and Ba 2015).
 *
 * Parameter vector (ORC_MLP_NPARAMS doubles): W1 [64][96], W2 [64][64], b2 [64],
 * W3 [64][64], b3 [64], W4 [64][64], b4 [64], row-major [out][in].
 * Records are 12 floats: x.xyz, alpha, n.xyz, weight, wo.xyz, cluster (the bits
 * of a uint32).
 */
#include <math.h>
#include <stdint.h>
#include <string.h>

#include "ckr_oracle.h"

#define IN ORC_MLP_IN
#define H ORC_MLP_HIDDEN
#define OUT ORC_MLP_OUT

enum { OFF_W1 = 0, OFF_W2 = OFF_W1 + H * IN, OFF_B2 = OFF_W2 + H * H, OFF_W3 = OFF_B2 + H, OFF_B3 = OFF_W3 + H * H,
       OFF_W4 = OFF_B3 + H, OFF_B4 = OFF_W4 + OUT * H, OFF_END = OFF_B4 + OUT };

void orc_mlp_features(const float *rec, const double *centre, double scale, double *f) {
  for (int c = 0; c < 3; ++c) {
    double p = ((double)rec[c] - centre[c]) * scale;
    for (int k = 0; k < ORC_MLP_FREQS; ++k) {
      double a = ldexp(p, k) * 3.14159265358979323846;
      f[24 * c + 2 * k] = sin(a);
      f[24 * c + 2 * k + 1] = cos(a);
    }
  }
  for (int j = 0; j < 3; ++j) {
    f[72 + j] = rec[4 + j];
    f[75 + j] = rec[8 + j];
  }
  f[78] = rec[3];
  f[79] = 1.0;
  for (int j = 80; j < IN; ++j) f[j] = 0.0;
}

static void dense(const double *W, const double *b, const double *x, int nout, int nin, int relu, double *y) {
  for (int o = 0; o < nout; ++o) {
    double s = b ? b[o] : 0.0;
    for (int i = 0; i < nin; ++i) s += W[o * nin + i] * x[i];
    y[o] = relu && s < 0 ? 0.0 : s;
  }
}

static void forward1(const double *P, const double *f, uint32_t C, double *h1, double *h2, double *h3, double *p) {
  double z[OUT];
  dense(P + OFF_W1, NULL, f, H, IN, 1, h1);
  dense(P + OFF_W2, P + OFF_B2, h1, H, H, 1, h2);
  dense(P + OFF_W3, P + OFF_B3, h2, H, H, 1, h3);
  dense(P + OFF_W4, P + OFF_B4, h3, OUT, H, 0, z);
  double mx = -1e300;
  for (uint32_t j = 0; j < C; ++j) mx = z[j] > mx ? z[j] : mx;
  double sum = 0;
  for (uint32_t j = 0; j < OUT; ++j) {
    p[j] = j < C ? exp(z[j] - mx) : 0.0;
    sum += p[j];
  }
  for (uint32_t j = 0; j < OUT; ++j) p[j] /= sum;
}

void orc_mlp_forward(const double *params, const float *rec12, uint32_t n, const double *centre, double scale,
                     uint32_t nclusters, double *probs) {
  double f[IN], h1[H], h2[H], h3[H];
  for (uint32_t r = 0; r < n; ++r) {
    orc_mlp_features(rec12 + 12 * (size_t)r, centre, scale, f);
    forward1(params, f, nclusters, h1, h2, h3, probs + OUT * (size_t)r);
  }
}

int orc_mlp_loss_grad(const double *params, const float *rec12, uint32_t n, const double *centre, double scale,
                      uint32_t nclusters, double *grad, double *loss) {
  memset(grad, 0, sizeof(double) * OFF_END);
  *loss = 0;
  double wsum = 0;
  for (uint32_t r = 0; r < n; ++r) wsum += rec12[12 * (size_t)r + 7];
  if (!(wsum > 0) || n == 0) return 0;
  const double wbar = wsum / n;
  double f[IN], h1[H], h2[H], h3[H], p[OUT], g4[OUT], g3[H], g2[H], g1[H];
  for (uint32_t r = 0; r < n; ++r) {
    const float *rec = rec12 + 12 * (size_t)r;
    double w = rec[7];
    if (!(w > 0)) continue;
    uint32_t k;
    memcpy(&k, rec + 11, 4);
    orc_mlp_features(rec, centre, scale, f);
    forward1(params, f, nclusters, h1, h2, h3, p);
    double a = w / (wbar * n);
    *loss -= a * log(p[k]);
    for (int j = 0; j < OUT; ++j) g4[j] = j < (int)nclusters ? a * (p[j] - (j == (int)k ? 1.0 : 0.0)) : 0.0;
    for (int o = 0; o < OUT; ++o) {
      grad[OFF_B4 + o] += g4[o];
      for (int i = 0; i < H; ++i) grad[OFF_W4 + o * H + i] += g4[o] * h3[i];
    }
    for (int i = 0; i < H; ++i) {
      double s = 0;
      for (int o = 0; o < OUT; ++o) s += params[OFF_W4 + o * H + i] * g4[o];
      g3[i] = h3[i] > 0 ? s : 0.0;
    }
    for (int o = 0; o < H; ++o) {
      grad[OFF_B3 + o] += g3[o];
      for (int i = 0; i < H; ++i) grad[OFF_W3 + o * H + i] += g3[o] * h2[i];
    }
    for (int i = 0; i < H; ++i) {
      double s = 0;
      for (int o = 0; o < H; ++o) s += params[OFF_W3 + o * H + i] * g3[o];
      g2[i] = h2[i] > 0 ? s : 0.0;
    }
    for (int o = 0; o < H; ++o) {
      grad[OFF_B2 + o] += g2[o];
      for (int i = 0; i < H; ++i) grad[OFF_W2 + o * H + i] += g2[o] * h1[i];
    }
    for (int i = 0; i < H; ++i) {
      double s = 0;
      for (int o = 0; o < H; ++o) s += params[OFF_W2 + o * H + i] * g2[o];
      g1[i] = h1[i] > 0 ? s : 0.0;
    }
    for (int o = 0; o < H; ++o)
      for (int i = 0; i < IN; ++i) grad[OFF_W1 + o * IN + i] += g1[o] * f[i];
  }
  return 1;
}

void orc_mlp_adam(double *params, double *m, double *v, const double *grad, uint32_t n, uint32_t step, double lr,
                  double beta1, double beta2, double eps) {
  double c1 = 1.0 - pow(beta1, (double)step), c2 = 1.0 - pow(beta2, (double)step);
  for (uint32_t i = 0; i < n; ++i) {
    m[i] = beta1 * m[i] + (1.0 - beta1) * grad[i];
    v[i] = beta2 * v[i] + (1.0 - beta2) * grad[i] * grad[i];
    params[i] -= lr * (m[i] / c1) / (sqrt(v[i] / c2) + eps);
  }
}
