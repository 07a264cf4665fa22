// Host-side parameters of the exponential-of-semicircle (ES) NUFFT kernel
// phi(z) = exp(beta (sqrt(1 - z^2) - 1)) (Barnett, Magland & af Klinteberg
// 2019), shared by the FP32 and FP64 plans: fine-grid sizes, the width and
// shape for a tolerance, and the kernel's Fourier transform at the modes.
#pragma once

#include <math.h>

#include <vector>

namespace spf {

// Smallest even n' >= n whose only prime factors are 2, 3 and 5.
inline int es_next_smooth_even(int n) {
  if (n < 2) n = 2;
  if (n & 1) ++n;
  for (;; n += 2) {
    int m = n;
    for (int p : {2, 3, 5})
      while (m % p == 0) m /= p;
    if (m == 1) return n;
  }
}

// Gauss-Legendre nodes/weights on [-1, 1] by Newton iteration on P_q.
inline void es_gauss_legendre(int q, std::vector<double> &x, std::vector<double> &wt) {
  x.assign(q, 0.0);
  wt.assign(q, 0.0);
  for (int i = 0; i < q; ++i) {
    double z = cos(M_PI * (i + 0.75) / (q + 0.5));
    double dp = 1.0;
    for (int it = 0; it < 100; ++it) {
      double p0 = 1.0, p1 = z;
      for (int k = 2; k <= q; ++k) {
        double pk = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
        p0 = p1;
        p1 = pk;
      }
      dp = q * (z * p1 - p0) / (z * z - 1.0);
      double dz = p1 / dp;
      z -= dz;
      if (fabs(dz) < 1e-15) break;
    }
    x[i] = z;
    wt[i] = 2.0 / ((1.0 - z * z) * dp * dp);
  }
}

// Width for tolerance eps at upsampling sigma, clamped to [w_min, w_max].
inline int es_width_for(double eps, double sigma, int w_min, int w_max) {
  int w;
  if (sigma == 2.0) {
    w = (int)ceil(-log10(eps / 10.0));
  } else {
    w = (int)ceil(log(1.0 / eps) / (M_PI * sqrt(1.0 - 1.0 / sigma)));
  }
  if (w < w_min) w = w_min;
  if (w > w_max) w = w_max;
  return w;
}

inline double es_beta_for(int w, double sigma) {
  if (sigma == 2.0) {
    double bon = (w == 2) ? 2.20 : (w == 3) ? 2.26 : (w == 4) ? 2.38 : 2.30;
    return bon * w;
  }
  return 0.97 * M_PI * w * (1.0 - 1.0 / (2.0 * sigma));
}

// 1 / p(k) for the m centred modes k = -floor(m/2) .., where
// p(k) = int_{-w/2}^{w/2} phi(2t/w) cos(k h t) dt, h = 2 pi / n, by
// (4w + 40)-point Gauss-Legendre quadrature on [0, w/2] (phi is even).
inline std::vector<double> es_inverse_kernel_ft(int m, int n, int w, double beta) {
  std::vector<double> xq, wq;
  es_gauss_legendre(4 * w + 40, xq, wq);
  std::vector<double> out(m);
  double h = 2.0 * M_PI / n;
  for (int i = 0; i < m; ++i) {
    double k = (double)(i - m / 2);
    double s = 0.0;
    for (size_t q = 0; q < xq.size(); ++q) {
      double t = 0.25 * w * (xq[q] + 1.0);
      double z = 2.0 * t / w;
      double phi = exp(beta * (sqrt(fmax(1.0 - z * z, 0.0)) - 1.0));
      s += 0.25 * w * wq[q] * phi * cos(k * h * t);
    }
    out[i] = 1.0 / (2.0 * s);
  }
  return out;
}

}  // namespace spf
