/*
 * ORACLE -- test infrastructure only.  Nothing in the product path links,
 * loads or calls this file; only tests/, __graft_entry__.smoke() and the
 * CPU-baseline leg of bench.py use it, and only as the checker.
 *
 * FP64 CPU restatement of the 3D non-uniform FFT that Spinifel calls through
 * finufft / cufinufft (spinifel/extern/nufft_ext.py:248-327,420-487 and
 * spinifel/autocorrelation.py:32-61,97-128).  finufft itself is a git
 * submodule that is not checked out in the reference, so this restates the
 * published method (Barnett, Magland, af Klinteberg, "A parallel non-uniform
 * fast Fourier transform library based on an exponential of semicircle
 * kernel", SIAM J. Sci. Comput. 41(5), 2019):
 *
 *   type 2:  c_j = sum_k f_k exp(isign * i k.x_j)
 *   type 1:  f_k = sum_j c_j exp(isign * i k.x_j)
 *
 * with modes k in [-floor(m/2), ceil(m/2)-1] per axis (finufft mode order 0),
 * the first coordinate bound to axis 0 of a C-ordered array (the reference
 * swaps H and L before handing a C array to the Fortran-ordered library,
 * spinifel/extern/cufinufft_ext.py:120-122).
 *
 * This file holds the O(N) pieces (spreading and interpolation with the
 * kernel phi(z) = exp(beta (sqrt(1 - z^2) - 1)), |z| < 1) and the exact
 * direct sums used to pin them.  The FFT and deconvolution glue is numpy
 * (oracle/nufft.py).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

static inline double es_kernel(double z, double beta) {
  double s = 1.0 - z * z;
  if (s <= 0.0) return 0.0;
  return exp(beta * (sqrt(s) - 1.0));
}

double orc_es_kernel(double z, double beta) { return es_kernel(z, beta); }

/* Integer grid offsets and weights along one axis.  x is in radians; the
 * fine grid has n points with spacing 2 pi / n, index l <-> position l*h
 * (periodic).  Returns the first (unwrapped) index; w weights written. */
static inline long axis_weights(double x, int n, int w, double beta, double *wt) {
  double t = x * (double)n / (2.0 * M_PI);
  long l0 = (long)ceil(t - 0.5 * w);
  for (int a = 0; a < w; ++a) {
    double z = 2.0 * ((double)(l0 + a) - t) / (double)w;
    wt[a] = es_kernel(z, beta);
  }
  return l0;
}

static inline long wrap(long i, long n) {
  long r = i % n;
  return r < 0 ? r + n : r;
}

/* c_j = sum_l U_l phi(x_j - l h): complex fine grid U (interleaved re/im,
 * C order n1 x n2 x n3), output interleaved complex. */
void orc_interp(int n1, int n2, int n3, const double *U, int64_t npts,
                const double *x, const double *y, const double *z, int w,
                double beta, double *out) {
#pragma omp parallel for schedule(static)
  for (int64_t j = 0; j < npts; ++j) {
    double wx[32], wy[32], wz[32];
    long i0 = axis_weights(x[j], n1, w, beta, wx);
    long j0 = axis_weights(y[j], n2, w, beta, wy);
    long k0 = axis_weights(z[j], n3, w, beta, wz);
    double re = 0.0, im = 0.0;
    for (int a = 0; a < w; ++a) {
      long ia = wrap(i0 + a, n1);
      for (int b = 0; b < w; ++b) {
        long jb = wrap(j0 + b, n2);
        double wab = wx[a] * wy[b];
        const double *row = U + 2 * ((ia * n2 + jb) * (long)n3);
        double rr = 0.0, ri = 0.0;
        for (int c = 0; c < w; ++c) {
          long kc = wrap(k0 + c, n3);
          rr += wz[c] * row[2 * kc];
          ri += wz[c] * row[2 * kc + 1];
        }
        re += wab * rr;
        im += wab * ri;
      }
    }
    out[2 * j] = re;
    out[2 * j + 1] = im;
  }
}

/* G_l += c_j phi(x_j - l h): complex strengths c (interleaved), complex fine
 * grid G accumulated in place. */
void orc_spread(int n1, int n2, int n3, double *G, int64_t npts,
                const double *x, const double *y, const double *z,
                const double *c, int w, double beta) {
#pragma omp parallel for schedule(static)
  for (int64_t j = 0; j < npts; ++j) {
    double wx[32], wy[32], wz[32];
    long i0 = axis_weights(x[j], n1, w, beta, wx);
    long j0 = axis_weights(y[j], n2, w, beta, wy);
    long k0 = axis_weights(z[j], n3, w, beta, wz);
    double cr = c[2 * j], ci = c[2 * j + 1];
    for (int a = 0; a < w; ++a) {
      long ia = wrap(i0 + a, n1);
      for (int b = 0; b < w; ++b) {
        long jb = wrap(j0 + b, n2);
        double wab = wx[a] * wy[b];
        double *row = G + 2 * ((ia * n2 + jb) * (long)n3);
        for (int cc = 0; cc < w; ++cc) {
          long kc = wrap(k0 + cc, n3);
          double v = wab * wz[cc];
#pragma omp atomic
          row[2 * kc] += v * cr;
#pragma omp atomic
          row[2 * kc + 1] += v * ci;
        }
      }
    }
  }
}

/* Per-point 1D exponentials exp(isign i k x) for k = -floor(m/2) .. */
static void axis_exp(double x, int m, int isign, double *er, double *ei) {
  int k0 = -(m / 2);
  for (int a = 0; a < m; ++a) {
    double ph = (double)isign * (double)(k0 + a) * x;
    er[a] = cos(ph);
    ei[a] = sin(ph);
  }
}

/* Exact type 2: c_j = sum_k f_k exp(isign i k.x_j); f complex m1 x m2 x m3
 * C order, modes centred.  O(npts * m^3). */
void orc_nudft_t2(int m1, int m2, int m3, const double *f, int64_t npts,
                  const double *x, const double *y, const double *z,
                  int isign, double *out) {
#pragma omp parallel
  {
    double *e1 = (double *)malloc(sizeof(double) * 2 * (m1 + m2 + m3));
    double *e1r = e1, *e1i = e1 + m1;
    double *e2r = e1 + 2 * m1, *e2i = e2r + m2;
    double *e3r = e1 + 2 * (m1 + m2), *e3i = e3r + m3;
#pragma omp for schedule(static)
    for (int64_t j = 0; j < npts; ++j) {
      axis_exp(x[j], m1, isign, e1r, e1i);
      axis_exp(y[j], m2, isign, e2r, e2i);
      axis_exp(z[j], m3, isign, e3r, e3i);
      double sr = 0.0, si = 0.0;
      for (int a = 0; a < m1; ++a) {
        double ar = 0.0, ai = 0.0;
        for (int b = 0; b < m2; ++b) {
          const double *row = f + 2 * (((long)a * m2 + b) * m3);
          double br = 0.0, bi = 0.0;
          for (int c = 0; c < m3; ++c) {
            double fr = row[2 * c], fi = row[2 * c + 1];
            br += fr * e3r[c] - fi * e3i[c];
            bi += fr * e3i[c] + fi * e3r[c];
          }
          ar += br * e2r[b] - bi * e2i[b];
          ai += br * e2i[b] + bi * e2r[b];
        }
        sr += ar * e1r[a] - ai * e1i[a];
        si += ar * e1i[a] + ai * e1r[a];
      }
      out[2 * j] = sr;
      out[2 * j + 1] = si;
    }
    free(e1);
  }
}

/* Exact type 1: f_k = sum_j c_j exp(isign i k.x_j).  Parallel over the
 * first mode axis so that no two threads write the same output. */
void orc_nudft_t1(int m1, int m2, int m3, const double *c, int64_t npts,
                  const double *x, const double *y, const double *z,
                  int isign, double *f) {
  memset(f, 0, sizeof(double) * 2 * (size_t)m1 * m2 * m3);
#pragma omp parallel
  {
    double *e = (double *)malloc(sizeof(double) * 2 * (m2 + m3));
    double *e2r = e, *e2i = e + m2, *e3r = e + 2 * m2, *e3i = e3r + m3;
#pragma omp for schedule(static)
    for (int a = 0; a < m1; ++a) {
      double ka = (double)(a - m1 / 2);
      for (int64_t j = 0; j < npts; ++j) {
        double ph = (double)isign * ka * x[j];
        double pr = cos(ph), pi = sin(ph);
        double cr = c[2 * j] * pr - c[2 * j + 1] * pi;
        double ci = c[2 * j] * pi + c[2 * j + 1] * pr;
        axis_exp(y[j], m2, isign, e2r, e2i);
        axis_exp(z[j], m3, isign, e3r, e3i);
        for (int b = 0; b < m2; ++b) {
          double br = cr * e2r[b] - ci * e2i[b];
          double bi = cr * e2i[b] + ci * e2r[b];
          double *row = f + 2 * (((long)a * m2 + b) * m3);
          for (int cc = 0; cc < m3; ++cc) {
            row[2 * cc] += br * e3r[cc] - bi * e3i[cc];
            row[2 * cc + 1] += br * e3i[cc] + bi * e3r[cc];
          }
        }
      }
    }
    free(e);
  }
}

/* The CUDA KNN distance of the reference
 * (spinifel/sequential/orientation_matching_sp.cu:22-519): for every
 * (data image d, reference r) the sum over the first 16*floor(P/16) pixels
 * of (data - ref)^2, row-major [d][r].  FP64 accumulation. */
void orc_knn_eudist(const double *ref, const double *data, int64_t n_ref,
                    int64_t n_data, int64_t n_pix, double *out) {
  int64_t used = (n_pix / 16) * 16;
#pragma omp parallel for schedule(static)
  for (int64_t d = 0; d < n_data; ++d) {
    const double *xd = data + d * n_pix;
    for (int64_t r = 0; r < n_ref; ++r) {
      const double *xr = ref + r * n_pix;
      double s = 0.0;
      for (int64_t p = 0; p < used; ++p) {
        double t = xd[p] - xr[p];
        s += t * t;
      }
      out[d * n_ref + r] = s;
    }
  }
}
