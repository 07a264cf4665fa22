// FP64 3D type-2 / type-1 NUFFT with the exponential-of-semicircle kernel:
// the reference's own tolerance (eps = 1e-12 in double,
// spinifel/extern/nufft_ext.py:62, finufft_ext.py:70-94), which an FP32 grid
// cannot reach (its floor is about 1e-7).  Kernel widths 2..16.
//
// Same layout and conventions as the FP32 plan of nufft.cu, in double:
//   fine   : n1*n2*n3 complex128, the upsampled grid (cuFFT Z2Z);
//   re_pad : Re of the type-2 fine grid with a periodic halo of
//            p = ceil(w/2)+1 cells per side (no modulo in the inner loops);
//   im_pad : Im (only when requested);
//   acc_pad: padded accumulator of type-1 spreading, folded before the FFT.
// Points (radians) map to fine-grid coordinate t = x n / (2 pi), wrapped into
// [-n/2, n/2); the footprint is l0 .. l0+w-1 with l0 = ceil(t - w/2).
//
// GB300 runs FP64 at about 1/64 of its FP32 rate, so these kernels are
// bound by the FP64 pipe (W^3 FMAs per point); the grid (tens of MB) stays
// in L2 and is read through L1 without shared-memory staging.
#include <cufft.h>
#include <math.h>

#include <vector>

#include "common.cuh"
#include "es_params.cuh"

struct spf_nufft64_plan_s {
  int dev = 0;
  int m[3] = {0, 0, 0};
  int n[3] = {0, 0, 0};
  int np[3] = {0, 0, 0};
  int pad = 0;
  int w = 0;
  double beta = 0, sigma = 2.0, eps = 1e-12;
  double *inv_p[3] = {nullptr, nullptr, nullptr};
  double2 *fine = nullptr;
  double *re_pad = nullptr;
  double *im_pad = nullptr;
  double *acc_pad = nullptr;
  cufftHandle fft = 0;
  bool fft_ok = false;
};

namespace spf {
namespace f64 {

struct Geom {
  int n1, n2, n3;
  int p1, p2, p3;
  int off1, off2, off3;
  double beta;
  double inv_half_w;
};

static Geom geom_of(const spf_nufft64_plan_s *P) {
  Geom g;
  g.n1 = P->n[0]; g.n2 = P->n[1]; g.n3 = P->n[2];
  g.p1 = P->np[0]; g.p2 = P->np[1]; g.p3 = P->np[2];
  g.off1 = P->n[0] / 2 + P->pad;
  g.off2 = P->n[1] / 2 + P->pad;
  g.off3 = P->n[2] / 2 + P->pad;
  g.beta = P->beta;
  g.inv_half_w = 2.0 / P->w;
  return g;
}

// Padded first index and the W kernel values along one axis for a point at
// x (radians) with grid scale s = n / (2 pi) (times the caller's coordinate
// scale); t is wrapped into [-n/2, n/2).
template <int W>
__device__ __forceinline__ int axis_setup(double x, double s, int n, int off, double beta,
                                          double inv_half_w, double *wt) {
  const double fn = (double)n;
  double t = __dmul_rn(x, s);
  t = __dsub_rn(t, __dmul_rn(fn, floor(__dadd_rn(__ddiv_rn(t, fn), 0.5))));
  const double l0 = ceil(__dsub_rn(t, 0.5 * W));
#pragma unroll
  for (int a = 0; a < W; ++a) {
    const double z = (l0 + (double)a - t) * inv_half_w;
    const double q = fmax(fma(-z, z, 1.0), 0.0);
    wt[a] = exp(beta * (sqrt(q) - 1.0));
  }
  return (int)l0 + off;
}

template <int W>
__device__ __forceinline__ double interp_point(const double *__restrict__ grid, const Geom &g,
                                               double x1, double s1, double x2, double s2,
                                               double x3, double s3) {
  double w1[W], w2[W], w3[W];
  const int i0 = axis_setup<W>(x1, s1, g.n1, g.off1, g.beta, g.inv_half_w, w1);
  const int j0 = axis_setup<W>(x2, s2, g.n2, g.off2, g.beta, g.inv_half_w, w2);
  const int k0 = axis_setup<W>(x3, s3, g.n3, g.off3, g.beta, g.inv_half_w, w3);
  double acc = 0.0;
#pragma unroll 1
  for (int a = 0; a < W; ++a) {
    double acc_a = 0.0;
    const double *plane = grid + ((size_t)(i0 + a) * g.p2 + j0) * g.p3 + k0;
#pragma unroll
    for (int b = 0; b < W; ++b) {
      const double *row = plane + (size_t)b * g.p3;
      double r = 0.0;
#pragma unroll
      for (int c = 0; c < W; ++c) r = fma(w3[c], __ldg(row + c), r);
      acc_a = fma(w2[b], r, acc_a);
    }
    acc = fma(w1[a], acc_a, acc);
  }
  return acc;
}

// Rotation of pixel position q by the inverse (transpose) of R(quat)
// (quat = [w,x,y,z]; spinifel/extern/nufft_ext.py:59-60 inverts the
// skopi quaternion2rot3d matrix), in double.
__device__ __forceinline__ void rotate_inv(const double *__restrict__ quat, double qx, double qy,
                                           double qz, double &h, double &k, double &l) {
  const double q0 = quat[0], q1 = quat[1], q2 = quat[2], q3 = quat[3];
  const double r00 = 1.0 - 2.0 * (q2 * q2 + q3 * q3), r01 = 2.0 * (q1 * q2 - q0 * q3),
               r02 = 2.0 * (q1 * q3 + q0 * q2);
  const double r10 = 2.0 * (q1 * q2 + q0 * q3), r11 = 1.0 - 2.0 * (q1 * q1 + q3 * q3),
               r12 = 2.0 * (q2 * q3 - q0 * q1);
  const double r20 = 2.0 * (q1 * q3 - q0 * q2), r21 = 2.0 * (q2 * q3 + q0 * q1),
               r22 = 1.0 - 2.0 * (q1 * q1 + q2 * q2);
  h = r00 * qx + r10 * qy + r20 * qz;
  k = r01 * qx + r11 * qy + r21 * qz;
  l = r02 * qx + r12 * qy + r22 * qz;
}

// b[k mod n] = f_k * support_k / (p1 p2 p3), complex fine grid pre-zeroed.
__global__ void k_scatter_modes(const double *__restrict__ f, const double *__restrict__ sup,
                                int m1, int m2, int m3, int n1, int n2, int n3,
                                const double *__restrict__ ip1, const double *__restrict__ ip2,
                                const double *__restrict__ ip3, double2 *__restrict__ fine) {
  const int64_t total = (int64_t)m1 * m2 * m3;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int c = (int)(idx % m3);
    const int b = (int)((idx / m3) % m2);
    const int a = (int)(idx / ((int64_t)m2 * m3));
    double v = f[idx];
    if (sup) v *= sup[idx];
    v *= ip1[a] * ip2[b] * ip3[c];
    const int fa = ((a - m1 / 2) % n1 + n1) % n1;
    const int fb = ((b - m2 / 2) % n2 + n2) % n2;
    const int fc = ((c - m3 / 2) % n3 + n3) % n3;
    fine[((int64_t)fa * n2 + fb) * n3 + fc] = make_double2(v, 0.0);
  }
}

// re_pad[i] = Re fine[(i - off) mod n] (and Im), every padded cell.
__global__ void k_fill_padded(const double2 *__restrict__ fine, Geom g,
                              double *__restrict__ re_pad, double *__restrict__ im_pad) {
  const int64_t total = (int64_t)g.p1 * g.p2 * g.p3;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int k = (int)(idx % g.p3);
    const int j = (int)((idx / g.p3) % g.p2);
    const int i = (int)(idx / ((int64_t)g.p2 * g.p3));
    const int a = ((i - g.off1) % g.n1 + g.n1) % g.n1;
    const int b = ((j - g.off2) % g.n2 + g.n2) % g.n2;
    const int c = ((k - g.off3) % g.n3 + g.n3) % g.n3;
    const double2 v = fine[((int64_t)a * g.n2 + b) * g.n3 + c];
    re_pad[idx] = v.x;
    if (im_pad) im_pad[idx] = v.y;
  }
}

template <int W>
__global__ void __launch_bounds__(128)
    k_interp(const double *__restrict__ re_pad, const double *__restrict__ im_pad, Geom g,
             const double *__restrict__ x, const double *__restrict__ y,
             const double *__restrict__ z, int64_t npts, double *__restrict__ out_re,
             double *__restrict__ out_im) {
  const double sc1 = g.n1 * (0.5 / M_PI), sc2 = g.n2 * (0.5 / M_PI), sc3 = g.n3 * (0.5 / M_PI);
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < npts;
       j += (int64_t)gridDim.x * blockDim.x) {
    out_re[j] = interp_point<W>(re_pad, g, x[j], sc1, y[j], sc2, z[j], sc3);
    if (out_im) out_im[j] = interp_point<W>(im_pad, g, x[j], sc1, y[j], sc2, z[j], sc3);
  }
}

// Slicing: point (o, p) = scale * R(q_o)^-1 ppr[:, p]; out[o * n_pix + p] = Re c.
template <int W>
__global__ void __launch_bounds__(128)
    k_slice(const double *__restrict__ re_pad, Geom g, const double *__restrict__ quats,
            const double *__restrict__ ppr, int64_t n_pix, double s1, double s2, double s3,
            double *__restrict__ out) {
  const int64_t o = blockIdx.x;
  const int64_t p = blockIdx.y * (int64_t)blockDim.x + threadIdx.x;
  if (p >= n_pix) return;
  double h, k, l;
  rotate_inv(quats + 4 * o, ppr[p], ppr[n_pix + p], ppr[2 * n_pix + p], h, k, l);
  out[o * n_pix + p] = interp_point<W>(re_pad, g, h, s1, k, s2, l, s3);
}

template <int W>
__global__ void __launch_bounds__(128)
    k_spread(double *__restrict__ acc_pad, Geom g, const double *__restrict__ x,
             const double *__restrict__ y, const double *__restrict__ z,
             const double *__restrict__ c, int64_t npts) {
  const double sc1 = g.n1 * (0.5 / M_PI), sc2 = g.n2 * (0.5 / M_PI), sc3 = g.n3 * (0.5 / M_PI);
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < npts;
       j += (int64_t)gridDim.x * blockDim.x) {
    double w1[W], w2[W], w3[W];
    const int i0 = axis_setup<W>(x[j], sc1, g.n1, g.off1, g.beta, g.inv_half_w, w1);
    const int j0 = axis_setup<W>(y[j], sc2, g.n2, g.off2, g.beta, g.inv_half_w, w2);
    const int k0 = axis_setup<W>(z[j], sc3, g.n3, g.off3, g.beta, g.inv_half_w, w3);
    const double cj = c[j];
#pragma unroll
    for (int q = 0; q < W; ++q) w3[q] *= cj;
#pragma unroll 1
    for (int a = 0; a < W; ++a) {
#pragma unroll 1
      for (int b = 0; b < W; ++b) {
        const double wab = w1[a] * w2[b];
        double *row = acc_pad + ((size_t)(i0 + a) * g.p2 + (j0 + b)) * g.p3 + k0;
#pragma unroll
        for (int q = 0; q < W; ++q) atomicAdd(row + q, wab * w3[q]);
      }
    }
  }
}

// fine[l] = sum of acc_pad[i] over padded i == l + off (mod n), Im = 0.
__global__ void k_fold(const double *__restrict__ acc_pad, Geom g, double2 *__restrict__ fine) {
  const int64_t total = (int64_t)g.n1 * g.n2 * g.n3;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int c = (int)(idx % g.n3);
    const int b = (int)((idx / g.n3) % g.n2);
    const int a = (int)(idx / ((int64_t)g.n2 * g.n3));
    // padded indices i = l + off - n*s for the s that keep i in [0, p)
    double v = 0.0;
    for (int i = (a + g.off1) % g.n1; i < g.p1; i += g.n1)
      for (int j = (b + g.off2) % g.n2; j < g.p2; j += g.n2)
        for (int k = (c + g.off3) % g.n3; k < g.p3; k += g.n3)
          v += acc_pad[((int64_t)i * g.p2 + j) * g.p3 + k];
    fine[idx] = make_double2(v, 0.0);
  }
}

// modes[k] = fine[k mod n] / (p1 p2 p3)
__global__ void k_extract(const double2 *__restrict__ fine, int m1, int m2, int m3, int n1,
                          int n2, int n3, const double *__restrict__ ip1,
                          const double *__restrict__ ip2, const double *__restrict__ ip3,
                          double *__restrict__ out_re, double *__restrict__ out_im) {
  const int64_t total = (int64_t)m1 * m2 * m3;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int c = (int)(idx % m3);
    const int b = (int)((idx / m3) % m2);
    const int a = (int)(idx / ((int64_t)m2 * m3));
    const int fa = ((a - m1 / 2) % n1 + n1) % n1;
    const int fb = ((b - m2 / 2) % n2 + n2) % n2;
    const int fc = ((c - m3 / 2) % n3 + n3) % n3;
    const double2 v = fine[((int64_t)fa * n2 + fb) * n3 + fc];
    const double s = ip1[a] * ip2[b] * ip3[c];
    out_re[idx] = v.x * s;
    if (out_im) out_im[idx] = v.y * s;
  }
}

#define SPF_W64_DISPATCH(w, KERNEL_CALL)                           \
  switch (w) {                                                     \
    case 2: { constexpr int W = 2; KERNEL_CALL; break; }           \
    case 3: { constexpr int W = 3; KERNEL_CALL; break; }           \
    case 4: { constexpr int W = 4; KERNEL_CALL; break; }           \
    case 5: { constexpr int W = 5; KERNEL_CALL; break; }           \
    case 6: { constexpr int W = 6; KERNEL_CALL; break; }           \
    case 7: { constexpr int W = 7; KERNEL_CALL; break; }           \
    case 8: { constexpr int W = 8; KERNEL_CALL; break; }           \
    case 9: { constexpr int W = 9; KERNEL_CALL; break; }           \
    case 10: { constexpr int W = 10; KERNEL_CALL; break; }         \
    case 11: { constexpr int W = 11; KERNEL_CALL; break; }         \
    case 12: { constexpr int W = 12; KERNEL_CALL; break; }         \
    case 13: { constexpr int W = 13; KERNEL_CALL; break; }         \
    case 14: { constexpr int W = 14; KERNEL_CALL; break; }         \
    case 15: { constexpr int W = 15; KERNEL_CALL; break; }         \
    case 16: { constexpr int W = 16; KERNEL_CALL; break; }         \
    default: set_error("unsupported kernel width %d", w); return SPF_ERR_UNSUPPORTED; \
  }

static int check_plan(spf_nufft64_plan P, const char *what) {
  if (!P) {
    set_error("%s: plan is NULL", what);
    return SPF_ERR_ARG;
  }
  int dev = -1;
  cudaGetDevice(&dev);
  if (dev != P->dev) {
    set_error("%s: plan was made on device %d, current device is %d", what, P->dev, dev);
    return SPF_ERR_ARG;
  }
  return SPF_OK;
}

static int fft_exec(spf_nufft64_plan P, int isign, cudaStream_t s, const char *what) {
  if (cufftSetStream(P->fft, s) != CUFFT_SUCCESS) {
    set_error("%s: cufftSetStream failed", what);
    return SPF_ERR_CUDA;
  }
  cufftResult r = cufftExecZ2Z(P->fft, reinterpret_cast<cufftDoubleComplex *>(P->fine),
                               reinterpret_cast<cufftDoubleComplex *>(P->fine),
                               isign < 0 ? CUFFT_FORWARD : CUFFT_INVERSE);
  if (r != CUFFT_SUCCESS) {
    set_error("%s: cufftExecZ2Z failed (%d)", what, (int)r);
    return SPF_ERR_CUDA;
  }
  count_launch();
  return SPF_OK;
}

// points per thread-block for the FP64 kernels, and the scale of the
// coordinate (radians) to the fine grid per axis
static void grid_scales(const spf_nufft64_plan_s *P, double scale, double *s) {
  for (int d = 0; d < 3; ++d) s[d] = scale * P->n[d] / (2.0 * M_PI);
}

}  // namespace f64
}  // namespace spf

using namespace spf;
using namespace spf::f64;

extern "C" {

int spf_nufft64_plan_create(int m1, int m2, int m3, double eps, double upsampfac,
                            spf_nufft64_plan *out) {
  SPF_REQUIRE(out != nullptr, "spf_nufft64_plan_create: out is NULL");
  *out = nullptr;
  SPF_REQUIRE(m1 > 0 && m2 > 0 && m3 > 0 && m1 <= 2048 && m2 <= 2048 && m3 <= 2048,
              "spf_nufft64_plan_create: bad mode counts (%d, %d, %d)", m1, m2, m3);
  SPF_REQUIRE(eps >= 1e-15 && eps < 1, "spf_nufft64_plan_create: eps must be in [1e-15, 1)");
  const double sigma = upsampfac <= 0 ? 2.0 : upsampfac;
  SPF_REQUIRE(sigma >= 1.25 && sigma <= 4.0, "spf_nufft64_plan_create: upsampfac out of range");
  auto *P = new spf_nufft64_plan_s();
  cudaGetDevice(&P->dev);
  P->m[0] = m1; P->m[1] = m2; P->m[2] = m3;
  P->eps = eps;
  P->sigma = sigma;
  P->w = es_width_for(eps, sigma, 2, 16);
  P->beta = es_beta_for(P->w, sigma);
  P->pad = (P->w + 1) / 2 + 1;
  for (int d = 0; d < 3; ++d) {
    int want = (int)ceil(sigma * P->m[d]);
    if (want < 2 * P->w) want = 2 * P->w;
    P->n[d] = es_next_smooth_even(want);
    P->np[d] = P->n[d] + 2 * P->pad;
  }
  int st = SPF_OK;
  const size_t nfine = (size_t)P->n[0] * P->n[1] * P->n[2];
  const size_t npad = (size_t)P->np[0] * P->np[1] * P->np[2];
  for (int d = 0; d < 3 && st == SPF_OK; ++d) {
    auto v = es_inverse_kernel_ft(P->m[d], P->n[d], P->w, P->beta);
    st = check_cuda(cudaMalloc(&P->inv_p[d], v.size() * sizeof(double)), "plan64_create");
    if (st == SPF_OK)
      st = check_cuda(cudaMemcpy(P->inv_p[d], v.data(), v.size() * sizeof(double),
                                 cudaMemcpyHostToDevice), "plan64_create");
  }
  if (st == SPF_OK) st = check_cuda(cudaMalloc(&P->fine, nfine * sizeof(double2)), "plan64_create");
  if (st == SPF_OK) st = check_cuda(cudaMalloc(&P->re_pad, npad * sizeof(double)), "plan64_create");
  if (st == SPF_OK) {
    cufftResult r = cufftPlan3d(&P->fft, P->n[0], P->n[1], P->n[2], CUFFT_Z2Z);
    if (r != CUFFT_SUCCESS) {
      set_error("plan64_create: cufftPlan3d(%d,%d,%d) failed (%d)", P->n[0], P->n[1], P->n[2],
                (int)r);
      st = r == CUFFT_ALLOC_FAILED ? SPF_ERR_OOM : SPF_ERR_CUDA;
    } else {
      P->fft_ok = true;
    }
  }
  if (st != SPF_OK) {
    spf_nufft64_plan_destroy(P);
    return st;
  }
  *out = P;
  return SPF_OK;
}

int spf_nufft64_plan_destroy(spf_nufft64_plan P) {
  if (!P) return SPF_OK;
  int prev = -1;
  cudaGetDevice(&prev);
  if (prev != P->dev) cudaSetDevice(P->dev);
  for (int d = 0; d < 3; ++d) cudaFree(P->inv_p[d]);
  cudaFree(P->fine);
  cudaFree(P->re_pad);
  cudaFree(P->im_pad);
  cudaFree(P->acc_pad);
  if (P->fft_ok) cufftDestroy(P->fft);
  if (prev != P->dev && prev >= 0) cudaSetDevice(prev);
  delete P;
  return SPF_OK;
}

int spf_nufft64_plan_info(spf_nufft64_plan P, int *n_fine, int *width, double *beta,
                          int *n_padded) {
  SPF_REQUIRE(P != nullptr, "spf_nufft64_plan_info: plan is NULL");
  for (int d = 0; d < 3; ++d) {
    if (n_fine) n_fine[d] = P->n[d];
    if (n_padded) n_padded[d] = P->np[d];
  }
  if (width) *width = P->w;
  if (beta) *beta = P->beta;
  return SPF_OK;
}

int spf_nufft64_t2_set_modes(spf_nufft64_plan P, const double *d_modes, const double *d_support,
                             int isign, int want_imag, void *stream) {
  SPF_TRY(check_plan(P, "spf_nufft64_t2_set_modes"));
  SPF_REQUIRE(d_modes != nullptr, "spf_nufft64_t2_set_modes: modes is NULL");
  SPF_REQUIRE(isign == 1 || isign == -1, "spf_nufft64_t2_set_modes: isign must be +-1");
  cudaStream_t s = as_stream(stream);
  const size_t nfine = (size_t)P->n[0] * P->n[1] * P->n[2];
  const size_t npad = (size_t)P->np[0] * P->np[1] * P->np[2];
  if (want_imag && !P->im_pad)
    SPF_TRY(check_cuda(cudaMalloc(&P->im_pad, npad * sizeof(double)), "spf_nufft64_t2_set_modes"));
  SPF_TRY(check_cuda(cudaMemsetAsync(P->fine, 0, nfine * sizeof(double2), s),
                     "spf_nufft64_t2_set_modes"));
  const int64_t nm = (int64_t)P->m[0] * P->m[1] * P->m[2];
  k_scatter_modes<<<grid_for(nm, 256, 8 * 1024), 256, 0, s>>>(
      d_modes, d_support, P->m[0], P->m[1], P->m[2], P->n[0], P->n[1], P->n[2], P->inv_p[0],
      P->inv_p[1], P->inv_p[2], P->fine);
  SPF_TRY(check_launch("k_scatter_modes (f64)"));
  SPF_TRY(fft_exec(P, isign, s, "spf_nufft64_t2_set_modes"));
  const Geom g = geom_of(P);
  k_fill_padded<<<grid_for((int64_t)npad, 256, 16 * 1024), 256, 0, s>>>(
      P->fine, g, P->re_pad, want_imag ? P->im_pad : nullptr);
  return check_launch("k_fill_padded (f64)");
}

int spf_nufft64_t2_interp(spf_nufft64_plan P, const double *d_x, const double *d_y,
                          const double *d_z, int64_t npts, double *d_out_re, double *d_out_im,
                          void *stream) {
  SPF_TRY(check_plan(P, "spf_nufft64_t2_interp"));
  SPF_REQUIRE(npts >= 0, "spf_nufft64_t2_interp: npts < 0");
  if (npts == 0) return SPF_OK;
  SPF_REQUIRE(d_x && d_y && d_z && d_out_re, "spf_nufft64_t2_interp: NULL pointer");
  SPF_REQUIRE(!d_out_im || P->im_pad,
              "spf_nufft64_t2_interp: imaginary output needs set_modes(want_imag=1)");
  cudaStream_t s = as_stream(stream);
  const Geom g = geom_of(P);
  const int grid = grid_for(npts, 128, (int64_t)sm_count() * 32);
  SPF_W64_DISPATCH(P->w, (k_interp<W><<<grid, 128, 0, s>>>(P->re_pad, P->im_pad, g, d_x, d_y,
                                                              d_z, npts, d_out_re, d_out_im)));
  return check_launch("k_interp (f64)");
}

int spf_slice_t2_f64(spf_nufft64_plan P, const double *d_quats, int64_t n_orient,
                     const double *d_ppr, int64_t n_pix, double scale, double *d_out,
                     void *stream) {
  SPF_TRY(check_plan(P, "spf_slice_t2_f64"));
  SPF_REQUIRE(n_orient >= 0 && n_pix >= 0, "spf_slice_t2_f64: negative size");
  if (n_orient == 0 || n_pix == 0) return SPF_OK;
  SPF_REQUIRE(d_quats && d_ppr && d_out, "spf_slice_t2_f64: NULL pointer");
  SPF_REQUIRE(n_orient < (1LL << 31) && n_pix <= 65535LL * 128, "spf_slice_t2_f64: size too large");
  cudaStream_t s = as_stream(stream);
  const Geom g = geom_of(P);
  double sc[3];
  grid_scales(P, scale, sc);
  const dim3 grid((unsigned)n_orient, (unsigned)((n_pix + 127) / 128));
  SPF_W64_DISPATCH(P->w, (k_slice<W><<<grid, 128, 0, s>>>(P->re_pad, g, d_quats, d_ppr, n_pix,
                                                             sc[0], sc[1], sc[2], d_out)));
  return check_launch("k_slice (f64)");
}

int spf_nufft64_t1_zero(spf_nufft64_plan P, void *stream) {
  SPF_TRY(check_plan(P, "spf_nufft64_t1_zero"));
  const size_t npad = (size_t)P->np[0] * P->np[1] * P->np[2];
  if (!P->acc_pad)
    SPF_TRY(check_cuda(cudaMalloc(&P->acc_pad, npad * sizeof(double)), "spf_nufft64_t1_zero"));
  return check_cuda(cudaMemsetAsync(P->acc_pad, 0, npad * sizeof(double), as_stream(stream)),
                    "spf_nufft64_t1_zero");
}

int spf_nufft64_t1_spread(spf_nufft64_plan P, const double *d_x, const double *d_y,
                          const double *d_z, const double *d_c, int64_t npts, void *stream) {
  SPF_TRY(check_plan(P, "spf_nufft64_t1_spread"));
  SPF_REQUIRE(P->acc_pad != nullptr, "spf_nufft64_t1_spread: call spf_nufft64_t1_zero first");
  SPF_REQUIRE(npts >= 0, "spf_nufft64_t1_spread: npts < 0");
  if (npts == 0) return SPF_OK;
  SPF_REQUIRE(d_x && d_y && d_z && d_c, "spf_nufft64_t1_spread: NULL pointer");
  cudaStream_t s = as_stream(stream);
  const Geom g = geom_of(P);
  const int grid = grid_for(npts, 128, (int64_t)sm_count() * 32);
  SPF_W64_DISPATCH(P->w, (k_spread<W><<<grid, 128, 0, s>>>(P->acc_pad, g, d_x, d_y, d_z, d_c,
                                                              npts)));
  return check_launch("k_spread (f64)");
}

int spf_nufft64_t1_finish(spf_nufft64_plan P, int isign, double *d_out_re, double *d_out_im,
                          void *stream) {
  SPF_TRY(check_plan(P, "spf_nufft64_t1_finish"));
  SPF_REQUIRE(P->acc_pad != nullptr, "spf_nufft64_t1_finish: call spf_nufft64_t1_zero first");
  SPF_REQUIRE(isign == 1 || isign == -1, "spf_nufft64_t1_finish: isign must be +-1");
  SPF_REQUIRE(d_out_re != nullptr, "spf_nufft64_t1_finish: out_re is NULL");
  cudaStream_t s = as_stream(stream);
  const Geom g = geom_of(P);
  const int64_t nfine = (int64_t)P->n[0] * P->n[1] * P->n[2];
  k_fold<<<grid_for(nfine, 256, 16 * 1024), 256, 0, s>>>(P->acc_pad, g, P->fine);
  SPF_TRY(check_launch("k_fold (f64)"));
  SPF_TRY(fft_exec(P, isign, s, "spf_nufft64_t1_finish"));
  const int64_t nm = (int64_t)P->m[0] * P->m[1] * P->m[2];
  k_extract<<<grid_for(nm, 256, 16 * 1024), 256, 0, s>>>(
      P->fine, P->m[0], P->m[1], P->m[2], P->n[0], P->n[1], P->n[2], P->inv_p[0], P->inv_p[1],
      P->inv_p[2], d_out_re, d_out_im);
  return check_launch("k_extract (f64)");
}

}  // extern "C"
