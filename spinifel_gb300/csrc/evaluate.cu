// Reconstruction quality: Fourier shell correlation and volume alignment
// (eval/fsc.py, eval/align.py of the spinifel project), FP64.
//
// Alignment scores many candidate rotations of one volume against another:
// the reference materialises every rotated copy (scipy map_coordinates,
// order 1) and then takes Pearson correlations (align.py:36-120).  Here one
// kernel samples the rotated volume trilinearly on the fly and accumulates
// the correlation sums per rotation, so no rotated copy is stored; the
// volume being rotated is read through L1/L2 (8 neighbours per voxel).
// Sums use a fixed grid and order, so scores are reproducible.
#include <cufft.h>
#include <math.h>

#include "common.cuh"

namespace {

constexpr int SC_BLOCKS = 64;  // blocks per rotation (fixed: fixed summation order)
constexpr int SC_THREADS = 256;

struct Rot {
  double r[9];
};

// eval/geom.py:8-45 (same products and sums)
__device__ __forceinline__ Rot quat_rot(const double *q) {
  const double q01 = q[0] * q[1], q02 = q[0] * q[2], q03 = q[0] * q[3], q11 = q[1] * q[1],
               q12 = q[1] * q[2], q13 = q[1] * q[3], q22 = q[2] * q[2], q23 = q[2] * q[3],
               q33 = q[3] * q[3];
  Rot R;
  R.r[0] = 1. - 2. * (q22 + q33);
  R.r[1] = 2. * (q12 - q03);
  R.r[2] = 2. * (q13 + q02);
  R.r[3] = 2. * (q12 + q03);
  R.r[4] = 1. - 2. * (q11 + q33);
  R.r[5] = 2. * (q23 - q01);
  R.r[6] = 2. * (q13 - q02);
  R.r[7] = 2. * (q23 + q01);
  R.r[8] = 1. - 2. * (q11 + q22);
  return R;
}

// scipy.ndimage.map_coordinates(order=1, mode='constant', cval=0): a
// coordinate outside [0, M-1] on any axis gives 0, otherwise trilinear.
__device__ __forceinline__ double sample_linear(const double *__restrict__ v, int M, double u0,
                                                double u1, double u2) {
  const double top = (double)(M - 1);
  if (!(u0 >= 0.0 && u0 <= top && u1 >= 0.0 && u1 <= top && u2 >= 0.0 && u2 <= top)) return 0.0;
  const int i0 = min((int)floor(u0), M - 1), i1 = min((int)floor(u1), M - 1),
            i2 = min((int)floor(u2), M - 1);
  const double t0 = u0 - i0, t1 = u1 - i1, t2 = u2 - i2;
  const int j0 = min(i0 + 1, M - 1), j1 = min(i1 + 1, M - 1), j2 = min(i2 + 1, M - 1);
  const int64_t M2 = (int64_t)M * M;
  auto at = [&](int a, int b, int c) { return __ldg(v + a * M2 + (int64_t)b * M + c); };
  const double c00 = at(i0, i1, i2) * (1.0 - t2) + at(i0, i1, j2) * t2;
  const double c01 = at(i0, j1, i2) * (1.0 - t2) + at(i0, j1, j2) * t2;
  const double c10 = at(j0, i1, i2) * (1.0 - t2) + at(j0, i1, j2) * t2;
  const double c11 = at(j0, j1, i2) * (1.0 - t2) + at(j0, j1, j2) * t2;
  const double c0 = c00 * (1.0 - t1) + c01 * t1;
  const double c1 = c10 * (1.0 - t1) + c11 * t1;
  return c0 * (1.0 - t0) + c1 * t0;
}

// rotate_volume (align.py:36-67): output voxel f = (a*M + b)*M + c of the
// 'xy'-indexed meshgrid has (x, y, z) = (b, a, c) - M/2; T = R (x, y, z) +
// M/2 and the sample is taken at (T1, T0, T2).
__device__ __forceinline__ double rotated_at(const double *__restrict__ vol, int M, const Rot &R,
                                             int64_t f) {
  const int h = M / 2;
  const int c = (int)(f % M), b = (int)((f / M) % M), a = (int)(f / ((int64_t)M * M));
  const double x = (double)(b - h), y = (double)(a - h), z = (double)(c - h);
  const double T0 = R.r[0] * x + R.r[1] * y + R.r[2] * z + h;
  const double T1 = R.r[3] * x + R.r[4] * y + R.r[5] * z + h;
  const double T2 = R.r[6] * x + R.r[7] * y + R.r[8] * z + h;
  return sample_linear(vol, M, T1, T0, T2);
}

__device__ __forceinline__ double blk_sum(double v) {
  __shared__ double sh[SC_THREADS / 32];
  for (int o = 16; o >= 1; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) sh[w] = v;
  __syncthreads();
  v = 0.0;
  if (threadIdx.x < 32) {
    if (threadIdx.x < SC_THREADS / 32) v = sh[threadIdx.x];
    for (int o = 16; o >= 1; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  }
  __syncthreads();
  return v;
}

// partial[(q * SC_BLOCKS + b) * 3 + {0,1,2}] = sums of x, x^2, x y for rotation q
__global__ void __launch_bounds__(SC_THREADS)
    k_score_partial(const double *__restrict__ vol1, const double *__restrict__ vol2, int M,
                    const double *__restrict__ quats, double *__restrict__ partial) {
  const int q = blockIdx.y;
  const Rot R = quat_rot(quats + 4 * q);
  const int64_t n = (int64_t)M * M * M;
  double sx = 0.0, sxx = 0.0, sxy = 0.0;
  for (int64_t f = blockIdx.x * (int64_t)SC_THREADS + threadIdx.x; f < n;
       f += (int64_t)SC_BLOCKS * SC_THREADS) {
    const double x = rotated_at(vol1, M, R, f);
    const double y = vol2[f];
    sx += x;
    sxx = fma(x, x, sxx);
    sxy = fma(x, y, sxy);
  }
  sx = blk_sum(sx);
  sxx = blk_sum(sxx);
  sxy = blk_sum(sxy);
  if (threadIdx.x == 0) {
    double *p = partial + ((int64_t)q * SC_BLOCKS + blockIdx.x) * 3;
    p[0] = sx;
    p[1] = sxx;
    p[2] = sxy;
  }
}

// sums of y and y^2 of the fixed volume (scal[0], scal[1])
__global__ void __launch_bounds__(SC_THREADS)
    k_score_fixed(const double *__restrict__ vol2, int64_t n, double *__restrict__ scal) {
  double sy = 0.0, syy = 0.0;
  for (int64_t f = threadIdx.x; f < n; f += SC_THREADS) {
    const double y = vol2[f];
    sy += y;
    syy = fma(y, y, syy);
  }
  sy = blk_sum(sy);
  syy = blk_sum(syy);
  if (threadIdx.x == 0) {
    scal[0] = sy;
    scal[1] = syy;
  }
}

// Pearson correlation (align.py:69-90) from the sums:
// sum (x - mx)(y - my) / sqrt(sum (x - mx)^2 sum (y - my)^2)
__global__ void k_score_final(const double *__restrict__ partial, const double *__restrict__ scal,
                              int64_t n, int n_quat, double *__restrict__ cc) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n_quat) return;
  double sx = 0.0, sxx = 0.0, sxy = 0.0;
  for (int b = 0; b < SC_BLOCKS; ++b) {
    const double *p = partial + ((int64_t)q * SC_BLOCKS + b) * 3;
    sx += p[0];
    sxx += p[1];
    sxy += p[2];
  }
  const double nn = (double)n;
  const double mx = sx / nn, my = scal[0] / nn;
  const double num = sxy - nn * mx * my;
  const double vx = sxx - nn * mx * mx, vy = scal[1] - nn * my * my;
  cc[q] = num / (sqrt(vx) * sqrt(vy));
}

__global__ void k_rotate(const double *__restrict__ vol, int M, const double *__restrict__ quats,
                         double *__restrict__ out) {
  const int q = blockIdx.y;
  const Rot R = quat_rot(quats + 4 * q);
  const int64_t n = (int64_t)M * M * M;
  for (int64_t f = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; f < n;
       f += (int64_t)gridDim.x * blockDim.x)
    out[(int64_t)q * n + f] = rotated_at(vol, M, R, f);
}

// value of the full spectrum at (h, j, k) from a D2Z half spectrum
__device__ __forceinline__ double2 spec_at(const double2 *spec, int M, int h, int j, int k) {
  const int mh = M / 2 + 1;
  if (k < mh) return spec[((int64_t)h * M + j) * mh + k];
  const double2 z = spec[((int64_t)((M - h) % M) * M + (M - j) % M) * mh + (M - k)];
  return make_double2(z.x, -z.y);
}

// FSC shell sums (fsc.py:67-125): over the fftshifted grid, shell i holds the
// voxels with i*spacing < |q| < i*spacing + spacing, |q| = sqrt(x^2 + y^2 +
// z^2) * scale on the centred mesh coord^3; sums[3i..3i+2] += Re(F1 conj F2),
// |F1|^2, |F2|^2.
__global__ void k_fsc(const double2 *__restrict__ s1, const double2 *__restrict__ s2, int M,
                      const double *__restrict__ coord, double scale, double spacing,
                      int n_shells, double *__restrict__ sums) {
  const int64_t n = (int64_t)M * M * M;
  const int sh = (M + 1) / 2;  // fftshift: centred index c holds frequency index (c + sh) % M
  for (int64_t f = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; f < n;
       f += (int64_t)gridDim.x * blockDim.x) {
    const int c = (int)(f % M), b = (int)((f / M) % M), a = (int)(f / ((int64_t)M * M));
    const double x = coord[a], y = coord[b], z = coord[c];
    // numpy's norm over the last axis: ((x^2 + y^2) + z^2), no fused multiply-add
    const double s =
        __dmul_rn(sqrt(__dadd_rn(__dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y)), __dmul_rn(z, z))),
                  scale);
    const int i0 = (int)floor(s / spacing);
    bool any = false;
    double2 z1, z2;
    for (int i = max(i0 - 1, 0); i <= min(i0 + 1, n_shells - 1); ++i) {
      const double r = (double)i * spacing;
      if (!(s > r && s < r + spacing)) continue;
      if (!any) {
        z1 = spec_at(s1, M, (a + sh) % M, (b + sh) % M, (c + sh) % M);
        z2 = spec_at(s2, M, (a + sh) % M, (b + sh) % M, (c + sh) % M);
        any = true;
      }
      atomicAdd(sums + 3 * i, z1.x * z2.x + z1.y * z2.y);
      atomicAdd(sums + 3 * i + 1, z1.x * z1.x + z1.y * z1.y);
      atomicAdd(sums + 3 * i + 2, z2.x * z2.x + z2.y * z2.y);
    }
  }
}

}  // namespace

extern "C" {

int spf_eval_score_rotations(const double *d_vol1, const double *d_vol2, int M,
                             const double *d_quats, int64_t n_quat, double *d_cc, void *stream) {
  SPF_REQUIRE(M >= 2 && M <= 1024 && n_quat >= 0 && n_quat <= 65535,
              "spf_eval_score_rotations: M in 2..1024, n_quat in 0..65535");
  if (n_quat == 0) return SPF_OK;
  SPF_REQUIRE(d_vol1 && d_vol2 && d_quats && d_cc, "spf_eval_score_rotations: NULL pointer");
  cudaStream_t s = spf::as_stream(stream);
  double *partial = nullptr, *scal = nullptr;
  SPF_TRY(spf::check_cuda(cudaMallocAsync(&partial, n_quat * SC_BLOCKS * 3 * sizeof(double), s),
                          "spf_eval_score_rotations"));
  int st = spf::check_cuda(cudaMallocAsync(&scal, 2 * sizeof(double), s),
                           "spf_eval_score_rotations");
  const int64_t n = (int64_t)M * M * M;
  if (st == SPF_OK) {
    k_score_fixed<<<1, SC_THREADS, 0, s>>>(d_vol2, n, scal);
    st = spf::check_launch("k_score_fixed");
  }
  if (st == SPF_OK) {
    k_score_partial<<<dim3(SC_BLOCKS, (unsigned)n_quat), SC_THREADS, 0, s>>>(d_vol1, d_vol2, M,
                                                                             d_quats, partial);
    st = spf::check_launch("k_score_partial");
  }
  if (st == SPF_OK) {
    k_score_final<<<(unsigned)((n_quat + 127) / 128), 128, 0, s>>>(partial, scal, n, (int)n_quat,
                                                                    d_cc);
    st = spf::check_launch("k_score_final");
  }
  cudaFreeAsync(partial, s);
  if (scal) cudaFreeAsync(scal, s);
  return st;
}

int spf_eval_rotate_volume(const double *d_vol, int M, const double *d_quats, int64_t n_quat,
                           double *d_out, void *stream) {
  SPF_REQUIRE(M >= 2 && M <= 1024 && n_quat >= 0 && n_quat <= 65535,
              "spf_eval_rotate_volume: M in 2..1024, n_quat in 0..65535");
  if (n_quat == 0) return SPF_OK;
  SPF_REQUIRE(d_vol && d_quats && d_out, "spf_eval_rotate_volume: NULL pointer");
  const int64_t n = (int64_t)M * M * M;
  k_rotate<<<dim3(spf::grid_for(n, 256, 1024), (unsigned)n_quat), 256, 0,
             spf::as_stream(stream)>>>(d_vol, M, d_quats, d_out);
  return spf::check_launch("k_rotate");
}

int spf_eval_fsc_shells(const double *d_vol1, const double *d_vol2, int M, const double *d_coord,
                        double scale, double spacing, int n_shells, double *d_sums,
                        void *stream) {
  SPF_REQUIRE(M >= 2 && M <= 1024 && n_shells >= 1 && spacing > 0.0,
              "spf_eval_fsc_shells: bad sizes");
  SPF_REQUIRE(d_vol1 && d_vol2 && d_coord && d_sums, "spf_eval_fsc_shells: NULL pointer");
  cudaStream_t s = spf::as_stream(stream);
  const int64_t nh = (int64_t)M * M * (M / 2 + 1);
  double2 *s1 = nullptr, *s2 = nullptr;
  cufftHandle plan;
  if (cufftPlan3d(&plan, M, M, M, CUFFT_D2Z) != CUFFT_SUCCESS) {
    spf::set_error("spf_eval_fsc_shells: cufftPlan3d failed (M = %d)", M);
    return SPF_ERR_CUDA;
  }
  cufftSetStream(plan, s);
  int st = spf::check_cuda(cudaMallocAsync(&s1, nh * sizeof(double2), s), "spf_eval_fsc_shells");
  if (st == SPF_OK)
    st = spf::check_cuda(cudaMallocAsync(&s2, nh * sizeof(double2), s), "spf_eval_fsc_shells");
  if (st == SPF_OK &&
      (cufftExecD2Z(plan, const_cast<double *>(d_vol1), (cufftDoubleComplex *)s1) != CUFFT_SUCCESS ||
       cufftExecD2Z(plan, const_cast<double *>(d_vol2), (cufftDoubleComplex *)s2) != CUFFT_SUCCESS)) {
    spf::set_error("spf_eval_fsc_shells: D2Z failed");
    st = SPF_ERR_CUDA;
  }
  if (st == SPF_OK)
    st = spf::check_cuda(cudaMemsetAsync(d_sums, 0, 3 * n_shells * sizeof(double), s),
                         "spf_eval_fsc_shells");
  if (st == SPF_OK) {
    const int64_t n = (int64_t)M * M * M;
    k_fsc<<<spf::grid_for(n, 256, (int64_t)spf::sm_count() * 8), 256, 0, s>>>(
        s1, s2, M, d_coord, scale, spacing, n_shells, d_sums);
    st = spf::check_launch("k_fsc");
  }
  if (s1) cudaFreeAsync(s1, s);
  if (s2) cudaFreeAsync(s2, s);
  cudaStreamSynchronize(s);  // the plan's work is done before it is destroyed
  cufftDestroy(plan);
  return st;
}

}  // extern "C"
