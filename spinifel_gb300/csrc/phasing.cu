// Phase retrieval of the autocorrelation: ER / HIO iterations with
// shrink-wrap, device resident in FP64 (spinifel/sequential/phasing.py).
//
// Arrays follow the reference's convention: a trailing underscore means
// ifftshifted (phasing.py:27-40), so the FFT of rho_ is a plain fftn.  rho_
// is real, so its spectrum is Hermitian and every transform is a D2Z / Z2D
// on the M^3 grid (half spectrum [M][M][M/2+1]); the amplitude projection
// keeps that symmetry, so the C2R result is the real part the reference
// takes (phasing.py:186-188).  Reductions (max, mean, std, centre of mass)
// use a fixed grid and order, so a run is bit-reproducible.  An iteration is
// a fixed launch sequence without host synchronisation; only the recentring
// at the end reads three integers back (phasing.py:45-80 rounds on the host).
#include <cufft.h>
#include <math.h>

#include <vector>

#include "common.cuh"

namespace {

constexpr int PH_BLOCKS = 296;  // fixed so the reduction order is fixed
constexpr int PH_THREADS = 256;
constexpr int PH_MAX_TAPS = 65;  // Gaussian radius <= 32

struct GaussTaps {
  double w[PH_MAX_TAPS];  // w[0] centre, w[j] the weight at distance j
  int radius;
};

__host__ __device__ inline int ishift(int k, int M) { return (k + M / 2) % M; }
__host__ __device__ inline int fshift(int k, int M) { return (k + (M + 1) / 2) % M; }

__device__ __forceinline__ double ph_block_reduce(double v, bool is_max) {
  __shared__ double sh[PH_THREADS / 32];
  for (int o = 16; o >= 1; o >>= 1) {
    double u = __shfl_xor_sync(0xffffffffu, v, o);
    v = is_max ? fmax(v, u) : v + u;
  }
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) sh[w] = v;
  __syncthreads();
  v = is_max ? -INFINITY : 0.0;
  if (threadIdx.x < 32) {
    if (threadIdx.x < PH_THREADS / 32) v = sh[threadIdx.x];
    for (int o = 16; o >= 1; o >>= 1) {
      double u = __shfl_xor_sync(0xffffffffu, v, o);
      v = is_max ? fmax(v, u) : v + u;
    }
  }
  __syncthreads();
  return v;
}

// partial[b * 4 + q], q = 0..3, for the statistics below
enum RedKind { RED_MAX = 0, RED_SUM = 1, RED_SQDEV = 2, RED_ABSMAX = 3, RED_COM = 4 };

__global__ void __launch_bounds__(PH_THREADS)
    k_ph_partial(const double *__restrict__ x, int64_t n, int kind, const double *__restrict__ scal,
                 const double *__restrict__ coord, int M, double *__restrict__ partial) {
  const bool is_max = kind == RED_MAX || kind == RED_ABSMAX;
  double s[4] = {is_max ? -INFINITY : 0.0, 0.0, 0.0, 0.0};
  const double mean = kind == RED_SQDEV ? scal[1] : 0.0;
  for (int64_t i = blockIdx.x * (int64_t)PH_THREADS + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * PH_THREADS) {
    const double v = x[i];
    switch (kind) {
      case RED_MAX: s[0] = fmax(s[0], v); break;
      case RED_ABSMAX: s[0] = fmax(s[0], fabs(v)); break;
      case RED_SUM: s[0] += v; break;
      case RED_SQDEV: {
        const double d = __dsub_rn(v, mean);
        s[0] = __dadd_rn(s[0], __dmul_rn(d, d));
        break;
      }
      default: {  // centre of mass of |x| over the (shifted) coordinate grid
        const double a = fabs(v);
        const int k = (int)(i % M), j = (int)((i / M) % M), h = (int)(i / ((int64_t)M * M));
        s[0] += a;
        s[1] = __dadd_rn(s[1], __dmul_rn(a, coord[ishift(h, M)]));
        s[2] = __dadd_rn(s[2], __dmul_rn(a, coord[ishift(j, M)]));
        s[3] = __dadd_rn(s[3], __dmul_rn(a, coord[ishift(k, M)]));
      }
    }
  }
  const int nq = kind == RED_COM ? 4 : 1;
  for (int q = 0; q < nq; ++q) {
    double r = ph_block_reduce(s[q], is_max);
    if (threadIdx.x == 0) partial[blockIdx.x * 4 + q] = r;
  }
}

// scal[slot .. slot+nq) = reduction of the partials; RED_SUM and RED_SQDEV
// are divided by n (means).
__global__ void __launch_bounds__(PH_THREADS)
    k_ph_final(const double *__restrict__ partial, int kind, int64_t n, double *__restrict__ scal,
               int slot) {
  const bool is_max = kind == RED_MAX || kind == RED_ABSMAX;
  const int nq = kind == RED_COM ? 4 : 1;
  for (int q = 0; q < nq; ++q) {
    double v = is_max ? -INFINITY : 0.0;
    for (int i = threadIdx.x; i < PH_BLOCKS; i += PH_THREADS) {
      const double u = partial[i * 4 + q];
      v = is_max ? fmax(v, u) : v + u;
    }
    v = ph_block_reduce(v, is_max);
    if (threadIdx.x == 0) {
      if (kind == RED_SUM || kind == RED_SQDEV) v = v / (double)n;
      scal[slot + q] = v;
    }
  }
}

__global__ void k_ph_relu(const double *__restrict__ in, double *__restrict__ out, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    out[i] = fmax(in[i], 0.0);
}

__global__ void k_ph_abs(const double *__restrict__ in, double *__restrict__ out, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    out[i] = fabs(in[i]);
}

// 1-D Gaussian correlation along one axis of an M^3 array (scipy.ndimage
// correlate1d with symmetric weights: w0 x[c] + sum_j w_j (x[c-j] + x[c+j])),
// boundary 'wrap' (periodic) or 'constant' (zero outside).
__global__ void k_ph_gauss_axis(const double *__restrict__ in, double *__restrict__ out, int M,
                                int axis, GaussTaps taps, int wrap) {
  const int64_t n = (int64_t)M * M * M;
  const int64_t stride = axis == 0 ? (int64_t)M * M : (axis == 1 ? M : 1);
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int c = (int)((i / stride) % M);
    const int64_t base = i - (int64_t)c * stride;
    double acc = __dmul_rn(in[i], taps.w[0]);
    for (int j = 1; j <= taps.radius; ++j) {
      int lo = c - j, hi = c + j;
      double a = 0.0, b = 0.0;
      if (wrap) {
        lo = ((lo % M) + M) % M;
        hi = hi % M;
        a = in[base + lo * stride];
        b = in[base + hi * stride];
      } else {
        if (lo >= 0) a = in[base + lo * stride];
        if (hi < M) b = in[base + hi * stride];
      }
      acc = __dadd_rn(acc, __dmul_rn(__dadd_rn(a, b), taps.w[j]));
    }
    out[i] = acc;
  }
}

// out = ifftshift(in) (shift = +1) or fftshift(in) (shift = -1), 3-D
template <class T>
__global__ void k_ph_shift(const T *__restrict__ in, T *__restrict__ out, int M, int forward) {
  const int64_t n = (int64_t)M * M * M;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int k = (int)(i % M), j = (int)((i / M) % M), h = (int)(i / ((int64_t)M * M));
    const int sh = forward ? ishift(h, M) : fshift(h, M), sj = forward ? ishift(j, M) : fshift(j, M),
              sk = forward ? ishift(k, M) : fshift(k, M);
    out[i] = in[((int64_t)sh * M + sj) * M + sk];
  }
}

// amplitudes_ = sqrt(|fftn(ac_filt_)|) on the half spectrum
__global__ void k_ph_amp(const double2 *__restrict__ spec, double *__restrict__ amp, int64_t nh) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nh;
       i += (int64_t)gridDim.x * blockDim.x)
    amp[i] = sqrt(hypot(spec[i].x, spec[i].y));
}

// support_ = ifftshift(square) & (ac_filt_ > 1e-2 max(ac_filt_))  (phasing.py:84-107)
__global__ void k_ph_create_support(const double *__restrict__ ac_filt_, const double *__restrict__ scal,
                                    int M, int Mquat, uint8_t *__restrict__ support) {
  const int64_t n = (int64_t)M * M * M;
  const double thr = 1e-2 * scal[0];
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int k = (int)(i % M), j = (int)((i / M) % M), h = (int)(i / ((int64_t)M * M));
    const int ch = ishift(h, M), cj = ishift(j, M), ck = ishift(k, M);
    const bool sq = ch >= Mquat && ch < M - Mquat && cj >= Mquat && cj < M - Mquat &&
                    ck >= Mquat && ck < M - Mquat;
    support[i] = (uint8_t)(sq && ac_filt_[i] > thr);
  }
}

// Fourier projection (phasing.py:182-188): every mode but (0,0,0) gets the
// measured amplitude with the current phase; the 1/M^3 of the inverse FFT is
// folded in.
__global__ void k_ph_project(double2 *__restrict__ spec, const double *__restrict__ amp,
                             int64_t nh, double inv_n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nh;
       i += (int64_t)gridDim.x * blockDim.x) {
    double2 z = spec[i];
    if (i != 0) {
      const double r = hypot(z.x, z.y);
      if (r > 0.0) {
        z.x = amp[i] * (z.x / r);
        z.y = amp[i] * (z.y / r);
      } else {  // angle(0) = 0
        z.x = amp[i];
        z.y = 0.0;
      }
    }
    spec[i] = make_double2(z.x * inv_n, z.y * inv_n);
  }
}

// ER (phasing.py:130-147) and HIO (:151-169) real-space updates
__global__ void k_ph_update(double *__restrict__ rho, const double *__restrict__ rho_mod,
                            const uint8_t *__restrict__ support, int64_t n, int hio, double beta,
                            double rho_max) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double m = rho_mod[i];
    const bool star = support[i] && m > 0.0;
    double r;
    if (hio) {
      r = star ? m : __dsub_rn(rho[i], __dmul_rn(beta, m));
      if (m > rho_max) r = __dadd_rn(r, __dsub_rn(__dmul_rn(2.0 * beta, m), rho_max));
    } else {
      r = star ? m : 0.0;
      if (m > rho_max) r = rho_max;
    }
    rho[i] = r;
  }
}

// shrink-wrap threshold (phasing.py:193-221): scal[4] = std * weight or
// max|rho| * cutoff * weight; support_ = gauss > threshold
__global__ void k_ph_threshold(const double *__restrict__ scal, int method, double weight,
                               double cutoff, double *__restrict__ out) {
  if (threadIdx.x == 0 && blockIdx.x == 0)
    out[0] = method == 0 ? sqrt(scal[2]) * weight : scal[3] * cutoff * weight;
}

__global__ void k_ph_support_from(const double *__restrict__ g, const double *__restrict__ thr,
                                  uint8_t *__restrict__ support, int64_t n) {
  const double t = thr[0];
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    support[i] = (uint8_t)(g[i] > t);
}

// np.roll(x, -s, axis) on all three axes at once: out[i] = in[i + s]
template <class T>
__global__ void k_ph_roll(const T *__restrict__ in, T *__restrict__ out, int M, int s0, int s1,
                          int s2) {
  const int64_t n = (int64_t)M * M * M;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int k = (int)(i % M), j = (int)((i / M) % M), h = (int)(i / ((int64_t)M * M));
    const int a = (h + s0) % M, b = (j + s1) % M, c = (k + s2) % M;
    out[i] = in[((int64_t)a * M + b) * M + c];
  }
}

// value of the full spectrum at (h, j, k) from the D2Z half spectrum
__device__ __forceinline__ double2 half_at(const double2 *spec, int M, int h, int j, int k) {
  const int mh = M / 2 + 1;
  if (k < mh) return spec[((int64_t)h * M + j) * mh + k];
  const double2 z = spec[((int64_t)((M - h) % M) * M + (M - j) % M) * mh + (M - k)];
  return make_double2(z.x, -z.y);
}

// intensities_phased_ = |fftn(rho_)|^2 on the full grid
__global__ void k_ph_abs2_full(const double2 *__restrict__ spec, double *__restrict__ out, int M) {
  const int64_t n = (int64_t)M * M * M;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int k = (int)(i % M), j = (int)((i / M) % M), h = (int)(i / ((int64_t)M * M));
    const double2 z = half_at(spec, M, h, j, k);
    const double a = hypot(z.x, z.y);
    out[i] = a * a;
  }
}

// ac_phased = fftshift(|ifftn(I)|) = fftshift(|fftn(I)|) / M^3 for real I
__global__ void k_ph_ac_out(const double2 *__restrict__ spec, double *__restrict__ out, int M,
                            double inv_n) {
  const int64_t n = (int64_t)M * M * M;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int k = (int)(i % M), j = (int)((i / M) % M), h = (int)(i / ((int64_t)M * M));
    const double2 z = half_at(spec, M, fshift(h, M), fshift(j, M), fshift(k, M));
    out[i] = hypot(z.x, z.y) * inv_n;
  }
}

int grid_n(int64_t n) { return spf::grid_for(n, 256, (int64_t)spf::sm_count() * 8); }

}  // namespace

struct spf_phaser_s {
  int dev = 0;
  int M = 0;
  int64_t n = 0, nh = 0;
  cufftHandle d2z = 0, z2d = 0;
  bool have_d2z = false, have_z2d = false;
  double *amp = nullptr, *ac_filt = nullptr, *rho = nullptr, *rho_mod = nullptr, *tmp = nullptr,
         *tmp2 = nullptr, *partial = nullptr, *scal = nullptr, *coord = nullptr;
  uint8_t *support = nullptr, *support2 = nullptr;
  double2 *spec = nullptr;
};

namespace {

using spf::check_cuda;
using spf::check_launch;

int cufft_status(cufftResult r, const char *what) {
  if (r == CUFFT_SUCCESS) return SPF_OK;
  spf::set_error("%s: cuFFT error %d", what, (int)r);
  return r == CUFFT_ALLOC_FAILED ? SPF_ERR_OOM : SPF_ERR_CUDA;
}

int ph_check(spf_phaser_s *P, const char *what) {
  SPF_REQUIRE(P != nullptr, "%s: phaser is NULL", what);
  int dev = 0;
  cudaGetDevice(&dev);
  SPF_REQUIRE(dev == P->dev, "%s: current device %d is not the phaser's device %d", what, dev,
              P->dev);
  return SPF_OK;
}

GaussTaps gauss_taps(double sigma, double truncate) {
  // scipy.ndimage._gaussian_kernel1d: exp(-x^2 / (2 sigma^2)) over
  // |x| <= int(truncate * sigma + 0.5), normalised to sum 1
  GaussTaps t{};
  t.radius = (int)(truncate * sigma + 0.5);
  std::vector<double> phi(2 * t.radius + 1);
  double s = 0.0;
  for (int x = -t.radius; x <= t.radius; ++x) {
    phi[x + t.radius] = exp(-0.5 / (sigma * sigma) * (double)(x * x));
  }
  for (double v : phi) s += v;
  for (int j = 0; j <= t.radius; ++j) t.w[j] = phi[t.radius + j] / s;
  return t;
}

int gauss3(spf_phaser_s *P, const double *in, double *out, double *scratch, double sigma,
           int wrap, cudaStream_t s) {
  GaussTaps taps = gauss_taps(sigma, 2.0);
  SPF_REQUIRE(taps.radius < PH_MAX_TAPS / 2 + 1 && taps.radius >= 0,
              "phasing: Gaussian sigma %g too large", sigma);
  const int g = grid_n(P->n);
  // axis 0: in -> out, axis 1: out -> scratch, axis 2: scratch -> out
  k_ph_gauss_axis<<<g, 256, 0, s>>>(in, out, P->M, 0, taps, wrap);
  SPF_TRY(check_launch("k_ph_gauss_axis"));
  k_ph_gauss_axis<<<g, 256, 0, s>>>(out, scratch, P->M, 1, taps, wrap);
  SPF_TRY(check_launch("k_ph_gauss_axis"));
  k_ph_gauss_axis<<<g, 256, 0, s>>>(scratch, out, P->M, 2, taps, wrap);
  return check_launch("k_ph_gauss_axis");
}

int reduce(spf_phaser_s *P, const double *x, int kind, int slot, cudaStream_t s) {
  k_ph_partial<<<PH_BLOCKS, PH_THREADS, 0, s>>>(x, P->n, kind, P->scal, P->coord, P->M,
                                                 P->partial);
  SPF_TRY(check_launch("k_ph_partial"));
  k_ph_final<<<1, PH_THREADS, 0, s>>>(P->partial, kind, P->n, P->scal, slot);
  return check_launch("k_ph_final");
}

int iterate(spf_phaser_s *P, int n_loops, int hio, double beta, double rho_max, cudaStream_t s) {
  SPF_REQUIRE(n_loops >= 0, "phasing: n_loops < 0");
  cufftSetStream(P->d2z, s);
  cufftSetStream(P->z2d, s);
  const double inv_n = 1.0 / (double)P->n;
  for (int it = 0; it < n_loops; ++it) {
    SPF_TRY(cufft_status(cufftExecD2Z(P->d2z, P->rho, (cufftDoubleComplex *)P->spec), "D2Z"));
    k_ph_project<<<grid_n(P->nh), 256, 0, s>>>(P->spec, P->amp, P->nh, inv_n);
    SPF_TRY(check_launch("k_ph_project"));
    SPF_TRY(cufft_status(cufftExecZ2D(P->z2d, (cufftDoubleComplex *)P->spec, P->rho_mod), "Z2D"));
    k_ph_update<<<grid_n(P->n), 256, 0, s>>>(P->rho, P->rho_mod, P->support, P->n, hio, beta,
                                             rho_max);
    SPF_TRY(check_launch("k_ph_update"));
  }
  return SPF_OK;
}

}  // namespace

extern "C" {

int spf_phase_destroy(spf_phaser_s *P);

int spf_phase_create(int M, spf_phaser_s **out) {
  SPF_REQUIRE(out != nullptr, "spf_phase_create: out is NULL");
  *out = nullptr;
  SPF_REQUIRE(M >= 3 && M <= 1024, "spf_phase_create: M = %d out of range 3..1024", M);
  auto *P = new spf_phaser_s();
  cudaGetDevice(&P->dev);
  P->M = M;
  P->n = (int64_t)M * M * M;
  P->nh = (int64_t)M * M * (M / 2 + 1);
  int st = SPF_OK;
  auto alloc = [&](void **p, size_t bytes) {
    if (st == SPF_OK) st = check_cuda(cudaMalloc(p, bytes), "spf_phase_create");
  };
  alloc((void **)&P->amp, P->nh * sizeof(double));
  alloc((void **)&P->ac_filt, P->n * sizeof(double));
  alloc((void **)&P->rho, P->n * sizeof(double));
  alloc((void **)&P->rho_mod, P->n * sizeof(double));
  alloc((void **)&P->tmp, P->n * sizeof(double));
  alloc((void **)&P->tmp2, P->n * sizeof(double));
  alloc((void **)&P->partial, PH_BLOCKS * 4 * sizeof(double));
  alloc((void **)&P->scal, 16 * sizeof(double));
  alloc((void **)&P->coord, M * sizeof(double));
  alloc((void **)&P->support, P->n);
  alloc((void **)&P->support2, P->n);
  alloc((void **)&P->spec, P->nh * sizeof(double2));
  if (st == SPF_OK) {
    st = cufft_status(cufftPlan3d(&P->d2z, M, M, M, CUFFT_D2Z), "spf_phase_create: D2Z plan");
    P->have_d2z = st == SPF_OK;
  }
  if (st == SPF_OK) {
    st = cufft_status(cufftPlan3d(&P->z2d, M, M, M, CUFFT_Z2D), "spf_phase_create: Z2D plan");
    P->have_z2d = st == SPF_OK;
  }
  if (st == SPF_OK) {
    // midpoints of numpy.linspace(-1, 1, M + 1) (phasing.py:70-71), same arithmetic
    std::vector<double> ls(M + 1), mid(M);
    const double step = 2.0 / (double)M;
    for (int c = 0; c <= M; ++c) ls[c] = (double)c * step + -1.0;
    ls[M] = 1.0;
    for (int c = 0; c < M; ++c) mid[c] = (ls[c] + ls[c + 1]) / 2.0;
    st = check_cuda(cudaMemcpy(P->coord, mid.data(), M * sizeof(double), cudaMemcpyHostToDevice),
                    "spf_phase_create");
  }
  if (st == SPF_OK)
    st = check_cuda(cudaMemset(P->support, 0, P->n), "spf_phase_create");
  if (st == SPF_OK)
    st = check_cuda(cudaMemset(P->rho, 0, P->n * sizeof(double)), "spf_phase_create");
  if (st != SPF_OK) {
    spf_phase_destroy(P);
    return st;
  }
  *out = P;
  return SPF_OK;
}

int spf_phase_destroy(spf_phaser_s *P) {
  if (!P) return SPF_OK;
  if (P->have_d2z) cufftDestroy(P->d2z);
  if (P->have_z2d) cufftDestroy(P->z2d);
  void *bufs[] = {P->amp, P->ac_filt, P->rho,     P->rho_mod, P->tmp,      P->tmp2,
                  P->partial, P->scal, P->coord, P->support, P->support2, P->spec};
  for (void *b : bufs)
    if (b) cudaFree(b);
  delete P;
  return SPF_OK;
}

int spf_phase_set_ac(spf_phaser_s *P, const double *d_ac, void *stream) {
  SPF_TRY(ph_check(P, "spf_phase_set_ac"));
  SPF_REQUIRE(d_ac != nullptr, "spf_phase_set_ac: ac is NULL");
  cudaStream_t s = spf::as_stream(stream);
  const int g = grid_n(P->n);
  // ac_filt = gaussian_filter(max(ac, 0), mode='constant', sigma=1, truncate=2)
  k_ph_relu<<<g, 256, 0, s>>>(d_ac, P->tmp, P->n);
  SPF_TRY(check_launch("k_ph_relu"));
  SPF_TRY(gauss3(P, P->tmp, P->tmp2, P->rho_mod, 1.0, 0, s));
  // ac_filt_ = ifftshift(ac_filt); amplitudes_ = sqrt(|fftn(ac_filt_)|)
  k_ph_shift<double><<<g, 256, 0, s>>>(P->tmp2, P->ac_filt, P->M, 1);
  SPF_TRY(check_launch("k_ph_shift"));
  cufftSetStream(P->d2z, s);
  SPF_TRY(cufft_status(cufftExecD2Z(P->d2z, P->ac_filt, (cufftDoubleComplex *)P->spec),
                       "spf_phase_set_ac: D2Z"));
  k_ph_amp<<<grid_n(P->nh), 256, 0, s>>>(P->spec, P->amp, P->nh);
  return check_launch("k_ph_amp");
}

int spf_phase_create_support(spf_phaser_s *P, int Mquat, void *stream) {
  SPF_TRY(ph_check(P, "spf_phase_create_support"));
  SPF_REQUIRE(Mquat >= 0 && 2 * Mquat < P->M, "spf_phase_create_support: bad Mquat %d", Mquat);
  cudaStream_t s = spf::as_stream(stream);
  SPF_TRY(reduce(P, P->ac_filt, RED_MAX, 0, s));
  k_ph_create_support<<<grid_n(P->n), 256, 0, s>>>(P->ac_filt, P->scal, P->M, Mquat, P->support);
  return check_launch("k_ph_create_support");
}

int spf_phase_set_state(spf_phaser_s *P, const double *d_rho_, const uint8_t *d_support_,
                        void *stream) {
  SPF_TRY(ph_check(P, "spf_phase_set_state"));
  cudaStream_t s = spf::as_stream(stream);
  if (d_rho_)
    SPF_TRY(check_cuda(cudaMemcpyAsync(P->rho, d_rho_, P->n * sizeof(double),
                                       cudaMemcpyDeviceToDevice, s), "spf_phase_set_state"));
  if (d_support_)
    SPF_TRY(check_cuda(cudaMemcpyAsync(P->support, d_support_, P->n, cudaMemcpyDeviceToDevice, s),
                       "spf_phase_set_state"));
  return SPF_OK;
}

int spf_phase_get_state(spf_phaser_s *P, double *d_rho_, uint8_t *d_support_, void *stream) {
  SPF_TRY(ph_check(P, "spf_phase_get_state"));
  cudaStream_t s = spf::as_stream(stream);
  if (d_rho_)
    SPF_TRY(check_cuda(cudaMemcpyAsync(d_rho_, P->rho, P->n * sizeof(double),
                                       cudaMemcpyDeviceToDevice, s), "spf_phase_get_state"));
  if (d_support_)
    SPF_TRY(check_cuda(cudaMemcpyAsync(d_support_, P->support, P->n, cudaMemcpyDeviceToDevice, s),
                       "spf_phase_get_state"));
  return SPF_OK;
}

int spf_phase_er(spf_phaser_s *P, int n_loops, double rho_max, void *stream) {
  SPF_TRY(ph_check(P, "spf_phase_er"));
  return iterate(P, n_loops, 0, 0.0, rho_max, spf::as_stream(stream));
}

int spf_phase_hio(spf_phaser_s *P, int n_loops, double beta, double rho_max, void *stream) {
  SPF_TRY(ph_check(P, "spf_phase_hio"));
  return iterate(P, n_loops, 1, beta, rho_max, spf::as_stream(stream));
}

int spf_phase_shrink_wrap(spf_phaser_s *P, double sigma, int method, double weight, double cutoff,
                          void *stream) {
  SPF_TRY(ph_check(P, "spf_phase_shrink_wrap"));
  SPF_REQUIRE(method == 0 || method == 1, "spf_phase_shrink_wrap: method 0 (std) or 1 (max)");
  SPF_REQUIRE(sigma > 0.0, "spf_phase_shrink_wrap: sigma <= 0");
  cudaStream_t s = spf::as_stream(stream);
  const int g = grid_n(P->n);
  k_ph_abs<<<g, 256, 0, s>>>(P->rho, P->tmp, P->n);
  SPF_TRY(check_launch("k_ph_abs"));
  SPF_TRY(gauss3(P, P->tmp, P->tmp2, P->rho_mod, sigma, 1, s));  // rho_gauss_ in tmp2
  if (method == 0) {
    SPF_TRY(reduce(P, P->tmp2, RED_SUM, 1, s));    // scal[1] = mean
    SPF_TRY(reduce(P, P->tmp2, RED_SQDEV, 2, s));  // scal[2] = mean squared deviation
  } else {
    SPF_TRY(reduce(P, P->rho, RED_ABSMAX, 3, s));  // scal[3] = max |rho_|
  }
  k_ph_threshold<<<1, 32, 0, s>>>(P->scal, method, weight, cutoff, P->scal + 4);
  SPF_TRY(check_launch("k_ph_threshold"));
  k_ph_support_from<<<g, 256, 0, s>>>(P->tmp2, P->scal + 4, P->support, P->n);
  return check_launch("k_ph_support_from");
}

int spf_phase_run(spf_phaser_s *P, int n_phase_loops, int n_er, int n_hio, double beta,
                  double rho_max, int method, double weight, double cutoff, void *stream) {
  SPF_TRY(ph_check(P, "spf_phase_run"));
  SPF_REQUIRE(n_phase_loops >= 0 && n_er >= 0 && n_hio >= 0, "spf_phase_run: negative counts");
  // phasing.py:270-282
  for (int i = 0; i < n_phase_loops; ++i) {
    SPF_TRY(spf_phase_er(P, n_er, rho_max, stream));
    SPF_TRY(spf_phase_hio(P, n_hio, beta, rho_max, stream));
    SPF_TRY(spf_phase_er(P, n_er, rho_max, stream));
    SPF_TRY(spf_phase_shrink_wrap(P, 1.0, method, weight, cutoff, stream));
  }
  return spf_phase_er(P, n_er, rho_max, stream);
}

int spf_phase_finish(spf_phaser_s *P, double *d_ac_phased, int *h_shift, void *stream) {
  SPF_TRY(ph_check(P, "spf_phase_finish"));
  SPF_REQUIRE(d_ac_phased != nullptr, "spf_phase_finish: ac_phased is NULL");
  cudaStream_t s = spf::as_stream(stream);
  const int g = grid_n(P->n);
  // recenter (phasing.py:45-80): centre of mass of |rho_| on the shifted grid
  SPF_TRY(reduce(P, P->rho, RED_COM, 8, s));
  double com[4];
  SPF_TRY(check_cuda(cudaMemcpyAsync(com, P->scal + 8, sizeof(com), cudaMemcpyDeviceToHost, s),
                     "spf_phase_finish"));
  SPF_TRY(check_cuda(cudaStreamSynchronize(s), "spf_phase_finish"));
  int sh[3];
  for (int a = 0; a < 3; ++a) {
    const double v = com[1 + a] / com[0] * (double)P->M / 2.0;
    sh[a] = (int)nearbyint(v);  // numpy.round: half to even (default rounding mode)
    if (h_shift) h_shift[a] = sh[a];
  }
  int r[3];
  for (int a = 0; a < 3; ++a) r[a] = ((sh[a] % P->M) + P->M) % P->M;
  k_ph_roll<double><<<g, 256, 0, s>>>(P->rho, P->tmp, P->M, r[0], r[1], r[2]);
  SPF_TRY(check_launch("k_ph_roll"));
  k_ph_roll<uint8_t><<<g, 256, 0, s>>>(P->support, P->support2, P->M, r[0], r[1], r[2]);
  SPF_TRY(check_launch("k_ph_roll"));
  SPF_TRY(check_cuda(cudaMemcpyAsync(P->rho, P->tmp, P->n * sizeof(double),
                                     cudaMemcpyDeviceToDevice, s), "spf_phase_finish"));
  SPF_TRY(check_cuda(cudaMemcpyAsync(P->support, P->support2, P->n, cudaMemcpyDeviceToDevice, s),
                     "spf_phase_finish"));
  // ac_phased = fftshift(|ifftn(|fftn(rho_)|^2)|)
  cufftSetStream(P->d2z, s);
  SPF_TRY(cufft_status(cufftExecD2Z(P->d2z, P->rho, (cufftDoubleComplex *)P->spec), "D2Z"));
  k_ph_abs2_full<<<g, 256, 0, s>>>(P->spec, P->tmp, P->M);
  SPF_TRY(check_launch("k_ph_abs2_full"));
  SPF_TRY(cufft_status(cufftExecD2Z(P->d2z, P->tmp, (cufftDoubleComplex *)P->spec), "D2Z"));
  k_ph_ac_out<<<g, 256, 0, s>>>(P->spec, d_ac_phased, P->M, 1.0 / (double)P->n);
  return check_launch("k_ph_ac_out");
}

}  // extern "C"
