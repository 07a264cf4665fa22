// Device-resident conjugate-gradient solve of the autocorrelation merge
// (spinifel/sequential/autocorrelation.py:152-225):
//
//   W x = conv(x) + rlambda x + flambda reg(x),   d = A^H b + rlambda x0,
//   conv(x) = S . (ugrid_conv (*) (S . x)) / M^3           (Toeplitz form)
//           = S . Re T1(T2(S . x)) / (M_ups^3 M^3)         (direct form)
//   reg(x)  = S . Re fftshift(ifftn(fftn(ifftshift(S . x)) . ifftshift(F_anti)))
//
// ugrid_conv is the type 1 of ones onto the M_ups grid divided by M_ups^3
// (:158-166); only its modes -(M-1)..M-1 enter the product, so the circular
// convolution runs on an FFT grid of any smooth size L >= 2M-1 (R2C / C2R,
// the kernel's transform is real because ugrid_conv is real and even).  The
// regulariser is a size-M circular operation and uses exactly M; it runs in
// FP64 because flambda = 1e3 scales its FP32 rounding above the data term.
// For a prime M with smooth M - 1 (41, 151, ...) it runs as the Rader DFT
// of prime_dft.cu (the reference's complex fftn / ifftn, real part taken);
// otherwise as a cuFFT D2Z / Z2D pair on the half spectrum.
//
// CG follows scipy.sparse.linalg.cg (the solver the reference calls, :217)
// step for step: stop when ||r|| < rtol ||b||, at most maxiter iterations.
// x, r, p, q and every dot product are FP64; the Toeplitz product is FP32
// (R2C / C2R) after spf_merge_set_kernel and FP64 (D2Z / Z2D) after
// spf_merge_set_kernel_f64, the form for the reference's double-precision
// run.  Each
// iteration is a fixed sequence of launches with no host synchronisation
// (convergence is a device flag that turns later updates into no-ops), so a
// whole solve can be captured in one CUDA graph.
#include <cufft.h>

#include <vector>

#include "common.cuh"
#include "prime_dft.cuh"

#include "../../include/spinifel_gb300.h"

struct Sweep;
void free_sweep(Sweep *w);

struct spf_merge_s {
  int dev = 0;
  int M = 0, L = 0;
  int64_t n = 0;       // M^3
  int64_t nL = 0;      // L^3
  int64_t nLh = 0;     // L*L*(L/2+1)
  int64_t nMh = 0;     // M*M*(M/2+1)
  double rlambda = 0, flambda = 0;
  double conv_scale = 0;  // applied after the C2R of the Toeplitz product
  double direct_scale = 0;
  float *support = nullptr;    // M^3
  float *kernel_hat = nullptr; // nLh
  double *mask_hat = nullptr;  // nMh
  float *conv_in = nullptr;    // L^3
  float2 *conv_freq = nullptr; // nLh
  float *conv_out = nullptr;   // L^3
  double *reg_in = nullptr;    // M^3 (the regulariser runs in FP64: flambda = 1e3 would
  double2 *reg_freq = nullptr; // nMh  otherwise bury the data term in FP32 rounding)
  double *reg_out = nullptr;   // M^3
  float *modes = nullptr;      // M^3 (direct form input / output)
  float *t1_out = nullptr;     // M^3
  double *r = nullptr, *p = nullptr, *q = nullptr;
  double *partial = nullptr;   // reduction scratch
  double *scal = nullptr;      // device scalars
  int *flags = nullptr;        // [0] done, [1] iterations
  cufftHandle r2c_L = 0, c2r_L = 0, r2c_M = 0, c2r_M = 0;
  bool plans_ok = false;    // the L-grid pair
  // FP64 Toeplitz product (spf_merge_set_kernel_f64): D2Z / Z2D on the L grid
  bool conv64 = false;
  double *kernel_hat64 = nullptr;  // nLh
  double *conv_in64 = nullptr;     // L^3, zero outside the M^3 corner
  double2 *conv_freq64 = nullptr;  // nLh
  double *conv_out64 = nullptr;    // L^3
  cufftHandle d2z_L = 0, z2d_L = 0;
  bool plans64_ok = false;
  bool m_plans_ok = false;  // the M-grid D2Z / Z2D pair (regulariser without Rader)
  // regulariser of a prime M with smooth M - 1: Rader DFT and the full
  // real multiplier ifftshift(F_anti) on M^3
  spf::PrimeDft *pd = nullptr;
  double *mask_full = nullptr;
  // direct form
  spf_nufft_plan_s *nufft = nullptr;
  const float *quats = nullptr, *ppr = nullptr, *weights = nullptr;
  int64_t n_orient = 0, n_pix = 0;
  int det[3] = {0, 0, 0};
  bool sorted = false;
  double coord_scale = 0;
  struct Sweep *sweep = nullptr;  // batched buffers of spf_merge_cg_sweep
};

// device scalar slots
enum { S_RHO = 0, S_RHO_PREV, S_ALPHA, S_BETA, S_PQ, S_ATOL, S_BNORM, S_COUNT };

extern "C" int spf_nufft_t2_set_modes(spf_nufft_plan_s *, const float *, const float *, int, int,
                                      void *);
extern "C" int spf_nufft_t1_zero(spf_nufft_plan_s *, void *);
extern "C" int spf_nufft_t1_finish(spf_nufft_plan_s *, int, float *, float *, void *);
extern "C" int spf_nufft_interp_spread_orient(spf_nufft_plan_s *, const float *, int64_t,
                                              const float *, int64_t, double, const float *,
                                              void *);
extern "C" int spf_nufft_interp_spread_det(spf_nufft_plan_s *, const float *, int64_t,
                                           const float *, int, int, int, double, const float *,
                                           void *);
extern "C" int spf_nufft_sort_orient(spf_nufft_plan_s *, const float *, int64_t, const float *,
                                     int64_t, double, void *);
extern "C" int spf_nufft_interp_spread_sorted(spf_nufft_plan_s *, const float *, void *);

namespace spf {
namespace cg {

constexpr int RED_BLOCKS = 296;  // 2 x 148+; fixed so the reduction order is fixed
constexpr int RED_THREADS = 256;

static int next_smooth(int n) {
  for (;; ++n) {
    int m = n;
    for (int p : {2, 3, 5, 7})
      while (m % p == 0) m /= p;
    if (m == 1) return n;
  }
}

__device__ __forceinline__ double block_sum(double v) {
  __shared__ double sh[RED_THREADS / 32];
  for (int o = 16; o >= 1; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) sh[w] = v;
  __syncthreads();
  v = 0.0;
  if (threadIdx.x < 32) {
    v = threadIdx.x < RED_THREADS / 32 ? sh[threadIdx.x] : 0.0;
    for (int o = 16; o >= 1; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  }
  __syncthreads();
  return v;
}

__global__ void __launch_bounds__(RED_THREADS)
    k_dot_partial(const double *__restrict__ a, const double *__restrict__ b, int64_t n,
                  double *__restrict__ partial) {
  double s = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)RED_THREADS + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * RED_THREADS)
    s = fma(a[i], b[i], s);
  s = block_sum(s);
  if (threadIdx.x == 0) partial[blockIdx.x] = s;
}

__device__ __forceinline__ double sum_partials(const double *partial) {
  double v = 0.0;
  for (int i = threadIdx.x; i < RED_BLOCKS; i += RED_THREADS) v += partial[i];
  return block_sum(v);
}

// stage 0: ||b|| -> atol; zero the counters
__global__ void k_cg_init(const double *partial, double rtol, double *scal, int *flags) {
  double bb = sum_partials(partial);
  if (threadIdx.x == 0) {
    double bn = sqrt(bb);
    scal[S_BNORM] = bn;
    scal[S_ATOL] = rtol * bn;
    scal[S_RHO_PREV] = 1.0;
    flags[0] = bn == 0.0 ? 1 : 0;
    flags[1] = 0;
  }
}

// stage 1: rho = r.r, convergence test, beta
__global__ void k_cg_stage1(const double *partial, int it, double *scal, int *flags,
                            double *hist) {
  double rho = sum_partials(partial);
  if (threadIdx.x == 0) {
    if (hist) hist[it] = sqrt(rho);
    if (!flags[0]) {
      if (sqrt(rho) < scal[S_ATOL]) {
        flags[0] = 1;
      } else {
        scal[S_RHO] = rho;
        scal[S_BETA] = it > 0 ? rho / scal[S_RHO_PREV] : 0.0;
      }
    }
  }
}

// stage 2: alpha = rho / p.q
__global__ void k_cg_stage2(const double *partial, double *scal, const int *flags) {
  double pq = sum_partials(partial);
  if (threadIdx.x == 0 && !flags[0]) {
    scal[S_PQ] = pq;
    scal[S_ALPHA] = scal[S_RHO] / pq;
    scal[S_RHO_PREV] = scal[S_RHO];
  }
}

// p = r + beta p; operator inputs (S . p in FP32) for both forms
__global__ void k_cg_update_p(double *__restrict__ p, const double *__restrict__ r,
                              const double *__restrict__ scal, const int *__restrict__ flags,
                              const float *__restrict__ S, int M, int L, float *__restrict__ conv_in,
                              double *__restrict__ conv_in64, double *__restrict__ reg_in,
                              float *__restrict__ modes) {
  const bool done = flags[0] != 0;
  const double beta = scal[S_BETA];
  const int64_t n = (int64_t)M * M * M;
  const int h = M / 2;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    double pv = p[i];
    if (!done) {
      pv = r[i] + beta * pv;
      p[i] = pv;
    }
    double vd = pv * (double)S[i];
    float v = (float)vd;
    const unsigned iu = (unsigned)i;  // M^3 < 2^31 (M <= 1024)
    int c = (int)(iu % M), b = (int)((iu / M) % M), a = (int)(iu / (unsigned)(M * M));
    if (conv_in) conv_in[((int64_t)a * L + b) * L + c] = v;
    if (conv_in64) conv_in64[((int64_t)a * L + b) * L + c] = vd;
    if (modes) modes[i] = v;
    // ifftshift: reg_in[j] = in[(j + M/2) mod M]  <=>  in[i] lands at j = (i - M/2) mod M
    int ja = (a - h + M) % M, jb = (b - h + M) % M, jc = (c - h + M) % M;
    reg_in[((int64_t)ja * M + jb) * M + jc] = vd;
  }
}

// apply to a plain vector (x0 or a test vector): same as update_p without the CG update
__global__ void k_load_input(const double *__restrict__ x, const float *__restrict__ S, int M,
                             int L, float *__restrict__ conv_in, double *__restrict__ conv_in64,
                             double *__restrict__ reg_in, float *__restrict__ modes) {
  const int64_t n = (int64_t)M * M * M;
  const int h = M / 2;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    double vd = x[i] * (double)S[i];
    float v = (float)vd;
    const unsigned iu = (unsigned)i;  // M^3 < 2^31 (M <= 1024)
    int c = (int)(iu % M), b = (int)((iu / M) % M), a = (int)(iu / (unsigned)(M * M));
    if (conv_in) conv_in[((int64_t)a * L + b) * L + c] = v;
    if (conv_in64) conv_in64[((int64_t)a * L + b) * L + c] = vd;
    if (modes) modes[i] = v;
    int ja = (a - h + M) % M, jb = (b - h + M) % M, jc = (c - h + M) % M;
    reg_in[((int64_t)ja * M + jb) * M + jc] = vd;
  }
}

__global__ void k_mul_real(float2 *__restrict__ z, const float *__restrict__ w, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    float s = w[i];
    float2 v = z[i];
    z[i] = make_float2(v.x * s, v.y * s);
  }
}

__global__ void k_mul_real_d(double2 *__restrict__ z, const double *__restrict__ w, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    double s = w[i];
    double2 v = z[i];
    z[i] = make_double2(v.x * s, v.y * s);
  }
}

// q = S conv * cs + rlambda x + flambda S reg / M^3, and the partial p.q
// (conv from the Toeplitz product on the L grid, or from t1_out for the
// direct form)
__global__ void __launch_bounds__(RED_THREADS)
    k_assemble(const double *__restrict__ x, const float *__restrict__ S, int M, int L,
               const float *__restrict__ conv_out, const double *__restrict__ conv_out64,
               const float *__restrict__ t1_out,
               double conv_scale, const double *__restrict__ reg_out, double rlambda,
               double flambda, double *__restrict__ q, double *__restrict__ partial) {
  const int64_t n = (int64_t)M * M * M;
  const int h = M / 2;
  const double reg_scale = 1.0 / ((double)M * M * M);
  double s = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)RED_THREADS + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * RED_THREADS) {
    const unsigned iu = (unsigned)i;  // M^3 < 2^31 (M <= 1024)
    int c = (int)(iu % M), b = (int)((iu / M) % M), a = (int)(iu / (unsigned)(M * M));
    double sv = S[i];
    const int64_t li = ((int64_t)a * L + b) * L + c;
    double cv = conv_out64 ? conv_out64[li] : conv_out ? (double)conv_out[li] : (double)t1_out[i];
    // fftshift: out[i] = reg_out[(i - M/2) mod M]
    int ja = (a - h + M) % M, jb = (b - h + M) % M, jc = (c - h + M) % M;
    double rv = reg_out[((int64_t)ja * M + jb) * M + jc];
    double xv = x[i];
    double qv = sv * cv * conv_scale + rlambda * xv + flambda * sv * rv * reg_scale;
    q[i] = qv;
    s = fma(xv, qv, s);
  }
  s = block_sum(s);
  if (partial && threadIdx.x == 0) partial[blockIdx.x] = s;
}

__global__ void k_cg_update_xr(double *__restrict__ x, double *__restrict__ r,
                               const double *__restrict__ p, const double *__restrict__ q,
                               const double *__restrict__ scal, int *__restrict__ flags,
                               int64_t n) {
  if (flags[0]) return;
  const double alpha = scal[S_ALPHA];
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    x[i] = fma(alpha, p[i], x[i]);
    r[i] = fma(-alpha, q[i], r[i]);
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) flags[1] += 1;
}

// r = b - q (q = W x0), or r = b when x0 is zero
__global__ void k_sub(const double *__restrict__ b, const double *__restrict__ q,
                      double *__restrict__ r, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    r[i] = q ? b[i] - q[i] : b[i];
}

// kernel_hat: g[m] = ugrid_conv[d + Mu/2] at m = d mod L for |d| <= M-1
template <typename Tin, typename Tout>
__global__ void k_embed_kernel(const Tin *__restrict__ ugrid_conv, int Mu, int M, int L,
                               Tout *__restrict__ g) {
  const int64_t nL = (int64_t)L * L * L;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nL;
       i += (int64_t)gridDim.x * blockDim.x) {
    int m3 = (int)(i % L), m2 = (int)((i / L) % L), m1 = (int)(i / ((int64_t)L * L));
    int d1 = m1 <= L / 2 ? m1 : m1 - L;
    int d2 = m2 <= L / 2 ? m2 : m2 - L;
    int d3 = m3 <= L / 2 ? m3 : m3 - L;
    Tout v = Tout(0);
    if (abs(d1) <= M - 1 && abs(d2) <= M - 1 && abs(d3) <= M - 1) {
      int a = d1 + Mu / 2, b = d2 + Mu / 2, c = d3 + Mu / 2;
      if (a >= 0 && a < Mu && b >= 0 && b < Mu && c >= 0 && c < Mu)
        v = (Tout)ugrid_conv[((int64_t)a * Mu + b) * Mu + c];
    }
    g[i] = v;
  }
}

__global__ void k_real_part(const float2 *__restrict__ z, float *__restrict__ out, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    out[i] = z[i].x;
}

__global__ void k_real_part_d(const double2 *__restrict__ z, double *__restrict__ out,
                              int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    out[i] = z[i].x;
}

// mask_hat on the R2C half spectrum: the even part (H(m) + H(-m)) / 2 of
// H(m) = F_anti[(m + M/2) mod M].  For real input, Re(ifftn(fftn(y) . H))
// (the reference's regulariser) equals the C2R transform of
// rfftn(y) . (even part of H); F_anti from linspace is not always exactly
// centrosymmetric (rounding at |q| = pi/ovs flips boundary cells, 28 of them
// at M = 31), so H itself would differ there.
__global__ void k_mask_half(const float *__restrict__ F, int M, double *__restrict__ out) {
  const int Mh = M / 2 + 1;
  const int64_t n = (int64_t)M * M * Mh;
  const int h = M / 2;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    int m3 = (int)(i % Mh), m2 = (int)((i / Mh) % M), m1 = (int)(i / ((int64_t)M * Mh));
    int a = (m1 + h) % M, b = (m2 + h) % M, c = (m3 + h) % M;
    int na = (M - m1 + h) % M, nb = (M - m2 + h) % M, nc = (M - m3 + h) % M;
    out[i] = 0.5 * ((double)F[((int64_t)a * M + b) * M + c] +
                    (double)F[((int64_t)na * M + nb) * M + nc]);
  }
}

// mask_full[m] = F_anti[(m + M/2) mod M] on the whole M^3 spectrum
__global__ void k_mask_full(const float *__restrict__ F, int M, double *__restrict__ out) {
  const int64_t n = (int64_t)M * M * M;
  const int h = M / 2;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    int m3 = (int)(i % M), m2 = (int)((i / M) % M), m1 = (int)(i / ((int64_t)M * M));
    int a = (m1 + h) % M, b = (m2 + h) % M, c = (m3 + h) % M;
    out[i] = F[((int64_t)a * M + b) * M + c];
  }
}

static int cufft_ok(cufftResult r, const char *what) {
  if (r == CUFFT_SUCCESS) {
    count_launch();
    return SPF_OK;
  }
  set_error("%s: cuFFT error %d", what, (int)r);
  return r == CUFFT_ALLOC_FAILED ? SPF_ERR_OOM : SPF_ERR_CUDA;
}

static int grid1(int64_t n) { return grid_for(n, 256, (int64_t)sm_count() * 8); }

// conv part of the operator from conv_in / reg_in / modes already loaded
static int apply_operator_core(spf_merge_s *G, bool direct, cudaStream_t s) {
  if (!direct && G->conv64) {
    cufftSetStream(G->d2z_L, s);
    cufftSetStream(G->z2d_L, s);
    SPF_TRY(cufft_ok(cufftExecD2Z(G->d2z_L, G->conv_in64,
                                  reinterpret_cast<cufftDoubleComplex *>(G->conv_freq64)),
                     "conv D2Z"));
    k_mul_real_d<<<grid1(G->nLh), 256, 0, s>>>(G->conv_freq64, G->kernel_hat64, G->nLh);
    SPF_TRY(check_launch("k_mul_real_d"));
    SPF_TRY(cufft_ok(cufftExecZ2D(G->z2d_L, reinterpret_cast<cufftDoubleComplex *>(G->conv_freq64),
                                  G->conv_out64),
                     "conv Z2D"));
  } else if (!direct) {
    cufftSetStream(G->r2c_L, s);
    cufftSetStream(G->c2r_L, s);
    SPF_TRY(cufft_ok(cufftExecR2C(G->r2c_L, G->conv_in, reinterpret_cast<cufftComplex *>(G->conv_freq)),
                     "conv R2C"));
    k_mul_real<<<grid1(G->nLh), 256, 0, s>>>(G->conv_freq, G->kernel_hat, G->nLh);
    SPF_TRY(check_launch("k_mul_real"));
    SPF_TRY(cufft_ok(cufftExecC2R(G->c2r_L, reinterpret_cast<cufftComplex *>(G->conv_freq), G->conv_out),
                     "conv C2R"));
  } else {
    SPF_TRY(spf_nufft_t2_set_modes(G->nufft, G->modes, nullptr, -1, 0, s));
    SPF_TRY(spf_nufft_t1_zero(G->nufft, s));
    if (G->sorted)
      SPF_TRY(spf_nufft_interp_spread_sorted(G->nufft, G->weights, s));
    else if (G->det[0] > 0)
      SPF_TRY(spf_nufft_interp_spread_det(G->nufft, G->quats, G->n_orient, G->ppr, G->det[0],
                                          G->det[1], G->det[2], G->coord_scale, G->weights, s));
    else
      SPF_TRY(spf_nufft_interp_spread_orient(G->nufft, G->quats, G->n_orient, G->ppr, G->n_pix,
                                             G->coord_scale, G->weights, s));
    SPF_TRY(spf_nufft_t1_finish(G->nufft, +1, G->t1_out, nullptr, s));
  }
  if (G->pd) return prime_dft_filter(G->pd, G->reg_in, G->mask_full, G->reg_out, s);
  cufftSetStream(G->r2c_M, s);
  cufftSetStream(G->c2r_M, s);
  SPF_TRY(cufft_ok(cufftExecD2Z(G->r2c_M, G->reg_in,
                                reinterpret_cast<cufftDoubleComplex *>(G->reg_freq)),
                   "reg D2Z"));
  k_mul_real_d<<<grid1(G->nMh), 256, 0, s>>>(G->reg_freq, G->mask_hat, G->nMh);
  SPF_TRY(check_launch("k_mul_real_d"));
  return cufft_ok(cufftExecZ2D(G->c2r_M, reinterpret_cast<cufftDoubleComplex *>(G->reg_freq),
                               G->reg_out),
                  "reg Z2D");
}

}  // namespace cg
}  // namespace spf

using namespace spf;
using namespace spf::cg;

extern "C" {

int spf_merge_destroy(spf_merge_s *G);

int spf_merge_create(int M, int M_ups, double rlambda, double flambda, const float *d_support,
                     const float *d_antisupport, spf_merge_s **out) {
  SPF_REQUIRE(out != nullptr, "spf_merge_create: out is NULL");
  *out = nullptr;
  SPF_REQUIRE(M >= 3 && M <= 1024 && M_ups >= 2 * M - 1, "spf_merge_create: bad M / M_ups");
  SPF_REQUIRE(d_support && d_antisupport, "spf_merge_create: NULL pointer");
  auto *G = new spf_merge_s();
  cudaGetDevice(&G->dev);
  G->M = M;
  G->L = next_smooth(2 * M - 1);
  G->n = (int64_t)M * M * M;
  G->nL = (int64_t)G->L * G->L * G->L;
  G->nLh = (int64_t)G->L * G->L * (G->L / 2 + 1);
  G->nMh = (int64_t)M * M * (M / 2 + 1);
  G->rlambda = rlambda;
  G->flambda = flambda;
  G->conv_scale = 1.0 / ((double)M * M * M) / (double)G->nL;
  G->direct_scale = 1.0 / ((double)M_ups * M_ups * M_ups) / ((double)M * M * M);
  int st = SPF_OK;
  auto alloc = [&](void **p, size_t bytes) {
    if (st == SPF_OK) st = check_cuda(cudaMalloc(p, bytes), "spf_merge_create");
  };
  alloc((void **)&G->support, G->n * sizeof(float));
  alloc((void **)&G->kernel_hat, G->nLh * sizeof(float));
  const bool rader = prime_dft_applies(M) && tune_get(SPF_TUNE_PRIME_DFT, 1) == 1;
  if (rader) {
    alloc((void **)&G->mask_full, G->n * sizeof(double));
    if (st == SPF_OK) st = prime_dft_create(M, 1, &G->pd);
  } else {
    alloc((void **)&G->mask_hat, G->nMh * sizeof(double));
    alloc((void **)&G->reg_freq, G->nMh * sizeof(double2));
  }
  alloc((void **)&G->conv_in, G->nL * sizeof(float));
  alloc((void **)&G->conv_freq, G->nLh * sizeof(float2));
  alloc((void **)&G->conv_out, G->nL * sizeof(float));
  alloc((void **)&G->reg_in, G->n * sizeof(double));
  alloc((void **)&G->reg_out, G->n * sizeof(double));
  alloc((void **)&G->modes, G->n * sizeof(float));
  alloc((void **)&G->t1_out, G->n * sizeof(float));
  alloc((void **)&G->r, G->n * sizeof(double));
  alloc((void **)&G->p, G->n * sizeof(double));
  alloc((void **)&G->q, G->n * sizeof(double));
  alloc((void **)&G->partial, RED_BLOCKS * sizeof(double));
  alloc((void **)&G->scal, S_COUNT * sizeof(double));
  alloc((void **)&G->flags, 2 * sizeof(int));
  if (st == SPF_OK) {
    bool ok = cufftPlan3d(&G->r2c_L, G->L, G->L, G->L, CUFFT_R2C) == CUFFT_SUCCESS &&
              cufftPlan3d(&G->c2r_L, G->L, G->L, G->L, CUFFT_C2R) == CUFFT_SUCCESS;
    G->plans_ok = ok;
    if (ok && !G->pd) {
      ok = cufftPlan3d(&G->r2c_M, M, M, M, CUFFT_D2Z) == CUFFT_SUCCESS &&
           cufftPlan3d(&G->c2r_M, M, M, M, CUFFT_Z2D) == CUFFT_SUCCESS;
      G->m_plans_ok = ok;
    }
    if (!ok) {
      set_error("spf_merge_create: cufftPlan3d failed (L = %d, M = %d)", G->L, M);
      st = SPF_ERR_CUDA;
    }
  }
  if (st == SPF_OK) {
    st = check_cuda(cudaMemcpy(G->support, d_support, G->n * sizeof(float),
                               cudaMemcpyDeviceToDevice), "spf_merge_create");
  }
  if (st == SPF_OK) {
    cudaMemset(G->conv_in, 0, G->nL * sizeof(float));
    cudaMemset(G->kernel_hat, 0, G->nLh * sizeof(float));
    if (G->pd) {
      k_mask_full<<<grid1(G->n), 256>>>(d_antisupport, M, G->mask_full);
      st = check_launch("k_mask_full");
    } else {
      k_mask_half<<<grid1(G->nMh), 256>>>(d_antisupport, M, G->mask_hat);
      st = check_launch("k_mask_half");
    }
  }
  if (st == SPF_OK) st = check_cuda(cudaDeviceSynchronize(), "spf_merge_create");
  if (st != SPF_OK) {
    spf_merge_destroy(G);
    return st;
  }
  *out = G;
  return SPF_OK;
}

int spf_merge_destroy(spf_merge_s *G) {
  if (!G) return SPF_OK;
  void *bufs[] = {G->support, G->kernel_hat, G->mask_hat, G->conv_in, G->conv_freq,
                  G->conv_out, G->reg_in, G->reg_freq, G->reg_out, G->modes, G->t1_out,
                  G->r, G->p, G->q, G->partial, G->scal, G->flags, G->mask_full,
                  G->kernel_hat64, G->conv_in64, G->conv_freq64, G->conv_out64};
  for (void *b : bufs) cudaFree(b);
  free_sweep(G->sweep);
  prime_dft_free(G->pd);
  if (G->plans_ok) {
    cufftDestroy(G->r2c_L);
    cufftDestroy(G->c2r_L);
  }
  if (G->m_plans_ok) {
    cufftDestroy(G->r2c_M);
    cufftDestroy(G->c2r_M);
  }
  if (G->plans64_ok) {
    cufftDestroy(G->d2z_L);
    cufftDestroy(G->z2d_L);
  }
  delete G;
  return SPF_OK;
}

int spf_merge_info(spf_merge_s *G, int *fft_size) {
  SPF_REQUIRE(G != nullptr, "spf_merge_info: NULL");
  if (fft_size) *fft_size = G->L;
  return SPF_OK;
}

int spf_merge_set_kernel(spf_merge_s *G, const float *d_ugrid_conv, int M_ups, void *stream) {
  SPF_REQUIRE(G && d_ugrid_conv, "spf_merge_set_kernel: NULL pointer");
  SPF_REQUIRE(M_ups >= 2 * G->M - 1, "spf_merge_set_kernel: M_ups < 2M-1");
  cudaStream_t s = as_stream(stream);
  k_embed_kernel<<<grid1(G->nL), 256, 0, s>>>(d_ugrid_conv, M_ups, G->M, G->L, G->conv_out);
  SPF_TRY(check_launch("k_embed_kernel"));
  cufftSetStream(G->r2c_L, s);
  SPF_TRY(cufft_ok(cufftExecR2C(G->r2c_L, G->conv_out, reinterpret_cast<cufftComplex *>(G->conv_freq)),
                   "kernel R2C"));
  k_real_part<<<grid1(G->nLh), 256, 0, s>>>(G->conv_freq, G->kernel_hat, G->nLh);
  SPF_TRY(check_launch("k_real_part"));
  G->conv64 = false;
  return SPF_OK;
}

int spf_merge_set_kernel_f64(spf_merge_s *G, const double *d_ugrid_conv, int M_ups,
                             void *stream) {
  SPF_REQUIRE(G && d_ugrid_conv, "spf_merge_set_kernel_f64: NULL pointer");
  SPF_REQUIRE(M_ups >= 2 * G->M - 1, "spf_merge_set_kernel_f64: M_ups < 2M-1");
  cudaStream_t s = as_stream(stream);
  if (!G->plans64_ok) {
    int st = SPF_OK;
    auto alloc = [&](void **p, size_t bytes) {
      if (st == SPF_OK) st = check_cuda(cudaMalloc(p, bytes), "spf_merge_set_kernel_f64");
    };
    alloc((void **)&G->kernel_hat64, G->nLh * sizeof(double));
    alloc((void **)&G->conv_in64, G->nL * sizeof(double));
    alloc((void **)&G->conv_freq64, G->nLh * sizeof(double2));
    alloc((void **)&G->conv_out64, G->nL * sizeof(double));
    SPF_TRY(st);
    SPF_TRY(check_cuda(cudaMemsetAsync(G->conv_in64, 0, G->nL * sizeof(double), s),
                       "spf_merge_set_kernel_f64"));
    if (cufftPlan3d(&G->d2z_L, G->L, G->L, G->L, CUFFT_D2Z) != CUFFT_SUCCESS) {
      set_error("spf_merge_set_kernel_f64: cufftPlan3d D2Z (L = %d) failed", G->L);
      return SPF_ERR_CUDA;
    }
    if (cufftPlan3d(&G->z2d_L, G->L, G->L, G->L, CUFFT_Z2D) != CUFFT_SUCCESS) {
      cufftDestroy(G->d2z_L);
      set_error("spf_merge_set_kernel_f64: cufftPlan3d Z2D (L = %d) failed", G->L);
      return SPF_ERR_CUDA;
    }
    G->plans64_ok = true;
  }
  // the FP64 product's kernel ...
  k_embed_kernel<<<grid1(G->nL), 256, 0, s>>>(d_ugrid_conv, M_ups, G->M, G->L, G->conv_out64);
  SPF_TRY(check_launch("k_embed_kernel (f64)"));
  cufftSetStream(G->d2z_L, s);
  SPF_TRY(cufft_ok(cufftExecD2Z(G->d2z_L, G->conv_out64,
                                reinterpret_cast<cufftDoubleComplex *>(G->conv_freq64)),
                   "kernel D2Z"));
  k_real_part_d<<<grid1(G->nLh), 256, 0, s>>>(G->conv_freq64, G->kernel_hat64, G->nLh);
  SPF_TRY(check_launch("k_real_part_d"));
  // ... and the FP32 one, rounded, which the batched sweep reads
  k_embed_kernel<<<grid1(G->nL), 256, 0, s>>>(d_ugrid_conv, M_ups, G->M, G->L, G->conv_out);
  SPF_TRY(check_launch("k_embed_kernel"));
  cufftSetStream(G->r2c_L, s);
  SPF_TRY(cufft_ok(cufftExecR2C(G->r2c_L, G->conv_out, reinterpret_cast<cufftComplex *>(G->conv_freq)),
                   "kernel R2C"));
  k_real_part<<<grid1(G->nLh), 256, 0, s>>>(G->conv_freq, G->kernel_hat, G->nLh);
  SPF_TRY(check_launch("k_real_part"));
  G->conv64 = true;
  return SPF_OK;
}

int spf_merge_set_direct(spf_merge_s *G, spf_nufft_plan_s *plan, const float *d_quats,
                         int64_t n_orient, const float *d_ppr, int64_t n_pix, int det_panels,
                         int det_nx, int det_ny, double coord_scale, const float *d_weights) {
  SPF_REQUIRE(G && plan && d_quats && d_ppr, "spf_merge_set_direct: NULL pointer");
  SPF_REQUIRE(det_panels <= 0 || (int64_t)det_panels * det_nx * det_ny == n_pix,
              "spf_merge_set_direct: detector shape does not match n_pix");
  G->det[0] = det_panels > 0 ? det_panels : 0;
  G->det[1] = det_nx;
  G->det[2] = det_ny;
  G->nufft = plan;
  G->quats = d_quats;
  G->ppr = d_ppr;
  G->weights = d_weights;
  G->n_orient = n_orient;
  G->n_pix = n_pix;
  G->coord_scale = coord_scale;
  // the points are fixed for the solve: sort them by fine-grid bin once
  G->sorted = false;
  SPF_TRY(spf_nufft_sort_orient(plan, d_quats, n_orient, d_ppr, n_pix, coord_scale, nullptr));
  G->sorted = true;
  return SPF_OK;
}

// y = W x (form: 0 Toeplitz, 1 direct)
int spf_merge_apply(spf_merge_s *G, int form, const double *d_x, double *d_y, void *stream) {
  SPF_REQUIRE(G && d_x && d_y, "spf_merge_apply: NULL pointer");
  SPF_REQUIRE(form == 0 || (form == 1 && G->nufft), "spf_merge_apply: bad form / no direct set-up");
  cudaStream_t s = as_stream(stream);
  bool direct = form == 1;
  const bool c64 = !direct && G->conv64;
  k_load_input<<<grid1(G->n), 256, 0, s>>>(d_x, G->support, G->M, G->L,
                                           (direct || c64) ? nullptr : G->conv_in,
                                           c64 ? G->conv_in64 : nullptr, G->reg_in,
                                           direct ? G->modes : nullptr);
  SPF_TRY(check_launch("k_load_input"));
  SPF_TRY(apply_operator_core(G, direct, s));
  k_assemble<<<RED_BLOCKS, RED_THREADS, 0, s>>>(
      d_x, G->support, G->M, G->L, (direct || c64) ? nullptr : G->conv_out,
      c64 ? G->conv_out64 : nullptr, G->t1_out,
      direct ? G->direct_scale : G->conv_scale, G->reg_out, G->rlambda, G->flambda, d_y, nullptr);
  return check_launch("k_assemble");
}

// CG from x (x0 in, solution out).  hist (maxiter floats of ||r||, may be
// NULL) and the iteration count are left on the device; iters_out (device
// int, may be NULL) receives the count.
int spf_merge_cg(spf_merge_s *G, int form, const double *d_b, double *d_x, int x0_is_zero,
                 int maxiter, double rtol, double *d_hist, int *d_iters_out, void *stream) {
  SPF_REQUIRE(G && d_b && d_x, "spf_merge_cg: NULL pointer");
  SPF_REQUIRE(maxiter >= 0, "spf_merge_cg: maxiter < 0");
  SPF_REQUIRE(form == 0 || (form == 1 && G->nufft), "spf_merge_cg: bad form / no direct set-up");
  cudaStream_t s = as_stream(stream);
  bool direct = form == 1;
  const bool c64 = !direct && G->conv64;
  const int64_t n = G->n;
  // r = b - W x0
  if (x0_is_zero) {
    k_sub<<<grid1(n), 256, 0, s>>>(d_b, nullptr, G->r, n);
    SPF_TRY(check_launch("k_sub"));
  } else {
    SPF_TRY(spf_merge_apply(G, form, d_x, G->q, stream));
    k_sub<<<grid1(n), 256, 0, s>>>(d_b, G->q, G->r, n);
    SPF_TRY(check_launch("k_sub"));
  }
  k_dot_partial<<<RED_BLOCKS, RED_THREADS, 0, s>>>(d_b, d_b, n, G->partial);
  SPF_TRY(check_launch("k_dot_partial"));
  k_cg_init<<<1, RED_THREADS, 0, s>>>(G->partial, rtol, G->scal, G->flags);
  SPF_TRY(check_launch("k_cg_init"));
  SPF_TRY(check_cuda(cudaMemsetAsync(G->p, 0, n * sizeof(double), s), "spf_merge_cg"));
  for (int it = 0; it < maxiter; ++it) {
    k_dot_partial<<<RED_BLOCKS, RED_THREADS, 0, s>>>(G->r, G->r, n, G->partial);
    SPF_TRY(check_launch("k_dot_partial"));
    k_cg_stage1<<<1, RED_THREADS, 0, s>>>(G->partial, it, G->scal, G->flags, d_hist);
    SPF_TRY(check_launch("k_cg_stage1"));
    k_cg_update_p<<<grid1(n), 256, 0, s>>>(G->p, G->r, G->scal, G->flags, G->support, G->M, G->L,
                                           (direct || c64) ? nullptr : G->conv_in,
                                           c64 ? G->conv_in64 : nullptr, G->reg_in,
                                           direct ? G->modes : nullptr);
    SPF_TRY(check_launch("k_cg_update_p"));
    SPF_TRY(apply_operator_core(G, direct, s));
    k_assemble<<<RED_BLOCKS, RED_THREADS, 0, s>>>(
        G->p, G->support, G->M, G->L, (direct || c64) ? nullptr : G->conv_out,
        c64 ? G->conv_out64 : nullptr, G->t1_out,
        direct ? G->direct_scale : G->conv_scale, G->reg_out, G->rlambda, G->flambda, G->q,
        G->partial);
    SPF_TRY(check_launch("k_assemble"));
    k_cg_stage2<<<1, RED_THREADS, 0, s>>>(G->partial, G->scal, G->flags);
    SPF_TRY(check_launch("k_cg_stage2"));
    k_cg_update_xr<<<grid1(n), 256, 0, s>>>(d_x, G->r, G->p, G->q, G->scal, G->flags, n);
    SPF_TRY(check_launch("k_cg_update_xr"));
  }
  if (d_iters_out)
    SPF_TRY(check_cuda(cudaMemcpyAsync(d_iters_out, G->flags + 1, sizeof(int),
                                       cudaMemcpyDeviceToDevice, s), "spf_merge_cg"));
  return SPF_OK;
}

int spf_cg_solve(spf_merge_s *G, int form, const double *d_b, double *d_x, int x0_is_zero,
                 int maxiter, double rtol, double *d_hist, int *d_iters, void *stream) {
  return spf_merge_cg(G, form, d_b, d_x, x0_is_zero, maxiter, rtol, d_hist, d_iters, stream);
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Regularisation sweep: the MPI merge gives every rank its own
// (rlambda, flambda) and keeps the result the L-curve rule picks
// (spinifel/mpi/autocorrelation.py:64-68, 173-214).  Here the n systems
//   W_l x = c conv(x) + rlambda_l x + flambda_l reg(x) = ADb + rlambda_l x0
// (c = 1 for the sequential merge's scaling, M^3 for the MPI merge, whose
// kernel transform is not divided by M^3: mpi/autocorrelation.py:95-104)
// run as one batched CG on one GPU: every vector is [n][M^3], each pointwise
// and CG launch covers all systems (blockIdx.y, or one block per system for
// the scalar stages), and the transforms run system by system with the
// single-system plans; the regulariser runs batched (Rader over all systems
// while their buffers fit in L2 together, else system by system; batched
// D2Z / Z2D for a non-prime M).  Each system keeps its own CG scalars and
// stops on scipy's rule independently.
// per-system stride of the sweep's L-grid arrays: L^3 rounded up to 64
// floats, so that every system's array starts on a 256-byte boundary (cuFFT
// rejects an R2C input at an odd float offset)
__host__ __device__ __forceinline__ int64_t sweep_stride(int L) {
  return ((int64_t)L * L * L + 63) / 64 * 64;
}

struct Sweep {
  int nl = 0;
  double *r = nullptr, *p = nullptr, *q = nullptr, *d = nullptr, *lam = nullptr;
  float *conv_in = nullptr, *conv_out = nullptr;
  float2 *conv_freq = nullptr;
  double *reg_in = nullptr, *reg_out = nullptr;
  double2 *reg_freq = nullptr;
  double *partial = nullptr, *scal = nullptr;
  int *flags = nullptr;
  // regulariser of a non-prime M: batched D2Z / Z2D over the systems (their
  // strides handled by cuFFT; per-system offsets of an odd M^3 doubles are
  // not aligned for single-system transforms)
  cufftHandle d2z = 0, z2d = 0;
  bool m_plans = false;
  spf::PrimeDft *pd = nullptr;  // prime M: the Rader regulariser over all systems at once
};

void free_sweep(Sweep *w) {
  if (!w) return;
  void *bufs[] = {w->r,       w->p,        w->q,         w->d,       w->lam,
                  w->conv_in, w->conv_out, w->conv_freq, w->reg_in,  w->reg_out,
                  w->reg_freq, w->partial, w->scal,      w->flags};
  for (void *b : bufs)
    if (b) cudaFree(b);
  if (w->m_plans) {
    cufftDestroy(w->d2z);
    cufftDestroy(w->z2d);
  }
  spf::prime_dft_free(w->pd);
  delete w;
}

namespace spf {
namespace cg {

static int make_sweep(spf_merge_s *G, int nl) {
  if (G->sweep && G->sweep->nl == nl) return SPF_OK;
  free_sweep(G->sweep);
  G->sweep = nullptr;
  auto *w = new Sweep();
  w->nl = nl;
  const int64_t n = G->n;
  int st = SPF_OK;
  auto alloc = [&](void **ptr, size_t bytes) {
    if (st == SPF_OK) st = check_cuda(cudaMalloc(ptr, bytes), "spf_merge_cg_sweep");
  };
  alloc((void **)&w->r, nl * n * sizeof(double));
  alloc((void **)&w->p, nl * n * sizeof(double));
  alloc((void **)&w->q, nl * n * sizeof(double));
  alloc((void **)&w->d, nl * n * sizeof(double));
  alloc((void **)&w->lam, 2 * nl * sizeof(double));
  const int64_t sL = sweep_stride(G->L);
  alloc((void **)&w->conv_in, nl * sL * sizeof(float));
  alloc((void **)&w->conv_out, nl * sL * sizeof(float));
  alloc((void **)&w->conv_freq, nl * G->nLh * sizeof(float2));
  alloc((void **)&w->reg_in, nl * n * sizeof(double));
  alloc((void **)&w->reg_out, nl * n * sizeof(double));
  // the Rader buffers (two complex M^3 arrays per system) of all systems
  // together in L2: one batched regulariser; otherwise system by system with
  // the operator's own (one system's buffers stay in L2: 110 MB at M = 151)
  const bool batched_rader = (double)nl * 2.0 * (double)n * 16.0 <= 96.0 * (1 << 20);
  if (G->pd && batched_rader && st == SPF_OK) st = prime_dft_create(G->M, nl, &w->pd);
  if (!G->pd) alloc((void **)&w->reg_freq, nl * G->nMh * sizeof(double2));
  if (st == SPF_OK && !G->pd) {
    int dm[3] = {G->M, G->M, G->M};
    int em[3] = {G->M, G->M, G->M / 2 + 1};
    bool ok =
        cufftPlanMany(&w->d2z, 3, dm, dm, 1, (int)n, em, 1, (int)G->nMh, CUFFT_D2Z, nl) ==
            CUFFT_SUCCESS &&
        cufftPlanMany(&w->z2d, 3, dm, em, 1, (int)G->nMh, dm, 1, (int)n, CUFFT_Z2D, nl) ==
            CUFFT_SUCCESS;
    w->m_plans = ok;
    if (!ok) {
      set_error("spf_merge_cg_sweep: batched cuFFT plans failed (n = %d)", nl);
      st = SPF_ERR_CUDA;
    }
  }
  alloc((void **)&w->partial, nl * RED_BLOCKS * sizeof(double));
  alloc((void **)&w->scal, nl * S_COUNT * sizeof(double));
  alloc((void **)&w->flags, nl * 2 * sizeof(int));
  if (st == SPF_OK)
    st = check_cuda(cudaMemset(w->conv_in, 0, nl * sL * sizeof(float)), "spf_merge_cg_sweep");
  if (st != SPF_OK) {
    free_sweep(w);
    return st;
  }
  G->sweep = w;
  return SPF_OK;
}

// d_l = adb + rlambda_l x0 and x_l = x0 (0 when x0 is NULL)
__global__ void k_sw_rhs(const double *__restrict__ adb, const double *__restrict__ x0,
                         const double *__restrict__ lam, double *__restrict__ d,
                         double *__restrict__ x, int64_t n) {
  const int l = blockIdx.y;
  const double rl = lam[2 * l];
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double v = x0 ? x0[i] : 0.0;
    d[l * n + i] = adb[i] + rl * v;
    x[l * n + i] = v;
  }
}

// operator inputs of every system: S.v into the padded L grid (FP32) and the
// ifftshifted M grid (FP64); with p/r/scal/flags the CG update p = r + beta p
// comes first (systems that stopped keep p)
__global__ void k_sw_load(double *__restrict__ v, const double *__restrict__ r,
                          const double *__restrict__ scal, const int *__restrict__ flags,
                          const float *__restrict__ S, int M, int L, float *__restrict__ conv_in,
                          double *__restrict__ reg_in) {
  const int l = blockIdx.y;
  const int64_t n = (int64_t)M * M * M, sL = sweep_stride(L);
  const bool update = r != nullptr && !flags[2 * l];
  const double beta = r ? scal[l * S_COUNT + S_BETA] : 0.0;
  const int h = M / 2;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    double pv = v[l * n + i];
    if (update) {
      pv = r[l * n + i] + beta * pv;
      v[l * n + i] = pv;
    }
    const double vd = pv * (double)S[i];
    const unsigned iu = (unsigned)i;  // M^3 < 2^31 (M <= 1024)
    const int c = (int)(iu % M), b = (int)((iu / M) % M), a = (int)(iu / (unsigned)(M * M));
    conv_in[l * sL + ((int64_t)a * L + b) * L + c] = (float)vd;
    const int ja = (a - h + M) % M, jb = (b - h + M) % M, jc = (c - h + M) % M;
    reg_in[l * n + ((int64_t)ja * M + jb) * M + jc] = vd;
  }
}

__global__ void k_sw_mul(float2 *__restrict__ z, const float *__restrict__ w, int64_t n,
                         int64_t total) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const float s = w[i % n];
    const float2 v = z[i];
    z[i] = make_float2(v.x * s, v.y * s);
  }
}

__global__ void k_sw_mul_d(double2 *__restrict__ z, const double *__restrict__ w, int64_t n,
                           int64_t total) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double s = w[i % n];
    const double2 v = z[i];
    z[i] = make_double2(v.x * s, v.y * s);
  }
}

// q_l = W_l v_l and the partials of v_l . q_l
__global__ void __launch_bounds__(RED_THREADS)
    k_sw_assemble(const double *__restrict__ v, const float *__restrict__ S, int M, int L,
                  const float *__restrict__ conv_out, double conv_scale,
                  const double *__restrict__ reg_out, const double *__restrict__ lam,
                  double *__restrict__ q, double *__restrict__ partial) {
  const int l = blockIdx.y;
  const int64_t n = (int64_t)M * M * M, sL = sweep_stride(L);
  const int h = M / 2;
  const double reg_scale = 1.0 / ((double)M * M * M);
  const double rl = lam[2 * l], fl = lam[2 * l + 1];
  double s = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)RED_THREADS + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * RED_THREADS) {
    const unsigned iu = (unsigned)i;  // M^3 < 2^31 (M <= 1024)
    const int c = (int)(iu % M), b = (int)((iu / M) % M), a = (int)(iu / (unsigned)(M * M));
    const double sv = S[i];
    const double cv = (double)conv_out[l * sL + ((int64_t)a * L + b) * L + c];
    const int ja = (a - h + M) % M, jb = (b - h + M) % M, jc = (c - h + M) % M;
    const double rv = reg_out[l * n + ((int64_t)ja * M + jb) * M + jc];
    const double xv = v[l * n + i];
    const double qv = sv * cv * conv_scale + rl * xv + fl * sv * rv * reg_scale;
    q[l * n + i] = qv;
    s = fma(xv, qv, s);
  }
  s = block_sum(s);
  if (threadIdx.x == 0) partial[l * RED_BLOCKS + blockIdx.x] = s;
}

__global__ void __launch_bounds__(RED_THREADS)
    k_sw_dot(const double *__restrict__ a, const double *__restrict__ b, int64_t n,
             double *__restrict__ partial) {
  const int l = blockIdx.y;
  double s = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)RED_THREADS + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * RED_THREADS)
    s = fma(a[l * n + i], b[l * n + i], s);
  s = block_sum(s);
  if (threadIdx.x == 0) partial[l * RED_BLOCKS + blockIdx.x] = s;
}

// out_l = a_l - b_l
__global__ void k_sw_sub(const double *__restrict__ a, const double *__restrict__ b,
                         double *__restrict__ out, int64_t n) {
  const int l = blockIdx.y;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    out[l * n + i] = a[l * n + i] - b[l * n + i];
}

// one block per system: the scalar stages of the single-system CG
__global__ void k_sw_init(const double *partial, double rtol, double *scal, int *flags) {
  const int l = blockIdx.x;
  const double bb = sum_partials(partial + l * RED_BLOCKS);
  if (threadIdx.x == 0) {
    const double bn = sqrt(bb);
    double *sc = scal + l * S_COUNT;
    sc[S_BNORM] = bn;
    sc[S_ATOL] = rtol * bn;
    sc[S_RHO_PREV] = 1.0;
    flags[2 * l] = bn == 0.0 ? 1 : 0;
    flags[2 * l + 1] = 0;
  }
}

__global__ void k_sw_stage1(const double *partial, int it, double *scal, int *flags,
                            double *hist, int maxiter) {
  const int l = blockIdx.x;
  const double rho = sum_partials(partial + l * RED_BLOCKS);
  if (threadIdx.x == 0) {
    double *sc = scal + l * S_COUNT;
    if (hist) hist[(int64_t)l * maxiter + it] = sqrt(rho);
    if (!flags[2 * l]) {
      if (sqrt(rho) < sc[S_ATOL]) {
        flags[2 * l] = 1;
      } else {
        sc[S_RHO] = rho;
        sc[S_BETA] = it > 0 ? rho / sc[S_RHO_PREV] : 0.0;
      }
    }
  }
}

__global__ void k_sw_stage2(const double *partial, double *scal, const int *flags) {
  const int l = blockIdx.x;
  const double pq = sum_partials(partial + l * RED_BLOCKS);
  if (threadIdx.x == 0 && !flags[2 * l]) {
    double *sc = scal + l * S_COUNT;
    sc[S_PQ] = pq;
    sc[S_ALPHA] = sc[S_RHO] / pq;
    sc[S_RHO_PREV] = sc[S_RHO];
  }
}

__global__ void k_sw_update_xr(double *__restrict__ x, double *__restrict__ r,
                               const double *__restrict__ p, const double *__restrict__ q,
                               const double *__restrict__ scal, int *__restrict__ flags,
                               int64_t n) {
  const int l = blockIdx.y;
  if (flags[2 * l]) return;
  const double alpha = scal[l * S_COUNT + S_ALPHA];
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    x[l * n + i] = fma(alpha, p[l * n + i], x[l * n + i]);
    r[l * n + i] = fma(-alpha, q[l * n + i], r[l * n + i]);
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) flags[2 * l + 1] += 1;
}

// norms[2l] = sqrt(partials of slot 0), norms[2l+1] = sqrt(slot 1)
__global__ void k_sw_norm(const double *partial, double *norms, int slot) {
  const int l = blockIdx.x;
  const double v = sum_partials(partial + l * RED_BLOCKS);
  if (threadIdx.x == 0) norms[2 * l + slot] = sqrt(v);
}

__global__ void k_sw_iters(const int *flags, int *iters, int nl) {
  const int l = blockIdx.x * blockDim.x + threadIdx.x;
  if (l < nl) iters[l] = flags[2 * l + 1];
}

// W v for all systems (v already loaded into conv_in / reg_in): q = W v, and
// the partials of v . q
static int sweep_operator(spf_merge_s *G, Sweep *w, const double *v, double conv_factor,
                          cudaStream_t s) {
  // the convolution transforms run system by system with the single-system
  // plans (batched 3-D cuFFT plans measured slower); the regulariser runs
  // batched when the systems' buffers fit in L2 together; the pointwise and
  // CG kernels cover all systems per launch
  const int nl = w->nl;
  cufftSetStream(G->r2c_L, s);
  cufftSetStream(G->c2r_L, s);
  for (int l = 0; l < nl; ++l)
    SPF_TRY(cufft_ok(cufftExecR2C(G->r2c_L, w->conv_in + l * sweep_stride(G->L),
                                  reinterpret_cast<cufftComplex *>(w->conv_freq + l * G->nLh)),
                     "sweep conv R2C"));
  k_sw_mul<<<grid1(nl * G->nLh), 256, 0, s>>>(w->conv_freq, G->kernel_hat, G->nLh, nl * G->nLh);
  SPF_TRY(check_launch("k_sw_mul"));
  for (int l = 0; l < nl; ++l)
    SPF_TRY(cufft_ok(cufftExecC2R(G->c2r_L,
                                  reinterpret_cast<cufftComplex *>(w->conv_freq + l * G->nLh),
                                  w->conv_out + l * sweep_stride(G->L)),
                     "sweep conv C2R"));
  if (w->pd) {
    SPF_TRY(prime_dft_filter(w->pd, w->reg_in, G->mask_full, w->reg_out, s));
  } else if (G->pd) {
    for (int l = 0; l < nl; ++l)
      SPF_TRY(prime_dft_filter(G->pd, w->reg_in + l * G->n, G->mask_full, w->reg_out + l * G->n,
                               s));
  } else {
    cufftSetStream(w->d2z, s);
    cufftSetStream(w->z2d, s);
    SPF_TRY(cufft_ok(cufftExecD2Z(w->d2z, w->reg_in,
                                  reinterpret_cast<cufftDoubleComplex *>(w->reg_freq)),
                     "sweep reg D2Z"));
    k_sw_mul_d<<<grid1(nl * G->nMh), 256, 0, s>>>(w->reg_freq, G->mask_hat, G->nMh,
                                                  nl * G->nMh);
    SPF_TRY(check_launch("k_sw_mul_d"));
    SPF_TRY(cufft_ok(cufftExecZ2D(w->z2d, reinterpret_cast<cufftDoubleComplex *>(w->reg_freq),
                                  w->reg_out),
                     "sweep reg Z2D"));
  }
  k_sw_assemble<<<dim3(RED_BLOCKS, nl), RED_THREADS, 0, s>>>(
      v, G->support, G->M, G->L, w->conv_out, G->conv_scale * conv_factor, w->reg_out, w->lam,
      w->q, w->partial);
  return check_launch("k_sw_assemble");
}

}  // namespace cg
}  // namespace spf

extern "C" int spf_merge_cg_sweep(spf_merge_s *G, int n_lambda, double conv_factor,
                                  const double *h_rlambda, const double *h_flambda,
                                  const double *d_adb,
                                  const double *d_x0, double *d_x, int maxiter, double rtol,
                                  double *d_norms, double *d_hist, int *d_iters, void *stream) {
  using namespace spf::cg;
  SPF_REQUIRE(G && h_rlambda && h_flambda && d_adb && d_x, "spf_merge_cg_sweep: NULL pointer");
  SPF_REQUIRE(n_lambda >= 1 && n_lambda <= 64, "spf_merge_cg_sweep: n_lambda in 1..64");
  SPF_REQUIRE(maxiter >= 0, "spf_merge_cg_sweep: maxiter < 0");
  int dev = 0;
  cudaGetDevice(&dev);
  SPF_REQUIRE(dev == G->dev, "spf_merge_cg_sweep: wrong device");
  SPF_TRY(make_sweep(G, n_lambda));
  Sweep *w = G->sweep;
  cudaStream_t s = spf::as_stream(stream);
  const int nl = n_lambda;
  const int64_t n = G->n;
  std::vector<double> lam(2 * nl);
  for (int l = 0; l < nl; ++l) {
    lam[2 * l] = h_rlambda[l];
    lam[2 * l + 1] = h_flambda[l];
  }
  SPF_TRY(check_cuda(cudaMemcpyAsync(w->lam, lam.data(), 2 * nl * sizeof(double),
                                     cudaMemcpyHostToDevice, s), "spf_merge_cg_sweep"));
  // the host copy must stay valid until the copy ran
  SPF_TRY(check_cuda(cudaStreamSynchronize(s), "spf_merge_cg_sweep"));
  const dim3 gb(grid1(n), nl);
  k_sw_rhs<<<gb, 256, 0, s>>>(d_adb, d_x0, w->lam, w->d, d_x, n);
  SPF_TRY(check_launch("k_sw_rhs"));
  // r = d - W x0
  if (d_x0) {
    k_sw_load<<<gb, 256, 0, s>>>(d_x, nullptr, nullptr, nullptr, G->support, G->M, G->L,
                                 w->conv_in, w->reg_in);
    SPF_TRY(check_launch("k_sw_load"));
    SPF_TRY(sweep_operator(G, w, d_x, conv_factor, s));
    k_sw_sub<<<gb, 256, 0, s>>>(w->d, w->q, w->r, n);
  } else {
    SPF_TRY(check_cuda(cudaMemcpyAsync(w->r, w->d, nl * n * sizeof(double),
                                       cudaMemcpyDeviceToDevice, s), "spf_merge_cg_sweep"));
  }
  SPF_TRY(check_launch("k_sw_sub"));
  k_sw_dot<<<dim3(RED_BLOCKS, nl), RED_THREADS, 0, s>>>(w->d, w->d, n, w->partial);
  SPF_TRY(check_launch("k_sw_dot"));
  k_sw_init<<<nl, RED_THREADS, 0, s>>>(w->partial, rtol, w->scal, w->flags);
  SPF_TRY(check_launch("k_sw_init"));
  SPF_TRY(check_cuda(cudaMemsetAsync(w->p, 0, nl * n * sizeof(double), s), "spf_merge_cg_sweep"));
  for (int it = 0; it < maxiter; ++it) {
    k_sw_dot<<<dim3(RED_BLOCKS, nl), RED_THREADS, 0, s>>>(w->r, w->r, n, w->partial);
    SPF_TRY(check_launch("k_sw_dot"));
    k_sw_stage1<<<nl, RED_THREADS, 0, s>>>(w->partial, it, w->scal, w->flags, d_hist, maxiter);
    SPF_TRY(check_launch("k_sw_stage1"));
    k_sw_load<<<gb, 256, 0, s>>>(w->p, w->r, w->scal, w->flags, G->support, G->M, G->L,
                                 w->conv_in, w->reg_in);
    SPF_TRY(check_launch("k_sw_load"));
    SPF_TRY(sweep_operator(G, w, w->p, conv_factor, s));
    k_sw_stage2<<<nl, RED_THREADS, 0, s>>>(w->partial, w->scal, w->flags);
    SPF_TRY(check_launch("k_sw_stage2"));
    k_sw_update_xr<<<gb, 256, 0, s>>>(d_x, w->r, w->p, w->q, w->scal, w->flags, n);
    SPF_TRY(check_launch("k_sw_update_xr"));
  }
  if (d_iters) {
    k_sw_iters<<<(nl + 63) / 64, 64, 0, s>>>(w->flags, d_iters, nl);
    SPF_TRY(check_launch("k_sw_iters"));
  }
  if (d_norms) {  // ||x_l|| and ||W_l x_l - d_l|| (the reference's v1, v2)
    k_sw_dot<<<dim3(RED_BLOCKS, nl), RED_THREADS, 0, s>>>(d_x, d_x, n, w->partial);
    SPF_TRY(check_launch("k_sw_dot"));
    k_sw_norm<<<nl, RED_THREADS, 0, s>>>(w->partial, d_norms, 0);
    SPF_TRY(check_launch("k_sw_norm"));
    k_sw_load<<<gb, 256, 0, s>>>(d_x, nullptr, nullptr, nullptr, G->support, G->M, G->L,
                                 w->conv_in, w->reg_in);
    SPF_TRY(check_launch("k_sw_load"));
    SPF_TRY(sweep_operator(G, w, d_x, conv_factor, s));
    k_sw_sub<<<gb, 256, 0, s>>>(w->q, w->d, w->r, n);
    SPF_TRY(check_launch("k_sw_sub"));
    k_sw_dot<<<dim3(RED_BLOCKS, nl), RED_THREADS, 0, s>>>(w->r, w->r, n, w->partial);
    SPF_TRY(check_launch("k_sw_dot"));
    k_sw_norm<<<nl, RED_THREADS, 0, s>>>(w->partial, d_norms, 1);
    SPF_TRY(check_launch("k_sw_norm"));
  }
  return SPF_OK;
}
