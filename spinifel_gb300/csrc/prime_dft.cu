// FP64 3-D DFT of a prime size p by Rader's algorithm, for the merge's
// regulariser on the model grid (spinifel/sequential/autocorrelation.py:
// 116-128 applies fftn / ifftn on M^3 with M = 4 Mquat + 1, often prime:
// 41, 151).  cuFFT runs prime sizes as Bluestein transforms of a padded
// length >= 2p - 1 (343 for p = 151); Rader's algorithm turns the size-p
// DFT into one cyclic convolution of length p - 1 (150 = 2 3 5^2 for
// p = 151), which cuFFT runs natively, so each 1-D transform costs two
// length-(p-1) FFTs instead of two length-343 ones.
//
// With g a primitive root mod p, n = g^m (input) and k = g^-q (output), for
// k != 0:  X[g^-q] = x[0] + sum_m x[g^m] w^(g^(m-q)) = x[0] + (a (*) b)[q]
// with a[m] = x[g^m], b[j] = w^(g^-j), w = exp(-+2 pi i / p); X[0] = sum x.
// The convolution runs as IFFT(FFT(a) . FFT(b) / (p - 1)) with FFT(b) / (p - 1)
// precomputed on the host in double precision.  X[0] is x[0] plus the DC term
// of FFT(a).  A 3-D transform is three passes, one per axis; each pass
// gathers the lines along its axis into Rader order, runs the batched
// cuFFT Z2Z pair, and scatters back.
#include <cufft.h>

#include <cmath>
#include <vector>

#include "common.cuh"
#include "prime_dft.cuh"

namespace spf {
namespace pdft {

static bool is_prime(int n) {
  if (n < 2) return false;
  for (int d = 2; (int64_t)d * d <= n; ++d)
    if (n % d == 0) return false;
  return true;
}

static bool smooth(int n) {
  for (int f : {2, 3, 5, 7})
    while (n % f == 0) n /= f;
  return n == 1;
}

static int64_t powmod(int64_t b, int64_t e, int64_t m) {
  int64_t r = 1;
  b %= m;
  while (e > 0) {
    if (e & 1) r = r * b % m;
    b = b * b % m;
    e >>= 1;
  }
  return r;
}

static int primitive_root(int p) {
  std::vector<int> fac;
  int n = p - 1;
  for (int f = 2; f * f <= n; ++f)
    if (n % f == 0) {
      fac.push_back(f);
      while (n % f == 0) n /= f;
    }
  if (n > 1) fac.push_back(n);
  for (int g = 2; g < p; ++g) {
    bool ok = true;
    for (int f : fac)
      if (powmod(g, (p - 1) / f, p) == 1) {
        ok = false;
        break;
      }
    if (ok) return g;
  }
  return -1;
}

// element idx of the [nb][p][p][p] array -> (line, position along axis ax);
// 32-bit arithmetic (nb p^3 < 2^31, checked at creation)
__device__ __forceinline__ void line_of(unsigned idx, unsigned p, int ax, unsigned &line,
                                        int &n) {
  const unsigned p2 = p * p, p3 = p2 * p;
  const unsigned sys = idx / p3;
  const unsigned r = idx - sys * p3;
  const unsigned i0 = r / p2, r2 = r - i0 * p2;
  const unsigned i1 = r2 / p, i2 = r2 - i1 * p;
  unsigned u, v;
  if (ax == 2) {
    n = (int)i2; u = i0; v = i1;
  } else if (ax == 1) {
    n = (int)i1; u = i0; v = i2;
  } else {
    n = (int)i0; u = i1; v = i2;
  }
  line = sys * p2 + u * p + v;
}

// a[line][pinv[n]] = x[line, n] (n >= 1), x0[line] = x[line, 0]; the input
// is the real array xr (imaginary part 0) or the complex array z
__global__ void k_pd_gather(const double *__restrict__ xr, const double2 *__restrict__ z, int p,
                            int ax, int64_t total, const int16_t *__restrict__ pinv,
                            double2 *__restrict__ a, double2 *__restrict__ x0) {
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    unsigned line;
    int n;
    line_of((unsigned)idx, (unsigned)p, ax, line, n);
    const double2 v = xr ? make_double2(xr[idx], 0.0) : z[idx];
    if (n == 0)
      x0[line] = v;
    else
      a[(int64_t)line * (p - 1) + pinv[n]] = v;
  }
}

// a *= bh (per position), keeping the DC term of FFT(a) first
__global__ void k_pd_mul(double2 *__restrict__ a, const double2 *__restrict__ bh, int pm1,
                         int64_t total, double2 *__restrict__ dc) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const unsigned iu = (unsigned)i;  // lines (p - 1) < 2^31
    const int m = (int)(iu % (unsigned)pm1);
    const double2 v = a[i];
    if (m == 0) dc[iu / (unsigned)pm1] = v;
    const double2 b = bh[m];
    a[i] = make_double2(v.x * b.x - v.y * b.y, v.x * b.y + v.y * b.x);
  }
}

// X[line, n] = x0 + c[qinv[n]] (n >= 1), X[line, 0] = x0 + dc; optionally
// times the real multiplier h[idx mod p^3]; written to z, or its real part
// to re_out
__global__ void k_pd_scatter(const double2 *__restrict__ a, const double2 *__restrict__ x0,
                             const double2 *__restrict__ dc, int p, int ax, int64_t total,
                             const int16_t *__restrict__ qinv, const double *__restrict__ h,
                             double2 *__restrict__ z, double *__restrict__ re_out) {
  const int64_t p3 = (int64_t)p * p * p;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    unsigned line;
    int n;
    line_of((unsigned)idx, (unsigned)p, ax, line, n);
    const double2 b = x0[line];
    const double2 c = n == 0 ? dc[line] : a[(int64_t)line * (p - 1) + qinv[n]];
    double2 X = make_double2(b.x + c.x, b.y + c.y);
    if (h) {
      const double s = h[(unsigned)idx % (unsigned)p3];
      X = make_double2(X.x * s, X.y * s);
    }
    if (re_out)
      re_out[idx] = X.x;
    else
      z[idx] = X;
  }
}

}  // namespace pdft

bool prime_dft_applies(int p) {
  return p >= 5 && p <= 32767 && pdft::is_prime(p) && pdft::smooth(p - 1);
}

void prime_dft_free(PrimeDft *d) {
  if (!d) return;
  void *bufs[] = {d->pinv, d->qinv, d->bf, d->bi, d->a, d->x0, d->dc, d->z};
  for (void *b : bufs)
    if (b) cudaFree(b);
  if (d->plan_ok) cufftDestroy(d->plan);
  delete d;
}

int prime_dft_create(int p, int nb, PrimeDft **out) {
  using namespace pdft;
  *out = nullptr;
  SPF_REQUIRE(prime_dft_applies(p) && nb >= 1, "prime_dft_create: size %d not supported", p);
  SPF_REQUIRE((int64_t)nb * p * p * p < (1LL << 31), "prime_dft_create: %d x %d^3 too large", nb,
              p);
  const int g = primitive_root(p);
  SPF_REQUIRE(g > 0, "prime_dft_create: no primitive root of %d", p);
  auto *d = new PrimeDft();
  d->p = p;
  d->nb = nb;
  d->lines = (int64_t)nb * p * p;
  const int pm1 = p - 1;
  // index tables: pinv[g^m] = m, qinv[g^-q] = q
  std::vector<int16_t> pinv(p, 0), qinv(p, 0);
  const int64_t ginv = powmod(g, p - 2, p);
  for (int m = 0; m < pm1; ++m) {
    pinv[powmod(g, m, p)] = (int16_t)m;
    qinv[powmod(ginv, m, p)] = (int16_t)m;
  }
  // FFT_{p-1}(b) / (p-1) for both signs, b[j] = exp(-+2 pi i g^-j / p),
  // summed directly in double precision (angles reduced to integers mod p
  // and mod p - 1 before scaling)
  std::vector<double2> bf(pm1), bi(pm1);
  for (int k = 0; k < pm1; ++k) {
    double fr = 0, fi = 0, ir = 0, ii = 0;
    for (int j = 0; j < pm1; ++j) {
      const double tb = 2.0 * M_PI * (double)powmod(ginv, j, p) / p;
      const double tf = 2.0 * M_PI * (double)(((int64_t)j * k) % pm1) / pm1;
      // forward kernel exp(-i tb) times exp(-i tf); inverse exp(+i tb) exp(-i tf)
      fr += std::cos(tb + tf);
      fi += -std::sin(tb + tf);
      ir += std::cos(tb - tf);
      ii += std::sin(tb - tf);
    }
    bf[k] = make_double2(fr / pm1, fi / pm1);
    bi[k] = make_double2(ir / pm1, ii / pm1);
  }
  int st = SPF_OK;
  auto alloc = [&](void **ptr, size_t bytes) {
    if (st == SPF_OK) st = check_cuda(cudaMalloc(ptr, bytes), "prime_dft_create");
  };
  alloc((void **)&d->pinv, p * sizeof(int16_t));
  alloc((void **)&d->qinv, p * sizeof(int16_t));
  alloc((void **)&d->bf, pm1 * sizeof(double2));
  alloc((void **)&d->bi, pm1 * sizeof(double2));
  alloc((void **)&d->a, (size_t)d->lines * pm1 * sizeof(double2));
  alloc((void **)&d->x0, (size_t)d->lines * sizeof(double2));
  alloc((void **)&d->dc, (size_t)d->lines * sizeof(double2));
  alloc((void **)&d->z, (size_t)d->lines * p * sizeof(double2));
  if (st == SPF_OK) {
    int n[1] = {pm1};
    bool ok = cufftPlanMany(&d->plan, 1, n, nullptr, 1, pm1, nullptr, 1, pm1, CUFFT_Z2Z,
                            (int)d->lines) == CUFFT_SUCCESS;
    d->plan_ok = ok;
    if (!ok) {
      set_error("prime_dft_create: cufftPlanMany(%d x %lld) failed", pm1, (long long)d->lines);
      st = SPF_ERR_CUDA;
    }
  }
  auto upload = [&](void *dst, const void *src, size_t bytes) {
    if (st == SPF_OK)
      st = check_cuda(cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice), "prime_dft_create");
  };
  upload(d->pinv, pinv.data(), p * sizeof(int16_t));
  upload(d->qinv, qinv.data(), p * sizeof(int16_t));
  upload(d->bf, bf.data(), pm1 * sizeof(double2));
  upload(d->bi, bi.data(), pm1 * sizeof(double2));
  if (st != SPF_OK) {
    prime_dft_free(d);
    return st;
  }
  *out = d;
  return SPF_OK;
}

// one axis pass of the forward (sign -1) or inverse (sign +1, unnormalised)
// DFT; the input is xr (real) or d->z, the output d->z (times h) or the real
// part into re_out
static int axis_pass(PrimeDft *d, int ax, int sign, const double *xr, const double *h,
                     double *re_out, cudaStream_t s) {
  using namespace pdft;
  const int p = d->p, pm1 = p - 1;
  const int64_t total = d->lines * p, na = d->lines * pm1;
  const int grid = grid_for(total, 256, (int64_t)sm_count() * 8);
  k_pd_gather<<<grid, 256, 0, s>>>(xr, d->z, p, ax, total, d->pinv, d->a, d->x0);
  SPF_TRY(check_launch("k_pd_gather"));
  cufftSetStream(d->plan, s);
  auto *ca = reinterpret_cast<cufftDoubleComplex *>(d->a);
  if (cufftExecZ2Z(d->plan, ca, ca, CUFFT_FORWARD) != CUFFT_SUCCESS) {
    set_error("prime_dft: cufftExecZ2Z failed");
    return SPF_ERR_CUDA;
  }
  count_launch();
  k_pd_mul<<<grid_for(na, 256, (int64_t)sm_count() * 8), 256, 0, s>>>(
      d->a, sign < 0 ? d->bf : d->bi, pm1, na, d->dc);
  SPF_TRY(check_launch("k_pd_mul"));
  if (cufftExecZ2Z(d->plan, ca, ca, CUFFT_INVERSE) != CUFFT_SUCCESS) {
    set_error("prime_dft: cufftExecZ2Z failed");
    return SPF_ERR_CUDA;
  }
  count_launch();
  k_pd_scatter<<<grid, 256, 0, s>>>(d->a, d->x0, d->dc, p, ax, total, d->qinv, h, d->z, re_out);
  return check_launch("k_pd_scatter");
}

int prime_dft_filter(PrimeDft *d, const double *in, const double *h, double *out,
                     cudaStream_t s) {
  // forward along axes 2, 1, 0 (the multiplier applied with the last), then
  // the unnormalised inverse, keeping the real part
  SPF_TRY(axis_pass(d, 2, -1, in, nullptr, nullptr, s));
  SPF_TRY(axis_pass(d, 1, -1, nullptr, nullptr, nullptr, s));
  SPF_TRY(axis_pass(d, 0, -1, nullptr, h, nullptr, s));
  SPF_TRY(axis_pass(d, 2, +1, nullptr, nullptr, nullptr, s));
  SPF_TRY(axis_pass(d, 1, +1, nullptr, nullptr, nullptr, s));
  return axis_pass(d, 0, +1, nullptr, nullptr, out, s);
}

}  // namespace spf
