// 3D type-1 / type-2 NUFFT with the exponential-of-semicircle (ES) kernel,
// FP32 on the device, for the Spinifel slicing and merge operators.
//
// Layout in HBM (per plan):
//   fine   : n1*n2*n3 complex64, the upsampled grid the FFT works on;
//   re_pad : (n1+2p)(n2+2p)(n3+2p) float, Re of the type-2 fine grid with a
//            periodic halo of p = ceil(w/2)+1 cells on every side, so that a
//            kernel footprint never wraps (no modulo in the inner loop);
//   im_pad : same for Im (only when requested);
//   acc_pad: padded real grid that type-1 spreading accumulates into; the
//            halo is folded back onto the periodic grid before the FFT.
// A point x (radians) sits at fine-grid coordinate t = x n / (2 pi), wrapped
// into [-n/2, n/2); its footprint is the w cells l0 .. l0+w-1 with
// l0 = ceil(t - w/2), stored at padded index l + n/2 + p.
#include <cufft.h>
#include <math.h>

#include <vector>

#include "common.cuh"
#include "tma.cuh"
#include "es_params.cuh"

struct spf_nufft_plan_s {
  int dev = 0;
  int m[3] = {0, 0, 0};
  int n[3] = {0, 0, 0};
  int np[3] = {0, 0, 0};
  int pad = 0;
  int w = 0;
  double beta = 0, sigma = 2.0, eps = 1e-6;
  float *inv_p[3] = {nullptr, nullptr, nullptr};  // 1 / kernel FT per mode
  float2 *fine = nullptr;
  float *re_pad = nullptr;
  float *im_pad = nullptr;
  float *acc_pad = nullptr;
  cufftHandle fft = 0;
  bool fft_ok = false;
  // bin-sorted orientation points (spf_nufft_sort_orient)
  int32_t *sorted = nullptr;   // point indices o * n_pix + p, grouped by bin
  int4 *items = nullptr;       // (bin, start, count, 0) work items
  int64_t n_items = 0, n_sorted = 0, sorted_cap = 0, items_cap = 0;
  int nb[3] = {0, 0, 0};
  const float *s_quats = nullptr, *s_ppr = nullptr;
  const float *s_x = nullptr, *s_y = nullptr, *s_z = nullptr;  // explicit points instead
  int64_t s_n_orient = 0, s_n_pix = 0;
  double s_scale = 0;
};

namespace spf {

static int next_smooth_even(int n) { return es_next_smooth_even(n); }

// FP32 cannot resolve tolerances finer than w = 8 (the FP64 plan of
// nufft_f64.cu serves those)
static int es_width(double eps, double sigma) { return es_width_for(eps, sigma, 3, 8); }

static double es_beta(int w, double sigma) { return es_beta_for(w, sigma); }

static std::vector<float> inverse_kernel_ft(int m, int n, int w, double beta) {
  std::vector<double> d = es_inverse_kernel_ft(m, n, w, beta);
  return std::vector<float>(d.begin(), d.end());
}

// ---------------------------------------------------------------------------
// device helpers
// ---------------------------------------------------------------------------

struct GridGeom {
  int n1, n2, n3;     // fine grid
  int p1, p2, p3;     // padded dims
  int off1, off2, off3;  // n/2 + pad
  float beta;
  float half_w;
  float inv_half_w;   // 2 / w
};

static GridGeom geom_of(const spf_nufft_plan_s *P) {
  GridGeom g;
  g.n1 = P->n[0]; g.n2 = P->n[1]; g.n3 = P->n[2];
  g.p1 = P->np[0]; g.p2 = P->np[1]; g.p3 = P->np[2];
  g.off1 = P->n[0] / 2 + P->pad;
  g.off2 = P->n[1] / 2 + P->pad;
  g.off3 = P->n[2] / 2 + P->pad;
  g.beta = (float)P->beta;
  g.half_w = 0.5f * P->w;
  g.inv_half_w = 2.0f / P->w;
  return g;
}

__device__ __forceinline__ float es_eval(float z, float beta) {
  float s = fmaxf(1.0f - z * z, 0.0f);
  return expf(beta * (sqrtf(s) - 1.0f));
}

// ES kernel exp(beta (sqrt(1 - z^2) - 1)) from the hardware approximations
// (sqrt.approx, ex2.approx: relative errors near 2^-22, far below the
// kernel's own approximation error at any eps >= 1e-7); beta_log2e = beta log2(e)
__device__ __forceinline__ float es_eval_approx(float z, float beta_log2e) {
  const float s = fmaxf(fmaf(-z, z, 1.0f), 0.0f);
  float r, e;
  asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(s));
  const float x = beta_log2e * (r - 1.0f);
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(e) : "f"(x));
  return e;
}

// Padded first index and the W weights along one axis for the point at
// x (in units of the coordinate scale) with grid scale s: t = x s in grid
// units, wrapped into [-n/2, n/2).  The index arithmetic uses explicitly
// rounded operations (no contraction), so every kernel that places a point
// computes the same cell for it.
template <int W>
__device__ __forceinline__ int axis_setup(float x, float s, int n, int off, float beta,
                                          float inv_half_w, float *wt) {
  float fn = (float)n;
  float t = __fmul_rn(x, s);
  t = __fsub_rn(t, __fmul_rn(fn, floorf(__fadd_rn(__fdiv_rn(t, fn), 0.5f))));
  float l0 = ceilf(__fsub_rn(t, 0.5f * W));
#pragma unroll
  for (int a = 0; a < W; ++a) {
    float z = (l0 + (float)a - t) * inv_half_w;
    wt[a] = es_eval(z, beta);
  }
  return (int)l0 + off;
}

// axis_setup with the kernel values from es_eval_approx (the type-2 slicing
// kernels: every kernel that slices through here gives the same bits)
template <int W>
__device__ __forceinline__ int axis_setup_approx(float x, float s, int n, int off,
                                                 float beta_log2e, float inv_half_w, float *wt) {
  float fn = (float)n;
  float t = __fmul_rn(x, s);
  t = __fsub_rn(t, __fmul_rn(fn, floorf(__fadd_rn(__fdiv_rn(t, fn), 0.5f))));
  float l0 = ceilf(__fsub_rn(t, 0.5f * W));
#pragma unroll
  for (int a = 0; a < W; ++a) wt[a] = es_eval_approx((l0 + (float)a - t) * inv_half_w, beta_log2e);
  return (int)l0 + off;
}

template <int W>
__device__ __forceinline__ float interp_point(const float *__restrict__ grid, const GridGeom &g,
                                              float x1, float s1, float x2, float s2, float x3,
                                              float s3) {
  float w1[W], w2[W], w3[W];
  const float bl2 = g.beta * 1.4426950408889634f;
  int i0 = axis_setup_approx<W>(x1, s1, g.n1, g.off1, bl2, g.inv_half_w, w1);
  int j0 = axis_setup_approx<W>(x2, s2, g.n2, g.off2, bl2, g.inv_half_w, w2);
  int k0 = axis_setup_approx<W>(x3, s3, g.n3, g.off3, bl2, g.inv_half_w, w3);
  float acc = 0.0f;
#pragma unroll
  for (int a = 0; a < W; ++a) {
    float acc_a = 0.0f;
#pragma unroll
    for (int b = 0; b < W; ++b) {
      const float *row = grid + ((size_t)(i0 + a) * g.p2 + (j0 + b)) * g.p3 + k0;
      float r = 0.0f;
#pragma unroll
      for (int c = 0; c < W; ++c) r = fmaf(w3[c], __ldg(row + c), r);
      acc_a = fmaf(w2[b], r, acc_a);
    }
    acc = fmaf(w1[a], acc_a, acc);
  }
  return acc;
}

template <int W>
__device__ __forceinline__ void spread_point(float *__restrict__ grid, const GridGeom &g, float x1,
                                             float s1, float x2, float s2, float x3, float s3,
                                             float c) {
  float w1[W], w2[W], w3[W];
  int i0 = axis_setup<W>(x1, s1, g.n1, g.off1, g.beta, g.inv_half_w, w1);
  int j0 = axis_setup<W>(x2, s2, g.n2, g.off2, g.beta, g.inv_half_w, w2);
  int k0 = axis_setup<W>(x3, s3, g.n3, g.off3, g.beta, g.inv_half_w, w3);
#pragma unroll
  for (int c3 = 0; c3 < W; ++c3) w3[c3] *= c;
#pragma unroll
  for (int a = 0; a < W; ++a) {
#pragma unroll
    for (int b = 0; b < W; ++b) {
      float wab = w1[a] * w2[b];
      float *row = grid + ((size_t)(i0 + a) * g.p2 + (j0 + b)) * g.p3 + k0;
#pragma unroll
      for (int c3 = 0; c3 < W; ++c3) atomicAdd(row + c3, wab * w3[c3]);
    }
  }
}

// Rotation of pixel position q by the inverse of R(quat) (quat = [w,x,y,z],
// spinifel/extern/nufft_ext.py:59-60 with eval/geom.py:9-48), scaled.
__device__ __forceinline__ void rotate_inv(const float *__restrict__ quat, float qx, float qy,
                                           float qz, float s, float &h, float &k, float &l) {
  float q0 = quat[0], q1 = quat[1], q2 = quat[2], q3 = quat[3];
  float r00 = 1.f - 2.f * (q2 * q2 + q3 * q3), r01 = 2.f * (q1 * q2 - q0 * q3),
        r02 = 2.f * (q1 * q3 + q0 * q2);
  float r10 = 2.f * (q1 * q2 + q0 * q3), r11 = 1.f - 2.f * (q1 * q1 + q3 * q3),
        r12 = 2.f * (q2 * q3 - q0 * q1);
  float r20 = 2.f * (q1 * q3 - q0 * q2), r21 = 2.f * (q2 * q3 + q0 * q1),
        r22 = 1.f - 2.f * (q1 * q1 + q2 * q2);
  // R^-1 = R^T for a unit quaternion (explicitly rounded: no contraction)
  h = __fmul_rn(s, __fadd_rn(__fadd_rn(__fmul_rn(r00, qx), __fmul_rn(r10, qy)), __fmul_rn(r20, qz)));
  k = __fmul_rn(s, __fadd_rn(__fadd_rn(__fmul_rn(r01, qx), __fmul_rn(r11, qy)), __fmul_rn(r21, qz)));
  l = __fmul_rn(s, __fadd_rn(__fadd_rn(__fmul_rn(r02, qx), __fmul_rn(r12, qy)), __fmul_rn(r22, qz)));
}

// ---------------------------------------------------------------------------
// kernels
// ---------------------------------------------------------------------------

// b[k mod n] = f_k * support_k / (p1 p2 p3), complex fine grid pre-zeroed.
__global__ void k_t2_scatter_modes(const float *__restrict__ f, const float *__restrict__ sup,
                                   int m1, int m2, int m3, int n1, int n2, int n3,
                                   const float *__restrict__ ip1, const float *__restrict__ ip2,
                                   const float *__restrict__ ip3, float2 *__restrict__ fine) {
  int64_t total = (int64_t)m1 * m2 * m3;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    int c = (int)(idx % m3);
    int b = (int)((idx / m3) % m2);
    int a = (int)(idx / ((int64_t)m2 * m3));
    float v = f[idx];
    if (sup) v *= sup[idx];
    v *= ip1[a] * ip2[b] * ip3[c];
    int fa = ((a - m1 / 2) % n1 + n1) % n1;
    int fb = ((b - m2 / 2) % n2 + n2) % n2;
    int fc = ((c - m3 / 2) % n3 + n3) % n3;
    fine[((int64_t)fa * n2 + fb) * n3 + fc] = make_float2(v, 0.0f);
  }
}

// re_pad[i] = Re fine[(i - off) mod n] (and Im), for every padded cell.
__global__ void k_t2_fill_padded(const float2 *__restrict__ fine, GridGeom g, float im_sign,
                                 float *__restrict__ re_pad, float *__restrict__ im_pad) {
  int64_t total = (int64_t)g.p1 * g.p2 * g.p3;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    int k = (int)(idx % g.p3);
    int j = (int)((idx / g.p3) % g.p2);
    int i = (int)(idx / ((int64_t)g.p2 * g.p3));
    int a = ((i - g.off1) % g.n1 + g.n1) % g.n1;
    int b = ((j - g.off2) % g.n2 + g.n2) % g.n2;
    int c = ((k - g.off3) % g.n3 + g.n3) % g.n3;
    float2 v = fine[((int64_t)a * g.n2 + b) * g.n3 + c];
    re_pad[idx] = v.x;
    if (im_pad) im_pad[idx] = im_sign * v.y;
  }
}

template <int W>
__global__ void k_t2_interp(const float *__restrict__ re_pad, const float *__restrict__ im_pad,
                            GridGeom g, const float *__restrict__ x, const float *__restrict__ y,
                            const float *__restrict__ z, int64_t npts, float *__restrict__ out_re,
                            float *__restrict__ out_im) {
  const float sc1 = g.n1 * (float)(0.5 / M_PI), sc2 = g.n2 * (float)(0.5 / M_PI),
              sc3 = g.n3 * (float)(0.5 / M_PI);
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < npts;
       j += (int64_t)gridDim.x * blockDim.x) {
    out_re[j] = interp_point<W>(re_pad, g, x[j], sc1, y[j], sc2, z[j], sc3);
    if (out_im) out_im[j] = interp_point<W>(im_pad, g, x[j], sc1, y[j], sc2, z[j], sc3);
  }
}

template <int W>
__global__ void k_slice_t2(const float *__restrict__ re_pad, GridGeom g,
                           const float *__restrict__ quats, const float *__restrict__ ppr,
                           int64_t n_pix, float scale1, float scale2, float scale3,
                           float *__restrict__ out, __nv_bfloat16 *__restrict__ out_bf16) {
  int64_t o = blockIdx.x;
  int64_t p = blockIdx.y * (int64_t)blockDim.x + threadIdx.x;
  if (p >= n_pix) return;
  float h, k, l;
  rotate_inv(quats + 4 * o, ppr[p], ppr[n_pix + p], ppr[2 * n_pix + p], 1.0f, h, k, l);
  float v = interp_point<W>(re_pad, g, h, scale1, k, scale2, l, scale3);
  int64_t idx = o * n_pix + p;
  out[idx] = v;
  if (out_bf16) out_bf16[idx] = __float2bfloat16_rn(v);
}

// Shared-memory boxes of the padded grid: a box of di x dj x dk cells at
// (imin, jmin, kmin), stored with plane stride sp and row stride sr floats.  Rows are
// walked by half-warps (dk <= 16) or warps with the lanes along the fastest
// axis, so the global side is coalesced and there is one division per row,
// not per cell.
struct BoxShape {
  int imin, jmin, kmin, di, dj, dk;
  int sp, sr;  // plane and row strides in floats: cell (ii, jj, kk) at ii*sp + jj*sr + kk
};

template <class F>
__device__ __forceinline__ void box_rows(const BoxShape &b, F &&f) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const bool half = b.dk <= 16;
  const int l = half ? (lane & 15) : lane;
  const int step = half ? 16 : 32;
  const int rpw = half ? 2 : 1;
  const int rows = b.di * b.dj;
  for (int r = warp * rpw + (half ? (lane >> 4) : 0); r < rows; r += nw * rpw) {
    const int ii = r / b.dj, jj = r - ii * b.dj;
    for (int kk = l; kk < b.dk; kk += step) f(ii, jj, kk, ii * b.sp + jj * b.sr + kk);
  }
}

__device__ __forceinline__ size_t box_global(const GridGeom &g, const BoxShape &b, int ii, int jj,
                                             int kk) {
  return ((size_t)(b.imin + ii) * g.p2 + (b.jmin + jj)) * g.p3 + b.kmin + kk;
}

// Box fill: thread t loads cells t, t + blockDim.x, ... (coalesced along the
// fastest axis), four loads in flight before their stores; the cell index
// advances by a mixed-radix step instead of a division per cell.
__device__ __forceinline__ void box_load(float *box, const float *__restrict__ grid,
                                         const GridGeom &g, const BoxShape &b) {
  constexpr int U = 4;
  const int vol = b.di * b.dj * b.dk;
  const int nt = blockDim.x;
  int idx = threadIdx.x;
  int kk = idx % b.dk, jj = (idx / b.dk) % b.dj, ii = idx / (b.dk * b.dj);
  const int stk = nt % b.dk, stj = (nt / b.dk) % b.dj, sti = nt / (b.dk * b.dj);
  while (idx < vol) {
    float v[U];
    int dst[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      dst[u] = -1;
      v[u] = 0.0f;
      if (idx < vol) {
        dst[u] = ii * b.sp + jj * b.sr + kk;
        v[u] = __ldg(grid + box_global(g, b, ii, jj, kk));
      }
      idx += nt;
      kk += stk;
      jj += stj;
      ii += sti;
      if (kk >= b.dk) {
        kk -= b.dk;
        ++jj;
      }
      if (jj >= b.dj) {
        jj -= b.dj;
        ++ii;
      }
    }
#pragma unroll
    for (int u = 0; u < U; ++u)
      if (dst[u] >= 0) box[dst[u]] = v[u];
  }
}

// Box fill with 16-byte loads, for a padded grid whose rows are 16-byte
// aligned (p3 % 4 == 0): each box row [kmin, kmin + dk) is read as the
// aligned quads from kmin & ~3, which never leave the grid row; unit (row,
// quad) goes to thread unit mod blockDim.x, four loads in flight, and each
// quad stores the cells that lie inside the box row.  Fills the same cells
// with the same values as box_load, in about a third of the instructions.
__device__ __forceinline__ void box_load_q(float *box, const float *__restrict__ grid,
                                           const GridGeom &g, const BoxShape &b) {
  constexpr int U = 2;
  const int lead = b.kmin & 3;
  const int nq = (lead + b.dk + 3) >> 2;
  const int units = b.di * b.dj * nq;
  const int nt = blockDim.x;
  const int p3q = g.p3 >> 2, p2q = g.p2 * p3q;
  const float4 *base = reinterpret_cast<const float4 *>(
      grid + ((size_t)b.imin * g.p2 + b.jmin) * g.p3 + (b.kmin - lead));
  int u = threadIdx.x;
  int q = u % nq, r = u / nq;
  int jj = r % b.dj, ii = r / b.dj;
  const int stq = nt % nq, str = nt / nq;
  const int stj = str % b.dj, sti = str / b.dj;
  while (u < units) {
    float4 v[U];
    int row[U], c0[U];
    bool ok[U];
#pragma unroll
    for (int x = 0; x < U; ++x) {
      ok[x] = u < units;
      row[x] = ii * b.sp + jj * b.sr;
      c0[x] = 4 * q - lead;
      if (ok[x]) v[x] = __ldg(base + (ii * p2q + jj * p3q + q));
      u += nt;
      q += stq;
      jj += stj;
      ii += sti;
      if (q >= nq) {
        q -= nq;
        ++jj;
      }
      if (jj >= b.dj) {
        jj -= b.dj;
        ++ii;
      }
    }
#pragma unroll
    for (int x = 0; x < U; ++x) {
      if (!ok[x]) continue;
      const float e[4] = {v[x].x, v[x].y, v[x].z, v[x].w};
#pragma unroll
      for (int t = 0; t < 4; ++t) {
        const int c = c0[x] + t;
        if (c >= 0 && c < b.dk) box[row[x] + c] = e[t];
      }
    }
  }
}

__device__ __forceinline__ void box_flush(const float *box, float *__restrict__ grid,
                                          const GridGeom &g, const BoxShape &b) {
  box_rows(b, [&](int ii, int jj, int kk, int s) {
    const float v = box[s];
    if (v != 0.0f) atomicAdd(grid + box_global(g, b, ii, jj, kk), v);
  });
}

// Slicing on a multi-panel detector [n_panels][nx][ny]: a CTA of 256 threads
// takes a 16 x 16 pixel patch of one panel at one orientation, so its points
// are neighbours on the Ewald sphere.  It finds the bounding box of their
// kernel footprints in the padded fine grid, stages that box in shared memory
// (coalesced along the fastest axis) and interpolates from there; a box too
// large for shared memory (a patch seen edge-on) reads the grid directly.
// The arithmetic per point is that of k_slice_t2, so the values are identical.
constexpr int SLICE_PATCH = 16;

// Pixel of thread t within its 16 x 16 patch: warp w takes the 4 x 8 block at
// rows 4 (w / 2), columns 8 (w % 2), so a warp's 32 pixels are compact on the
// detector, their footprints overlap more and their shared-memory reads hit
// fewer distinct cells.
__device__ __forceinline__ int patch_dx(int t) { return ((t >> 5) >> 1) * 4 + ((t & 31) >> 3); }
__device__ __forceinline__ int patch_dy(int t) { return ((t >> 5) & 1) * 8 + (t & 7); }
constexpr int SLICE_SMEM_FLOATS = 11264;  // 44 KB

// Tile shapes of the slicing kernel (256 threads, one pixel each): the patch
// is px x py pixels of a panel and each warp takes a wx x wy block of it.
// The shape decides how many distinct box rows a warp's loads touch (bank
// conflicts) and the box's size; which is fastest depends on the detector's
// pixel spacing in grid cells, so the autotuner picks it
// (SPF_TUNE_SLICE_SHAPE).  Every shape gives the same bits.
//
// search picks the box's row and plane strides per CTA: a lane's W^3 loads
// all sit at fixed offsets from its footprint start, so the bank of that
// start, ((li * sj + lj) * sk + lk) mod 32, fixes the warp's bank conflicts
// for the whole interpolation.  The CTA scores 16 candidate strides (sj = dj
// + 0..3, sk = dk + 0..3) by the number of distinct banks its warps'
// footprint starts hit (one warp-wide OR of bank bits per candidate) and
// keeps the best one that fits in shared memory.
struct PatchShape {
  int px, py, wx, wy, search;
};
constexpr int N_SLICE_SHAPES = 8;
constexpr int SLICE_SEARCH = 4;  // candidates per stride
__host__ __device__ inline PatchShape slice_shape(int code) {
  switch (code) {
    case 1: return PatchShape{16, 16, 8, 4, 0};
    case 2: return PatchShape{8, 32, 2, 16, 0};
    case 3: return PatchShape{8, 32, 4, 8, 0};
    case 4: return PatchShape{32, 8, 8, 4, 0};
    case 5: return PatchShape{32, 8, 16, 2, 0};
    case 6: return PatchShape{16, 16, 4, 8, 1};
    case 7: return PatchShape{16, 16, 8, 4, 1};
    default: return PatchShape{16, 16, 4, 8, 0};
  }
}

template <int W, bool SEARCH>
__global__ void __launch_bounds__(256)
    k_slice_t2_det(const float *__restrict__ re_pad, GridGeom g, const float *__restrict__ quats,
                   const float *__restrict__ ppr, int n_panels, int nx, int ny, float scale1,
                   float scale2, float scale3, float *__restrict__ out,
                   __nv_bfloat16 *__restrict__ out_bf16, PatchShape ps) {
  __shared__ float box[SLICE_SMEM_FLOATS];
  constexpr int NCAND = SLICE_SEARCH * SLICE_SEARCH;
  __shared__ int bb[7];
  __shared__ int score[8][NCAND];
  const int64_t o = blockIdx.x;
  const int patches_y = (ny + ps.py - 1) / ps.py;
  const int patches_x = (nx + ps.px - 1) / ps.px;
  const int pid = blockIdx.y;
  const int panel = pid / (patches_x * patches_y);
  const int rem = pid % (patches_x * patches_y);
  const int t = (int)threadIdx.x, warp = t >> 5, lane = t & 31;
  const int warps_y = ps.py / ps.wy;
  const int px = (rem / patches_y) * ps.px + (warp / warps_y) * ps.wx + lane / ps.wy;
  const int py = (rem % patches_y) * ps.py + (warp % warps_y) * ps.wy + lane % ps.wy;
  const bool valid = px < nx && py < ny && panel < n_panels;
  const int64_t n_pix = (int64_t)n_panels * nx * ny;
  const int64_t p = ((int64_t)panel * nx + (valid ? px : 0)) * ny + (valid ? py : 0);
  if (threadIdx.x < 6) bb[threadIdx.x] = (threadIdx.x < 3) ? INT32_MAX : INT32_MIN;
  __syncthreads();
  float h, k, l;
  rotate_inv(quats + 4 * o, ppr[p], ppr[n_pix + p], ppr[2 * n_pix + p], 1.0f, h, k, l);
  float w1[W], w2[W], w3[W];
  const float bl2 = g.beta * 1.4426950408889634f;
  int i0 = axis_setup_approx<W>(h, scale1, g.n1, g.off1, bl2, g.inv_half_w, w1);
  int j0 = axis_setup_approx<W>(k, scale2, g.n2, g.off2, bl2, g.inv_half_w, w2);
  int k0 = axis_setup_approx<W>(l, scale3, g.n3, g.off3, bl2, g.inv_half_w, w3);
  {
    int mi = valid ? i0 : INT32_MAX, mj = valid ? j0 : INT32_MAX, mk = valid ? k0 : INT32_MAX;
    int xi = valid ? i0 : INT32_MIN, xj = valid ? j0 : INT32_MIN, xk = valid ? k0 : INT32_MIN;
    mi = __reduce_min_sync(0xffffffffu, mi);
    mj = __reduce_min_sync(0xffffffffu, mj);
    mk = __reduce_min_sync(0xffffffffu, mk);
    xi = __reduce_max_sync(0xffffffffu, xi);
    xj = __reduce_max_sync(0xffffffffu, xj);
    xk = __reduce_max_sync(0xffffffffu, xk);
    if ((threadIdx.x & 31) == 0) {
      atomicMin(&bb[0], mi);
      atomicMin(&bb[1], mj);
      atomicMin(&bb[2], mk);
      atomicMax(&bb[3], xi);
      atomicMax(&bb[4], xj);
      atomicMax(&bb[5], xk);
    }
  }
  __syncthreads();
  const int imin = bb[0], jmin = bb[1], kmin = bb[2];
  const int di = bb[3] - imin + W, dj = bb[4] - jmin + W, dk = bb[5] - kmin + W;
  // odd row strides spread neighbouring points' rows over the banks
  int sj = dj | 1, sk = dk | 1;
  if (SEARCH && bb[3] >= imin) {
    const int li = i0 - imin, lj = j0 - jmin, lk = k0 - kmin;
    const unsigned vmask = valid ? 0xffffffffu : 0u;
    unsigned mine = 0;  // lane c keeps candidate c's bank bits
#pragma unroll
    for (int a = 0; a < SLICE_SEARCH; ++a) {
      const int r = li * (dj + a) + lj;
      int start = r * dk + lk;
#pragma unroll
      for (int b = 0; b < SLICE_SEARCH; ++b) {
        const unsigned m = __reduce_or_sync(0xffffffffu, (1u << (start & 31)) & vmask);
        if (lane == a * SLICE_SEARCH + b) mine = m;
        start += r;
      }
    }
    if (lane < NCAND) score[warp][lane] = __popc(mine);
    __syncthreads();
    if (warp == 0) {
      const int sjc = dj + lane / SLICE_SEARCH, skc = dk + lane % SLICE_SEARCH;
      int tot = 0;
      if (lane < NCAND)
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) tot += score[w][lane];
      const bool fits = lane < NCAND && (int64_t)di * sjc * skc <= SLICE_SMEM_FLOATS;
      // most distinct banks; ties go to the lower candidate (the smaller box)
      const int key = fits ? (tot << 5) | (31 - lane) : -1;
      const int best = __reduce_max_sync(0xffffffffu, key);
      if (lane == 0) bb[6] = best < 0 ? -1 : 31 - (best & 31);
    }
    __syncthreads();
    if (bb[6] >= 0) {
      sj = dj + bb[6] / SLICE_SEARCH;
      sk = dk + bb[6] % SLICE_SEARCH;
    }
  }
  const int64_t svol = (int64_t)di * sj * sk;
  float acc = 0.0f;
  if (bb[3] >= imin && svol <= SLICE_SMEM_FLOATS) {
    const BoxShape shape{imin, jmin, kmin, di, dj, dk, sj * sk, sk};
    if ((g.p3 & 3) == 0)
      box_load_q(box, re_pad, g, shape);
    else
      box_load(box, re_pad, g, shape);
    __syncthreads();
    // only valid points' footprints are inside the box
    if (!valid) return;
    const int li = i0 - imin, lj = j0 - jmin, lk = k0 - kmin;
#pragma unroll
    for (int a = 0; a < W; ++a) {
      float acc_a = 0.0f;
#pragma unroll
      for (int b = 0; b < W; ++b) {
        const float *row = box + ((li + a) * sj + (lj + b)) * sk + lk;
        float r = 0.0f;
#pragma unroll
        for (int c = 0; c < W; ++c) r = fmaf(w3[c], row[c], r);
        acc_a = fmaf(w2[b], r, acc_a);
      }
      acc = fmaf(w1[a], acc_a, acc);
    }
  } else {
    if (!valid) return;
#pragma unroll
    for (int a = 0; a < W; ++a) {
      float acc_a = 0.0f;
#pragma unroll
      for (int b = 0; b < W; ++b) {
        const float *row = re_pad + ((size_t)(i0 + a) * g.p2 + (j0 + b)) * g.p3 + k0;
        float r = 0.0f;
#pragma unroll
        for (int c = 0; c < W; ++c) r = fmaf(w3[c], __ldg(row + c), r);
        acc_a = fmaf(w2[b], r, acc_a);
      }
      acc = fmaf(w1[a], acc_a, acc);
    }
  }
  if (!valid) return;
  int64_t idx = o * n_pix + p;
  out[idx] = acc;
  if (out_bf16) out_bf16[idx] = __float2bfloat16_rn(acc);
}

// Shared pieces of the patch kernels: pixel of this thread, its footprint and
// the CTA's bounding box of footprints.
struct PatchPoint {
  bool valid;
  int64_t p;
  int i0, j0, k0;
};

template <int W>
__device__ __forceinline__ PatchPoint patch_point(const GridGeom &g, const float *__restrict__ quat,
                                                  const float *__restrict__ ppr, int n_panels,
                                                  int nx, int ny, float s1, float s2, float s3,
                                                  float *w1, float *w2, float *w3) {
  const int patches_y = (ny + SLICE_PATCH - 1) / SLICE_PATCH;
  const int patches_x = (nx + SLICE_PATCH - 1) / SLICE_PATCH;
  const int pid = blockIdx.y;
  const int panel = pid / (patches_x * patches_y);
  const int rem = pid % (patches_x * patches_y);
  const int px = (rem / patches_y) * SLICE_PATCH + patch_dx((int)threadIdx.x);
  const int py = (rem % patches_y) * SLICE_PATCH + patch_dy((int)threadIdx.x);
  PatchPoint pt;
  pt.valid = px < nx && py < ny && panel < n_panels;
  const int64_t n_pix = (int64_t)n_panels * nx * ny;
  pt.p = ((int64_t)panel * nx + (pt.valid ? px : 0)) * ny + (pt.valid ? py : 0);
  float h, k, l;
  rotate_inv(quat, ppr[pt.p], ppr[n_pix + pt.p], ppr[2 * n_pix + pt.p], 1.0f, h, k, l);
  pt.i0 = axis_setup<W>(h, s1, g.n1, g.off1, g.beta, g.inv_half_w, w1);
  pt.j0 = axis_setup<W>(k, s2, g.n2, g.off2, g.beta, g.inv_half_w, w2);
  pt.k0 = axis_setup<W>(l, s3, g.n3, g.off3, g.beta, g.inv_half_w, w3);
  return pt;
}

// bb must be shared int[6]; returns false when no thread of the CTA is valid
__device__ __forceinline__ bool patch_box(const PatchPoint &pt, int *bb) {
  if (threadIdx.x < 6) bb[threadIdx.x] = (threadIdx.x < 3) ? INT32_MAX : INT32_MIN;
  __syncthreads();
  int mi = pt.valid ? pt.i0 : INT32_MAX, mj = pt.valid ? pt.j0 : INT32_MAX;
  int mk = pt.valid ? pt.k0 : INT32_MAX;
  int xi = pt.valid ? pt.i0 : INT32_MIN, xj = pt.valid ? pt.j0 : INT32_MIN;
  int xk = pt.valid ? pt.k0 : INT32_MIN;
  mi = __reduce_min_sync(0xffffffffu, mi);
  mj = __reduce_min_sync(0xffffffffu, mj);
  mk = __reduce_min_sync(0xffffffffu, mk);
  xi = __reduce_max_sync(0xffffffffu, xi);
  xj = __reduce_max_sync(0xffffffffu, xj);
  xk = __reduce_max_sync(0xffffffffu, xk);
  if ((threadIdx.x & 31) == 0) {
    atomicMin(&bb[0], mi);
    atomicMin(&bb[1], mj);
    atomicMin(&bb[2], mk);
    atomicMax(&bb[3], xi);
    atomicMax(&bb[4], xj);
    atomicMax(&bb[5], xk);
  }
  __syncthreads();
  return bb[3] >= bb[0];
}

// Type-1 spreading on a multi-panel detector: the CTA's 256 points spread
// into a shared-memory copy of their footprint box (shared atomics), which is
// then added to the padded accumulator once per cell (W^3 global atomics per
// point become about (box volume / 256)).  Boxes too large for shared memory
// spread straight to global memory.
constexpr int SPREAD_SMEM_FLOATS = 11264;

template <int W, bool INTERP>
__global__ void __launch_bounds__(256)
    k_spread_det(const float *__restrict__ re_pad, float *__restrict__ acc_pad, GridGeom g,
                 const float *__restrict__ quats, const float *__restrict__ ppr, int n_panels,
                 int nx, int ny, float s1, float s2, float s3, const float *__restrict__ vals) {
  __shared__ float box[SPREAD_SMEM_FLOATS];
  __shared__ int bb[6];
  const int64_t o = blockIdx.x;
  const int64_t n_pix = (int64_t)n_panels * nx * ny;
  float w1[W], w2[W], w3[W];
  PatchPoint pt = patch_point<W>(g, quats + 4 * o, ppr, n_panels, nx, ny, s1, s2, s3, w1, w2, w3);
  if (!patch_box(pt, bb)) return;
  const int imin = bb[0], jmin = bb[1], kmin = bb[2];
  const int di = bb[3] - imin + W, dj = bb[4] - jmin + W, dk = bb[5] - kmin + W;
  const int64_t vol = (int64_t)di * dj * dk;
  const bool staged = vol <= SPREAD_SMEM_FLOATS;
  const BoxShape shape{imin, jmin, kmin, di, dj, dk, dj * dk, dk};
  float v = 0.0f;
  if constexpr (INTERP) {
    // interpolate from the type-2 grid first (staged through the same box)
    if (staged) {
      box_load(box, re_pad, g, shape);
      __syncthreads();
    }
    const int li = pt.i0 - imin, lj = pt.j0 - jmin, lk = pt.k0 - kmin;
    if (pt.valid) {  // only valid points' footprints are inside the box
#pragma unroll
      for (int a = 0; a < W; ++a) {
        float acc_a = 0.0f;
#pragma unroll
        for (int b = 0; b < W; ++b) {
          const float *row = staged ? box + ((li + a) * dj + (lj + b)) * dk + lk
                                    : re_pad + ((size_t)(pt.i0 + a) * g.p2 + (pt.j0 + b)) * g.p3 +
                                          pt.k0;
          float r = 0.0f;
#pragma unroll
          for (int c = 0; c < W; ++c) r = fmaf(w3[c], row[c], r);
          acc_a = fmaf(w2[b], r, acc_a);
        }
        v = fmaf(w1[a], acc_a, v);
      }
      if (vals) v *= vals[o * n_pix + pt.p];
    }
    if (staged) __syncthreads();  // everyone has read the box before it is reused
  } else {
    v = vals[o * n_pix + pt.p];
  }
  if (!pt.valid) v = 0.0f;
  if (staged) {
    for (int idx = threadIdx.x; idx < (int)vol; idx += blockDim.x) box[idx] = 0.0f;
    __syncthreads();
    if (v != 0.0f) {
      const int li = pt.i0 - imin, lj = pt.j0 - jmin, lk = pt.k0 - kmin;
#pragma unroll
      for (int a = 0; a < W; ++a) {
#pragma unroll
        for (int b = 0; b < W; ++b) {
          float wab = w1[a] * w2[b] * v;
          float *row = box + ((li + a) * dj + (lj + b)) * dk + lk;
#pragma unroll
          for (int c = 0; c < W; ++c) atomicAdd(row + c, wab * w3[c]);
        }
      }
    }
    __syncthreads();
    box_flush(box, acc_pad, g, shape);
  } else if (v != 0.0f) {
#pragma unroll
    for (int a = 0; a < W; ++a) {
#pragma unroll
      for (int b = 0; b < W; ++b) {
        float wab = w1[a] * w2[b] * v;
        float *row = acc_pad + ((size_t)(pt.i0 + a) * g.p2 + (pt.j0 + b)) * g.p3 + pt.k0;
#pragma unroll
        for (int c = 0; c < W; ++c) atomicAdd(row + c, wab * w3[c]);
      }
    }
  }
}

template <int W>
__global__ void k_t1_spread(float *__restrict__ acc_pad, GridGeom g, const float *__restrict__ x,
                            const float *__restrict__ y, const float *__restrict__ z,
                            const float *__restrict__ c, int64_t npts) {
  const float sc1 = g.n1 * (float)(0.5 / M_PI), sc2 = g.n2 * (float)(0.5 / M_PI),
              sc3 = g.n3 * (float)(0.5 / M_PI);
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < npts;
       j += (int64_t)gridDim.x * blockDim.x) {
    float cj = c[j];
    if (cj == 0.0f) continue;
    spread_point<W>(acc_pad, g, x[j], sc1, y[j], sc2, z[j], sc3, cj);
  }
}

template <int W>
__global__ void k_t1_spread_orient(float *__restrict__ acc_pad, GridGeom g,
                                   const float *__restrict__ quats, const float *__restrict__ ppr,
                                   int64_t n_pix, float scale1, float scale2, float scale3,
                                   const float *__restrict__ c) {
  int64_t o = blockIdx.x;
  int64_t p = blockIdx.y * (int64_t)blockDim.x + threadIdx.x;
  if (p >= n_pix) return;
  float cj = c[o * n_pix + p];
  if (cj == 0.0f) return;
  float h, k, l;
  rotate_inv(quats + 4 * o, ppr[p], ppr[n_pix + p], ppr[2 * n_pix + p], 1.0f, h, k, l);
  spread_point<W>(acc_pad, g, h, scale1, k, scale2, l, scale3, cj);
}

// Fused type 2 -> type 1 at the same points (the direct A^H D A operator):
// each point interpolates Re of the type-2 fine grid, multiplies by its
// weight and spreads the result back with the same kernel weights.
template <int W>
__global__ void k_interp_spread_orient(const float *__restrict__ re_pad,
                                       float *__restrict__ acc_pad, GridGeom g,
                                       const float *__restrict__ quats,
                                       const float *__restrict__ ppr, int64_t n_pix, float scale1,
                                       float scale2, float scale3,
                                       const float *__restrict__ weights) {
  int64_t o = blockIdx.x;
  int64_t p = blockIdx.y * (int64_t)blockDim.x + threadIdx.x;
  if (p >= n_pix) return;
  float h, k, l;
  rotate_inv(quats + 4 * o, ppr[p], ppr[n_pix + p], ppr[2 * n_pix + p], 1.0f, h, k, l);
  float w1[W], w2[W], w3[W];
  int i0 = axis_setup<W>(h, scale1, g.n1, g.off1, g.beta, g.inv_half_w, w1);
  int j0 = axis_setup<W>(k, scale2, g.n2, g.off2, g.beta, g.inv_half_w, w2);
  int k0 = axis_setup<W>(l, scale3, g.n3, g.off3, g.beta, g.inv_half_w, w3);
  float acc = 0.0f;
#pragma unroll
  for (int a = 0; a < W; ++a) {
    float acc_a = 0.0f;
#pragma unroll
    for (int b = 0; b < W; ++b) {
      const float *row = re_pad + ((size_t)(i0 + a) * g.p2 + (j0 + b)) * g.p3 + k0;
      float r = 0.0f;
#pragma unroll
      for (int c = 0; c < W; ++c) r = fmaf(w3[c], __ldg(row + c), r);
      acc_a = fmaf(w2[b], r, acc_a);
    }
    acc = fmaf(w1[a], acc_a, acc);
  }
  if (weights) acc *= weights[o * n_pix + p];
  if (acc == 0.0f) return;
#pragma unroll
  for (int c = 0; c < W; ++c) w3[c] *= acc;
#pragma unroll
  for (int a = 0; a < W; ++a) {
#pragma unroll
    for (int b = 0; b < W; ++b) {
      float wab = w1[a] * w2[b];
      float *row = acc_pad + ((size_t)(i0 + a) * g.p2 + (j0 + b)) * g.p3 + k0;
#pragma unroll
      for (int c = 0; c < W; ++c) atomicAdd(row + c, wab * w3[c]);
    }
  }
}

// ---------------------------------------------------------------------------
// bin-sorted points: 8^3-cell bins of the padded grid
// ---------------------------------------------------------------------------
constexpr int BIN = 8;
constexpr int BIN_CHUNK = 2048;      // default points per work item (big bins are split)
constexpr int BIN_CHUNK_MAX = 8192;  // largest item SPF_TUNE_SORT_ITEM may pick: the cell
                                     // sort stages an item in 48 KB of dynamic shared memory
constexpr size_t CELLSORT_SMEM = (size_t)BIN_CHUNK_MAX * (sizeof(int32_t) + sizeof(int16_t));

// The points of the sorted passes: orientation points (point o * n_pix + p
// is pixel p of the detector rotated by quaternion o, coordinates made in the
// kernel) or explicit coordinates x, y, z.
struct PointSrc {
  const float *quats, *ppr;
  int64_t n_pix;
  const float *x, *y, *z;
  __device__ __forceinline__ void coords(int64_t i, float &h, float &k, float &l) const {
    if (x) {
      h = x[i];
      k = y[i];
      l = z[i];
      return;
    }
    const int64_t o = i / n_pix, p = i % n_pix;
    rotate_inv(quats + 4 * o, ppr[p], ppr[n_pix + p], ppr[2 * n_pix + p], 1.0f, h, k, l);
  }
};

template <int W>
__device__ __forceinline__ int point_bin(const GridGeom &g, const int *nb, float h, float k, float l,
                                         float s1, float s2, float s3) {
  float w[W];
  int i0 = axis_setup<W>(h, s1, g.n1, g.off1, g.beta, g.inv_half_w, w);
  int j0 = axis_setup<W>(k, s2, g.n2, g.off2, g.beta, g.inv_half_w, w);
  int k0 = axis_setup<W>(l, s3, g.n3, g.off3, g.beta, g.inv_half_w, w);
  return ((i0 / BIN) * nb[1] + (j0 / BIN)) * nb[2] + (k0 / BIN);
}

struct BinDims {
  int nb[3];
};

template <int W>
__global__ void k_bin_count(GridGeom g, BinDims bd, PointSrc src, int64_t n, float s1, float s2,
                            float s3, int32_t *__restrict__ bin_of, int32_t *__restrict__ counts) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    float h, k, l;
    src.coords(i, h, k, l);
    int b = point_bin<W>(g, bd.nb, h, k, l, s1, s2, s3);
    bin_of[i] = b;
    atomicAdd(counts + b, 1);
  }
}

// exclusive prefix sum of n ints, one block of 1024 threads
__global__ void __launch_bounds__(1024) k_scan(const int32_t *__restrict__ in, int64_t n,
                                               int32_t *__restrict__ out) {
  __shared__ int32_t part[1024];
  const int t = threadIdx.x;
  const int64_t per = (n + 1023) / 1024;
  const int64_t lo = t * per, hi = lo + per < n ? lo + per : n;
  int32_t s = 0;
  for (int64_t i = lo; i < hi; ++i) s += in[i];
  part[t] = s;
  __syncthreads();
  for (int off = 1; off < 1024; off <<= 1) {
    int32_t v = t >= off ? part[t - off] : 0;
    __syncthreads();
    part[t] += v;
    __syncthreads();
  }
  int32_t run = t > 0 ? part[t - 1] : 0;
  for (int64_t i = lo; i < hi; ++i) {
    out[i] = run;
    run += in[i];
  }
}

__global__ void k_bin_scatter(const int32_t *__restrict__ bin_of, int64_t n,
                              const int32_t *__restrict__ offsets, int32_t *__restrict__ cursor,
                              int32_t *__restrict__ sorted) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    int b = bin_of[i];
    int pos = atomicAdd(cursor + b, 1);
    sorted[offsets[b] + pos] = (int32_t)i;
  }
}

// Padded first footprint index of a point along one axis: the index
// arithmetic of axis_setup without the weights (same explicitly rounded
// operations, so the cell agrees with the one the kernels use).
template <int W>
__device__ __forceinline__ int axis_cell(float x, float s, int n, int off) {
  float fn = (float)n;
  float t = __fmul_rn(x, s);
  t = __fsub_rn(t, __fmul_rn(fn, floorf(__fadd_rn(__fdiv_rn(t, fn), 0.5f))));
  return (int)ceilf(__fsub_rn(t, 0.5f * W)) + off;
}

// Orders the points of each work item by their first footprint cell within
// the bin (a counting sort over the 8^3 cells in shared memory), so that
// points sharing a footprint are consecutive.  The point set of every item is
// unchanged; only its order within the item is.
template <int W>
__global__ void __launch_bounds__(256)
    k_item_cellsort(GridGeom g, BinDims bd, const int4 *__restrict__ items,
                    int32_t *__restrict__ sorted, PointSrc src, float s1, float s2, float s3,
                    unsigned int *__restrict__ err) {
  constexpr int NC = BIN * BIN * BIN;
  extern __shared__ __align__(16) unsigned char cs_smem[];  // CELLSORT_SMEM bytes
  int32_t *idx = reinterpret_cast<int32_t *>(cs_smem);              // BIN_CHUNK_MAX
  int16_t *key = reinterpret_cast<int16_t *>(idx + BIN_CHUNK_MAX);  // BIN_CHUNK_MAX
  __shared__ int32_t cnt[NC];
  const int4 it = items[blockIdx.x];
  if (it.z > BIN_CHUNK_MAX) {  // an item larger than the staging arrays is never read
    if (threadIdx.x == 0 && err) atomicExch(err, (unsigned int)(-SPF_ERR_ARG));
    return;
  }
  const int b = it.x;
  const int bi = b / (bd.nb[1] * bd.nb[2]), bj = (b / bd.nb[2]) % bd.nb[1], bk = b % bd.nb[2];
  const int i0b = bi * BIN, j0b = bj * BIN, k0b = bk * BIN;
  for (int t = threadIdx.x; t < NC; t += blockDim.x) cnt[t] = 0;
  __syncthreads();
  for (int q = threadIdx.x; q < it.z; q += blockDim.x) {
    const int32_t pi = sorted[it.y + q];
    float h, k, l;
    src.coords(pi, h, k, l);
    const int ci = min(max(axis_cell<W>(h, s1, g.n1, g.off1) - i0b, 0), BIN - 1);
    const int cj = min(max(axis_cell<W>(k, s2, g.n2, g.off2) - j0b, 0), BIN - 1);
    const int ck = min(max(axis_cell<W>(l, s3, g.n3, g.off3) - k0b, 0), BIN - 1);
    const int kk = (ci * BIN + cj) * BIN + ck;
    idx[q] = pi;
    key[q] = (int16_t)kk;
    atomicAdd(&cnt[kk], 1);
  }
  __syncthreads();
  if (threadIdx.x < 32) {  // exclusive scan of the NC counters by one warp
    constexpr int PER = NC / 32;
    const int lane = threadIdx.x;
    int local = 0;
#pragma unroll
    for (int u = 0; u < PER; ++u) local += cnt[lane * PER + u];
    int incl = local;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int v = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += v;
    }
    int run = incl - local;
#pragma unroll
    for (int u = 0; u < PER; ++u) {
      const int c = cnt[lane * PER + u];
      cnt[lane * PER + u] = run;
      run += c;
    }
  }
  __syncthreads();
  for (int q = threadIdx.x; q < it.z; q += blockDim.x) {
    const int pos = atomicAdd(&cnt[key[q]], 1);
    sorted[it.y + pos] = idx[q];
  }
}

// Fused type 2 -> weight -> type 1 over bin-sorted points.  A CTA takes one
// work item (up to 2,048 points of one 8^3-cell bin, ordered by footprint
// cell), stages the bin's footprint box of the type-2 grid in shared memory,
// and accumulates the spread into a second box that is added to the type-1
// accumulator at the end.  A warp serves one point at a time.  Lane
// (g, c) = (lane / 8, lane % 8) owns the two footprint rows b = g and b = g + 4
// (second axis) at offset c along the fastest axis over the W planes of the
// slowest axis.  Consecutive points with the same footprint cell touch the
// same 2W cells per lane, so a lane keeps their box values and their pending
// spread in registers for the whole run: it reads the box, and adds to the
// spread box (shared atomics), only when the cell changes.  The separable
// weights are shuffled in once per point (w1 for the plane, w2 * w3 for the
// lane's two rows).  With a row stride of 24 floats the 32 lanes of either
// row set fall on 32 distinct banks.  Each point's coordinates are computed
// once by one lane and broadcast; lanes 0-7 / 8-15 / 16-23 evaluate the
// kernel on axes 1 / 2 / 3.
constexpr int SORTED_ROW_STRIDE = 24;
constexpr int SORTED_THREADS = 256;




template <int W, bool INTERP>
__global__ void __launch_bounds__(SORTED_THREADS, 4)
    k_interp_spread_sorted(const float *__restrict__ re_pad, float *__restrict__ acc_pad,
                           GridGeom g, BinDims bd, const int4 *__restrict__ items,
                           const int32_t *__restrict__ sorted, PointSrc src, float s1, float s2,
                           float s3, const float *__restrict__ weights,
                           const __grid_constant__ CUtensorMap tmap, int use_tma,
                           unsigned int *__restrict__ err) {
  static_assert(W <= 8, "eight lanes per footprint row, two rows per lane");
  constexpr int D = BIN + W - 1;
  constexpr int SR = SORTED_ROW_STRIDE;
  constexpr int SP = D * SR;
  static_assert(D <= SR, "row stride holds a footprint row");
  __shared__ __align__(128) float tbox[INTERP ? D * SP : 1];
  __shared__ __align__(8) uint64_t tbar;
  __shared__ float abox[D * SP];
  __shared__ float4 pt_tw[SORTED_THREADS];  // per warp: 32 prepared points
  __shared__ int pt_key[SORTED_THREADS];
  const int4 it = items[blockIdx.x];
  const int b = it.x;
  const int bi = b / (bd.nb[1] * bd.nb[2]), bj = (b / bd.nb[2]) % bd.nb[1], bk = b % bd.nb[2];
  const int i0b = bi * BIN, j0b = bj * BIN, k0b = bk * BIN;
  const int di = min(D, g.p1 - i0b), dj = min(D, g.p2 - j0b), dk = min(D, g.p3 - k0b);
  const BoxShape shape{i0b, j0b, k0b, di, dj, dk, SP, SR};
  // the bin's box is a regular tile of the padded grid: one TMA copy of
  // D x D x SR floats (the row stride's extra cells and cells past the grid
  // end come along or read as zero; no footprint reaches them), else a
  // cooperative load
  if (INTERP) {
    if (use_tma) {
      if (threadIdx.x == 0) {
        mbar_init(&tbar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        mbar_arrive_expect_tx(&tbar, (uint32_t)(D * SP * sizeof(float)));
        tma_load_3d(tbox, &tmap, &tbar, k0b, j0b, i0b);
      }
    } else {
      box_load(tbox, re_pad, g, shape);
    }
  }
  box_rows(shape, [&](int, int, int, int s) { abox[s] = 0.0f; });
  __syncthreads();
  if (INTERP && use_tma) {
    constexpr uint64_t TMA_TIMEOUT_NS = 1000000000ull;
    const bool late = !mbar_wait_for(&tbar, 0, TMA_TIMEOUT_NS);
    if (__syncthreads_or(late)) {
      // the copy gave no sign within the bound: report it, let it land, and
      // leave the item out
      if (threadIdx.x == 0 && err) atomicExch(err, (unsigned int)(-SPF_ERR_TIMEOUT));
      mbar_wait_for(&tbar, 0, TMA_TIMEOUT_NS);
      return;
    }
  }
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const int grp = lane >> 3;  // row set of the lane; kernel axis for the weights
  const int c = lane & 7;     // offset along the fastest axis
  const int r0 = grp, r1 = grp + 4;
  const bool ok0 = c < W && r0 < W, ok1 = c < W && r1 < W;
  const int lane_off0 = r0 * SR + c, lane_off1 = r1 * SR + c;
  const int warp = threadIdx.x >> 5;
  const int nwarps = SORTED_THREADS / 32;
  // the run: footprint cell (packed li, lj, lk) held in registers, its box
  // values and its spread not yet added
  int cur = -1, cur_base = 0;
  float2 pend[W];  // spread not yet added at the lane's two cells of plane a
  float2 xc[W];    // box values at the lane's two cells of plane a
  auto flush = [&]() {
#pragma unroll
    for (int a = 0; a < W; ++a) {
      if (ok0) atomicAdd(&abox[cur_base + lane_off0 + a * SP], pend[a].x);
      if (ok1) atomicAdd(&abox[cur_base + lane_off1 + a * SP], pend[a].y);
    }
  };
  // the lane's kernel axis: position of its first footprint index in the
  // packed cell key, and the offset from box to grid index
  const int ax = grp < 3 ? grp : 2;
  const int ax_shift = 10 - 5 * ax;
  const int ax_base = ax == 0 ? i0b - g.off1 : (ax == 1 ? j0b - g.off2 : k0b - g.off3);
  const float beta_log2e = g.beta * 1.4426950408889634f;
  const float fn1 = (float)g.n1, fn2 = (float)g.n2, fn3 = (float)g.n3;
  float4 *my_tw = pt_tw + warp * 32;
  int *my_key = pt_key + warp * 32;
  for (int q0 = warp * 32; q0 < it.z; q0 += nwarps * 32) {
    const int cnt = min(32, it.z - q0);
    // lane L prepares point q0 + L (same arithmetic as axis_setup / the bin sort)
    // into the warp's slots: (t1, t2, t3, weight) and the packed first cell
    // in the box, or -1 for a point outside the box
    if (lane < cnt) {
      const int32_t pi = sorted[it.y + q0 + lane];
      const float pw = weights ? weights[pi] : 1.0f;
      float h, k, l;
      src.coords(pi, h, k, l);
      float t1 = __fmul_rn(h, s1), t2 = __fmul_rn(k, s2), t3 = __fmul_rn(l, s3);
      t1 = __fsub_rn(t1, __fmul_rn(fn1, floorf(__fadd_rn(__fdiv_rn(t1, fn1), 0.5f))));
      t2 = __fsub_rn(t2, __fmul_rn(fn2, floorf(__fadd_rn(__fdiv_rn(t2, fn2), 0.5f))));
      t3 = __fsub_rn(t3, __fmul_rn(fn3, floorf(__fadd_rn(__fdiv_rn(t3, fn3), 0.5f))));
      const int li = (int)ceilf(__fsub_rn(t1, 0.5f * W)) + g.off1 - i0b;
      const int lj = (int)ceilf(__fsub_rn(t2, 0.5f * W)) + g.off2 - j0b;
      const int lk = (int)ceilf(__fsub_rn(t3, 0.5f * W)) + g.off3 - k0b;
      const bool inside =
          li >= 0 && lj >= 0 && lk >= 0 && li + W <= di && lj + W <= dj && lk + W <= dk;
      if (!inside && err)  // cannot happen for a correctly binned point; never read outside
        atomicExch(err, (unsigned int)(-SPF_ERR_CUDA));
      my_tw[lane] = make_float4(t1, t2, t3, pw);
      my_key[lane] = inside ? (li << 10) | (lj << 5) | lk : -1;  // li, lj, lk < 32
    }
    __syncwarp();
    const float *my_twf = reinterpret_cast<const float *>(my_tw);
    for (int j = 0; j < cnt; ++j) {
      const int key = my_key[j];
      if (key < 0) continue;
      // first footprint index along the lane's kernel axis, as a float (exact)
      const int la = ((key >> ax_shift) & 31) + ax_base;
      const float tt = my_twf[4 * j + ax];
      const float kw = (c < W && grp < 3)
                           ? es_eval_approx(((float)la + (float)c - tt) * g.inv_half_w, beta_log2e)
                           : 0.0f;
      const float w3c = __shfl_sync(FULL, kw, 16 + c);
      const float u0 = __shfl_sync(FULL, kw, 8 + r0) * w3c;
      const float u1 = __shfl_sync(FULL, kw, 8 + (r1 & 7)) * w3c;
      float w1[W];
#pragma unroll
      for (int a = 0; a < W; ++a) w1[a] = __shfl_sync(FULL, kw, a);
      if (key != cur) {  // warp-uniform
        if (cur >= 0) flush();
        cur = key;
        cur_base = (key >> 10) * SP + ((key >> 5) & 31) * SR + (key & 31);
#pragma unroll
        for (int a = 0; a < W; ++a) {
          pend[a] = make_float2(0.0f, 0.0f);
          if (INTERP)
            xc[a] = make_float2(ok0 ? tbox[cur_base + lane_off0 + a * SP] : 0.0f,
                                ok1 ? tbox[cur_base + lane_off1 + a * SP] : 0.0f);
        }
      }
      float v = my_twf[4 * j + 3];  // the point's weight (1 without weights)
      if (INTERP) {
        // interpolate: plane a, the lane's two rows (one packed FMA per plane)
        float2 sx = make_float2(0.0f, 0.0f);
#pragma unroll
        for (int a = 0; a < W; ++a) sx = ffma2(make_float2(w1[a], w1[a]), xc[a], sx);
        float part = fmaf(u1, sx.y, u0 * sx.x);
#pragma unroll
        for (int m = 16; m >= 1; m >>= 1) part += __shfl_xor_sync(FULL, part, m);
        v *= part;
      }
      const float2 vv = make_float2(u0 * v, u1 * v);
#pragma unroll
      for (int a = 0; a < W; ++a) pend[a] = ffma2(make_float2(w1[a], w1[a]), vv, pend[a]);
    }
    __syncwarp();  // the slots are rewritten by the next chunk
  }
  if (cur >= 0) flush();
  __syncthreads();
  box_flush(abox, acc_pad, g, shape);
}

// fine[l] = sum of acc_pad[i] over padded i == l + off (mod n)  (Im = 0).
__global__ void k_t1_fold(const float *__restrict__ acc_pad, GridGeom g,
                          float2 *__restrict__ fine) {
  int64_t total = (int64_t)g.n1 * g.n2 * g.n3;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    int c = (int)(idx % g.n3);
    int b = (int)((idx / g.n3) % g.n2);
    int a = (int)(idx / ((int64_t)g.n2 * g.n3));
    int ia[2], ib[2], ic[2];
    int na = 0, nb = 0, nc = 0;
    int i0 = (a + g.off1) % g.n1;
    ia[na++] = i0;
    if (i0 + g.n1 < g.p1) ia[na++] = i0 + g.n1;
    int j0 = (b + g.off2) % g.n2;
    ib[nb++] = j0;
    if (j0 + g.n2 < g.p2) ib[nb++] = j0 + g.n2;
    int k0 = (c + g.off3) % g.n3;
    ic[nc++] = k0;
    if (k0 + g.n3 < g.p3) ic[nc++] = k0 + g.n3;
    float s = 0.0f;
    for (int u = 0; u < na; ++u)
      for (int v = 0; v < nb; ++v)
        for (int q = 0; q < nc; ++q)
          s += acc_pad[((int64_t)ia[u] * g.p2 + ib[v]) * g.p3 + ic[q]];
    fine[idx] = make_float2(s, 0.0f);
  }
}

// modes[k] = fine[k mod n] / (p1 p2 p3)
__global__ void k_t1_extract(const float2 *__restrict__ fine, int m1, int m2, int m3, int n1,
                             int n2, int n3, const float *__restrict__ ip1,
                             const float *__restrict__ ip2, const float *__restrict__ ip3,
                             float *__restrict__ out_re, float *__restrict__ out_im) {
  int64_t total = (int64_t)m1 * m2 * m3;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    int c = (int)(idx % m3);
    int b = (int)((idx / m3) % m2);
    int a = (int)(idx / ((int64_t)m2 * m3));
    int fa = ((a - m1 / 2) % n1 + n1) % n1;
    int fb = ((b - m2 / 2) % n2 + n2) % n2;
    int fc = ((c - m3 / 2) % n3 + n3) % n3;
    float2 v = fine[((int64_t)fa * n2 + fb) * n3 + fc];
    float s = ip1[a] * ip2[b] * ip3[c];
    out_re[idx] = v.x * s;
    if (out_im) out_im[idx] = v.y * s;
  }
}

// ---------------------------------------------------------------------------
// dispatch on the kernel width
// ---------------------------------------------------------------------------

#define SPF_W_DISPATCH(w, KERNEL_CALL)              \
  switch (w) {                                      \
    case 3: { constexpr int W = 3; KERNEL_CALL; break; } \
    case 4: { constexpr int W = 4; KERNEL_CALL; break; } \
    case 5: { constexpr int W = 5; KERNEL_CALL; break; } \
    case 6: { constexpr int W = 6; KERNEL_CALL; break; } \
    case 7: { constexpr int W = 7; KERNEL_CALL; break; } \
    case 8: { constexpr int W = 8; KERNEL_CALL; break; } \
    default: set_error("unsupported kernel width %d", w); return SPF_ERR_UNSUPPORTED; \
  }

static int check_plan(spf_nufft_plan P, const char *what) {
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

static int fft_exec(spf_nufft_plan P, int isign, cudaStream_t s, const char *what) {
  if (cufftSetStream(P->fft, s) != CUFFT_SUCCESS) {
    set_error("%s: cufftSetStream failed", what);
    return SPF_ERR_CUDA;
  }
  cufftResult r = cufftExecC2C(P->fft, reinterpret_cast<cufftComplex *>(P->fine),
                               reinterpret_cast<cufftComplex *>(P->fine),
                               isign < 0 ? CUFFT_FORWARD : CUFFT_INVERSE);
  if (r != CUFFT_SUCCESS) {
    set_error("%s: cufftExecC2C failed (%d)", what, (int)r);
    return SPF_ERR_CUDA;
  }
  count_launch();
  return SPF_OK;
}

}  // namespace spf

using namespace spf;

extern "C" {

int spf_nufft_plan_create(int m1, int m2, int m3, double eps, double upsampfac,
                          spf_nufft_plan *out) {
  SPF_REQUIRE(out != nullptr, "spf_nufft_plan_create: out is NULL");
  *out = nullptr;
  SPF_REQUIRE(m1 > 0 && m2 > 0 && m3 > 0 && m1 <= 4096 && m2 <= 4096 && m3 <= 4096,
              "spf_nufft_plan_create: bad mode counts (%d, %d, %d)", m1, m2, m3);
  SPF_REQUIRE(eps > 0 && eps < 1, "spf_nufft_plan_create: eps must be in (0, 1)");
  double sigma = upsampfac <= 0 ? 2.0 : upsampfac;
  SPF_REQUIRE(sigma >= 1.25 && sigma <= 4.0, "spf_nufft_plan_create: upsampfac out of range");
  auto *P = new spf_nufft_plan_s();
  cudaGetDevice(&P->dev);
  P->m[0] = m1; P->m[1] = m2; P->m[2] = m3;
  P->eps = eps;
  P->sigma = sigma;
  P->w = es_width(eps, sigma);
  P->beta = es_beta(P->w, sigma);
  P->pad = (P->w + 1) / 2 + 1;
  for (int d = 0; d < 3; ++d) {
    int md = P->m[d];
    int want = (int)ceil(sigma * md);
    if (want < 2 * P->w) want = 2 * P->w;
    P->n[d] = next_smooth_even(want);
    P->np[d] = P->n[d] + 2 * P->pad;
  }
  // rows of the padded grid start on 16-byte boundaries (the slicing box is
  // filled with 16-byte loads); the extra cells are never inside a footprint
  P->np[2] = (P->np[2] + 3) & ~3;
  int st = SPF_OK;
  size_t nfine = (size_t)P->n[0] * P->n[1] * P->n[2];
  size_t npad = (size_t)P->np[0] * P->np[1] * P->np[2];
  for (int d = 0; d < 3 && st == SPF_OK; ++d) {
    auto v = inverse_kernel_ft(P->m[d], P->n[d], P->w, P->beta);
    st = check_cuda(cudaMalloc(&P->inv_p[d], v.size() * sizeof(float)), "plan_create");
    if (st == SPF_OK)
      st = check_cuda(cudaMemcpy(P->inv_p[d], v.data(), v.size() * sizeof(float),
                                 cudaMemcpyHostToDevice), "plan_create");
  }
  if (st == SPF_OK) st = check_cuda(cudaMalloc(&P->fine, nfine * sizeof(float2)), "plan_create");
  if (st == SPF_OK) st = check_cuda(cudaMalloc(&P->re_pad, npad * sizeof(float)), "plan_create");
  if (st == SPF_OK) st = check_cuda(cudaMalloc(&P->acc_pad, npad * sizeof(float)), "plan_create");
  if (st == SPF_OK) {
    cufftResult r = cufftPlan3d(&P->fft, P->n[0], P->n[1], P->n[2], CUFFT_C2C);
    if (r != CUFFT_SUCCESS) {
      set_error("plan_create: cufftPlan3d(%d,%d,%d) failed (%d)", P->n[0], P->n[1], P->n[2], (int)r);
      st = r == CUFFT_ALLOC_FAILED ? SPF_ERR_OOM : SPF_ERR_CUDA;
    } else {
      P->fft_ok = true;
    }
  }
  if (st != SPF_OK) {
    spf_nufft_plan_destroy(P);
    return st;
  }
  *out = P;
  return SPF_OK;
}

int spf_nufft_plan_destroy(spf_nufft_plan P) {
  if (!P) return SPF_OK;
  int prev = -1;
  cudaGetDevice(&prev);
  if (prev != P->dev) cudaSetDevice(P->dev);
  for (int d = 0; d < 3; ++d) cudaFree(P->inv_p[d]);
  cudaFree(P->fine);
  cudaFree(P->re_pad);
  cudaFree(P->im_pad);
  cudaFree(P->acc_pad);
  cudaFree(P->sorted);
  cudaFree(P->items);
  if (P->fft_ok) cufftDestroy(P->fft);
  if (prev != P->dev && prev >= 0) cudaSetDevice(prev);
  delete P;
  return SPF_OK;
}

int spf_nufft_plan_info(spf_nufft_plan P, int *n_fine, int *width, double *beta, int *n_padded) {
  SPF_REQUIRE(P != nullptr, "spf_nufft_plan_info: plan is NULL");
  for (int d = 0; d < 3; ++d) {
    if (n_fine) n_fine[d] = P->n[d];
    if (n_padded) n_padded[d] = P->np[d];
  }
  if (width) *width = P->w;
  if (beta) *beta = P->beta;
  return SPF_OK;
}

int spf_nufft_t2_set_modes(spf_nufft_plan P, const float *d_modes, const float *d_support,
                           int isign, int want_imag, void *stream) {
  SPF_TRY(check_plan(P, "spf_nufft_t2_set_modes"));
  SPF_REQUIRE(d_modes != nullptr, "spf_nufft_t2_set_modes: modes is NULL");
  SPF_REQUIRE(isign == 1 || isign == -1, "spf_nufft_t2_set_modes: isign must be +-1");
  cudaStream_t s = as_stream(stream);
  size_t nfine = (size_t)P->n[0] * P->n[1] * P->n[2];
  size_t npad = (size_t)P->np[0] * P->np[1] * P->np[2];
  if (want_imag && !P->im_pad)
    SPF_TRY(check_cuda(cudaMalloc(&P->im_pad, npad * sizeof(float)), "spf_nufft_t2_set_modes"));
  SPF_TRY(check_cuda(cudaMemsetAsync(P->fine, 0, nfine * sizeof(float2), s), "t2_set_modes"));
  int64_t nm = (int64_t)P->m[0] * P->m[1] * P->m[2];
  k_t2_scatter_modes<<<grid_for(nm, 256, 8 * 1024), 256, 0, s>>>(
      d_modes, d_support, P->m[0], P->m[1], P->m[2], P->n[0], P->n[1], P->n[2], P->inv_p[0],
      P->inv_p[1], P->inv_p[2], P->fine);
  SPF_TRY(check_launch("k_t2_scatter_modes"));
  SPF_TRY(fft_exec(P, isign, s, "spf_nufft_t2_set_modes"));
  GridGeom g = geom_of(P);
  k_t2_fill_padded<<<grid_for((int64_t)npad, 256, 16 * 1024), 256, 0, s>>>(
      P->fine, g, 1.0f, P->re_pad, want_imag ? P->im_pad : nullptr);
  return check_launch("k_t2_fill_padded");
}

int spf_nufft_t2_interp(spf_nufft_plan P, const float *d_x, const float *d_y, const float *d_z,
                        int64_t npts, float *d_out_re, float *d_out_im, void *stream) {
  SPF_TRY(check_plan(P, "spf_nufft_t2_interp"));
  SPF_REQUIRE(npts >= 0, "spf_nufft_t2_interp: npts < 0");
  if (npts == 0) return SPF_OK;
  SPF_REQUIRE(d_x && d_y && d_z && d_out_re, "spf_nufft_t2_interp: NULL pointer");
  SPF_REQUIRE(!d_out_im || P->im_pad,
              "spf_nufft_t2_interp: imaginary output needs set_modes(want_imag=1)");
  cudaStream_t s = as_stream(stream);
  GridGeom g = geom_of(P);
  int grid = grid_for(npts, 256, (int64_t)sm_count() * 16);
  SPF_W_DISPATCH(P->w, (k_t2_interp<W><<<grid, 256, 0, s>>>(P->re_pad, P->im_pad, g, d_x, d_y,
                                                               d_z, npts, d_out_re, d_out_im)));
  return check_launch("k_t2_interp");
}

int spf_slice_t2(spf_nufft_plan P, const float *d_quats, int64_t n_orient, const float *d_ppr,
                 int64_t n_pix, double scale, float *d_out, void *d_out_bf16, void *stream) {
  SPF_TRY(check_plan(P, "spf_slice_t2"));
  SPF_REQUIRE(n_orient >= 0 && n_pix >= 0, "spf_slice_t2: negative size");
  if (n_orient == 0 || n_pix == 0) return SPF_OK;
  SPF_REQUIRE(d_quats && d_ppr && d_out, "spf_slice_t2: NULL pointer");
  SPF_REQUIRE(n_orient < (1LL << 31) && n_pix <= 65535LL * 256, "spf_slice_t2: size too large");
  cudaStream_t s = as_stream(stream);
  GridGeom g = geom_of(P);
  float s1 = (float)(scale * P->n[0] / (2.0 * M_PI));
  float s2 = (float)(scale * P->n[1] / (2.0 * M_PI));
  float s3 = (float)(scale * P->n[2] / (2.0 * M_PI));
  dim3 grid((unsigned)n_orient, (unsigned)((n_pix + 255) / 256));
  auto *bf = reinterpret_cast<__nv_bfloat16 *>(d_out_bf16);
  SPF_W_DISPATCH(P->w, (k_slice_t2<W><<<grid, 256, 0, s>>>(P->re_pad, g, d_quats, d_ppr, n_pix,
                                                              s1, s2, s3, d_out, bf)));
  return check_launch("k_slice_t2");
}

int spf_slice_t2_det(spf_nufft_plan P, const float *d_quats, int64_t n_orient, const float *d_ppr,
                     int n_panels, int nx, int ny, double scale, float *d_out, void *d_out_bf16,
                     void *stream) {
  SPF_TRY(check_plan(P, "spf_slice_t2_det"));
  SPF_REQUIRE(n_orient >= 0 && n_panels >= 0 && nx >= 0 && ny >= 0,
              "spf_slice_t2_det: negative size");
  if (n_orient == 0 || n_panels == 0 || nx == 0 || ny == 0) return SPF_OK;
  SPF_REQUIRE(d_quats && d_ppr && d_out, "spf_slice_t2_det: NULL pointer");
  const int code = (int)tune_get(SPF_TUNE_SLICE_SHAPE, 0);
  const PatchShape ps = slice_shape(code >= 0 && code < N_SLICE_SHAPES ? code : 0);
  int64_t patches = (int64_t)n_panels * ((nx + ps.px - 1) / ps.px) * ((ny + ps.py - 1) / ps.py);
  SPF_REQUIRE(n_orient < (1LL << 31) && patches <= 65535, "spf_slice_t2_det: size too large");
  cudaStream_t s = as_stream(stream);
  GridGeom g = geom_of(P);
  float s1 = (float)(scale * P->n[0] / (2.0 * M_PI));
  float s2 = (float)(scale * P->n[1] / (2.0 * M_PI));
  float s3 = (float)(scale * P->n[2] / (2.0 * M_PI));
  dim3 grid((unsigned)n_orient, (unsigned)patches);
  auto *bf = reinterpret_cast<__nv_bfloat16 *>(d_out_bf16);
  if (ps.search) {
    SPF_W_DISPATCH(P->w, (k_slice_t2_det<W, true><<<grid, 256, 0, s>>>(
                             P->re_pad, g, d_quats, d_ppr, n_panels, nx, ny, s1, s2, s3, d_out,
                             bf, ps)));
  } else {
    SPF_W_DISPATCH(P->w, (k_slice_t2_det<W, false><<<grid, 256, 0, s>>>(
                             P->re_pad, g, d_quats, d_ppr, n_panels, nx, ny, s1, s2, s3, d_out,
                             bf, ps)));
  }
  return check_launch("k_slice_t2_det");
}

int spf_nufft_t1_zero(spf_nufft_plan P, void *stream) {
  SPF_TRY(check_plan(P, "spf_nufft_t1_zero"));
  size_t npad = (size_t)P->np[0] * P->np[1] * P->np[2];
  return check_cuda(cudaMemsetAsync(P->acc_pad, 0, npad * sizeof(float), as_stream(stream)),
                    "spf_nufft_t1_zero");
}

int spf_nufft_t1_spread(spf_nufft_plan P, const float *d_x, const float *d_y, const float *d_z,
                        const float *d_c, int64_t npts, void *stream) {
  SPF_TRY(check_plan(P, "spf_nufft_t1_spread"));
  SPF_REQUIRE(npts >= 0, "spf_nufft_t1_spread: npts < 0");
  if (npts == 0) return SPF_OK;
  SPF_REQUIRE(d_x && d_y && d_z && d_c, "spf_nufft_t1_spread: NULL pointer");
  cudaStream_t s = as_stream(stream);
  GridGeom g = geom_of(P);
  int grid = grid_for(npts, 256, (int64_t)sm_count() * 16);
  SPF_W_DISPATCH(P->w, (k_t1_spread<W><<<grid, 256, 0, s>>>(P->acc_pad, g, d_x, d_y, d_z, d_c,
                                                               npts)));
  return check_launch("k_t1_spread");
}

int spf_nufft_t1_spread_orient(spf_nufft_plan P, const float *d_quats, int64_t n_orient,
                               const float *d_ppr, int64_t n_pix, double scale, const float *d_c,
                               void *stream) {
  SPF_TRY(check_plan(P, "spf_nufft_t1_spread_orient"));
  SPF_REQUIRE(n_orient >= 0 && n_pix >= 0, "spf_nufft_t1_spread_orient: negative size");
  if (n_orient == 0 || n_pix == 0) return SPF_OK;
  SPF_REQUIRE(d_quats && d_ppr && d_c, "spf_nufft_t1_spread_orient: NULL pointer");
  SPF_REQUIRE(n_orient < (1LL << 31) && n_pix <= 65535LL * 256,
              "spf_nufft_t1_spread_orient: size too large");
  cudaStream_t s = as_stream(stream);
  GridGeom g = geom_of(P);
  float s1 = (float)(scale * P->n[0] / (2.0 * M_PI));
  float s2 = (float)(scale * P->n[1] / (2.0 * M_PI));
  float s3 = (float)(scale * P->n[2] / (2.0 * M_PI));
  dim3 grid((unsigned)n_orient, (unsigned)((n_pix + 255) / 256));
  SPF_W_DISPATCH(P->w, (k_t1_spread_orient<W><<<grid, 256, 0, s>>>(P->acc_pad, g, d_quats, d_ppr,
                                                                      n_pix, s1, s2, s3, d_c)));
  return check_launch("k_t1_spread_orient");
}

int spf_nufft_interp_spread_orient(spf_nufft_plan P, const float *d_quats, int64_t n_orient,
                                   const float *d_ppr, int64_t n_pix, double scale,
                                   const float *d_weights, void *stream) {
  SPF_TRY(check_plan(P, "spf_nufft_interp_spread_orient"));
  SPF_REQUIRE(n_orient >= 0 && n_pix >= 0, "spf_nufft_interp_spread_orient: negative size");
  if (n_orient == 0 || n_pix == 0) return SPF_OK;
  SPF_REQUIRE(d_quats && d_ppr, "spf_nufft_interp_spread_orient: NULL pointer");
  SPF_REQUIRE(n_orient < (1LL << 31) && n_pix <= 65535LL * 256,
              "spf_nufft_interp_spread_orient: size too large");
  cudaStream_t s = as_stream(stream);
  GridGeom g = geom_of(P);
  float s1 = (float)(scale * P->n[0] / (2.0 * M_PI));
  float s2 = (float)(scale * P->n[1] / (2.0 * M_PI));
  float s3 = (float)(scale * P->n[2] / (2.0 * M_PI));
  dim3 grid((unsigned)n_orient, (unsigned)((n_pix + 255) / 256));
  SPF_W_DISPATCH(P->w, (k_interp_spread_orient<W><<<grid, 256, 0, s>>>(
                           P->re_pad, P->acc_pad, g, d_quats, d_ppr, n_pix, s1, s2, s3,
                           d_weights)));
  return check_launch("k_interp_spread_orient");
}

static int spread_det(spf_nufft_plan P, bool interp, const float *d_quats, int64_t n_orient,
                      const float *d_ppr, int n_panels, int nx, int ny, double scale,
                      const float *d_vals, void *stream, const char *name) {
  SPF_TRY(check_plan(P, name));
  SPF_REQUIRE(n_orient >= 0 && n_panels >= 0 && nx >= 0 && ny >= 0, "%s: negative size", name);
  if (n_orient == 0 || n_panels == 0 || nx == 0 || ny == 0) return SPF_OK;
  SPF_REQUIRE(d_quats && d_ppr && (interp || d_vals), "%s: NULL pointer", name);
  int64_t patches = (int64_t)n_panels * ((nx + SLICE_PATCH - 1) / SLICE_PATCH) *
                    ((ny + SLICE_PATCH - 1) / SLICE_PATCH);
  SPF_REQUIRE(n_orient < (1LL << 31) && patches <= 65535, "%s: size too large", name);
  cudaStream_t s = as_stream(stream);
  GridGeom g = geom_of(P);
  float s1 = (float)(scale * P->n[0] / (2.0 * M_PI));
  float s2 = (float)(scale * P->n[1] / (2.0 * M_PI));
  float s3 = (float)(scale * P->n[2] / (2.0 * M_PI));
  dim3 grid((unsigned)n_orient, (unsigned)patches);
  if (interp) {
    SPF_W_DISPATCH(P->w, (k_spread_det<W, true><<<grid, 256, 0, s>>>(
                             P->re_pad, P->acc_pad, g, d_quats, d_ppr, n_panels, nx, ny, s1, s2, s3,
                             d_vals)));
  } else {
    SPF_W_DISPATCH(P->w, (k_spread_det<W, false><<<grid, 256, 0, s>>>(
                             P->re_pad, P->acc_pad, g, d_quats, d_ppr, n_panels, nx, ny, s1, s2, s3,
                             d_vals)));
  }
  return check_launch(name);
}

int spf_nufft_t1_spread_det(spf_nufft_plan P, const float *d_quats, int64_t n_orient,
                            const float *d_ppr, int n_panels, int nx, int ny, double scale,
                            const float *d_c, void *stream) {
  return spread_det(P, false, d_quats, n_orient, d_ppr, n_panels, nx, ny, scale, d_c, stream,
                    "spf_nufft_t1_spread_det");
}

int spf_nufft_interp_spread_det(spf_nufft_plan P, const float *d_quats, int64_t n_orient,
                                const float *d_ppr, int n_panels, int nx, int ny, double scale,
                                const float *d_weights, void *stream) {
  return spread_det(P, true, d_quats, n_orient, d_ppr, n_panels, nx, ny, scale, d_weights, stream,
                    "spf_nufft_interp_spread_det");
}

// bin sort of n points (orientation or explicit) for the sorted passes
static int sort_points(spf_nufft_plan P, PointSrc src, int64_t n, double scale, void *stream) {
  SPF_REQUIRE(n < (1LL << 31), "spf_nufft_sort: more than 2^31 points");
  cudaStream_t s = as_stream(stream);
  GridGeom g = geom_of(P);
  BinDims bd;
  for (int d = 0; d < 3; ++d) bd.nb[d] = P->nb[d] = (P->np[d] + BIN - 1) / BIN;
  const int64_t n_bins = (int64_t)bd.nb[0] * bd.nb[1] * bd.nb[2];
  float s1 = (float)(scale * P->n[0] / (2.0 * M_PI));
  float s2 = (float)(scale * P->n[1] / (2.0 * M_PI));
  float s3 = (float)(scale * P->n[2] / (2.0 * M_PI));
  // temporaries
  int32_t *bin_of = nullptr, *counts = nullptr, *offsets = nullptr, *cursor = nullptr;
  int st = check_cuda(cudaMalloc(&bin_of, (n > 0 ? n : 1) * sizeof(int32_t)), "sort_orient");
  if (st == SPF_OK) st = check_cuda(cudaMalloc(&counts, n_bins * 3 * sizeof(int32_t)), "sort_orient");
  if (st == SPF_OK && n > P->sorted_cap) {
    cudaFree(P->sorted);
    P->sorted = nullptr;
    st = check_cuda(cudaMalloc(&P->sorted, n * sizeof(int32_t)), "sort_orient");
    if (st == SPF_OK) P->sorted_cap = n;
  }
  if (st == SPF_OK) {
    offsets = counts + n_bins;
    cursor = counts + 2 * n_bins;
    cudaMemsetAsync(counts, 0, n_bins * 3 * sizeof(int32_t), s);
    int grid = grid_for(n, 256, (int64_t)sm_count() * 16);
    SPF_W_DISPATCH(P->w, (k_bin_count<W><<<grid, 256, 0, s>>>(g, bd, src, n, s1, s2, s3, bin_of,
                                                                 counts)));
    st = check_launch("k_bin_count");
  }
  if (st == SPF_OK) {
    k_scan<<<1, 1024, 0, s>>>(counts, n_bins, offsets);
    st = check_launch("k_scan");
  }
  if (st == SPF_OK) {
    k_bin_scatter<<<grid_for(n, 256, (int64_t)sm_count() * 16), 256, 0, s>>>(bin_of, n, offsets,
                                                                            cursor, P->sorted);
    st = check_launch("k_bin_scatter");
  }
  // work items: every non-empty bin, big bins split into BIN_CHUNK points
  std::vector<int32_t> h_counts, h_offsets;
  if (st == SPF_OK) {
    h_counts.resize(n_bins);
    h_offsets.resize(n_bins);
    st = check_cuda(cudaMemcpyAsync(h_counts.data(), counts, n_bins * sizeof(int32_t),
                                    cudaMemcpyDeviceToHost, s), "sort_orient");
    if (st == SPF_OK)
      st = check_cuda(cudaMemcpyAsync(h_offsets.data(), offsets, n_bins * sizeof(int32_t),
                                      cudaMemcpyDeviceToHost, s), "sort_orient");
    if (st == SPF_OK) st = check_cuda(cudaStreamSynchronize(s), "sort_orient");
  }
  cudaFree(bin_of);
  cudaFree(counts);
  if (st != SPF_OK) return st;
  std::vector<int4> h_items;
  int32_t chunk = (int32_t)tune_get(SPF_TUNE_SORT_ITEM, BIN_CHUNK);
  if (chunk < 1 || chunk > BIN_CHUNK_MAX) chunk = BIN_CHUNK;  // the cell sort stages <= the max
  for (int64_t b = 0; b < n_bins; ++b)
    for (int32_t c = 0; c < h_counts[b]; c += chunk)
      h_items.push_back(make_int4((int)b, h_offsets[b] + c,
                                  h_counts[b] - c < chunk ? h_counts[b] - c : chunk, 0));
  if ((int64_t)h_items.size() > P->items_cap) {
    cudaFree(P->items);
    P->items = nullptr;
    SPF_TRY(check_cuda(cudaMalloc(&P->items, (h_items.size() + 1) * sizeof(int4)), "sort_orient"));
    P->items_cap = (int64_t)h_items.size();
  }
  if (!h_items.empty())
    SPF_TRY(check_cuda(cudaMemcpy(P->items, h_items.data(), h_items.size() * sizeof(int4),
                                  cudaMemcpyHostToDevice), "sort_orient"));
  P->n_items = (int64_t)h_items.size();
  P->n_sorted = n;
  if (P->n_items > 0) {  // points sharing a footprint cell become consecutive
    SPF_W_DISPATCH(P->w, (cudaFuncSetAttribute(k_item_cellsort<W>,
                                               cudaFuncAttributeMaxDynamicSharedMemorySize,
                                               (int)CELLSORT_SMEM),
                          k_item_cellsort<W><<<(unsigned)P->n_items, 256, CELLSORT_SMEM, s>>>(
                             g, bd, P->items, P->sorted, src, s1, s2, s3,
                             device_error_word())));
    SPF_TRY(check_launch("k_item_cellsort"));
  }
  P->s_quats = src.quats;
  P->s_ppr = src.ppr;
  P->s_n_pix = src.n_pix;
  P->s_x = src.x;
  P->s_y = src.y;
  P->s_z = src.z;
  P->s_scale = scale;
  return SPF_OK;
}

int spf_nufft_sort_orient(spf_nufft_plan P, const float *d_quats, int64_t n_orient,
                          const float *d_ppr, int64_t n_pix, double scale, void *stream) {
  SPF_TRY(check_plan(P, "spf_nufft_sort_orient"));
  SPF_REQUIRE(n_orient >= 0 && n_pix >= 0, "spf_nufft_sort_orient: negative size");
  SPF_REQUIRE(d_quats && d_ppr, "spf_nufft_sort_orient: NULL pointer");
  SPF_REQUIRE(n_pix > 0 || n_orient == 0, "spf_nufft_sort_orient: n_pix = 0");
  SPF_TRY(sort_points(P, PointSrc{d_quats, d_ppr, n_pix > 0 ? n_pix : 1, nullptr, nullptr, nullptr},
                      n_orient * n_pix, scale, stream));
  P->s_n_orient = n_orient;
  return SPF_OK;
}

int spf_nufft_sort_points(spf_nufft_plan P, const float *d_x, const float *d_y,
                          const float *d_z, int64_t n, void *stream) {
  SPF_TRY(check_plan(P, "spf_nufft_sort_points"));
  SPF_REQUIRE(n >= 0, "spf_nufft_sort_points: negative size");
  SPF_REQUIRE(n == 0 || (d_x && d_y && d_z), "spf_nufft_sort_points: NULL pointer");
  SPF_TRY(sort_points(P, PointSrc{nullptr, nullptr, 1, d_x, d_y, d_z}, n, 1.0, stream));
  P->s_n_orient = 0;
  return SPF_OK;
}

static int sorted_pass(spf_nufft_plan P, const float *d_weights, bool interp, const char *what,
                       void *stream) {
  SPF_TRY(check_plan(P, what));
  SPF_REQUIRE(P->sorted != nullptr && P->n_sorted > 0 || P->n_items == 0,
              "%s: call spf_nufft_sort_orient first", what);
  if (P->n_items == 0) return SPF_OK;
  cudaStream_t s = as_stream(stream);
  GridGeom g = geom_of(P);
  BinDims bd;
  for (int d = 0; d < 3; ++d) bd.nb[d] = P->nb[d];
  float s1 = (float)(P->s_scale * P->n[0] / (2.0 * M_PI));
  float s2 = (float)(P->s_scale * P->n[1] / (2.0 * M_PI));
  float s3 = (float)(P->s_scale * P->n[2] / (2.0 * M_PI));
  SPF_REQUIRE(P->n_items < (1LL << 31), "%s: too many items", what);
  const PointSrc src{P->s_quats, P->s_ppr, P->s_n_pix, P->s_x, P->s_y, P->s_z};
  // TMA map of the padded grid for the bins' boxes (rows are 16-byte aligned)
  CUtensorMap tmap;
  memset(&tmap, 0, sizeof(tmap));
  int use_tma = 0;
  auto encode = tensor_map_encoder();
  if (interp && (g.p3 & 3) == 0 && encode) {
    const int D = BIN + P->w - 1;
    cuuint64_t dims[3] = {(cuuint64_t)g.p3, (cuuint64_t)g.p2, (cuuint64_t)g.p1};
    cuuint64_t strides[2] = {(cuuint64_t)g.p3 * sizeof(float),
                             (cuuint64_t)g.p3 * g.p2 * sizeof(float)};
    cuuint32_t box[3] = {(cuuint32_t)SORTED_ROW_STRIDE, (cuuint32_t)D, (cuuint32_t)D};
    cuuint32_t estr[3] = {1, 1, 1};
    use_tma = encode(&tmap, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, P->re_pad, dims, strides, box,
                     estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                     CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
  }
  if (interp) {
    SPF_W_DISPATCH(P->w, (k_interp_spread_sorted<W, true>
                          <<<(unsigned)P->n_items, SORTED_THREADS, 0, s>>>(
                              P->re_pad, P->acc_pad, g, bd, P->items, P->sorted, src, s1, s2,
                              s3, d_weights, tmap, use_tma, device_error_word())));
  } else {
    SPF_W_DISPATCH(P->w, (k_interp_spread_sorted<W, false>
                          <<<(unsigned)P->n_items, SORTED_THREADS, 0, s>>>(
                              P->re_pad, P->acc_pad, g, bd, P->items, P->sorted, src, s1, s2,
                              s3, d_weights, tmap, 0, device_error_word())));
  }
  return check_launch(what);
}

int spf_nufft_interp_spread_sorted(spf_nufft_plan P, const float *d_weights, void *stream) {
  return sorted_pass(P, d_weights, true, "spf_nufft_interp_spread_sorted", stream);
}

int spf_nufft_spread_sorted(spf_nufft_plan P, const float *d_values, void *stream) {
  return sorted_pass(P, d_values, false, "spf_nufft_spread_sorted", stream);
}

int spf_nufft_t1_finish(spf_nufft_plan P, int isign, float *d_out_re, float *d_out_im,
                        void *stream) {
  SPF_TRY(check_plan(P, "spf_nufft_t1_finish"));
  SPF_REQUIRE(isign == 1 || isign == -1, "spf_nufft_t1_finish: isign must be +-1");
  SPF_REQUIRE(d_out_re != nullptr, "spf_nufft_t1_finish: out_re is NULL");
  cudaStream_t s = as_stream(stream);
  GridGeom g = geom_of(P);
  int64_t nfine = (int64_t)P->n[0] * P->n[1] * P->n[2];
  k_t1_fold<<<grid_for(nfine, 256, 16 * 1024), 256, 0, s>>>(P->acc_pad, g, P->fine);
  SPF_TRY(check_launch("k_t1_fold"));
  SPF_TRY(fft_exec(P, isign, s, "spf_nufft_t1_finish"));
  int64_t nm = (int64_t)P->m[0] * P->m[1] * P->m[2];
  k_t1_extract<<<grid_for(nm, 256, 16 * 1024), 256, 0, s>>>(
      P->fine, P->m[0], P->m[1], P->m[2], P->n[0], P->n[1], P->n[2], P->inv_p[0], P->inv_p[1],
      P->inv_p[2], d_out_re, d_out_im);
  return check_launch("k_t1_extract");
}

int spf_spread_t1(spf_nufft_plan P, const float *d_x, const float *d_y, const float *d_z,
                  const float *d_c, int64_t npts, int isign, float *d_out_re, float *d_out_im,
                  void *stream) {
  SPF_TRY(spf_nufft_t1_zero(P, stream));
  SPF_TRY(spf_nufft_t1_spread(P, d_x, d_y, d_z, d_c, npts, stream));
  return spf_nufft_t1_finish(P, isign, d_out_re, d_out_im, stream);
}

int spf_fft_deconv(spf_nufft_plan P, int type, int isign, const float *d_modes_in,
                   const float *d_support, float *d_modes_out_re, float *d_modes_out_im,
                   void *stream) {
  if (type == 2) {
    SPF_REQUIRE(!d_modes_out_re && !d_modes_out_im,
                "spf_fft_deconv: type 2 keeps its result in the plan (outputs must be NULL)");
    return spf_nufft_t2_set_modes(P, d_modes_in, d_support, isign, 0, stream);
  }
  SPF_REQUIRE(type == 1, "spf_fft_deconv: type must be 1 or 2");
  SPF_REQUIRE(!d_modes_in && !d_support,
              "spf_fft_deconv: type 1 reads the plan's accumulator (inputs must be NULL)");
  return spf_nufft_t1_finish(P, isign, d_modes_out_re, d_modes_out_im, stream);
}

}  // extern "C"
