// Plain (SIMT) distance kernels: the drop-in for the reference's CUDA KNN
// module and the FP32 distance + argmin that SNM computes with cuBLAS + CUB.
//
// Both operands are row-major with the pixel axis contiguous ("K-major"):
// images [n_img][n_pix] and references [n_ref][n_pix].  A CTA computes a
// 128 x 128 tile of (image, reference) pairs with 256 threads, each thread an
// 8 x 8 register tile, K staged through shared memory in steps of 16 pixels
// with register double-buffering.  The tile order is grouped (8 image tiles
// per group) so that CTAs resident at the same time share image and
// reference rows in L2.
#include "common.cuh"

namespace spf {

constexpr int TB_M = 128;  // image rows per CTA
constexpr int TB_N = 128;  // reference rows per CTA
constexpr int TB_K = 16;
constexpr int TB_THREADS = 256;
constexpr int GROUP_M = 8;

enum class Mode { DIFF, DOT };

template <typename T>
struct TileLoader {
  // 128 rows x 16 k per tile = 2048 elements, 8 per thread as 2 x 4.
  T v[2][4];
  __device__ __forceinline__ void load(const T *__restrict__ base, int64_t n_rows, int64_t ld,
                                       int64_t K, int64_t row0, int64_t k0, bool vec) {
    int tid = threadIdx.x;
#pragma unroll
    for (int i = 0; i < 2; ++i) {
      int idx = tid + i * TB_THREADS;
      int r = idx >> 2;
      int kq = (idx & 3) * 4;
      int64_t row = row0 + r;
      int64_t k = k0 + kq;
      if (row < n_rows) {
        const T *p = base + row * ld + k;
        if constexpr (sizeof(T) == 4) {
          if (vec && k + 3 < K) {
            float4 f = __ldg(reinterpret_cast<const float4 *>(p));
            v[i][0] = f.x; v[i][1] = f.y; v[i][2] = f.z; v[i][3] = f.w;
            continue;
          }
        }
#pragma unroll
        for (int j = 0; j < 4; ++j) v[i][j] = (k + j < K) ? __ldg(p + j) : T(0);
      } else {
#pragma unroll
        for (int j = 0; j < 4; ++j) v[i][j] = T(0);
      }
    }
  }
  __device__ __forceinline__ void store(T (*s)[TB_M + 4]) {
    int tid = threadIdx.x;
#pragma unroll
    for (int i = 0; i < 2; ++i) {
      int idx = tid + i * TB_THREADS;
      int r = idx >> 2;
      int kq = (idx & 3) * 4;
#pragma unroll
      for (int j = 0; j < 4; ++j) s[kq + j][r] = v[i][j];
    }
  }
};

__device__ __forceinline__ void tile_coords(int64_t n_img_tiles, int64_t n_ref_tiles,
                                            int group_m, int64_t &mt, int64_t &nt) {
  int64_t bid = blockIdx.x;
  int64_t per_group = (int64_t)group_m * n_ref_tiles;
  int64_t group = bid / per_group;
  int64_t first_m = group * group_m;
  int64_t gm = n_img_tiles - first_m;
  if (gm > group_m) gm = group_m;
  int64_t in = bid % per_group;
  mt = first_m + in % gm;
  nt = in / gm;
}

// acc[i][j] accumulates for image row (ty*4 + i%4 + 64*(i/4)) and reference
// row (tx*4 + j%4 + 64*(j/4)) of the tile.
template <typename T, Mode MODE>
__device__ __forceinline__ void tile_mainloop(const T *__restrict__ A, int64_t n_a,
                                              const T *__restrict__ B, int64_t n_b, int64_t ld,
                                              int64_t K, int64_t a0, int64_t b0, T acc[8][8],
                                              T (*As)[TB_K][TB_M + 4],
                                              T (*Bs)[TB_K][TB_N + 4]) {
  const int tx = threadIdx.x & 15;
  const int ty = threadIdx.x >> 4;
  const bool vec = (sizeof(T) == 4) && (ld % 4 == 0) && aligned(A, 16) && aligned(B, 16);
#pragma unroll
  for (int i = 0; i < 8; ++i)
#pragma unroll
    for (int j = 0; j < 8; ++j) acc[i][j] = T(0);
  TileLoader<T> la, lb;
  int64_t ktiles = (K + TB_K - 1) / TB_K;
  if (ktiles == 0) return;
  la.load(A, n_a, ld, K, a0, 0, vec);
  lb.load(B, n_b, ld, K, b0, 0, vec);
  la.store(As[0]);
  lb.store(Bs[0]);
  __syncthreads();
  for (int64_t kt = 0; kt < ktiles; ++kt) {
    int cur = kt & 1;
    bool more = kt + 1 < ktiles;
    if (more) {
      la.load(A, n_a, ld, K, a0, (kt + 1) * TB_K, vec);
      lb.load(B, n_b, ld, K, b0, (kt + 1) * TB_K, vec);
    }
#pragma unroll
    for (int k = 0; k < TB_K; ++k) {
      T a[8], b[8];
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        a[i] = As[cur][k][ty * 4 + i];
        a[i + 4] = As[cur][k][64 + ty * 4 + i];
        b[i] = Bs[cur][k][tx * 4 + i];
        b[i + 4] = Bs[cur][k][64 + tx * 4 + i];
      }
      if constexpr (sizeof(T) == 4) {
        // two outputs per instruction (packed sub / fma, each lane the same
        // IEEE operation as below, so every output's chain is unchanged)
#pragma unroll
        for (int i = 0; i < 8; ++i)
#pragma unroll
          for (int j = 0; j < 8; j += 2) {
            const float2 ai = make_float2(a[i], a[i]), bj = make_float2(b[j], b[j + 1]);
            const float2 c = make_float2(acc[i][j], acc[i][j + 1]);
            float2 r;
            if constexpr (MODE == Mode::DIFF) {
              const float2 d = fsub2(ai, bj);
              r = ffma2(d, d, c);
            } else {
              r = ffma2(ai, bj, c);
            }
            acc[i][j] = r.x;
            acc[i][j + 1] = r.y;
          }
      } else {
#pragma unroll
        for (int i = 0; i < 8; ++i)
#pragma unroll
          for (int j = 0; j < 8; ++j) {
            if constexpr (MODE == Mode::DIFF) {
              T d = a[i] - b[j];
              acc[i][j] = fma(d, d, acc[i][j]);
            } else {
              acc[i][j] = fma(a[i], b[j], acc[i][j]);
            }
          }
      }
    }
    if (more) {
      la.store(As[cur ^ 1]);
      lb.store(Bs[cur ^ 1]);
    }
    __syncthreads();
  }
}

// out[d][r] = sum_{p < K} (data[d][p] - ref[r][p])^2
template <typename T>
__global__ void __launch_bounds__(TB_THREADS) k_knn_eudist(const T *__restrict__ ref,
                                                           const T *__restrict__ data,
                                                           int64_t n_ref, int64_t n_data,
                                                           int64_t ld, int64_t K,
                                                           T *__restrict__ out, int group_m) {
  __shared__ __align__(16) T As[2][TB_K][TB_M + 4];
  __shared__ __align__(16) T Bs[2][TB_K][TB_N + 4];
  int64_t n_img_tiles = (n_data + TB_M - 1) / TB_M;
  int64_t n_ref_tiles = (n_ref + TB_N - 1) / TB_N;
  int64_t mt, nt;
  tile_coords(n_img_tiles, n_ref_tiles, group_m, mt, nt);
  T acc[8][8];
  tile_mainloop<T, Mode::DIFF>(data, n_data, ref, n_ref, ld, K, mt * TB_M, nt * TB_N, acc, As,
                               Bs);
  const int tx = threadIdx.x & 15;
  const int ty = threadIdx.x >> 4;
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    int64_t d = mt * TB_M + ty * 4 + (i & 3) + 64 * (i >> 2);
    if (d >= n_data) continue;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      int64_t r = nt * TB_N + tx * 4 + (j & 3) + 64 * (j >> 2);
      if (r < n_ref) out[d * n_ref + r] = acc[i][j];
    }
  }
}

// Running argmin of x2 + s2 - 2 x.s, packed (order key << 32 | index).
__global__ void __launch_bounds__(TB_THREADS) k_dist_argmin_f32(
    const float *__restrict__ img, const float *__restrict__ img_sq, int64_t n_img,
    const float *__restrict__ ref, const float *__restrict__ ref_sq, int64_t n_ref, int64_t K,
    int64_t ref_offset, unsigned long long *__restrict__ best, int group_m) {
  __shared__ __align__(16) float As[2][TB_K][TB_M + 4];
  __shared__ __align__(16) float Bs[2][TB_K][TB_N + 4];
  int64_t n_img_tiles = (n_img + TB_M - 1) / TB_M;
  int64_t n_ref_tiles = (n_ref + TB_N - 1) / TB_N;
  int64_t mt, nt;
  tile_coords(n_img_tiles, n_ref_tiles, group_m, mt, nt);
  float acc[8][8];
  tile_mainloop<float, Mode::DOT>(img, n_img, ref, n_ref, K, K, mt * TB_M, nt * TB_N, acc, As,
                                  Bs);
  const int tx = threadIdx.x & 15;
  const int ty = threadIdx.x >> 4;
  float s2[8];
  int64_t rr[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    rr[j] = nt * TB_N + tx * 4 + (j & 3) + 64 * (j >> 2);
    s2[j] = rr[j] < n_ref ? ref_sq[rr[j]] : 0.0f;
  }
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    int64_t d = mt * TB_M + ty * 4 + (i & 3) + 64 * (i >> 2);
    float x2 = d < n_img ? img_sq[d] : 0.0f;
    unsigned long long key = ~0ULL;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      if (rr[j] < n_ref) {
        float dist = __fsub_rn(__fadd_rn(x2, s2[j]), __fmul_rn(2.0f, acc[i][j]));
        unsigned long long k2 =
            ((unsigned long long)float_key(dist) << 32) | (unsigned long long)(rr[j] + ref_offset);
        key = k2 < key ? k2 : key;
      }
    }
    // the 16 threads with this ty hold the other columns of the row
#pragma unroll
    for (int o = 8; o >= 1; o >>= 1) {
      unsigned long long other = __shfl_xor_sync(0xffffffffu, key, o, 16);
      key = other < key ? other : key;
    }
    if (tx == 0 && d < n_img && key != ~0ULL) atomicMin(best + d, key);
  }
}

__global__ void k_best_init(unsigned long long *best, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    best[i] = ~0ULL;
}

__global__ void k_best_unpack(const unsigned long long *__restrict__ best, int64_t n,
                              int32_t *__restrict__ idx, float *__restrict__ dist) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    unsigned long long b = best[i];
    if (idx) idx[i] = (b == ~0ULL) ? -1 : (int32_t)(b & 0xffffffffu);
    if (dist) dist[i] = key_float((uint32_t)(b >> 32));
  }
}

// FP64 running argmin over the rows of a distance block [n_img][n_ref]: one
// warp per image; the lowest column wins ties within the block, and the
// running best changes only on a strictly smaller distance (earlier blocks
// hold lower reference indices), as argmin over the whole row would.
__global__ void k_argmin_rows_f64(const double *__restrict__ dist, int64_t n_img, int64_t n_ref,
                                  int64_t ref_offset, double *__restrict__ best_dist,
                                  int64_t *__restrict__ best_idx) {
  const int lane = threadIdx.x & 31;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < n_img;
       i += nwarps) {
    const double *row = dist + i * n_ref;
    double bd = INFINITY;
    int64_t bi = -1;
    for (int64_t r = lane; r < n_ref; r += 32) {
      const double d = row[r];
      if (d < bd) {  // lanes walk their columns in increasing order
        bd = d;
        bi = r;
      }
    }
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) {
      const double od = __shfl_xor_sync(0xffffffffu, bd, o);
      const int64_t oi = __shfl_xor_sync(0xffffffffu, bi, o);
      if (oi >= 0 && (bi < 0 || od < bd || (od == bd && oi < bi))) {
        bd = od;
        bi = oi;
      }
    }
    if (lane == 0 && bi >= 0 && (best_idx[i] < 0 || bd < best_dist[i])) {
      best_dist[i] = bd;
      best_idx[i] = bi + ref_offset;
    }
  }
}

__global__ void k_best64_init(double *best_dist, int64_t *best_idx, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    best_dist[i] = INFINITY;
    best_idx[i] = -1;
  }
}

// sum of squares per row (FP64 accumulation, one warp per row)
__global__ void k_row_sqnorm(const float *__restrict__ x, int64_t n_rows, int64_t n_pix,
                             float *__restrict__ out) {
  int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  int nwarps = (gridDim.x * blockDim.x) >> 5;
  for (int64_t r = warp; r < n_rows; r += nwarps) {
    const float *p = x + r * n_pix;
    double s = 0.0;
    for (int64_t k = lane; k < n_pix; k += 32) {
      double v = p[k];
      s = fma(v, v, s);
    }
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) out[r] = (float)s;
  }
}

// uint16 counts -> f32 (+ bf16) (+ squared norm, 4-norm); one CTA of 256
// threads per frame (a warp per frame left 10,000 frames in just over one
// wave of resident warps, half the time spent in the tail).  The squared norm
// of integer counts is summed exactly in 64-bit integers (at most 65535^2 *
// n_pix, far below 2^64) and rounded once to float, the same value an exact
// FP64 sum gives; the 4-norm (FP64) is only computed when asked for.  Rows
// move as 16-byte vectors (8 counts) when aligned, four loads in flight per
// thread.
constexpr int INGEST_THREADS = 256;

__global__ void __launch_bounds__(INGEST_THREADS)
    k_ingest_u16(const uint16_t *__restrict__ in, int64_t n_img, int64_t n_pix,
                 float *__restrict__ f32, __nv_bfloat16 *__restrict__ bf, int64_t ld,
                 float *__restrict__ sq, float *__restrict__ n4, int vec) {
  constexpr int NW = INGEST_THREADS / 32;
  __shared__ unsigned long long sh2[NW];
  __shared__ double sh4[NW];
  const int t = (int)threadIdx.x, lane = t & 31, wid = t >> 5;
  const bool want4 = n4 != nullptr;
  for (int64_t r = blockIdx.x; r < n_img; r += gridDim.x) {
    const uint16_t *p = in + r * n_pix;
    unsigned long long s2 = 0;
    double s4 = 0.0;
    if (vec) {
      const uint4 *pv = reinterpret_cast<const uint4 *>(p);
      float4 *fv = reinterpret_cast<float4 *>(f32 + r * n_pix);
      uint4 *bv = bf ? reinterpret_cast<uint4 *>(bf + r * ld) : nullptr;
      const int64_t n8 = n_pix / 8;
      constexpr int U = 4;
      for (int64_t k0 = t; k0 < n8; k0 += INGEST_THREADS * U) {
        uint4 raw[U];
#pragma unroll
        for (int u = 0; u < U; ++u)
          if (k0 + INGEST_THREADS * u < n8) raw[u] = __ldg(pv + k0 + INGEST_THREADS * u);
#pragma unroll
        for (int u = 0; u < U; ++u) {
          const int64_t k = k0 + INGEST_THREADS * u;
          if (k >= n8) break;
          const uint32_t w[4] = {raw[u].x, raw[u].y, raw[u].z, raw[u].w};
          float v[8];
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            const uint32_t lo = w[q] & 0xffffu, hi = w[q] >> 16;
            v[2 * q] = (float)lo;
            v[2 * q + 1] = (float)hi;
            s2 += (unsigned long long)(lo * lo) + (unsigned long long)(hi * hi);
            if (want4) {
              const double a = (double)lo * (double)lo, b = (double)hi * (double)hi;
              s4 = fma(a, a, s4);
              s4 = fma(b, b, s4);
            }
          }
          fv[2 * k] = make_float4(v[0], v[1], v[2], v[3]);
          fv[2 * k + 1] = make_float4(v[4], v[5], v[6], v[7]);
          if (bv) {
            uint4 o;
            uint32_t *ow = reinterpret_cast<uint32_t *>(&o);
#pragma unroll
            for (int q = 0; q < 4; ++q) {
              __nv_bfloat162 h = __floats2bfloat162_rn(v[2 * q], v[2 * q + 1]);
              ow[q] = *reinterpret_cast<uint32_t *>(&h);
            }
            bv[k] = o;
          }
        }
      }
    } else {
      for (int64_t k = t; k < n_pix; k += INGEST_THREADS) {
        const uint32_t c = p[k];
        const float v = (float)c;
        f32[r * n_pix + k] = v;
        if (bf) bf[r * ld + k] = __float2bfloat16_rn(v);
        s2 += (unsigned long long)(c * c);
        if (want4) {
          const double a = (double)c * (double)c;
          s4 = fma(a, a, s4);
        }
      }
    }
    if (bf)
      for (int64_t k = n_pix + t; k < ld; k += INGEST_THREADS)
        bf[r * ld + k] = __float2bfloat16_rn(0.0f);
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) {
      s2 += __shfl_xor_sync(0xffffffffu, s2, o);
      if (want4) s4 += __shfl_xor_sync(0xffffffffu, s4, o);
    }
    if (lane == 0) {
      sh2[wid] = s2;
      sh4[wid] = s4;
    }
    __syncthreads();
    if (t == 0) {
      unsigned long long a2 = 0;
      double a4 = 0.0;
      for (int w = 0; w < NW; ++w) {
        a2 += sh2[w];
        a4 += sh4[w];
      }
      if (sq) sq[r] = __ull2float_rn(a2);
      if (n4) n4[r] = (float)sqrt(a4);
    }
    __syncthreads();  // the partial sums are reused by the next frame
  }
}

// dst[i] = src[rows[i]] for rows of row_bytes bytes (16-byte chunks when aligned)
__global__ void k_gather_rows16(const uint4 *__restrict__ src, int64_t row_chunks,
                                const int64_t *__restrict__ rows, int64_t n,
                                uint4 *__restrict__ dst) {
  int64_t total = n * row_chunks;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    int64_t i = e / row_chunks, c = e % row_chunks;
    dst[e] = src[rows[i] * row_chunks + c];
  }
}

__global__ void k_gather_rows1(const unsigned char *__restrict__ src, int64_t row_bytes,
                               const int64_t *__restrict__ rows, int64_t n,
                               unsigned char *__restrict__ dst) {
  int64_t total = n * row_bytes;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    int64_t i = e / row_bytes, c = e % row_bytes;
    dst[e] = src[rows[i] * row_bytes + c];
  }
}

// dst[rows[i]] = src[i], rows of row_bytes bytes
__global__ void k_scatter_rows1(const unsigned char *__restrict__ src, int64_t row_bytes,
                                const int64_t *__restrict__ rows, int64_t n,
                                unsigned char *__restrict__ dst) {
  int64_t total = n * row_bytes;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    int64_t i = e / row_bytes, c = e % row_bytes;
    dst[rows[i] * row_bytes + c] = src[e];
  }
}

__global__ void k_f32_to_bf16(const float *__restrict__ src, int64_t n_rows, int64_t n_pix,
                              __nv_bfloat16 *__restrict__ dst, int64_t ld) {
  int64_t total = n_rows * ld;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    int64_t r = i / ld, p = i % ld;
    dst[i] = __float2bfloat16_rn(p < n_pix ? src[r * n_pix + p] : 0.0f);
  }
}

// k smallest of each row, ascending, ties to the lower index; warp per row.
template <typename T>
__global__ void k_topk(const T *__restrict__ dist, int64_t n_rows, int64_t n_cols, int k,
                       int32_t *__restrict__ out) {
  constexpr int KMAX = 32;
  int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  int nwarps = (gridDim.x * blockDim.x) >> 5;
  for (int64_t r = warp; r < n_rows; r += nwarps) {
    T d[KMAX];
    int32_t ix[KMAX];
    int cnt = 0;
    const T *row = dist + r * n_cols;
    for (int64_t c = lane; c < n_cols; c += 32) {
      T v = row[c];
      int32_t ci = (int32_t)c;
      // columns arrive in increasing order per lane, so an equal value never
      // displaces an existing entry (lower index wins)
      if (cnt < k) {
        int pos = cnt++;
        while (pos > 0 && d[pos - 1] > v) {
          d[pos] = d[pos - 1];
          ix[pos] = ix[pos - 1];
          --pos;
        }
        d[pos] = v;
        ix[pos] = ci;
      } else if (v < d[k - 1]) {
        int pos = k - 1;
        while (pos > 0 && d[pos - 1] > v) {
          d[pos] = d[pos - 1];
          ix[pos] = ix[pos - 1];
          --pos;
        }
        d[pos] = v;
        ix[pos] = ci;
      }
    }
    int head = 0;
    for (int t = 0; t < k; ++t) {
      T hv = head < cnt ? d[head] : T(0);
      int32_t hi = head < cnt ? ix[head] : INT32_MAX;
      bool valid = head < cnt;
      // warp min by (valid, value, index)
      T bv = hv;
      int32_t bi = hi;
      bool bvalid = valid;
#pragma unroll
      for (int o = 16; o >= 1; o >>= 1) {
        T ov = __shfl_xor_sync(0xffffffffu, bv, o);
        int32_t oi = __shfl_xor_sync(0xffffffffu, bi, o);
        bool ovalid = __shfl_xor_sync(0xffffffffu, (int)bvalid, o);
        bool take = ovalid && (!bvalid || ov < bv || (ov == bv && oi < bi));
        if (take) {
          bv = ov;
          bi = oi;
          bvalid = true;
        }
      }
      if (valid && hi == bi) ++head;
      if (lane == 0) out[r * k + t] = bvalid ? bi : -1;
    }
  }
}

}  // namespace spf

using namespace spf;

template <typename T>
static int knn_eudist(const T *ref, const T *data, int64_t n_ref, int64_t n_data, int64_t n_pix,
                      T *out, void *stream, const char *name) {
  SPF_REQUIRE(n_ref >= 0 && n_data >= 0 && n_pix >= 0, "%s: negative size", name);
  if (n_ref == 0 || n_data == 0) return SPF_OK;
  SPF_REQUIRE(ref && data && out, "%s: NULL pointer", name);
  int64_t K = (n_pix / 16) * 16;  // the reference kernel drops the ragged tail
  int64_t tiles = ((n_data + TB_M - 1) / TB_M) * ((n_ref + TB_N - 1) / TB_N);
  SPF_REQUIRE(tiles < (1LL << 31), "%s: too many tiles", name);
  int group_m = (int)tune_get(SPF_TUNE_FP32_GROUP_M, GROUP_M);
  k_knn_eudist<T><<<(unsigned)tiles, TB_THREADS, 0, as_stream(stream)>>>(ref, data, n_ref, n_data,
                                                                          n_pix, K, out, group_m);
  return check_launch(name);
}

template <typename T>
static int knn_topk(const T *dist, int64_t n_data, int64_t n_ref, int k, int32_t *idx,
                    void *stream, const char *name) {
  SPF_REQUIRE(n_data >= 0 && n_ref >= 0, "%s: negative size", name);
  SPF_REQUIRE(k >= 1 && k <= 32, "%s: k must be in [1, 32]", name);
  SPF_REQUIRE(k <= n_ref || n_data == 0, "%s: k > n_ref", name);
  if (n_data == 0) return SPF_OK;
  SPF_REQUIRE(dist && idx, "%s: NULL pointer", name);
  int blocks = grid_for(n_data * 32, 256, (int64_t)sm_count() * 32);
  k_topk<T><<<blocks, 256, 0, as_stream(stream)>>>(dist, n_data, n_ref, k, idx);
  return check_launch(name);
}

extern "C" {

int spf_knn_eudist_f32(const float *d_ref, const float *d_data, int64_t n_ref, int64_t n_data,
                       int64_t n_pix, float *d_out, void *stream) {
  return knn_eudist<float>(d_ref, d_data, n_ref, n_data, n_pix, d_out, stream,
                           "spf_knn_eudist_f32");
}

int spf_knn_eudist_f64(const double *d_ref, const double *d_data, int64_t n_ref, int64_t n_data,
                       int64_t n_pix, double *d_out, void *stream) {
  return knn_eudist<double>(d_ref, d_data, n_ref, n_data, n_pix, d_out, stream,
                            "spf_knn_eudist_f64");
}

int spf_knn_topk_f32(const float *d_dist, int64_t n_data, int64_t n_ref, int k, int32_t *d_idx,
                     void *stream) {
  return knn_topk<float>(d_dist, n_data, n_ref, k, d_idx, stream, "spf_knn_topk_f32");
}

int spf_knn_topk_f64(const double *d_dist, int64_t n_data, int64_t n_ref, int k, int32_t *d_idx,
                     void *stream) {
  return knn_topk<double>(d_dist, n_data, n_ref, k, d_idx, stream, "spf_knn_topk_f64");
}

int spf_row_sqnorm_f32(const float *d_x, int64_t n_rows, int64_t n_pix, float *d_out,
                       void *stream) {
  SPF_REQUIRE(n_rows >= 0 && n_pix >= 0, "spf_row_sqnorm_f32: negative size");
  if (n_rows == 0) return SPF_OK;
  SPF_REQUIRE(d_x && d_out, "spf_row_sqnorm_f32: NULL pointer");
  int blocks = grid_for(n_rows * 32, 256, (int64_t)sm_count() * 32);
  k_row_sqnorm<<<blocks, 256, 0, as_stream(stream)>>>(d_x, n_rows, n_pix, d_out);
  return check_launch("spf_row_sqnorm_f32");
}

int spf_frames_ingest_u16(const uint16_t *d_counts, int64_t n_img, int64_t n_pix, float *d_f32,
                          void *d_bf16, int64_t ld, float *d_sq, float *d_n4, void *stream) {
  SPF_REQUIRE(n_img >= 0 && n_pix >= 0, "spf_frames_ingest_u16: negative size");
  SPF_REQUIRE(!d_bf16 || ld >= n_pix, "spf_frames_ingest_u16: ld < n_pix");
  if (n_img == 0 || n_pix == 0) return SPF_OK;
  SPF_REQUIRE(d_counts && d_f32, "spf_frames_ingest_u16: NULL pointer");
  // one CTA per frame; frames beyond 2^24 are taken by a grid-stride loop
  const int blocks = (int)std::min<int64_t>(n_img, int64_t(1) << 24);
  const int vec = n_pix % 8 == 0 && aligned(d_counts, 16) && aligned(d_f32, 16) &&
                  (!d_bf16 || (aligned(d_bf16, 16) && ld % 8 == 0));
  k_ingest_u16<<<blocks, INGEST_THREADS, 0, as_stream(stream)>>>(
      d_counts, n_img, n_pix, d_f32, reinterpret_cast<__nv_bfloat16 *>(d_bf16), ld, d_sq, d_n4,
      vec);
  return check_launch("spf_frames_ingest_u16");
}

int spf_gather_rows(const void *d_src, int64_t n_src_rows, int64_t row_bytes,
                    const int64_t *d_rows, int64_t n, void *d_dst, void *stream) {
  SPF_REQUIRE(n >= 0 && row_bytes >= 0 && n_src_rows >= 0, "spf_gather_rows: negative size");
  if (n == 0 || row_bytes == 0) return SPF_OK;
  SPF_REQUIRE(d_src && d_rows && d_dst, "spf_gather_rows: NULL pointer");
  cudaStream_t s = as_stream(stream);
  if (row_bytes % 16 == 0 && aligned(d_src, 16) && aligned(d_dst, 16)) {
    int64_t chunks = row_bytes / 16;
    k_gather_rows16<<<grid_for(n * chunks, 256, (int64_t)sm_count() * 16), 256, 0, s>>>(
        reinterpret_cast<const uint4 *>(d_src), chunks, d_rows, n,
        reinterpret_cast<uint4 *>(d_dst));
  } else {
    k_gather_rows1<<<grid_for(n * row_bytes, 256, (int64_t)sm_count() * 16), 256, 0, s>>>(
        reinterpret_cast<const unsigned char *>(d_src), row_bytes, d_rows, n,
        reinterpret_cast<unsigned char *>(d_dst));
  }
  return check_launch("spf_gather_rows");
}

int spf_scatter_rows(const void *d_src, int64_t row_bytes, const int64_t *d_rows, int64_t n,
                     void *d_dst, int64_t n_dst_rows, void *stream) {
  SPF_REQUIRE(n >= 0 && row_bytes >= 0 && n_dst_rows >= 0, "spf_scatter_rows: negative size");
  if (n == 0 || row_bytes == 0) return SPF_OK;
  SPF_REQUIRE(d_src && d_rows && d_dst, "spf_scatter_rows: NULL pointer");
  k_scatter_rows1<<<grid_for(n * row_bytes, 256, (int64_t)sm_count() * 16), 256, 0,
                    as_stream(stream)>>>(reinterpret_cast<const unsigned char *>(d_src), row_bytes,
                                         d_rows, n, reinterpret_cast<unsigned char *>(d_dst));
  return check_launch("spf_scatter_rows");
}

int spf_f32_to_bf16(const float *d_src, int64_t n_rows, int64_t n_pix, void *d_dst, int64_t ld,
                    void *stream) {
  SPF_REQUIRE(n_rows >= 0 && n_pix >= 0 && ld >= n_pix, "spf_f32_to_bf16: bad sizes");
  if (n_rows == 0 || ld == 0) return SPF_OK;
  SPF_REQUIRE(d_src && d_dst, "spf_f32_to_bf16: NULL pointer");
  k_f32_to_bf16<<<grid_for(n_rows * ld, 256, (int64_t)sm_count() * 64), 256, 0,
                  as_stream(stream)>>>(d_src, n_rows, n_pix,
                                       reinterpret_cast<__nv_bfloat16 *>(d_dst), ld);
  return check_launch("spf_f32_to_bf16");
}

int spf_best_init(uint64_t *d_best, int64_t n_img, void *stream) {
  SPF_REQUIRE(n_img >= 0, "spf_best_init: negative size");
  if (n_img == 0) return SPF_OK;
  SPF_REQUIRE(d_best != nullptr, "spf_best_init: NULL pointer");
  k_best_init<<<grid_for(n_img, 256, 4096), 256, 0, as_stream(stream)>>>(
      reinterpret_cast<unsigned long long *>(d_best), n_img);
  return check_launch("spf_best_init");
}

int spf_dist_argmin_f32(const float *d_img, const float *d_img_sq, int64_t n_img,
                        const float *d_ref, const float *d_ref_sq, int64_t n_ref, int64_t n_pix,
                        int64_t ref_offset, uint64_t *d_best, void *stream) {
  SPF_REQUIRE(n_img >= 0 && n_ref >= 0 && n_pix >= 0 && ref_offset >= 0,
              "spf_dist_argmin_f32: negative size");
  if (n_img == 0 || n_ref == 0) return SPF_OK;
  SPF_REQUIRE(d_img && d_img_sq && d_ref && d_ref_sq && d_best,
              "spf_dist_argmin_f32: NULL pointer");
  SPF_REQUIRE(ref_offset + n_ref < (1LL << 32), "spf_dist_argmin_f32: index exceeds 32 bits");
  int64_t tiles = ((n_img + TB_M - 1) / TB_M) * ((n_ref + TB_N - 1) / TB_N);
  SPF_REQUIRE(tiles < (1LL << 31), "spf_dist_argmin_f32: too many tiles");
  k_dist_argmin_f32<<<(unsigned)tiles, TB_THREADS, 0, as_stream(stream)>>>(
      d_img, d_img_sq, n_img, d_ref, d_ref_sq, n_ref, n_pix, ref_offset,
      reinterpret_cast<unsigned long long *>(d_best),
      (int)tune_get(SPF_TUNE_FP32_GROUP_M, GROUP_M));
  return check_launch("spf_dist_argmin_f32");
}

int spf_best_unpack(const uint64_t *d_best, int64_t n_img, int32_t *d_idx, float *d_dist,
                    void *stream) {
  SPF_REQUIRE(n_img >= 0, "spf_best_unpack: negative size");
  if (n_img == 0) return SPF_OK;
  SPF_REQUIRE(d_best != nullptr, "spf_best_unpack: NULL pointer");
  k_best_unpack<<<grid_for(n_img, 256, 4096), 256, 0, as_stream(stream)>>>(
      reinterpret_cast<const unsigned long long *>(d_best), n_img, d_idx, d_dist);
  return check_launch("spf_best_unpack");
}

int spf_dist_argmin_fp32(const float *d_img, const float *d_img_sq, int64_t n_img,
                         const float *d_ref, const float *d_ref_sq, int64_t n_ref, int64_t n_pix,
                         uint64_t *d_best, int32_t *d_idx, float *d_dist, void *stream) {
  SPF_REQUIRE(n_img == 0 || (d_idx && d_dist), "spf_dist_argmin_fp32: NULL output");
  SPF_TRY(spf_best_init(d_best, n_img, stream));
  SPF_TRY(spf_dist_argmin_f32(d_img, d_img_sq, n_img, d_ref, d_ref_sq, n_ref, n_pix, 0, d_best,
                              stream));
  return spf_best_unpack(d_best, n_img, d_idx, d_dist, stream);
}

int spf_dist_f64(const double *d_ref, const double *d_data, int64_t n_ref, int64_t n_data,
                 int64_t n_pix, double *d_out, void *stream) {
  SPF_REQUIRE(n_ref >= 0 && n_data >= 0 && n_pix >= 0, "spf_dist_f64: negative size");
  if (n_ref == 0 || n_data == 0) return SPF_OK;
  SPF_REQUIRE(d_ref && d_data && d_out, "spf_dist_f64: NULL pointer");
  const int64_t tiles = ((n_data + TB_M - 1) / TB_M) * ((n_ref + TB_N - 1) / TB_N);
  SPF_REQUIRE(tiles < (1LL << 31), "spf_dist_f64: too many tiles");
  const int group_m = (int)tune_get(SPF_TUNE_FP32_GROUP_M, GROUP_M);
  k_knn_eudist<double><<<(unsigned)tiles, TB_THREADS, 0, as_stream(stream)>>>(
      d_ref, d_data, n_ref, n_data, n_pix, n_pix, d_out, group_m);
  return check_launch("spf_dist_f64");
}

int spf_best64_init(double *d_best_dist, int64_t *d_best_idx, int64_t n_img, void *stream) {
  SPF_REQUIRE(n_img >= 0, "spf_best64_init: negative size");
  if (n_img == 0) return SPF_OK;
  SPF_REQUIRE(d_best_dist && d_best_idx, "spf_best64_init: NULL pointer");
  k_best64_init<<<grid_for(n_img, 256, 4096), 256, 0, as_stream(stream)>>>(d_best_dist,
                                                                           d_best_idx, n_img);
  return check_launch("spf_best64_init");
}

int spf_argmin_rows_f64(const double *d_dist, int64_t n_img, int64_t n_ref, int64_t ref_offset,
                        double *d_best_dist, int64_t *d_best_idx, void *stream) {
  SPF_REQUIRE(n_img >= 0 && n_ref >= 0 && ref_offset >= 0, "spf_argmin_rows_f64: negative size");
  if (n_img == 0 || n_ref == 0) return SPF_OK;
  SPF_REQUIRE(d_dist && d_best_dist && d_best_idx, "spf_argmin_rows_f64: NULL pointer");
  k_argmin_rows_f64<<<grid_for(n_img * 32, 256, (int64_t)sm_count() * 16), 256, 0,
                      as_stream(stream)>>>(d_dist, n_img, n_ref, ref_offset, d_best_dist,
                                           d_best_idx);
  return check_launch("spf_argmin_rows_f64");
}

}  // extern "C"
