// BF16 tensor-core orientation matching (tcgen05 + TMEM + TMA) with a fused
// per-image top-8, and the exact FP32 re-rank that restores the plain path's
// argmin.
//
// Distance: dist(i, r) = ||x_i||^2 + ||s_r||^2 - 2 x_i . s_r.  The x.s term is
// a GEMM X[n_img, K] . S[n_ref, K]^T, both operands K-major bf16.  One CTA
// (persistent, one per SM) computes 128 x 224 tiles (images x references):
//   warp 0   : TMA producer, 5-stage ring of (A 16 KB + B 28 KB) k-blocks of
//              64 pixels, 128-byte swizzle;
//   warp 1   : allocates 512 TMEM columns (two 128 x 224 FP32 accumulators,
//              256 columns apart) and issues tcgen05.mma kind::f16 (M128 N224
//              K16) from one lane;
//   warps 2-5: epilogue -- each thread owns one image row (TMEM lane), reads
//              its 224 accumulators with tcgen05.ld, forms s2 - 2 acc and keeps
//              the 8 smallest (ties to the lower index), then writes them to
//              the candidate buffer cand[n_tile][image][8].
// Accumulators are double-buffered so the epilogue of tile t overlaps the
// main loop of tile t+1.  Every mbarrier wait is bounded (1 s); on timeout
// the kernel records SPF_ERR_TIMEOUT in the device error word, stops issuing,
// drains its copies and frees TMEM before returning.
//
// The re-rank merges the candidates of all reference tiles into the per-frame
// top-8, recomputes those 8 distances in FP32 with exactly the plain path's
// arithmetic (so the values are bit-identical to it), and certifies the
// result: no reference outside the 8 can beat the re-ranked best when the
// 8th-best approximate distance exceeds it by more than the bf16 rounding
// error (10 sigma, sigma = 2 (u/sqrt 3) sqrt(sum_p x_p^2 max_r s_rp^2),
// u = 2^-8) plus the FP32 accumulation error of both paths.  Uncertified
// frames are flagged for an exact pass over all references.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <mutex>
#include <vector>

#include "common.cuh"
#include "tma.cuh"

namespace spf {
namespace bf16mm {

constexpr int BM = 128;
// 224 references per tile: a stage (A 16 KB + B 28 KB) leaves room for five
// stages in the 227 KB of shared memory a CTA may hold, one more than 256-row
// tiles allow, and the deeper ring rides out more of the L2-miss latency of
// the TMA loads (the tensor pipe idled a quarter of the cycles with four).
constexpr int BN = 224;
constexpr int BK = 64;  // bf16 elements = 128 bytes = one swizzle atom row
constexpr int STAGES = 5;
constexpr int ACC_STRIDE = 256;  // TMEM columns between the two accumulators
constexpr int A_BYTES = BM * BK * 2;
constexpr int B_BYTES = BN * BK * 2;
constexpr int STAGE_BYTES = A_BYTES + B_BYTES;
constexpr int THREADS = 192;
constexpr int TOPK = 8;
constexpr int GROUP_M = 16;
constexpr uint32_t TMEM_COLS = 512;
constexpr uint64_t TIMEOUT_NS = 1000000000ull;
constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + 1024 /*align*/ + 256 /*barriers*/;
static_assert(SMEM_BYTES <= 227 * 1024, "one CTA's shared memory");
static_assert(BN % 16 == 0 && BN <= 256 && BN <= ACC_STRIDE && 2 * ACC_STRIDE <= 512,
              "MMA N and the two TMEM accumulators");
static_assert((STAGES * A_BYTES) % 1024 == 0 && B_BYTES % 1024 == 0 && A_BYTES % 1024 == 0,
              "128-byte-swizzled stages start on 1024-byte boundaries");
static_assert(2 * STAGES * 8 + 5 * 8 + 8 <= 256, "barriers, TMEM slot and abort flag");

// Instruction descriptor, kind::f16: D = F32 (bits 4-5 = 1), A = B = BF16
// (bits 7-9, 10-12 = 1), both K-major, N >> 3 at bits 17-22, M >> 4 at 24-28.
constexpr uint32_t IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(BN >> 3) << 17) |
                           ((uint32_t)(BM >> 4) << 24);

// Bounded wait.  Returns false (and raises the CTA abort flag) on timeout or
// when another role of the CTA has already aborted.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, volatile int *abort) {
  if (mbar_try_wait(bar, parity)) return true;
  uint64_t t0 = globaltimer();
  for (uint32_t it = 1;; ++it) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((it & 255) == 0) {
      if (*abort) return false;
      if (globaltimer() - t0 > TIMEOUT_NS) {
        *abort = 1;
        return false;
      }
    }
  }
}

__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

__device__ __forceinline__ uint64_t sdesc_sw128(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);  // start address
  d |= (uint64_t)1 << 16;                    // leading byte offset (unused, swizzled K-major)
  d |= (uint64_t)(1024 >> 4) << 32;          // stride byte offset: 8 rows x 128 B
  d |= (uint64_t)1 << 46;                    // descriptor version
  d |= (uint64_t)2 << 61;                    // 128-byte swizzle
  return d;
}

__device__ __forceinline__ void umma_bf16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(IDESC), "r"(acc)
      : "memory");
}

__device__ __forceinline__ void umma_commit(uint64_t *bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&r)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
      "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
      "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]),
        "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]),
        "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

struct TopK {
  float d[TOPK];
  int32_t i[TOPK];
  __device__ __forceinline__ void clear() {
#pragma unroll
    for (int k = 0; k < TOPK; ++k) {
      d[k] = __int_as_float(0x7f800000);  // +inf
      i[k] = INT32_MAX;
    }
  }
  // insert with ties resolved towards the lower index (callers feed indices
  // in increasing order, so a strict < on the value keeps the earlier one)
  __device__ __forceinline__ void push(float v, int32_t j) {
    if (!(v < d[TOPK - 1])) return;
    d[TOPK - 1] = v;
    i[TOPK - 1] = j;
#pragma unroll
    for (int k = TOPK - 1; k > 0; --k) {
      bool sw = d[k] < d[k - 1];
      float td = sw ? d[k - 1] : d[k];
      int32_t ti = sw ? i[k - 1] : i[k];
      d[k - 1] = sw ? d[k] : d[k - 1];
      i[k - 1] = sw ? i[k] : i[k - 1];
      d[k] = td;
      i[k] = ti;
    }
  }
};

__device__ __forceinline__ void tile_of(int64_t t, int64_t n_m, int64_t n_n, int group_m,
                                        int64_t &m, int64_t &n) {
  int64_t per_group = (int64_t)group_m * n_n;
  int64_t g = t / per_group;
  int64_t first_m = g * group_m;
  int64_t gm = n_m - first_m < group_m ? n_m - first_m : group_m;
  int64_t r = t % per_group;
  m = first_m + r % gm;
  n = r / gm;
}

// RANGE = false: per-tile top-8 into cand_d / cand_i.
// RANGE = true : every reference with s2 - 2 acc <= thresh[row] is appended to
//                list[row * cap ..] (count[row] holds the number found, which
//                may exceed cap: the caller then treats the row as overflowed).
template <bool RANGE>
__global__ void __launch_bounds__(THREADS, 1)
    k_dist_topk_bf16(const __grid_constant__ CUtensorMap tmap_a,
                     const __grid_constant__ CUtensorMap tmap_b, const float *__restrict__ ref_sq,
                     int64_t n_img, int64_t n_ref, int64_t n_pix, float *__restrict__ cand_d,
                     int32_t *__restrict__ cand_i, const float *__restrict__ thresh,
                     int32_t *__restrict__ list, int32_t *__restrict__ count, int cap,
                     int group_m, unsigned int *__restrict__ err) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t *smem = reinterpret_cast<uint8_t *>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~static_cast<uintptr_t>(1023));
  uint8_t *sA = smem;
  uint8_t *sB = smem + STAGES * A_BYTES;
  uint64_t *bars = reinterpret_cast<uint64_t *>(smem + STAGES * STAGE_BYTES);
  uint64_t *full = bars;
  uint64_t *empty = bars + STAGES;
  uint64_t *acc_full = bars + 2 * STAGES;
  uint64_t *acc_empty = bars + 2 * STAGES + 2;
  uint64_t *done = bars + 2 * STAGES + 4;
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bars + 2 * STAGES + 5);
  volatile int *abort = reinterpret_cast<volatile int *>(tmem_slot + 1);

  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  const int64_t n_m = (n_img + BM - 1) / BM;
  const int64_t n_n = (n_ref + BN - 1) / BN;
  const int64_t n_tiles = n_m * n_n;
  const int nkb = (int)((n_pix + BK - 1) / BK);

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&acc_full[b], 1);
      mbar_init(&acc_empty[b], 128);
    }
    mbar_init(done, 1);
    *abort = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tmem_slot)),
                 "r"(TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem_base = *tmem_slot;

  if (warp == 0) {
    if (lane == 0) {
      // ---------------- TMA producer ----------------
      uint32_t it = 0;
      bool ok = true;
      for (int64_t t = blockIdx.x; t < n_tiles && ok; t += gridDim.x) {
        int64_t m, n;
        tile_of(t, n_m, n_n, group_m, m, n);
        for (int kb = 0; kb < nkb; ++kb, ++it) {
          int s = it % STAGES;
          uint32_t ph = (it / STAGES) & 1;
          if (!mbar_wait(&empty[s], ph ^ 1, abort)) {
            ok = false;
            break;
          }
          mbar_arrive_expect_tx(&full[s], STAGE_BYTES);
          tma_load_2d(sA + s * A_BYTES, &tmap_a, &full[s], kb * BK, (int)(m * BM));
          tma_load_2d(sB + s * B_BYTES, &tmap_b, &full[s], kb * BK, (int)(n * BN));
        }
      }
      // drain: every issued copy must have landed before the CTA exits
      uint32_t first = it > (uint32_t)STAGES ? it - STAGES : 0;
      for (uint32_t j = first; j < it; ++j) {
        int s = j % STAGES;
        uint32_t ph = (j / STAGES) & 1;
        uint64_t t0 = globaltimer();
        while (!mbar_try_wait(&full[s], ph) && globaltimer() - t0 < TIMEOUT_NS) {
        }
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      // ---------------- MMA issuer ----------------
      uint32_t it = 0, tc = 0;
      bool ok = true;
      for (int64_t t = blockIdx.x; t < n_tiles && ok; t += gridDim.x, ++tc) {
        uint32_t b = tc & 1, use = tc >> 1;
        if (!mbar_wait(&acc_empty[b], (use & 1) ^ 1, abort)) break;
        tc_fence_after();
        uint32_t d_tmem = tmem_base + b * ACC_STRIDE;
        for (int kb = 0; kb < nkb; ++kb, ++it) {
          int s = it % STAGES;
          uint32_t ph = (it / STAGES) & 1;
          if (!mbar_wait(&full[s], ph, abort)) {
            ok = false;
            break;
          }
          tc_fence_after();
          uint32_t a0 = smem_u32(sA + s * A_BYTES);
          uint32_t b0 = smem_u32(sB + s * B_BYTES);
#pragma unroll
          for (int k = 0; k < BK / 16; ++k) {
            umma_bf16(d_tmem, sdesc_sw128(a0 + k * 32), sdesc_sw128(b0 + k * 32),
                      (kb | k) != 0 ? 1u : 0u);
          }
          umma_commit(&empty[s]);
        }
        if (!ok) break;
        umma_commit(&acc_full[b]);
      }
      // all issued MMAs complete before TMEM is released
      umma_commit(done);
      uint64_t t0 = globaltimer();
      while (!mbar_try_wait(done, 0) && globaltimer() - t0 < TIMEOUT_NS) {
      }
    }
  } else {
    // ---------------- epilogue (warps 2..5) ----------------
    const int q = warp & 3;  // TMEM lane quarter this warp may access
    uint32_t tc = 0;
    for (int64_t t = blockIdx.x; t < n_tiles; t += gridDim.x, ++tc) {
      int64_t m, n;
      tile_of(t, n_m, n_n, group_m, m, n);
      uint32_t b = tc & 1, use = tc >> 1;
      // one lane waits, the warp follows (tcgen05.ld below is warp-collective)
      int ok = 1;
      if (lane == 0) ok = mbar_wait(&acc_full[b], use & 1, abort) ? 1 : 0;
      ok = __shfl_sync(0xffffffffu, ok, 0);
      if (!ok) break;
      tc_fence_after();
      const int64_t row = m * BM + q * 32 + lane;
      const int64_t col0 = n * BN;
      if constexpr (RANGE) {
        const float thr = row < n_img ? thresh[row] : -__int_as_float(0x7f800000);
#pragma unroll 1
        for (int c = 0; c < BN / 32; ++c) {
          uint32_t r[32];
          tmem_ld32(tmem_base + ((uint32_t)(q * 32) << 16) + b * ACC_STRIDE + c * 32, r);
#pragma unroll
          for (int j = 0; j < 32; ++j) {
            int64_t col = col0 + c * 32 + j;
            if (col < n_ref) {
              float v = __ldg(ref_sq + col) - 2.0f * __uint_as_float(r[j]);
              if (v <= thr) {
                int pos = atomicAdd(count + row, 1);
                if (pos < cap) list[row * cap + pos] = (int32_t)col;
              }
            }
          }
        }
        tc_fence_before();
        mbar_arrive(&acc_empty[b]);
      } else {
        TopK top;
        top.clear();
#pragma unroll 1
        for (int c = 0; c < BN / 32; ++c) {
          uint32_t r[32];
          tmem_ld32(tmem_base + ((uint32_t)(q * 32) << 16) + b * ACC_STRIDE + c * 32, r);
#pragma unroll
          for (int j = 0; j < 32; ++j) {
            int64_t col = col0 + c * 32 + j;
            if (col < n_ref) {
              float v = __ldg(ref_sq + col) - 2.0f * __uint_as_float(r[j]);
              top.push(v, (int32_t)col);
            }
          }
        }
        tc_fence_before();
        mbar_arrive(&acc_empty[b]);
        if (row < n_img) {
          size_t base = ((size_t)n * n_img + row) * TOPK;
          float4 *pd = reinterpret_cast<float4 *>(cand_d + base);
          int4 *pi = reinterpret_cast<int4 *>(cand_i + base);
          pd[0] = make_float4(top.d[0], top.d[1], top.d[2], top.d[3]);
          pd[1] = make_float4(top.d[4], top.d[5], top.d[6], top.d[7]);
          pi[0] = make_int4(top.i[0], top.i[1], top.i[2], top.i[3]);
          pi[1] = make_int4(top.i[4], top.i[5], top.i[6], top.i[7]);
        }
      }
    }
  }

  __syncthreads();
  if (threadIdx.x == 0 && *abort) atomicExch(err, (unsigned int)(-SPF_ERR_TIMEOUT));
  tc_fence_after();
  if (warp == 1) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem_base),
                 "r"(TMEM_COLS)
                 : "memory");
  }
}

// Waits on an mbarrier that nothing arrives at, through the same bounded wait
// the GEMM uses, and reports what the wait returned: the self-test of the
// timeout path (the wait must give up, raise the abort flag and leave the
// device usable).
__global__ void k_wait_selftest(uint64_t timeout_ns, unsigned int *err, int *result) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    uint64_t t0 = globaltimer();
    bool ok = true;
    while (!mbar_try_wait(&bar, 0)) {
      if (globaltimer() - t0 > timeout_ns) {
        ok = false;
        break;
      }
    }
    result[0] = ok ? 1 : 0;
    result[1] = (int)((globaltimer() - t0) / 1000000ull);  // ms waited
    if (!ok) atomicExch(err, (unsigned int)(-SPF_ERR_TIMEOUT));
    // complete the barrier's phase so no waiter can remain
    mbar_arrive(&bar);
  }
}

// ---------------------------------------------------------------------------
// merge + exact FP32 re-rank
// ---------------------------------------------------------------------------
constexpr int RR_THREADS = 256;
constexpr float U_BF16 = 1.0f / 256.0f;    // unit roundoff of bf16 (8 significant bits)
constexpr float U_FP32 = 5.9604645e-8f;    // 2^-24
constexpr float CERT_SIGMAS = 10.0f;

__device__ __forceinline__ bool lex_less(float a, int32_t ia, float b, int32_t ib) {
  return a < b || (a == b && ia < ib);
}

// Block per frame: the 8 smallest candidates over all reference tiles (by
// distance, then index), written to mrg[frame] (tile 0's slot of the
// candidate buffers when mrg is that slot, the older layout); and the frame's
// bf16 error variance term V = sum_p x_p^2 max_r s_rp^2 (negated when some
// x_p is not exact in bf16) into work[frame].
__global__ void __launch_bounds__(RR_THREADS)
    k_merge_top8(const float *__restrict__ cand_d, const int32_t *__restrict__ cand_i,
                 int64_t n_tiles, const float *__restrict__ img, int64_t n_img,
                 const float *__restrict__ m2, int64_t n_pix, float *__restrict__ work,
                 float *__restrict__ mrg_d, int32_t *__restrict__ mrg_i) {
  __shared__ float s_d[RR_THREADS / 32][TOPK];
  __shared__ int32_t s_i[RR_THREADS / 32][TOPK];
  __shared__ float s_v[RR_THREADS / 32];
  __shared__ int s_x[RR_THREADS / 32];
  const int64_t im = blockIdx.x;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (im >= n_img) return;
  float d[TOPK];
  int32_t ix[TOPK];
#pragma unroll
  for (int k = 0; k < TOPK; ++k) {
    d[k] = __int_as_float(0x7f800000);
    ix[k] = INT32_MAX;
  }
  const int64_t total = n_tiles * TOPK;
  for (int64_t c = tid; c < total; c += RR_THREADS) {
    int64_t tile = c / TOPK, k = c % TOPK;
    size_t off = ((size_t)tile * n_img + im) * TOPK + k;
    float v = cand_d[off];
    int32_t j = cand_i[off];
    if (!lex_less(v, j, d[TOPK - 1], ix[TOPK - 1])) continue;
    d[TOPK - 1] = v;
    ix[TOPK - 1] = j;
#pragma unroll
    for (int q = TOPK - 1; q > 0; --q) {
      bool sw = lex_less(d[q], ix[q], d[q - 1], ix[q - 1]);
      float td = sw ? d[q - 1] : d[q];
      int32_t ti = sw ? ix[q - 1] : ix[q];
      d[q - 1] = sw ? d[q] : d[q - 1];
      ix[q - 1] = sw ? ix[q] : ix[q - 1];
      d[q] = td;
      ix[q] = ti;
    }
  }
  // frame error term (coalesced pass over the frame)
  float V = 0.0f;
  int inexact = 0;
  const float *x = img + im * n_pix;
  for (int64_t p = tid; p < n_pix; p += RR_THREADS) {
    float xv = x[p];
    V = fmaf(xv * xv, __ldg(m2 + p), V);
    inexact |= (__bfloat162float(__float2bfloat16_rn(xv)) != xv);
  }
  // warp merge of the per-thread lists: 8 rounds of a lexicographic minimum
  int head = 0;
  for (int r = 0; r < TOPK; ++r) {
    float hv = head < TOPK ? d[head] : __int_as_float(0x7f800000);
    int32_t hi = head < TOPK ? ix[head] : INT32_MAX;
    float bv = hv;
    int32_t bi = hi;
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) {
      float ov = __shfl_xor_sync(0xffffffffu, bv, o);
      int32_t oi = __shfl_xor_sync(0xffffffffu, bi, o);
      if (lex_less(ov, oi, bv, bi)) {
        bv = ov;
        bi = oi;
      }
    }
    if (head < TOPK && hv == bv && hi == bi) ++head;
    if (lane == 0) {
      s_d[warp][r] = bv;
      s_i[warp][r] = bi;
    }
  }
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1) {
    V += __shfl_xor_sync(0xffffffffu, V, o);
    inexact |= __shfl_xor_sync(0xffffffffu, inexact, o);
  }
  if (lane == 0) {
    s_v[warp] = V;
    s_x[warp] = inexact;
  }
  __syncthreads();
  if (warp == 0) {
    float a0 = s_d[lane >> 3][lane & 7], a1 = s_d[4 + (lane >> 3)][lane & 7];
    int32_t j0 = s_i[lane >> 3][lane & 7], j1 = s_i[4 + (lane >> 3)][lane & 7];
    if (lex_less(a1, j1, a0, j0)) {
      float tv = a0; a0 = a1; a1 = tv;
      int32_t tj = j0; j0 = j1; j1 = tj;
    }
    int h = 0;
    for (int r = 0; r < TOPK; ++r) {
      float hv = h == 0 ? a0 : (h == 1 ? a1 : __int_as_float(0x7f800000));
      int32_t hi = h == 0 ? j0 : (h == 1 ? j1 : INT32_MAX);
      float bv = hv;
      int32_t bi = hi;
#pragma unroll
      for (int o = 16; o >= 1; o >>= 1) {
        float ov = __shfl_xor_sync(0xffffffffu, bv, o);
        int32_t oi = __shfl_xor_sync(0xffffffffu, bi, o);
        if (lex_less(ov, oi, bv, bi)) {
          bv = ov;
          bi = oi;
        }
      }
      if (h < 2 && hv == bv && hi == bi) ++h;
      if (lane == 0) {
        size_t off = (size_t)im * TOPK + r;
        mrg_d[off] = bv;
        mrg_i[off] = bi;
      }
    }
    if (lane == 0) {
      float vt = 0.0f;
      int ex = 0;
      for (int w = 0; w < RR_THREADS / 32; ++w) {
        vt += s_v[w];
        ex |= s_x[w];
      }
      work[im] = ex ? -vt : vt;
    }
  }
}

// Exact FP32 distances of the 8 candidates of each frame, computed with the
// arithmetic of the plain kernel (k_dist_argmin_f32): acc = fma(x_p, s_p, acc)
// for p = 0 .. n_pix-1 in order, then (x2 + s2) - 2 acc, so the re-ranked
// values are bit-identical to the plain path's.  A CTA takes 4 frames (32
// (frame, candidate) chains, one per lane of warp 0); all its warps stream the
// 4 frame rows and 32 candidate rows through shared memory in 64-pixel
// chunks, RXE_STAGES - 1 chunks in flight (cp.async groups issued by warps
// 1-3 while warp 0 runs the chains), rows padded to 68 floats so that the
// chains' 16-byte reads of 8 consecutive rows fall on distinct banks.  Small
// stages keep 29 KB of shared memory per CTA, so many CTAs (and their loads)
// are resident per SM.  Lane 0 of each group of 8 keeps the lexicographic
// minimum and evaluates the certificate.
// The certificate's band: a bound on |approximate - exact| distance for any
// reference (CERT_SIGMAS sigma of the bf16 rounding, per-pixel bound, plus
// the FP32 accumulation error of both paths).
__device__ __forceinline__ float cert_band(float V, float x2, float ref_sq_max, int64_t n_pix) {
  float vs = V < 0.0f ? -2.0f * V : V;  // x rounding doubles the variance term
  float sig16 = 2.0f * U_BF16 * 0.57735027f * sqrtf(vs);
  float sig32 = U_FP32 * sqrtf((float)n_pix) * (x2 + ref_sq_max);
  return CERT_SIGMAS * (sig16 + 2.0f * sig32);
}

// A candidate whose approximate distance exceeds the best approximate one by
// more than twice the band cannot be the exact minimum (its exact distance
// is above the band's upper end for the best candidate), so its row is not
// read: only the candidates near the best are re-ranked.
__device__ __forceinline__ bool rerank_skip(const float *cand_d, int64_t im, int c, float band) {
  return c > 0 && cand_d[(size_t)im * TOPK + c] > cand_d[(size_t)im * TOPK] + 2.0f * band;
}

constexpr int RX_FRAMES = 4;
constexpr int RX_ROWS = RX_FRAMES * (TOPK + 1);  // 4 frame rows + 32 candidate rows
constexpr int RX_THREADS = 128;
constexpr int RXE_CHUNK = 64;                    // re-rank kernels: pixels per stage
constexpr int RXE_STRIDE = RXE_CHUNK + 4;
constexpr int RXE_STAGES = 3;

__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(smem)), "l"(gmem)
               : "memory");
}

__global__ void __launch_bounds__(RX_THREADS)
    k_rerank_exact(const float *__restrict__ cand_d, const int32_t *__restrict__ cand_i,
                   const float *__restrict__ img, const float *__restrict__ img_sq,
                   int64_t n_img, const float *__restrict__ ref, const float *__restrict__ ref_sq,
                   int64_t n_ref, float ref_sq_max, int64_t n_pix, int64_t ref_offset,
                   float *__restrict__ work, int32_t *__restrict__ out_idx,
                   float *__restrict__ out_dist, int32_t *__restrict__ uncertified,
                   int32_t *__restrict__ out_top) {
  extern __shared__ __align__(16) float rx[];  // [RXE_STAGES][RX_ROWS][RXE_STRIDE]
  __shared__ const float *rows[RX_ROWS];
  const int tid = threadIdx.x;
  const int64_t f0 = (int64_t)blockIdx.x * RX_FRAMES;
  // row table: r < 4 -> frame rows, r >= 4 -> candidate rows (frame (r-4)/8)
  if (tid < RX_ROWS) {
    const float *ptr = nullptr;
    if (tid < RX_FRAMES) {
      int64_t im = f0 + tid;
      if (im < n_img) ptr = img + im * n_pix;
    } else {
      int q = tid - RX_FRAMES;
      int64_t im = f0 + q / TOPK;
      if (im < n_img) {
        int32_t j = cand_i[(size_t)im * TOPK + (q % TOPK)];
        float band = cert_band(work[im], img_sq[im], ref_sq_max, n_pix);
        // an index outside [0, n_ref) (a candidate slot the GEMM did not
        // write) is never read
        if (j >= 0 && j < n_ref && !rerank_skip(cand_d, im, q % TOPK, band))
          ptr = ref + (int64_t)j * n_pix;
      }
    }
    rows[tid] = ptr;
  }
  __syncthreads();
  const int64_t nchunks = (n_pix + RXE_CHUNK - 1) / RXE_CHUNK;
  const bool vec = (n_pix % 4) == 0 && aligned(img, 16) && aligned(ref, 16);
  // asynchronous 16-byte copies of one chunk of every row (ragged ends by
  // plain loads)
  // (a chunk past the end issues nothing; its group is still committed so
  // that the group count stays one per chunk)
  auto stage = [&](int buf, int64_t chunk) {
    float *dst = rx + (size_t)buf * RX_ROWS * RXE_STRIDE;
    const int64_t base = chunk * RXE_CHUNK;
    if (tid < 32) return;  // warp 0 runs the chains; warps 1.. stage
    for (int e = tid - 32; chunk < nchunks && e < RX_ROWS * (RXE_CHUNK / 4);
         e += RX_THREADS - 32) {
      int r = e / (RXE_CHUNK / 4), q4 = (e % (RXE_CHUNK / 4)) * 4;
      const float *src = rows[r];
      // a row without source (a skipped candidate, a list slot past the end,
      // a frame past the last) is not staged: its chain's result is discarded
      if (!src) continue;
      int64_t p = base + q4;
      float *d = dst + r * RXE_STRIDE + q4;
      if (vec && p + 3 < n_pix) {
        cp_async16(d, src + p);
      } else {
#pragma unroll
        for (int u = 0; u < 4; ++u) d[u] = p + u < n_pix ? __ldg(src + p + u) : 0.0f;
      }
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
  };
  // chain of lane l of warp 0: frame l / 8, candidate l % 8
  const int lane = tid & 31;
  const int fr = lane / TOPK;
  const int crow = RX_FRAMES + lane;
  float acc = 0.0f;
#pragma unroll
  for (int st = 0; st < RXE_STAGES - 1; ++st) stage(st, st);
  for (int64_t ch = 0; ch < nchunks; ++ch) {
    const int cur = (int)(ch % RXE_STAGES);
    // chunk ch has landed (groups complete in order; RXE_STAGES - 2 younger
    // ones may still be in flight) and is visible to every thread; every
    // thread is also done with the buffer the next stage overwrites
    asm volatile("cp.async.wait_group %0;" ::"n"(RXE_STAGES - 2) : "memory");
    __syncthreads();
    stage((int)((ch + RXE_STAGES - 1) % RXE_STAGES), ch + RXE_STAGES - 1);
    if (tid < 32) {
      const float *xb = rx + (size_t)cur * RX_ROWS * RXE_STRIDE + fr * RXE_STRIDE;
      const float *sb = rx + (size_t)cur * RX_ROWS * RXE_STRIDE + crow * RXE_STRIDE;
      const int64_t lim = n_pix - ch * RXE_CHUNK;
      if (lim >= RXE_CHUNK) {
#pragma unroll 4
        for (int k = 0; k < RXE_CHUNK; k += 4) {  // 16-byte reads, same FMA order
          const float4 xv = *reinterpret_cast<const float4 *>(xb + k);
          const float4 sv = *reinterpret_cast<const float4 *>(sb + k);
          acc = fmaf(xv.x, sv.x, acc);
          acc = fmaf(xv.y, sv.y, acc);
          acc = fmaf(xv.z, sv.z, acc);
          acc = fmaf(xv.w, sv.w, acc);
        }
      } else {
        for (int k = 0; k < (int)lim; ++k) acc = fmaf(xb[k], sb[k], acc);
      }
    }
  }
  asm volatile("cp.async.wait_group 0;" ::: "memory");
  if (tid >= 32) return;
  const int64_t im = f0 + fr;
  const int c = lane % TOPK;
  const bool live = im < n_img;
  const int64_t imc = live ? im : 0;
  int32_t j = cand_i[(size_t)imc * TOPK + c];
  float x2 = live ? img_sq[imc] : 0.0f;
  const float band = live ? cert_band(work[imc], x2, ref_sq_max, n_pix) : 0.0f;
  const bool valid = live && j >= 0 && j < n_ref && !rerank_skip(cand_d, imc, c, band);
  float dist = valid ? __fsub_rn(__fadd_rn(x2, ref_sq[j]), __fmul_rn(2.0f, acc))
                     : __int_as_float(0x7f800000);
  int32_t jj = valid ? j : INT32_MAX;
#pragma unroll
  for (int o = 4; o >= 1; o >>= 1) {
    float od = __shfl_xor_sync(0xffffffffu, dist, o, TOPK);
    int32_t oj = __shfl_xor_sync(0xffffffffu, jj, o, TOPK);
    if (lex_less(od, oj, dist, jj)) {
      dist = od;
      jj = oj;
    }
  }
  if (!live) return;
  if (out_top) out_top[im * TOPK + c] = (j == INT32_MAX) ? -1 : (int32_t)(j + ref_offset);
  if (c != 0) return;
  out_idx[im] = jj == INT32_MAX ? -1 : (int32_t)(jj + ref_offset);
  if (out_dist) out_dist[im] = dist;
  if (!uncertified) return;
  // certificate: every reference outside the 8 has approximate distance
  // >= d8 (+ x2), and its plain-path distance differs from that by at most
  // the bf16 rounding error (CERT_SIGMAS sigma, per-pixel bound) plus the
  // FP32 accumulation error of both paths; the re-ranked best must lie below
  int32_t j7 = cand_i[(size_t)im * TOPK + TOPK - 1];
  int cert = 1;
  if (j7 != INT32_MAX) {
    float d8 = cand_d[(size_t)im * TOPK + TOPK - 1] + x2;
    cert = (d8 - band - dist) > 0.0f ? 1 : 0;
  }
  uncertified[im] = cert ? 0 : 1;
  // the range that must be searched when the frame is not certified: every
  // reference whose approximate distance (without x2) lies within the band
  // of the re-ranked best
  work[im] = (dist - x2) + band;
}

constexpr size_t RX_SMEM = (size_t)RXE_STAGES * RX_ROWS * RXE_STRIDE * sizeof(float);

// Exact FP32 distances (plain-path arithmetic) for every listed candidate of
// every frame; the per-frame lexicographic minimum is folded into best[]
// (packed order key << 32 | index, as spf_dist_argmin_f32 keeps it).  A CTA
// takes one frame and walks its list 32 candidates at a time: warps 1-3
// stream the frame row and the 32 candidate rows through shared memory in
// 64-pixel chunks (cp.async, the stages of k_rerank_exact) while warp 0 runs
// the 32 sequential FMA chains.
constexpr int RL_ROWS = 33;

__global__ void __launch_bounds__(RX_THREADS)
    k_rerank_list(const int32_t *__restrict__ list, const int32_t *__restrict__ count, int cap,
                  const float *__restrict__ img, const float *__restrict__ img_sq, int64_t n_img,
                  const float *__restrict__ ref, const float *__restrict__ ref_sq, int64_t n_pix,
                  int64_t ref_offset, unsigned long long *__restrict__ best) {
  extern __shared__ __align__(16) float rx[];  // [RXE_STAGES][RL_ROWS][RXE_STRIDE]
  __shared__ const float *rows[RL_ROWS];
  const int64_t im = blockIdx.x;
  const int tid = threadIdx.x, lane = tid & 31;
  if (im >= n_img) return;
  int cnt = count[im];
  // a count above the cap marks a list that is incomplete (overflowed, or a
  // saturated tile list that may hide references, with fewer than cap entries
  // written): the caller settles that frame another way, so nothing is read
  if (cnt > cap) cnt = 0;
  const int64_t nchunks = (n_pix + RXE_CHUNK - 1) / RXE_CHUNK;
  const bool vec = (n_pix % 4) == 0 && aligned(img, 16) && aligned(ref, 16);
  unsigned long long kbest = ~0ULL;
  for (int g0 = 0; g0 < cnt; g0 += 32) {
    __syncthreads();  // the previous group is done with rows[] and the buffers
    if (tid < RL_ROWS) {
      const float *ptr = nullptr;
      if (tid == 0) {
        ptr = img + im * n_pix;
      } else if (g0 + tid - 1 < cnt) {
        ptr = ref + (int64_t)list[im * cap + g0 + tid - 1] * n_pix;
      }
      rows[tid] = ptr;
    }
    __syncthreads();
    // warps 1.. stage the chunks (an empty group past the end keeps one
    // group per chunk); warp 0 runs the chains
    auto stage = [&](int buf, int64_t chunk) {
      if (tid < 32) return;
      float *dst = rx + (size_t)buf * RL_ROWS * RXE_STRIDE;
      const int64_t base = chunk * RXE_CHUNK;
      for (int e = tid - 32; chunk < nchunks && e < RL_ROWS * (RXE_CHUNK / 4);
           e += RX_THREADS - 32) {
        int r = e / (RXE_CHUNK / 4), q4 = (e % (RXE_CHUNK / 4)) * 4;
        const float *src = rows[r];
        if (!src) continue;  // a slot past the list's end: its chain is discarded
        int64_t p = base + q4;
        float *d = dst + r * RXE_STRIDE + q4;
        if (vec && p + 3 < n_pix) {
          cp_async16(d, src + p);
        } else {
#pragma unroll
          for (int u = 0; u < 4; ++u) d[u] = p + u < n_pix ? __ldg(src + p + u) : 0.0f;
        }
      }
      asm volatile("cp.async.commit_group;" ::: "memory");
    };
    float acc = 0.0f;
#pragma unroll
    for (int st = 0; st < RXE_STAGES - 1; ++st) stage(st, st);
    for (int64_t ch = 0; ch < nchunks; ++ch) {
      const int cur = (int)(ch % RXE_STAGES);
      asm volatile("cp.async.wait_group %0;" ::"n"(RXE_STAGES - 2) : "memory");
      __syncthreads();
      stage((int)((ch + RXE_STAGES - 1) % RXE_STAGES), ch + RXE_STAGES - 1);
      if (tid < 32) {
        const float *xb = rx + (size_t)cur * RL_ROWS * RXE_STRIDE;
        const float *sb = xb + (1 + lane) * RXE_STRIDE;
        const int64_t lim = n_pix - ch * RXE_CHUNK;
        if (lim >= RXE_CHUNK) {
#pragma unroll 4
          for (int k = 0; k < RXE_CHUNK; k += 4) {  // 16-byte reads, same FMA order
            const float4 xv = *reinterpret_cast<const float4 *>(xb + k);
            const float4 sv = *reinterpret_cast<const float4 *>(sb + k);
            acc = fmaf(xv.x, sv.x, acc);
            acc = fmaf(xv.y, sv.y, acc);
            acc = fmaf(xv.z, sv.z, acc);
            acc = fmaf(xv.w, sv.w, acc);
          }
        } else {
          for (int k = 0; k < (int)lim; ++k) acc = fmaf(xb[k], sb[k], acc);
        }
      }
    }
    asm volatile("cp.async.wait_group 0;" ::: "memory");
    if (tid < 32 && g0 + lane < cnt) {
      int32_t j = list[im * cap + g0 + lane];
      float dist = __fsub_rn(__fadd_rn(img_sq[im], ref_sq[j]), __fmul_rn(2.0f, acc));
      unsigned long long key =
          ((unsigned long long)float_key(dist) << 32) | (unsigned long long)(j + ref_offset);
      kbest = key < kbest ? key : kbest;
    }
  }
  if (tid < 32) {
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) {
      unsigned long long other = __shfl_xor_sync(0xffffffffu, kbest, o);
      kbest = other < kbest ? other : kbest;
    }
    if (lane == 0 && kbest != ~0ULL) atomicMin(best + im, kbest);
  }
}

constexpr size_t RL_SMEM = (size_t)RXE_STAGES * RL_ROWS * RXE_STRIDE * sizeof(float);

// column maxima of squares: out[p] = max_r x[r, p]^2
__global__ void k_col_maxsq(const float *__restrict__ x, int64_t n_rows, int64_t n_pix,
                            float *__restrict__ out) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n_pix;
       p += (int64_t)gridDim.x * blockDim.x) {
    float m = 0.0f;
    for (int64_t r = 0; r < n_rows; ++r) {
      float v = x[r * n_pix + p];
      m = fmaxf(m, v * v);
    }
    out[p] = m;
  }
}

// sum of squares and sqrt(sum of fourth powers) per row, FP64 accumulation
__global__ void k_row_norms(const float *__restrict__ x, int64_t n_rows, int64_t n_pix,
                            float *__restrict__ sq, float *__restrict__ n4) {
  int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  int nwarps = (gridDim.x * blockDim.x) >> 5;
  for (int64_t r = warp; r < n_rows; r += nwarps) {
    const float *p = x + r * n_pix;
    double s2 = 0.0, s4 = 0.0;
    for (int64_t k = lane; k < n_pix; k += 32) {
      double v = p[k];
      double v2 = v * v;
      s2 += v2;
      s4 = fma(v2, v2, s4);
    }
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) {
      s2 += __shfl_xor_sync(0xffffffffu, s2, o);
      s4 += __shfl_xor_sync(0xffffffffu, s4, o);
    }
    if (lane == 0) {
      if (sq) sq[r] = (float)s2;
      if (n4) n4[r] = (float)sqrt(s4);
    }
  }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
// k_rerank_exact uses RX_SMEM (29 KB) of dynamic shared memory
static int rerank_smem_attr() {
  static bool done[64] = {false};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64 || done[dev]) return SPF_OK;
  SPF_TRY(check_cuda(cudaFuncSetAttribute(k_rerank_exact,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)RX_SMEM),
                     "k_rerank_exact"));
  done[dev] = true;
  return SPF_OK;
}

static int make_map(CUtensorMap *map, const void *base, int64_t rows, int64_t ld, int box_rows) {
  auto fn = tensor_map_encoder();
  if (!fn) {
    set_error("cuTensorMapEncodeTiled is not available from the driver");
    return SPF_ERR_UNSUPPORTED;
  }
  cuuint64_t dims[2] = {(cuuint64_t)ld, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)(ld * 2)};
  cuuint32_t box[2] = {(cuuint32_t)BK, (cuuint32_t)box_rows};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(base), dims,
                  strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                  CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    set_error("cuTensorMapEncodeTiled failed (%d)", (int)r);
    return SPF_ERR_ARG;
  }
  return SPF_OK;
}

}  // namespace bf16mm
}  // namespace spf

using namespace spf;
using namespace spf::bf16mm;

extern "C" {

int64_t spf_dist_topk_bf16_tiles(int64_t n_ref) { return (n_ref + BN - 1) / BN; }

int64_t spf_dist_topk_bf16_tile_refs(void) { return BN; }

static int launch_bf16(bool range, const void *d_img_bf16, int64_t n_img, const void *d_ref_bf16,
                       int64_t n_ref, int64_t n_pix, int64_t ld, const float *d_ref_sq,
                       float *d_cand_d, int32_t *d_cand_i, const float *d_thresh,
                       int32_t *d_list, int32_t *d_count, int cap, void *stream,
                       const char *name) {
  SPF_REQUIRE(n_img >= 0 && n_ref >= 0 && n_pix >= 0, "%s: negative size", name);
  if (n_img == 0 || n_ref == 0) return SPF_OK;
  SPF_REQUIRE(d_img_bf16 && d_ref_bf16 && d_ref_sq, "%s: NULL pointer", name);
  SPF_REQUIRE(ld >= n_pix && ld % 8 == 0,
              "%s: row stride ld must be >= n_pix and a multiple of 8", name);
  SPF_REQUIRE(aligned(d_img_bf16, 16) && aligned(d_ref_bf16, 16),
              "%s: operands must be 16-byte aligned", name);
  SPF_REQUIRE(n_img < (1LL << 31) && n_ref < (1LL << 31) && ld < (1LL << 31),
              "%s: size too large", name);
  int dev = 0;
  cudaGetDevice(&dev);
  int major = 0, minor = 0;
  cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev);
  cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev);
  if (major != 10 || minor != 3) {
    set_error("%s: needs sm_103 (GB300), device is sm_%d%d", name, major, minor);
    return SPF_ERR_UNSUPPORTED;
  }
  CUtensorMap ma, mb;
  SPF_TRY(make_map(&ma, d_img_bf16, n_img, ld, BM));
  SPF_TRY(make_map(&mb, d_ref_bf16, n_ref, ld, BN));
  static bool attr_set[2][64] = {{false}};
  if (dev >= 0 && dev < 64 && !attr_set[range][dev]) {
    cudaError_t e = range ? cudaFuncSetAttribute(k_dist_topk_bf16<true>,
                                                 cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                 SMEM_BYTES)
                          : cudaFuncSetAttribute(k_dist_topk_bf16<false>,
                                                 cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                 SMEM_BYTES);
    SPF_TRY(check_cuda(e, name));
    attr_set[range][dev] = true;
  }
  unsigned int *err = device_error_word();
  SPF_REQUIRE(err != nullptr, "%s: no device error word", name);
  int64_t tiles = ((n_img + BM - 1) / BM) * ((n_ref + BN - 1) / BN);
  int64_t max_grid = tune_get(SPF_TUNE_BF16_GRID, sm_count());
  int grid = (int)(tiles < max_grid ? tiles : max_grid);
  int group_m = (int)tune_get(SPF_TUNE_BF16_GROUP_M, GROUP_M);
  if (range)
    k_dist_topk_bf16<true><<<grid, THREADS, SMEM_BYTES, as_stream(stream)>>>(
        ma, mb, d_ref_sq, n_img, n_ref, n_pix, nullptr, nullptr, d_thresh, d_list, d_count, cap,
        group_m, err);
  else
    k_dist_topk_bf16<false><<<grid, THREADS, SMEM_BYTES, as_stream(stream)>>>(
        ma, mb, d_ref_sq, n_img, n_ref, n_pix, d_cand_d, d_cand_i, nullptr, nullptr, nullptr, 0,
        group_m, err);
  return check_launch(name);
}

int spf_dist_topk_bf16(const void *d_img_bf16, int64_t n_img, const void *d_ref_bf16,
                       int64_t n_ref, int64_t n_pix, int64_t ld, const float *d_ref_sq,
                       float *d_cand_d, int32_t *d_cand_i, void *stream) {
  SPF_REQUIRE(n_img == 0 || n_ref == 0 || (d_cand_d && d_cand_i),
              "spf_dist_topk_bf16: NULL candidate buffer");
  SPF_REQUIRE(aligned(d_cand_d, 16) && aligned(d_cand_i, 16),
              "spf_dist_topk_bf16: candidate buffers must be 16-byte aligned");
  return launch_bf16(false, d_img_bf16, n_img, d_ref_bf16, n_ref, n_pix, ld, d_ref_sq, d_cand_d,
                     d_cand_i, nullptr, nullptr, nullptr, 0, stream, "spf_dist_topk_bf16");
}

int spf_dist_range_bf16(const void *d_img_bf16, int64_t n_img, const void *d_ref_bf16,
                        int64_t n_ref, int64_t n_pix, int64_t ld, const float *d_ref_sq,
                        const float *d_thresh, int32_t *d_list, int32_t *d_count, int cap,
                        void *stream) {
  SPF_REQUIRE(cap >= 1 && cap <= 4096, "spf_dist_range_bf16: cap must be in [1, 4096]");
  SPF_REQUIRE(n_img == 0 || n_ref == 0 || (d_thresh && d_list && d_count),
              "spf_dist_range_bf16: NULL pointer");
  if (n_img > 0)
    SPF_TRY(check_cuda(cudaMemsetAsync(d_count, 0, n_img * sizeof(int32_t), as_stream(stream)),
                       "spf_dist_range_bf16"));
  return launch_bf16(true, d_img_bf16, n_img, d_ref_bf16, n_ref, n_pix, ld, d_ref_sq, nullptr,
                     nullptr, d_thresh, d_list, d_count, cap, stream, "spf_dist_range_bf16");
}

int spf_rerank_list_fp32(const int32_t *d_list, const int32_t *d_count, int cap,
                         const float *d_img, const float *d_img_sq, int64_t n_img,
                         const float *d_ref, const float *d_ref_sq, int64_t n_pix,
                         int64_t ref_offset, uint64_t *d_best, void *stream) {
  SPF_REQUIRE(n_img >= 0 && n_pix >= 0 && cap >= 1, "spf_rerank_list_fp32: bad size");
  if (n_img == 0) return SPF_OK;
  SPF_REQUIRE(d_list && d_count && d_img && d_img_sq && d_ref && d_ref_sq && d_best,
              "spf_rerank_list_fp32: NULL pointer");
  SPF_REQUIRE(n_img < (1LL << 31), "spf_rerank_list_fp32: too many frames");
  static bool attr[64] = {false};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev >= 0 && dev < 64 && !attr[dev]) {
    SPF_TRY(check_cuda(cudaFuncSetAttribute(k_rerank_list,
                                            cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            (int)RL_SMEM),
                       "spf_rerank_list_fp32"));
    attr[dev] = true;
  }
  k_rerank_list<<<(unsigned)n_img, RX_THREADS, RL_SMEM, as_stream(stream)>>>(
      d_list, d_count, cap, d_img, d_img_sq, n_img, d_ref, d_ref_sq, n_pix, ref_offset,
      reinterpret_cast<unsigned long long *>(d_best));
  return check_launch("k_rerank_list");
}

}  // extern "C" (reopened below)

namespace spf {
namespace bf16mm {

// Block per open frame (rows[r]): every candidate of every reference tile
// whose approximate distance lies within the frame's bound thresh[r] goes to
// list[r][...] (count[r] of them; the order does not matter to the re-rank).
// The tile lists hold each tile's 8 smallest approximate distances, so they
// contain every in-bound reference of the tile unless all 8 are in bound: the
// tile may then hold more, and count[r] is set above the cap so that the
// caller searches that frame by the range GEMM.
__global__ void __launch_bounds__(256)
    k_scan_band(const float *__restrict__ cand_d, const int32_t *__restrict__ cand_i,
                int64_t n_tiles, int64_t n_img, const int64_t *__restrict__ rows,
                const float *__restrict__ thresh, int32_t *__restrict__ list,
                int32_t *__restrict__ count, int cap) {
  __shared__ int cnt, sat;
  const int64_t r = blockIdx.x;
  const int64_t im = rows[r];
  const float T = thresh[r];
  if (threadIdx.x == 0) {
    cnt = 0;
    sat = 0;
  }
  __syncthreads();
  for (int64_t t = threadIdx.x; t < n_tiles; t += blockDim.x) {
    const size_t off = ((size_t)t * n_img + im) * TOPK;
    int valid = 0, inband = 0;
#pragma unroll
    for (int k = 0; k < TOPK; ++k) {
      const int32_t j = cand_i[off + k];
      if (j == INT32_MAX) continue;
      ++valid;
      if (cand_d[off + k] <= T) {
        ++inband;
        const int pos = atomicAdd(&cnt, 1);
        if (pos < cap) list[r * (int64_t)cap + pos] = j;
      }
    }
    if (valid == TOPK && inband == TOPK) sat = 1;
  }
  __syncthreads();
  if (threadIdx.x == 0) count[r] = sat ? cap + 1 : cnt;
}

}  // namespace bf16mm
}  // namespace spf

extern "C" {

int spf_scan_band_bf16(const float *d_cand_d, const int32_t *d_cand_i, int64_t n_tiles,
                       int64_t n_img, const int64_t *d_rows, int64_t n_rows,
                       const float *d_thresh, int32_t *d_list, int32_t *d_count, int cap,
                       void *stream) {
  SPF_REQUIRE(n_tiles >= 0 && n_img >= 0 && n_rows >= 0 && cap >= 1,
              "spf_scan_band_bf16: bad sizes");
  if (n_rows == 0) return SPF_OK;
  SPF_REQUIRE(d_cand_d && d_cand_i && d_rows && d_thresh && d_list && d_count,
              "spf_scan_band_bf16: NULL pointer");
  SPF_REQUIRE(n_rows < (1LL << 31), "spf_scan_band_bf16: too many rows");
  spf::bf16mm::k_scan_band<<<(unsigned)n_rows, 256, 0, as_stream(stream)>>>(
      d_cand_d, d_cand_i, n_tiles, n_img, d_rows, d_thresh, d_list, d_count, cap);
  return check_launch("k_scan_band");
}

int spf_complete_open(const float *d_cand_d, const int32_t *d_cand_i, int64_t n_tiles,
                      const void *d_img_bf16, const float *d_img, const float *d_img_sq,
                      const float *d_work, int64_t n_img, const int64_t *d_rows, int64_t n_rows,
                      const void *d_ref_bf16, const float *d_ref, const float *d_ref_sq,
                      int64_t n_ref, int64_t n_pix, int64_t ld, int32_t *d_idx, float *d_dist,
                      int64_t *h_stats, void *stream) {
  SPF_REQUIRE(n_rows >= 0 && n_img >= 0, "spf_complete_open: bad sizes");
  if (h_stats) h_stats[0] = h_stats[1] = h_stats[2] = 0;
  if (n_rows == 0) return SPF_OK;
  SPF_REQUIRE(d_cand_d && d_cand_i && d_img_bf16 && d_img && d_img_sq && d_work && d_rows &&
                  d_ref_bf16 && d_ref && d_ref_sq && d_idx && d_dist,
              "spf_complete_open: NULL pointer");
  constexpr int CAP = 512;
  cudaStream_t s = as_stream(stream);
  void *sv = stream;
  std::vector<void *> bufs;
  int st = SPF_OK;
  auto get = [&](size_t bytes) -> void * {
    void *p = nullptr;
    if (st == SPF_OK)
      st = check_cuda(cudaMallocAsync(&p, bytes < 16 ? 16 : bytes, s), "spf_complete_open");
    if (p) bufs.push_back(p);
    return p;
  };
  const int64_t nr = n_rows;
  float *f32_c = (float *)get((size_t)nr * n_pix * 4);
  float *sq_c = (float *)get(nr * 4), *thr_c = (float *)get(nr * 4);
  int32_t *lst = (int32_t *)get((size_t)nr * CAP * 4), *cnt = (int32_t *)get(nr * 4);
  uint64_t *best = (uint64_t *)get(nr * 8);
  int64_t *sub = (int64_t *)get(nr * 8);
  void *bf_c = get((size_t)nr * ld * 2);
  std::vector<int32_t> h_cnt(nr);
  std::vector<int64_t> h_rows(nr);
  if (st == SPF_OK) st = spf_gather_rows(d_img, n_img, n_pix * 4, d_rows, nr, f32_c, sv);
  if (st == SPF_OK) st = spf_gather_rows(d_img_sq, n_img, 4, d_rows, nr, sq_c, sv);
  if (st == SPF_OK) st = spf_gather_rows(d_work, n_img, 4, d_rows, nr, thr_c, sv);
  // 1) the kept tile lists: every in-bound candidate, re-ranked exactly
  if (st == SPF_OK)
    st = spf_scan_band_bf16(d_cand_d, d_cand_i, n_tiles, n_img, d_rows, nr, thr_c, lst, cnt, CAP,
                            sv);
  if (st == SPF_OK) st = spf_best_init(best, nr, sv);
  if (st == SPF_OK)
    st = spf_rerank_list_fp32(lst, cnt, CAP, f32_c, sq_c, nr, d_ref, d_ref_sq, n_pix, 0, best, sv);
  if (st == SPF_OK) st = spf_best_unpack(best, nr, d_idx, d_dist, sv);
  if (st == SPF_OK)
    st = check_cuda(cudaMemcpyAsync(h_cnt.data(), cnt, nr * 4, cudaMemcpyDeviceToHost, s),
                    "spf_complete_open");
  if (st == SPF_OK)
    st = check_cuda(cudaMemcpyAsync(h_rows.data(), d_rows, nr * 8, cudaMemcpyDeviceToHost, s),
                    "spf_complete_open");
  if (st == SPF_OK) st = check_cuda(cudaStreamSynchronize(s), "spf_complete_open");
  // 2) frames whose tile lists may hide references: the range GEMM, then
  //    (a list over the cap) the plain pass
  std::vector<int64_t> over_pos;  // positions within the rows
  for (int64_t k = 0; st == SPF_OK && k < nr; ++k)
    if (h_cnt[k] > CAP) over_pos.push_back(k);
  if (h_stats) h_stats[0] = (int64_t)over_pos.size();
  for (int pass = 0; pass < 2 && st == SPF_OK && !over_pos.empty(); ++pass) {
    const int64_t no = (int64_t)over_pos.size();
    std::vector<int64_t> h_sub(over_pos);
    st = check_cuda(cudaMemcpyAsync(sub, h_sub.data(), no * 8, cudaMemcpyHostToDevice, s),
                    "spf_complete_open");
    // compact copies of those rows (frame data indexed within the gathered rows)
    float *f32_o = (float *)get((size_t)no * n_pix * 4);
    float *sq_o = (float *)get(no * 4), *thr_o = (float *)get(no * 4);
    int32_t *idx_o = (int32_t *)get(no * 4);
    float *dist_o = (float *)get(no * 4);
    int64_t *frames_o = (int64_t *)get(no * 8);
    if (st == SPF_OK) st = spf_gather_rows(f32_c, nr, n_pix * 4, sub, no, f32_o, sv);
    if (st == SPF_OK) st = spf_gather_rows(sq_c, nr, 4, sub, no, sq_o, sv);
    if (st == SPF_OK) st = spf_gather_rows(thr_c, nr, 4, sub, no, thr_o, sv);
    if (st == SPF_OK) st = spf_best_init(best, no, sv);
    std::vector<int32_t> h_c2(no, 0);
    std::vector<int64_t> h_fr(no);
    if (pass == 0) {
      for (int64_t k = 0; k < no; ++k) h_fr[k] = h_rows[over_pos[k]];
      if (st == SPF_OK)
        st = check_cuda(cudaMemcpyAsync(frames_o, h_fr.data(), no * 8, cudaMemcpyHostToDevice, s),
                        "spf_complete_open");
      if (st == SPF_OK) st = spf_gather_rows(d_img_bf16, n_img, ld * 2, frames_o, no, bf_c, sv);
      if (st == SPF_OK)
        st = spf_dist_range_bf16(bf_c, no, d_ref_bf16, n_ref, n_pix, ld, d_ref_sq, thr_o, lst,
                                 cnt, CAP, sv);
      if (st == SPF_OK)
        st = spf_rerank_list_fp32(lst, cnt, CAP, f32_o, sq_o, no, d_ref, d_ref_sq, n_pix, 0, best,
                                  sv);
      if (st == SPF_OK)
        st = check_cuda(cudaMemcpyAsync(h_c2.data(), cnt, no * 4, cudaMemcpyDeviceToHost, s),
                        "spf_complete_open");
    } else if (st == SPF_OK) {
      st = spf_dist_argmin_f32(f32_o, sq_o, no, d_ref, d_ref_sq, n_ref, n_pix, 0, best, sv);
    }
    if (st == SPF_OK) st = spf_best_unpack(best, no, idx_o, dist_o, sv);
    // the completed rows go back into d_idx / d_dist at their positions
    if (st == SPF_OK) st = spf_scatter_rows(idx_o, 4, sub, no, d_idx, nr, sv);
    if (st == SPF_OK) st = spf_scatter_rows(dist_o, 4, sub, no, d_dist, nr, sv);
    if (st == SPF_OK) st = check_cuda(cudaStreamSynchronize(s), "spf_complete_open");
    std::vector<int64_t> next;
    for (int64_t k = 0; pass == 0 && k < no; ++k)
      if (h_c2[k] > CAP) next.push_back(over_pos[k]);
    if (pass == 0 && h_stats) h_stats[1] = (int64_t)next.size();
    over_pos.swap(next);
  }
  for (void *p : bufs) cudaFreeAsync(p, s);
  return st;
}

static int rerank_impl(const char *name, float *d_cand_d, int32_t *d_cand_i, int64_t n_tiles,
                       const float *d_img, const float *d_img_sq, int64_t n_img,
                       const float *d_ref, const float *d_ref_sq, const float *d_ref_m2,
                       float ref_sq_max, int64_t n_ref, int64_t n_pix, int64_t ref_offset,
                       float *d_work, int32_t *d_idx, float *d_dist, int32_t *d_uncertified,
                       int32_t *d_top8, float *d_mrg_d, int32_t *d_mrg_i, void *stream) {
  SPF_REQUIRE(n_img >= 0 && n_ref >= 0 && n_pix >= 0 && n_tiles >= 0,
              "%s: negative size", name);
  if (n_img == 0) return SPF_OK;
  SPF_REQUIRE(d_cand_d && d_cand_i && d_img && d_img_sq && d_ref && d_ref_sq && d_ref_m2 &&
                  d_work && d_idx && d_mrg_d && d_mrg_i,
              "%s: NULL pointer", name);
  SPF_REQUIRE(n_tiles == (n_ref + BN - 1) / BN, "%s: n_tiles does not match n_ref", name);
  SPF_REQUIRE(n_img < (1LL << 28), "%s: too many images", name);
  cudaStream_t s = as_stream(stream);
  k_merge_top8<<<(unsigned)n_img, RR_THREADS, 0, s>>>(d_cand_d, d_cand_i, n_tiles, d_img, n_img,
                                                      d_ref_m2, n_pix, d_work, d_mrg_d, d_mrg_i);
  SPF_TRY(check_launch("k_merge_top8"));
  SPF_TRY(rerank_smem_attr());
  k_rerank_exact<<<(unsigned)((n_img + RX_FRAMES - 1) / RX_FRAMES), RX_THREADS, RX_SMEM, s>>>(
      d_mrg_d, d_mrg_i, d_img, d_img_sq, n_img, d_ref, d_ref_sq, n_ref, ref_sq_max, n_pix,
      ref_offset, d_work, d_idx, d_dist, d_uncertified, d_top8);
  return check_launch("k_rerank_exact");
}

int spf_rerank_fp32(float *d_cand_d, int32_t *d_cand_i, int64_t n_tiles, const float *d_img,
                    const float *d_img_sq, int64_t n_img, const float *d_ref,
                    const float *d_ref_sq, const float *d_ref_m2, float ref_sq_max,
                    int64_t n_ref, int64_t n_pix, int64_t ref_offset, float *d_work,
                    int32_t *d_idx, float *d_dist, int32_t *d_uncertified, int32_t *d_top8,
                    void *stream) {
  return rerank_impl("spf_rerank_fp32", d_cand_d, d_cand_i, n_tiles, d_img, d_img_sq, n_img,
                     d_ref, d_ref_sq, d_ref_m2, ref_sq_max, n_ref, n_pix, ref_offset, d_work,
                     d_idx, d_dist, d_uncertified, d_top8, d_cand_d, d_cand_i, stream);
}

int spf_rerank_fp32_keep(const float *d_cand_d, const int32_t *d_cand_i, int64_t n_tiles,
                         const float *d_img, const float *d_img_sq, int64_t n_img,
                         const float *d_ref, const float *d_ref_sq, const float *d_ref_m2,
                         float ref_sq_max, int64_t n_ref, int64_t n_pix, int64_t ref_offset,
                         float *d_work, int32_t *d_idx, float *d_dist, int32_t *d_uncertified,
                         float *d_merged_d, int32_t *d_merged_i, void *stream) {
  return rerank_impl("spf_rerank_fp32_keep", const_cast<float *>(d_cand_d),
                     const_cast<int32_t *>(d_cand_i), n_tiles, d_img, d_img_sq, n_img, d_ref,
                     d_ref_sq, d_ref_m2, ref_sq_max, n_ref, n_pix, ref_offset, d_work, d_idx,
                     d_dist, d_uncertified, nullptr, d_merged_d, d_merged_i, stream);
}

int spf_col_maxsq_f32(const float *d_x, int64_t n_rows, int64_t n_pix, float *d_out,
                      void *stream) {
  SPF_REQUIRE(n_rows >= 0 && n_pix >= 0, "spf_col_maxsq_f32: negative size");
  if (n_pix == 0) return SPF_OK;
  SPF_REQUIRE(d_x && d_out, "spf_col_maxsq_f32: NULL pointer");
  k_col_maxsq<<<grid_for(n_pix, 256, 4096), 256, 0, as_stream(stream)>>>(d_x, n_rows, n_pix,
                                                                          d_out);
  return check_launch("spf_col_maxsq_f32");
}

int spf_selftest_bounded_wait(int64_t timeout_ms, int *d_result, void *stream) {
  SPF_REQUIRE(timeout_ms > 0 && timeout_ms <= 5000, "spf_selftest_bounded_wait: 1..5000 ms");
  SPF_REQUIRE(d_result != nullptr, "spf_selftest_bounded_wait: NULL pointer");
  unsigned int *err = device_error_word();
  SPF_REQUIRE(err != nullptr, "spf_selftest_bounded_wait: no device error word");
  k_wait_selftest<<<1, 32, 0, as_stream(stream)>>>((uint64_t)timeout_ms * 1000000ull, err,
                                                   d_result);
  return check_launch("k_wait_selftest");
}

int spf_row_norms_f32(const float *d_x, int64_t n_rows, int64_t n_pix, float *d_sq, float *d_n4,
                      void *stream) {
  SPF_REQUIRE(n_rows >= 0 && n_pix >= 0, "spf_row_norms_f32: negative size");
  if (n_rows == 0) return SPF_OK;
  SPF_REQUIRE(d_x != nullptr, "spf_row_norms_f32: NULL pointer");
  int blocks = grid_for(n_rows * 32, 256, (int64_t)sm_count() * 32);
  k_row_norms<<<blocks, 256, 0, as_stream(stream)>>>(d_x, n_rows, n_pix, d_sq, d_n4);
  return check_launch("spf_row_norms_f32");
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Matching without device allocation.
//
// Some callers cannot call cudaMalloc: code that records its work inside a
// CUDA stream capture (an allocation there breaks the capture), and online
// data-acquisition processes that fix their GPU memory when they start and
// must not allocate while frames stream in.  spf_match_bf16_static gives them
// the bf16 tensor-core top-8 + exact FP32 re-rank with its scratch (the
// candidate buffer, the re-rank work area and the device error word) in the
// file-scope array below instead of caller- or library-allocated memory.
// The array is part of this library's device image: every GPU that loads the
// library holds it (STATIC_SCRATCH_BYTES = 2 x 8 MiB of candidates + 16 KiB of
// per-frame work + 256 B for the error word) until the process exits.  All
// calls on a device share it and it keeps the last call's contents, so calls
// that overlap on the GPU (different streams, or different host threads)
// race; serialise them.  The call clears the error word first; the GEMM then
// writes every candidate slot the re-rank reads, unless a bounded wait gives
// up, in which case the re-rank skips indices outside [0, n_ref), the call's
// outputs are marked void (idx -1, distance NaN, uncertified 1) and the error
// word keeps the code for spf_device_error.
// ---------------------------------------------------------------------------
namespace spf {
namespace bf16mm {

constexpr int64_t STATIC_MAX_TILE_FRAMES = SPF_STATIC_MAX_TILE_FRAMES;  // tiles(n_ref) * n_img
constexpr int64_t STATIC_MAX_FRAMES = SPF_STATIC_MAX_FRAMES;
constexpr size_t STATIC_CAND_BYTES = (size_t)STATIC_MAX_TILE_FRAMES * TOPK * 4;
constexpr size_t STATIC_WORK_BYTES = (size_t)STATIC_MAX_FRAMES * 4;
constexpr size_t STATIC_SCRATCH_BYTES = 2 * STATIC_CAND_BYTES + STATIC_WORK_BYTES + 256;

static __device__ __align__(256) unsigned char g_match_scratch[STATIC_SCRATCH_BYTES];

// After a GEMM that gave up a bounded wait (*err != 0): idx -1, distance
// NaN and uncertified for every frame of the call.
// Test hook (SPF_TUNE_STATIC_ABORT_TEST): records a given-up wait, as the
// GEMM's own timeout path does, so that the void answers and their report
// can be checked without making any wait run out.
__global__ void k_static_inject_timeout(unsigned int *__restrict__ err) {
  if (threadIdx.x == 0 && blockIdx.x == 0) atomicExch(err, (unsigned int)(-SPF_ERR_TIMEOUT));
}

__global__ void k_static_abort_mark(const unsigned int *__restrict__ err, int64_t n_img,
                                    int32_t *__restrict__ idx, float *__restrict__ dist,
                                    int32_t *__restrict__ unc) {
  if (*err == 0u) return;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n_img;
       i += (int64_t)gridDim.x * blockDim.x) {
    idx[i] = -1;
    if (dist) dist[i] = __int_as_float(0x7fc00000);
    if (unc) unc[i] = 1;
  }
}

// Device address of g_match_scratch per device, looked up once with the
// device current (host code cannot use the symbol itself as an address).
static std::mutex g_static_mu;
static unsigned char *g_static_ptr[64] = {nullptr};
static bool g_static_attr[64] = {false};

static int static_scratch(int dev, unsigned char **out) {
  std::lock_guard<std::mutex> lk(g_static_mu);
  if (!g_static_ptr[dev]) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_match_scratch);
    if (e != cudaSuccess || p == nullptr) {
      set_error("spf_match_bf16_static: cudaGetSymbolAddress failed: %s", cudaGetErrorString(e));
      return SPF_ERR_CUDA;
    }
    g_static_ptr[dev] = static_cast<unsigned char *>(p);
  }
  if (!g_static_attr[dev]) {
    SPF_TRY(check_cuda(cudaFuncSetAttribute(k_dist_topk_bf16<false>,
                                            cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            SMEM_BYTES),
                       "spf_match_bf16_static"));
    g_static_attr[dev] = true;
  }
  *out = g_static_ptr[dev];
  return SPF_OK;
}

}  // namespace bf16mm

// The static path's error word on the current device, or NULL while no
// static call has set the path up on it (read by spf_device_error).
unsigned int *static_match_error_word() {
  using namespace bf16mm;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
  std::lock_guard<std::mutex> lk(g_static_mu);
  if (!g_static_ptr[dev]) return nullptr;
  return reinterpret_cast<unsigned int *>(g_static_ptr[dev] + 2 * STATIC_CAND_BYTES +
                                          STATIC_WORK_BYTES);
}

}  // namespace spf

extern "C" int spf_match_bf16_static(const void *d_img_bf16, const float *d_img,
                                     const float *d_img_sq, int64_t n_img,
                                     const void *d_ref_bf16, const float *d_ref,
                                     const float *d_ref_sq, const float *d_ref_m2,
                                     float ref_sq_max, int64_t n_ref, int64_t n_pix, int64_t ld,
                                     int32_t *d_idx, float *d_dist, int32_t *d_uncertified,
                                     void *stream) {
  using namespace spf;
  using namespace spf::bf16mm;
  const char *name = "spf_match_bf16_static";
  SPF_REQUIRE(n_img >= 0 && n_ref >= 0 && n_pix >= 0, "%s: negative size", name);
  if (n_img == 0) return SPF_OK;
  SPF_REQUIRE(n_ref > 0, "%s: no references", name);
  const int64_t tiles = (n_ref + BN - 1) / BN;
  SPF_REQUIRE(n_img <= STATIC_MAX_FRAMES,
              "%s: %lld frames exceed the static scratch limit of %lld frames per call", name,
              (long long)n_img, (long long)STATIC_MAX_FRAMES);
  SPF_REQUIRE(tiles * n_img <= STATIC_MAX_TILE_FRAMES,
              "%s: ceil(n_ref/%d) * n_img = %lld exceeds the static scratch limit of %lld "
              "(split the references or the frames)",
              name, BN, (long long)(tiles * n_img), (long long)STATIC_MAX_TILE_FRAMES);
  SPF_REQUIRE(d_img_bf16 && d_img && d_img_sq && d_ref_bf16 && d_ref && d_ref_sq && d_ref_m2 &&
                  d_idx,
              "%s: NULL pointer", name);
  SPF_REQUIRE(ld >= n_pix && ld % 8 == 0, "%s: ld must be >= n_pix and a multiple of 8", name);
  SPF_REQUIRE(aligned(d_img_bf16, 16) && aligned(d_ref_bf16, 16),
              "%s: bf16 operands must be 16-byte aligned", name);
  SPF_REQUIRE(n_ref < (1LL << 31) && ld < (1LL << 31), "%s: size too large", name);
  int dev = 0;
  SPF_TRY(check_cuda(cudaGetDevice(&dev), name));
  SPF_REQUIRE(dev >= 0 && dev < 64, "%s: device index out of range", name);
  int major = 0, minor = 0;
  cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev);
  cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev);
  if (major != 10 || minor != 3) {
    set_error("%s: needs sm_103 (GB300), device is sm_%d%d", name, major, minor);
    return SPF_ERR_UNSUPPORTED;
  }
  unsigned char *base = nullptr;
  SPF_TRY(static_scratch(dev, &base));
  float *cand_d = reinterpret_cast<float *>(base);
  int32_t *cand_i = reinterpret_cast<int32_t *>(base + STATIC_CAND_BYTES);
  float *work = reinterpret_cast<float *>(base + 2 * STATIC_CAND_BYTES);
  unsigned int *err =
      reinterpret_cast<unsigned int *>(base + 2 * STATIC_CAND_BYTES + STATIC_WORK_BYTES);
  cudaStream_t s = as_stream(stream);
  SPF_TRY(check_cuda(cudaMemsetAsync(err, 0, sizeof(unsigned int), s), name));
  CUtensorMap ma, mb;
  SPF_TRY(make_map(&ma, d_img_bf16, n_img, ld, BM));
  SPF_TRY(make_map(&mb, d_ref_bf16, n_ref, ld, BN));
  int64_t gemm_tiles = ((n_img + BM - 1) / BM) * tiles;
  int grid = (int)(gemm_tiles < sm_count() ? gemm_tiles : sm_count());
  k_dist_topk_bf16<false><<<grid, THREADS, SMEM_BYTES, s>>>(ma, mb, d_ref_sq, n_img, n_ref,
                                                            n_pix, cand_d, cand_i, nullptr,
                                                            nullptr, nullptr, 0, GROUP_M, err);
  SPF_TRY(check_launch("k_dist_topk_bf16 (static scratch)"));
  if (tune_get(SPF_TUNE_STATIC_ABORT_TEST, 0)) {
    k_static_inject_timeout<<<1, 32, 0, s>>>(err);
    SPF_TRY(check_launch("k_static_inject_timeout"));
  }
  k_merge_top8<<<(unsigned)n_img, RR_THREADS, 0, s>>>(cand_d, cand_i, tiles, d_img, n_img,
                                                      d_ref_m2, n_pix, work, cand_d, cand_i);
  SPF_TRY(check_launch("k_merge_top8 (static scratch)"));
  SPF_TRY(rerank_smem_attr());
  k_rerank_exact<<<(unsigned)((n_img + RX_FRAMES - 1) / RX_FRAMES), RX_THREADS, RX_SMEM, s>>>(
      cand_d, cand_i, d_img, d_img_sq, n_img, d_ref, d_ref_sq, n_ref, ref_sq_max, n_pix, 0, work,
      d_idx, d_dist, d_uncertified, nullptr);
  SPF_TRY(check_launch("k_rerank_exact (static scratch)"));
  // a GEMM that gave up a bounded wait left candidate slots unwritten: the
  // call's answers are then void, and every frame says so
  k_static_abort_mark<<<grid_for(n_img, 256, 1024), 256, 0, s>>>(err, n_img, d_idx, d_dist,
                                                                d_uncertified);
  return check_launch("k_static_abort_mark");
}
