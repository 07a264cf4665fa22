// Shared helpers for the spinifel_gb300 CUDA library: status handling,
// thread-local error text, launch accounting and small device utilities.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include <atomic>
#include <string>

#include "../../include/spinifel_gb300.h"

namespace spf {

// Thread-local message of the last failure on this host thread.
void set_error(const char *fmt, ...);
const char *get_error();

// Count of kernels launched by this library (all threads).
extern std::atomic<uint64_t> g_launches;
inline void count_launch(uint64_t n = 1) { g_launches.fetch_add(n, std::memory_order_relaxed); }

// Device-side error word (per device; bounded waits write codes here).
unsigned int *device_error_word();
// The error word of the matching path without device allocation
// (spf_match_bf16_static) on the current device; NULL until that path has
// been set up on it.
unsigned int *static_match_error_word();

inline cudaStream_t as_stream(void *s) { return reinterpret_cast<cudaStream_t>(s); }

// Check the launch that was just issued; returns an SPF status.
inline int check_launch(const char *what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error("%s: launch failed: %s", what, cudaGetErrorString(e));
    return SPF_ERR_LAUNCH;
  }
  count_launch();
  return SPF_OK;
}

inline int check_cuda(cudaError_t e, const char *what) {
  if (e == cudaSuccess) return SPF_OK;
  set_error("%s: %s", what, cudaGetErrorString(e));
  return e == cudaErrorMemoryAllocation ? SPF_ERR_OOM : SPF_ERR_CUDA;
}

#define SPF_REQUIRE(cond, ...)          \
  do {                                  \
    if (!(cond)) {                      \
      ::spf::set_error(__VA_ARGS__);    \
      return SPF_ERR_ARG;               \
    }                                   \
  } while (0)

#define SPF_TRY(expr)              \
  do {                             \
    int _st = (expr);              \
    if (_st != SPF_OK) return _st; \
  } while (0)

__host__ __device__ inline bool aligned(const void *p, size_t a) { return (reinterpret_cast<uintptr_t>(p) % a) == 0; }

// Order-preserving map of a float to uint32 (negative values included), so
// that unsigned comparison of the result orders the floats.
__host__ __device__ inline uint32_t float_key(float f) {
#ifdef __CUDA_ARCH__
  uint32_t u = __float_as_uint(f);
#else
  uint32_t u;
  memcpy(&u, &f, 4);
#endif
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

__host__ __device__ inline float key_float(uint32_t k) {
  uint32_t u = (k & 0x80000000u) ? (k & 0x7fffffffu) : ~k;
#ifdef __CUDA_ARCH__
  return __uint_as_float(u);
#else
  float f;
  memcpy(&f, &u, 4);
  return f;
#endif
}

inline int grid_for(int64_t n, int block, int64_t cap = 1 << 30) {
  int64_t g = (n + block - 1) / block;
  if (g < 1) g = 1;
  if (g > cap) g = cap;
  return (int)g;
}

int sm_count();

// Runtime tunables (set by the autotuner through spf_tune_set).
int64_t tune_get(int param, int64_t dflt);

// d = a * b + c on two FP32 lanes in one instruction (fma.rn.f32x2, sm_100
// family): each lane is an IEEE round-to-nearest fma, bit-identical to fmaf
__device__ __forceinline__ float2 ffma2(float2 a, float2 b, float2 c) {
  float2 d;
  asm("{\n\t.reg .b64 ra, rb, rc, rd;\n\t"
      "mov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\tmov.b64 rc, {%6, %7};\n\t"
      "fma.rn.f32x2 rd, ra, rb, rc;\n\tmov.b64 {%0, %1}, rd;\n\t}"
      : "=f"(d.x), "=f"(d.y)
      : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y), "f"(c.x), "f"(c.y));
  return d;
}

// d = a - b on two FP32 lanes in one instruction (sub.rn.f32x2)
__device__ __forceinline__ float2 fsub2(float2 a, float2 b) {
  float2 d;
  asm("{\n\t.reg .b64 ra, rb, rd;\n\t"
      "mov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\t"
      "sub.rn.f32x2 rd, ra, rb;\n\tmov.b64 {%0, %1}, rd;\n\t}"
      : "=f"(d.x), "=f"(d.y)
      : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
  return d;
}

}  // namespace spf
