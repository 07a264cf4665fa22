// Library-wide state: error text, launch counter, device error word.
#include <stdarg.h>
#include <string.h>

#include <mutex>

#include "common.cuh"

namespace spf {

static thread_local char t_error[1024] = "";
std::atomic<uint64_t> g_launches{0};

void set_error(const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(t_error, sizeof(t_error), fmt, ap);
  va_end(ap);
}

const char *get_error() { return t_error; }

// One error word per device, in device memory, allocated on first use.
static std::mutex g_err_mu;
static unsigned int *g_err_words[64] = {nullptr};

unsigned int *device_error_word() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
  std::lock_guard<std::mutex> lk(g_err_mu);
  if (!g_err_words[dev]) {
    void *p = nullptr;
    if (cudaMalloc(&p, sizeof(unsigned int)) != cudaSuccess) return nullptr;
    cudaMemset(p, 0, sizeof(unsigned int));
    g_err_words[dev] = static_cast<unsigned int *>(p);
  }
  return g_err_words[dev];
}

static std::atomic<int64_t> g_tune[16];
static std::atomic<bool> g_tune_set[16];

int64_t tune_get(int param, int64_t dflt) {
  if (param <= 0 || param >= 16 || !g_tune_set[param].load()) return dflt;
  return g_tune[param].load();
}

int sm_count() {
  static int cached[64] = {0};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) return 152;
  if (!cached[dev]) {
    int n = 0;
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    cached[dev] = n > 0 ? n : 152;
  }
  return cached[dev];
}

}  // namespace spf

extern "C" {

const char *spf_version(void) { return "spinifel_gb300 0.1 (sm_103a)"; }

const char *spf_status_string(int status) {
  switch (status) {
    case SPF_OK: return "ok";
    case SPF_ERR_ARG: return "bad argument";
    case SPF_ERR_OOM: return "out of device memory";
    case SPF_ERR_TIMEOUT: return "device wait timed out";
    case SPF_ERR_LAUNCH: return "kernel launch failed";
    case SPF_ERR_CUDA: return "CUDA error";
    case SPF_ERR_UNSUPPORTED: return "unsupported";
    default: return "unknown status";
  }
}

const char *spf_last_error(void) { return spf::get_error(); }

uint64_t spf_launch_count(void) { return spf::g_launches.load(); }

int spf_tune_set(int param, int64_t value) {
  SPF_REQUIRE(param >= 1 && param <= 7, "spf_tune_set: unknown parameter %d", param);
  if (param == SPF_TUNE_STATIC_ABORT_TEST)
    SPF_REQUIRE(value == 0 || value == 1, "spf_tune_set: the abort test switch is 0 or 1");
  if (param == SPF_TUNE_PRIME_DFT)
    SPF_REQUIRE(value >= 0 && value <= 2, "spf_tune_set: prime DFT choice is 0, 1 or 2");
  if (param == SPF_TUNE_SLICE_SHAPE)
    SPF_REQUIRE(value >= 0 && value <= 7, "spf_tune_set: slicing tile shape is 0 .. 7");
  if (param == SPF_TUNE_SORT_ITEM)
    SPF_REQUIRE(value == 0 || (value >= 256 && value <= 8192),
                "spf_tune_set: sort item size is 256 .. 8192 (0 = default)");
  if (param == SPF_TUNE_BF16_GROUP_M || param == SPF_TUNE_FP32_GROUP_M)
    SPF_REQUIRE(value >= 0 && value <= 1024, "spf_tune_set: group size out of range");
  if (param == SPF_TUNE_BF16_GRID)
    SPF_REQUIRE(value >= 0 && value <= 4096, "spf_tune_set: grid size out of range");
  if (value == 0) {
    spf::g_tune_set[param].store(false);
  } else {
    spf::g_tune[param].store(value);
    spf::g_tune_set[param].store(true);
  }
  return SPF_OK;
}

int spf_tune_get(int param, int64_t *value) {
  SPF_REQUIRE(param >= 1 && param <= 7 && value, "spf_tune_get: bad arguments");
  *value = spf::tune_get(param, 0);
  return SPF_OK;
}

int spf_device_error(void *stream, int *h_code) {
  SPF_REQUIRE(h_code != nullptr, "spf_device_error: h_code is NULL");
  unsigned int *w = spf::device_error_word();
  if (!w) {
    spf::set_error("spf_device_error: no device error word");
    return SPF_ERR_CUDA;
  }
  unsigned int v = 0, sv = 0;
  cudaStream_t s = spf::as_stream(stream);
  // the static matching path keeps its own word (it may not allocate)
  unsigned int *ws = spf::static_match_error_word();
  SPF_TRY(spf::check_cuda(cudaMemcpyAsync(&v, w, sizeof(v), cudaMemcpyDeviceToHost, s),
                          "spf_device_error"));
  if (ws)
    SPF_TRY(spf::check_cuda(cudaMemcpyAsync(&sv, ws, sizeof(sv), cudaMemcpyDeviceToHost, s),
                            "spf_device_error"));
  SPF_TRY(spf::check_cuda(cudaStreamSynchronize(s), "spf_device_error"));
  SPF_TRY(spf::check_cuda(cudaMemsetAsync(w, 0, sizeof(unsigned int), s), "spf_device_error"));
  if (ws)
    SPF_TRY(spf::check_cuda(cudaMemsetAsync(ws, 0, sizeof(unsigned int), s), "spf_device_error"));
  *h_code = (int)(v ? v : sv);
  return SPF_OK;
}

}  // extern "C"
