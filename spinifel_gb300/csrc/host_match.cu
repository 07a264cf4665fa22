// Batch matching from host memory in one call: the drop-in for the
// reference's synchronous slicing_and_match matching step
// (spinifel/sequential/orientation_matching.py:113-186), which takes host
// frames and returns host indices, with the copies overlapped by the work.
//
// The frames are split into chunks (2,560 frames by default).  A copy stream
// moves the chunks host -> device one after another, an ingest stream turns
// each landed chunk into FP32, bf16 and norms, and the caller's stream runs
// the bf16 tcgen05 top-8 and the exact FP32 re-rank of each chunk in order.
// The copies (211 GB/s from pinned memory on GB300) and the ingest (a
// bandwidth-bound pass that shares the SMs with the one-CTA-per-SM GEMM) of
// chunk k + 1 run under the GEMM of chunk k, so only the first chunk's copy
// and ingest are exposed.  The GEMMs stay on one stream: two GEMMs that run
// at once stream the references twice and fall off the tensor roofline.
// Chunks may also double from a small first chunk; over 1e5 references that
// is slower (every chunk streams all references once).
// Each chunk keeps its per-tile candidate lists; the frames the certificate
// leaves open are completed at the end in one pass over all chunks (their
// in-band list entries re-ranked exactly; no second pass over the references
// unless a tile list may hide one); indices and distances are copied back.
// Scratch comes from the device's stream-ordered pool (cudaMallocAsync),
// whose release threshold is raised once so that repeated calls reuse the
// memory.
#include <algorithm>
#include <mutex>
#include <vector>

#include "common.cuh"

namespace {

struct Scratch {
  cudaStream_t s;
  std::vector<void *> bufs;
  int st = SPF_OK;
  explicit Scratch(cudaStream_t stream) : s(stream) {}
  template <class T>
  T *get(size_t bytes) {
    void *p = nullptr;
    if (st == SPF_OK)
      st = spf::check_cuda(cudaMallocAsync(&p, std::max<size_t>(bytes, 16), s),
                           "spf_match_bf16_host: cudaMallocAsync");
    if (p) bufs.push_back(p);
    return static_cast<T *>(p);
  }
  ~Scratch() {
    for (void *p : bufs) cudaFreeAsync(p, s);
  }
};

void keep_pool_memory(int dev) {
  static std::mutex mu;
  static bool done[64] = {false};
  std::lock_guard<std::mutex> lk(mu);
  if (dev < 0 || dev >= 64 || done[dev]) return;
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
    uint64_t keep = UINT64_MAX;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
  }
  done[dev] = true;
}

// Chunks of the batch as (first frame, frames): chunk_frames > 0 fixed
// chunks; 0 fixed chunks of 2,560 frames; < 0 chunks doubling from
// -chunk_frames.  A doubling plan folds a remainder smaller than half a chunk
// into the last chunk.
std::vector<std::pair<int64_t, int64_t>> chunk_plan(int64_t n_img, int64_t chunk_frames) {
  std::vector<std::pair<int64_t, int64_t>> plan;
  const bool grow = chunk_frames < 0;
  int64_t size = chunk_frames > 0 ? chunk_frames : (chunk_frames < 0 ? -chunk_frames : 2560);
  for (int64_t r0 = 0; r0 < n_img;) {
    const int64_t rem = n_img - r0;
    int64_t n = std::min(size, rem);
    if (grow && rem - n < n / 2) n = rem;
    plan.emplace_back(r0, n);
    r0 += n;
    if (grow && size < (int64_t(1) << 40)) size *= 2;
  }
  return plan;
}

}  // namespace

extern "C" int spf_match_bf16_host(const uint16_t *h_counts, int64_t n_img,
                                   const void *d_ref_bf16, const float *d_ref,
                                   const float *d_ref_sq, const float *d_ref_m2, float ref_sq_max,
                                   int64_t n_ref, int64_t n_pix, int64_t ld,
                                   int64_t chunk_frames, int32_t *h_idx, float *h_dist,
                                   int64_t *h_stats, void *stream) {
  SPF_REQUIRE(n_img >= 0 && n_ref > 0 && n_pix > 0 && ld >= n_pix && ld % 8 == 0,
              "spf_match_bf16_host: bad sizes");
  if (h_stats) h_stats[0] = h_stats[1] = h_stats[2] = 0;
  if (n_img == 0) return SPF_OK;
  SPF_REQUIRE(h_counts && d_ref_bf16 && d_ref && d_ref_sq && d_ref_m2 && h_idx,
              "spf_match_bf16_host: NULL pointer");
  SPF_REQUIRE(chunk_frames >= -(int64_t(1) << 30), "spf_match_bf16_host: bad chunk_frames");
  const std::vector<std::pair<int64_t, int64_t>> plan = chunk_plan(n_img, chunk_frames);
  const int64_t n_chunks = (int64_t)plan.size();
  SPF_REQUIRE(n_chunks <= 4096, "spf_match_bf16_host: more than 4096 chunks");
  int dev = 0;
  cudaGetDevice(&dev);
  keep_pool_memory(dev);
  cudaStream_t s = spf::as_stream(stream);
  void *sv = s;
  const int64_t tiles = spf_dist_topk_bf16_tiles(n_ref);
  int st = SPF_OK;
  cudaStream_t cs = nullptr, is = nullptr;
  std::vector<cudaEvent_t> ev;
  auto new_event = [&](cudaEvent_t *e) {
    *e = nullptr;
    if (st == SPF_OK)
      st = spf::check_cuda(cudaEventCreateWithFlags(e, cudaEventDisableTiming),
                           "spf_match_bf16_host");
    if (*e) ev.push_back(*e);
  };
  // chunk k's tile lists start at frame offset r0 of the candidate arrays
  auto cand_at = [&](auto *base, int64_t k) { return base + (size_t)tiles * plan[k].first * 8; };
  {
    Scratch W(s);
    uint16_t *u16 = W.get<uint16_t>((size_t)n_img * n_pix * 2);
    float *f32 = W.get<float>((size_t)n_img * n_pix * 4);
    char *bf16 = W.get<char>((size_t)n_img * ld * 2);
    float *sq = W.get<float>(n_img * 4);
    float *work = W.get<float>(n_img * 4), *dist = W.get<float>(n_img * 4);
    int32_t *idx = W.get<int32_t>(n_img * 4), *unc = W.get<int32_t>(n_img * 4);
    // every chunk keeps its tile lists for the completion of its open frames
    float *cand_d = W.get<float>((size_t)tiles * n_img * 8 * 4);
    int32_t *cand_i = W.get<int32_t>((size_t)tiles * n_img * 8 * 4);
    float *mrg_d = W.get<float>((size_t)n_img * 8 * 4);
    int32_t *mrg_i = W.get<int32_t>((size_t)n_img * 8 * 4);
    st = W.st;
    for (cudaStream_t *x : {&cs, &is})
      if (st == SPF_OK)
        st = spf::check_cuda(cudaStreamCreateWithFlags(x, cudaStreamNonBlocking),
                             "spf_match_bf16_host");
    // the scratch above is ordered on s; the other streams must not run ahead of it
    cudaEvent_t ready;
    new_event(&ready);
    if (st == SPF_OK) st = spf::check_cuda(cudaEventRecord(ready, s), "spf_match_bf16_host");
    for (cudaStream_t x : {cs, is})
      if (st == SPF_OK)
        st = spf::check_cuda(cudaStreamWaitEvent(x, ready, 0), "spf_match_bf16_host");
    for (int64_t k = 0; k < n_chunks && st == SPF_OK; ++k) {
      const int64_t r0 = plan[k].first, n = plan[k].second;
      cudaEvent_t copied, ingested;
      new_event(&copied);
      new_event(&ingested);
      if (st == SPF_OK)
        st = spf::check_cuda(cudaMemcpyAsync(u16 + r0 * n_pix, h_counts + r0 * n_pix,
                                             (size_t)n * n_pix * 2, cudaMemcpyHostToDevice, cs),
                             "spf_match_bf16_host: frames to device");
      if (st == SPF_OK) st = spf::check_cuda(cudaEventRecord(copied, cs), "spf_match_bf16_host");
      if (st == SPF_OK)
        st = spf::check_cuda(cudaStreamWaitEvent(is, copied, 0), "spf_match_bf16_host");
      if (st == SPF_OK)
        st = spf_frames_ingest_u16(u16 + r0 * n_pix, n, n_pix, f32 + r0 * n_pix, bf16 + r0 * ld * 2,
                                   ld, sq + r0, nullptr, is);
      if (st == SPF_OK) st = spf::check_cuda(cudaEventRecord(ingested, is), "spf_match_bf16_host");
      if (st == SPF_OK)
        st = spf::check_cuda(cudaStreamWaitEvent(s, ingested, 0), "spf_match_bf16_host");
      if (st == SPF_OK)
        st = spf_dist_topk_bf16(bf16 + r0 * ld * 2, n, d_ref_bf16, n_ref, n_pix, ld, d_ref_sq,
                                cand_at(cand_d, k), cand_at(cand_i, k), sv);
      if (st == SPF_OK)
        st = spf_rerank_fp32_keep(cand_at(cand_d, k), cand_at(cand_i, k), tiles, f32 + r0 * n_pix,
                                  sq + r0, n, d_ref, d_ref_sq, d_ref_m2, ref_sq_max, n_ref, n_pix,
                                  0, work + r0, idx + r0, dist + r0, unc + r0, mrg_d + r0 * 8,
                                  mrg_i + r0 * 8, sv);
    }
    // the caller's stream waits for everything queued on the copy and ingest
    // streams, also after an error, so that no copy can outlive the scratch
    // (whose frees are ordered on s) or the caller's host buffer
    for (cudaStream_t x : {cs, is}) {
      cudaEvent_t joined = nullptr;
      if (x && cudaEventCreateWithFlags(&joined, cudaEventDisableTiming) == cudaSuccess) {
        ev.push_back(joined);
        if (cudaEventRecord(joined, x) == cudaSuccess) cudaStreamWaitEvent(s, joined, 0);
      }
    }
    // results and the open frames back to the host
    std::vector<int32_t> h_unc(n_img);
    std::vector<float> h_d(h_dist ? 0 : n_img);
    float *dist_out = h_dist ? h_dist : h_d.data();
    if (st == SPF_OK)
      st = spf::check_cuda(cudaMemcpyAsync(h_idx, idx, n_img * 4, cudaMemcpyDeviceToHost, s),
                           "spf_match_bf16_host");
    if (st == SPF_OK)
      st = spf::check_cuda(cudaMemcpyAsync(dist_out, dist, n_img * 4, cudaMemcpyDeviceToHost, s),
                           "spf_match_bf16_host");
    if (st == SPF_OK)
      st = spf::check_cuda(cudaMemcpyAsync(h_unc.data(), unc, n_img * 4, cudaMemcpyDeviceToHost, s),
                           "spf_match_bf16_host");
    if (st == SPF_OK) st = spf::check_cuda(cudaStreamSynchronize(s), "spf_match_bf16_host");
    int64_t n_bad = 0, n_range = 0, n_plain = 0;
    // completion of the open frames of all chunks in one pass: each chunk's
    // kept tile lists are scanned into one list array, then one exact
    // re-rank over every open frame; a frame whose tile lists may hide
    // references is completed by spf_complete_open (range GEMM, plain pass)
    constexpr int CAP = 512;
    std::vector<int64_t> rows_g, rows_l, off(n_chunks + 1, 0);
    for (int64_t k = 0; k < n_chunks; ++k) {
      const int64_t r0 = plan[k].first, n = plan[k].second;
      off[k] = (int64_t)rows_g.size();
      for (int64_t i = 0; i < n; ++i)
        if (h_unc[r0 + i]) {
          rows_g.push_back(r0 + i);
          rows_l.push_back(i);
        }
    }
    off[n_chunks] = (int64_t)rows_g.size();
    const int64_t nb = (int64_t)rows_g.size();
    n_bad = nb;
    if (st == SPF_OK && nb > 0) {
      Scratch C(s);
      int64_t *d_rg = C.get<int64_t>(nb * 8), *d_rl = C.get<int64_t>(nb * 8);
      float *f32_c = C.get<float>((size_t)nb * n_pix * 4);
      float *sq_c = C.get<float>(nb * 4), *thr_c = C.get<float>(nb * 4);
      int32_t *lst = C.get<int32_t>((size_t)nb * CAP * 4), *cnt = C.get<int32_t>(nb * 4);
      uint64_t *best = C.get<uint64_t>(nb * 8);
      int32_t *idx2 = C.get<int32_t>(nb * 4);
      float *dist2 = C.get<float>(nb * 4);
      st = C.st;
      std::vector<int32_t> h_i2(nb), h_cnt(nb);
      std::vector<float> h_d2(nb);
      if (st == SPF_OK)
        st = spf::check_cuda(cudaMemcpyAsync(d_rg, rows_g.data(), nb * 8, cudaMemcpyHostToDevice, s),
                             "spf_match_bf16_host");
      if (st == SPF_OK)
        st = spf::check_cuda(cudaMemcpyAsync(d_rl, rows_l.data(), nb * 8, cudaMemcpyHostToDevice, s),
                             "spf_match_bf16_host");
      if (st == SPF_OK) st = spf_gather_rows(f32, n_img, n_pix * 4, d_rg, nb, f32_c, sv);
      if (st == SPF_OK) st = spf_gather_rows(sq, n_img, 4, d_rg, nb, sq_c, sv);
      if (st == SPF_OK) st = spf_gather_rows(work, n_img, 4, d_rg, nb, thr_c, sv);
      for (int64_t k = 0; st == SPF_OK && k < n_chunks; ++k) {
        const int64_t nk = off[k + 1] - off[k];
        if (!nk) continue;
        const int64_t n = plan[k].second;
        st = spf_scan_band_bf16(cand_at(cand_d, k), cand_at(cand_i, k), tiles, n, d_rl + off[k], nk,
                                thr_c + off[k], lst + off[k] * CAP, cnt + off[k], CAP, sv);
      }
      if (st == SPF_OK) st = spf_best_init(best, nb, sv);
      if (st == SPF_OK)
        st = spf_rerank_list_fp32(lst, cnt, CAP, f32_c, sq_c, nb, d_ref, d_ref_sq, n_pix, 0, best,
                                  sv);
      if (st == SPF_OK) st = spf_best_unpack(best, nb, idx2, dist2, sv);
      if (st == SPF_OK)
        st = spf::check_cuda(cudaMemcpyAsync(h_i2.data(), idx2, nb * 4, cudaMemcpyDeviceToHost, s),
                             "spf_match_bf16_host");
      if (st == SPF_OK)
        st = spf::check_cuda(cudaMemcpyAsync(h_d2.data(), dist2, nb * 4, cudaMemcpyDeviceToHost, s),
                             "spf_match_bf16_host");
      if (st == SPF_OK)
        st = spf::check_cuda(cudaMemcpyAsync(h_cnt.data(), cnt, nb * 4, cudaMemcpyDeviceToHost, s),
                             "spf_match_bf16_host");
      if (st == SPF_OK) st = spf::check_cuda(cudaStreamSynchronize(s), "spf_match_bf16_host");
      for (int64_t j = 0; st == SPF_OK && j < nb; ++j)
        if (h_cnt[j] <= CAP) {
          h_idx[rows_g[j]] = h_i2[j];
          dist_out[rows_g[j]] = h_d2[j];
        }
      // the rare frames whose tile lists may hide references, per chunk
      for (int64_t k = 0; st == SPF_OK && k < n_chunks; ++k) {
        const int64_t r0 = plan[k].first, n = plan[k].second;
        std::vector<int64_t> ov;
        for (int64_t j = off[k]; j < off[k + 1]; ++j)
          if (h_cnt[j] > CAP) ov.push_back(rows_l[j]);
        if (ov.empty()) continue;
        const int64_t no = (int64_t)ov.size();
        int64_t hs[3] = {0, 0, 0};
        std::vector<int32_t> o_i(no);
        std::vector<float> o_d(no);
        st = spf::check_cuda(cudaMemcpyAsync(d_rl, ov.data(), no * 8, cudaMemcpyHostToDevice, s),
                             "spf_match_bf16_host");
        if (st == SPF_OK)
          st = spf_complete_open(cand_at(cand_d, k), cand_at(cand_i, k), tiles, bf16 + r0 * ld * 2,
                                 f32 + r0 * n_pix, sq + r0, work + r0, n, d_rl, no, d_ref_bf16,
                                 d_ref, d_ref_sq, n_ref, n_pix, ld, idx2, dist2, hs, sv);
        if (st == SPF_OK)
          st = spf::check_cuda(cudaMemcpyAsync(o_i.data(), idx2, no * 4, cudaMemcpyDeviceToHost, s),
                               "spf_match_bf16_host");
        if (st == SPF_OK)
          st = spf::check_cuda(cudaMemcpyAsync(o_d.data(), dist2, no * 4, cudaMemcpyDeviceToHost, s),
                               "spf_match_bf16_host");
        if (st == SPF_OK) st = spf::check_cuda(cudaStreamSynchronize(s), "spf_match_bf16_host");
        for (int64_t j = 0; st == SPF_OK && j < no; ++j) {
          h_idx[r0 + ov[j]] = o_i[j];
          dist_out[r0 + ov[j]] = o_d[j];
        }
        n_range += hs[0];
        n_plain += hs[1];
      }
    }
    if (h_stats) {
      h_stats[0] = n_bad;
      h_stats[1] = n_range;
      h_stats[2] = n_plain;
    }
  }
  cudaStreamSynchronize(s);  // the scratch frees are ordered before the streams go
  for (cudaEvent_t e : ev) cudaEventDestroy(e);
  for (cudaStream_t x : {cs, is})
    if (x) cudaStreamDestroy(x);
  return st;
}
