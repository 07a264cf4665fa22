// Native continuous-batching orientation server (C ABI spf_serve_*).
//
// The reference matches frames in one synchronous loop per MPI rank
// (spinifel/sequential/orientation_matching.py:113-186 called from
// spinifel/mpi/main.py:151-279); streaming use needs a server that keeps the
// references resident and batches whatever has arrived.  One host thread per
// server admits queued requests FIFO into a free slot (frame capacity and an
// HBM budget permitting), launches the slot's work on the slot's own stream
// (copy in, ingest, bf16 tcgen05 top-8 + exact FP32 re-rank, copy out) and
// polls the slots' events, so the copies and re-rank of one slot overlap the
// tensor-core work of another.  Frames the re-rank certificate leaves open
// get the certified completion (the in-band references of the kept per-tile
// candidate lists re-ranked exactly; the range GEMM and the plain pass only
// where those lists may hide references) before their request is delivered.  A frame's result depends only on that frame
// and the references, so batching never changes an answer.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "common.cuh"

namespace spf {
namespace {

constexpr int kRangeCap = 512;

double steady_seconds() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch())
      .count();
}

struct Request {
  int64_t ticket = 0;
  const uint16_t *h_counts = nullptr;
  int64_t n = 0;
  int32_t *h_idx = nullptr;
  float *h_dist = nullptr;
  double arrival = 0.0;
  bool pinned = false;
  bool done = false;
  int status = SPF_OK;
  std::string msg;
};

struct Slot {
  cudaStream_t stream = nullptr;
  cudaEvent_t ev_start = nullptr, ev_done = nullptr;
  int64_t cap = 0;
  // device buffers
  uint16_t *u16 = nullptr;
  float *f32 = nullptr, *sq = nullptr, *n4 = nullptr;
  void *bf16 = nullptr;
  float *cand_d = nullptr, *work = nullptr, *dist = nullptr, *mrg_d = nullptr;
  int32_t *cand_i = nullptr, *idx = nullptr, *unc = nullptr, *mrg_i = nullptr;
  uint64_t *best = nullptr;
  int64_t *rows = nullptr;
  float *f32_c = nullptr, *sq_c = nullptr, *thr_c = nullptr, *dist2 = nullptr;
  int32_t *lst = nullptr, *cnt = nullptr, *idx2 = nullptr;
  // pinned host buffers
  uint16_t *h_stage = nullptr;
  int32_t *h_idx = nullptr, *h_unc = nullptr, *h_idx2 = nullptr, *h_cnt = nullptr;
  float *h_dist = nullptr, *h_dist2 = nullptr;
  int64_t *h_rows = nullptr;
  unsigned int *h_err = nullptr;
  // the batch in flight
  std::vector<Request *> reqs;
  int64_t n = 0, bytes = 0;
  int stage = 0;  // 0 free, 1 matching, 2 completing uncertified frames
  std::vector<int64_t> bad;
};

}  // namespace

struct Server {
  int device = 0;
  int path = 0;  // 0 bf16 tensor cores + re-rank, 1 plain FP32
  const void *ref_bf16 = nullptr;
  const float *ref = nullptr, *ref_sq = nullptr, *ref_m2 = nullptr;
  float ref_sq_max = 0.f;
  int64_t n_ref = 0, n_pix = 0, ld = 0, tiles = 0, slot_frames = 0;
  int64_t per_frame_bytes = 0, budget = 0, in_use = 0;
  unsigned int *err_word = nullptr;

  std::vector<std::unique_ptr<Slot>> slots;
  std::deque<Slot *> free_slots;
  std::vector<Slot *> busy;  // server thread only
  std::deque<Request *> pending;
  std::unordered_map<int64_t, Request *> tickets;
  std::vector<double> latencies_ms;
  int64_t next_ticket = 1;
  double stat[8] = {0};  // requests, frames, launches, uncertified, overflow, gpu ms, budget waits

  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  bool stop = false;
  std::thread thread;

  ~Server();
  int alloc_slot(Slot &s);
  void free_slot(Slot &s);
  std::vector<Slot *> admit();  // under mu
  int launch(Slot &s);
  int complete_stage1(Slot &s, bool *finished);
  int complete_stage2(Slot &s);
  void deliver(Slot &s, int status, const char *msg);  // takes mu
  void run();
};

namespace {

template <class T>
int dev_alloc(T **p, size_t n) {
  void *v = nullptr;
  int st = check_cuda(cudaMalloc(&v, std::max<size_t>(n, 1)), "spf_serve_create: cudaMalloc");
  *p = static_cast<T *>(v);
  return st;
}

template <class T>
int host_alloc(T **p, size_t n) {
  void *v = nullptr;
  int st = check_cuda(cudaHostAlloc(&v, std::max<size_t>(n, 1), cudaHostAllocDefault),
                      "spf_serve_create: cudaHostAlloc");
  *p = static_cast<T *>(v);
  return st;
}

}  // namespace

int Server::alloc_slot(Slot &s) {
  const int64_t c = slot_frames;
  s.cap = c;
  SPF_TRY(check_cuda(cudaStreamCreateWithFlags(&s.stream, cudaStreamNonBlocking), "spf_serve_create"));
  SPF_TRY(check_cuda(cudaEventCreate(&s.ev_start), "spf_serve_create"));
  SPF_TRY(check_cuda(cudaEventCreate(&s.ev_done), "spf_serve_create"));
  SPF_TRY(dev_alloc(&s.u16, c * n_pix * 2));
  SPF_TRY(dev_alloc(&s.f32, c * n_pix * 4));
  SPF_TRY(dev_alloc(&s.sq, c * 4));
  SPF_TRY(dev_alloc(&s.n4, c * 4));
  SPF_TRY(dev_alloc(&s.bf16, c * ld * 2));
  SPF_TRY(dev_alloc(&s.cand_d, tiles * c * 8 * 4));
  SPF_TRY(dev_alloc(&s.cand_i, tiles * c * 8 * 4));
  SPF_TRY(dev_alloc(&s.mrg_d, c * 8 * 4));
  SPF_TRY(dev_alloc(&s.mrg_i, c * 8 * 4));
  SPF_TRY(dev_alloc(&s.work, c * 4));
  SPF_TRY(dev_alloc(&s.dist, c * 4));
  SPF_TRY(dev_alloc(&s.idx, c * 4));
  SPF_TRY(dev_alloc(&s.unc, c * 4));
  SPF_TRY(dev_alloc(&s.best, c * 8));
  SPF_TRY(dev_alloc(&s.rows, c * 8));
  SPF_TRY(dev_alloc(&s.f32_c, c * n_pix * 4));
  SPF_TRY(dev_alloc(&s.sq_c, c * 4));
  SPF_TRY(dev_alloc(&s.thr_c, c * 4));
  SPF_TRY(dev_alloc(&s.dist2, c * 4));
  SPF_TRY(dev_alloc(&s.idx2, c * 4));
  SPF_TRY(dev_alloc(&s.cnt, c * 4));
  SPF_TRY(dev_alloc(&s.lst, c * kRangeCap * 4));
  SPF_TRY(host_alloc(&s.h_stage, c * n_pix * 2));
  SPF_TRY(host_alloc(&s.h_idx, c * 4));
  SPF_TRY(host_alloc(&s.h_unc, c * 4));
  SPF_TRY(host_alloc(&s.h_idx2, c * 4));
  SPF_TRY(host_alloc(&s.h_cnt, c * 4));
  SPF_TRY(host_alloc(&s.h_dist, c * 4));
  SPF_TRY(host_alloc(&s.h_dist2, c * 4));
  SPF_TRY(host_alloc(&s.h_rows, c * 8));
  SPF_TRY(host_alloc(&s.h_err, 4));
  return SPF_OK;
}

void Server::free_slot(Slot &s) {
  if (s.stream) cudaStreamSynchronize(s.stream);
  void *dev[] = {s.u16, s.f32,  s.sq,    s.n4,   s.bf16, s.cand_d, s.cand_i, s.mrg_d,
                 s.mrg_i, s.work, s.dist, s.idx, s.unc, s.best, s.rows, s.f32_c,
                 s.sq_c, s.thr_c, s.dist2, s.idx2, s.cnt, s.lst};
  for (void *p : dev)
    if (p) cudaFree(p);
  void *host[] = {s.h_stage, s.h_idx, s.h_unc, s.h_idx2, s.h_cnt, s.h_dist, s.h_dist2,
                  s.h_rows, s.h_err};
  for (void *p : host)
    if (p) cudaFreeHost(p);
  if (s.ev_start) cudaEventDestroy(s.ev_start);
  if (s.ev_done) cudaEventDestroy(s.ev_done);
  if (s.stream) cudaStreamDestroy(s.stream);
}

Server::~Server() {
  for (auto &s : slots) free_slot(*s);
  for (auto &kv : tickets) delete kv.second;  // every queued request also has a ticket
}

std::vector<Slot *> Server::admit() {
  std::vector<Slot *> out;
  while (!free_slots.empty() && !pending.empty()) {
    Slot *s = free_slots.front();
    int64_t n = 0, bytes = 0;
    s->reqs.clear();
    while (!pending.empty()) {
      Request *r = pending.front();
      int64_t need = r->n * per_frame_bytes;
      if (n + r->n > s->cap || in_use + bytes + need > budget) break;
      pending.pop_front();
      s->reqs.push_back(r);
      n += r->n;
      bytes += need;
    }
    if (s->reqs.empty()) {
      stat[6] += 1;
      break;
    }
    free_slots.pop_front();
    s->n = n;
    s->bytes = bytes;
    in_use += bytes;
    out.push_back(s);
  }
  return out;
}

int Server::launch(Slot &s) {
  cudaStream_t st = s.stream;
  void *sv = st;
  SPF_TRY(check_cuda(cudaEventRecord(s.ev_start, st), "spf_serve: event"));
  int64_t row = 0;
  for (Request *r : s.reqs) {
    const size_t bytes = (size_t)(r->n * n_pix * 2);
    const void *src = r->h_counts;
    if (!r->pinned) {  // pageable input: through the slot's pinned staging rows
      memcpy(s.h_stage + row * n_pix, r->h_counts, bytes);
      src = s.h_stage + row * n_pix;
    }
    SPF_TRY(check_cuda(cudaMemcpyAsync(s.u16 + row * n_pix, src, bytes, cudaMemcpyHostToDevice, st),
                       "spf_serve: frames to device"));
    row += r->n;
  }
  const int64_t n = s.n;
  SPF_TRY(spf_frames_ingest_u16(s.u16, n, n_pix, s.f32, s.bf16, ld, s.sq, nullptr, sv));
  if (path == 0) {
    SPF_TRY(spf_dist_topk_bf16(s.bf16, n, ref_bf16, n_ref, n_pix, ld, ref_sq, s.cand_d, s.cand_i,
                               sv));
    SPF_TRY(spf_rerank_fp32_keep(s.cand_d, s.cand_i, tiles, s.f32, s.sq, n, ref, ref_sq, ref_m2,
                                 ref_sq_max, n_ref, n_pix, 0, s.work, s.idx, s.dist, s.unc,
                                 s.mrg_d, s.mrg_i, sv));
    SPF_TRY(check_cuda(cudaMemcpyAsync(s.h_unc, s.unc, n * 4, cudaMemcpyDeviceToHost, st),
                       "spf_serve: flags to host"));
  } else {
    SPF_TRY(spf_best_init(s.best, n, sv));
    SPF_TRY(spf_dist_argmin_f32(s.f32, s.sq, n, ref, ref_sq, n_ref, n_pix, 0, s.best, sv));
    SPF_TRY(spf_best_unpack(s.best, n, s.idx, s.dist, sv));
    memset(s.h_unc, 0, n * 4);
  }
  SPF_TRY(check_cuda(cudaMemcpyAsync(s.h_idx, s.idx, n * 4, cudaMemcpyDeviceToHost, st),
                     "spf_serve: indices to host"));
  SPF_TRY(check_cuda(cudaMemcpyAsync(s.h_dist, s.dist, n * 4, cudaMemcpyDeviceToHost, st),
                     "spf_serve: distances to host"));
  SPF_TRY(check_cuda(cudaMemcpyAsync(s.h_err, err_word, 4, cudaMemcpyDeviceToHost, st),
                     "spf_serve: error word"));
  SPF_TRY(check_cuda(cudaEventRecord(s.ev_done, st), "spf_serve: event"));
  s.stage = 1;
  return SPF_OK;
}

// Stage 1 landed on the host: enqueue the certified completion of the open
// frames from the kept tile lists (no host wait) or report the slot finished.
int Server::complete_stage1(Slot &s, bool *finished) {
  float ms = 0.f;
  if (cudaEventElapsedTime(&ms, s.ev_start, s.ev_done) == cudaSuccess) {
    std::lock_guard<std::mutex> g(mu);
    stat[5] += ms;
  }
  s.bad.clear();
  for (int64_t i = 0; i < s.n; ++i)
    if (s.h_unc[i]) s.bad.push_back(i);
  if (s.bad.empty()) {
    *finished = true;
    return SPF_OK;
  }
  *finished = false;
  cudaStream_t st = s.stream;
  void *sv = st;
  const int64_t nb = (int64_t)s.bad.size();
  std::copy(s.bad.begin(), s.bad.end(), s.h_rows);
  SPF_TRY(check_cuda(cudaMemcpyAsync(s.rows, s.h_rows, nb * 8, cudaMemcpyHostToDevice, st),
                     "spf_serve: rows to device"));
  SPF_TRY(spf_gather_rows(s.f32, s.n, n_pix * 4, s.rows, nb, s.f32_c, sv));
  SPF_TRY(spf_gather_rows(s.sq, s.n, 4, s.rows, nb, s.sq_c, sv));
  SPF_TRY(spf_gather_rows(s.work, s.n, 4, s.rows, nb, s.thr_c, sv));
  // every in-bound reference from the kept tile lists of the matching pass
  SPF_TRY(spf_scan_band_bf16(s.cand_d, s.cand_i, tiles, s.n, s.rows, nb, s.thr_c, s.lst, s.cnt,
                             kRangeCap, sv));
  SPF_TRY(spf_best_init(s.best, nb, sv));
  SPF_TRY(spf_rerank_list_fp32(s.lst, s.cnt, kRangeCap, s.f32_c, s.sq_c, nb, ref, ref_sq, n_pix,
                               0, s.best, sv));
  SPF_TRY(spf_best_unpack(s.best, nb, s.idx2, s.dist2, sv));
  SPF_TRY(check_cuda(cudaMemcpyAsync(s.h_idx2, s.idx2, nb * 4, cudaMemcpyDeviceToHost, st),
                     "spf_serve: completion to host"));
  SPF_TRY(check_cuda(cudaMemcpyAsync(s.h_dist2, s.dist2, nb * 4, cudaMemcpyDeviceToHost, st),
                     "spf_serve: completion to host"));
  SPF_TRY(check_cuda(cudaMemcpyAsync(s.h_cnt, s.cnt, nb * 4, cudaMemcpyDeviceToHost, st),
                     "spf_serve: completion to host"));
  SPF_TRY(check_cuda(cudaMemcpyAsync(s.h_err, err_word, 4, cudaMemcpyDeviceToHost, st),
                     "spf_serve: error word"));
  SPF_TRY(check_cuda(cudaEventRecord(s.ev_done, st), "spf_serve: event"));
  s.stage = 2;
  std::lock_guard<std::mutex> g(mu);
  stat[3] += (double)nb;
  return SPF_OK;
}

// Stage 2 landed: fold the list re-rank into the slot's results.  A frame
// whose tile lists may hide references (or whose list is over its cap) is
// completed by spf_complete_open -- the range GEMM, then the plain pass --
// while the server thread waits (rare).
int Server::complete_stage2(Slot &s) {
  const int64_t nb = (int64_t)s.bad.size();
  std::vector<int64_t> over;
  for (int64_t j = 0; j < nb; ++j) {
    if (s.h_cnt[j] > kRangeCap) {
      over.push_back(s.bad[j]);
    } else {
      s.h_idx[s.bad[j]] = s.h_idx2[j];
      s.h_dist[s.bad[j]] = s.h_dist2[j];
    }
  }
  if (over.empty()) return SPF_OK;
  cudaStream_t st = s.stream;
  void *sv = st;
  const int64_t no = (int64_t)over.size();
  for (int64_t k = 0; k < no; ++k) s.h_rows[k] = over[k];
  SPF_TRY(check_cuda(cudaMemcpyAsync(s.rows, s.h_rows, no * 8, cudaMemcpyHostToDevice, st),
                     "spf_serve: rows to device"));
  int64_t hs[3];
  SPF_TRY(spf_complete_open(s.cand_d, s.cand_i, tiles, s.bf16, s.f32, s.sq, s.work, s.n, s.rows,
                            no, ref_bf16, ref, ref_sq, n_ref, n_pix, ld, s.idx2, s.dist2, hs, sv));
  SPF_TRY(check_cuda(cudaMemcpyAsync(s.h_idx2, s.idx2, no * 4, cudaMemcpyDeviceToHost, st),
                     "spf_serve: completion to host"));
  SPF_TRY(check_cuda(cudaMemcpyAsync(s.h_dist2, s.dist2, no * 4, cudaMemcpyDeviceToHost, st),
                     "spf_serve: completion to host"));
  SPF_TRY(check_cuda(cudaStreamSynchronize(st), "spf_serve: completion"));
  for (int64_t k = 0; k < no; ++k) {
    s.h_idx[over[k]] = s.h_idx2[k];
    s.h_dist[over[k]] = s.h_dist2[k];
  }
  std::lock_guard<std::mutex> g(mu);
  stat[4] += (double)no;
  return SPF_OK;
}

void Server::deliver(Slot &s, int status, const char *msg) {
  const double now = steady_seconds();
  if (status == SPF_OK) {  // results into the callers' buffers before they are told
    int64_t row = 0;
    for (Request *r : s.reqs) {
      if (r->h_idx) memcpy(r->h_idx, s.h_idx + row, r->n * 4);
      if (r->h_dist) memcpy(r->h_dist, s.h_dist + row, r->n * 4);
      row += r->n;
    }
  }
  std::lock_guard<std::mutex> lk(mu);
  for (Request *r : s.reqs) {
    r->status = status;
    if (status != SPF_OK) r->msg = msg ? msg : "spf_serve: request failed";
    r->done = true;
    latencies_ms.push_back((now - r->arrival) * 1e3);
    stat[0] += 1;
    stat[1] += (double)r->n;
  }
  s.reqs.clear();
  in_use -= s.bytes;
  s.n = s.bytes = 0;
  s.stage = 0;
  free_slots.push_back(&s);
  cv_done.notify_all();
}

void Server::run() {
  cudaSetDevice(device);
  std::unique_lock<std::mutex> lk(mu);
  for (;;) {
    if (stop && pending.empty() && busy.empty()) break;
    std::vector<Slot *> launched = admit();
    if (launched.empty() && busy.empty()) {
      cv_work.wait_for(lk, std::chrono::milliseconds(1));
      continue;
    }
    lk.unlock();
    for (Slot *s : launched) {
      int st = launch(*s);
      {
        std::lock_guard<std::mutex> g(mu);
        stat[2] += 1;
      }
      if (st != SPF_OK) {
        std::string m = get_error();
        cudaStreamSynchronize(s->stream);
        deliver(*s, st, m.c_str());
        continue;
      }
      busy.push_back(s);
    }
    std::vector<Slot *> still;
    for (Slot *s : busy) {
      cudaError_t q = cudaEventQuery(s->ev_done);
      if (q == cudaErrorNotReady) {
        still.push_back(s);
        continue;
      }
      int st = q == cudaSuccess ? SPF_OK : check_cuda(q, "spf_serve: stream");
      if (st == SPF_OK && *s->h_err != 0) {
        set_error("spf_serve: device error word %u (a bounded device wait gave up)", *s->h_err);
        st = SPF_ERR_TIMEOUT;
      }
      if (st == SPF_OK && s->stage == 1) {
        bool finished = false;
        st = complete_stage1(*s, &finished);
        if (st == SPF_OK && !finished) {
          still.push_back(s);
          continue;
        }
      } else if (st == SPF_OK) {
        st = complete_stage2(*s);
      }
      std::string m = st == SPF_OK ? std::string() : std::string(get_error());
      if (st != SPF_OK) cudaStreamSynchronize(s->stream);
      deliver(*s, st, m.c_str());
    }
    busy.swap(still);
    if (!busy.empty() && launched.empty()) std::this_thread::sleep_for(std::chrono::microseconds(50));
    lk.lock();
  }
}

}  // namespace spf

// The opaque handle of the C ABI.
struct spf_server_s : spf::Server {};

extern "C" {

double spf_serve_clock(void) { return spf::steady_seconds(); }

int spf_serve_create(int device, const void *d_ref_bf16, const float *d_ref, const float *d_ref_sq,
                     const float *d_ref_m2, float ref_sq_max, int64_t n_ref, int64_t n_pix,
                     int64_t ld, int path, int64_t slot_frames, int n_slots, int64_t hbm_budget,
                     spf_server *out) {
  SPF_REQUIRE(out != nullptr, "spf_serve_create: out is NULL");
  *out = nullptr;
  SPF_REQUIRE(path == 0 || path == 1, "spf_serve_create: path must be 0 (bf16) or 1 (fp32)");
  SPF_REQUIRE(d_ref && d_ref_sq && (path == 1 || (d_ref_bf16 && d_ref_m2)),
              "spf_serve_create: reference buffers are NULL");
  SPF_REQUIRE(n_ref > 0 && n_pix > 0 && ld >= n_pix && ld % 8 == 0,
              "spf_serve_create: bad sizes (n_ref %lld, n_pix %lld, ld %lld)", (long long)n_ref,
              (long long)n_pix, (long long)ld);
  SPF_REQUIRE(slot_frames >= 1 && slot_frames <= 65536 && n_slots >= 1 && n_slots <= 16,
              "spf_serve_create: slot_frames in 1..65536 and n_slots in 1..16");
  SPF_REQUIRE(n_ref <= INT32_MAX, "spf_serve_create: n_ref too large");
  SPF_REQUIRE(device >= 0, "spf_serve_create: bad device");
  SPF_TRY(spf::check_cuda(cudaSetDevice(device), "spf_serve_create"));
  auto srv = std::make_unique<spf_server_s>();
  spf::Server &s = *srv;
  s.device = device;
  s.path = path;
  s.ref_bf16 = d_ref_bf16;
  s.ref = d_ref;
  s.ref_sq = d_ref_sq;
  s.ref_m2 = d_ref_m2;
  s.ref_sq_max = ref_sq_max;
  s.n_ref = n_ref;
  s.n_pix = n_pix;
  s.ld = ld;
  s.tiles = spf_dist_topk_bf16_tiles(n_ref);
  s.slot_frames = slot_frames;
  s.per_frame_bytes = n_pix * (2 + 4) + ld * 2 + 16 + s.tiles * 8 * 8 + 16;
  s.budget = hbm_budget > 0 ? hbm_budget : s.per_frame_bytes * slot_frames * n_slots;
  SPF_REQUIRE(s.budget >= s.per_frame_bytes, "spf_serve_create: HBM budget smaller than one frame");
  s.err_word = spf::device_error_word();
  if (!s.err_word) {
    spf::set_error("spf_serve_create: no device error word");
    return SPF_ERR_CUDA;
  }
  for (int i = 0; i < n_slots; ++i) {
    s.slots.emplace_back(new spf::Slot());
    SPF_TRY(s.alloc_slot(*s.slots.back()));
    s.free_slots.push_back(s.slots.back().get());
  }
  s.thread = std::thread([&s] { s.run(); });
  *out = srv.release();
  return SPF_OK;
}

int spf_serve_submit(spf_server srv, const uint16_t *h_counts, int64_t n_frames, int32_t *h_idx,
                     float *h_dist, double arrival, int64_t *ticket) {
  SPF_REQUIRE(srv && h_counts && ticket, "spf_serve_submit: NULL argument");
  spf::Server &s = *srv;
  SPF_REQUIRE(n_frames >= 1 && n_frames <= s.slot_frames,
              "spf_serve_submit: a request holds 1..%lld frames", (long long)s.slot_frames);
  SPF_REQUIRE(n_frames * s.per_frame_bytes <= s.budget,
              "spf_serve_submit: request larger than the HBM budget");
  auto *r = new spf::Request();
  r->h_counts = h_counts;
  r->n = n_frames;
  r->h_idx = h_idx;
  r->h_dist = h_dist;
  r->arrival = arrival >= 0.0 ? arrival : spf::steady_seconds();
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, h_counts) == cudaSuccess)
    r->pinned = a.type == cudaMemoryTypeHost;
  cudaGetLastError();  // an unregistered pointer is not an error here
  {
    std::lock_guard<std::mutex> lk(s.mu);
    if (s.stop) {
      delete r;
      spf::set_error("spf_serve_submit: server is closing");
      return SPF_ERR_ARG;
    }
    r->ticket = s.next_ticket++;
    s.tickets[r->ticket] = r;
    s.pending.push_back(r);
  }
  s.cv_work.notify_one();
  *ticket = r->ticket;
  return SPF_OK;
}

int spf_serve_wait(spf_server srv, int64_t ticket, int64_t timeout_ms, int *done) {
  SPF_REQUIRE(srv && done, "spf_serve_wait: NULL argument");
  spf::Server &s = *srv;
  *done = 0;
  std::unique_lock<std::mutex> lk(s.mu);
  auto it = s.tickets.find(ticket);
  SPF_REQUIRE(it != s.tickets.end(), "spf_serve_wait: unknown ticket %lld", (long long)ticket);
  spf::Request *r = it->second;
  auto ready = [r] { return r->done; };
  if (timeout_ms < 0) {
    s.cv_done.wait(lk, ready);
  } else if (!s.cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), ready)) {
    return SPF_OK;
  }
  *done = 1;
  int st = r->status;
  if (st != SPF_OK) spf::set_error("%s", r->msg.c_str());
  s.tickets.erase(it);
  delete r;
  return st;
}

int spf_serve_stats(spf_server srv, double *h_out, int n_out) {
  SPF_REQUIRE(srv && h_out && n_out >= 0, "spf_serve_stats: bad arguments");
  spf::Server &s = *srv;
  std::lock_guard<std::mutex> lk(s.mu);
  double v[9];
  for (int i = 0; i < 7; ++i) v[i] = s.stat[i];
  std::vector<double> lat(s.latencies_ms);
  v[7] = v[8] = 0.0;
  if (!lat.empty()) {
    std::sort(lat.begin(), lat.end());
    auto pct = [&lat](double p) {  // linear interpolation between order statistics
      double x = p * (double)(lat.size() - 1);
      size_t i = (size_t)x;
      double f = x - (double)i;
      return i + 1 < lat.size() ? lat[i] * (1.0 - f) + lat[i + 1] * f : lat[i];
    };
    v[7] = pct(0.50);
    v[8] = pct(0.99);
  }
  for (int i = 0; i < n_out && i < 9; ++i) h_out[i] = v[i];
  return SPF_OK;
}

int spf_serve_latencies(spf_server srv, double *h_ms, int64_t cap, int64_t *n) {
  SPF_REQUIRE(srv && n && (cap == 0 || h_ms), "spf_serve_latencies: bad arguments");
  spf::Server &s = *srv;
  std::lock_guard<std::mutex> lk(s.mu);
  *n = (int64_t)s.latencies_ms.size();
  int64_t k = std::min<int64_t>(cap, *n);
  if (k > 0) memcpy(h_ms, s.latencies_ms.data(), k * sizeof(double));
  return SPF_OK;
}

int spf_serve_destroy(spf_server srv) {
  if (!srv) return SPF_OK;
  {
    std::lock_guard<std::mutex> lk(srv->mu);
    srv->stop = true;
  }
  srv->cv_work.notify_all();
  if (srv->thread.joinable()) srv->thread.join();
  delete srv;
  return SPF_OK;
}

}  // extern "C"
