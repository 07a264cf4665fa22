"""Continuous-batching orientation server.

Frames arrive in requests of 1..512 frames.  The server keeps the reference
slices resident in HBM (FP32 for the exact re-rank, bf16 for the tensor
cores) and runs a scheduler thread that

  * admits pending requests into a free *slot* as long as the slot's frame
    capacity and the HBM budget allow (several requests share one launch:
    continuous batching, not a queue of single requests);
  * stages each admitted request's uint16 frames host -> device on the slot's
    own CUDA stream, ingests them (FP32, bf16, norms), runs the bf16 tcgen05
    distance + top-8 kernel and the exact FP32 re-rank, and copies the indices
    back -- so the copies and re-rank of one slot overlap the tensor-core work
    of another;
  * completes requests as their slot's event fires, re-matching exactly
    (plain FP32 over all references) any frame whose certificate failed.

Each frame's result depends only on that frame and the references (the
distance of a frame row never mixes with other rows), so a request gets the
same answer alone or batched with others; tests/test_gpu_serving.py checks
that.  Latency is measured from a request's arrival time to the moment its
result is on the host.
"""
from __future__ import annotations

import collections
import ctypes
import threading
import time
from concurrent.futures import Future
from dataclasses import dataclass, field

import numpy as np
import torch

from . import _lib, matching


@dataclass
class Request:
    frames: torch.Tensor            # [n, n_pix] int16/uint16 bit pattern, pinned host
    arrival: float                  # time.perf_counter() at arrival
    future: Future = field(default_factory=Future)
    n: int = 0
    done_at: float = 0.0


class _Slot:
    def __init__(self, device, cap: int, n_pix: int, ld: int, n_tiles: int):
        self.stream = torch.cuda.Stream(device=device)
        self.cap = cap
        self.u16 = torch.empty(cap, n_pix, dtype=torch.int16, device=device)
        self.frames = matching.FrameSet.__new__(matching.FrameSet)
        self.frames.n_pix, self.frames.ld = n_pix, ld
        self.f32 = torch.empty(cap, n_pix, dtype=torch.float32, device=device)
        self.bf16 = torch.empty(cap, ld, dtype=torch.bfloat16, device=device)
        self.sq = torch.empty(cap, dtype=torch.float32, device=device)
        self.n4 = torch.empty(cap, dtype=torch.float32, device=device)
        self.cand_d = torch.empty(n_tiles * cap * 8, dtype=torch.float32, device=device)
        self.cand_i = torch.empty(n_tiles * cap * 8, dtype=torch.int32, device=device)
        self.idx = torch.empty(cap, dtype=torch.int32, device=device)
        self.dist = torch.empty(cap, dtype=torch.float32, device=device)
        self.unc = torch.empty(cap, dtype=torch.int32, device=device)
        self.work = torch.empty(cap, dtype=torch.float32, device=device)
        self.host_out = torch.empty(2, cap, dtype=torch.int32).pin_memory()
        # completion buffers, allocated once: pinning memory while other work
        # runs on the device can wait for that work
        self.host_rows = torch.empty(cap, dtype=torch.int64).pin_memory()
        self.host_bad = torch.empty(2, cap, dtype=torch.int32).pin_memory()
        self.event = torch.cuda.Event(enable_timing=True)
        self.t_start = torch.cuda.Event(enable_timing=True)
        self.requests: list[Request] = []
        self.n = 0
        self.bytes = 0
        self.stage = 0       # 0 free, 1 matching, 2 completing uncertified frames
        self.result = None
        self.bad = None
        self.keep = None

    def view(self, n):
        fs = self.frames
        fs.n = n
        fs.f32, fs.bf16, fs.sq, fs.n4 = self.f32[:n], self.bf16[:n], self.sq[:n], self.n4[:n]
        return fs


class OrientationServer:
    """Serve orientation requests against resident references.

    refs          : matching.ReferenceSet (resident FP32 + bf16 slices)
    slot_frames   : frame capacity of one launch (a multiple of 128 is best)
    n_slots       : launches that may be in flight at once (each has a stream)
    hbm_budget    : bytes the in-flight slots may use for frames + candidates;
                    a request is admitted only while the total stays within it
    path          : "bf16" (tensor cores + re-rank) or "fp32" (plain path)
    """

    def __init__(self, refs: "matching.ReferenceSet", slot_frames: int = 512, n_slots: int = 3,
                 hbm_budget: int | None = None, path: str = "bf16"):
        self.refs = refs
        self.device = refs.f32.device
        self.path = path
        self.n_pix, self.ld = refs.n_pix, refs.ld
        self.n_tiles = int(_lib.lib().spf_dist_topk_bf16_tiles(refs.n_ref))
        self.slot_frames = slot_frames
        self.per_frame_bytes = (self.n_pix * (2 + 4) + self.ld * 2 + 16 +
                                self.n_tiles * 8 * 8 + 16)
        slot_bytes = self.per_frame_bytes * slot_frames
        self.hbm_budget = hbm_budget if hbm_budget is not None else slot_bytes * n_slots
        if self.hbm_budget < self.per_frame_bytes:
            raise ValueError("HBM budget smaller than one frame")
        self.slots = [_Slot(self.device, slot_frames, self.n_pix, self.ld, self.n_tiles)
                      for _ in range(n_slots)]
        self.free = collections.deque(self.slots)
        self.busy: list[_Slot] = []
        self.pending: collections.deque[Request] = collections.deque()
        self.in_use_bytes = 0
        self.lock = threading.Condition()
        self.stop_flag = False
        self.completed: list[Request] = []
        self.stats = collections.Counter()
        self.thread = threading.Thread(target=self._loop, daemon=True)
        self.thread.start()

    # ---------------------------------------------------------------- client
    def submit(self, frames_u16: torch.Tensor, arrival: float | None = None) -> Future:
        if frames_u16.dim() != 2 or frames_u16.shape[1] != self.n_pix:
            raise ValueError(f"frames must be [n, {self.n_pix}]")
        if frames_u16.dtype not in (torch.int16, torch.uint16):
            raise TypeError("frames must be 16-bit photon counts")
        n = frames_u16.shape[0]
        if n == 0 or n > self.slot_frames:
            raise ValueError(f"a request holds 1..{self.slot_frames} frames")
        if not frames_u16.is_pinned():
            frames_u16 = frames_u16.pin_memory()
        r = Request(frames_u16, arrival if arrival is not None else time.perf_counter(), n=n)
        with self.lock:
            if self.stop_flag:
                raise RuntimeError("server stopped")
            self.pending.append(r)
            self.lock.notify()
        return r.future

    def close(self):
        with self.lock:
            self.stop_flag = True
            self.lock.notify()
        self.thread.join()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # ------------------------------------------------------------- scheduler
    def _admit(self):
        """Fill free slots from the pending queue (FIFO), within the budget."""
        launched = []
        while self.free and self.pending:
            slot = self.free[0]
            take = []
            n = 0
            bytes_ = 0
            while self.pending:
                r = self.pending[0]
                need = r.n * self.per_frame_bytes
                if n + r.n > slot.cap or self.in_use_bytes + bytes_ + need > self.hbm_budget:
                    break
                take.append(self.pending.popleft())
                n += r.n
                bytes_ += need
            if not take:
                self.stats["budget_waits"] += 1
                break
            self.free.popleft()
            slot.requests, slot.n, slot.bytes = take, n, bytes_
            self.in_use_bytes += bytes_
            launched.append(slot)
        return launched

    def _launch(self, slot: _Slot):
        t0 = time.perf_counter()
        with torch.cuda.stream(slot.stream):
            slot.t_start.record(slot.stream)
            row = 0
            for r in slot.requests:
                slot.u16[row:row + r.n].copy_(r.frames, non_blocking=True)
                row += r.n
            n = slot.n
            fs = slot.view(n)
            matching.ingest_u16(slot.u16[:n], fs.f32, fs.bf16, fs.sq, None)
            sh = _lib.stream_handle(slot.stream)
            if self.path == "bf16":
                _lib.call("spf_dist_topk_bf16", _lib.ptr(fs.bf16), n, _lib.ptr(self.refs.bf16),
                          self.refs.n_ref, self.n_pix, self.ld, _lib.ptr(self.refs.sq),
                          _lib.ptr(slot.cand_d[:self.n_tiles * n * 8]),
                          _lib.ptr(slot.cand_i[:self.n_tiles * n * 8]), sh)
                _lib.call("spf_rerank_fp32", _lib.ptr(slot.cand_d[:self.n_tiles * n * 8]),
                          _lib.ptr(slot.cand_i[:self.n_tiles * n * 8]), self.n_tiles,
                          _lib.ptr(fs.f32), _lib.ptr(fs.sq), n,
                          _lib.ptr(self.refs.f32), _lib.ptr(self.refs.sq), _lib.ptr(self.refs.m2),
                          float(self.refs.sq_max), self.refs.n_ref, self.n_pix, 0,
                          _lib.ptr(slot.work[:n]), _lib.ptr(slot.idx[:n]),
                          _lib.ptr(slot.dist[:n]), _lib.ptr(slot.unc[:n]), None, sh)
                slot.host_out[1, :n].copy_(slot.unc[:n], non_blocking=True)
            else:
                best = torch.empty(n, dtype=torch.int64, device=self.device)
                _lib.call("spf_best_init", _lib.ptr(best), n, sh)
                _lib.call("spf_dist_argmin_f32", _lib.ptr(fs.f32), _lib.ptr(fs.sq), n,
                          _lib.ptr(self.refs.f32), _lib.ptr(self.refs.sq), self.refs.n_ref,
                          self.n_pix, 0, _lib.ptr(best), sh)
                _lib.call("spf_best_unpack", _lib.ptr(best), n, _lib.ptr(slot.idx[:n]),
                          _lib.ptr(slot.dist[:n]), sh)
                slot.host_out[1, :n].zero_()
            slot.host_out[0, :n].copy_(slot.idx[:n], non_blocking=True)
            slot.event.record(slot.stream)
        self.stats["launches"] += 1
        self.stats["frames"] += slot.n
        self.stats["t_launch_ms"] += (time.perf_counter() - t0) * 1e3

    def _finish_stage1(self, slot: _Slot) -> bool:
        """Called when a slot's match has landed on the host.  Frames the
        top-8 certificate left open get the certified completion (range query
        on the tensor cores + exact re-rank of the list), enqueued on the
        slot's stream without waiting; returns True when the slot is done."""
        n = slot.n
        slot.result = slot.host_out[0, :n].numpy().copy()
        unc = slot.host_out[1, :n].numpy()
        bad = np.flatnonzero(unc)
        slot.bad = bad
        if not bad.size:
            return True
        t0 = time.perf_counter()
        with torch.cuda.stream(slot.stream):
            nb = int(bad.size)
            slot.host_rows[:nb].copy_(torch.from_numpy(bad.astype(np.int64)))
            rows = slot.host_rows[:nb].to(self.device, non_blocking=True)
            self.stats["t_c_rows_ms"] += (time.perf_counter() - t0) * 1e3
            fs = slot.view(n)
            sh0 = slot.stream
            bf = matching.gather_rows(fs.bf16, rows, stream=sh0)
            f32 = matching.gather_rows(fs.f32, rows, stream=sh0)
            sq = matching.gather_rows(fs.sq.view(-1, 1), rows, stream=sh0).view(-1)
            thresh = matching.gather_rows(slot.work[:n].view(-1, 1), rows, stream=sh0).view(-1)
            cap = matching.RANGE_CAP
            lst = torch.empty(nb * cap, dtype=torch.int32, device=self.device)
            cnt = torch.empty(nb, dtype=torch.int32, device=self.device)
            sh = _lib.stream_handle(slot.stream)
            self.stats["t_c_gather_ms"] += (time.perf_counter() - t0) * 1e3
            _lib.call("spf_dist_range_bf16", _lib.ptr(bf), nb, _lib.ptr(self.refs.bf16),
                      self.refs.n_ref, self.n_pix, self.ld, _lib.ptr(self.refs.sq),
                      _lib.ptr(thresh), _lib.ptr(lst), _lib.ptr(cnt), cap, sh)
            self.stats["t_c_range_ms"] += (time.perf_counter() - t0) * 1e3
            tr = matching.BestTracker(nb, self.device)
            _lib.call("spf_rerank_list_fp32", _lib.ptr(lst), _lib.ptr(cnt), cap, _lib.ptr(f32),
                      _lib.ptr(sq), nb, _lib.ptr(self.refs.f32), _lib.ptr(self.refs.sq),
                      self.n_pix, 0, _lib.ptr(tr.best), sh)
            i2, _ = tr.result()
            slot.host_bad[0, :nb].copy_(i2, non_blocking=True)
            slot.host_bad[1, :nb].copy_(cnt, non_blocking=True)
            slot.keep = (f32, sq)
            slot.event.record(slot.stream)
        self.stats["uncertified"] += int(bad.size)
        self.stats["t_complete_ms"] += (time.perf_counter() - t0) * 1e3
        return False

    def _finish_stage2(self, slot: _Slot):
        nb = int(slot.bad.size)
        idx2 = slot.host_bad[0, :nb].numpy().copy()
        cnt = slot.host_bad[1, :nb].numpy()
        over = np.flatnonzero(cnt > matching.RANGE_CAP)
        if over.size:
            # a list longer than the cap: exact pass over all references (rare)
            f32, sq = slot.keep
            with torch.cuda.stream(slot.stream):
                sel = torch.as_tensor(over, dtype=torch.int64, device=self.device)
                tr = matching.BestTracker(int(over.size), self.device)
                tr.update_fp32(matching.gather_rows(f32, sel),
                               matching.gather_rows(sq.view(-1, 1), sel).view(-1),
                               self.refs.f32, self.refs.sq, 0)
                i3, _ = tr.result()
                idx2 = idx2.copy()
                idx2[over] = i3.cpu().numpy()
            self.stats["range_overflow"] += int(over.size)
        slot.result[slot.bad] = idx2
        slot.keep = None

    def _deliver(self, slot: _Slot):
        now = time.perf_counter()
        row = 0
        for r in slot.requests:
            r.done_at = now
            r.future.set_result(slot.result[row:row + r.n].astype(np.int64))
            row += r.n
            self.completed.append(r)
        self.in_use_bytes -= slot.bytes
        slot.requests, slot.n, slot.bytes = [], 0, 0
        slot.stage = 0

    def _loop(self):
        torch.cuda.set_device(self.device)
        while True:
            with self.lock:
                if self.stop_flag and not self.pending and not self.busy:
                    return
                launched = self._admit()
                if not launched and not self.busy:
                    self.lock.wait(timeout=0.001)
                    continue
            for slot in launched:
                try:
                    self._launch(slot)
                    slot.stage = 1
                except Exception as e:  # surface the failure to the requests
                    for r in slot.requests:
                        r.future.set_exception(e)
                    with self.lock:
                        self.in_use_bytes -= slot.bytes
                        slot.requests, slot.n, slot.bytes = [], 0, 0
                        self.free.append(slot)
                    continue
                self.busy.append(slot)
            still = []
            for slot in self.busy:
                if not slot.event.query():
                    still.append(slot)
                    continue
                if slot.stage == 1:
                    self.stats["t_gpu_ms"] += slot.t_start.elapsed_time(slot.event)
                    if not self._finish_stage1(slot):
                        slot.stage = 2  # completion enqueued; its event re-recorded
                        still.append(slot)
                        continue
                else:
                    self._finish_stage2(slot)
                self._deliver(slot)
                with self.lock:
                    self.free.append(slot)
            self.busy = still
            if self.busy and not launched:
                time.sleep(0.0001)

    # ---------------------------------------------------------------- report
    def latency_ms(self):
        lat = np.array([(r.done_at - r.arrival) * 1e3 for r in self.completed])
        return lat


class _NativeFuture:
    """Result of one request to the native server (the Future API subset
    run_schedule uses)."""

    def __init__(self, server: "NativeOrientationServer", ticket: int, n: int, keep):
        self._srv, self._ticket, self._keep = server, ticket, keep
        self._idx = np.empty(n, dtype=np.int32)
        self._dist = np.empty(n, dtype=np.float32)
        self._done = False

    def _ptrs(self):
        return (ctypes.c_void_p(self._idx.ctypes.data), ctypes.c_void_p(self._dist.ctypes.data))

    def done(self) -> bool:
        if not self._done:
            self._wait(0)
        return self._done

    def _wait(self, timeout_ms: int):
        flag = ctypes.c_int(0)
        _lib.call("spf_serve_wait", self._srv._h, self._ticket, int(timeout_ms),
                  ctypes.byref(flag))
        if flag.value:
            self._done = True
            self._keep = None
            self._srv._inflight.pop(self._ticket, None)

    def result(self, timeout: float | None = None) -> np.ndarray:
        if not self._done:
            self._wait(-1 if timeout is None else int(timeout * 1e3))
            if not self._done:
                raise TimeoutError("request not complete")
        return self._idx.astype(np.int64)

    @property
    def distances(self) -> np.ndarray:
        self.result()
        return self._dist


class NativeOrientationServer:
    """The continuous-batching server of the C ABI (spf_serve_*): admission,
    launches and completion run on a native thread of the library, so no
    Python code sits between a request's arrival and its result.  Same
    constructor arguments and submit / close / latency_ms as
    OrientationServer; stats are read from the library."""

    def __init__(self, refs: "matching.ReferenceSet", slot_frames: int = 512, n_slots: int = 3,
                 hbm_budget: int | None = None, path: str = "bf16"):
        if path not in ("bf16", "fp32"):
            raise ValueError("path is 'bf16' or 'fp32'")
        self.refs = refs
        self.n_pix = refs.n_pix
        self.slot_frames = slot_frames
        self.device = refs.f32.device
        h = ctypes.c_void_p()
        _lib.call("spf_serve_create", self.device.index or 0, _lib.ptr(refs.bf16),
                  _lib.ptr(refs.f32), _lib.ptr(refs.sq), _lib.ptr(refs.m2),
                  float(refs.sq_max), refs.n_ref, refs.n_pix, refs.ld,
                  0 if path == "bf16" else 1, slot_frames, n_slots, int(hbm_budget or 0),
                  ctypes.byref(h))
        self._h = h
        self._inflight = {}  # ticket -> future: its buffers stay alive until the library is done

    def submit(self, frames_u16: torch.Tensor, arrival: float | None = None) -> _NativeFuture:
        if frames_u16.dim() != 2 or frames_u16.shape[1] != self.n_pix:
            raise ValueError(f"frames must be [n, {self.n_pix}]")
        if frames_u16.dtype not in (torch.int16, torch.uint16) or frames_u16.is_cuda:
            raise TypeError("frames must be 16-bit photon counts in host memory")
        if not frames_u16.is_contiguous():
            frames_u16 = frames_u16.contiguous()
        n = int(frames_u16.shape[0])
        # arrival is on time.perf_counter(); the library measures on its own clock
        t_lib = -1.0
        if arrival is not None:
            t_lib = float(_lib.lib().spf_serve_clock()) - (time.perf_counter() - arrival)
        fut = _NativeFuture(self, 0, n, frames_u16)
        ticket = ctypes.c_int64(0)
        pi, pd = fut._ptrs()
        _lib.call("spf_serve_submit", self._h, ctypes.c_void_p(frames_u16.data_ptr()), n, pi, pd,
                  t_lib, ctypes.byref(ticket))
        fut._ticket = ticket.value
        self._inflight[ticket.value] = fut
        return fut

    @property
    def stats(self) -> dict:
        v = (ctypes.c_double * 9)()
        _lib.call("spf_serve_stats", self._h, v, 9)
        keys = ("requests", "frames", "launches", "uncertified", "range_overflow", "t_gpu_ms",
                "budget_waits", "p50_ms", "p99_ms")
        return dict(zip(keys, list(v)))

    def latency_ms(self) -> np.ndarray:
        n = ctypes.c_int64(0)
        _lib.call("spf_serve_latencies", self._h, None, 0, ctypes.byref(n))
        out = np.empty(n.value, dtype=np.float64)
        _lib.call("spf_serve_latencies", self._h,
                  out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), n.value, ctypes.byref(n))
        return out

    def close(self):
        if self._h:
            _lib.call("spf_serve_destroy", self._h)  # completes every queued request
            self._h = None
            self._inflight.clear()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def poisson_schedule(total_frames: int, rate_fps: float, rng: np.random.Generator,
                     max_batch: int = 512):
    """Request sizes log-uniform in [1, max_batch] and Poisson arrival times
    whose mean frame rate is rate_fps; returns [(t_arrival, n_frames)]."""
    out = []
    t = 0.0
    n = 0
    mean_size = (max_batch - 1) / np.log(max_batch)  # mean of log-uniform on [1, max_batch]
    rate_req = rate_fps / mean_size
    while n < total_frames:
        size = int(np.clip(np.round(np.exp(rng.uniform(0, np.log(max_batch)))), 1, max_batch))
        size = min(size, total_frames - n)
        t += rng.exponential(1.0 / rate_req)
        out.append((t, size))
        n += size
    return out


def run_schedule(server: OrientationServer, frames_u16_host: torch.Tensor, schedule,
                 time_scale: float = 1.0):
    """Replay a schedule against the server in real time; returns the
    futures and the (arrival, n) list actually used."""
    futures = []
    t0 = time.perf_counter()
    row = 0
    for t_arr, n in schedule:
        target = t0 + t_arr * time_scale
        while True:
            now = time.perf_counter()
            if now >= target:
                break
            time.sleep(min(0.0005, target - now))
        if row + n > frames_u16_host.shape[0]:
            row = 0
        futures.append(server.submit(frames_u16_host[row:row + n], arrival=target))
        row += n
    results = [f.result() for f in futures]
    return results
