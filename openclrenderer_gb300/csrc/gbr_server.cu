// gbr_server.cu — the serving loop: resident scenes, HBM-budgeted admission,
// continuous batching per scene, overlap across scenes, latency statistics.
//
// Threads: submit() runs on the caller's thread; each scene has a worker
// thread with its own CUDA stream and device output pool.  Admission is FIFO
// over all scenes: a request is admitted when the bytes of everything
// admitted plus its own fit the budget; it then waits in its scene's pending
// queue.  A worker takes every pending request of its scene (up to the batch
// limits) as one batch, renders it with one launch per stage
// (render_batch), copies each result to the request's host buffers, completes
// the requests and releases their bytes, which admits more.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <thread>
#include <vector>

#include "../../include/gbr.h"
#include "gbr_scene.h"
#include "gbr_internal.h"

namespace {

using Clock = std::chrono::steady_clock;

double ms_between(Clock::time_point a, Clock::time_point b) {
  return std::chrono::duration<double, std::milli>(b - a).count();
}

struct Req {
  gbr_request r;
  uint64_t id;
  uint64_t bytes;
  Clock::time_point t_submit, t_launch, t_admit;
};

// Device outputs of one batch; two per worker so that a batch renders while
// the previous one's results are still being copied to host memory.
struct Pool {
  uint8_t* p = nullptr;
  size_t bytes = 0;
  cudaEvent_t free_ev = nullptr;  // recorded after the pool's last copy
  bool used = false;
};

struct Worker;

// A batch in flight: completed from the stream by a host callback.
struct Flight {
  gbr_server* server;
  Worker* worker;
  std::vector<Req> batch;
  Clock::time_point t_launch;
  gbr_status status;
};

struct Worker {
  uint32_t scene_index = 0;
  gbr_scene* scene = nullptr;
  cudaStream_t stream = nullptr;
  std::deque<Req> pending;
  std::thread thread;
  Pool pools[2];
  int next_pool = 0;
};

}  // namespace

struct gbr_server {
  gbr_server_config cfg{};
  int device = 0;
  std::vector<Worker*> workers;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<Req> waiting;  // not yet admitted (FIFO)
  std::deque<gbr_completion> done;
  std::vector<double> latencies;
  uint64_t admitted_bytes = 0, peak_bytes = 0;
  uint64_t next_id = 1, submitted = 0, completed = 0, rejected = 0, batches = 0, batch_views = 0;
  uint64_t pixels_completed = 0;
  uint64_t in_system = 0;  // submitted, not completed
  uint32_t inflight = 0;   // batches launched, not completed
  bool stop = false;
  bool started = false;
  Clock::time_point t_first, t_last;
};

namespace {

// Admit waiting requests in FIFO order while the budget allows (lock held).
void admit_locked(gbr_server* s) {
  bool any = false;
  while (!s->waiting.empty()) {
    Req& q = s->waiting.front();
    if (s->admitted_bytes + q.bytes > s->cfg.hbm_budget_bytes) break;
    q.t_admit = Clock::now();
    s->admitted_bytes += q.bytes;
    s->peak_bytes = std::max(s->peak_bytes, s->admitted_bytes);
    s->workers[q.r.scene]->pending.push_back(q);
    s->waiting.pop_front();
    any = true;
  }
  if (any) s->cv_work.notify_all();
}

gbr_status ensure_pool(Pool& pl, size_t bytes) {
  if (pl.used && cudaEventSynchronize(pl.free_ev) != cudaSuccess) return GBR_CUDA_ERROR;
  if (bytes <= pl.bytes) return GBR_OK;
  if (pl.p) cudaFree(pl.p);
  pl.p = nullptr;
  pl.bytes = 0;
  if (cudaMalloc(&pl.p, bytes) != cudaSuccess) {
    cudaGetLastError();
    return GBR_OOM;
  }
  pl.bytes = bytes;
  return GBR_OK;
}

void complete(gbr_server* s, std::vector<Req>& batch, gbr_status st, Clock::time_point t_launch);

// Runs on a driver thread when the stream reaches the end of a batch's copies.
void CUDART_CB on_batch_done(void* data) {
  Flight* f = static_cast<Flight*>(data);
  complete(f->server, f->batch, f->status, f->t_launch);
  delete f;
}

void worker_loop(gbr_server* s, Worker* w) {
  cudaSetDevice(s->device);
  const uint32_t max_views = s->cfg.max_batch_views ? s->cfg.max_batch_views : 64;
  const uint64_t max_pix = s->cfg.max_batch_pixels ? s->cfg.max_batch_pixels : 33177600ull;
  for (;;) {
    std::vector<Req> batch;
    {
      std::unique_lock<std::mutex> lk(s->mu);
      s->cv_work.wait(lk, [&] { return s->stop || !w->pending.empty(); });
      if (s->stop && w->pending.empty()) return;
      // a batching window from the oldest pending request, cut short when
      // the batch limits are reached or the server stops
      if (s->cfg.batch_window_us) {
        const Clock::time_point until = w->pending.front().t_admit + std::chrono::microseconds(s->cfg.batch_window_us);
        s->cv_work.wait_until(lk, until, [&] {
          if (s->stop) return true;
          uint64_t pix = 0;
          for (const Req& q : w->pending) pix += (uint64_t)q.r.view.width * q.r.view.height;
          return w->pending.size() >= max_views || pix >= max_pix;
        });
      }
      // a slot on the GPU: requests arriving meanwhile join this batch
      if (s->cfg.max_inflight)
        s->cv_work.wait(lk, [&] { return s->stop || s->inflight < s->cfg.max_inflight; });
      s->inflight++;
      uint64_t pix = 0;
      while (!w->pending.empty() && batch.size() < max_views) {
        const Req& q = w->pending.front();
        const uint64_t p = (uint64_t)q.r.view.width * (uint64_t)q.r.view.height;
        if (!batch.empty() && pix + p > max_pix) break;
        pix += p;
        batch.push_back(q);
        w->pending.pop_front();
      }
    }
    const Clock::time_point t_launch = Clock::now();
    // device outputs: depth, id, rgba per view, packed in the worker's pool
    size_t bytes = 0;
    std::vector<size_t> offs(batch.size());
    for (size_t i = 0; i < batch.size(); i++) {
      offs[i] = bytes;
      bytes += (size_t)batch[i].r.view.width * batch[i].r.view.height * 12 + 256;
    }
    Pool& pl = w->pools[w->next_pool];
    w->next_pool ^= 1;
    gbr_status st = ensure_pool(pl, bytes);
    std::vector<gbr_camera> cams(batch.size());
    std::vector<gbr_view> views(batch.size());
    std::vector<gbr_outputs> outs(batch.size());
    // a pinned, mapped RGBA buffer is written by kernel3 itself (no copy)
    std::vector<uint8_t*> direct(batch.size(), nullptr);
    for (size_t i = 0; i < batch.size() && st == GBR_OK; i++) {
      const size_t P = (size_t)batch[i].r.view.width * batch[i].r.view.height;
      uint8_t* b = pl.p + offs[i];
      cams[i] = batch[i].r.cam;
      views[i] = batch[i].r.view;
      direct[i] = gbr::mapped_host_alias(batch[i].r.rgba);
      outs[i] = gbr_outputs{reinterpret_cast<uint32_t*>(b), reinterpret_cast<uint32_t*>(b + 4 * P),
                            direct[i] ? direct[i] : b + 8 * P, nullptr};
    }
    if (st == GBR_OK)
      st = gbr_render_batch(w->scene, (uint32_t)batch.size(), cams.data(), views.data(), outs.data(), w->stream);
    if (st == GBR_OK) {
      for (size_t i = 0; i < batch.size() && st == GBR_OK; i++) {
        const size_t P = (size_t)batch[i].r.view.width * batch[i].r.view.height;
        const gbr_request& r = batch[i].r;
        if (r.depth && cudaMemcpyAsync(r.depth, outs[i].depth, 4 * P, cudaMemcpyDeviceToHost, w->stream) != cudaSuccess)
          st = GBR_CUDA_ERROR;
        if (r.id && cudaMemcpyAsync(r.id, outs[i].id, 4 * P, cudaMemcpyDeviceToHost, w->stream) != cudaSuccess)
          st = GBR_CUDA_ERROR;
        if (r.rgba && !direct[i] &&
            cudaMemcpyAsync(r.rgba, outs[i].rgba, 4 * P, cudaMemcpyDeviceToHost, w->stream) != cudaSuccess)
          st = GBR_CUDA_ERROR;
      }
    }
    if (st == GBR_OK) {
      Flight* f = new Flight{s, w, std::move(batch), t_launch, GBR_OK};
      if (cudaEventRecord(pl.free_ev, w->stream) == cudaSuccess &&
          cudaLaunchHostFunc(w->stream, on_batch_done, f) == cudaSuccess) {
        pl.used = true;
        continue;  // completed from the stream; take the next batch now
      }
      batch = std::move(f->batch);
      delete f;
      st = GBR_CUDA_ERROR;
    }
    cudaStreamSynchronize(w->stream);
    complete(s, batch, st, t_launch);
  }
}

void complete(gbr_server* s, std::vector<Req>& batch, gbr_status st, Clock::time_point t_launch) {
  const Clock::time_point t_done = Clock::now();
  {
    std::lock_guard<std::mutex> lk(s->mu);
    for (const Req& q : batch) {
      gbr_completion c{};
      c.request_id = q.id;
      c.user_tag = q.r.user_tag;
      c.status = st;
      c.batch_views = (uint32_t)batch.size();
      c.latency_ms = ms_between(q.t_submit, t_done);
      c.queue_ms = ms_between(q.t_submit, t_launch);
      s->done.push_back(c);
      s->admitted_bytes -= q.bytes;
      s->completed++;
      s->in_system--;
      if (st == GBR_OK) {
        s->latencies.push_back(c.latency_ms);
        s->pixels_completed += (uint64_t)q.r.view.width * q.r.view.height;
      }
    }
    s->batches++;
    s->batch_views += batch.size();
    s->inflight--;
    s->t_last = t_done;
    admit_locked(s);
  }
  s->cv_done.notify_all();
  s->cv_work.notify_all();  // a GPU slot is free
}

}  // namespace

extern "C" {

gbr_status gbr_server_create(gbr_scene* const* scenes, uint32_t n, const gbr_server_config* cfg, gbr_server** out) {
  if (!out || !cfg || !scenes || n == 0) return GBR_INVALID_ARG;
  *out = nullptr;
  gbr_server* s = new gbr_server();
  s->cfg = *cfg;
  if (s->cfg.hbm_budget_bytes == 0) s->cfg.hbm_budget_bytes = 8ull << 30;
  cudaGetDevice(&s->device);
  for (uint32_t i = 0; i < n; i++) {
    if (!scenes[i]) {
      for (Worker* w : s->workers) delete w;
      delete s;
      return GBR_INVALID_ARG;
    }
    Worker* w = new Worker();
    w->scene_index = i;
    w->scene = scenes[i];
    if (cudaStreamCreateWithFlags(&w->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&w->pools[0].free_ev, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&w->pools[1].free_ev, cudaEventDisableTiming) != cudaSuccess) {
      delete w;
      for (Worker* x : s->workers) delete x;
      delete s;
      return GBR_CUDA_ERROR;
    }
    s->workers.push_back(w);
  }
  for (Worker* w : s->workers) w->thread = std::thread(worker_loop, s, w);
  *out = s;
  return GBR_OK;
}

gbr_status gbr_server_submit(gbr_server* s, const gbr_request* req, uint64_t* request_id) {
  if (!s || !req) return GBR_INVALID_ARG;
  if (req->scene >= s->workers.size()) return GBR_INVALID_ARG;
  const gbr_view& v = req->view;
  if (v.width < 1 || v.height < 1 || v.width > gbr::kMaxWalkWidth || v.height > gbr::kMaxWalkHeight)
    return GBR_INVALID_ARG;
  Req q;
  q.r = *req;
  q.bytes = gbr::view_device_bytes(v.width, v.height);
  q.t_submit = Clock::now();
  std::lock_guard<std::mutex> lk(s->mu);
  if (q.bytes > s->cfg.hbm_budget_bytes) {
    s->rejected++;
    return GBR_ADMISSION_REJECTED;
  }
  q.id = s->next_id++;
  if (request_id) *request_id = q.id;
  if (!s->started) {
    s->started = true;
    s->t_first = q.t_submit;
  }
  s->submitted++;
  s->in_system++;
  s->waiting.push_back(q);
  admit_locked(s);
  return GBR_OK;
}

gbr_status gbr_server_poll(gbr_server* s, gbr_completion* out, uint32_t cap, uint32_t* n, int32_t wait_ms) {
  if (!s || !n || (cap && !out)) return GBR_INVALID_ARG;
  std::unique_lock<std::mutex> lk(s->mu);
  if (s->done.empty() && wait_ms != 0) {
    if (wait_ms < 0)
      s->cv_done.wait(lk, [&] { return !s->done.empty() || s->in_system == 0; });
    else
      s->cv_done.wait_for(lk, std::chrono::milliseconds(wait_ms), [&] { return !s->done.empty(); });
  }
  uint32_t k = 0;
  while (k < cap && !s->done.empty()) {
    out[k++] = s->done.front();
    s->done.pop_front();
  }
  *n = k;
  return GBR_OK;
}

gbr_status gbr_server_drain(gbr_server* s) {
  if (!s) return GBR_INVALID_ARG;
  std::unique_lock<std::mutex> lk(s->mu);
  s->cv_done.wait(lk, [&] { return s->in_system == 0; });
  return GBR_OK;
}

gbr_status gbr_server_drain_for(gbr_server* s, int32_t timeout_ms) {
  if (!s) return GBR_INVALID_ARG;
  if (timeout_ms < 0) return gbr_server_drain(s);
  std::unique_lock<std::mutex> lk(s->mu);
  if (!s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), [&] { return s->in_system == 0; }))
    return gbr::fail(GBR_DEVICE_TIMEOUT, "%llu requests still in the system after %d ms",
                (unsigned long long)s->in_system, timeout_ms);
  return GBR_OK;
}

gbr_status gbr_server_stats_get(gbr_server* s, gbr_server_stats* out) {
  if (!s || !out) return GBR_INVALID_ARG;
  std::lock_guard<std::mutex> lk(s->mu);
  gbr_server_stats st{};
  st.submitted = s->submitted;
  st.completed = s->completed;
  st.rejected = s->rejected;
  st.batches = s->batches;
  st.pixels_completed = s->pixels_completed;
  st.peak_admitted_bytes = s->peak_bytes;
  std::vector<double> l = s->latencies;
  if (!l.empty()) {
    std::sort(l.begin(), l.end());
    auto pct = [&](double p) { return l[std::min(l.size() - 1, (size_t)(p * (l.size() - 1) + 0.5))]; };
    st.p50_ms = pct(0.50);
    st.p99_ms = pct(0.99);
    double sum = 0;
    for (double x : l) sum += x;
    st.mean_ms = sum / l.size();
  }
  st.mean_batch_views = s->batches ? (double)s->batch_views / s->batches : 0.0;
  st.wall_s = s->started ? ms_between(s->t_first, s->t_last) / 1e3 : 0.0;
  *out = st;
  return GBR_OK;
}

gbr_status gbr_server_destroy(gbr_server* s) {
  if (!s) return GBR_OK;
  {
    std::unique_lock<std::mutex> lk(s->mu);
    s->cv_done.wait(lk, [&] { return s->in_system == 0; });
  }
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
  }
  s->cv_work.notify_all();
  for (Worker* w : s->workers) {
    if (w->thread.joinable()) w->thread.join();
    if (w->stream) cudaStreamSynchronize(w->stream);
    for (Pool& pl : w->pools) {
      if (pl.p) cudaFree(pl.p);
      if (pl.free_ev) cudaEventDestroy(pl.free_ev);
    }
    if (w->stream) cudaStreamDestroy(w->stream);
    delete w;
  }
  delete s;
  return GBR_OK;
}

}  // extern "C"
