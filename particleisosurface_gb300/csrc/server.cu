// Request loop: continuous batching of frame reconstructions on one GPU.
//
// The reference reconstructs one frame per process run (runOurs,
// src/main.cpp:330-405).  Here a server owns `slots` worker threads, each
// with its own context (CUDA stream); requests queue in arrival order and a
// worker admits the head request when its estimated device footprint fits in
// the memory budget next to the frames already resident (at least one frame
// is always admitted).  Admitted frames run concurrently, their kernels
// overlapping on the device; results stay in host memory until fetched.
// Each frame's computation is the same as pi_run's, so a result does not
// depend on what else runs beside it.
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "internal.h"

namespace pisurf {

extern thread_local std::string g_last_error;

static double now_ms() {
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// Device bytes of one frame, per particle plus a fixed part (hash grid and
// per-particle arrays ~160 B, octree nodes and per-level sample buffers and
// extraction sort buffers ~2 KB at the configurations' surface densities).
static size_t frame_bytes_estimate(long long n) { return (size_t)n * 2304 + (64ull << 20); }

struct Request {
  uint64_t ticket = 0;
  pi_params P;
  std::vector<float> xyz;
  long long n = 0;
  size_t est = 0;
  double t_submit = 0, t_start = 0, t_done = 0;
  bool done = false;
  int rc = 0;
  std::string err;
  std::vector<float> verts;
  std::vector<int32_t> tris;
};

}  // namespace pisurf

struct pi_server {
  int device = 0;
  int slots = 1;
  size_t budget = 0;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<std::shared_ptr<pisurf::Request>> queue;
  std::unordered_map<uint64_t, std::shared_ptr<pisurf::Request>> live;
  size_t reserved = 0;
  int in_flight = 0, max_in_flight = 0;
  long long completed = 0;
  uint64_t next_ticket = 1;
  bool stop = false;
  std::vector<std::thread> workers;
};

namespace pisurf {

static void worker_main(pi_server* s, int slot) {
  pi_ctx* ctx = nullptr;
  int rc0 = pi_ctx_create(s->device, 0, &ctx);
  // without a server budget a worker keeps one frame for all its requests
  // (device buffers and events carry over); with a budget each request's
  // memory is returned when it completes, as admission assumes
  pi_frame* kept = nullptr;
  const bool reuse = s->budget == 0;
  for (;;) {
    std::shared_ptr<Request> r;
    {
      std::unique_lock<std::mutex> lk(s->mu);
      s->cv_work.wait(lk, [&] {
        if (s->stop) return true;
        if (s->queue.empty()) return false;
        const size_t need = s->queue.front()->est;
        return s->in_flight == 0 || s->budget == 0 || s->reserved + need <= s->budget;
      });
      if (s->stop && s->queue.empty()) break;
      if (s->queue.empty()) continue;
      r = s->queue.front();
      s->queue.pop_front();
      s->reserved += r->est;
      s->in_flight++;
      if (s->in_flight > s->max_in_flight) s->max_in_flight = s->in_flight;
    }
    r->t_start = now_ms();
    int rc = rc0;
    std::string err = rc0 ? std::string(pi_last_error()) : std::string();
    if (!rc) {
      pi_frame* f = nullptr;
      if (reuse && kept) {
        try {
          check_params(&r->P);
          kept->P = r->P;
          frame_clear(kept, 0);
          f = kept;
        } catch (const std::exception& e) {
          rc = PI_ERR_INVALID;
          g_last_error = e.what();
        }
      } else {
        rc = pi_frame_create(ctx, &r->P, &f);
        if (!rc && reuse) kept = f;
      }
      if (!rc) rc = pi_frame_upload(f, r->xyz.data(), r->n);
      if (!rc) rc = pi_run(f);
      int64_t nv = 0, nt = 0;
      if (!rc) rc = pi_mesh_counts(f, &nv, &nt);
      if (!rc) {
        r->verts.resize((size_t)nv * 3);
        r->tris.resize((size_t)nt * 3);
        rc = pi_mesh_get(f, r->verts.data(), r->tris.data(), nullptr);
      }
      if (rc) err = pi_last_error();
      if (f && f != kept) pi_frame_destroy(f);
    }
    r->xyz.clear();
    r->xyz.shrink_to_fit();
    {
      std::lock_guard<std::mutex> lk(s->mu);
      r->rc = rc;
      r->err = err;
      r->t_done = now_ms();
      r->done = true;
      s->reserved -= r->est;
      s->in_flight--;
      s->completed++;
    }
    s->cv_done.notify_all();
    s->cv_work.notify_all();
  }
  if (kept) pi_frame_destroy(kept);
  if (ctx) pi_ctx_destroy(ctx);
  (void)slot;
}

}  // namespace pisurf

using namespace pisurf;

#define SRV_BEGIN try {
#define SRV_END                                   \
  }                                               \
  catch (const std::invalid_argument& e) {        \
    g_last_error = e.what();                      \
    return PI_ERR_INVALID;                        \
  }                                               \
  catch (const std::exception& e) {               \
    g_last_error = e.what();                      \
    return PI_ERR_CUDA;                           \
  }                                               \
  return PI_OK;

extern "C" {

int pi_server_create(int device, int slots, size_t budget_bytes, pi_server** out) {
  SRV_BEGIN
  if (!out || slots < 1 || slots > 64) throw std::invalid_argument("bad server arguments");
  int ndev = 0;
  PI_CUDA(cudaGetDeviceCount(&ndev));
  if (device < 0 || device >= ndev) throw std::invalid_argument("no such CUDA device");
  pi_server* s = new pi_server();
  s->device = device;
  s->slots = slots;
  s->budget = budget_bytes;
  for (int k = 0; k < slots; ++k) s->workers.emplace_back(worker_main, s, k);
  *out = s;
  SRV_END
}

int pi_server_submit(pi_server* s, const pi_params* p, const float* xyz, int64_t n, uint64_t* ticket) {
  SRV_BEGIN
  if (!s || !p || !xyz || n <= 0 || !ticket) throw std::invalid_argument("bad submit arguments");
  auto r = std::make_shared<Request>();
  r->P = *p;
  r->n = n;
  r->xyz.assign(xyz, xyz + 3 * n);
  r->est = frame_bytes_estimate(n);
  r->t_submit = now_ms();
  {
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->stop) throw std::invalid_argument("server is stopping");
    r->ticket = s->next_ticket++;
    s->live[r->ticket] = r;
    s->queue.push_back(r);
    *ticket = r->ticket;
  }
  s->cv_work.notify_all();
  SRV_END
}

int pi_server_poll(pi_server* s, uint64_t ticket, int* done) {
  SRV_BEGIN
  if (!s || !done) throw std::invalid_argument("null argument");
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->live.find(ticket);
  if (it == s->live.end()) throw std::invalid_argument("unknown ticket");
  *done = it->second->done ? 1 : 0;
  SRV_END
}

int pi_server_wait(pi_server* s, uint64_t ticket, int64_t* nverts, int64_t* ntris, double* latency_ms,
                   double* queue_ms) {
  SRV_BEGIN
  if (!s) throw std::invalid_argument("null server");
  std::shared_ptr<Request> r;
  {
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->live.find(ticket);
    if (it == s->live.end()) throw std::invalid_argument("unknown ticket");
    r = it->second;
    s->cv_done.wait(lk, [&] { return r->done; });
  }
  if (nverts) *nverts = (int64_t)(r->verts.size() / 3);
  if (ntris) *ntris = (int64_t)(r->tris.size() / 3);
  if (latency_ms) *latency_ms = r->t_done - r->t_submit;
  if (queue_ms) *queue_ms = r->t_start - r->t_submit;
  if (r->rc) {
    g_last_error = r->err;
    return r->rc;
  }
  SRV_END
}

int pi_server_fetch(pi_server* s, uint64_t ticket, float* verts, int32_t* tris) {
  SRV_BEGIN
  if (!s) throw std::invalid_argument("null server");
  std::shared_ptr<Request> r;
  {
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->live.find(ticket);
    if (it == s->live.end()) throw std::invalid_argument("unknown ticket");
    r = it->second;
    s->cv_done.wait(lk, [&] { return r->done; });
    s->live.erase(it);
  }
  if (r->rc) {
    g_last_error = r->err;
    return r->rc;
  }
  if (verts && !r->verts.empty()) std::memcpy(verts, r->verts.data(), sizeof(float) * r->verts.size());
  if (tris && !r->tris.empty()) std::memcpy(tris, r->tris.data(), sizeof(int32_t) * r->tris.size());
  SRV_END
}

int pi_server_stats(pi_server* s, int64_t* completed, int64_t* in_flight, int64_t* max_in_flight,
                    int64_t* queued, int64_t* bytes_reserved) {
  SRV_BEGIN
  if (!s) throw std::invalid_argument("null server");
  std::lock_guard<std::mutex> lk(s->mu);
  if (completed) *completed = s->completed;
  if (in_flight) *in_flight = s->in_flight;
  if (max_in_flight) *max_in_flight = s->max_in_flight;
  if (queued) *queued = (int64_t)s->queue.size();
  if (bytes_reserved) *bytes_reserved = (int64_t)s->reserved;
  SRV_END
}

int pi_server_destroy(pi_server* s) {
  SRV_BEGIN
  if (!s) return PI_OK;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
  }
  s->cv_work.notify_all();
  for (auto& t : s->workers) t.join();
  delete s;
  SRV_END
}

}  // extern "C"
