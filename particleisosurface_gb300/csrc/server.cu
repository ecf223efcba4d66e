// Request loop: continuous batching of frame reconstructions on one GPU.
//
// The reference reconstructs one frame per run of its driver loop (runOurs,
// src/main.cpp:330-405).  Here a server owns `slots` worker threads, each
// with its own context (CUDA stream); requests queue in arrival order and a
// worker admits a request when its device-memory reservation fits in the
// budget next to the frames in flight and the resident frame states (one
// frame is always admitted when nothing else holds memory).  Admitted frames
// run concurrently, their kernels overlapping on the device; results stay in
// host memory until fetched.  Each frame's computation is the same as
// pi_run's, so a result does not depend on what else runs beside it.
//
// Admission.  A request reserves an estimate of its frame's device bytes;
// with a budget, the worker's context is capped at that reservation, so a
// frame cannot take more than it was admitted with: a frame that needs more
// fails inside the worker with PI_ERR_NOMEM and goes back to the head of the
// queue with its reservation doubled, up to the whole budget (a frame that
// needs more than the whole budget fails with PI_ERR_NOMEM).  When the head request
// does not fit, up to kLookahead requests behind it may pass it if they fit,
// but no request is passed more than kMaxBypass times, so a large request
// cannot starve.
//
// Resident frame states.  After a request completes its frame (hash grid,
// anisotropy, octree, mesh and their device buffers) stays resident in the
// worker that built it, tagged with the request's sequence (the steps of one
// advected particle set, pi_server_submit_seq).  The next step of that
// sequence goes to the worker holding it when that worker is idle, and is
// reconstructed in the resident frame's buffers.  At most one frame state is
// resident per worker (`slots` in all); with a budget the resident bytes
// count against it and idle workers give their frames back, least recently
// used first, when an admission needs the room.
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <algorithm>
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
// per-particle arrays ~190 B, octree nodes, per-level sample buffers and
// extraction tables ~2-3 KB at the configurations' surface densities; the
// fixed part covers the per-cell bucket tables and the corner bitmap of
// small frames).
constexpr size_t kEstPerParticle = 3072, kEstFixed = 128ull << 20;

constexpr int kLookahead = 16;  // queued requests that may pass a blocked head
constexpr int kMaxBypass = 8;   // times one request may be passed

struct Request {
  uint64_t ticket = 0;
  uint64_t seq = 0;  // sequence id (0: none)
  pi_params P;
  std::vector<float> xyz;
  long long n = 0;
  size_t est = 0;
  int bypassed = 0;
  int retries = 0;
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
  size_t est_per_particle = pisurf::kEstPerParticle, est_fixed = pisurf::kEstFixed;
  size_t reserved = 0;  // reservations of the frames in flight
  int in_flight = 0, max_in_flight = 0;
  long long completed = 0, bypasses = 0, retries = 0, resident_hits = 0;
  uint64_t next_ticket = 1;
  long long clock = 0;  // request starts, for the least-recently-used order
  bool stop = false;
  // per worker: busy, the sequence of its resident frame (0: none or
  // anonymous), the resident frame's device bytes (counted with a budget),
  // its last use, and whether an admission asked it to release the frame
  std::vector<char> busy;
  std::vector<uint64_t> res_seq;
  std::vector<size_t> res_bytes;
  std::vector<long long> res_used;
  std::vector<char> drop;  // the worker must release its resident frame
  std::vector<std::thread> workers;
};

namespace pisurf {

static size_t resident_total(const pi_server* s) {
  size_t t = 0;
  for (size_t b : s->res_bytes) t += b;
  return t;
}

// Under s->mu: the worker that should run request r next to `slot`'s
// choice: the idle worker holding r's sequence, else `slot` itself.
static int owner_for(const pi_server* s, const Request& r, int slot) {
  if (r.seq == 0) return slot;
  for (int w = 0; w < s->slots; ++w)
    if (s->res_seq[w] == r.seq) return s->busy[w] ? slot : w;
  return slot;
}

// Under s->mu: whether r fits now next to the frames in flight and the
// resident frames (this worker's own resident frame is replaced by r's).
// When it would fit once idle workers gave their resident frames back, those
// workers (least recently used first) are asked to release them, and r is
// admitted after they have.
static bool fits(pi_server* s, const Request& r, int self) {
  if (s->budget == 0) return true;
  const size_t res = resident_total(s) - s->res_bytes[self];
  if (s->in_flight == 0 && res == 0) return true;  // alone: always admitted
  if (s->reserved + res + r.est <= s->budget) return true;
  std::vector<int> idle;
  for (int w = 0; w < s->slots; ++w)
    if (w != self && !s->busy[w] && s->res_bytes[w] && !s->drop[w]) idle.push_back(w);
  std::sort(idle.begin(), idle.end(), [&](int a, int b) { return s->res_used[a] < s->res_used[b]; });
  size_t need = s->reserved + res + r.est;
  std::vector<int> release;
  for (int w : idle) {
    if (need <= s->budget || (s->in_flight == 0 && need == r.est)) break;
    need -= s->res_bytes[w];
    release.push_back(w);
  }
  if (need > s->budget && !(s->in_flight == 0 && need == r.est)) return false;
  for (int w : release) s->drop[w] = 1;
  if (!release.empty()) s->cv_work.notify_all();
  return false;
}

// Under s->mu: the index in the queue of the request this worker may start,
// or -1.
static int pick(pi_server* s, int slot) {
  const int nq = (int)s->queue.size();
  const int look = std::min(nq, 1 + kLookahead);
  for (int i = 0; i < look; ++i) {
    const Request& r = *s->queue[i];
    if (i > 0 && s->queue[0]->bypassed >= kMaxBypass) break;
    if (owner_for(s, r, slot) != slot) continue;  // the idle holder of its sequence takes it
    if (fits(s, r, slot)) return i;
  }
  return -1;
}

static void worker_main(pi_server* s, int slot) {
  pi_ctx* ctx = nullptr;
  int rc0 = pi_ctx_create(s->device, 0, &ctx);
  // the frame of the worker's last request stays resident (its device
  // buffers, events and results), and the next request reuses it
  pi_frame* kept = nullptr;
  for (;;) {
    std::shared_ptr<Request> r;
    {
      std::unique_lock<std::mutex> lk(s->mu);
      int at = -1;
      s->cv_work.wait(lk, [&] {
        if (s->drop[slot]) return true;
        if (s->stop && s->queue.empty()) return true;
        at = pick(s, slot);
        return at >= 0;
      });
      if (s->drop[slot]) {
        // an admission elsewhere needs this worker's resident bytes
        lk.unlock();
        if (kept) pi_frame_destroy(kept);
        kept = nullptr;
        lk.lock();
        s->drop[slot] = 0;
        s->res_bytes[slot] = 0;
        s->res_seq[slot] = 0;
        s->cv_work.notify_all();
        continue;
      }
      if (at < 0) break;  // stopping, queue empty
      r = s->queue[at];
      if (at > 0) {
        s->queue[0]->bypassed++;
        s->bypasses++;
      }
      s->queue.erase(s->queue.begin() + at);
      if (r->seq && s->res_seq[slot] == r->seq) s->resident_hits++;
      // this worker's resident frame is reused (or replaced) by r: its bytes
      // are now part of r's reservation
      s->res_bytes[slot] = 0;
      s->res_seq[slot] = 0;
      s->busy[slot] = 1;
      s->reserved += r->est;
      s->in_flight++;
      s->res_used[slot] = ++s->clock;
      if (s->in_flight > s->max_in_flight) s->max_in_flight = s->in_flight;
    }
    r->t_start = now_ms();
    int rc = rc0;
    std::string err = rc0 ? std::string(pi_last_error()) : std::string();
    size_t held = 0;
    if (!rc) {
      // a budget caps the context at the request's reservation (at most the
      // whole budget); a resident frame holding more than that is given back
      // first
      ctx->budget = s->budget ? std::min(r->est, s->budget) : 0;
      if (kept && s->budget && (size_t)ctx->used.load() > r->est) {
        pi_frame_destroy(kept);
        kept = nullptr;
      }
      pi_frame* f = nullptr;
      if (kept) {
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
        if (!rc) kept = f;
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
      if (rc && kept) {
        // a failed frame is not kept: its buffers go back
        pi_frame_destroy(kept);
        kept = nullptr;
      }
      held = (size_t)ctx->used.load();
    }
    bool requeue = false;
    {
      std::lock_guard<std::mutex> lk(s->mu);
      s->reserved -= r->est;
      s->in_flight--;
      s->busy[slot] = 0;
      if (rc == PI_ERR_NOMEM && s->budget && r->est < s->budget) {
        // the frame needs more than its reservation: back to the head with
        // twice as much, at most the whole budget
        r->est = std::min(r->est * 2, s->budget);
        r->retries++;
        s->retries++;
        s->queue.push_front(r);
        requeue = true;
      } else {
        if (!rc) {
          s->res_seq[slot] = r->seq;
          s->res_bytes[slot] = s->budget ? held : 0;
        }
        r->xyz.clear();
        r->xyz.shrink_to_fit();
        r->rc = rc;
        r->err = err;
        r->t_done = now_ms();
        r->done = true;
        s->completed++;
      }
    }
    (void)requeue;
    s->cv_done.notify_all();
    s->cv_work.notify_all();
  }
  if (kept) pi_frame_destroy(kept);
  if (ctx) pi_ctx_destroy(ctx);
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
  s->busy.assign(slots, 0);
  s->res_seq.assign(slots, 0);
  s->res_bytes.assign(slots, 0);
  s->res_used.assign(slots, 0);
  s->drop.assign(slots, 0);
  for (int k = 0; k < slots; ++k) s->workers.emplace_back(worker_main, s, k);
  *out = s;
  SRV_END
}

int pi_server_submit_seq(pi_server* s, const pi_params* p, const float* xyz, int64_t n, uint64_t sequence,
                         uint64_t* ticket) {
  SRV_BEGIN
  if (!s || !p || !xyz || n <= 0 || !ticket) throw std::invalid_argument("bad submit arguments");
  auto r = std::make_shared<Request>();
  r->seq = sequence;
  r->P = *p;
  r->n = n;
  r->xyz.assign(xyz, xyz + 3 * n);
  {
    std::lock_guard<std::mutex> lk(s->mu);
    r->est = (size_t)n * s->est_per_particle + s->est_fixed;
  }
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

int pi_server_submit(pi_server* s, const pi_params* p, const float* xyz, int64_t n, uint64_t* ticket) {
  return pi_server_submit_seq(s, p, xyz, n, 0, ticket);
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

int pi_server_set_estimate(pi_server* s, size_t bytes_per_particle, size_t fixed_bytes) {
  SRV_BEGIN
  if (!s || bytes_per_particle == 0) throw std::invalid_argument("bad estimate");
  std::lock_guard<std::mutex> lk(s->mu);
  s->est_per_particle = bytes_per_particle;
  s->est_fixed = fixed_bytes;
  SRV_END
}

int pi_server_info(pi_server* s, int64_t* out8) {
  SRV_BEGIN
  if (!s || !out8) throw std::invalid_argument("null argument");
  std::lock_guard<std::mutex> lk(s->mu);
  int resident = 0;
  for (int w = 0; w < s->slots; ++w) resident += (s->res_seq[w] != 0 || s->res_bytes[w] != 0) ? 1 : 0;
  out8[0] = s->completed;
  out8[1] = (int64_t)s->reserved;
  out8[2] = (int64_t)resident_total(s);
  out8[3] = resident;
  out8[4] = s->bypasses;
  out8[5] = s->retries;
  out8[6] = s->resident_hits;
  out8[7] = (int64_t)s->budget;
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
