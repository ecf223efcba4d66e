// C ABI (include/pisurf.h): context and frame lifecycle, stage
// orchestration, dumps and queries.  SurfReconstructor::Run
// (src/surface_reconstructor.cpp:409-479) is pi_run.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <algorithm>
#include <cstdlib>
#include <memory>
#include <mutex>
#include <new>
#include <stdexcept>
#include <string>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "internal.h"

namespace pisurf {

struct NoMem : std::runtime_error {
  using std::runtime_error::runtime_error;
};
struct StateError : std::runtime_error {
  using std::runtime_error::runtime_error;
};

thread_local std::string g_last_error;

void ctx_account(pi_ctx* c, long long delta) {
  if (!c) return;
  long long now = c->used.fetch_add(delta) + delta;
  if (delta > 0 && c->budget && now > (long long)c->budget) {
    c->used.fetch_sub(delta);
    throw NoMem("device memory budget exceeded: need " + std::to_string(now) + " bytes, budget " +
                std::to_string(c->budget));
  }
}

template <class T>
void DBuf<T>::alloc(pi_ctx* c, cudaStream_t st, size_t count) {
  release();
  if (count == 0) count = 1;
  ctx_account(c, (long long)(count * sizeof(T)));
  void* q = nullptr;
  cudaError_t e = cudaMallocAsync(&q, count * sizeof(T), st);
  if (e != cudaSuccess) {
    ctx_account(c, -(long long)(count * sizeof(T)));
    (void)cudaGetLastError();
    if (e == cudaErrorMemoryAllocation) throw NoMem("cudaMallocAsync: out of device memory");
    throw CudaError(std::string("cudaMallocAsync: ") + cudaGetErrorString(e), (int)e);
  }
  p = static_cast<T*>(q);
  n = count;
  ctx = c;
  s = st;
}

template <class T>
void DBuf<T>::grow(pi_ctx* c, cudaStream_t st, size_t count, size_t keep) {
  if (count <= n) return;
  T* old = p;
  size_t oldn = n;
  pi_ctx* oc = ctx;
  cudaStream_t os = s;
  p = nullptr;
  n = 0;
  alloc(c, st, count);
  if (old) {
    keep = keep < oldn ? keep : oldn;  // never past the old allocation
    if (keep) PI_CUDA(cudaMemcpyAsync(p, old, keep * sizeof(T), cudaMemcpyDeviceToDevice, st));
    cudaFreeAsync(old, os);
    ctx_account(oc, -(long long)(oldn * sizeof(T)));
  }
}

template <class T>
void DBuf<T>::release() {
  if (p) {
    cudaFreeAsync(p, s);
    ctx_account(ctx, -(long long)(n * sizeof(T)));
  }
  p = nullptr;
  n = 0;
}

template struct DBuf<float>;
template struct DBuf<float4>;
template struct DBuf<int>;
template struct DBuf<int4>;
template struct DBuf<int2>;
template struct DBuf<unsigned>;
template struct DBuf<int8_t>;
template struct DBuf<uint64_t>;
template struct DBuf<unsigned long long>;
template struct DBuf<long long>;
template struct DBuf<MultiGridView>;

// Bspline_kernel (src/evaluator.cpp:383-396) with the reference's types:
// float in, polynomial in double, float out.
float bspline_host(float ratio, float sigma) {
  if (ratio < 2) {
    if (ratio <= 1) return (float)(sigma * (1 - 1.5 * std::pow(ratio, 2) + 0.75 * std::pow(ratio, 3)));
    float tmq = 2 - ratio;
    return (float)(sigma * (0.25 * std::pow(tmq, 3)));
  }
  return 0.0f;
}

void counters_reset(pi_frame* f) {
  cudaStream_t s = f->ctx->stream;
  if (f->dcount.n < (size_t)kCounterWords) f->dcount.alloc(f->ctx, s, kCounterWords);
  PI_CUDA(cudaMemsetAsync(f->dcount.p, 0, sizeof(unsigned long long) * kCounterWords, s));
}

void counters_read(pi_frame* f, unsigned long long out[kCounters]) {
  cudaStream_t s = f->ctx->stream;
  std::vector<unsigned long long> h(kCounterWords);
  PI_CUDA(cudaMemcpyAsync(h.data(), f->dcount.p, sizeof(unsigned long long) * kCounterWords,
                          cudaMemcpyDeviceToHost, s));
  PI_CUDA(cudaStreamSynchronize(s));
  for (int w = 0; w < kCounters; ++w) {
    out[w] = 0;
    for (int k = 0; k < kStripes; ++k) out[w] += h[((size_t)w * kStripes + k) * 4];
  }
}

void counters_snapshot(pi_frame* f, int slot) {
  PI_CUDA(cudaMemcpyAsync(f->ctx->hpin + (size_t)slot * kCounterWords, f->dcount.p,
                          sizeof(unsigned long long) * kCounterWords, cudaMemcpyDeviceToHost, f->ctx->stream));
  f->pin_pending |= 1 << slot;
}

static void fold_counters(const unsigned long long* h, unsigned long long out[kCounters]) {
  for (int w = 0; w < kCounters; ++w) {
    out[w] = 0;
    for (int k = 0; k < kStripes; ++k) out[w] += h[((size_t)w * kStripes + k) * 4];
  }
}

void resolve_pending(pi_frame* f) {
  qef_join(f);
  topology_join(f);
  if (!f->ev_pending && !f->pin_pending) return;
  PI_CUDA(cudaStreamSynchronize(f->ctx->stream));
  for (int k = 0; k < 8; ++k)
    if (f->ev_pending & (1 << k)) {
      float ms = 0;
      PI_CUDA(cudaEventElapsedTime(&ms, f->ev[2 * k], f->ev[2 * k + 1]));
      f->stage_ms[k] += ms;
    }
  f->ev_pending = 0;
  const unsigned long long* h = f->ctx->hpin;
  unsigned long long c[kCounters];
  pi_ctx* ctx = f->ctx;
  if (f->pin_pending & (1 << kPinAniso)) {
    fold_counters(h + (size_t)kPinAniso * kCounterWords, c);
    f->fp64Count = (long long)c[0];
  }
  if (f->pin_pending & (1 << kPinOctree)) {
    fold_counters(h + (size_t)kPinOctree * kCounterWords, c);
    // the reference's NodeCalcNode evaluates the field at the leaf's node
    // point whether or not its vertex is accepted (src/iso_method_ours.cpp:
    // 161-173): one more reference call per leaf solved
    f->fieldEvals = (long long)(c[C_REF_EVALS] + c[C_QEF_LEAVES]);
    f->doneEvals = (long long)(c[C_DONE_CHUNK] + c[C_DONE_THREAD] + c[C_DONE_LEAF] + c[C_QEF_EVALS]);
    f->pairs = (long long)c[C_SAMPLE_PAIRS];
    f->qefAccepted = (long long)c[C_QEF_ACCEPTED];
    f->qefSingular = (long long)c[C_QEF_SINGULAR];
    if (c[C_STAGE_TIMEOUT])
      throw CudaError("a bulk-staging wait of the field evaluation ran out; the frame's values are void", 0);
    if (ctx->profile) {
      ctx->group_pairs[PG_CHUNK] += (int64_t)c[C_PAIRS_CHUNK];
      ctx->group_pairs[PG_THREAD] += (int64_t)c[C_PAIRS_THREAD];
      ctx->group_pairs[PG_LEAF] += (int64_t)c[C_PAIRS_LEAF];
      ctx->group_units[PG_CHUNK] += (int64_t)c[C_DONE_CHUNK];
      ctx->group_units[PG_THREAD] += (int64_t)c[C_DONE_THREAD];
      ctx->group_units[PG_LEAF] += (int64_t)c[C_DONE_LEAF];
      ctx->group_units[PG_QEF] += (int64_t)c[C_QEF_LEAVES];
    }
  }
  if (f->pin_pending & (1 << kPinExtract)) {
    fold_counters(h + (size_t)kPinExtract * kCounterWords, c);
    f->nDual = (long long)c[C_DUAL];
    f->bisectEvals = (long long)c[C_BISECT_EVALS];
    f->fieldEvals += (long long)c[C_BISECT_EVALS];
    f->doneEvals += (long long)c[C_BISECT_EVALS];
    f->pairs += (long long)c[C_BISECT_PAIRS];
    if (ctx->profile) {
      ctx->group_pairs[PG_BISECT] += (int64_t)c[C_BISECT_PAIRS];
      ctx->group_units[PG_BISECT] += (int64_t)c[C_BISECT_EVALS];
    }
  }
  if (f->pin_pending & (1 << kPinValid)) {
    const int valid = *reinterpret_cast<const int*>(h + (size_t)kPinSlots * kCounterWords);
    f->g.nInvalid = (int)(f->N - valid);
  }
  f->pin_pending = 0;
}

void prof_begin(pi_ctx* c, cudaStream_t s, int g) {
  if (!c->profile) return;
  cudaEvent_t e;
  PI_CUDA(cudaEventCreate(&e));
  PI_CUDA(cudaEventRecord(e, s));
  c->prof_events[g].push_back(e);
}
void prof_end(pi_ctx* c, cudaStream_t s, int g) {
  if (!c->profile) return;
  cudaEvent_t e;
  PI_CUDA(cudaEventCreate(&e));
  PI_CUDA(cudaEventRecord(e, s));
  c->prof_events[g].push_back(e);
  c->group_launches[g]++;
}

// Reads every pending event pair into the group times.
static void prof_collect(pi_ctx* c) {
  for (int g = 0; g < kProfGroups; ++g) {
    auto& ev = c->prof_events[g];
    for (size_t i = 0; i + 1 < ev.size(); i += 2) {
      float t = 0;
      PI_CUDA(cudaEventElapsedTime(&t, ev[i], ev[i + 1]));
      c->group_ms[g] += t;
    }
    for (auto e : ev) cudaEventDestroy(e);
    ev.clear();
  }
}

// resizeRootBoxConstR (src/surface_reconstructor.cpp:97-122),
// CalculateMaxScalarConstR / RecommendIsoValueConstR (src/evaluator.cpp:272-335)
static void host_root_and_scalars(pi_frame* f) {
  const float r = f->P.radius;
  const float* bb = f->bbox6;
  float maxLen = std::max({(bb[1] - bb[0]), (bb[3] - bb[2]), (bb[5] - bb[4])});
  // all particles at one point: log2(0) would make the reference's depth
  // undefined; the search then starts at depth 0
  const float cells = std::ceil(maxLen / r);
  int dmax = cells >= 1.0f ? int(std::ceil(std::log2(cells))) : 0;
  float resizeLen = (float)(std::pow(2, dmax) * r);
  while (resizeLen - maxLen < (4.0f * r * 2)) {
    dmax++;
    resizeLen = (float)(std::pow(2, dmax) * r);
  }
  f->rootH = resizeLen / 2;
  for (int i = 0; i < 3; ++i) f->rootC[i] = (bb[i * 2] + bb[i * 2 + 1]) / 2;
  f->dmax = dmax;
  f->dmin = dmax - (f->singleLayer ? 1 : 3);
  const float sqrt2 = 1.4142135623730950488016887242097f;
  const float sqrt3 = 1.7320508075688772935274463415059f;
  float k = 0;
  k += bspline_host(0.0f, f->sigma);
  k += bspline_host(1.0f, f->sigma) * 6;
  k += bspline_host(sqrt2, f->sigma) * 12;
  k += bspline_host(sqrt3, f->sigma) * 8;
  f->maxScalar = k;
  f->iso = bspline_host((float)0.01, f->sigma);
}

static void ev_record(pi_frame* f, int i) {
  if (!f->ev[i]) PI_CUDA(cudaEventCreate(&f->ev[i]));
  PI_CUDA(cudaEventRecord(f->ev[i], f->ctx->stream));
}
// Stage slot k's time is read by resolve_pending, at the end of the API call
// (or, for an upload, at the next one that synchronises).
static void ev_close(pi_frame* f, int stage_slot) { f->ev_pending |= 1 << stage_slot; }

static void need(const pi_frame* f, int stage) {
  if (f->stage < stage) throw StateError("stage called before the stages it depends on");
}

// The uniform grid, the box query and the FP64 oracle are built for one
// hash grid (a constant radius).
static void const_radius_only(const pi_frame* f) {
  if (f->varR) throw StateError("not available with per-particle radii");
}

// An NVTX range per stage (names as the reference's printf stage titles), so
// a timeline tool shows the stages; free when no tool is attached.
struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
};

static void run_stage(pi_frame* f, int target) {
  // target: 2 hash, 3 aniso, 4 normals, 5 octree, 6 mesh
  if (f->stage >= target) return;
  need(f, target - 1);
  static const char* const names[7] = {"", "", "pisurf hash grid", "pisurf anisotropy", "pisurf normals",
                                        "pisurf octree", "pisurf extraction"};
  NvtxRange range(names[target]);
  const int slot = target == 2 ? 1 : target == 3 ? 2 : target == 4 ? 3 : target == 5 ? 4 : 6;
  ev_record(f, 2 * slot);
  switch (target) {
    case 2:
      if (f->varR)
        stage_hashgrid_vr(f);
      else
        stage_hashgrid(f);
      break;
    case 3:
      if (f->varR)
        stage_aniso_vr(f);
      else
        stage_aniso(f);
      break;
    case 4:
      if (f->varR)
        host_root_and_scalars_vr(f);
      else
        host_root_and_scalars(f);
      if (f->P.max_depth > 0 && f->dmax > f->P.max_depth)
        throw std::length_error("octree depth " + std::to_string(f->dmax) + " exceeds max_depth " +
                                std::to_string(f->P.max_depth));
      stage_normals(f);
      break;
    case 5:
      stage_octree(f);
      break;
    case 6:
      stage_extract(f);
      break;
  }
  ev_record(f, 2 * slot + 1);
  ev_close(f, slot);
  f->stage = target;
}

void check_params(const pi_params* p) {
  if (!(std::isfinite(p->radius) && p->radius > 0)) throw std::invalid_argument("radius must be positive");
  if (!(std::isfinite(p->smooth_factor) && p->smooth_factor > 0))
    throw std::invalid_argument("smooth_factor must be positive");
  if (p->splash != 0 && p->splash != 1) throw std::invalid_argument("splash must be 0 or 1");
}

// Back to `stage` (0: nothing uploaded, 1: particles uploaded) with every
// result and counter cleared; device buffers are kept for reuse.
void frame_clear(pi_frame* f, int stage) {
  qef_join(f);
  topology_join(f);
  f->stage = stage;
  f->f64_ready = false;
  f->nNodes = f->nV = f->nT = f->nDual = 0;
  f->fieldEvals = f->pairs = f->bisectEvals = f->fp64Count = f->nLeaves = f->nEmpty = 0;
  f->doneEvals = 0;
  f->qefAccepted = f->qefSingular = 0;
  f->nSplash = 0;
  f->ev_pending = f->pin_pending = 0;
  for (int k = 0; k < 8; ++k) f->stage_ms[k] = 0;
}

}  // namespace pisurf

using namespace pisurf;

#define PI_API_BEGIN try {
#define PI_API_END                                 \
  }                                                \
  catch (const NoMem& e) {                         \
    g_last_error = e.what();                       \
    return PI_ERR_NOMEM;                           \
  }                                                \
  catch (const StateError& e) {                    \
    g_last_error = e.what();                       \
    return PI_ERR_STATE;                           \
  }                                                \
  catch (const CudaError& e) {                     \
    g_last_error = e.what();                       \
    return PI_ERR_CUDA;                            \
  }                                                \
  catch (const std::invalid_argument& e) {         \
    g_last_error = e.what();                       \
    return PI_ERR_INVALID;                         \
  }                                                \
  catch (const std::length_error& e) {             \
    g_last_error = e.what();                       \
    return PI_ERR_LIMIT;                           \
  }                                                \
  catch (const std::bad_alloc& e) {                \
    g_last_error = "host allocation failed";       \
    return PI_ERR_NOMEM;                           \
  }                                                \
  catch (const std::exception& e) {                \
    g_last_error = e.what();                       \
    return PI_ERR_CUDA;                            \
  }                                                \
  return PI_OK;

#define PI_CHECK(cond, msg)                 \
  do {                                      \
    if (!(cond)) throw std::invalid_argument(msg); \
  } while (0)

static void set_device(pi_ctx* c) { PI_CUDA(cudaSetDevice(c->device)); }

template <class T>
static std::vector<T> d2h(const T* d, size_t n, cudaStream_t s) {
  std::vector<T> h(n);
  if (n) PI_CUDA(cudaMemcpyAsync(h.data(), d, sizeof(T) * n, cudaMemcpyDeviceToHost, s));
  PI_CUDA(cudaStreamSynchronize(s));
  return h;
}


extern "C" {

const char* pi_last_error(void) { return g_last_error.c_str(); }
const char* pi_version(void) { return "particleisosurface_gb300 0.1 (sm_103a)"; }

void pi_params_default(pi_params* p) {
  if (!p) return;
  std::memset(p, 0, sizeof(*p));
  p->radius = 0.01f;
  p->smooth_factor = 2.0f;
  p->iso_factor = 1.9f;
  p->qef = 0;
  p->max_depth = 0;
}

int pi_ctx_create(int device, size_t budget_bytes, pi_ctx** out) {
  PI_API_BEGIN
  PI_CHECK(out, "out is null");
  *out = nullptr;
  int ndev = 0;
  PI_CUDA(cudaGetDeviceCount(&ndev));
  PI_CHECK(device >= 0 && device < ndev, "no such CUDA device");
  std::unique_ptr<pi_ctx> c(new pi_ctx());
  c->device = device;
  c->budget = budget_bytes;
  PI_CUDA(cudaSetDevice(device));
  PI_CUDA(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
  PI_CUDA(cudaDeviceGetAttribute(&c->smCount, cudaDevAttrMultiProcessorCount, device));
  PI_CUDA(cudaMallocHost(&c->hpin, sizeof(unsigned long long) * (size_t)kPinWords));
  PI_CUDA(cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking));
  PI_CUDA(cudaStreamCreateWithFlags(&c->qef_stream, cudaStreamNonBlocking));
  PI_CUDA(cudaStreamCreateWithFlags(&c->topo_stream, cudaStreamNonBlocking));
  PI_CUDA(cudaEventCreateWithFlags(&c->ev_topo_in, cudaEventDisableTiming));
  PI_CUDA(cudaEventCreateWithFlags(&c->ev_topo_done, cudaEventDisableTiming));
  PI_CUDA(cudaEventCreateWithFlags(&c->ev_topo_read, cudaEventDisableTiming));
  PI_CUDA(cudaEventCreateWithFlags(&c->ev_qef_in, cudaEventDisableTiming));
  PI_CUDA(cudaEventCreateWithFlags(&c->ev_qef_done, cudaEventDisableTiming));
  c->coop_blocks = top_levels_grid(device, c->smCount);
  PI_CUDA(cudaEventCreateWithFlags(&c->ev_tris_ready, cudaEventDisableTiming));
  PI_CUDA(cudaEventCreateWithFlags(&c->ev_tris_copied, cudaEventDisableTiming));
  PI_CUDA(cudaEventCreateWithFlags(&c->ev_read, cudaEventDisableTiming));
  cudaMemPool_t pool;
  PI_CUDA(cudaDeviceGetDefaultMemPool(&pool, device));
  uint64_t thr = UINT64_MAX;
  PI_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr));
  *out = c.release();
  PI_API_END
}

static void ctx_release(pi_ctx* c) {
  if (c->refs.fetch_sub(1) != 1) return;
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  if (c->topo_stream) {
    cudaStreamSynchronize(c->topo_stream);
    cudaStreamDestroy(c->topo_stream);
  }
  for (cudaEvent_t e : {c->ev_topo_in, c->ev_topo_done, c->ev_topo_read})
    if (e) cudaEventDestroy(e);
  for (auto& ev : c->prof_events)
    for (auto e : ev) cudaEventDestroy(e);
  if (c->hpin) cudaFreeHost(c->hpin);
  if (c->copy_stream) {
    cudaStreamSynchronize(c->copy_stream);
    cudaStreamDestroy(c->copy_stream);
  }
  if (c->qef_stream) {
    cudaStreamSynchronize(c->qef_stream);
    cudaStreamDestroy(c->qef_stream);
  }
  if (c->ev_qef_in) cudaEventDestroy(c->ev_qef_in);
  if (c->ev_qef_done) cudaEventDestroy(c->ev_qef_done);
  if (c->ev_tris_ready) cudaEventDestroy(c->ev_tris_ready);
  if (c->ev_tris_copied) cudaEventDestroy(c->ev_tris_copied);
  if (c->ev_read) cudaEventDestroy(c->ev_read);
  cudaStreamDestroy(c->stream);
  (void)cudaGetLastError();
  delete c;
}

int pi_ctx_destroy(pi_ctx* c) {
  PI_API_BEGIN
  if (!c) return PI_OK;
  if (c->recon) {
    pi_frame* r = c->recon;
    c->recon = nullptr;
    pi_frame_destroy(r);
  }
  // frames still alive keep the context (and its stream) until they are destroyed
  ctx_release(c);
  PI_API_END
}

int pi_ctx_stats(const pi_ctx* c, uint64_t* launches, uint64_t* bytes) {
  PI_API_BEGIN
  PI_CHECK(c, "ctx is null");
  if (launches) *launches = g_launches.load(std::memory_order_relaxed);
  if (bytes) *bytes = (uint64_t)c->used.load();
  PI_API_END
}

int pi_ctx_profile(pi_ctx* c, int enable) {
  PI_API_BEGIN
  PI_CHECK(c, "ctx is null");
  c->profile = enable != 0;
  PI_API_END
}

int pi_ctx_kernel_time(pi_ctx* c, double* total_ms, int64_t* launches, int64_t* pairs, int64_t* evals) {
  PI_API_BEGIN
  PI_CHECK(c, "ctx is null");
  set_device(c);
  PI_CUDA(cudaStreamSynchronize(c->stream));
  prof_collect(c);
  // field evaluation at octree samples: the chunked, per-sample and
  // leaf-value groups together
  double ms = 0;
  int64_t l = 0, p = 0, u = 0;
  for (int g : {PG_CHUNK, PG_THREAD, PG_LEAF}) {
    ms += c->group_ms[g];
    l += c->group_launches[g];
    p += c->group_pairs[g];
    u += c->group_units[g];
    c->group_ms[g] = 0;
    c->group_launches[g] = c->group_pairs[g] = c->group_units[g] = 0;
  }
  if (total_ms) *total_ms = ms;
  if (launches) *launches = l;
  if (pairs) *pairs = p;
  if (evals) *evals = u;
  PI_API_END
}

int pi_ctx_kernel_groups(pi_ctx* c, int32_t ngroups, double* ms, int64_t* launches, int64_t* pairs,
                         int64_t* units) {
  PI_API_BEGIN
  PI_CHECK(c && ms && launches && pairs && units, "null argument");
  PI_CHECK(ngroups >= 1 && ngroups <= kProfGroups, "ngroups out of range");
  set_device(c);
  PI_CUDA(cudaStreamSynchronize(c->stream));
  prof_collect(c);
  for (int g = 0; g < ngroups; ++g) {
    ms[g] = c->group_ms[g];
    launches[g] = c->group_launches[g];
    pairs[g] = c->group_pairs[g];
    units[g] = c->group_units[g];
    c->group_ms[g] = 0;
    c->group_launches[g] = c->group_pairs[g] = c->group_units[g] = 0;
  }
  PI_API_END
}

void* pi_ctx_stream(pi_ctx* c) { return c ? (void*)c->stream : nullptr; }

int pi_ctx_tune(pi_ctx* c, int32_t samples_per_lane) {
  PI_API_BEGIN
  PI_CHECK(c, "ctx is null");
  PI_CHECK(samples_per_lane == 0 || samples_per_lane == 1 || samples_per_lane == 2 || samples_per_lane == 4,
           "samples per lane must be 0, 1, 2 or 4");
  c->eval_forced = samples_per_lane;
  c->eval_cfg[0] = c->eval_cfg[1] = 0;
  PI_API_END
}

int pi_ctx_tuning(const pi_ctx* c, int32_t* out2) {
  PI_API_BEGIN
  PI_CHECK(c && out2, "null argument");
  for (int k = 0; k < 2; ++k)
    out2[k] = c->eval_forced ? c->eval_forced : c->eval_cfg[k] ? kEvalTable[c->eval_cfg[k] - 1].K : 0;
  PI_API_END
}

int pi_ctx_tune_config(pi_ctx* c, int32_t index) {
  PI_API_BEGIN
  PI_CHECK(c, "ctx is null");
  PI_CHECK(index >= -1 && index < kEvalConfigs, "configuration index out of range");
  c->eval_forced = 0;
  c->eval_cfg[0] = c->eval_cfg[1] = index + 1;
  PI_API_END
}

int pi_ctx_tune_qef_parts(pi_ctx* c, int32_t parts) {
  PI_API_BEGIN
  PI_CHECK(c, "ctx is null");
  PI_CHECK(parts >= 1 && parts <= kMaxQefParts, "QEF parts out of range");
  c->qef_parts = parts;
  PI_API_END
}

int pi_ctx_qef_parts(const pi_ctx* c, int32_t* out) {
  PI_API_BEGIN
  PI_CHECK(c && out, "null argument");
  *out = c->qef_parts;
  PI_API_END
}

int pi_ctx_tuning_config(const pi_ctx* c, int32_t* out8) {
  PI_API_BEGIN
  PI_CHECK(c && out8, "null argument");
  for (int k = 0; k < 2; ++k) {
    int cfg = c->eval_cfg[k] - 1;
    if (c->eval_forced) cfg = c->eval_forced == 1 ? 0 : c->eval_forced == 2 ? 1 : 2;
    out8[4 * k] = cfg >= 0 ? kEvalTable[cfg].K : 0;
    out8[4 * k + 1] = cfg >= 0 ? kEvalTable[cfg].W : 0;
    out8[4 * k + 2] = cfg >= 0 ? kEvalTable[cfg].CB : 0;
    out8[4 * k + 3] = cfg >= 0 ? kEvalTable[cfg].bulk : 0;
  }
  PI_API_END
}

int pi_eval_configs(void) { return kEvalConfigs; }

int pi_frame_create(pi_ctx* c, const pi_params* p, pi_frame** out) {
  PI_API_BEGIN
  PI_CHECK(c && p && out, "null argument");
  check_params(p);
  *out = nullptr;
  pi_frame* f = new pi_frame();
  f->ctx = c;
  f->P = *p;
  c->refs.fetch_add(1);
  *out = f;
  PI_API_END
}

int pi_frame_destroy(pi_frame* f) {
  PI_API_BEGIN
  if (!f) return PI_OK;
  pi_ctx* c = f->ctx;
  set_device(c);
  qef_join(f);  // the frees below follow any QEF work in flight
  topology_fence(f);  // and the topology stream's frees follow the context stream's work
  for (auto& e : f->ev)
    if (e) cudaEventDestroy(e);
  delete f;  // device buffers are freed on the context stream
  ctx_release(c);
  PI_API_END
}

int pi_frame_upload(pi_frame* f, const float* xyz, int64_t n) {
  PI_API_BEGIN
  PI_CHECK(f && xyz && n > 0, "bad upload arguments");
  PI_CHECK(n < (1LL << 31), "more than 2^31 particles");
  set_device(f->ctx);
  ev_record(f, 0);
  stage_upload_host(f, xyz, n);
  ev_record(f, 1);
  ev_close(f, 0);
  f->stage = 1;
  f->varR = false;
  PI_API_END
}

int pi_frame_upload_radii(pi_frame* f, const float* radii, int64_t n) {
  PI_API_BEGIN
  PI_CHECK(f && radii && n > 0, "bad radii arguments");
  need(f, 1);
  set_device(f->ctx);
  stage_upload_radii(f, radii, n);
  frame_clear(f, 1);
  PI_API_END
}

int pi_frame_grid(const pi_frame* f, int32_t k, float* bounding6, int32_t* dims3, float* cell_size, int64_t* count,
                  int64_t* offset_base, int32_t* radius_id) {
  PI_API_BEGIN
  PI_CHECK(f && bounding6 && dims3 && cell_size && count && offset_base && radius_id, "null argument");
  need(f, 2);
  if (!f->varR) {
    PI_CHECK(k == 0, "no such grid");
    for (int q = 0; q < 6; ++q) bounding6[q] = f->g.bounding[q];
    dims3[0] = f->g.nx, dims3[1] = f->g.ny, dims3[2] = f->g.nz;
    *cell_size = f->g.cell;
    *count = f->N;
    *offset_base = 0;
    *radius_id = -1;
  } else {
    PI_CHECK(k >= 0 && k < (int)f->bins.size(), "no such grid");
    const BinHost& b = f->bins[k];
    for (int q = 0; q < 6; ++q) bounding6[q] = b.bounding[q];
    dims3[0] = b.nx, dims3[1] = b.ny, dims3[2] = b.nz;
    *cell_size = b.cell;
    *count = b.count;
    *offset_base = b.offBase;
    *radius_id = b.radius_id;
  }
  PI_API_END
}

int pi_frame_upload_device(pi_frame* f, const float* d_xyz, int64_t n) {
  PI_API_BEGIN
  PI_CHECK(f && d_xyz && n > 0, "bad upload arguments");
  PI_CHECK(n < (1LL << 31), "more than 2^31 particles");
  set_device(f->ctx);
  stage_upload_device(f, d_xyz, n);
  f->stage = 1;
  f->varR = false;
  PI_API_END
}

int pi_frame_reset(pi_frame* f) {
  PI_API_BEGIN
  PI_CHECK(f, "frame is null");
  need(f, 1);
  frame_clear(f, 1);
  PI_API_END
}

int pi_hashgrid_build(pi_frame* f) {
  PI_API_BEGIN
  PI_CHECK(f, "frame is null");
  set_device(f->ctx);
  run_stage(f, 2);
  resolve_pending(f);
  PI_API_END
}
int pi_aniso_compute(pi_frame* f) {
  PI_API_BEGIN
  PI_CHECK(f, "frame is null");
  set_device(f->ctx);
  run_stage(f, 3);
  resolve_pending(f);
  PI_API_END
}
int pi_normals_compute(pi_frame* f) {
  PI_API_BEGIN
  PI_CHECK(f, "frame is null");
  set_device(f->ctx);
  run_stage(f, 4);
  resolve_pending(f);
  PI_API_END
}
int pi_octree_build(pi_frame* f) {
  PI_API_BEGIN
  PI_CHECK(f, "frame is null");
  set_device(f->ctx);
  run_stage(f, 5);
  resolve_pending(f);
  PI_API_END
}
int pi_extract_mesh(pi_frame* f) {
  PI_API_BEGIN
  PI_CHECK(f, "frame is null");
  set_device(f->ctx);
  run_stage(f, 6);
  resolve_pending(f);
  PI_API_END
}
// One JSON line per completed frame, appended to the file named by the
// PISURF_METRICS environment variable (unset: nothing is written).  The
// reference prints its stage times and frontier sizes instead
// (src/surface_reconstructor.cpp:322-470).
static void metrics_record(const pi_frame* f) {
  static const char* path = std::getenv("PISURF_METRICS");
  if (!path || !*path) return;
  static std::mutex mu;
  std::lock_guard<std::mutex> lk(mu);
  FILE* fp = std::fopen(path, "a");
  if (!fp) return;
  std::fprintf(fp,
               "{\"particles\": %lld, \"depth_max\": %d, \"nodes\": %lld, \"leaves\": %lld, "
               "\"dual_cells\": %lld, \"vertices\": %lld, \"triangles\": %lld, \"field_evals\": %lld, "
               "\"field_evals_performed\": %lld, \"candidate_pairs\": %lld, \"qef_accepted\": %lld, "
               "\"stage_ms\": {\"hash\": %.4f, \"aniso\": %.4f, \"normals\": %.4f, \"octree\": %.4f, "
               "\"qef\": %.4f, \"extract\": %.4f}}\n",
               f->N, f->dmax, f->nNodes, f->nLeaves, f->nDual, f->nV, f->nT, f->fieldEvals, f->doneEvals, f->pairs,
               f->qefAccepted, f->stage_ms[1], f->stage_ms[2], f->stage_ms[3], f->stage_ms[4], f->stage_ms[5],
               f->stage_ms[6]);
  std::fclose(fp);
}

int pi_run(pi_frame* f) {
  PI_API_BEGIN
  PI_CHECK(f, "frame is null");
  set_device(f->ctx);
  need(f, 1);
  const bool fresh = f->stage < 6;
  // the octree's last QEF level may overlap the extraction's topology
  f->defer_qef_join = true;
  f->extract_follows = true;
  try {
    for (int t = 2; t <= 6; ++t) run_stage(f, t);
  } catch (...) {
    f->defer_qef_join = f->extract_follows = false;
    topology_join(f);
    throw;
  }
  f->defer_qef_join = f->extract_follows = false;
  resolve_pending(f);
  if (fresh) metrics_record(f);
  PI_API_END
}

int pi_frame_info_get(const pi_frame* f, pi_frame_info* o) {
  PI_API_BEGIN
  PI_CHECK(f && o, "null argument");
  resolve_pending(const_cast<pi_frame*>(f));
  std::memset(o, 0, sizeof(*o));
  o->num_particles = f->N;
  o->num_invalid_keys = f->g.nInvalid;
  for (int k = 0; k < 6; ++k) o->bounding[k] = f->g.bounding[k];
  o->cell_size = f->g.cell;
  o->xyz_cell_num[0] = f->g.nx;
  o->xyz_cell_num[1] = f->g.ny;
  o->xyz_cell_num[2] = f->g.nz;
  o->cell_num = f->g.cellNum;
  o->depth_max = f->dmax;
  o->depth_min = f->dmin;
  for (int k = 0; k < 3; ++k) o->root_center[k] = f->rootC[k];
  o->root_half = f->rootH;
  o->iso_value = f->iso;
  o->max_scalar = f->maxScalar;
  o->influence2 = f->influ2;
  o->sigma = f->sigma;
  o->num_nodes = f->nNodes;
  o->num_leaves = f->nLeaves;
  o->num_empty = f->nEmpty;
  o->num_dual_cells = f->nDual;
  o->num_vertices = f->nV;
  o->num_triangles = f->nT;
  o->field_evals = f->fieldEvals;
  o->candidate_pairs = f->pairs;
  o->bisection_evals = f->bisectEvals;
  o->fp64_eigen = f->fp64Count;
  for (int k = 0; k < 8; ++k) o->stage_ms[k] = f->stage_ms[k];
  o->qef_accepted = f->qefAccepted;
  o->qef_singular = f->qefSingular;
  o->grid_pairs = f->gridPairs;
  o->field_evals_performed = f->doneEvals;
  o->num_grids = f->varR ? (int32_t)f->bins.size() : (f->stage >= 2 ? 1 : 0);
  o->radius_min = f->varR ? f->vrMinR : f->P.radius;
  o->radius_max = f->varR ? f->vrMaxR : f->P.radius;
  o->num_splash = f->nSplash;
  PI_API_END
}

int pi_mesh_counts(const pi_frame* f, int64_t* nv, int64_t* nt) {
  PI_API_BEGIN
  PI_CHECK(f && nv && nt, "null argument");
  need(f, 6);
  *nv = f->nV;
  *nt = f->nT;
  PI_API_END
}

int pi_mesh_get(pi_frame* f, float* verts, int32_t* tris, uint64_t* vkeys) {
  PI_API_BEGIN
  PI_CHECK(f, "frame is null");
  need(f, 6);
  set_device(f->ctx);
  cudaStream_t s = f->ctx->stream;
  if (verts && f->nV) PI_CUDA(cudaMemcpyAsync(verts, f->mv.p, sizeof(float) * 3 * f->nV, cudaMemcpyDeviceToHost, s));
  if (tris && f->nT) PI_CUDA(cudaMemcpyAsync(tris, f->mt.p, sizeof(int) * 3 * f->nT, cudaMemcpyDeviceToHost, s));
  if (vkeys && f->nV)
    PI_CUDA(cudaMemcpyAsync(vkeys, f->mk.p, sizeof(uint64_t) * 2 * f->nV, cudaMemcpyDeviceToHost, s));
  PI_CUDA(cudaStreamSynchronize(s));
  PI_API_END
}

int pi_mesh_write_obj(pi_frame* f, const char* path) {
  PI_API_BEGIN
  PI_CHECK(f && path, "null argument");
  need(f, 6);
  std::vector<float> v(3 * f->nV);
  std::vector<int> t(3 * f->nT);
  int rc = pi_mesh_get(f, v.data(), t.data(), nullptr);
  if (rc) return rc;
  FILE* fp = std::fopen(path, "w");
  PI_CHECK(fp, "cannot open output file");
  for (long long i = 0; i < f->nV; ++i) std::fprintf(fp, "v %f %f %f\n", v[3 * i], v[3 * i + 1], v[3 * i + 2]);
  for (long long i = 0; i < f->nT; ++i) std::fprintf(fp, "f %d %d %d\n", t[3 * i] + 1, t[3 * i + 1] + 1, t[3 * i + 2] + 1);
  std::fclose(fp);
  PI_API_END
}

int pi_fp64_aniso(pi_frame* f, double* xmeans3, double* g9, double* det) {
  PI_API_BEGIN
  PI_CHECK(f, "frame is null");
  need(f, 2);
  const_radius_only(f);
  set_device(f->ctx);
  fp64_aniso_get(f, xmeans3, g9, det);
  PI_API_END
}

int pi_fp64_eval_field(pi_frame* f, const float* pts, int64_t m, double* scalar, double* grad) {
  PI_API_BEGIN
  PI_CHECK(f && pts && scalar && m > 0, "bad arguments");
  need(f, 2);
  const_radius_only(f);
  set_device(f->ctx);
  cudaStream_t s = f->ctx->stream;
  DBuf<float> dp;
  DBuf<double> dv, dg;
  dp.alloc(f->ctx, s, m * 3);
  dv.alloc(f->ctx, s, m);
  if (grad) dg.alloc(f->ctx, s, m * 3);
  PI_CUDA(cudaMemcpyAsync(dp.p, pts, sizeof(float) * 3 * m, cudaMemcpyHostToDevice, s));
  fp64_eval(f, dp.p, m, dv.p, grad ? dg.p : nullptr);
  PI_CUDA(cudaMemcpyAsync(scalar, dv.p, sizeof(double) * m, cudaMemcpyDeviceToHost, s));
  if (grad) PI_CUDA(cudaMemcpyAsync(grad, dg.p, sizeof(double) * 3 * m, cudaMemcpyDeviceToHost, s));
  PI_CUDA(cudaStreamSynchronize(s));
  PI_API_END
}

int pi_fp64_scalars(const pi_frame* f, double* out4) {
  PI_API_BEGIN
  PI_CHECK(f && out4, "null argument");
  fp64_scalars(f, out4);
  PI_API_END
}

int pi_eval_field(pi_frame* f, const float* pts, int64_t m, float* scalar, float* grad) {
  PI_API_BEGIN
  PI_CHECK(f && pts && scalar && m > 0, "bad arguments");
  need(f, 4);
  set_device(f->ctx);
  cudaStream_t s = f->ctx->stream;
  DBuf<float> dp, dv, dg;
  dp.alloc(f->ctx, s, m * 3);
  dv.alloc(f->ctx, s, m);
  if (grad) dg.alloc(f->ctx, s, m * 3);
  PI_CUDA(cudaMemcpyAsync(dp.p, pts, sizeof(float) * 3 * m, cudaMemcpyHostToDevice, s));
  eval_points(f, dp.p, m, dv.p, grad ? dg.p : nullptr);
  PI_CUDA(cudaMemcpyAsync(scalar, dv.p, sizeof(float) * m, cudaMemcpyDeviceToHost, s));
  if (grad) PI_CUDA(cudaMemcpyAsync(grad, dg.p, sizeof(float) * 3 * m, cudaMemcpyDeviceToHost, s));
  PI_CUDA(cudaStreamSynchronize(s));
  PI_API_END
}

int pi_grid_dims(pi_frame* f, int32_t* dims3, float* box6, int64_t* npoints) {
  PI_API_BEGIN
  PI_CHECK(f && dims3, "bad arguments");
  need(f, 2);
  const_radius_only(f);
  float box[6];
  int steps[3], dims[3];
  uniform_grid_host(f, box, steps, dims);
  for (int i = 0; i < 3; ++i) dims3[i] = dims[i];
  if (box6)
    for (int i = 0; i < 6; ++i) box6[i] = box[i];
  if (npoints) *npoints = (int64_t)dims[0] * dims[1] * dims[2];
  PI_API_END
}

int pi_grid_sample_device(pi_frame* f, float* d_values, int64_t cap) {
  PI_API_BEGIN
  PI_CHECK(f && d_values, "bad arguments");
  need(f, 4);
  const_radius_only(f);
  set_device(f->ctx);
  const long long total = grid_sample(f, d_values, cap);
  if (total > cap) throw std::length_error("value buffer too small for the lattice");
  PI_API_END
}

int pi_grid_sample(pi_frame* f, float* values, int64_t cap) {
  PI_API_BEGIN
  PI_CHECK(f && values, "bad arguments");
  need(f, 4);
  const_radius_only(f);
  set_device(f->ctx);
  cudaStream_t s = f->ctx->stream;
  const long long total = grid_sample(f, nullptr, 0);
  if (total > cap) throw std::length_error("value buffer too small for the lattice");
  DBuf<float> dv;
  dv.alloc(f->ctx, s, total);
  grid_sample(f, dv.p, total);
  PI_CUDA(cudaMemcpyAsync(values, dv.p, sizeof(float) * total, cudaMemcpyDeviceToHost, s));
  PI_CUDA(cudaStreamSynchronize(s));
  PI_API_END
}

int pi_grid_write_vti(pi_frame* f, const char* path) {
  PI_API_BEGIN
  PI_CHECK(f && path, "bad arguments");
  need(f, 4);
  const_radius_only(f);
  set_device(f->ctx);
  float box[6];
  int steps[3], dims[3];
  uniform_grid_host(f, box, steps, dims);
  const long long total = (long long)dims[0] * dims[1] * dims[2];
  std::vector<float> v((size_t)total);
  {
    cudaStream_t s = f->ctx->stream;
    DBuf<float> dv;
    dv.alloc(f->ctx, s, total);
    grid_sample(f, dv.p, total);
    PI_CUDA(cudaMemcpyAsync(v.data(), dv.p, sizeof(float) * total, cudaMemcpyDeviceToHost, s));
    PI_CUDA(cudaStreamSynchronize(s));
  }
  FILE* fp = std::fopen(path, "wb");
  if (!fp) throw std::invalid_argument(std::string("cannot open ") + path);
  const float r = f->P.radius;
  std::fprintf(fp,
               "<?xml version=\"1.0\"?>\n"
               "<VTKFile type=\"ImageData\" version=\"1.0\" byte_order=\"LittleEndian\" header_type=\"UInt64\">\n"
               "  <ImageData WholeExtent=\"0 %d 0 %d 0 %d\" Origin=\"%.9g %.9g %.9g\" Spacing=\"%.9g %.9g %.9g\">\n"
               "    <Piece Extent=\"0 %d 0 %d 0 %d\">\n"
               "      <PointData Scalars=\"scalars\">\n"
               "        <DataArray type=\"Float32\" Name=\"scalars\" format=\"appended\" offset=\"0\"/>\n"
               "      </PointData>\n"
               "    </Piece>\n"
               "  </ImageData>\n"
               "  <AppendedData encoding=\"raw\">\n_",
               dims[0] - 1, dims[1] - 1, dims[2] - 1, box[0], box[2], box[4], r, r, r, dims[0] - 1, dims[1] - 1,
               dims[2] - 1);
  const uint64_t nbytes = sizeof(float) * (uint64_t)total;
  unsigned char hdr[8];
  for (int k = 0; k < 8; ++k) hdr[k] = (unsigned char)((nbytes >> (8 * k)) & 0xffu);
  std::fwrite(hdr, 1, 8, fp);
  std::vector<unsigned char> le((size_t)nbytes);
  for (long long i = 0; i < total; ++i) {
    uint32_t u;
    std::memcpy(&u, &v[(size_t)i], 4);
    for (int k = 0; k < 4; ++k) le[(size_t)i * 4 + k] = (unsigned char)((u >> (8 * k)) & 0xffu);
  }
  std::fwrite(le.data(), 1, le.size(), fp);
  std::fprintf(fp, "\n  </AppendedData>\n</VTKFile>\n");
  const bool ok = std::ferror(fp) == 0;
  std::fclose(fp);
  if (!ok) throw std::invalid_argument(std::string("write failed: ") + path);
  PI_API_END
}

int pi_load_csv(const char* path, float* xyz, float* radius, int64_t cap, int64_t* n, int32_t* cols4) {
  PI_API_BEGIN
  PI_CHECK(path && n, "bad arguments");
  int cols[4];
  const long long rows = load_csv(path, xyz, radius, xyz ? cap : 0, cols);
  *n = rows;
  if (cols4)
    for (int i = 0; i < 4; ++i) cols4[i] = cols[i];
  if (xyz && rows > cap) throw std::length_error("buffer holds fewer rows than the file");
  PI_API_END
}

int pi_load_hdf5(const char* path, float* xyz, float* radius, int64_t cap, int64_t* n) {
  PI_API_BEGIN
  PI_CHECK(path && n, "bad arguments");
  long long rows = 0;
  *n = 0;
  try {
    load_hdf5(path, xyz, radius, xyz ? cap : 0, radius != nullptr, &rows);
  } catch (...) {
    *n = rows;
    throw;
  }
  *n = rows;
  PI_API_END
}

int pi_hdf5_dataset(const char* path, const char* name, double* out, int64_t cap, int64_t* count,
                    int64_t* dims8, int32_t* rank) {
  PI_API_BEGIN
  PI_CHECK(path && name && count, "bad arguments");
  std::vector<uint64_t> dims;
  const std::vector<double> v = load_hdf5_dataset(path, name, &dims);
  *count = (int64_t)v.size();
  if (rank) *rank = (int32_t)dims.size();
  if (dims8)
    for (size_t i = 0; i < dims.size() && i < 8; ++i) dims8[i] = (int64_t)dims[i];
  if (out) {
    if ((int64_t)v.size() > cap) throw std::length_error("buffer holds fewer values than the dataset");
    std::memcpy(out, v.data(), sizeof(double) * v.size());
  }
  PI_API_END
}

int pi_load_xdmf(const char* dir, const char* xdmf_file, int32_t target_frame, char* out, int64_t cap,
                 int64_t* len, int32_t* frames) {
  PI_API_BEGIN
  PI_CHECK(dir && xdmf_file && len, "bad arguments");
  const std::vector<std::string> v = load_xdmf(dir, xdmf_file, target_frame);
  std::string s;
  for (size_t i = 0; i < v.size(); ++i) s += (i ? "\n" : "") + v[i];
  *len = (int64_t)s.size() + 1;
  if (frames) *frames = (int32_t)v.size();
  if (out) {
    if (*len > cap) throw std::length_error("buffer too small for the frame list");
    std::memcpy(out, s.c_str(), s.size() + 1);
  }
  PI_API_END
}

int pi_write_ply(const char* path, const float* verts, int64_t nv, const int32_t* tris, int64_t nt,
                 int32_t one_based) {
  PI_API_BEGIN
  PI_CHECK(path && nv >= 0 && nt >= 0 && (verts || nv == 0) && (tris || nt == 0), "bad arguments");
  write_ply(path, verts, nv, tris, nt, one_based);
  PI_API_END
}

int pi_mesh_write_ply(pi_frame* f, const char* path) {
  PI_API_BEGIN
  PI_CHECK(f && path, "bad arguments");
  need(f, 6);
  set_device(f->ctx);
  cudaStream_t s = f->ctx->stream;
  std::vector<float> v((size_t)f->nV * 3);
  std::vector<int32_t> t((size_t)f->nT * 3);
  if (f->nV) PI_CUDA(cudaMemcpyAsync(v.data(), f->mv.p, sizeof(float) * v.size(), cudaMemcpyDeviceToHost, s));
  if (f->nT) PI_CUDA(cudaMemcpyAsync(t.data(), f->mt.p, sizeof(int32_t) * t.size(), cudaMemcpyDeviceToHost, s));
  PI_CUDA(cudaStreamSynchronize(s));
  write_ply(path, v.data(), f->nV, t.data(), f->nT, 0);
  PI_API_END
}

int pi_hashgrid_neighbors(pi_frame* f, const float* pts, int64_t m, int64_t* offsets, int32_t* idx, int64_t cap,
                          int64_t* total) {
  PI_API_BEGIN
  PI_CHECK(f && pts && offsets && total && m > 0, "bad arguments");
  need(f, 2);
  set_device(f->ctx);
  std::vector<long long> off(m + 1);
  long long t = neighbors(f, pts, m, off.data(), idx, idx ? cap : 0);
  for (long long i = 0; i <= m; ++i) offsets[i] = off[i];
  *total = t;
  if (t > cap) throw std::length_error("neighbour buffer too small");
  PI_API_END
}

int pi_hashgrid_in_box(pi_frame* f, const float* b1, const float* b2, int32_t* idx, int64_t cap, int64_t* total) {
  PI_API_BEGIN
  PI_CHECK(f && b1 && b2 && total, "bad arguments");
  need(f, 2);
  const_radius_only(f);
  set_device(f->ctx);
  long long t = in_box(f, b1, b2, idx, idx ? cap : 0);
  *total = t;
  if (t > cap) throw std::length_error("index buffer too small");
  PI_API_END
}

static size_t dump_size(const pi_frame* f, int what) {
  switch (what) {
    case PI_DUMP_KEYS: return sizeof(int64_t) * f->N;
    case PI_DUMP_INDEX_LIST: return sizeof(int32_t) * f->N;
    case PI_DUMP_CELL_OFFSETS: return sizeof(int32_t) * (f->varR ? f->off.n : f->g.cellNum + 1);
    case PI_DUMP_GRID_OF: return sizeof(int32_t) * f->N;
    case PI_DUMP_XMEANS: return sizeof(float) * 3 * f->N;
    case PI_DUMP_G: return sizeof(float) * 9 * f->N;
    case PI_DUMP_DET: return sizeof(float) * f->N;
    case PI_DUMP_NORMALS: return sizeof(float) * 3 * f->N;
    case PI_DUMP_NODES: return sizeof(pi_node) * f->nNodes;
    case PI_DUMP_FP64_FLAGS: return sizeof(int8_t) * f->N;
    case PI_DUMP_SPLASH: return sizeof(int8_t) * f->N;
    case PI_DUMP_VERTEX_EDGES: return sizeof(int32_t) * 2 * f->nV;
    case PI_DUMP_QEF_SAMPLES: return f->P.qef ? sizeof(float) * 27 * f->nNodes : 0;
  }
  return 0;
}

int pi_stage_dump_size(const pi_frame* f, int what, size_t* bytes) {
  PI_API_BEGIN
  PI_CHECK(f && bytes, "null argument");
  *bytes = dump_size(f, what);
  PI_CHECK(*bytes || what == PI_DUMP_NODES, "unknown dump");
  PI_API_END
}

int pi_stage_dump(pi_frame* f, int what, void* buf, size_t bytes) {
  PI_API_BEGIN
  PI_CHECK(f && buf, "null argument");
  size_t need_b = dump_size(f, what);
  PI_CHECK(bytes >= need_b, "dump buffer too small");
  set_device(f->ctx);
  cudaStream_t s = f->ctx->stream;
  const long long N = f->N;
  auto sorted_to_orig = [&](const std::vector<float>& src, int w, float* dst) {
    std::vector<uint32_t> sidx = d2h(f->sidx.p, N, s);
    for (long long t = 0; t < N; ++t)
      for (int k = 0; k < w; ++k) dst[(size_t)sidx[t] * w + k] = src[(size_t)t * w + k];
  };
  switch (what) {
    case PI_DUMP_KEYS: {
      need(f, 2);
      auto k = d2h(f->key.p, N, s);
      int64_t* o = (int64_t*)buf;
      for (long long i = 0; i < N; ++i) o[i] = k[i];
      break;
    }
    case PI_DUMP_INDEX_LIST: {
      need(f, 2);
      auto k = d2h(f->sidx.p, N, s);
      std::memcpy(buf, k.data(), sizeof(int32_t) * N);
      break;
    }
    case PI_DUMP_CELL_OFFSETS: {
      need(f, 2);
      const size_t m = f->varR ? f->off.n : (size_t)f->g.cellNum + 1;
      auto k = d2h(f->off.p, m, s);
      std::memcpy(buf, k.data(), sizeof(int32_t) * m);
      break;
    }
    case PI_DUMP_GRID_OF: {
      need(f, 2);
      if (f->varR) {
        auto k = d2h(f->pbin.p, N, s);
        std::memcpy(buf, k.data(), sizeof(int32_t) * N);
      } else {
        std::memset(buf, 0, sizeof(int32_t) * N);
      }
      break;
    }
    case PI_DUMP_XMEANS: {
      need(f, 3);
      auto x = d2h(f->xm.p, N, s);
      std::vector<float> v(3 * N);
      for (long long t = 0; t < N; ++t) v[3 * t] = x[t].x, v[3 * t + 1] = x[t].y, v[3 * t + 2] = x[t].z;
      sorted_to_orig(v, 3, (float*)buf);
      break;
    }
    case PI_DUMP_G: {
      need(f, 3);
      sorted_to_orig(d2h(f->gfull.p, 9 * N, s), 9, (float*)buf);
      break;
    }
    case PI_DUMP_DET: {
      need(f, 3);
      sorted_to_orig(d2h(f->det.p, N, s), 1, (float*)buf);
      break;
    }
    case PI_DUMP_NORMALS: {
      need(f, 4);
      auto x = d2h(f->nrm.p, N, s);
      std::vector<float> v(3 * N);
      for (long long t = 0; t < N; ++t) v[3 * t] = x[t].x, v[3 * t + 1] = x[t].y, v[3 * t + 2] = x[t].z;
      sorted_to_orig(v, 3, (float*)buf);
      break;
    }
    case PI_DUMP_VERTEX_EDGES: {
      need(f, 6);
      if (f->nV) PI_CUDA(cudaMemcpyAsync(buf, f->vedge.p, sizeof(int2) * f->nV, cudaMemcpyDeviceToHost, s));
      PI_CUDA(cudaStreamSynchronize(s));
      break;
    }
    case PI_DUMP_SPLASH: {
      need(f, 3);
      int8_t* o = (int8_t*)buf;
      if (!f->P.splash) {
        std::memset(o, 0, N);
        break;
      }
      auto x = d2h(f->spl.p, N, s);
      std::vector<uint32_t> sidx = d2h(f->sidx.p, N, s);
      for (long long t = 0; t < N; ++t) o[sidx[t]] = x[t];
      break;
    }
    case PI_DUMP_FP64_FLAGS: {
      need(f, 3);
      auto x = d2h(f->f64flag.p, N, s);
      std::vector<uint32_t> sidx = d2h(f->sidx.p, N, s);
      int8_t* o = (int8_t*)buf;
      for (long long t = 0; t < N; ++t) o[sidx[t]] = x[t];
      break;
    }
    case PI_DUMP_NODES: {
      need(f, 5);
      const long long n = f->nNodes;
      auto c = d2h(f->nd_c.p, n, s);
      auto v = d2h(f->nd_v.p, n, s);
      auto id = d2h(f->nd_id.p, n, s);
      auto par = d2h(f->nd_parent.p, n, s);
      auto ch = d2h(f->nd_child.p, n, s);
      auto ty = d2h(f->nd_type.p, n, s);
      auto de = d2h(f->nd_depth.p, n, s);
      auto sc = d2h(f->nd_sc.p, n, s);
      auto cu = d2h(f->nd_curv.p, n, s);
      pi_node* o = (pi_node*)buf;
      for (long long i = 0; i < n; ++i) {
        o[i].id = id[i];
        o[i].center[0] = c[i].x, o[i].center[1] = c[i].y, o[i].center[2] = c[i].z;
        o[i].half = c[i].w;
        o[i].node[0] = v[i].x, o[i].node[1] = v[i].y, o[i].node[2] = v[i].z, o[i].node[3] = v[i].w;
        o[i].curv = cu[i];
        o[i].parent = par[i];
        o[i].first_child = ch[i];
        o[i].depth = de[i];
        o[i].type = ty[i];
        o[i].signchange = sc[i];
        o[i].pad = 0;
      }
      break;
    }
    case PI_DUMP_QEF_SAMPLES: {
      need(f, 5);
      PI_CHECK(f->P.qef, "QEF samples exist only in qef mode");
      auto x = d2h(f->nd_samp.p, 27 * f->nNodes, s);
      std::memcpy(buf, x.data(), sizeof(float) * 27 * f->nNodes);
      break;
    }
    default:
      throw std::invalid_argument("unknown dump");
  }
  PI_API_END
}

int pi_reconstruct(pi_ctx* c, const pi_params* p, const float* xyz, int64_t n, float* verts, int64_t max_verts,
                   int32_t* tris, int64_t max_tris, int64_t* nverts, int64_t* ntris) {
  PI_API_BEGIN
  PI_CHECK(c && p && xyz && nverts && ntris, "null argument");
  check_params(p);
  // without a budget the context keeps this call's frame for the next one,
  // so that its device buffers and events carry over; with a budget the
  // frame's memory is returned at the end of the call
  const bool keep = c->budget == 0;
  pi_frame* f = nullptr;
  if (keep && c->recon) {
    f = c->recon;
    f->P = *p;
    frame_clear(f, 0);
  } else {
    int rc = pi_frame_create(c, p, &f);
    if (rc) return rc;
    if (keep) c->recon = f;
  }
  struct Guard {
    pi_frame* f;
    bool keep;
    ~Guard() {
      // the triangle copy reads the frame and writes the caller's buffer:
      // it ends before the call does, on every path
      if (f->tris_sent) cudaEventSynchronize(f->ctx->ev_tris_copied);
      f->host_tris = nullptr;
      f->host_tcap = 0;
      f->tris_sent = false;
      if (!keep) pi_frame_destroy(f);
    }
  } guard{f, keep};
  f->host_tris = tris;
  f->host_tcap = tris ? max_tris : 0;
  f->tris_sent = false;
  int rc = 0;
  rc = pi_frame_upload(f, xyz, n);
  if (rc) return rc;
  rc = pi_run(f);
  if (rc) return rc;
  *nverts = f->nV;
  *ntris = f->nT;
  if (f->nV > max_verts || f->nT > max_tris) throw std::length_error("mesh buffers too small");
  rc = pi_mesh_get(f, verts, f->tris_sent ? nullptr : tris, nullptr);
  if (rc) return rc;
  PI_API_END
}

int pi_dmc_table(int32_t* trans, int8_t* flip, int32_t* code) {
  PI_API_BEGIN
  PI_CHECK(trans && flip && code, "null argument");
  int t[256][8], c[256];
  bool fl[256];
  dmc_host_table(t, fl, c);
  for (int i = 0; i < 256; ++i) {
    for (int k = 0; k < 8; ++k) trans[8 * i + k] = t[i][k];
    flip[i] = fl[i] ? 1 : 0;
    code[i] = c[i];
  }
  PI_API_END
}

}  // extern "C"
