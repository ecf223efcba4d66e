// Shared device/host helpers for the particle-isosurface CUDA library.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <cstdio>
#include <stdexcept>
#include <string>

namespace pisurf {

// Library-wide count of kernel launches (read by pi_ctx_stats).  Launches
// come from many host threads at once (the request loop's workers, one
// caller thread per frame), so the count is atomic; relaxed order suffices
// for a statistic.
extern std::atomic<unsigned long long> g_launches;
inline void count_launch() { g_launches.fetch_add(1ull, std::memory_order_relaxed); }

struct CudaError : std::runtime_error {
  int code;
  CudaError(const std::string& s, int c) : std::runtime_error(s), code(c) {}
};

// Throws on failure after clearing the runtime's last-error slot, so that a
// failed call is reported once and does not surface again at a later launch.
#define PI_CUDA(call)                                                                   \
  do {                                                                                  \
    cudaError_t _e = (call);                                                            \
    if (_e != cudaSuccess) {                                                            \
      (void)cudaGetLastError();                                                         \
      throw ::pisurf::CudaError(std::string(#call) + ": " + cudaGetErrorString(_e) +    \
                                    " (" + __FILE__ + ":" + std::to_string(__LINE__) + \
                                    ")",                                                \
                                (int)_e);                                               \
    }                                                                                   \
  } while (0)

// Launch wrapper: counts the launch and checks the launch error.
#define PI_LAUNCH(kernel, grid, block, smem, stream, ...)                 \
  do {                                                                    \
    if ((grid) > 0) {                                                     \
      kernel<<<(grid), (block), (smem), (stream)>>>(__VA_ARGS__);         \
      ::pisurf::count_launch();                                           \
      PI_CUDA(cudaGetLastError());                                        \
    }                                                                     \
  } while (0)

inline unsigned int div_up(long long a, long long b) { return (unsigned int)((a + b - 1) / b); }

// The reference compares floats with double literals (the float promoted to
// double): `cellsize - r < 1e-8`, `curv < 0.99` (src/surface_reconstructor.cpp:
// 247,262) and the 0.1 / 0.9 snap of the bisection (src/visitorextract.cpp:
// 71-80).  None of these literals is a float, so for a float x each
// comparison equals one float comparison with the float next to the literal:
// (double)x < d  <=>  x < (smallest float above d), and
// (double)x > d  <=>  x > (largest float below d).
// This keeps the decisions off the FP64 pipe, which is narrow on this GPU.
constexpr float kAbove1em8 = 0x1.5798fp-27f;  // smallest float above 1e-8
constexpr float kAbove099 = 0x1.fae148p-1f;   // smallest float above 0.99
constexpr float kAbove01 = 0x1.99999ap-4f;    // smallest float above 0.1
constexpr float kBelow09 = 0x1.ccccccp-1f;    // largest float below 0.9

// Striped device event counters (see stripe_add in device.cuh): kCounters
// counters x 64 stripes, 32 bytes apart.
constexpr int kStripes = 64;
enum Counter : int {
  C_REF_EVALS = 0,     // SingleEval calls the reference makes for octree samples and leaf values
  C_SAMPLE_PAIRS = 1,  // candidate pairs of every octree sampling kernel
  C_DUAL = 2,          // dual cells
  C_BISECT_EVALS = 3,  // bisection midpoints evaluated (one chain per mesh vertex)
  C_BISECT_PAIRS = 4,  // their candidate pairs
  C_QEF_ACCEPTED = 5,
  C_QEF_SINGULAR = 6,
  C_QEF_EVALS = 7,     // SingleEval at accepted QEF vertices
  C_PAIRS_CHUNK = 8,   // candidate pairs of the chunked sampling kernel (k_q_eval)
  C_PAIRS_THREAD = 9,  // ... of the per-sample kernel (k_q_eval_thread)
  C_PAIRS_LEAF = 10,   // ... of the leaf-value kernel (k_leaf_level)
  C_DONE_CHUNK = 11,   // evaluations performed by k_q_eval (distinct samples)
  C_QEF_LEAVES = 12,   // leaves whose QEF k_qef solved
  C_DONE_THREAD = 13,  // evaluations performed by k_q_eval_thread (distinct samples)
  C_DONE_LEAF = 14,    // evaluations performed by k_leaf_level (one per leaf)
  C_STAGE_TIMEOUT = 15,  // bulk-staging waits that ran out (an error: the frame's values are void)
  kCounters = 16
};
constexpr int kCounterWords = kCounters * kStripes * 4;

// Kernel groups timed with CUDA events when a context profiles (roofline
// reporting): field evaluation at octree samples in chunks (k_q_eval), one
// thread per sample (k_q_eval_thread), leaf values (k_leaf_level); edge
// bisection (k_bisect); the FP64 QEF (k_qef); the uniform-grid sampler
// (k_grid_eval).
enum ProfGroup : int { PG_CHUNK = 0, PG_THREAD = 1, PG_LEAF = 2, PG_BISECT = 3, PG_QEF = 4, PG_GRID = 5, kProfGroups = 6 };

// ---------------------------------------------------------------------------
// Scan (exclusive, int32) and stable LSD radix sort (u32/u64 keys, u32
// values).  Implemented in sort.cu.
// ---------------------------------------------------------------------------
struct Workspace;  // forward

// out[i] = sum_{k<i} in[i]; returns nothing; total written to *d_total if
// non-null.  in and out may alias.  tmp must hold scan_tmp_ints(n) ints.
size_t scan_tmp_ints(long long n);
void exclusive_scan_i32(const int* in, int* out, long long n, int* d_total, int* tmp,
                        cudaStream_t s);

// Sorts (keys, vals) by the bits [0, bits) of the key, stably.  Uses
// keys_alt/vals_alt as ping-pong buffers; the sorted result is returned in
// the pointers *keys/*vals (which may be swapped with the alt buffers).
// tmp must hold radix_tmp_ints(n) ints.
size_t radix_tmp_ints(long long n);
void radix_sort_u32(uint32_t** keys, uint32_t** vals, uint32_t** keys_alt, uint32_t** vals_alt,
                    long long n, int bits, int* tmp, cudaStream_t s);
void radix_sort_u64(uint64_t** keys, uint32_t** vals, uint64_t** keys_alt, uint32_t** vals_alt,
                    long long n, int bits, int* tmp, cudaStream_t s);

// iota: v[i] = i
void iota_u32(uint32_t* v, long long n, cudaStream_t s);

}  // namespace pisurf
