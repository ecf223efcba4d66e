// Exclusive scan and stable LSD radix sort.
//
// Used to order particles into hash cells (a stable sort by cell key keeps
// particle-index order inside a cell), to build the dense cell offset table,
// to compact octree frontiers and to deduplicate dual-grid vertices, mesh
// vertices and triangles.
//
// Scan: reduce -> single-block top scan -> down-sweep, tiles of 2048 ints.
// Radix sort: 8-bit digits; per pass a per-tile digit histogram, an exclusive
// scan of the digit-major histogram table, and a scatter in which each tile
// ranks its keys stably with warp match masks.  No kernel waits on another
// block, so nothing can spin.
#include "common.cuh"

namespace pisurf {

std::atomic<unsigned long long> g_launches{0};

static constexpr int kThreads = 256;
static constexpr int kItems = 8;
static constexpr int kTile = kThreads * kItems;

__device__ __forceinline__ int warp_incl_scan(int v) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int n = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += n;
  }
  return v;
}

// Block-wide exclusive scan of one int per thread (blockDim.x == 256 or
// 1024); returns the exclusive prefix and writes the block total.
template <int NT>
__device__ __forceinline__ int block_excl_scan(int v, int* s_warp, int* total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int inc = warp_incl_scan(v);
  if (lane == 31) s_warp[warp] = inc;
  __syncthreads();
  if (warp == 0) {
    int w = lane < NT / 32 ? s_warp[lane] : 0;
    int wi = warp_incl_scan(w);
    if (lane < NT / 32) s_warp[lane] = wi - w;
    if (lane == NT / 32 - 1) *total = wi;
  }
  __syncthreads();
  int r = inc - v + s_warp[warp];
  __syncthreads();
  return r;
}

__global__ void k_scan_reduce(const int* __restrict__ in, long long n, int* __restrict__ sums) {
  __shared__ int s_warp[32];
  __shared__ int s_total;
  long long base = (long long)blockIdx.x * kTile;
  int acc = 0;
#pragma unroll
  for (int i = 0; i < kItems; ++i) {
    long long idx = base + (long long)i * kThreads + threadIdx.x;
    if (idx < n) acc += in[idx];
  }
  block_excl_scan<kThreads>(acc, s_warp, &s_total);
  if (threadIdx.x == 0) sums[blockIdx.x] = s_total;
}

__global__ void k_scan_top(int* __restrict__ sums, int nb, int* __restrict__ d_total) {
  __shared__ int s_warp[32];
  __shared__ int s_total;
  int carry = 0;
  for (int base = 0; base < nb; base += 1024) {
    int i = base + threadIdx.x;
    int v = i < nb ? sums[i] : 0;
    int ex = block_excl_scan<1024>(v, s_warp, &s_total);
    if (i < nb) sums[i] = ex + carry;
    carry += s_total;
    __syncthreads();
  }
  if (threadIdx.x == 0 && d_total) *d_total = carry;
}

// Tile index with one padding word per 32, so that a thread's run of
// kItems consecutive elements and a warp's coalesced row both fall in
// distinct banks.
__device__ __forceinline__ int tpad(int i) { return i + (i >> 5); }

// Down-sweep of one tile: the block's exclusive scan plus the tile's offset
// (sums[blockIdx.x]; 0 when sums is null, the single-tile case, which also
// writes the total to *d_total when given).
__global__ void k_scan_down(const int* __restrict__ in, int* __restrict__ out, long long n,
                            const int* __restrict__ sums, int* __restrict__ d_total) {
  __shared__ int s_tile[kTile + kTile / 32];
  __shared__ int s_warp[32];
  __shared__ int s_total;
  long long base = (long long)blockIdx.x * kTile;
#pragma unroll
  for (int i = 0; i < kItems; ++i) {
    long long idx = base + (long long)i * kThreads + threadIdx.x;
    s_tile[tpad(i * kThreads + threadIdx.x)] = idx < n ? in[idx] : 0;
  }
  __syncthreads();
  int loc[kItems];
  int acc = 0;
#pragma unroll
  for (int i = 0; i < kItems; ++i) {
    loc[i] = acc;
    acc += s_tile[tpad(threadIdx.x * kItems + i)];
  }
  int ex = block_excl_scan<kThreads>(acc, s_warp, &s_total) + (sums ? sums[blockIdx.x] : 0);
  if (!sums && d_total && threadIdx.x == 0) *d_total = s_total;
#pragma unroll
  for (int i = 0; i < kItems; ++i) s_tile[tpad(threadIdx.x * kItems + i)] = ex + loc[i];
  __syncthreads();
#pragma unroll
  for (int i = 0; i < kItems; ++i) {
    long long idx = base + (long long)i * kThreads + threadIdx.x;
    if (idx < n) out[idx] = s_tile[tpad(i * kThreads + threadIdx.x)];
  }
}

size_t scan_tmp_ints(long long n) { return (size_t)div_up(n > 0 ? n : 1, kTile) + 32; }

void exclusive_scan_i32(const int* in, int* out, long long n, int* d_total, int* tmp,
                        cudaStream_t s) {
  if (n <= 0) {
    if (d_total) PI_CUDA(cudaMemsetAsync(d_total, 0, sizeof(int), s));
    return;
  }
  unsigned nb = div_up(n, kTile);
  if (nb == 1) {  // one tile: one launch
    PI_LAUNCH(k_scan_down, 1, kThreads, 0, s, in, out, n, nullptr, d_total);
    return;
  }
  PI_LAUNCH(k_scan_reduce, nb, kThreads, 0, s, in, n, tmp);
  PI_LAUNCH(k_scan_top, 1, 1024, 0, s, tmp, (int)nb, d_total);
  PI_LAUNCH(k_scan_down, nb, kThreads, 0, s, in, out, n, tmp, nullptr);
}

// ---------------------------------------------------------------------------
// radix sort
// ---------------------------------------------------------------------------
template <class K>
__global__ void k_rs_hist(const K* __restrict__ keys, long long n, int shift, int* __restrict__ hist,
                          int nt) {
  __shared__ int h[256];
  h[threadIdx.x] = 0;
  __syncthreads();
  long long base = (long long)blockIdx.x * kTile;
#pragma unroll
  for (int i = 0; i < kItems; ++i) {
    long long idx = base + (long long)i * kThreads + threadIdx.x;
    if (idx < n) atomicAdd(&h[(int)((keys[idx] >> shift) & 255)], 1);
  }
  __syncthreads();
  hist[(long long)threadIdx.x * nt + blockIdx.x] = h[threadIdx.x];
}

template <class K>
__global__ void k_rs_scatter(const K* __restrict__ kin, const uint32_t* __restrict__ vin,
                             K* __restrict__ kout, uint32_t* __restrict__ vout, long long n, int shift,
                             const int* __restrict__ offs, int nt) {
  __shared__ int run[256];
  __shared__ int wc[kThreads / 32][256];
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  run[t] = offs[(long long)t * nt + blockIdx.x];
#pragma unroll
  for (int w = 0; w < kThreads / 32; ++w) wc[w][t] = 0;
  __syncthreads();
  const unsigned lt = (1u << lane) - 1u;
  long long base = (long long)blockIdx.x * kTile;
  for (int r = 0; r < kItems; ++r) {
    long long idx = base + (long long)r * kThreads + t;
    bool valid = idx < n;
    K key = valid ? kin[idx] : K(0);
    uint32_t val = valid ? vin[idx] : 0u;
    int d = valid ? (int)((key >> shift) & 255) : 256;
    unsigned peers = __match_any_sync(0xffffffffu, d);
    int leader = __ffs(peers) - 1;
    int rank = __popc(peers & lt);
    int cnt = __popc(peers);
    if (valid && lane == leader) wc[warp][d] = cnt;
    __syncthreads();
    if (valid) {
      int pos = run[d] + rank;
      for (int w = 0; w < warp; ++w) pos += wc[w][d];
      kout[pos] = key;
      vout[pos] = val;
    }
    __syncthreads();
    if (valid && lane == leader) {
      atomicAdd(&run[d], cnt);
      wc[warp][d] = 0;
    }
    __syncthreads();
  }
}

size_t radix_tmp_ints(long long n) {
  size_t nt = div_up(n > 0 ? n : 1, kTile);
  return 256 * nt + scan_tmp_ints((long long)(256 * nt)) + 32;
}

template <class K>
static void radix_sort(K** keys, uint32_t** vals, K** kalt, uint32_t** valt, long long n, int bits,
                       int* tmp, cudaStream_t s) {
  if (n <= 1 || bits <= 0) return;
  int nt = (int)div_up(n, kTile);
  int* hist = tmp;
  int* stmp = tmp + 256 * (size_t)nt;
  for (int shift = 0; shift < bits; shift += 8) {
    PI_LAUNCH(k_rs_hist<K>, nt, kThreads, 0, s, *keys, n, shift, hist, nt);
    exclusive_scan_i32(hist, hist, 256LL * nt, nullptr, stmp, s);
    PI_LAUNCH(k_rs_scatter<K>, nt, kThreads, 0, s, *keys, *vals, *kalt, *valt, n, shift, hist, nt);
    std::swap(*keys, *kalt);
    std::swap(*vals, *valt);
  }
}

void radix_sort_u32(uint32_t** keys, uint32_t** vals, uint32_t** kalt, uint32_t** valt, long long n,
                    int bits, int* tmp, cudaStream_t s) {
  radix_sort<uint32_t>(keys, vals, kalt, valt, n, bits, tmp, s);
}
void radix_sort_u64(uint64_t** keys, uint32_t** vals, uint64_t** kalt, uint32_t** valt, long long n,
                    int bits, int* tmp, cudaStream_t s) {
  radix_sort<uint64_t>(keys, vals, kalt, valt, n, bits, tmp, s);
}

__global__ void k_iota(uint32_t* v, long long n) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) v[i] = (uint32_t)i;
}
void iota_u32(uint32_t* v, long long n, cudaStream_t s) {
  PI_LAUNCH(k_iota, div_up(n, 256), 256, 0, s, v, n);
}

}  // namespace pisurf
