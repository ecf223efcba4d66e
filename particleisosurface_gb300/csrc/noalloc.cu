// Hash-grid build that allocates no device memory.
//
// Some host programs cannot let a library allocate GPU memory once they are
// running: a solver that reserves the whole device for its own pool at
// start-up (any further cudaMalloc then fails), or a control loop whose
// latency budget forbids the allocator's first-touch stalls and whose rules
// ban allocation after initialisation.  pi_hashgrid_build_noalloc serves them:
// the caller passes device buffers for the particles and for every output,
// and the temporaries of the build (sort keys, ping-pong buffers, digit
// histograms, scan partials, bounding-box words) live in g_noalloc_scratch, a
// fixed array in this library's device image.  Each GPU that loads the
// library holds that array (12.5 MiB) until the process exits.
//
// The array is shared by every call on a device and keeps whatever the last
// call left in it.  Nothing in it needs to start at zero: each word the build
// reads was written earlier in the same call.  The caller's cell-offset
// output is cleared by the call.  Two calls whose GPU work overlaps (different
// streams, no ordering between them) race on the array and corrupt each other.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>

#include "internal.h"

namespace pisurf {

// Kernels of the regular hash-grid build (grid.cu), reused unchanged.
__global__ void k_bbox(const float* __restrict__ xyz, long long n, unsigned* __restrict__ misc);
__global__ void k_init_misc(unsigned* misc);
__global__ void k_keys(const float* __restrict__ xyz, long long n, float b0, float b2, float b4, float cell,
                       int nx, int ny, int nz, int* __restrict__ key, uint32_t* __restrict__ skey,
                       uint32_t* __restrict__ sidx);
__global__ void k_cell_count(const int* __restrict__ key, long long n, int* __restrict__ cnt);

static constexpr long long kMaxParticles = PI_NOALLOC_MAX_PARTICLES;
static constexpr long long kMaxCells = PI_NOALLOC_MAX_CELLS;
static constexpr long long kTileItems = 2048;  // sort.cu tile
static constexpr long long kTiles = (kMaxParticles + kTileItems - 1) / kTileItems;
static constexpr long long kRadixTmp = 256 * kTiles + ((256 * kTiles + kTileItems - 1) / kTileItems + 32) + 32;
static constexpr long long kScanTmp = (kMaxCells + 1 + kTileItems - 1) / kTileItems + 32;
static constexpr long long kTmpInts = kRadixTmp > kScanTmp ? kRadixTmp : kScanTmp;
// layout in 32-bit words: misc[16] | skey[N] | key_alt[N] | val_alt[N] | tmp
static constexpr long long kMiscWords = 16;
static constexpr long long kScratchWords = kMiscWords + 3 * kMaxParticles + kTmpInts;

static __device__ __align__(256) uint32_t g_noalloc_scratch[kScratchWords];

// Device address of g_noalloc_scratch per device, looked up once with that
// device current.
static uint32_t* scratch_on_current_device() {
  static std::mutex mu;
  static uint32_t* addr[256] = {nullptr};
  int dev = -1;
  PI_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 256) throw std::length_error("device ordinal out of range");
  std::lock_guard<std::mutex> lk(mu);
  if (!addr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess)
      throw CudaError(std::string("cudaGetSymbolAddress(g_noalloc_scratch): ") + cudaGetErrorString(e), (int)e);
    addr[dev] = static_cast<uint32_t*>(p);
  }
  return addr[dev];
}

static float dec_bound(unsigned e) {
  unsigned b = (e & 0x80000000u) ? (e & 0x7fffffffu) : ~e;
  float f;
  std::memcpy(&f, &b, 4);
  return f;
}

extern thread_local std::string g_last_error;

}  // namespace pisurf

using namespace pisurf;

extern "C" int pi_hashgrid_build_noalloc(const float* d_xyz, int64_t n, float radius, int32_t* d_keys,
                                         int32_t* d_index_list, int32_t* d_cell_offsets,
                                         int64_t cell_offsets_len, float* bounding_out6,
                                         int32_t* xyz_cell_num_out3, int64_t* cell_num_out, void* stream) {
  try {
    if (!d_xyz || !d_keys || !d_index_list || !d_cell_offsets || !bounding_out6 || !xyz_cell_num_out3 ||
        !cell_num_out)
      throw std::invalid_argument("null argument");
    if (n <= 0) throw std::invalid_argument("n must be positive");
    if (!(std::isfinite(radius) && radius > 0)) throw std::invalid_argument("radius must be positive");
    if (n > kMaxParticles)
      throw std::length_error("pi_hashgrid_build_noalloc: " + std::to_string(n) + " particles exceed the limit of " +
                              std::to_string(kMaxParticles));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    uint32_t* scr = scratch_on_current_device();
    unsigned* misc = scr;
    uint32_t* skey = scr + kMiscWords;
    uint32_t* kalt = skey + kMaxParticles;
    uint32_t* valt = kalt + kMaxParticles;
    int* tmp = reinterpret_cast<int*>(valt + kMaxParticles);
    if ((long long)radix_tmp_ints(n) > kTmpInts) throw std::length_error("scratch layout too small");

    PI_LAUNCH(k_init_misc, 1, 32, 0, s, misc);
    int dev = 0, sms = 0;
    PI_CUDA(cudaGetDevice(&dev));
    PI_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    int blocks = (int)std::min<long long>(div_up(n, 256), (long long)sms * 8);
    PI_LAUNCH(k_bbox, blocks, 256, 0, s, d_xyz, (long long)n, misc);
    unsigned h[8];
    PI_CUDA(cudaMemcpyAsync(h, misc, sizeof(h), cudaMemcpyDeviceToHost, s));
    PI_CUDA(cudaStreamSynchronize(s));
    if (h[6]) throw std::invalid_argument("non-finite particle coordinate");
    float bb[6];
    for (int k = 0; k < 6; ++k) bb[k] = dec_bound(h[k]);
    // HashGrid ctor (src/hash_grid.cpp:4-34), the same float expressions as the regular build
    const float cell = radius * 4.0f;
    float bounding[6];
    for (int i = 0; i < 3; ++i) {
      float length = (std::ceil((bb[i * 2 + 1] - bb[i * 2]) / cell)) * cell;
      float center = (bb[i * 2] + bb[i * 2 + 1]) / 2;
      bounding[i * 2] = center - length / 2;
      bounding[i * 2 + 1] = center + length / 2;
    }
    for (int k = 0; k < 6; ++k) bounding_out6[k] = bounding[k];
    int nn[3];
    long long cellNum = 0;
    try {
      cellNum = grid_cell_counts(bounding, cell, kMaxCells, nn);
    } catch (const std::length_error& e) {
      *cell_num_out = -1;
      throw std::length_error(std::string("pi_hashgrid_build_noalloc: ") + e.what());
    }
    for (int k = 0; k < 3; ++k) xyz_cell_num_out3[k] = nn[k];
    *cell_num_out = cellNum;
    if (cell_offsets_len < cellNum + 1)
      throw std::length_error("pi_hashgrid_build_noalloc: cell offset buffer needs " +
                              std::to_string(cellNum + 1) + " entries");
    int bits = 0;
    while (bits < 63 && (1LL << bits) <= cellNum + 1) ++bits;

    PI_LAUNCH(k_keys, div_up(n, 256), 256, 0, s, d_xyz, (long long)n, bounding[0], bounding[2], bounding[4], cell,
              nn[0], nn[1], nn[2], d_keys, skey, reinterpret_cast<uint32_t*>(d_index_list));
    uint32_t *k = skey, *v = reinterpret_cast<uint32_t*>(d_index_list), *ka = kalt, *va = valt;
    radix_sort_u32(&k, &v, &ka, &va, n, bits, tmp, s);
    if (v != reinterpret_cast<uint32_t*>(d_index_list))
      PI_CUDA(cudaMemcpyAsync(d_index_list, v, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, s));
    PI_CUDA(cudaMemsetAsync(d_cell_offsets, 0, sizeof(int32_t) * (cellNum + 1), s));
    PI_LAUNCH(k_cell_count, div_up(n, 256), 256, 0, s, d_keys, (long long)n, d_cell_offsets);
    exclusive_scan_i32(d_cell_offsets, d_cell_offsets, cellNum + 1, nullptr, tmp, s);
    PI_CUDA(cudaStreamSynchronize(s));
    return PI_OK;
  } catch (const CudaError& e) {
    g_last_error = e.what();
    return PI_ERR_CUDA;
  } catch (const std::invalid_argument& e) {
    g_last_error = e.what();
    return PI_ERR_INVALID;
  } catch (const std::length_error& e) {
    g_last_error = e.what();
    return PI_ERR_LIMIT;
  } catch (const std::exception& e) {
    g_last_error = e.what();
    return PI_ERR_CUDA;
  }
}
