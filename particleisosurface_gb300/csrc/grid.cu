// K1: hash grid.  loadRootBox (src/surface_reconstructor.cpp:30-49) and the
// constant-radius HashGrid (src/hash_grid.cpp:4-139): bounding box, cell keys,
// stable radix sort of particles by key, dense cell offset table, and the
// gather of positions into cell order.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <stdexcept>
#include <string>

#include "device.cuh"
#include "internal.h"

namespace pisurf {

// Order-preserving float <-> uint encoding for atomic min/max.
__device__ __forceinline__ unsigned fenc(float f) {
  unsigned b = __float_as_uint(f);
  return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
static inline float fdec(unsigned e) {
  unsigned b = (e & 0x80000000u) ? (e & 0x7fffffffu) : ~e;
  float f;
  std::memcpy(&f, &b, 4);
  return f;
}

// misc[0..5] = enc(min x, max x, min y, max y, min z, max z); misc[6] = count
// of non-finite coordinates.
__global__ void k_bbox(const float* __restrict__ xyz, long long n, unsigned* __restrict__ misc) {
  unsigned mn[3] = {0xffffffffu, 0xffffffffu, 0xffffffffu}, mx[3] = {0u, 0u, 0u};
  unsigned bad = 0;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      float v = xyz[3 * i + k];
      if (!isfinite(v)) {
        ++bad;
        continue;
      }
      unsigned e = fenc(v);
      mn[k] = min(mn[k], e);
      mx[k] = max(mx[k], e);
    }
  }
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    for (int o = 16; o > 0; o >>= 1) {
      mn[k] = min(mn[k], __shfl_xor_sync(0xffffffffu, mn[k], o));
      mx[k] = max(mx[k], __shfl_xor_sync(0xffffffffu, mx[k], o));
    }
  }
  for (int o = 16; o > 0; o >>= 1) bad += __shfl_xor_sync(0xffffffffu, bad, o);
  // the block's warps combine in shared memory, so that each block issues one
  // set of atomics (all blocks hit the same seven words)
  __shared__ unsigned s_v[32][7];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) {
    for (int k = 0; k < 3; ++k) {
      s_v[warp][2 * k] = mn[k];
      s_v[warp][2 * k + 1] = mx[k];
    }
    s_v[warp][6] = bad;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const int nw = (blockDim.x + 31) >> 5;
    for (int w = 1; w < nw; ++w)
      for (int k = 0; k < 3; ++k) {
        s_v[0][2 * k] = min(s_v[0][2 * k], s_v[w][2 * k]);
        s_v[0][2 * k + 1] = max(s_v[0][2 * k + 1], s_v[w][2 * k + 1]);
      }
    for (int w = 1; w < nw; ++w) s_v[0][6] += s_v[w][6];
    for (int k = 0; k < 3; ++k) {
      atomicMin(misc + 2 * k, s_v[0][2 * k]);
      atomicMax(misc + 2 * k + 1, s_v[0][2 * k + 1]);
    }
    if (s_v[0][6]) atomicAdd(misc + 6, s_v[0][6]);
  }
}

__global__ void k_init_misc(unsigned* misc) {
  int t = threadIdx.x;
  if (t < 6) misc[t] = (t & 1) ? 0u : 0xffffffffu;
  if (t >= 6 && t < 16) misc[t] = 0;
}

// CalcXYZIdx + CalcCellHash (src/hash_grid.cpp:124-139) per particle; key -1
// outside the grid.  skey = key + 1 so that key -1 sorts first, as the
// reference's std::sort on long long keys does.
__global__ void k_keys(const float* __restrict__ xyz, long long n, float b0, float b2, float b4,
                       float cell, int nx, int ny, int nz, int* __restrict__ key,
                       uint32_t* __restrict__ skey, uint32_t* __restrict__ sidx) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float x = xyz[3 * i], y = xyz[3 * i + 1], z = xyz[3 * i + 2];
  int cx = (int)__fdiv_rn(__fsub_rn(x, b0), cell);
  int cy = (int)__fdiv_rn(__fsub_rn(y, b2), cell);
  int cz = (int)__fdiv_rn(__fsub_rn(z, b4), cell);
  int k = -1;
  if (cx >= 0 && cx < nx && cy >= 0 && cy < ny && cz >= 0 && cz < nz)
    k = (int)(((long long)cz * ny + cy) * nx + cx);
  key[i] = k;
  skey[i] = (uint32_t)(k + 1);
  sidx[i] = (uint32_t)i;
}

__global__ void k_cell_count(const int* __restrict__ key, long long n, int* __restrict__ cnt) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int k = key[i];
  if (k >= 0) atomicAdd(cnt + k, 1);
}

__global__ void k_gather_pos(const float* __restrict__ xyz, const uint32_t* __restrict__ sidx, long long n,
                             float4* __restrict__ pos) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  uint32_t i = sidx[t];
  pos[t] = make_float4(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2], 0.f);
}

void stage_upload_host(pi_frame* f, const float* xyz, long long n) {
  cudaStream_t s = f->ctx->stream;
  f->N = n;
  f->xyz.alloc(f->ctx, s, (size_t)n * 3);
  PI_CUDA(cudaMemcpyAsync(f->xyz.p, xyz, sizeof(float) * 3 * n, cudaMemcpyHostToDevice, s));
}

void stage_upload_device(pi_frame* f, const float* d_xyz, long long n) {
  cudaStream_t s = f->ctx->stream;
  f->N = n;
  f->xyz.alloc(f->ctx, s, (size_t)n * 3);
  PI_CUDA(cudaMemcpyAsync(f->xyz.p, d_xyz, sizeof(float) * 3 * n, cudaMemcpyDeviceToDevice, s));
}

long long grid_cell_counts(const float bounding[6], float cell, long long max_cells, int nn[3]) {
  double total = 1.0;
  for (int i = 0; i < 3; ++i) {
    // XYZCellNum (src/hash_grid.cpp:24-27): ceil of a float quotient; a
    // tiny radius makes it too large for an int, so it is checked as a float
    // (NaN and infinity fail the test too) before the conversion
    const float q = std::ceil((bounding[i * 2 + 1] - bounding[i * 2]) / cell);
    if (!(q <= (float)max_cells))
      throw std::length_error("hash grid axis of " + std::to_string(q) + " cells exceeds the limit of " +
                              std::to_string(max_cells) + " cells (radius too small for the particle box)");
    nn[i] = std::max(int(q), 1);
    total *= nn[i];
  }
  if (total > (double)max_cells)
    throw std::length_error("hash grid of " + std::to_string((long long)total) + " cells exceeds the limit of " +
                            std::to_string(max_cells) + " cells");
  return (long long)nn[0] * nn[1] * nn[2];
}

static int bits_for(long long v) {
  int b = 0;
  while (b < 63 && (1LL << b) <= v) ++b;
  return b;
}

void stage_hashgrid(pi_frame* f) {
  cudaStream_t s = f->ctx->stream;
  f->f64_ready = false;
  const long long n = f->N;
  f->misc.alloc(f->ctx, s, 16);
  PI_LAUNCH(k_init_misc, 1, 32, 0, s, f->misc.p);
  int blocks = (int)std::min<long long>(div_up(n, 256), (long long)f->ctx->smCount * 2);
  PI_LAUNCH(k_bbox, blocks, 256, 0, s, f->xyz.p, n, f->misc.p);
  unsigned h[8];
  PI_CUDA(cudaMemcpyAsync(h, f->misc.p, sizeof(unsigned) * 8, cudaMemcpyDeviceToHost, s));
  PI_CUDA(cudaStreamSynchronize(s));
  if (h[6]) throw std::invalid_argument("non-finite particle coordinate");
  float bb[6];
  for (int k = 0; k < 6; ++k) bb[k] = fdec(h[k]);
  f->singleLayer = (bb[0] == bb[1] || bb[2] == bb[3] || bb[4] == bb[5]);

  // HashGrid ctor (src/hash_grid.cpp:4-34), same float expressions.
  GridHost& g = f->g;
  const float cell = f->P.radius * 4.0f;
  g.cell = cell;
  for (int i = 0; i < 3; ++i) {
    float length = (std::ceil((bb[i * 2 + 1] - bb[i * 2]) / cell)) * cell;
    float center = (bb[i * 2] + bb[i * 2 + 1]) / 2;
    g.bounding[i * 2] = center - length / 2;
    g.bounding[i * 2 + 1] = center + length / 2;
  }
  int nn[3];
  // FindStartEnd stores keys in an int (src/hash_grid.cpp:105).
  g.cellNum = grid_cell_counts(g.bounding, cell, (1LL << 31) - 2, nn);
  g.nx = nn[0], g.ny = nn[1], g.nz = nn[2];
  g.bits = bits_for(g.cellNum + 1);
  f->key.alloc(f->ctx, s, n);
  f->skey.alloc(f->ctx, s, n);
  f->sidx.alloc(f->ctx, s, n);
  f->u32a.alloc(f->ctx, s, n);
  f->u32b.alloc(f->ctx, s, n);
  size_t tmpn = std::max(radix_tmp_ints(n), scan_tmp_ints(g.cellNum + 1));
  f->tmp.alloc(f->ctx, s, tmpn);
  PI_LAUNCH(k_keys, div_up(n, 256), 256, 0, s, f->xyz.p, n, g.bounding[0], g.bounding[2],
            g.bounding[4], cell, g.nx, g.ny, g.nz, f->key.p, f->skey.p, f->sidx.p);
  uint32_t *k = f->skey.p, *v = f->sidx.p, *ka = f->u32a.p, *va = f->u32b.p;
  radix_sort_u32(&k, &v, &ka, &va, n, g.bits, f->tmp.p, s);
  if (k != f->skey.p) {
    PI_CUDA(cudaMemcpyAsync(f->skey.p, k, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, s));
    PI_CUDA(cudaMemcpyAsync(f->sidx.p, v, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, s));
  }
  f->off.alloc(f->ctx, s, g.cellNum + 1);
  PI_CUDA(cudaMemsetAsync(f->off.p, 0, sizeof(int) * (g.cellNum + 1), s));
  PI_LAUNCH(k_cell_count, div_up(n, 256), 256, 0, s, f->key.p, n, f->off.p);
  exclusive_scan_i32(f->off.p, f->off.p, g.cellNum + 1, nullptr, f->tmp.p, s);
  f->pos.alloc(f->ctx, s, n);
  PI_LAUNCH(k_gather_pos, div_up(n, 256), 256, 0, s, f->xyz.p, f->sidx.p, n, f->pos.p);
  // the valid-key count (offset table total) reaches g.nInvalid in
  // resolve_pending; nothing before the end of the call reads it
  PI_CUDA(cudaMemcpyAsync(reinterpret_cast<int*>(f->ctx->hpin + (size_t)kPinSlots * kCounterWords),
                          f->off.p + g.cellNum, sizeof(int), cudaMemcpyDeviceToHost, s));
  f->pin_pending |= 1 << kPinValid;
  // loadRootBox result kept for the octree root (resizeRootBoxConstR)
  for (int k2 = 0; k2 < 6; ++k2) f->bbox6[k2] = bb[k2];
}

}  // namespace pisurf
