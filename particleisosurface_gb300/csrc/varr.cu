// Variable radius: the reference's SurfReconstructor with per-particle radii
// (IS_CONST_RADIUS false), with its neighbour query switched on.
//
//   - MultiLevelSearcher (src/multi_level_reseacher.cpp:6-77): radii binned
//     into bins about minRadius / 2 wide; per non-empty bin a HashGrid of the
//     bin's particles (src/hash_grid.cpp:36-69) whose cell is the bin's
//     largest radius times 4, over the bin's bounding box.  Here every
//     particle gets the key of its bin's grid, and one stable radix sort by
//     (grid, key + 1) puts each grid's particles in cell order one grid after
//     the other; the offsets of all grids live in one table (device.cuh,
//     MultiGridView).  GetNeighbors is the bins' 27-cell lists in bin order.
//   - resizeRootBoxVarR (src/surface_reconstructor.cpp:124-149),
//     CalculateMaxScalarVarR / RecommendIsoValueVarR (src/evaluator.cpp:
//     293-361), per-particle Influnce2 and Sigma (:16-29).
//
// The reference's own code of this path is dead (the neighbour queries are
// commented out at src/evaluator.cpp:68,105,670,733), and two of its pieces
// are broken: MultiLevelSearcher::GetNeighbors indexes its searchers with
// the bin index (the wrong grid once an earlier bin is empty) and
// GetInBoxParticles maps particle indices through the bin's index list a
// second time.  Here each non-empty bin's grid is queried in bin order and
// its particle indices are used as they are, as the oracle does.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <stdexcept>
#include <string>

#include "device.cuh"
#include "internal.h"

namespace pisurf {

__global__ void k_bbox(const float* __restrict__ xyz, long long n, unsigned* __restrict__ misc);
__global__ void k_init_misc(unsigned* misc);

__device__ __forceinline__ unsigned vr_fenc(float f) {
  unsigned b = __float_as_uint(f);
  return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
static float vr_fdec(unsigned e) {
  unsigned b = (e & 0x80000000u) ? (e & 0x7fffffffu) : ~e;
  float f;
  std::memcpy(&f, &b, 4);
  return f;
}

// Per-grid bounding boxes: bb[6 * g + k] encoded min / max, combined per
// block in shared memory (at most kMaxBins grids).
__global__ void k_vr_bin_bbox(const float* __restrict__ xyz, const int* __restrict__ pbin, long long n, int ng,
                              unsigned* __restrict__ bb) {
  __shared__ unsigned s[kMaxBins * 6];
  for (int k = threadIdx.x; k < ng * 6; k += blockDim.x) s[k] = (k & 1) ? 0u : 0xffffffffu;
  __syncthreads();
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int g = pbin[i];
    for (int k = 0; k < 3; ++k) {
      const unsigned e = vr_fenc(xyz[3 * i + k]);
      atomicMin(s + 6 * g + 2 * k, e);
      atomicMax(s + 6 * g + 2 * k + 1, e);
    }
  }
  __syncthreads();
  for (int k = threadIdx.x; k < ng * 6; k += blockDim.x) {
    if (k & 1)
      atomicMax(bb + k, s[k]);
    else
      atomicMin(bb + k, s[k]);
  }
}

// Key of each particle in its grid (CalcXYZIdx + CalcCellHash,
// src/hash_grid.cpp:124-139, -1 outside) and the sort key (grid, key + 1).
__global__ void k_vr_keys(const float* __restrict__ xyz, const int* __restrict__ pbin, long long n,
                          const MultiGridView* __restrict__ mg, int kbits, int* __restrict__ key,
                          uint64_t* __restrict__ skey, uint32_t* __restrict__ sidx) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int b = pbin[i];
  const BinGrid g = mg->g[b];
  const int cx = (int)__fdiv_rn(__fsub_rn(xyz[3 * i], g.b0), g.cell);
  const int cy = (int)__fdiv_rn(__fsub_rn(xyz[3 * i + 1], g.b2), g.cell);
  const int cz = (int)__fdiv_rn(__fsub_rn(xyz[3 * i + 2], g.b4), g.cell);
  int k = -1;
  if (cx >= 0 && cx < g.nx && cy >= 0 && cy < g.ny && cz >= 0 && cz < g.nz)
    k = (int)(((long long)cz * g.ny + cy) * g.nx + cx);
  key[i] = k;
  skey[i] = ((uint64_t)b << kbits) | (uint64_t)(uint32_t)(k + 1);
  sidx[i] = (uint32_t)i;
}

// Cell counts into the concatenated offset table; a grid's key -1 particles
// count in its extra last entry, so that after the exclusive scan the grid's
// cell c starts at (grid's first sorted position) + (valid keys before c),
// the reference's StartList shifted by the grid's key -1 particles
// (src/hash_grid.cpp:103-122, 141-162).
__global__ void k_vr_cell_count(const int* __restrict__ key, const int* __restrict__ pbin, long long n,
                                const MultiGridView* __restrict__ mg, const long long* __restrict__ cellnum,
                                int* __restrict__ cnt) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int b = pbin[i];
  const int k = key[i];
  atomicAdd(cnt + mg->g[b].offBase + (k >= 0 ? (long long)k : cellnum[b]), 1);
}

__global__ void k_vr_gather_pos(const float* __restrict__ xyz, const float* __restrict__ rad,
                                const float4* __restrict__ vrc, const uint32_t* __restrict__ sidx, long long n,
                                float4* __restrict__ pos, float4* __restrict__ vrcs) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const uint32_t i = sidx[t];
  pos[t] = make_float4(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2], rad[i]);
  vrcs[t] = vrc[i];
}

void stage_upload_radii(pi_frame* f, const float* radii, long long n) {
  if (n != f->N) throw std::invalid_argument("radii: one per particle of the frame");
  for (long long i = 0; i < n; ++i)
    if (!(std::isfinite(radii[i]) && radii[i] > 0)) throw std::invalid_argument("radii must be positive");
  if (f->P.qef) throw std::invalid_argument("the QEF vertices are not available with per-particle radii");
  if (f->P.splash) throw std::invalid_argument("splash particles are not available with per-particle radii");
  f->hrad.assign(radii, radii + n);
  // Evaluator ctor, variable radius (src/evaluator.cpp:16-29): Influnce2 and
  // Sigma from 2 r in the reference's float / double mix, and the neighbour
  // radius nI = 4 r of compute_xMeans / compute_G_Yus with 1 / nI^3 (the
  // constant-radius stage computes the same four numbers from its radius)
  std::vector<float4> c((size_t)n);
  for (long long i = 0; i < n; ++i) {
    const float r = radii[i];
    const float nI = r * 4.0f;
    c[i] = make_float4((float)std::pow(r * 2.0f, 2), (float)(1 / std::pow(r * 2.0f, 6)), nI,
                       (float)(1.0 / ((double)nI * nI * nI)));
  }
  cudaStream_t s = f->ctx->stream;
  f->rad.alloc(f->ctx, s, n);
  f->vrc.alloc(f->ctx, s, n);
  PI_CUDA(cudaMemcpyAsync(f->rad.p, radii, sizeof(float) * n, cudaMemcpyHostToDevice, s));
  PI_CUDA(cudaMemcpyAsync(f->vrc.p, c.data(), sizeof(float4) * n, cudaMemcpyHostToDevice, s));
  PI_CUDA(cudaStreamSynchronize(s));  // the host staging vector goes out of scope
  f->varR = true;
}

void stage_hashgrid_vr(pi_frame* f) {
  pi_ctx* c = f->ctx;
  cudaStream_t s = c->stream;
  const long long n = f->N;
  const std::vector<float>& R = f->hrad;
  // loadRootBox over all particles (the octree root)
  f->misc.alloc(c, s, 16);
  PI_LAUNCH(k_init_misc, 1, 32, 0, s, f->misc.p);
  PI_LAUNCH(k_bbox, (int)std::min<long long>(div_up(n, 256), (long long)c->smCount * 2), 256, 0, s, f->xyz.p, n,
            f->misc.p);
  unsigned h[8];
  PI_CUDA(cudaMemcpyAsync(h, f->misc.p, sizeof(unsigned) * 8, cudaMemcpyDeviceToHost, s));
  // MultiLevelSearcher bins (src/multi_level_reseacher.cpp:9-45), the
  // reference's float arithmetic
  const float maxRadius = (float)(*std::max_element(R.begin(), R.end()) * 1.01);
  const float minRadius = (float)(*std::min_element(R.begin(), R.end()) * 0.99);
  float bin_extent = (float)(minRadius * 0.5);
  const int nbins = std::max(int(std::ceil((maxRadius - minRadius) / bin_extent)), 1);
  bin_extent = (maxRadius - minRadius) / nbins;
  std::vector<std::pair<float, float>> bounds(nbins);
  for (int i = 0; i < nbins; i++)
    bounds[i] = {minRadius + (i * bin_extent), std::min(minRadius + ((i + 1) * bin_extent), maxRadius)};
  std::vector<int> which(n);
  std::vector<long long> per(nbins, 0);
  double sum = 0;
  for (long long i = 0; i < n; ++i) {
    int k = -1;
    for (int b = 0; b < nbins; ++b)
      if (R[i] >= bounds[b].first && R[i] <= bounds[b].second) {
        k = b;
        break;
      }
    if (k < 0) throw std::invalid_argument("a radius falls outside the searcher's bins");
    which[i] = k;
    per[k]++;
    sum += R[i];
  }
  float avg = (float)(sum / n);
  f->vrMinR = minRadius;
  f->vrMaxR = maxRadius;
  f->vrAvgR = std::min(std::max(avg, minRadius), maxRadius);
  // non-empty bins become grids, in bin order
  std::vector<int> grid_of(nbins, -1);
  f->bins.clear();
  for (int b = 0; b < nbins; ++b)
    if (per[b]) {
      grid_of[b] = (int)f->bins.size();
      BinHost bh{};
      bh.bin = b;
      bh.count = per[b];
      bh.radius_id = -1;
      f->bins.push_back(bh);
    }
  const int ng = (int)f->bins.size();
  if (ng > kMaxBins)
    throw std::length_error("per-particle radii span " + std::to_string(ng) + " radius bins, more than " +
                            std::to_string(kMaxBins));
  std::vector<int> pbin(n);
  for (long long i = 0; i < n; ++i) {
    const int g = grid_of[which[i]];
    pbin[i] = g;
    int& rid = f->bins[g].radius_id;
    if (rid < 0 || R[i] > R[rid]) rid = (int)i;  // the first of equal maxima
  }
  f->pbin.alloc(c, s, n);
  PI_CUDA(cudaMemcpyAsync(f->pbin.p, pbin.data(), sizeof(int) * n, cudaMemcpyHostToDevice, s));
  DBuf<unsigned> bb;
  bb.alloc(c, s, 6 * ng);
  std::vector<unsigned> init(6 * ng);
  for (int k = 0; k < 6 * ng; ++k) init[k] = (k & 1) ? 0u : 0xffffffffu;
  PI_CUDA(cudaMemcpyAsync(bb.p, init.data(), sizeof(unsigned) * 6 * ng, cudaMemcpyHostToDevice, s));
  PI_LAUNCH(k_vr_bin_bbox, (int)std::min<long long>(div_up(n, 256), (long long)c->smCount * 2), 256, 0, s, f->xyz.p,
            f->pbin.p, n, ng, bb.p);
  std::vector<unsigned> hb(6 * ng);
  PI_CUDA(cudaMemcpyAsync(hb.data(), bb.p, sizeof(unsigned) * 6 * ng, cudaMemcpyDeviceToHost, s));
  PI_CUDA(cudaStreamSynchronize(s));
  if (h[6]) throw std::invalid_argument("non-finite particle coordinate");
  float box[6];
  for (int k = 0; k < 6; ++k) box[k] = vr_fdec(h[k]);
  f->singleLayer = (box[0] == box[1] || box[2] == box[3] || box[4] == box[5]);
  for (int k = 0; k < 6; ++k) f->bbox6[k] = box[k];
  // each grid: HashGrid var-R ctor (src/hash_grid.cpp:46-61)
  MultiGridView mv{};
  mv.nb = ng;
  long long offTotal = 0, start = 0;
  int kbits = 1;
  for (int g = 0; g < ng; ++g) {
    BinHost& bh = f->bins[g];
    float b6[6];
    for (int k = 0; k < 6; ++k) b6[k] = vr_fdec(hb[6 * g + k]);
    bh.cell = R[bh.radius_id] * 4.0f;
    for (int i = 0; i < 3; ++i) {
      float length = ((std::ceil((b6[i * 2 + 1] - b6[i * 2]) / bh.cell)) * bh.cell);
      float center = (b6[i * 2] + b6[i * 2 + 1]) / 2;
      bh.bounding[i * 2] = center - length / 2;
      bh.bounding[i * 2 + 1] = center + length / 2;
    }
    int nn[3];
    bh.cellNum = grid_cell_counts(bh.bounding, bh.cell, (1LL << 31) - 2, nn);
    bh.nx = nn[0], bh.ny = nn[1], bh.nz = nn[2];
    bh.offBase = (int)offTotal;
    bh.start = start;
    start += bh.count;
    offTotal += bh.cellNum + 1;
    if (offTotal >= (1LL << 31) - 1) throw std::length_error("the radius bins' grids hold >= 2^31 cells");
    mv.g[g] = BinGrid{bh.bounding[0], bh.bounding[2], bh.bounding[4], bh.cell, bh.nx, bh.ny, bh.nz, bh.offBase};
    while ((1LL << kbits) <= bh.cellNum + 1) ++kbits;
  }
  f->off.alloc(c, s, offTotal + 1);
  mv.off = f->off.p;
  f->mgv.alloc(c, s, 1);
  PI_CUDA(cudaMemcpyAsync(f->mgv.p, &mv, sizeof(MultiGridView), cudaMemcpyHostToDevice, s));
  // keys, the sort by (grid, key + 1), offsets, positions (radius in .w)
  int gbits = 0;
  while ((1 << gbits) < ng) ++gbits;
  DBuf<uint64_t> sk, ska;
  DBuf<uint32_t> sia;
  f->key.alloc(c, s, n);
  f->sidx.alloc(c, s, n);
  sk.alloc(c, s, n);
  ska.alloc(c, s, n);
  sia.alloc(c, s, n);
  f->tmp.alloc(c, s, std::max(radix_tmp_ints(n), scan_tmp_ints(offTotal + 1)));
  PI_LAUNCH(k_vr_keys, div_up(n, 256), 256, 0, s, f->xyz.p, f->pbin.p, n, f->mgv.p, kbits, f->key.p, sk.p,
            f->sidx.p);
  uint64_t *k = sk.p, *ka = ska.p;
  uint32_t *v = f->sidx.p, *va = sia.p;
  radix_sort_u64(&k, &v, &ka, &va, n, kbits + gbits, f->tmp.p, s);
  if (v != f->sidx.p) PI_CUDA(cudaMemcpyAsync(f->sidx.p, v, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, s));
  DBuf<long long> cn;
  cn.alloc(c, s, ng);
  std::vector<long long> hcn(ng);
  for (int g = 0; g < ng; ++g) hcn[g] = f->bins[g].cellNum;
  PI_CUDA(cudaMemcpyAsync(cn.p, hcn.data(), sizeof(long long) * ng, cudaMemcpyHostToDevice, s));
  PI_CUDA(cudaMemsetAsync(f->off.p, 0, sizeof(int) * (offTotal + 1), s));
  PI_LAUNCH(k_vr_cell_count, div_up(n, 256), 256, 0, s, f->key.p, f->pbin.p, n, f->mgv.p, cn.p, f->off.p);
  exclusive_scan_i32(f->off.p, f->off.p, offTotal + 1, nullptr, f->tmp.p, s);
  f->pos.alloc(c, s, n);
  f->vrcs.alloc(c, s, n);
  PI_LAUNCH(k_vr_gather_pos, div_up(n, 256), 256, 0, s, f->xyz.p, f->rad.p, f->vrc.p, f->sidx.p, n, f->pos.p,
            f->vrcs.p);
  // the frame's grid fields describe the first grid (pi_frame_info)
  GridHost& gh = f->g;
  const BinHost& b0 = f->bins[0];
  for (int q = 0; q < 6; ++q) gh.bounding[q] = b0.bounding[q];
  gh.cell = b0.cell;
  gh.nx = b0.nx, gh.ny = b0.ny, gh.nz = b0.nz;
  gh.cellNum = b0.cellNum;
  gh.nInvalid = 0;
  gh.bits = kbits + gbits;
  PI_CUDA(cudaStreamSynchronize(s));
}

// Bspline_kernel (src/evaluator.cpp:383-396) with the reference's float /
// double mix.
static float bspline_ref(float ratio, float sigma) {
  if (ratio < 2) {
    if (ratio <= 1) return (float)(sigma * (1 - 1.5 * std::pow(ratio, 2) + 0.75 * std::pow(ratio, 3)));
    float tmq = 2 - ratio;
    return (float)(sigma * (0.25 * std::pow(tmq, 3)));
  }
  return 0.0f;
}

void host_root_and_scalars_vr(pi_frame* f) {
  // resizeRootBoxVarR (src/surface_reconstructor.cpp:124-149)
  const float minR = f->vrMinR, maxR = f->vrMaxR;
  const float* bb = f->bbox6;
  float maxLen = std::max({(bb[1] - bb[0]), (bb[3] - bb[2]), (bb[5] - bb[4])});
  const float cells = std::ceil(maxLen / minR);
  int dmax = cells >= 1.0f ? int(std::ceil(std::log2(cells))) : 0;
  float resizeLen = (float)(std::pow(2, dmax) * minR);
  while (resizeLen - maxLen < (4.0f * maxR * 2)) {
    dmax++;
    resizeLen = (float)(std::pow(2, dmax) * minR);
  }
  f->rootH = resizeLen / 2;
  for (int i = 0; i < 3; ++i) f->rootC[i] = (bb[i * 2] + bb[i * 2 + 1]) / 2;
  f->dmax = dmax;
  const float cmax = std::ceil(maxLen / maxR);
  const int dr = cmax >= 1.0f ? int(std::ceil(std::log2(cmax))) : 0;
  f->dmin = std::min(dr - 1, dmax - 2);
  // CalculateMaxScalarVarR / RecommendIsoValueVarR (src/evaluator.cpp:293-361)
  // over the grids' radius particles; Sigma_j = 1 / (2 r_j)^6 from the
  // constructor's default smoothing factor (src/evaluator.cpp:24-28)
  const float sqrt2 = 1.4142135623730950488016887242097f;
  const float sqrt3 = 1.7320508075688772935274463415059f;
  float mx = 0, rec = 0;
  for (const BinHost& bh : f->bins) {
    const float smooth = f->hrad[bh.radius_id] * 2.0f;
    const float sg = (float)(1 / std::pow(smooth, 6));
    float k = 0;
    k += bspline_ref(0.0f, sg);
    k += bspline_ref(1.0f, sg) * 6;
    k += bspline_ref(sqrt2, sg) * 12;
    k += bspline_ref(sqrt3, sg) * 8;
    if (k > mx) mx = k;
    const float v = bspline_ref(0.25f, sg);
    if (v > rec) rec = v;
  }
  f->maxScalar = mx;
  f->iso = rec;
  // the smallest radius's constants, for the frame info
  const float smin = *std::min_element(f->hrad.begin(), f->hrad.end()) * 2.0f;
  f->influ2 = (float)std::pow(smin, 2);
  f->sigma = (float)(1 / std::pow(smin, 6));
}

}  // namespace pisurf
