// UniformGrid (src/marching.cpp): the field sampled on a uniform lattice of
// spacing r over the particles' box (the reference's dense-grid mode, written
// to a VTK image there).
//   - UniformGrid::resizeRootBoxConstR (:42-55): per axis
//     resizeLen = ceil(length / r) r + 4 r around the box centre,
//     steps = int(resizeLen / r), dims = steps + 1;
//   - UniformGrid::gridSampling (:72-93): SingleEval at
//     (steps - i) / steps * min + i / steps * max per axis, x fastest.
// The lattice points of one hash cell form a contiguous index run along each
// axis (the cell index is monotonic in the coordinate), so a chunk is a
// (x-run, y-run, z-run) triple: at most 5 x 5 x 5 points, all with the same
// 27-cell candidate list, evaluated by one warp (chunk_field, 4 per lane).
#include <cmath>
#include <vector>

#include "chunk.cuh"
#include "internal.h"

namespace pisurf {

constexpr int kGridWarps = 8;
constexpr int kRunMax = 5;  // points per axis run: a cell is 4r, the spacing r

void uniform_grid_host(const pi_frame* f, float box[6], int steps[3], int dims[3]) {
  const float r = f->P.radius;
  for (int i = 0; i < 3; i++) {
    const float center = (f->bbox6[i * 2] + f->bbox6[i * 2 + 1]) / 2;
    const float length = f->bbox6[i * 2 + 1] - f->bbox6[i * 2];
    const float resizeLen = std::ceil(length / r) * r + r * 4;
    box[i * 2] = center - resizeLen / 2;
    box[i * 2 + 1] = center + resizeLen / 2;
    steps[i] = int(resizeLen / r);
    dims[i] = steps[i] + 1;
  }
}

struct GridRuns {
  const float* coord[3];  // lattice coordinate per index, per axis
  const int* run[3];      // run k of an axis covers indices [run[k], run[k + 1])
  int nrun[3];
  int dims[3];
};

__global__ void __launch_bounds__(32 * kGridWarps, 3) k_grid_eval(GridView g, PartView P, float iso, GridRuns R,
                                                                 float* __restrict__ out,
                                                                 unsigned long long* __restrict__ counters) {
  __shared__ __align__(16) float s_stage[kGridWarps][kStageFloats];
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  const ChunkStage st{s_stage[wib]};
  const long long nchunks = (long long)R.nrun[0] * R.nrun[1] * R.nrun[2];
  const long long nwarps = (long long)gridDim.x * kGridWarps;
  long long pairs = 0;
  for (long long ci = (long long)blockIdx.x * kGridWarps + wib; ci < nchunks; ci += nwarps) {
    const int rx = (int)(ci % R.nrun[0]), ry = (int)((ci / R.nrun[0]) % R.nrun[1]),
              rz = (int)(ci / ((long long)R.nrun[0] * R.nrun[1]));
    const int x0 = __ldg(R.run[0] + rx), kx = __ldg(R.run[0] + rx + 1) - x0;
    const int y0 = __ldg(R.run[1] + ry), ky = __ldg(R.run[1] + ry + 1) - y0;
    const int z0 = __ldg(R.run[2] + rz), kz = __ldg(R.run[2] + rz + 1) - z0;
    const int npts = kx * ky * kz;
    float x[4], y[4], z[4];
    bool act[4], slots[4];
    long long idx[4];
#pragma unroll
    for (int m = 0; m < 4; ++m) {
      const int p = lane + 32 * m;
      act[m] = p < npts;
      slots[m] = npts > 32 * m;  // warp-uniform
      x[m] = y[m] = z[m] = __int_as_float(0x7fc00000);  // NaN: no term for an invalid point
      idx[m] = 0;
      if (act[m]) {
        const int ix = x0 + p % kx, iy = y0 + (p / kx) % ky, iz = z0 + p / (kx * ky);
        x[m] = __ldg(R.coord[0] + ix);
        y[m] = __ldg(R.coord[1] + iy);
        z[m] = __ldg(R.coord[2] + iz);
        idx[m] = ((long long)iz * R.dims[1] + iy) * R.dims[0] + ix;
      }
    }
    int cx, cy, cz;
    cell_of(g, __shfl_sync(0xffffffffu, x[0], 0), __shfl_sync(0xffffffffu, y[0], 0),
            __shfl_sync(0xffffffffu, z[0], 0), cx, cy, cz);
    float sum[4];
    chunk_field<4>(g, P, cx, cy, cz, x, y, z, act, slots, st, sum, pairs);
#pragma unroll
    for (int m = 0; m < 4; ++m)
      if (act[m]) out[idx[m]] = iso - sum[m];
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) pairs += __shfl_xor_sync(0xffffffffu, pairs, o);
  if (lane == 0 && pairs) stripe_add(counters, 1, (unsigned long long)pairs);
}

// Host restatement of cell_coord (same IEEE float expression, truncation,
// clamp to [-2, n + 1]).
static int host_cell_coord(float p, float lo, float cell, int n) {
  const float q = (p - lo) / cell;
  int c = (int)q;
  c = c < -2 ? -2 : c;
  c = c > n + 1 ? n + 1 : c;
  return c;
}

long long grid_sample(pi_frame* f, float* d_out, long long cap) {
  pi_ctx* ctx = f->ctx;
  cudaStream_t s = ctx->stream;
  float box[6];
  int steps[3], dims[3];
  uniform_grid_host(f, box, steps, dims);
  const long long total = (long long)dims[0] * dims[1] * dims[2];
  if (!d_out || cap < total) return total;
  const GridHost& gh = f->g;
  const float b[3] = {gh.bounding[0], gh.bounding[2], gh.bounding[4]};
  const int n[3] = {gh.nx, gh.ny, gh.nz};
  std::vector<float> coord[3];
  std::vector<int> run[3];
  for (int a = 0; a < 3; ++a) {
    coord[a].resize(dims[a]);
    const float mn = box[2 * a], mx = box[2 * a + 1];
    int prev = 0, len = 0;
    for (int i = 0; i < dims[a]; ++i) {
      // the reference's expression, float arithmetic
      const float v = float(steps[a] - i) / float(steps[a]) * mn + float(i) / float(steps[a]) * mx;
      coord[a][i] = v;
      const int c = host_cell_coord(v, b[a], gh.cell, n[a]);
      if (i == 0 || c != prev || len == kRunMax) {
        run[a].push_back(i);
        len = 0;
      }
      prev = c;
      ++len;
    }
    run[a].push_back(dims[a]);
  }
  DBuf<float> dc[3];
  DBuf<int> dr[3];
  GridRuns R;
  for (int a = 0; a < 3; ++a) {
    dc[a].alloc(ctx, s, coord[a].size());
    dr[a].alloc(ctx, s, run[a].size());
    PI_CUDA(cudaMemcpyAsync(dc[a].p, coord[a].data(), sizeof(float) * coord[a].size(), cudaMemcpyHostToDevice, s));
    PI_CUDA(cudaMemcpyAsync(dr[a].p, run[a].data(), sizeof(int) * run[a].size(), cudaMemcpyHostToDevice, s));
    R.coord[a] = dc[a].p;
    R.run[a] = dr[a].p;
    R.nrun[a] = (int)run[a].size() - 1;
    R.dims[a] = dims[a];
  }
  const long long nchunks = (long long)R.nrun[0] * R.nrun[1] * R.nrun[2];
  static thread_local int occ[64] = {0};
  const int dev = ctx->device & 63;
  if (occ[dev] == 0) {
    int nb = 0;
    PI_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_grid_eval, 32 * kGridWarps, 0));
    occ[dev] = nb > 0 ? nb : 1;
  }
  const int blocks = (int)std::min<long long>((long long)ctx->smCount * occ[dev], div_up(nchunks, kGridWarps));
  counters_reset(f);
  GridView g{gh.bounding[0], gh.bounding[2], gh.bounding[4], gh.cell, gh.nx, gh.ny, gh.nz, f->off.p};
  PartView P{f->pos.p, f->xm.p, f->ga.p, f->gb.p, f->xlo.p};
  prof_begin(ctx, s, PG_GRID);
  PI_LAUNCH(k_grid_eval, blocks, 32 * kGridWarps, 0, s, g, P, f->iso, R, d_out, f->dcount.p);
  prof_end(ctx, s, PG_GRID);
  unsigned long long cnt[kCounters];
  counters_read(f, cnt);
  f->gridPairs = (long long)cnt[1];
  return total;
}

}  // namespace pisurf
