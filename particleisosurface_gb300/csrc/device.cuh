// Device views of a frame and the per-point field evaluation shared by the
// normal, octree-sampling and edge-bisection kernels.
//
// Layout in HBM (all per-particle arrays are in hash-cell order, i.e. the
// order of the reference's HashGrid::IndexList, src/hash_grid.cpp:71-85):
//   pos[N]   float4 (x, y, z, 0)           particle positions
//   xm[N]    float4 (xmean, cull radius^2)  smoothed centres (GlobalxMeans)
//   ga[N]    float4 (a00, a01, a02, a11)    A = G / (2r), symmetric
//   gb[N]    float4 (a12, a22, det*Sigma, 0)
//   nrm[N]   float4 (normal, |normal|)      PariclesNormals
//   off[C+1] int    cell c holds sorted positions [off[c], off[c+1])
// off[] counts only particles with a valid cell key while positions index the
// full sorted array, whose front holds the particles with key -1: this is the
// reference's StartList/EndList + IndexList pairing (src/hash_grid.cpp:103-162)
// including its shift when such particles exist.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"

namespace pisurf {

struct GridView {
  float b0, b2, b4;  // Bounding[0], [2], [4]
  float cell;        // CellSize = 4r
  int nx, ny, nz;
  const int* off;
};

struct PartView {
  const float4* pos;
  const float4* xm;   // (centre rounded to float, cull radius^2)
  const float4* ga;
  const float4* gb;
  const float4* xlo;  // (centre - rounded centre, 0): the low part of the centre
};

// Event counters (field evaluations, candidate pairs, ...) striped over 64
// slots 32 bytes apart, so that many warps adding to one counter do not
// serialise on a single address.  Counter w, stripe k lives at
// c[(w * kStripes + k) * 4]; the host sums the stripes.
__device__ __forceinline__ void stripe_add(unsigned long long* c, int w, unsigned long long v) {
  if (v) atomicAdd(c + ((size_t)w * kStripes + (blockIdx.x & (kStripes - 1))) * 4, v);
}

struct Kahan {
  float s = 0.f, c = 0.f;
  __device__ __forceinline__ void add(float v) {
    float y = __fsub_rn(v, c);
    float t = __fadd_rn(s, y);
    c = __fsub_rn(__fsub_rn(t, s), y);
    s = t;
  }
};

// HashGrid::CalcXYZIdx (src/hash_grid.cpp:124-129): IEEE float subtract and
// divide, truncation toward zero.  Clamped to [-2, n+1] so that neighbour
// arithmetic cannot overflow; cells outside [0, n) are skipped either way.
__device__ __forceinline__ int cell_coord(float p, float lo, float cell, int n) {
  float q = __fdiv_rn(__fsub_rn(p, lo), cell);
  int c = (int)q;  // cvt.rzi
  c = c < -2 ? -2 : c;
  c = c > n + 1 ? n + 1 : c;
  return c;
}

// cell_coord that also returns the quotient (p - lo) / cell it truncates.
__device__ __forceinline__ int cell_coord_q(float p, float lo, float cell, int n, float& q) {
  q = __fdiv_rn(__fsub_rn(p, lo), cell);
  int c = (int)q;
  c = c < -2 ? -2 : c;
  c = c > n + 1 ? n + 1 : c;
  return c;
}

__device__ __forceinline__ void cell_of(const GridView& g, float x, float y, float z, int& cx,
                                        int& cy, int& cz) {
  cx = cell_coord(x, g.b0, g.cell, g.nx);
  cy = cell_coord(y, g.b2, g.cell, g.ny);
  cz = cell_coord(z, g.b4, g.cell, g.nz);
}

// Row (z, y) of the 3x3x3 neighbourhood of cell (cx, ., .): the cells
// x in [cx-1, cx+1] are consecutive keys, so their particles are the single
// contiguous range [*s, *e).  Returns false if the row is outside the grid.
__device__ __forceinline__ bool nb_row(const GridView& g, int cx, int y, int z, int* s, int* e) {
  if (z < 0 || z >= g.nz || y < 0 || y >= g.ny) return false;
  int x0 = cx - 1 < 0 ? 0 : cx - 1;
  int x1 = cx + 1 > g.nx - 1 ? g.nx - 1 : cx + 1;
  if (x0 > x1) return false;
  long long base = ((long long)z * g.ny + y) * g.nx;
  *s = __ldg(g.off + base + x0);
  *e = __ldg(g.off + base + x1 + 1);
  return *s < *e;
}

// Cubic B-spline of ratio q = sqrt(s2) in [0, 2) without the Sigma factor
// (Bspline_kernel, src/evaluator.cpp:383-396).
__device__ __forceinline__ float bspline_s2(float s2) {
  // sqrt(s2) as s2 / sqrt(s2); the floor only changes q for s2 < 1e-30,
  // where b1 rounds to 1 either way
  float q = s2 * rsqrtf(fmaxf(s2, 1e-30f));
  float b1 = fmaf(s2, fmaf(0.75f, q, -1.5f), 1.0f);
  float t = 2.0f - q;
  float b2 = 0.25f * t * t * t;
  return q <= 1.0f ? b1 : b2;
}

// u = A d for the symmetric A stored in (ga, gb).
__device__ __forceinline__ void amul(const float4& a, const float4& b, float dx, float dy, float dz,
                                     float& u0, float& u1, float& u2) {
  u0 = fmaf(a.x, dx, fmaf(a.y, dy, a.z * dz));
  u1 = fmaf(a.y, dx, fmaf(a.w, dy, b.x * dz));
  u2 = fmaf(a.z, dx, fmaf(b.x, dy, b.y * dz));
}

// The kernel terms of the candidates [s, e) at q, added to acc in candidate
// order.  32 candidates at a time: first the cheap |d|^2 < R^2 test of each
// into a bit mask, then the kernel terms of the set bits in candidate order,
// so that a warp runs the costly part as often as its busiest lane needs it
// rather than once per candidate any lane needs.
__device__ __forceinline__ void field_row(const PartView& P, int s, int e, float qx, float qy, float qz,
                                          Kahan& acc) {
  for (int j0 = s; j0 < e; j0 += 32) {
    const int cnt = min(32, e - j0);
    unsigned m = 0u;
    for (int k = 0; k < cnt; ++k) {
      const float4 x = __ldg(P.xm + j0 + k);
      const float dx = qx - x.x, dyy = qy - x.y, dzz = qz - x.z;
      const float e2 = fmaf(dx, dx, fmaf(dyy, dyy, dzz * dzz));
      m |= (e2 < x.w ? 1u : 0u) << k;
    }
    while (m) {
      const int j = j0 + __ffs(m) - 1;
      m &= m - 1u;
      const float4 x = __ldg(P.xm + j);
      const float dx = qx - x.x, dyy = qy - x.y, dzz = qz - x.z;
      const float4 a = __ldg(P.ga + j);
      const float4 b = __ldg(P.gb + j);
      const float4 lo = __ldg(P.xlo + j);
      float u0, u1, u2;
      amul(a, b, dx - lo.x, dyy - lo.y, dzz - lo.z, u0, u1, u2);
      const float s2 = fmaf(u0, u0, fmaf(u1, u1, u2 * u2));
      if (s2 < 4.0f) acc.add(b.z * bspline_s2(s2));
    }
  }
}

// Sum over the 27-cell candidates of particle kernel values at q: the
// sum in Evaluator::SingleEval (src/evaluator.cpp:60-87) without the
// iso - sum step.  Compensated (Kahan) FP32 accumulation.
__device__ __forceinline__ float field_sum(const GridView& g, const PartView& P, float qx, float qy,
                                           float qz, long long* npairs) {
  int cx, cy, cz;
  cell_of(g, qx, qy, qz, cx, cy, cz);
  Kahan acc;
  long long pairs = 0;
  for (int dz = -1; dz <= 1; ++dz)
    for (int dy = -1; dy <= 1; ++dy) {
      int s, e;
      if (!nb_row(g, cx, cy + dy, cz + dz, &s, &e)) continue;
      pairs += e - s;
      field_row(P, s, e, qx, qy, qz, acc);
    }
  if (npairs) *npairs += pairs;
  return acc.s;
}

// ---------------------------------------------------------------------------
// Variable radius: the particles binned by radius (MultiLevelSearcher,
// src/multi_level_reseacher.cpp:6-77), one hash grid per non-empty bin with
// the cell size of the bin's largest radius times 4.  Particles are sorted by
// (bin, cell key + 1, particle); off[] holds every bin's cell offsets one
// bin after the other (cellNum + 1 entries per bin, offBase its first), with
// bin b's entries counted from the bin's first sorted position and the
// reference's shift by the bin's key -1 particles kept.  A point's candidate
// list is the bins' 27-cell lists in bin order (GetNeighbors).
// ---------------------------------------------------------------------------
constexpr int kMaxBins = 32;

struct BinGrid {
  float b0, b2, b4, cell;
  int nx, ny, nz;
  int offBase;
};

struct MultiGridView {
  int nb;
  const int* off;
  BinGrid g[kMaxBins];
};

__device__ __forceinline__ bool bin_row(const BinGrid& g, const int* off, int cx, int y, int z, int* s, int* e) {
  if (z < 0 || z >= g.nz || y < 0 || y >= g.ny) return false;
  const int x0 = cx - 1 < 0 ? 0 : cx - 1;
  const int x1 = cx + 1 > g.nx - 1 ? g.nx - 1 : cx + 1;
  if (x0 > x1) return false;
  const long long base = (long long)g.offBase + ((long long)z * g.ny + y) * g.nx;
  *s = __ldg(off + base + x0);
  *e = __ldg(off + base + x1 + 1);
  return *s < *e;
}

// SingleEval's sum with the variable-radius candidate list; the per-particle
// records already hold each particle's A = G / (2 r_j), det * Sigma_j and
// support radius.
__device__ __forceinline__ float field_sum_vr(const MultiGridView& m, const PartView& P, float qx, float qy,
                                              float qz, long long* npairs) {
  Kahan acc;
  long long pairs = 0;
  for (int b = 0; b < m.nb; ++b) {
    const BinGrid g = m.g[b];
    const int cx = cell_coord(qx, g.b0, g.cell, g.nx), cy = cell_coord(qy, g.b2, g.cell, g.ny),
              cz = cell_coord(qz, g.b4, g.cell, g.nz);
    for (int dz = -1; dz <= 1; ++dz)
      for (int dy = -1; dy <= 1; ++dy) {
        int s, e;
        if (!bin_row(g, m.off, cx, cy + dy, cz + dz, &s, &e)) continue;
        pairs += e - s;
        field_row(P, s, e, qx, qy, qz, acc);
      }
  }
  if (npairs) *npairs += pairs;
  return acc.s;
}

}  // namespace pisurf
