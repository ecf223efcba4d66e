// Warp-cooperative field evaluation for a chunk of query points that share
// one hash cell, hence one 27-cell candidate list (Evaluator::SingleEval,
// src/evaluator.cpp:60-87).  Lane l holds points l, l + 32, ... (K per lane).
//
// The warp tests 32 candidates at a time against the chunk's bounding box: a
// candidate whose support radius R (|G d| < 2h needs |d| < R, stored as
// R^2 * 1.002 in xm.w) does not reach the box contributes to no point.
// Survivors' records are staged in shared memory in candidate order and every
// lane walks them, so each point's compensated sum sees the in-support terms
// in candidate order (the same terms and order as field_sum).
#pragma once
#include "device.cuh"

namespace pisurf {

constexpr int kCandBuf = 96;  // staged candidate records per warp

// Order-preserving map of a float onto a signed int (for warp min / max).
__device__ __forceinline__ int fkey(float v) {
  const int i = __float_as_int(v);
  return i >= 0 ? i : i ^ 0x7fffffff;
}
__device__ __forceinline__ float fkey_inv(int k) { return __int_as_float(k >= 0 ? k : k ^ 0x7fffffff); }

// 16-byte asynchronous copy global -> shared (cp.async, no register
// staging); completed by cp_async_wait_all before the records are read.
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// Per-warp staging buffers (shared memory), kCandBuf records each.
struct ChunkStage {
  float4* x;
  float4* a;
  float4* b;
  float4* l;
};

// Sums over the chunk's candidates for the K points of this lane.  act[m]
// marks the lane's valid points, and an invalid point's coordinates must be
// NaN (its s2 is then NaN and no term passes s2 < 4); slots[m]
// (warp-uniform) tells whether any lane holds a point m.  Returns the compensated sums in sum[]; adds the
// algorithmic candidate pairs of the lane's points to pairs.
template <int K>
__device__ __forceinline__ void chunk_field(const GridView& g, const PartView& P, int cx, int cy, int cz,
                                            const float (&qx)[K], const float (&qy)[K], const float (&qz)[K],
                                            const bool (&act)[K], const bool (&slots)[K], const ChunkStage& st,
                                            float (&sum)[K], long long& pairs) {
  const int lane = threadIdx.x & 31;
  const unsigned lt = (1u << lane) - 1u;
  // bounding box of the chunk's points
  const int kmin = 0x7fffffff, kmax = (int)0x80000000;
  int lx = kmin, ly = kmin, lz = kmin, hx = kmax, hy = kmax, hz = kmax;
  int nact = 0;
#pragma unroll
  for (int m = 0; m < K; ++m)
    if (act[m]) {
      lx = min(lx, fkey(qx[m]));
      ly = min(ly, fkey(qy[m]));
      lz = min(lz, fkey(qz[m]));
      hx = max(hx, fkey(qx[m]));
      hy = max(hy, fkey(qy[m]));
      hz = max(hz, fkey(qz[m]));
      ++nact;
    }
  const float blx = fkey_inv(__reduce_min_sync(0xffffffffu, lx));
  const float bly = fkey_inv(__reduce_min_sync(0xffffffffu, ly));
  const float blz = fkey_inv(__reduce_min_sync(0xffffffffu, lz));
  const float bhx = fkey_inv(__reduce_max_sync(0xffffffffu, hx));
  const float bhy = fkey_inv(__reduce_max_sync(0xffffffffu, hy));
  const float bhz = fkey_inv(__reduce_max_sync(0xffffffffu, hz));
  // compensated sums (Kahan), updated only for in-support terms
  float s[K], c[K];
#pragma unroll
  for (int m = 0; m < K; ++m) s[m] = c[m] = 0.f;
  int nc = 0;
  auto flush = [&]() {
    cp_async_wait_all();
    __syncwarp();
#pragma unroll 2
    for (int t = 0; t < nc; ++t) {
      const float4 x = st.x[t], ga = st.a[t], gb = st.b[t], lo = st.l[t];
#pragma unroll
      for (int m = 0; m < K; ++m) {
        if (!slots[m]) continue;  // warp-uniform
        float u0, u1, u2;
        amul(ga, gb, (qx[m] - x.x) - lo.x, (qy[m] - x.y) - lo.y, (qz[m] - x.z) - lo.z, u0, u1, u2);
        const float s2 = fmaf(u0, u0, fmaf(u1, u1, u2 * u2));
        if (s2 < 4.0f) {  // in support: one compensated step
          const float y = __fsub_rn(gb.z * bspline_s2(s2), c[m]);
          const float tt = __fadd_rn(s[m], y);
          c[m] = __fsub_rn(__fsub_rn(tt, s[m]), y);
          s[m] = tt;
        }
      }
    }
    __syncwarp();
    nc = 0;
  };
  for (int dz = -1; dz <= 1; ++dz)
    for (int dy = -1; dy <= 1; ++dy) {
      int rs, re;
      if (!nb_row(g, cx, cy + dy, cz + dz, &rs, &re)) continue;
      pairs += (long long)(re - rs) * nact;
      for (int j0 = rs; j0 < re; j0 += 32) {
        const int j = j0 + lane;
        bool pass = false;
        float4 x;
        if (j < re) {
          x = __ldg(P.xm + j);
          const float ex = fmaxf(fmaxf(blx - x.x, x.x - bhx), 0.f);
          const float ey = fmaxf(fmaxf(bly - x.y, x.y - bhy), 0.f);
          const float ez = fmaxf(fmaxf(blz - x.z, x.z - bhz), 0.f);
          pass = fmaf(ex, ex, fmaf(ey, ey, ez * ez)) < x.w;
        }
        const unsigned pm = __ballot_sync(0xffffffffu, pass);
        if (pass) {
          const int p = nc + __popc(pm & lt);
          st.x[p] = x;
          cp_async16(st.a + p, P.ga + j);
          cp_async16(st.b + p, P.gb + j);
          cp_async16(st.l + p, P.xlo + j);
        }
        nc += __popc(pm);
        if (nc > kCandBuf - 32) flush();
      }
    }
  flush();
#pragma unroll
  for (int m = 0; m < K; ++m) sum[m] = s[m];
}

}  // namespace pisurf
