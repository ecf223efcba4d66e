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

constexpr int kCandBuf = 96;  // staged candidate records per warp (default; k_q_eval tunes it)

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

// Per-warp staging buffer (shared memory): the staged candidates' records,
// one array of CB floats per component (structure of arrays), so that a
// component of two consecutive candidates is one 8-byte load feeding the
// packed FP32 instructions below.
enum : int {
  SC_X, SC_Y, SC_Z,        // centre, high part (xm)
  SC_LX, SC_LY, SC_LZ,     // centre, low part (xlo)
  SC_A0, SC_A1, SC_A2, SC_A3,  // A = G / h: a00 a01 a02 a11
  SC_B0, SC_B1, SC_B2,     // a12 a22 det * Sigma
  kStageComps
};
__host__ __device__ constexpr int stage_floats(int cb) { return kStageComps * cb; }  // per warp
constexpr int kStageFloats = stage_floats(kCandBuf);

struct ChunkStage {
  float* c;  // c[k * CB + t]: component k of staged candidate t
};

// 4-byte asynchronous copy global -> shared.
__device__ __forceinline__ void cp_async4(void* smem, const void* gmem) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(sa), "l"(gmem) : "memory");
}

template <int CB>
__device__ __forceinline__ float2 ld_pair(const ChunkStage& st, int k, int t) {
  return *reinterpret_cast<const float2*>(st.c + k * CB + t);
}

// The staged candidates [0, nc) against the lane's K points: two consecutive
// candidates per step with Blackwell's packed FP32 instructions, each term
// added to the point's compensated sum (s, c) in candidate order.
template <int K, int CB>
__device__ __forceinline__ void eval_staged(const ChunkStage& st, int nc, const float2 (&QX)[K], const float2 (&QY)[K],
                                            const float2 (&QZ)[K], const bool (&slots)[K], float (&s)[K],
                                            float (&c)[K]) {
  const float2 M1 = make_float2(-1.0f, -1.0f);
  auto kahan = [&](int m, float term) {
    const float y = __fsub_rn(term, c[m]);
    const float tt = __fadd_rn(s[m], y);
    c[m] = __fsub_rn(__fsub_rn(tt, s[m]), y);
    s[m] = tt;
  };
#pragma unroll 1
  for (int t = 0; t < nc; t += 2) {
    const bool two = t + 1 < nc;  // warp-uniform: a second candidate in this pair
    const float2 X = ld_pair<CB>(st, SC_X, t), Y = ld_pair<CB>(st, SC_Y, t), Z = ld_pair<CB>(st, SC_Z, t);
    const float2 LX = ld_pair<CB>(st, SC_LX, t), LY = ld_pair<CB>(st, SC_LY, t), LZ = ld_pair<CB>(st, SC_LZ, t);
    const float2 A0 = ld_pair<CB>(st, SC_A0, t), A1 = ld_pair<CB>(st, SC_A1, t), A2 = ld_pair<CB>(st, SC_A2, t),
                 A3 = ld_pair<CB>(st, SC_A3, t);
    const float2 B0 = ld_pair<CB>(st, SC_B0, t), B1 = ld_pair<CB>(st, SC_B1, t), B2 = ld_pair<CB>(st, SC_B2, t);
#pragma unroll
    for (int m = 0; m < K; ++m) {
      if (!slots[m]) continue;  // warp-uniform
      // d = (q - x) - lo
      const float2 dx = __ffma2_rn(LX, M1, __ffma2_rn(X, M1, QX[m]));
      const float2 dy = __ffma2_rn(LY, M1, __ffma2_rn(Y, M1, QY[m]));
      const float2 dz = __ffma2_rn(LZ, M1, __ffma2_rn(Z, M1, QZ[m]));
      // u = A d (amul), s2 = |u|^2
      const float2 u0 = __ffma2_rn(A0, dx, __ffma2_rn(A1, dy, __fmul2_rn(A2, dz)));
      const float2 u1 = __ffma2_rn(A1, dx, __ffma2_rn(A3, dy, __fmul2_rn(B0, dz)));
      const float2 u2 = __ffma2_rn(A2, dx, __ffma2_rn(B0, dy, __fmul2_rn(B1, dz)));
      const float2 s2 = __ffma2_rn(u0, u0, __ffma2_rn(u1, u1, __fmul2_rn(u2, u2)));
      const bool in0 = s2.x < 4.0f, in1 = two && s2.y < 4.0f;
      if (in0 || in1) {
        // bspline_s2 on both: q = s2 / sqrt(s2), b1 = 1 + s2 (0.75 q - 1.5),
        // b2 = 0.25 (2 - q)^3, q <= 1 ? b1 : b2
        const float2 r = make_float2(rsqrtf(fmaxf(s2.x, 1e-30f)), rsqrtf(fmaxf(s2.y, 1e-30f)));
        const float2 q = __fmul2_rn(s2, r);
        const float2 b1 = __ffma2_rn(s2, __ffma2_rn(make_float2(0.75f, 0.75f), q, make_float2(-1.5f, -1.5f)),
                                     make_float2(1.0f, 1.0f));
        const float2 tq = __ffma2_rn(q, M1, make_float2(2.0f, 2.0f));
        const float2 b2 = __fmul2_rn(__fmul2_rn(__fmul2_rn(make_float2(0.25f, 0.25f), tq), tq), tq);
        const float2 term = __fmul2_rn(B2, make_float2(q.x <= 1.0f ? b1.x : b2.x, q.y <= 1.0f ? b1.y : b2.y));
        if (in0) kahan(m, term.x);
        if (in1) kahan(m, term.y);
      }
    }
  }
}

// Sums over the chunk's candidates for the K points of this lane.  act[m]
// marks the lane's valid points, and an invalid point's coordinates must be
// NaN (its s2 is then NaN and no term passes s2 < 4); slots[m]
// (warp-uniform) tells whether any lane holds a point m.  Returns the
// compensated sums in sum[]; adds the algorithmic candidate pairs of the
// lane's points to pairs.
//
// Two consecutive staged candidates are evaluated together with Blackwell's
// packed FP32 instructions (__ffma2_rn, __fmul2_rn, __fadd2_rn: two IEEE
// round-to-nearest operations per instruction, each element rounded as the
// scalar instruction rounds it), from the offset q - x through the kernel
// term det * Sigma * B(|A d|).  The expressions are those of field_sum (a - b
// as fma(b, -1, a), exact in the product, one rounding), so every term is
// bit for bit the scalar one; the compensated sum then takes the two terms
// one after the other, in candidate order.
// CB staged candidates per warp (a multiple of 32 above 32); the flush
// points move with it, the terms and their order do not.
template <int K, int CB = kCandBuf>
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
  // the lane's points as packed pairs (q, q), built once per chunk
  float2 QX[K], QY[K], QZ[K];
#pragma unroll
  for (int m = 0; m < K; ++m) {
    QX[m] = make_float2(qx[m], qx[m]);
    QY[m] = make_float2(qy[m], qy[m]);
    QZ[m] = make_float2(qz[m], qz[m]);
  }
  // compensated sums (Kahan), updated only for in-support terms
  float s[K], c[K];
#pragma unroll
  for (int m = 0; m < K; ++m) s[m] = c[m] = 0.f;
  int nc = 0;
  auto flush = [&]() {
    cp_async_wait_all();
    __syncwarp();
    eval_staged<K, CB>(st, nc, QX, QY, QZ, slots, s, c);
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
          float* const c0 = st.c + p;
          c0[SC_X * CB] = x.x;
          c0[SC_Y * CB] = x.y;
          c0[SC_Z * CB] = x.z;
          const float* ga = reinterpret_cast<const float*>(P.ga + j);
          const float* gb = reinterpret_cast<const float*>(P.gb + j);
          const float* gl = reinterpret_cast<const float*>(P.xlo + j);
          cp_async4(c0 + SC_LX * CB, gl);
          cp_async4(c0 + SC_LY * CB, gl + 1);
          cp_async4(c0 + SC_LZ * CB, gl + 2);
          cp_async4(c0 + SC_A0 * CB, ga);
          cp_async4(c0 + SC_A1 * CB, ga + 1);
          cp_async4(c0 + SC_A2 * CB, ga + 2);
          cp_async4(c0 + SC_A3 * CB, ga + 3);
          cp_async4(c0 + SC_B0 * CB, gb);
          cp_async4(c0 + SC_B1 * CB, gb + 1);
          cp_async4(c0 + SC_B2 * CB, gb + 2);
        }
        nc += __popc(pm);
        if (nc > CB - 32) flush();
      }
    }
  flush();
#pragma unroll
  for (int m = 0; m < K; ++m) sum[m] = s[m];
}


// ---------------------------------------------------------------------------
// Bulk staging (configurations with `bulk` set in kEvalTable): each 27-cell
// row run is copied whole, in pieces of kBulkCap records, by 1D TMA bulk
// copies (cp.async.bulk, one per record array, completion counted on an
// mbarrier) into a per-warp AoS buffer; the warp then applies the same box
// test from shared memory and writes the survivors into the SoA buffer the
// evaluation loop reads.  Same candidates, same order, same values as
// chunk_field.  Waits are bounded: a wait that runs out counts
// C_STAGE_TIMEOUT (the host fails the frame), waits once more for the copies
// in flight and stops the warp.
// ---------------------------------------------------------------------------
constexpr int kBulkCap = 64;  // records per bulk piece

__device__ __forceinline__ void mbar_init(uint64_t* bar) {
  const unsigned a = (unsigned)__cvta_generic_to_shared(bar);
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(a) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
}

__device__ __forceinline__ void mbar_expect(uint64_t* bar, unsigned tx) {
  const unsigned b = (unsigned)__cvta_generic_to_shared(bar);
  asm volatile("{ .reg .b64 st; mbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1; }\n" ::"r"(b), "r"(tx)
               : "memory");
}

// 16-byte aligned global -> shared copy of `bytes` (a multiple of 16)
__device__ __forceinline__ void bulk_copy(float4* dst, const float4* src, unsigned bytes, uint64_t* bar) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  const unsigned b = (unsigned)__cvta_generic_to_shared(bar);
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(d),
               "l"(src), "r"(bytes), "r"(b)
               : "memory");
}

// Bounded wait for the barrier's phase `parity`; false when the limit ran out.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned parity) {
  const unsigned b = (unsigned)__cvta_generic_to_shared(bar);
  for (int it = 0; it < (1 << 22); ++it) {
    unsigned done;
    asm volatile(
        "{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p; }\n"
        : "=r"(done)
        : "r"(b), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

struct BulkStage {
  float4* rec;     // 4 x kBulkCap records: xm, xlo, ga, gb
  uint64_t* bar;   // the warp's barrier
  unsigned phase;  // parity of the next completion
};

// chunk_field with bulk staging; returns false after a wait ran out.
template <int K, int CB>
__device__ __forceinline__ bool chunk_field_bulk(const GridView& g, const PartView& P, int cx, int cy, int cz,
                                                 const float (&qx)[K], const float (&qy)[K], const float (&qz)[K],
                                                 const bool (&act)[K], const bool (&slots)[K], const ChunkStage& st,
                                                 BulkStage& bs, unsigned long long* counters, float (&sum)[K],
                                                 long long& pairs) {
  const int lane = threadIdx.x & 31;
  const unsigned lt = (1u << lane) - 1u;
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
  float2 QX[K], QY[K], QZ[K];
#pragma unroll
  for (int m = 0; m < K; ++m) {
    QX[m] = make_float2(qx[m], qx[m]);
    QY[m] = make_float2(qy[m], qy[m]);
    QZ[m] = make_float2(qz[m], qz[m]);
  }
  float s[K], c[K];
#pragma unroll
  for (int m = 0; m < K; ++m) s[m] = c[m] = 0.f;
  int nc = 0;
  auto flush = [&]() {
    __syncwarp();
    eval_staged<K, CB>(st, nc, QX, QY, QZ, slots, s, c);
    __syncwarp();
    nc = 0;
  };
  for (int dz = -1; dz <= 1; ++dz)
    for (int dy = -1; dy <= 1; ++dy) {
      int rs, re;
      if (!nb_row(g, cx, cy + dy, cz + dz, &rs, &re)) continue;
      pairs += (long long)(re - rs) * nact;
      for (int j0 = rs; j0 < re; j0 += kBulkCap) {
        const int cnt = min(kBulkCap, re - j0);
        const unsigned bytes = 16u * (unsigned)cnt;
        __syncwarp();  // every lane is done with the previous piece
        if (lane == 0) {
          asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
          mbar_expect(bs.bar, 4u * bytes);
          bulk_copy(bs.rec, P.xm + j0, bytes, bs.bar);
          bulk_copy(bs.rec + kBulkCap, P.xlo + j0, bytes, bs.bar);
          bulk_copy(bs.rec + 2 * kBulkCap, P.ga + j0, bytes, bs.bar);
          bulk_copy(bs.rec + 3 * kBulkCap, P.gb + j0, bytes, bs.bar);
        }
        if (!mbar_wait(bs.bar, bs.phase)) {
          if (lane == 0) stripe_add(counters, C_STAGE_TIMEOUT, 1ull);
          mbar_wait(bs.bar, bs.phase);  // the copies in flight, once more
          return false;
        }
        bs.phase ^= 1u;
        for (int k0 = 0; k0 < cnt; k0 += 32) {
          const int k = k0 + lane;
          bool pass = false;
          float4 x;
          if (k < cnt) {
            x = bs.rec[k];
            const float ex = fmaxf(fmaxf(blx - x.x, x.x - bhx), 0.f);
            const float ey = fmaxf(fmaxf(bly - x.y, x.y - bhy), 0.f);
            const float ez = fmaxf(fmaxf(blz - x.z, x.z - bhz), 0.f);
            pass = fmaf(ex, ex, fmaf(ey, ey, ez * ez)) < x.w;
          }
          const unsigned pm = __ballot_sync(0xffffffffu, pass);
          if (pass) {
            float* const c0 = st.c + nc + __popc(pm & lt);
            const float4 l = bs.rec[kBulkCap + k], a = bs.rec[2 * kBulkCap + k], b = bs.rec[3 * kBulkCap + k];
            c0[SC_X * CB] = x.x;
            c0[SC_Y * CB] = x.y;
            c0[SC_Z * CB] = x.z;
            c0[SC_LX * CB] = l.x;
            c0[SC_LY * CB] = l.y;
            c0[SC_LZ * CB] = l.z;
            c0[SC_A0 * CB] = a.x;
            c0[SC_A1 * CB] = a.y;
            c0[SC_A2 * CB] = a.z;
            c0[SC_A3 * CB] = a.w;
            c0[SC_B0 * CB] = b.x;
            c0[SC_B1 * CB] = b.y;
            c0[SC_B2 * CB] = b.z;
          }
          nc += __popc(pm);
          if (nc > CB - 32) flush();
        }
      }
    }
  flush();
#pragma unroll
  for (int m = 0; m < K; ++m) sum[m] = s[m];
  return true;
}

}  // namespace pisurf
