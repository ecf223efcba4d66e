// K4: adaptive octree, genIsoOurs state 0 (src/surface_reconstructor.cpp:326-407).
//
// The reference keeps a LIFO of nodes but processes the whole frontier at
// once (inProcessSize = 10^7), so refinement is breadth-first: one level per
// iteration.  Per level:
//   k_empty      emptiness of beforeSampleEval / checkEmptyAndCalcCurv
//                (:152-235): one warp per node, an existence test with early
//                exit over the hash cells that the node box grown by
//                r * smooth_factor touches.  Every particle strictly inside
//                the grown box lies in those cells (the float cell index is
//                monotonic in the coordinate), and they lie inside the
//                reference's block of box +- 1 cell, so the decision is the
//                reference's.
//   k_q_count_node / the 27 lattice samples and the centre of every non-empty
//   k_q_dedupe   node (TNode::GenerateSampling, src/iso_method_ours.cpp:52-75)
//                are bucketed by hash cell and octant with an atomic counting
//                sort, and points with bit-identical coordinates (shared by
//                neighbouring nodes) are evaluated once; the order inside a
//                bucket does not affect any result.
//   k_q_eval     field at the bucketed points (Evaluator::SingleEval,
//                src/evaluator.cpp:60-87): one warp per chunk of <= 32
//                samples of one bucket; the cell's 27-cell candidates are
//                filtered against the chunk's bounding box into shared
//                memory, then every lane walks the survivors (broadcast
//                loads, uniform loop bounds).
//   k_classify   afterSampleEval (:237-273): sign change against sample 0
//                (ballot), leaf by size, and the normal-coherence curvature
//                |sum n| / sum |n| computed only where the classification reads
//                it (nodes with a sign change that are not leaves by size).
//   k_spawn      8 children per INTERNAL node (TNode ctor,
//                src/iso_method_ours.cpp:25-38) after a scan of the flags.
#include <algorithm>
#include <cmath>

#include <cooperative_groups.h>

#include "chunk.cuh"
#include "device.cuh"
#include "internal.h"

namespace pisurf {

enum : int8_t { T_EMPTY = 0, T_INTERNAL = 1, T_LEAF = 2, T_UNCERTAIN = 3 };

constexpr int kQ = 28;  // 27 samples + the centre per node
constexpr int kSpawnWarps = 2;  // warps per block of k_spawn_scan (small blocks: a warp that scans a whole block does not hold up seven others)
// The leaf level with the QEF on runs in pi_ctx::qef_parts parts pipelined
// against the QEF stream; there the chunked evaluator leaves this many
// registers per SM free for k_qef's blocks (64 threads at up to 128
// registers: 8192 per block).
constexpr int kQefReserveRegs = 2 * 8192;

struct LevelArgs {
  GridView g;
  const float4* pos;
  const float4* nrm;
  float expand;  // r * smooth_factor
  float iso;
  float radius;
  long long lb, le;  // node range of the level
  int big;           // depth < D_min
  PartView P;
};

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Node box grown by `expand` and the block of hash cells it touches.
struct GrownBox {
  float lox, loy, loz, hix, hiy, hiz;
  int x0, x1, y0, y1, z0, z1;
};

__device__ __forceinline__ GrownBox grown_box(const GridView& g, float4 c, float expand) {
  GrownBox b;
  const float h = c.w;
  b.lox = __fsub_rn(__fsub_rn(c.x, h), expand);
  b.loy = __fsub_rn(__fsub_rn(c.y, h), expand);
  b.loz = __fsub_rn(__fsub_rn(c.z, h), expand);
  b.hix = __fadd_rn(__fadd_rn(c.x, h), expand);
  b.hiy = __fadd_rn(__fadd_rn(c.y, h), expand);
  b.hiz = __fadd_rn(__fadd_rn(c.z, h), expand);
  b.x0 = max(cell_coord(b.lox, g.b0, g.cell, g.nx), 0);
  b.y0 = max(cell_coord(b.loy, g.b2, g.cell, g.ny), 0);
  b.z0 = max(cell_coord(b.loz, g.b4, g.cell, g.nz), 0);
  b.x1 = min(cell_coord(b.hix, g.b0, g.cell, g.nx), g.nx - 1);
  b.y1 = min(cell_coord(b.hiy, g.b2, g.cell, g.ny), g.ny - 1);
  b.z1 = min(cell_coord(b.hiz, g.b4, g.cell, g.nz), g.nz - 1);
  return b;
}

// A particle counts for a node when it lies in the grown box and is not a
// splash particle (pos.w = 1, checkEmptyAndCalcCurv's CheckSplash test).
__device__ __forceinline__ bool inside(const GrownBox& b, float4 p) {
  return p.x > b.lox && p.x < b.hix && p.y > b.loy && p.y < b.hiy && p.z > b.loz && p.z < b.hiz && p.w == 0.f;
}

// Particle range of cell c (linear index over the block) of a grown box.
__device__ __forceinline__ void block_cell(const GridView& g, const GrownBox& b, int c, int* s, int* e) {
  const int nxb = b.x1 - b.x0 + 1, nyb = b.y1 - b.y0 + 1;
  const int x = b.x0 + c % nxb, y = b.y0 + (c / nxb) % nyb, z = b.z0 + c / (nxb * nyb);
  const long long k = ((long long)z * g.ny + y) * g.nx + x;
  *s = __ldg(g.off + k);
  *e = __ldg(g.off + k + 1);
}

__device__ __forceinline__ int block_cells(const GrownBox& b) {
  if (b.x0 > b.x1 || b.y0 > b.y1 || b.z0 > b.z1) return 0;
  return (b.x1 - b.x0 + 1) * (b.y1 - b.y0 + 1) * (b.z1 - b.z0 + 1);
}

__global__ void k_empty(LevelArgs a, const float4* __restrict__ nd_c, float4* __restrict__ nd_v,
                        int8_t* __restrict__ nd_type, float* __restrict__ nd_curv) {
  const long long node = a.lb + (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (node >= a.le) return;
  const GrownBox b = grown_box(a.g, nd_c[node], a.expand);
  // the block's rows (z, y) are spread over the lanes; each lane stops at the
  // first particle inside, the warp at the first batch of rows with a hit
  bool found = false;
  if (b.x0 <= b.x1 && b.y0 <= b.y1 && b.z0 <= b.z1) {
    const int nyb = b.y1 - b.y0 + 1;
    const int rows = (b.z1 - b.z0 + 1) * nyb;
    for (int r0 = 0; r0 < rows && !found; r0 += 32) {
      const int r = r0 + lane;
      bool hit = false;
      if (r < rows) {
        const int z = b.z0 + r / nyb, y = b.y0 + r % nyb;
        const long long base = ((long long)z * a.g.ny + y) * a.g.nx;
        const int s = __ldg(a.g.off + base + b.x0), e = __ldg(a.g.off + base + b.x1 + 1);
        for (int j = s; j < e; ++j)
          if (inside(b, __ldg(a.pos + j))) {
            hit = true;
            break;
          }
      }
      found = __any_sync(0xffffffffu, hit);
    }
  }
  if (lane == 0) {
    if (!found) {
      nd_type[node] = T_EMPTY;
      nd_curv[node] = 1.0f;  // area == 0
      float4 v = nd_v[node];
      v.w = a.iso;
      nd_v[node] = v;
    } else {
      nd_type[node] = a.big ? T_INTERNAL : T_UNCERTAIN;
      nd_curv[node] = -1.0f;  // not needed unless a sign change asks for it
    }
  }
}

// Sample s (< 27) of the node lattice, or the node position (s == 27).
__device__ __forceinline__ void sample_point(const float4 c, const float4 v, int s, float& qx, float& qy,
                                             float& qz) {
  if (s < 27) {
    const float h = c.w;
    const float tx = (s % 3) * 0.5f, ty = ((s / 3) % 3) * 0.5f, tz = (s / 9) * 0.5f;
    qx = __fadd_rn(__fmul_rn(1.0f - tx, __fsub_rn(c.x, h)), __fmul_rn(tx, __fadd_rn(c.x, h)));
    qy = __fadd_rn(__fmul_rn(1.0f - ty, __fsub_rn(c.y, h)), __fmul_rn(ty, __fadd_rn(c.y, h)));
    qz = __fadd_rn(__fmul_rn(1.0f - tz, __fsub_rn(c.z, h)), __fmul_rn(tz, __fadd_rn(c.z, h)));
  } else {
    qx = v.x, qy = v.y, qz = v.z;
  }
}

struct QArgs {
  GridView g;
  PartView P;
  float iso;
  long long lb, le;
  int ekx, eky;  // extended key strides (nx + 4, ny + 4)
  int octants;   // 1: buckets are cell octants, 0: whole cells
};

// Hash cell of a point as a key over the grid grown by 2 cells on each side
// (cell_coord clamps to [-2, n + 1]).
__device__ __forceinline__ int ext_key(const QArgs& a, int cx, int cy, int cz) {
  return ((cz + 2) * a.eky + (cy + 2)) * a.ekx + (cx + 2);
}

// Bucket of a sample: its hash cell (extended key, the cell of
// CalcXYZIdx), times 8 plus the octant of the cell it lies in when a.octants
// is set (from the same quotients), so that a chunk's points are close
// together.  One thread per node: a sample's coordinate on an axis is one of
// three values per node (t = 0, 1/2, 1), so the node needs 9 cell
// coordinates and octant bits (plus 3 for its position) rather than 84; the
// key separates by axis, so the 27 samples fall into the products of the
// per-axis runs of equal (cell, octant), counted with one atomic per
// distinct bucket.  The keys go through shared memory so that the block
// writes its nodes' keys as one contiguous run.
constexpr int kCountThreads = 128;
__global__ void __launch_bounds__(kCountThreads) k_q_count_node(QArgs a, const float4* __restrict__ nd_c,
                                                                const float4* __restrict__ nd_v,
                                                                const int8_t* __restrict__ nd_type,
                                                                int* __restrict__ qcnt, int* __restrict__ qkey) {
  __shared__ int s_key[kCountThreads * kQ];
  const long long t0 = (long long)blockIdx.x * kCountThreads;
  const long long node = a.lb + t0 + threadIdx.x;
  const long long nl = a.le - a.lb;
  int* const mine = s_key + threadIdx.x * kQ;
  if (node < a.le && nd_type[node] == T_UNCERTAIN) {
    const float4 c = nd_c[node], v = nd_v[node];
    const float h = c.w;
    const float cc[3] = {c.x, c.y, c.z}, vv[3] = {v.x, v.y, v.z};
    const float lo[3] = {a.g.b0, a.g.b2, a.g.b4};
    const int n[3] = {a.g.nx, a.g.ny, a.g.nz};
    int ck[3][4], ob[3][4];  // per axis: cell and octant bit of t = 0, 1/2, 1 and of the node position
#pragma unroll
    for (int ax = 0; ax < 3; ++ax) {
      const float mn = __fsub_rn(cc[ax], h), mx = __fadd_rn(cc[ax], h);
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        // sample_point's expression for t = k / 2 (k < 3), the position for k = 3
        const float tt = k * 0.5f;
        const float q = k < 3 ? __fadd_rn(__fmul_rn(1.0f - tt, mn), __fmul_rn(tt, mx)) : vv[ax];
        float f;
        ck[ax][k] = cell_coord_q(q, lo[ax], a.g.cell, n[ax], f);
        ob[ax][k] = f - (float)ck[ax][k] >= 0.5f ? 1 : 0;
      }
    }
    auto key = [&](int kx, int ky, int kz) {
      int k = ext_key(a, ck[0][kx], ck[1][ky], ck[2][kz]);
      if (a.octants) k = k * 8 + (ob[0][kx] | (ob[1][ky] << 1) | (ob[2][kz] << 2));
      return k;
    };
#pragma unroll
    for (int s = 0; s < 27; ++s) mine[s] = key(s % 3, (s / 3) % 3, s / 9);
    mine[27] = key(3, 3, 3);
    // runs of equal (cell, octant) per axis over t = 0, 1/2, 1 (both grow
    // with t, so equal values are adjacent): a run starts at k where the
    // value changes, and the samples whose indices all start runs carry the
    // count of their bucket (the product of the three run lengths)
    bool same[3][2];  // same[ax][k]: t = k / 2 and t = (k + 1) / 2 share a bucket component
    int len[3][3];    // run length from k (counted at run starts only)
#pragma unroll
    for (int ax = 0; ax < 3; ++ax) {
#pragma unroll
      for (int k = 0; k < 2; ++k)
        same[ax][k] = ck[ax][k] == ck[ax][k + 1] && (!a.octants || ob[ax][k] == ob[ax][k + 1]);
      len[ax][0] = 1 + (same[ax][0] ? 1 + (same[ax][1] ? 1 : 0) : 0);
      len[ax][1] = 1 + (same[ax][1] ? 1 : 0);
      len[ax][2] = 1;
    }
#pragma unroll
    for (int s = 0; s < 27; ++s) {
      const int kx = s % 3, ky = (s / 3) % 3, kz = s / 9;
      const bool start = (kx == 0 || !same[0][kx > 0 ? kx - 1 : 0]) && (ky == 0 || !same[1][ky > 0 ? ky - 1 : 0]) &&
                         (kz == 0 || !same[2][kz > 0 ? kz - 1 : 0]);
      if (start) atomicAdd(qcnt + mine[s], len[0][kx] * len[1][ky] * len[2][kz]);
    }
    atomicAdd(qcnt + mine[27], 1);
  } else {
#pragma unroll
    for (int s = 0; s < kQ; ++s) mine[s] = -1;
  }
  __syncthreads();
  // the block's keys: slots [t0 * kQ, (t0 + its nodes) * kQ) of the level
  const long long nodes = nl - t0 < kCountThreads ? nl - t0 : kCountThreads;
  const int total = (int)(nodes * kQ);
  int* const out = qkey + t0 * kQ;
  for (int i = threadIdx.x; i < total; i += kCountThreads) out[i] = s_key[i];
}

__device__ __forceinline__ uint32_t hash3(float x, float y, float z) {
  uint32_t h = __float_as_uint(x) * 0x9E3779B1u ^ __float_as_uint(y) * 0x85EBCA77u ^
               __float_as_uint(z) * 0xC2B2AE3Du;
  h ^= h >> 15;
  h *= 0x2C1B3C6Du;
  h ^= h >> 12;
  return h;
}

// Neighbouring nodes share lattice points, and most shared samples have the
// same float coordinates bit for bit (about 2.4 per point on liquid
// surfaces).  Equal coordinates give equal field values (same cell, same
// candidates, same summation order), so each distinct point is evaluated
// once.  Equal points share a bucket; bucket k owns hash slots
// [2 qoff[k], 2 qoff[k+1]) and a point's first inserter becomes its
// representative.  Representatives get consecutive places in the bucket's
// range of `order` (on a dense level k_q_chunks then cuts them into chunks, on
// a sparse level k_q_compact lists them in bucket order).
__global__ void k_q_dedupe(QArgs a, long long n, const float4* __restrict__ nd_c, const float4* __restrict__ nd_v,
                           const int* __restrict__ qkey, const int* __restrict__ qoff, unsigned* __restrict__ hslot,
                           int* __restrict__ ucnt, int* __restrict__ rep, int* __restrict__ order) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  const int k = i < n ? qkey[i] : -1;
  bool uniq = false;
  int place = 0;
  // the node's records load beside the key (the node index is valid for
  // every i < n)
  float4 nc = make_float4(0.f, 0.f, 0.f, 0.f), nv = nc;
  if (i < n) {
    const long long node = a.lb + i / kQ;
    nc = nd_c[node];
    nv = nd_v[node];
  }
  if (k >= 0) {
    float qx, qy, qz;
    sample_point(nc, nv, (int)(i % kQ), qx, qy, qz);
    const long long base = 2LL * qoff[k];
    const uint32_t m = 2u * (uint32_t)(qoff[k + 1] - qoff[k]);
    uint32_t pos = __umulhi(hash3(qx, qy, qz), m);
    int r = (int)i;
    for (uint32_t t = 0; t < m; ++t) {  // the region is at most half full
      unsigned cur = hslot[base + pos];
      if (cur == 0u) {
        cur = atomicCAS(hslot + base + pos, 0u, (unsigned)i + 1u);
        if (cur == 0u) break;  // first inserter: i represents the point
      }
      const long long j = (long long)cur - 1;
      const long long nj = a.lb + j / kQ;
      float px, py, pz;
      sample_point(nd_c[nj], nd_v[nj], (int)(j % kQ), px, py, pz);
      if (__float_as_uint(px) == __float_as_uint(qx) && __float_as_uint(py) == __float_as_uint(qy) &&
          __float_as_uint(pz) == __float_as_uint(qz)) {
        r = (int)j;
        break;
      }
      pos = pos + 1u == m ? 0u : pos + 1u;
    }
    rep[i] = r;
    uniq = r == (int)i;
  }
  // places for the representatives, one atomic per bucket and warp
  const unsigned um = __ballot_sync(0xffffffffu, uniq);
  const unsigned peers = __match_any_sync(0xffffffffu, uniq ? k : -1) & um;
  if (uniq) {
    const int leader = __ffs(peers) - 1;
    int b0 = 0;
    if (lane == leader) b0 = atomicAdd(ucnt + k, __popc(peers));
    b0 = __shfl_sync(peers, b0, leader);
    place = b0 + __popc(peers & ((1u << lane) - 1u));
    order[qoff[k] + place] = (int)i;
  }
}

// Chunks of a dense level: each bucket's distinct samples cut into runs of
// `chunk` places (bucket, first place); list order is arbitrary.
__global__ void k_q_chunks(long long nb, const int* __restrict__ ucnt, int chunk, int2* __restrict__ chunks,
                           int* __restrict__ nchunks) {
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  const int u = k < nb ? ucnt[k] : 0;
  const int c = (u + chunk - 1) / chunk;
  int incl = c;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int v = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += v;
  }
  const int total = __shfl_sync(0xffffffffu, incl, 31);
  if (total == 0) return;
  int base = 0;
  if (lane == 31) base = atomicAdd(nchunks, total);
  base = __shfl_sync(0xffffffffu, base, 31) + incl - c;
  for (int j = 0; j < c; ++j) chunks[base + j] = make_int2((int)k, j * chunk);
}

// The leaf level with the QEF on runs in parts, so that the FP64 QEF of one
// part's leaves (QEF stream) overlaps the FP32 sampling of the next part
// (context stream).  Parts are ranges of buckets (z-major cell order, then
// the octant), cut where the exclusive scan of the per-bucket sample slots
// qoff (qoff[nb] slots in all) crosses p / parts of the total.  pinfo holds
// kb[0 .. parts] (first bucket of each part), pb[0 .. parts] (chunk region of
// each part: qoff[kb[p]], since a part never has more chunks than sample
// slots) and the chunk counts cnt[0 .. parts - 1].
__global__ void k_part_bounds(const int* __restrict__ qoff, int nb, int parts, int* __restrict__ pinfo) {
  const int p = threadIdx.x;
  if (p > parts) return;
  int k = p == parts ? nb : 0;
  if (p > 0 && p < parts) {
    const long long target = (long long)qoff[nb] * p / parts;
    int lo = 0, hi = nb;  // smallest k with qoff[k] >= target
    while (lo < hi) {
      const int mid = (int)(((long long)lo + hi) / 2);
      if (qoff[mid] >= target)
        hi = mid;
      else
        lo = mid + 1;
    }
    k = lo;
  }
  pinfo[p] = k;
  pinfo[parts + 1 + p] = qoff[k];
  if (p < parts) pinfo[2 * (parts + 1) + p] = 0;
}

// Part of a bucket key (kb increasing, kb[0] = 0, kb[parts] = nb).
__device__ __forceinline__ int part_of(const int* __restrict__ kb, int parts, int k) {
  int p = 0;
  while (p + 1 < parts && kb[p + 1] <= k) ++p;
  return p;
}

// A node's part: that of its last lattice sample (the corner c + h on every
// axis), whose bucket is the largest of the node's 28: cell coordinates and
// octant bits grow with the coordinates, and the key orders them z, y, x,
// then the octant's z, y, x bits.  So all of a node's samples are evaluated
// once the parts up to its own are.  -1 for a node with no samples.
__global__ void k_node_part(long long nl, const int* __restrict__ qkey, const int* __restrict__ pinfo, int parts,
                            int8_t* __restrict__ npart) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nl) return;
  const int k = qkey[t * kQ + 26];
  npart[t] = k < 0 ? (int8_t)-1 : (int8_t)part_of(pinfo, parts, k);
}

// k_q_chunks with the chunks of part p in the region [pb[p], pb[p + 1]) of
// the list, cnt[p] of them (one atomic per part and warp).
__global__ void k_q_chunks_parts(long long nb, const int* __restrict__ ucnt, int chunk, int parts,
                                 int* __restrict__ pinfo, int2* __restrict__ chunks) {
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  const int u = k < nb ? ucnt[k] : 0;
  const int c = (u + chunk - 1) / chunk;
  const int p = k < nb ? part_of(pinfo, parts, (int)k) : parts - 1;
  const int* pb = pinfo + parts + 1;
  int* cnt = pinfo + 2 * (parts + 1);
  const unsigned peers = __match_any_sync(0xffffffffu, p);  // contiguous lanes: p grows with k
  // inclusive sum of c over this lane's part group, in lane order
  int incl = c;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int v = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += v;
  }
  // the group's sums are differences of the warp's inclusive sums
  const int leader = __ffs(peers) - 1, last = 31 - __clz(peers);
  const int before = __shfl_sync(0xffffffffu, incl - c, leader);  // exclusive sum at the group's first lane
  const int total = __shfl_sync(0xffffffffu, incl, last) - before;
  int base = 0;
  if (lane == leader && total > 0) base = atomicAdd(cnt + p, total);
  base = __shfl_sync(0xffffffffu, base, leader) + pb[p] + incl - c - before;
  for (int j = 0; j < c; ++j) chunks[base + j] = make_int2((int)k, j * chunk);
}

// Field at the samples of one chunk per warp (persistent, grid-stride over
// the chunks); a chunk holds up to 32 K samples and lane l holds samples
// l, l + 32, ..., K per lane (K, W and CB are autotuned per context, see
// eval_config_for).  All samples of a chunk share a hash cell, hence the
// 27-cell candidate list of Evaluator::SingleEval; chunk_field filters the
// candidates against the chunk's bounding box, stages the survivors in
// shared memory and sums in candidate order.
// Blocks of W warps, each with a staging buffer of CB candidates (static
// shared memory W * 13 * CB floats, plus 4 KiB per warp with bulk staging,
// at most 48 KiB); the register bound keeps 768 (K = 4) or 1024 threads per
// SM whatever W.  BULK selects the bulk (TMA) staging of chunk_field_bulk.
template <int K, int W, int CB, bool BULK>
__global__ void __launch_bounds__(32 * W, (K > 2 ? 24 : 32) / W) k_q_eval(QArgs a, const int* __restrict__ order,
                                                            const int* __restrict__ qoff,
                                                            const int* __restrict__ ucnt,
                                                            const int2* __restrict__ chunks,
                                                            const int* __restrict__ nchunks_ptr,
                                                            const int* __restrict__ cbeg_ptr,
                                                            const float4* __restrict__ nd_c,
                                                            const float4* __restrict__ nd_v,
                                                            float* __restrict__ qval,
                                                            unsigned long long* __restrict__ counters) {
  __shared__ __align__(16) float s_stage[W][stage_floats(CB)];
  __shared__ __align__(16) float4 s_bulk[BULK ? W : 1][BULK ? 4 * kBulkCap : 1];
  __shared__ __align__(8) uint64_t s_bar[W];
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  const ChunkStage st{s_stage[wib]};
  BulkStage bs{s_bulk[BULK ? wib : 0], &s_bar[wib], 0u};
  if (BULK) {
    if (lane == 0) mbar_init(bs.bar);
    __syncwarp();
  }
  // chunks [c0, c0 + count): a part of the level, or all of it from 0
  const int c0 = cbeg_ptr ? *cbeg_ptr : 0;
  const int cend = c0 + *nchunks_ptr;
  const int nwarps = gridDim.x * W;
  long long pairs = 0, done = 0;
  for (int ci = c0 + blockIdx.x * W + wib; ci < cend; ci += nwarps) {
    const int2 ch = chunks[ci];
    const int len = min(32 * K, __ldg(ucnt + ch.x) - ch.y);
    done += len;
    const int* ord = order + __ldg(qoff + ch.x) + ch.y;
    int q[K];
    float x[K], y[K], z[K];
    bool act[K], slots[K];
#pragma unroll
    for (int m = 0; m < K; ++m) {
      q[m] = 0;
      x[m] = y[m] = z[m] = __int_as_float(0x7fc00000);  // NaN: no term for an invalid point
      act[m] = lane + 32 * m < len;
      slots[m] = len > 32 * m;  // warp-uniform
      if (act[m]) {
        q[m] = ord[lane + 32 * m];
        const long long node = a.lb + q[m] / kQ;
        sample_point(nd_c[node], nd_v[node], q[m] % kQ, x[m], y[m], z[m]);
      }
    }
    int cx, cy, cz;
    cell_of(a.g, __shfl_sync(0xffffffffu, x[0], 0), __shfl_sync(0xffffffffu, y[0], 0),
            __shfl_sync(0xffffffffu, z[0], 0), cx, cy, cz);
    float sum[K];
    if (BULK) {
      if (!chunk_field_bulk<K, CB>(a.g, a.P, cx, cy, cz, x, y, z, act, slots, st, bs, counters, sum, pairs))
        return;  // a staging wait ran out: the frame fails (C_STAGE_TIMEOUT)
    } else {
      chunk_field<K, CB>(a.g, a.P, cx, cy, cz, x, y, z, act, slots, st, sum, pairs);
    }
#pragma unroll
    for (int m = 0; m < K; ++m)
      if (act[m]) qval[q[m]] = a.iso - sum[m];
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) pairs += __shfl_xor_sync(0xffffffffu, pairs, o);
  if (lane == 0) {
    stripe_add(counters, C_SAMPLE_PAIRS, (unsigned long long)pairs);
    stripe_add(counters, C_PAIRS_CHUNK, (unsigned long long)pairs);
    stripe_add(counters, C_DONE_CHUNK, (unsigned long long)done);
  }
}

// Sparse levels (a few distinct samples per bucket): one thread per distinct
// sample, each walking its own 27-cell candidate list (field_sum, the same
// tests and summation order as k_q_eval).  The list is in bucket order, so a
// warp's threads mostly share their cells and walk the same rows.
__global__ void __launch_bounds__(256, 4) k_q_eval_thread(QArgs a, const int* __restrict__ list,
                                                       const int* __restrict__ count_ptr,
                                                       const float4* __restrict__ nd_c,
                                                       const float4* __restrict__ nd_v, float* __restrict__ qval,
                                                       unsigned long long* __restrict__ counters) {
  const int n = *count_ptr;
  long long pairs = 0, done = 0;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    const int q = list[t];
    const long long node = a.lb + q / kQ;
    float qx, qy, qz;
    sample_point(nd_c[node], nd_v[node], q % kQ, qx, qy, qz);
    qval[q] = a.iso - field_sum(a.g, a.P, qx, qy, qz, &pairs);
    ++done;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    pairs += __shfl_xor_sync(0xffffffffu, pairs, o);
    done += __shfl_xor_sync(0xffffffffu, done, o);
  }
  if ((threadIdx.x & 31) == 0) {
    stripe_add(counters, C_SAMPLE_PAIRS, (unsigned long long)pairs);
    stripe_add(counters, C_PAIRS_THREAD, (unsigned long long)pairs);
    stripe_add(counters, C_DONE_THREAD, (unsigned long long)done);
  }
}

// Sparse levels: the distinct samples, placed per bucket by k_q_dedupe, made
// into one list in bucket order (ucum = exclusive scan of the bucket counts),
// so that neighbouring threads of k_q_eval_thread walk the same cells.
__global__ void k_q_compact(long long nb, const int* __restrict__ qoff, const int* __restrict__ ucnt,
                            const int* __restrict__ ucum, const int* __restrict__ order, int* __restrict__ list) {
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nb) return;
  const int u = ucnt[k];
  if (u == 0) return;
  const int* src = order + qoff[k];
  int* dst = list + ucum[k];
  for (int t = 0; t < u; ++t) dst[t] = src[t];
}

// Leaves by size without QEF: afterSampleEval (src/surface_reconstructor.cpp:
// 247-255) makes every node of size r a LEAF whose value is SingleEval at its
// position; the 27 lattice samples of GridEval only set a sign-change flag
// that nothing reads there (they feed NodeCalcNode, i.e. QEF mode only), so
// only the node position is evaluated.  The node's signchange stays 0.
__global__ void __launch_bounds__(256, 4) k_leaf_level(LevelArgs a, const float4* __restrict__ nd_c,
                                                       float4* __restrict__ nd_v, int8_t* __restrict__ nd_type,
                                                       unsigned long long* __restrict__ counters) {
  long long pairs = 0, evals = 0;
  for (long long node = a.lb + (long long)blockIdx.x * blockDim.x + threadIdx.x; node < a.le;
       node += (long long)gridDim.x * blockDim.x) {
    if (nd_type[node] != T_UNCERTAIN) continue;
    float4 v = nd_v[node];
    v.w = a.iso - field_sum(a.g, a.P, v.x, v.y, v.z, &pairs);
    nd_v[node] = v;
    nd_type[node] = T_LEAF;
    ++evals;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    pairs += __shfl_xor_sync(0xffffffffu, pairs, o);
    evals += __shfl_xor_sync(0xffffffffu, evals, o);
  }
  if ((threadIdx.x & 31) == 0) {
    stripe_add(counters, C_SAMPLE_PAIRS, (unsigned long long)pairs);
    stripe_add(counters, C_PAIRS_LEAF, (unsigned long long)pairs);
    stripe_add(counters, C_DONE_LEAF, (unsigned long long)evals);
    // the reference evaluates the 27 lattice samples (GridEval) and the
    // leaf value of each of these nodes
    stripe_add(counters, C_REF_EVALS, (unsigned long long)(28 * evals));
  }
}

__global__ void __launch_bounds__(64, 24) k_classify(LevelArgs a, const float* __restrict__ qval, const int* __restrict__ rep,
                           const float4* __restrict__ nd_c,
                           float4* __restrict__ nd_v, int8_t* __restrict__ nd_type, int8_t* __restrict__ nd_sc,
                           float* __restrict__ nd_curv, float* __restrict__ nd_samp, int qef, int curv_known,
                           unsigned long long* __restrict__ counters, const float* __restrict__ nd_minr) {
  const long long node = a.lb + (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (node >= a.le) return;
  // the node's type and its samples' representatives are loaded together
  // (the representative indices are valid whatever the type)
  const long long qb = (node - a.lb) * kQ;
  const int8_t ntype = nd_type[node];
  const int r = lane < kQ ? rep[qb + lane] : 0;
  const float4 c = nd_c[node];
  if (ntype != T_UNCERTAIN) return;  // warp-uniform
  const float val = lane < kQ ? qval[r] : 0.f;
  // GridEval sign change against sample 0, ">= 0" (src/evaluator.cpp:169-172)
  const unsigned pos_mask = __ballot_sync(0xffffffffu, lane < 27 && val >= 0.f);
  const bool origin = pos_mask & 1u;
  const bool signchange = origin ? (pos_mask != 0x07ffffffu) : (pos_mask != 0u);
  const float vc = __shfl_sync(0xffffffffu, val, 27);
  if (qef && lane < 27) nd_samp[node * 27 + lane] = val;
  const float cellsize = 2.0f * c.w;
  // leaf by size: the node is no larger than the radius (variable radius:
  // the smallest radius of the particles reaching it, src/surface_
  // reconstructor.cpp:156,203-208,247)
  const bool leaf_by_size = cellsize - (nd_minr ? nd_minr[node] : a.radius) < kAbove1em8;
  int8_t type = T_LEAF;
  float curv = -1.0f;
  if (!leaf_by_size && signchange && curv_known) {
    curv = nd_curv[node];  // summed by the parent's scan (k_spawn_scan)
    if (curv < kAbove099) type = T_INTERNAL;
  } else if (!leaf_by_size && signchange) {
    // checkEmptyAndCalcCurv sums over particles inside the grown box
    const GrownBox b = grown_box(a.g, c, a.expand);
    Kahan sx, sy, sz, ar;
    const int ncell = block_cells(b);
    for (int c0 = lane; c0 < ncell; c0 += 32) {
      int s, e;
      block_cell(a.g, b, c0, &s, &e);
      for (int j = s; j < e; ++j) {
        const float4 p = __ldg(a.pos + j);
        if (inside(b, p)) {
          const float4 nv = __ldg(a.nrm + j);
          sx.add(nv.x);
          sy.add(nv.y);
          sz.add(nv.z);
          ar.add(nv.w);
        }
      }
    }
    const float nx = warp_sum(sx.s - sx.c), ny = warp_sum(sy.s - sy.c), nz = warp_sum(sz.s - sz.c);
    const float area = warp_sum(ar.s - ar.c);
    curv = (area == 0.f) ? 1.0f : sqrtf(nx * nx + ny * ny + nz * nz) / area;
    if (curv < kAbove099) type = T_INTERNAL;
  }
  if (lane == 0) {
    nd_type[node] = type;
    nd_sc[node] = signchange ? 1 : 0;
    if (curv >= 0.f) nd_curv[node] = curv;
    if (type == T_LEAF) {
      float4 v = nd_v[node];
      v.w = vc;
      nd_v[node] = v;
    }
    stripe_add(counters, C_REF_EVALS, (unsigned long long)(27 + (type == T_LEAF ? 1 : 0)));
  }
}

// k_classify for a level that needs no particle scan: its nodes are leaves
// by size, or their curvature was summed by the parents' scan.  One thread
// per node gathers its 28 values (independent loads in flight together)
// instead of a warp per node; the decisions and values are k_classify's.
__global__ void __launch_bounds__(256) k_classify_thread(LevelArgs a, const float* __restrict__ qval,
                                                         const int* __restrict__ rep, const float4* __restrict__ nd_c,
                                                         float4* __restrict__ nd_v, int8_t* __restrict__ nd_type,
                                                         int8_t* __restrict__ nd_sc, float* __restrict__ nd_curv,
                                                         float* __restrict__ nd_samp, int qef,
                                                         unsigned long long* __restrict__ counters,
                                                         const int8_t* __restrict__ npart, int part) {
  const long long node = a.lb + (long long)blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long evals = 0;
  if (node < a.le && (!npart || npart[node - a.lb] == part) && nd_type[node] == T_UNCERTAIN) {
    const long long qb = (node - a.lb) * kQ;
    float val[kQ];
#pragma unroll
    for (int q = 0; q < kQ; ++q) val[q] = qval[__ldg(rep + qb + q)];
    // GridEval sign change against sample 0, ">= 0" (src/evaluator.cpp:169-172)
    const bool origin = val[0] >= 0.f;
    bool signchange = false;
#pragma unroll
    for (int q = 1; q < 27; ++q) signchange |= (val[q] >= 0.f) != origin;
    if (qef)
#pragma unroll
      for (int q = 0; q < 27; ++q) nd_samp[node * 27 + q] = val[q];
    const float4 c = nd_c[node];
    const float cellsize = 2.0f * c.w;
    const bool leaf_by_size = cellsize - a.radius < kAbove1em8;
    int8_t type = T_LEAF;
    if (!leaf_by_size && signchange && nd_curv[node] < kAbove099) type = T_INTERNAL;
    nd_type[node] = type;
    nd_sc[node] = signchange ? 1 : 0;
    if (type == T_LEAF) {
      float4 v = nd_v[node];
      v.w = val[27];
      nd_v[node] = v;
    }
    evals = 27 + (type == T_LEAF ? 1 : 0);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) evals += __shfl_xor_sync(0xffffffffu, evals, o);
  if ((threadIdx.x & 31) == 0) stripe_add(counters, C_REF_EVALS, evals);
}

__global__ void k_internal_flag(const int8_t* __restrict__ nd_type, long long lb, long long le,
                                int* __restrict__ flag) {
  long long i = lb + (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= le) return;
  flag[i - lb] = nd_type[i] == T_INTERNAL ? 1 : 0;
}

__global__ void k_spawn(long long lb, long long le, long long cbase, const int* __restrict__ rank,
                        const int8_t* nd_type, int child_depth, float4* __restrict__ nd_c,
                        float4* __restrict__ nd_v, uint64_t* __restrict__ nd_id, int* __restrict__ nd_parent,
                        int* __restrict__ nd_child, int8_t* nd_ctype, int8_t* __restrict__ nd_depth,
                        int8_t* __restrict__ nd_sc, float* __restrict__ nd_curv, int4* __restrict__ nd_org) {
  long long i = lb + (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= le) return;
  if (nd_type[i] != T_INTERNAL) {
    nd_child[i] = -1;
    return;
  }
  const long long b = cbase + 8LL * rank[i - lb];
  nd_child[i] = (int)b;
  const float4 pc = nd_c[i];
  const float hc = pc.w / 2;
  const uint64_t pid = nd_id[i];
  const int4 po = nd_org[i];
  const int hs = po.w >> 1;
  for (int k = 0; k < 8; ++k) {
    const float sx = (k & 1) ? hc : -hc, sy = (k & 2) ? hc : -hc, sz = (k & 4) ? hc : -hc;
    float4 cc = make_float4(__fadd_rn(pc.x, sx), __fadd_rn(pc.y, sy), __fadd_rn(pc.z, sz), hc);
    nd_c[b + k] = cc;
    nd_v[b + k] = make_float4(cc.x, cc.y, cc.z, 0.f);
    nd_id[b + k] = pid * 8ull + (uint64_t)k;
    nd_parent[b + k] = (int)i;
    nd_child[b + k] = -1;
    nd_ctype[b + k] = T_UNCERTAIN;
    nd_depth[b + k] = (int8_t)child_depth;
    nd_sc[b + k] = 0;
    nd_curv[b + k] = 0.f;
    nd_org[b + k] = make_int4(po.x + ((k & 1) ? hs : 0), po.y + ((k & 2) ? hs : 0), po.z + ((k & 4) ? hs : 0), hs);
  }
}

// Spawns the 8 children of each INTERNAL node and settles their emptiness
// and curvature sums in one scan of the parent's grown box: every child's box
// grown by r * smooth_factor lies inside the parent's, and each particle is
// tested against the children's float bounds exactly as the child itself
// would compute them (checkEmptyAndCalcCurv, src/surface_reconstructor.cpp:
// 152-222).  One warp per parent; lane k writes child k.
template <bool CURV>
__global__ void __launch_bounds__(32 * kSpawnWarps, CURV ? 16 : 24) k_spawn_scan(LevelArgs a, long long cbase, const int* __restrict__ rank,
                                                    int child_depth, float4* __restrict__ nd_c,
                                                    float4* __restrict__ nd_v, uint64_t* __restrict__ nd_id,
                                                    int* __restrict__ nd_parent, int* __restrict__ nd_child,
                                                    int8_t* nd_type, int8_t* __restrict__ nd_depth,
                                                    int8_t* __restrict__ nd_sc, float* __restrict__ nd_curv,
                                                    int4* __restrict__ nd_org) {
  __shared__ int s_row[kSpawnWarps][32];  // row starting at each element position of a batch
  const long long i = a.lb + (long long)blockIdx.x * kSpawnWarps + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  int* const srow = s_row[threadIdx.x >> 5];
  if (i >= a.le) return;
  if (nd_type[i] != T_INTERNAL) {
    if (lane == 0) nd_child[i] = -1;
    return;
  }
  const long long b = cbase + 8LL * rank[i - a.lb];
  const float4 pc = nd_c[i];
  const float hc = pc.w / 2;
  const float e = a.expand;
  const float pcs[3] = {pc.x, pc.y, pc.z};
  float ctr[3][2], clo[3][2], chi[3][2];
#pragma unroll
  for (int ax = 0; ax < 3; ++ax)
#pragma unroll
    for (int bit = 0; bit < 2; ++bit) {
      const float c = __fadd_rn(pcs[ax], bit ? hc : -hc);
      ctr[ax][bit] = c;
      clo[ax][bit] = __fsub_rn(__fsub_rn(c, hc), e);
      chi[ax][bit] = __fadd_rn(__fadd_rn(c, hc), e);
    }
  // the parent's grown box is the union: low child's lo to high child's hi
  const int x0 = max(cell_coord(clo[0][0], a.g.b0, a.g.cell, a.g.nx), 0);
  const int y0 = max(cell_coord(clo[1][0], a.g.b2, a.g.cell, a.g.ny), 0);
  const int z0 = max(cell_coord(clo[2][0], a.g.b4, a.g.cell, a.g.nz), 0);
  const int x1 = min(cell_coord(chi[0][1], a.g.b0, a.g.cell, a.g.nx), a.g.nx - 1);
  const int y1 = min(cell_coord(chi[1][1], a.g.b2, a.g.cell, a.g.ny), a.g.ny - 1);
  const int z1 = min(cell_coord(chi[2][1], a.g.b4, a.g.cell, a.g.nz), a.g.nz - 1);
  unsigned found = 0;
  float sum[CURV ? 8 : 1][4];
#pragma unroll
  for (int k = 0; k < (CURV ? 8 : 1); ++k) sum[k][0] = sum[k][1] = sum[k][2] = sum[k][3] = 0.f;
  if (x0 <= x1 && y0 <= y1 && z0 <= z1) {
    const int nyb = y1 - y0 + 1;
    const int rows = (z1 - z0 + 1) * nyb;
    // rows of the block, 32 at a time: lane r holds row r's particle range;
    // the concatenated ranges are then walked 32 particles at a time
    for (int r0 = 0; r0 < rows; r0 += 32) {
      if (!CURV && __reduce_or_sync(0xffffffffu, found) == 0xffu) break;  // all eight children non-empty
      const int r = r0 + lane;
      int rs = 0, rl = 0;
      if (r < rows) {
        const int z = z0 + r / nyb, y = y0 + r % nyb;
        const long long base = ((long long)z * a.g.ny + y) * a.g.nx;
        rs = __ldg(a.g.off + base + x0);
        rl = __ldg(a.g.off + base + x1 + 1) - rs;
      }
      int incl = rl;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int v = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += v;
      }
      const int excl = incl - rl;
      const int total = __shfl_sync(0xffffffffu, incl, 31);
      int carry = 0;  // row of the batch's element before its first
      for (int t0 = 0; t0 < total; t0 += 32) {
        if (!CURV && t0 > 0 && __reduce_or_sync(0xffffffffu, found) == 0xffu) break;
        const int t = t0 + lane;
        // row of element t: the non-empty row starting at the last position
        // <= t of this batch, else the row carried over from the batch before
        // (non-empty rows start at distinct positions)
        const bool starts = rl > 0 && excl >= t0 && excl < t0 + 32;
        __syncwarp();
        if (starts) srow[excl - t0] = lane;
        const unsigned smask = __reduce_or_sync(0xffffffffu, starts ? 1u << (excl - t0) : 0u);
        __syncwarp();
        const unsigned below = smask & (0xffffffffu >> (31 - lane));
        const int rr = below ? srow[31 - __clz(below)] : carry;
        carry = __shfl_sync(0xffffffffu, rr, 31);
        const int j = __shfl_sync(0xffffffffu, rs, rr) + (t - __shfl_sync(0xffffffffu, excl, rr));
        if (t >= total) continue;
        const float4 p = __ldg(a.pos + j);
        const int mx = ((p.x > clo[0][0] && p.x < chi[0][0]) ? 1 : 0) | ((p.x > clo[0][1] && p.x < chi[0][1]) ? 2 : 0);
        const int my = ((p.y > clo[1][0] && p.y < chi[1][0]) ? 1 : 0) | ((p.y > clo[1][1] && p.y < chi[1][1]) ? 2 : 0);
        const int mz = ((p.z > clo[2][0] && p.z < chi[2][0]) ? 1 : 0) | ((p.z > clo[2][1] && p.z < chi[2][1]) ? 2 : 0);
        if (mx && my && mz && p.w == 0.f) {  // splash particles (pos.w = 1) do not count
          unsigned m8 = 0;
#pragma unroll
          for (int k = 0; k < 8; ++k)
            if (((mx >> (k & 1)) & 1) && ((my >> ((k >> 1) & 1)) & 1) && ((mz >> ((k >> 2) & 1)) & 1)) m8 |= 1u << k;
          found |= m8;
          if (CURV) {
            const float4 nv = __ldg(a.nrm + j);
#pragma unroll
            for (int k = 0; k < (CURV ? 8 : 1); ++k)
              if ((m8 >> k) & 1u) {
                sum[k][0] += nv.x;
                sum[k][1] += nv.y;
                sum[k][2] += nv.z;
                sum[k][3] += nv.w;
              }
          }
        }
      }
    }
  }
  found = __reduce_or_sync(0xffffffffu, found);
  float mine[4] = {0.f, 0.f, 0.f, 0.f};
  if (CURV) {
#pragma unroll
    for (int k = 0; k < (CURV ? 8 : 1); ++k)
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const float t = warp_sum(sum[k][q]);
        if (lane == k) mine[q] = t;
      }
  }
  if (lane == 0) nd_child[i] = (int)b;
  if (lane < 8) {
    const int k = lane;
    const int4 po = nd_org[i];
    const int hs = po.w >> 1;
    const float4 cc = make_float4(ctr[0][k & 1], ctr[1][(k >> 1) & 1], ctr[2][(k >> 2) & 1], hc);
    const bool nonempty = (found >> k) & 1u;
    nd_c[b + k] = cc;
    nd_v[b + k] = make_float4(cc.x, cc.y, cc.z, nonempty ? 0.f : a.iso);
    nd_id[b + k] = nd_id[i] * 8ull + (uint64_t)k;
    nd_parent[b + k] = (int)i;
    nd_child[b + k] = -1;
    nd_type[b + k] = nonempty ? T_UNCERTAIN : T_EMPTY;
    nd_depth[b + k] = (int8_t)child_depth;
    nd_sc[b + k] = 0;
    nd_curv[b + k] = !CURV ? -1.0f
                     : (mine[3] == 0.f) ? 1.0f
                                        : sqrtf(mine[0] * mine[0] + mine[1] * mine[1] + mine[2] * mine[2]) / mine[3];
    nd_org[b + k] = make_int4(po.x + ((k & 1) ? hs : 0), po.y + ((k & 2) ? hs : 0), po.z + ((k & 4) ? hs : 0), hs);
  }
}

// The coarse levels (depth < D_min - 1) in one cooperative launch: their
// nodes are INTERNAL exactly when their grown box holds a particle, so a
// level is an emptiness test per node, a scan of the INTERNAL flags and the
// spawn of 8 children per INTERNAL node, the same steps (and results) as
// k_empty, k_internal_flag, the scan and k_spawn, with grid-wide barriers
// in place of launches and of the host's read of each level's size.  The
// levels are small (at most kTopLevelNodes nodes; the loop stops before a
// larger one), so block 0 scans the flags alone.  Node data written in the
// launch is read through the L2 (ld.global.cg), never the read-only path.
constexpr int kTopLevelNodes = 4096;
constexpr int kTopThreads = 256;

struct TopArgs {
  LevelArgs la;  // grid, particles, expand, iso (lb / le / big set per level)
  int dstop;     // levels 0 .. dstop - 1 at most
  long long* lv;     // level starts: level d is [lv[d], lv[d + 1])
  int* flag;         // kTopLevelNodes + 1
  int* depth_out;    // levels done
  float4* nd_c;
  float4* nd_v;
  uint64_t* nd_id;
  int* nd_parent;
  int* nd_child;
  int8_t* nd_type;
  int8_t* nd_depth;
  int8_t* nd_sc;
  float* nd_curv;
  int4* nd_org;
};

__global__ void __launch_bounds__(kTopThreads) k_top_levels(TopArgs t) {
  namespace cg = cooperative_groups;
  cg::grid_group grid = cg::this_grid();
  __shared__ int s_warp[kTopThreads / 32];
  __shared__ int s_carry;
  const int lane = threadIdx.x & 31;
  const long long gwarp = ((long long)blockIdx.x * kTopThreads + threadIdx.x) >> 5;
  const long long nwarps = (long long)gridDim.x * kTopThreads / 32;
  const long long gthread = (long long)blockIdx.x * kTopThreads + threadIdx.x;
  const long long nthreads = (long long)gridDim.x * kTopThreads;
  int depth = 0;
  for (;;) {
    const long long lb = __ldcg(t.lv + depth), le = __ldcg(t.lv + depth + 1);
    const long long n = le - lb;
    LevelArgs a = t.la;
    // emptiness: one warp per node (k_empty's test), INTERNAL if non-empty
    for (long long w = gwarp; w < n; w += nwarps) {
      const long long node = lb + w;
      const GrownBox b = grown_box(a.g, __ldcg(t.nd_c + node), a.expand);
      bool found = false;
      if (b.x0 <= b.x1 && b.y0 <= b.y1 && b.z0 <= b.z1) {
        const int nyb = b.y1 - b.y0 + 1;
        const int rows = (b.z1 - b.z0 + 1) * nyb;
        for (int r0 = 0; r0 < rows && !found; r0 += 32) {
          const int r = r0 + lane;
          bool hit = false;
          if (r < rows) {
            const int z = b.z0 + r / nyb, y = b.y0 + r % nyb;
            const long long base = ((long long)z * a.g.ny + y) * a.g.nx;
            const int s = __ldg(a.g.off + base + b.x0), e = __ldg(a.g.off + base + b.x1 + 1);
            for (int j = s; j < e; ++j)
              if (inside(b, __ldg(a.pos + j))) {
                hit = true;
                break;
              }
          }
          found = __any_sync(0xffffffffu, hit);
        }
      }
      if (lane == 0) {
        if (!found) {
          t.nd_type[node] = T_EMPTY;
          t.nd_curv[node] = 1.0f;  // area == 0
          float4 v = __ldcg(t.nd_v + node);
          v.w = a.iso;
          t.nd_v[node] = v;
        } else {
          t.nd_type[node] = T_INTERNAL;
          t.nd_curv[node] = -1.0f;
        }
        t.flag[w] = found ? 1 : 0;
      }
    }
    grid.sync();
    // exclusive scan of the flags by block 0; the next level's end
    if (blockIdx.x == 0) {
      if (threadIdx.x == 0) s_carry = 0;
      __syncthreads();
      for (long long b0 = 0; b0 < n; b0 += kTopThreads) {
        const long long i = b0 + threadIdx.x;
        const int v = i < n ? __ldcg(t.flag + i) : 0;
        int inc = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const int u = __shfl_up_sync(0xffffffffu, inc, o);
          if (lane >= o) inc += u;
        }
        if (lane == 31) s_warp[threadIdx.x >> 5] = inc;
        __syncthreads();
        int wbase = 0, total = 0;
        for (int k = 0; k < kTopThreads / 32; ++k) {
          if (k < (int)(threadIdx.x >> 5)) wbase += s_warp[k];
          total += s_warp[k];
        }
        if (i < n) t.flag[i] = s_carry + wbase + inc - v;
        __syncthreads();
        if (threadIdx.x == 0) s_carry += total;
        __syncthreads();
      }
      if (threadIdx.x == 0) t.lv[depth + 2] = le + 8LL * s_carry;
    }
    grid.sync();
    // spawn (k_spawn): children of the INTERNAL nodes from the level's end on
    for (long long w = gthread; w < n; w += nthreads) {
      const long long i = lb + w;
      if (__ldcg(t.nd_type + i) != T_INTERNAL) {
        t.nd_child[i] = -1;
        continue;
      }
      const long long b = le + 8LL * __ldcg(t.flag + w);
      t.nd_child[i] = (int)b;
      const float4 pc = __ldcg(t.nd_c + i);
      const float hc = pc.w / 2;
      const uint64_t pid = __ldcg(reinterpret_cast<const unsigned long long*>(t.nd_id) + i);
      const int4 po = __ldcg(t.nd_org + i);
      const int hs = po.w >> 1;
      for (int k = 0; k < 8; ++k) {
        const float sx = (k & 1) ? hc : -hc, sy = (k & 2) ? hc : -hc, sz = (k & 4) ? hc : -hc;
        const float4 cc = make_float4(__fadd_rn(pc.x, sx), __fadd_rn(pc.y, sy), __fadd_rn(pc.z, sz), hc);
        t.nd_c[b + k] = cc;
        t.nd_v[b + k] = make_float4(cc.x, cc.y, cc.z, 0.f);
        t.nd_id[b + k] = pid * 8ull + (uint64_t)k;
        t.nd_parent[b + k] = (int)i;
        t.nd_child[b + k] = -1;
        t.nd_type[b + k] = T_UNCERTAIN;
        t.nd_depth[b + k] = (int8_t)(depth + 1);
        t.nd_sc[b + k] = 0;
        t.nd_curv[b + k] = 0.f;
        t.nd_org[b + k] =
            make_int4(po.x + ((k & 1) ? hs : 0), po.y + ((k & 2) ? hs : 0), po.z + ((k & 4) ? hs : 0), hs);
      }
    }
    const long long next = __ldcg(t.lv + depth + 2) - le;  // written before the last barrier
    ++depth;
    if (next == 0 || depth >= t.dstop || next > kTopLevelNodes) break;  // the same for every thread
    grid.sync();
  }
  if (gthread == 0) *t.depth_out = depth;
}

int top_levels_grid(int device, int sm_count) {
  int coop = 0;
  if (cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, device) != cudaSuccess || !coop) {
    (void)cudaGetLastError();
    return 0;
  }
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_top_levels, kTopThreads, 0) != cudaSuccess ||
      per_sm < 1) {
    (void)cudaGetLastError();
    return 0;
  }
  // the coarse levels hold at most a few thousand nodes: half the SMs, one
  // block each, leave room for other contexts' kernels
  return std::max(1, std::min(per_sm * sm_count, sm_count / 2));
}

__global__ void k_root(float cx, float cy, float cz, float h, int size, float4* nd_c, float4* nd_v,
                       uint64_t* nd_id, int* nd_parent, int* nd_child, int8_t* nd_type, int8_t* nd_depth,
                       int8_t* nd_sc, float* nd_curv, int4* nd_org) {
  nd_c[0] = make_float4(cx, cy, cz, h);
  nd_v[0] = make_float4(cx, cy, cz, 0.f);
  nd_id[0] = 0;
  nd_parent[0] = -1;
  nd_child[0] = -1;
  nd_type[0] = T_UNCERTAIN;
  nd_depth[0] = 0;
  nd_sc[0] = 0;
  nd_curv[0] = 0.f;
  nd_org[0] = make_int4(0, 0, 0, size);
}

template <int K, int W, int CB, bool BULK>
static void launch_eval(pi_frame* f, int cfg, const QArgs& qa, long long qn, const int* order, const int* qoff,
                        const int* ucnt, const int2* chunks, const int* nchunks, const int* cbeg, int reserve,
                        float* qval, unsigned long long* counters) {
  pi_ctx* ctx = f->ctx;
  static thread_local int occ[64][kEvalConfigs] = {};
  static thread_local int regs[64][kEvalConfigs] = {};
  const int dev = ctx->device & 63;
  if (occ[dev][cfg] == 0) {
    int nb = 0;
    PI_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_q_eval<K, W, CB, BULK>, 32 * W, 0));
    cudaFuncAttributes fa;
    PI_CUDA(cudaFuncGetAttributes(&fa, k_q_eval<K, W, CB, BULK>));
    occ[dev][cfg] = nb > 0 ? nb : 1;
    regs[dev][cfg] = ((fa.numRegs + 7) / 8) * 8 * 32 * W;  // allocated per block: 8-register steps per thread
  }
  // reserve: registers per SM left to the QEF stream's kernel
  int per_sm = occ[dev][cfg];
  if (reserve > 0) per_sm = std::max(1, std::min(per_sm, (65536 - reserve) / regs[dev][cfg]));
  const int blocks = (int)std::min<long long>((long long)ctx->smCount * per_sm, div_up(qn, 32 * W));
  PI_LAUNCH((k_q_eval<K, W, CB, BULK>), blocks, 32 * W, 0, ctx->stream, qa, order, qoff, ucnt, chunks, nchunks,
            cbeg, f->nd_c.p, f->nd_v.p, qval, counters);
}

// The chunked evaluator's configurations: samples per lane K, warps per
// block W, staged candidates per warp CB, bulk (TMA) staging.  Index 1
// (K 2, W 8, CB 96, filter then cp.async) is the default; every
// configuration gives the same values (each sample's sum runs over the same
// candidates in the same order).
const EvalConfig kEvalTable[kEvalConfigs] = {{1, 8, 96, 0}, {2, 8, 96, 0}, {4, 8, 96, 0}, {2, 4, 96, 0},
                                             {4, 4, 96, 0}, {2, 8, 64, 0}, {4, 8, 64, 0}, {2, 16, 48, 0},
                                             {2, 4, 96, 1}, {4, 4, 96, 1}};

// Chunk list for configuration cfg, then the chunked evaluation.
static void eval_chunks(pi_frame* f, int cfg, const QArgs& qa, long long qn, const int* order, const int* qoff,
                        const int* ucnt, const int2* chunks, const int* nchunks, const int* cbeg, int reserve,
                        float* qval, unsigned long long* counters) {
#define PI_EVAL_CASE(i, k, w, cb, bulk) \
  case i:                               \
    launch_eval<k, w, cb, bulk>(f, i, qa, qn, order, qoff, ucnt, chunks, nchunks, cbeg, reserve, qval, counters); \
    break;
  switch (cfg) {
    PI_EVAL_CASE(0, 1, 8, 96, false)
    PI_EVAL_CASE(1, 2, 8, 96, false)
    PI_EVAL_CASE(2, 4, 8, 96, false)
    PI_EVAL_CASE(3, 2, 4, 96, false)
    PI_EVAL_CASE(4, 4, 4, 96, false)
    PI_EVAL_CASE(5, 2, 8, 64, false)
    PI_EVAL_CASE(6, 4, 8, 64, false)
    PI_EVAL_CASE(7, 2, 16, 48, false)
    PI_EVAL_CASE(8, 2, 4, 96, true)
    PI_EVAL_CASE(9, 4, 4, 96, true)
    default:
      throw std::logic_error("unknown evaluation configuration");
  }
#undef PI_EVAL_CASE
}

static void dense_eval(pi_frame* f, int cfg, const QArgs& qa, long long qn, long long nbuckets, const int* order,
                       const int* qoff, const int* ucnt, int2* chunks, int* nchunks, float* qval,
                       unsigned long long* counters) {
  cudaStream_t s = f->ctx->stream;
  const int K = kEvalTable[cfg].K;
  PI_CUDA(cudaMemsetAsync(nchunks, 0, sizeof(int), s));
  PI_LAUNCH(k_q_chunks, div_up(nbuckets, 256), 256, 0, s, nbuckets, ucnt, 32 * K, chunks, nchunks);
  eval_chunks(f, cfg, qa, qn, order, qoff, ucnt, chunks, nchunks, nullptr, 0, qval, counters);
}

// Configuration for a dense level of the given kind: the context's choice,
// or, the first time, the fastest of the table timed on this level (the
// evaluation is pure, so the runs give identical values).  A context whose K
// is fixed (pi_ctx_tune) runs that K with the default W and CB.
static int eval_config_for(pi_frame* f, int kind, const QArgs& qa, long long qn, long long nbuckets,
                           const int* order, const int* qoff, const int* ucnt, int2* chunks, int* nchunks,
                           float* qval) {
  pi_ctx* ctx = f->ctx;
  if (ctx->eval_forced) return ctx->eval_forced == 1 ? 0 : ctx->eval_forced == 2 ? 1 : 2;
  if (ctx->eval_cfg[kind]) return ctx->eval_cfg[kind] - 1;
  qef_join(f);  // time the trials without the QEF stream beside them
  cudaStream_t s = ctx->stream;
  cudaEvent_t e0, e1;
  PI_CUDA(cudaEventCreate(&e0));
  PI_CUDA(cudaEventCreate(&e1));
  float best = 1e30f;
  int bestc = 1;
  DBuf<unsigned long long> scratch;  // the trial runs' event counters are not the frame's
  scratch.alloc(ctx, s, kCounterWords);
  for (int c = 0; c < kEvalConfigs; ++c) {
    PI_CUDA(cudaEventRecord(e0, s));
    dense_eval(f, c, qa, qn, nbuckets, order, qoff, ucnt, chunks, nchunks, qval, scratch.p);
    PI_CUDA(cudaEventRecord(e1, s));
    PI_CUDA(cudaEventSynchronize(e1));
    float ms = 0.f;
    PI_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    if (ms < best) {
      best = ms;
      bestc = c;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  ctx->eval_cfg[kind] = bestc + 1;
  return bestc;
}

static void ensure_nodes(pi_frame* f, long long need) {
  // the QEF samples exist only in QEF mode, so a frame that switches it on
  // (pi_reconstruct reuses its frame across parameters) may hold node arrays
  // large enough and no samples yet
  const bool samp_ok = !f->P.qef || (long long)f->nd_samp.n >= need * 27;
  const bool minr_ok = !f->varR || (long long)f->nd_minr.n >= need;
  if ((long long)f->nd_c.n >= need && samp_ok && minr_ok) return;
  qef_join(f);  // the QEF in flight writes node arrays that are about to move
  long long cap = std::max<long long>(need, (long long)(f->nd_c.n * 3 / 2) + 1024);
  pi_ctx* c = f->ctx;
  cudaStream_t s = c->stream;
  long long keep = f->nNodes;
  f->nd_c.grow(c, s, cap, keep);
  f->nd_v.grow(c, s, cap, keep);
  f->nd_id.grow(c, s, cap, keep);
  f->nd_parent.grow(c, s, cap, keep);
  f->nd_child.grow(c, s, cap, keep);
  f->nd_type.grow(c, s, cap, keep);
  f->nd_depth.grow(c, s, cap, keep);
  f->nd_sc.grow(c, s, cap, keep);
  f->nd_curv.grow(c, s, cap, keep);
  f->nd_org.grow(c, s, cap, keep);
  if (f->P.qef) f->nd_samp.grow(c, s, cap * 27, keep * 27);
  if (f->varR) f->nd_minr.grow(c, s, cap, keep);
}

// ---------------------------------------------------------------------------
// Variable radius.  checkEmptyAndCalcCurv with per-particle radii
// (src/surface_reconstructor.cpp:152-222): a particle reaches a node when it
// lies strictly inside the node box grown by its own radius * smooth_factor;
// the node is empty when none does, else its curvature sums run over those
// particles and min_radius is their smallest radius, which makes the node a
// leaf by size when cellsize - min_radius < 1e-8 (:247).  One warp per node
// over the cells of every bin's grid that the box grown by the largest
// radius touches (the reference's GetInBoxParticles, box +- 1 cell, is a
// superset of these).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(64) k_vr_empty(const MultiGridView* __restrict__ mg, LevelArgs a,
                                                 float emax, const float4* __restrict__ nd_c,
                                                 float4* __restrict__ nd_v, int8_t* __restrict__ nd_type,
                                                 float* __restrict__ nd_curv, float* __restrict__ nd_minr) {
  const long long node = a.lb + (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (node >= a.le) return;
  const MultiGridView& m = *mg;
  const float4 c = nd_c[node];
  const float h = c.w;
  const float b1x = __fsub_rn(c.x, h), b1y = __fsub_rn(c.y, h), b1z = __fsub_rn(c.z, h);
  const float b2x = __fadd_rn(c.x, h), b2y = __fadd_rn(c.y, h), b2z = __fadd_rn(c.z, h);
  bool found = false;
  float minr = 3.402823466e38f;
  Kahan sx, sy, sz, ar;
  for (int b = 0; b < m.nb; ++b) {
    const BinGrid g = m.g[b];
    const int x0 = max(cell_coord(__fsub_rn(b1x, emax), g.b0, g.cell, g.nx), 0);
    const int y0 = max(cell_coord(__fsub_rn(b1y, emax), g.b2, g.cell, g.ny), 0);
    const int z0 = max(cell_coord(__fsub_rn(b1z, emax), g.b4, g.cell, g.nz), 0);
    const int x1 = min(cell_coord(__fadd_rn(b2x, emax), g.b0, g.cell, g.nx), g.nx - 1);
    const int y1 = min(cell_coord(__fadd_rn(b2y, emax), g.b2, g.cell, g.ny), g.ny - 1);
    const int z1 = min(cell_coord(__fadd_rn(b2z, emax), g.b4, g.cell, g.nz), g.nz - 1);
    if (x0 > x1 || y0 > y1 || z0 > z1) continue;
    const int nyb = y1 - y0 + 1;
    const int rows = (z1 - z0 + 1) * nyb;
    for (int r = lane; r < rows; r += 32) {
      const int z = z0 + r / nyb, y = y0 + r % nyb;
      const long long base = (long long)g.offBase + ((long long)z * g.ny + y) * g.nx;
      const int s = __ldg(m.off + base + x0), e = __ldg(m.off + base + x1 + 1);
      for (int j = s; j < e; ++j) {
        const float4 p = __ldg(a.pos + j);
        const float ej = p.w * a.expand;  // r_j * smooth_factor
        if (p.x > __fsub_rn(b1x, ej) && p.x < __fadd_rn(b2x, ej) && p.y > __fsub_rn(b1y, ej) &&
            p.y < __fadd_rn(b2y, ej) && p.z > __fsub_rn(b1z, ej) && p.z < __fadd_rn(b2z, ej)) {
          found = true;
          minr = fminf(minr, p.w);
          const float4 nv = __ldg(a.nrm + j);
          sx.add(nv.x);
          sy.add(nv.y);
          sz.add(nv.z);
          ar.add(nv.w);
        }
      }
    }
  }
  found = __any_sync(0xffffffffu, found);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) minr = fminf(minr, __shfl_xor_sync(0xffffffffu, minr, o));
  const float nx = warp_sum(sx.s - sx.c), ny = warp_sum(sy.s - sy.c), nz = warp_sum(sz.s - sz.c);
  const float area = warp_sum(ar.s - ar.c);
  if (lane == 0) {
    if (!found) {
      nd_type[node] = T_EMPTY;
      nd_curv[node] = 1.0f;
      float4 v = nd_v[node];
      v.w = a.iso;
      nd_v[node] = v;
    } else {
      // above D_min a node is INTERNAL unless it is a leaf by size already
      // (every particle reaching it is at least its size; afterSampleEval
      // tests the size first, :247): then it waits for its value
      const bool leaf_by_size = 2.0f * h - minr < kAbove1em8;
      nd_type[node] = (a.big && !leaf_by_size) ? T_INTERNAL : T_UNCERTAIN;
      nd_curv[node] = (area == 0.f) ? 1.0f : sqrtf(nx * nx + ny * ny + nz * nz) / area;
      nd_minr[node] = minr;
    }
  }
}

// Leaves by size above D_min (variable radius only): no GridEval there, the
// value is SingleEval at the node position (src/surface_reconstructor.cpp:
// 245-253).
__global__ void k_vr_big_leaf(const MultiGridView* __restrict__ mg, LevelArgs a, float4* __restrict__ nd_v,
                              int8_t* __restrict__ nd_type, unsigned long long* __restrict__ counters) {
  const long long node = a.lb + (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (node >= a.le || nd_type[node] != T_UNCERTAIN) return;
  float4 v = nd_v[node];
  v.w = a.iso - field_sum_vr(*mg, a.P, v.x, v.y, v.z, nullptr);
  nd_v[node] = v;
  nd_type[node] = T_LEAF;
  stripe_add(counters, C_REF_EVALS, 1ull);
  stripe_add(counters, C_DONE_THREAD, 1ull);
}

// Field at the distinct samples of a level, one thread per sample in bucket
// order, over the bins' candidate lists.
__global__ void __launch_bounds__(256, 4) k_vr_q_eval_thread(const MultiGridView* __restrict__ mg, QArgs a,
                                                             const int* __restrict__ list,
                                                             const int* __restrict__ count_ptr,
                                                             const float4* __restrict__ nd_c,
                                                             const float4* __restrict__ nd_v, float* __restrict__ qval,
                                                             unsigned long long* __restrict__ counters) {
  const int n = *count_ptr;
  long long pairs = 0, done = 0;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    const int q = list[t];
    const long long node = a.lb + q / kQ;
    float qx, qy, qz;
    sample_point(nd_c[node], nd_v[node], q % kQ, qx, qy, qz);
    qval[q] = a.iso - field_sum_vr(*mg, a.P, qx, qy, qz, &pairs);
    ++done;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    pairs += __shfl_xor_sync(0xffffffffu, pairs, o);
    done += __shfl_xor_sync(0xffffffffu, done, o);
  }
  if ((threadIdx.x & 31) == 0) {
    stripe_add(counters, C_SAMPLE_PAIRS, (unsigned long long)pairs);
    stripe_add(counters, C_PAIRS_THREAD, (unsigned long long)pairs);
    stripe_add(counters, C_DONE_THREAD, (unsigned long long)done);
  }
}

// genIsoOurs state 0 with per-particle radii: every level runs the
// emptiness scan above, then (depth >= D_min) the sampling, one thread per
// distinct sample, and the classification with each node's min_radius.
static void stage_octree_vr(pi_frame* f) {
  pi_ctx* ctx = f->ctx;
  cudaStream_t s = ctx->stream;
  f->nNodes = 0;
  f->levelBegin.clear();
  ensure_nodes(f, 1 << 16);
  if (!f->ev[kLevelEvent]) PI_CUDA(cudaEventCreateWithFlags(&f->ev[kLevelEvent], cudaEventDisableTiming));
  PI_LAUNCH(k_root, 1, 1, 0, s, f->rootC[0], f->rootC[1], f->rootC[2], f->rootH, 1 << f->dmax, f->nd_c.p,
            f->nd_v.p, f->nd_id.p, f->nd_parent.p, f->nd_child.p, f->nd_type.p, f->nd_depth.p, f->nd_sc.p,
            f->nd_curv.p, f->nd_org.p);
  f->nNodes = 1;
  // sample buckets: a grid of cells 4 * maxR over the root box (it holds
  // every sample), whole cells
  const float bcell = f->vrMaxR * 4.0f;
  const int bn = std::max(1, (int)std::ceil(2.0f * f->rootH / bcell));
  GridView bg{f->rootC[0] - f->rootH, f->rootC[1] - f->rootH, f->rootC[2] - f->rootH, bcell, bn, bn, bn, nullptr};
  PartView P{f->pos.p, f->xm.p, f->ga.p, f->gb.p, f->xlo.p};
  const int ekx = bn + 4, eky = bn + 4;
  const long long nb = (long long)ekx * eky * (bn + 4);
  counters_reset(f);
  DBuf<int> flag, qcnt, qkey, rep, order, ucnt, ucum;
  DBuf<unsigned> hslot;
  DBuf<float> qval;
  qcnt.alloc(ctx, s, nb + 2);
  ucnt.alloc(ctx, s, nb + 1);
  ucum.alloc(ctx, s, nb + 1);
  long long lb = 0, le = 1;
  for (int depth = 0; le > lb; ++depth) {
    f->levelBegin.push_back(lb);
    const long long nl = le - lb;
    LevelArgs la{bg, f->pos.p, f->nrm.p, f->P.smooth_factor, f->iso, f->vrMinR, lb, le, depth < f->dmin ? 1 : 0, P};
    PI_LAUNCH(k_vr_empty, div_up(nl, 2), 64, 0, s, f->mgv.p, la, f->vrMaxR * f->P.smooth_factor, f->nd_c.p,
              f->nd_v.p, f->nd_type.p, f->nd_curv.p, f->nd_minr.p);
    if (depth < f->dmin)
      PI_LAUNCH(k_vr_big_leaf, div_up(nl, 128), 128, 0, s, f->mgv.p, la, f->nd_v.p, f->nd_type.p, f->dcount.p);
    if (depth >= f->dmin) {
      const long long qn = nl * kQ;
      if (f->tmp.n < scan_tmp_ints(nb + 1)) f->tmp.alloc(ctx, s, scan_tmp_ints(nb + 1));
      qkey.alloc(ctx, s, qn);
      rep.alloc(ctx, s, qn);
      hslot.alloc(ctx, s, 2 * qn);
      qval.alloc(ctx, s, qn);
      order.alloc(ctx, s, qn);
      PI_CUDA(cudaMemsetAsync(qcnt.p, 0, sizeof(int) * (nb + 2), s));
      PI_CUDA(cudaMemsetAsync(ucnt.p, 0, sizeof(int) * (nb + 1), s));
      PI_CUDA(cudaMemsetAsync(hslot.p, 0, sizeof(unsigned) * 2 * qn, s));
      QArgs qa{bg, P, f->iso, lb, le, ekx, eky, 0};
      PI_LAUNCH(k_q_count_node, div_up(nl, kCountThreads), kCountThreads, 0, s, qa, f->nd_c.p, f->nd_v.p,
                f->nd_type.p, qcnt.p, qkey.p);
      exclusive_scan_i32(qcnt.p, qcnt.p, nb + 1, nullptr, f->tmp.p, s);
      PI_LAUNCH(k_q_dedupe, div_up(qn, 256), 256, 0, s, qa, qn, f->nd_c.p, f->nd_v.p, qkey.p, qcnt.p, hslot.p,
                ucnt.p, rep.p, order.p);
      int* list = reinterpret_cast<int*>(hslot.p);
      exclusive_scan_i32(ucnt.p, ucum.p, nb + 1, nullptr, f->tmp.p, s);
      PI_LAUNCH(k_q_compact, div_up(nb, 256), 256, 0, s, nb, qcnt.p, ucnt.p, ucum.p, order.p, list);
      prof_begin(ctx, s, PG_THREAD);
      PI_LAUNCH(k_vr_q_eval_thread, (int)std::min<long long>((long long)ctx->smCount * 8, div_up(qn, 256)), 256, 0,
                s, f->mgv.p, qa, list, ucum.p + nb, f->nd_c.p, f->nd_v.p, qval.p, f->dcount.p);
      prof_end(ctx, s, PG_THREAD);
      const int wpb = 2;
      PI_LAUNCH(k_classify, div_up(nl, wpb), 32 * wpb, 0, s, la, qval.p, rep.p, f->nd_c.p, f->nd_v.p, f->nd_type.p,
                f->nd_sc.p, f->nd_curv.p, f->nd_samp.p, 0, 1, f->dcount.p, (const float*)f->nd_minr.p);
    }
    flag.alloc(ctx, s, nl + 1);
    if (f->tmp.n < scan_tmp_ints(nl + 1)) f->tmp.alloc(ctx, s, scan_tmp_ints(nl + 1));
    PI_LAUNCH(k_internal_flag, div_up(nl, 256), 256, 0, s, f->nd_type.p, lb, le, flag.p);
    PI_CUDA(cudaMemsetAsync(flag.p + nl, 0, sizeof(int), s));
    exclusive_scan_i32(flag.p, flag.p, nl + 1, nullptr, f->tmp.p, s);
    int* const nint_h = reinterpret_cast<int*>(ctx->hpin + kPinSlots * kCounterWords + 1);
    PI_CUDA(cudaMemcpyAsync(nint_h, flag.p + nl, sizeof(int), cudaMemcpyDeviceToHost, s));
    PI_CUDA(cudaEventRecord(f->ev[kLevelEvent], s));
    f->nNodes = le;
    ensure_nodes(f, le + 8 * nl);
    PI_LAUNCH(k_spawn, div_up(nl, 256), 256, 0, s, lb, le, le, flag.p, f->nd_type.p, depth + 1, f->nd_c.p, f->nd_v.p,
              f->nd_id.p, f->nd_parent.p, f->nd_child.p, f->nd_type.p, f->nd_depth.p, f->nd_sc.p, f->nd_curv.p,
              f->nd_org.p);
    PI_CUDA(cudaEventSynchronize(f->ev[kLevelEvent]));
    const int nint = *nint_h;
    const long long newn = 8LL * nint;
    f->nNodes = le + newn;
    if (nint == 0 || depth >= f->dmax) break;
    lb = le;
    le = le + newn;
  }
  counters_snapshot(f, kPinOctree);
}

void stage_octree(pi_frame* f) {
  pi_ctx* ctx = f->ctx;
  cudaStream_t s = ctx->stream;
  if (f->dmax > 20) throw std::length_error("octree depth above 20");
  if (f->varR) {
    stage_octree_vr(f);
    return;
  }
  f->nNodes = 0;
  f->levelBegin.clear();
  ensure_nodes(f, 1 << 16);
  if (!f->ev[kLevelEvent]) PI_CUDA(cudaEventCreateWithFlags(&f->ev[kLevelEvent], cudaEventDisableTiming));
  PI_LAUNCH(k_root, 1, 1, 0, s, f->rootC[0], f->rootC[1], f->rootC[2], f->rootH, 1 << f->dmax, f->nd_c.p,
            f->nd_v.p, f->nd_id.p, f->nd_parent.p, f->nd_child.p, f->nd_type.p, f->nd_depth.p, f->nd_sc.p,
            f->nd_curv.p, f->nd_org.p);
  f->nNodes = 1;
  const GridHost& gh = f->g;
  GridView g{gh.bounding[0], gh.bounding[2], gh.bounding[4], gh.cell, gh.nx, gh.ny, gh.nz, f->off.p};
  PartView P{f->pos.p, f->xm.p, f->ga.p, f->gb.p, f->xlo.p};
  const int ekx = gh.nx + 4, eky = gh.ny + 4;
  const long long ek = (long long)ekx * eky * (gh.nz + 4) * 8;  // buckets: cell x octant
  counters_reset(f);
  DBuf<int> flag, qcnt, qkey, rep, order, ucnt, ucum;
  DBuf<unsigned> hslot;
  DBuf<int2> chunks;
  DBuf<float> qval;
  qcnt.alloc(ctx, s, ek + 2);  // bucket counts, total, chunk count
  ucnt.alloc(ctx, s, ek + 1);  // distinct points per bucket (+ 1 for the scan's total)
  ucum.alloc(ctx, s, ek + 1);  // exclusive scan of ucnt (sparse levels)
  long long lb = 0, le = 1;
  bool known = false;  // emptiness and curvature of this level settled by the parents' scan
  int depth0 = 0;
  if (f->dmin >= 2 && ctx->coop_blocks > 0) {
    // the coarse levels 0 .. D_min - 2 in one cooperative launch
    const int dstop = f->dmin - 1;
    DBuf<long long> lvd;
    DBuf<int> tflag, dout;
    lvd.alloc(ctx, s, dstop + 3);
    tflag.alloc(ctx, s, kTopLevelNodes + 1);
    dout.alloc(ctx, s, 1);
    long long* const lvh = reinterpret_cast<long long*>(ctx->hpin + kPinTopOffset);
    lvh[0] = 0;
    lvh[1] = 1;
    PI_CUDA(cudaMemcpyAsync(lvd.p, lvh, 2 * sizeof(long long), cudaMemcpyHostToDevice, s));
    TopArgs ta{LevelArgs{g, f->pos.p, f->nrm.p, f->P.radius * f->P.smooth_factor, f->iso, f->P.radius, 0, 0, 1, P},
               dstop,
               lvd.p,
               tflag.p,
               dout.p,
               f->nd_c.p,
               f->nd_v.p,
               f->nd_id.p,
               f->nd_parent.p,
               f->nd_child.p,
               f->nd_type.p,
               f->nd_depth.p,
               f->nd_sc.p,
               f->nd_curv.p,
               f->nd_org.p};
    void* args[] = {&ta};
    PI_CUDA(cudaLaunchCooperativeKernel((const void*)k_top_levels, dim3(ctx->coop_blocks), dim3(kTopThreads), args,
                                        0, s));
    count_launch();
    int* const dh = reinterpret_cast<int*>(lvh + kPinTopWords - 1);
    PI_CUDA(cudaMemcpyAsync(lvh, lvd.p, sizeof(long long) * (dstop + 2), cudaMemcpyDeviceToHost, s));
    PI_CUDA(cudaMemcpyAsync(dh, dout.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    PI_CUDA(cudaStreamSynchronize(s));
    depth0 = *dh;
    for (int d = 0; d < depth0; ++d) f->levelBegin.push_back(lvh[d]);
    lb = lvh[depth0];
    le = lvh[depth0 + 1];
    f->nNodes = le;
  }
  for (int depth = depth0; le > lb; ++depth) {
    f->levelBegin.push_back(lb);
    const long long nl = le - lb;
    LevelArgs la{g, f->pos.p, f->nrm.p, f->P.radius * f->P.smooth_factor, f->iso, f->P.radius, lb, le,
                 depth < f->dmin ? 1 : 0, P};
    // every node of the level has half size rootH / 2^depth (children halve exactly)
    const float cell_d = 2.0f * std::ldexp(f->rootH, -depth);
    const bool leaf_level = (double)(cell_d - f->P.radius) < 1e-8;
    // every non-empty node of a sampled leaf-by-size level becomes a leaf
    // (afterSampleEval returns before any INTERNAL test), so the tree is
    // final now: nothing spawns below this level.  Without the QEF the
    // extraction's topology, which reads only the tree, starts beside the
    // level's field values when the extraction follows; with the QEF it is
    // better left to run beside the last part's QEF at the extraction's start
    const bool last = depth >= f->dmin && leaf_level;
    const bool topo_early = last && f->extract_follows && !f->P.qef;
    if (topo_early) PI_CUDA(cudaEventRecord(ctx->ev_topo_in, s));
    const int wpb = 2;  // warps per block of the warp-per-node kernels (small blocks: uneven warps free their SM slots sooner)
    if (!known)
      PI_LAUNCH(k_empty, div_up(nl, wpb), 32 * wpb, 0, s, la, f->nd_c.p, f->nd_v.p, f->nd_type.p, f->nd_curv.p);
    if (depth >= f->dmin && leaf_level && !f->P.qef) {
      prof_begin(ctx, s, PG_LEAF);
      PI_LAUNCH(k_leaf_level, (int)std::min<long long>((long long)ctx->smCount * 8, div_up(nl, 256)), 256, 0, s, la,
                f->nd_c.p, f->nd_v.p, f->nd_type.p, f->dcount.p);
      prof_end(ctx, s, PG_LEAF);
    } else if (depth >= f->dmin) {
      const long long qn = nl * kQ;
      // buckets: cell octants on the leaf level, whole cells above it
      const int octants = depth == f->dmax ? 1 : 0;
      const long long nb = octants ? ek : ek / 8;
      if (f->tmp.n < scan_tmp_ints(nb + 1)) f->tmp.alloc(ctx, s, scan_tmp_ints(nb + 1));
      qkey.alloc(ctx, s, qn);
      rep.alloc(ctx, s, qn);
      hslot.alloc(ctx, s, 2 * qn);
      qval.alloc(ctx, s, qn);
      order.alloc(ctx, s, qn);
      chunks.alloc(ctx, s, qn);
      PI_CUDA(cudaMemsetAsync(qcnt.p, 0, sizeof(int) * (nb + 2), s));
      PI_CUDA(cudaMemsetAsync(ucnt.p, 0, sizeof(int) * (nb + 1), s));
      PI_CUDA(cudaMemsetAsync(hslot.p, 0, sizeof(unsigned) * 2 * qn, s));
      // the leaf level (node size r, samples r/2 apart) holds about 50
      // distinct samples per cell octant, the level above about 50 per cell;
      // coarser levels hold a few per cell
      const int dense = depth >= f->dmax - 1 ? 1 : 0;
      QArgs qa{g, P, f->iso, lb, le, ekx, eky, octants};
      PI_LAUNCH(k_q_count_node, div_up(nl, kCountThreads), kCountThreads, 0, s, qa, f->nd_c.p, f->nd_v.p,
                f->nd_type.p, qcnt.p, qkey.p);
      exclusive_scan_i32(qcnt.p, qcnt.p, nb + 1, nullptr, f->tmp.p, s);
      PI_LAUNCH(k_q_dedupe, div_up(qn, 256), 256, 0, s, qa, qn, f->nd_c.p, f->nd_v.p, qkey.p, qcnt.p, hslot.p,
                ucnt.p, rep.p, order.p);
      int* list = reinterpret_cast<int*>(hslot.p);  // the hash slots are free once the samples are placed
      if (!dense) {
        exclusive_scan_i32(ucnt.p, ucum.p, nb + 1, nullptr, f->tmp.p, s);
        PI_LAUNCH(k_q_compact, div_up(nb, 256), 256, 0, s, nb, qcnt.p, ucnt.p, ucum.p, order.p, list);
      }
      int cfg = 0;
      if (dense)
        cfg = eval_config_for(f, depth == f->dmax ? 0 : 1, qa, qn, nb, order.p, qcnt.p, ucnt.p, chunks.p,
                              qcnt.p + nb + 1, qval.p);
      if (dense && f->P.qef && depth == f->dmax && ctx->qef_parts > 1) {
        // the leaf level in parts: part p's QEF beside part p + 1's sampling
        const int parts = ctx->qef_parts;
        DBuf<int> pinfo;
        pinfo.alloc(ctx, s, 3 * (parts + 1));
        // the frame's array, so that it outlives the QEF stream's reads (the
        // QEF of this frame's coarser levels never reads it)
        DBuf<int8_t>& npart = f->npart;
        if (npart.n < (size_t)nl) npart.alloc(ctx, s, nl);
        PI_LAUNCH(k_part_bounds, 1, 128, 0, s, qcnt.p, (int)nb, parts, pinfo.p);
        PI_LAUNCH(k_node_part, div_up(nl, 256), 256, 0, s, nl, qkey.p, pinfo.p, parts, npart.p);
        PI_LAUNCH(k_q_chunks_parts, div_up(nb, 256), 256, 0, s, nb, ucnt.p, 32 * kEvalTable[cfg].K, parts, pinfo.p,
                  chunks.p);
        for (int p = 0; p < parts; ++p) {
          prof_begin(ctx, s, PG_CHUNK);
          // the grid is sized by the level (a part may hold fewer slots than
          // it has parts, and the blocks stride over the part's chunks)
          eval_chunks(f, cfg, qa, qn, order.p, qcnt.p, ucnt.p, chunks.p, pinfo.p + 2 * (parts + 1) + p,
                      pinfo.p + parts + 1 + p, kQefReserveRegs, qval.p, f->dcount.p);
          prof_end(ctx, s, PG_CHUNK);
          PI_LAUNCH(k_classify_thread, div_up(nl, 256), 256, 0, s, la, qval.p, rep.p, f->nd_c.p, f->nd_v.p,
                    f->nd_type.p, f->nd_sc.p, f->nd_curv.p, f->nd_samp.p, f->P.qef, f->dcount.p,
                    (const int8_t*)npart.p, p);
          qef_level(f, lb, le, depth, npart.p, p);
        }
      } else {
      const int pg = dense ? PG_CHUNK : PG_THREAD;
      prof_begin(ctx, s, pg);
      if (dense)
        dense_eval(f, cfg, qa, qn, nb, order.p, qcnt.p, ucnt.p, chunks.p, qcnt.p + nb + 1, qval.p, f->dcount.p);
      else
        PI_LAUNCH(k_q_eval_thread, (int)std::min<long long>((long long)ctx->smCount * 8, div_up(qn, 256)), 256, 0,
                  s, qa, list, ucum.p + nb, f->nd_c.p, f->nd_v.p, qval.p, f->dcount.p);
      prof_end(ctx, s, pg);
      if (known || leaf_level)  // no node needs a particle scan
        PI_LAUNCH(k_classify_thread, div_up(nl, 256), 256, 0, s, la, qval.p, rep.p, f->nd_c.p, f->nd_v.p,
                  f->nd_type.p, f->nd_sc.p, f->nd_curv.p, f->nd_samp.p, f->P.qef, f->dcount.p,
                  (const int8_t*)nullptr, 0);
      else
        PI_LAUNCH(k_classify, div_up(nl, wpb), 32 * wpb, 0, s, la, qval.p, rep.p, f->nd_c.p, f->nd_v.p,
                  f->nd_type.p, f->nd_sc.p, f->nd_curv.p, f->nd_samp.p, f->P.qef, known ? 1 : 0, f->dcount.p,
                  (const float*)nullptr);
      if (f->P.qef) qef_level(f, lb, le, depth);
      }
    }
    if (last) {
      f->nNodes = le;
      if (topo_early) topology_start(f);
      break;
    }
    flag.alloc(ctx, s, nl + 1);
    if (f->tmp.n < scan_tmp_ints(nl + 1)) f->tmp.alloc(ctx, s, scan_tmp_ints(nl + 1));
    PI_LAUNCH(k_internal_flag, div_up(nl, 256), 256, 0, s, f->nd_type.p, lb, le, flag.p);
    PI_CUDA(cudaMemsetAsync(flag.p + nl, 0, sizeof(int), s));
    exclusive_scan_i32(flag.p, flag.p, nl + 1, nullptr, f->tmp.p, s);
    // the number of INTERNAL nodes goes to pinned host memory and is read
    // while the spawn kernel runs, so that the device is still busy when the
    // host sizes the next level
    int* const nint_h = reinterpret_cast<int*>(ctx->hpin + kPinSlots * kCounterWords + 1);
    PI_CUDA(cudaMemcpyAsync(nint_h, flag.p + nl, sizeof(int), cudaMemcpyDeviceToHost, s));
    PI_CUDA(cudaEventRecord(f->ev[kLevelEvent], s));
    f->nNodes = le;
    ensure_nodes(f, le + 8 * nl);  // room for the children: at most 8 per node of the level
    known = depth + 1 >= f->dmin && depth < f->dmax;
    if (known) {
      // leaves by size never read their curvature (afterSampleEval returns
      // before the curvature test), so their parents only settle emptiness
      const float cell_child = 2.0f * std::ldexp(f->rootH, -(depth + 1));
      const int child_curv = (double)(cell_child - f->P.radius) < 1e-8 ? 0 : 1;
      if (child_curv)
        PI_LAUNCH(k_spawn_scan<true>, div_up(nl, kSpawnWarps), 32 * kSpawnWarps, 0, s, la, le, flag.p, depth + 1, f->nd_c.p,
                  f->nd_v.p, f->nd_id.p, f->nd_parent.p, f->nd_child.p, f->nd_type.p, f->nd_depth.p, f->nd_sc.p,
                  f->nd_curv.p, f->nd_org.p);
      else
        PI_LAUNCH(k_spawn_scan<false>, div_up(nl, kSpawnWarps), 32 * kSpawnWarps, 0, s, la, le, flag.p, depth + 1, f->nd_c.p,
                  f->nd_v.p, f->nd_id.p, f->nd_parent.p, f->nd_child.p, f->nd_type.p, f->nd_depth.p, f->nd_sc.p,
                  f->nd_curv.p, f->nd_org.p);
    } else {
      PI_LAUNCH(k_spawn, div_up(nl, 256), 256, 0, s, lb, le, le, flag.p, f->nd_type.p, depth + 1, f->nd_c.p,
                f->nd_v.p, f->nd_id.p, f->nd_parent.p, f->nd_child.p, f->nd_type.p, f->nd_depth.p, f->nd_sc.p,
                f->nd_curv.p, f->nd_org.p);
    }
    PI_CUDA(cudaEventSynchronize(f->ev[kLevelEvent]));
    const int nint = *nint_h;
    const long long newn = 8LL * nint;
    f->nNodes = le + newn;
    // depth D_max nodes are leaves by size, so nothing spawns past it
    if (nint == 0 || depth >= f->dmax) break;
    lb = le;
    le = le + newn;
  }
  // the last level's QEF may run on while the extraction builds the mesh
  // topology (stage_extract joins it before it reads node values, and takes
  // the octree's counters then)
  if (f->defer_qef_join && f->qef_inflight) return;
  qef_join(f);
  counters_snapshot(f, kPinOctree);
}

}  // namespace pisurf
