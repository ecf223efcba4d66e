// K6: dual-grid extraction, genIsoOurs state 1 (src/surface_reconstructor.cpp:290-323).
//
// The reference walks the octree recursively (include/traverse.h) and visits
// every interior octree vertex once with the 8 leaves around it
// (VisitorExtract::on_vert, src/visitorextract.cpp:229-256).  Those vertices
// are exactly the corners of leaves that lie strictly inside the root box, so
// here they are enumerated in parallel:
//   1. every leaf marks its interior corners (integer lattice at D_max) in
//      a Morton-indexed lattice bitmap (sort + unique above D_max = 10); the
//      set bits in index order are the dual vertices, in Z order;
//   2. per vertex, the leaf containing each of the 8 octants is found by
//      descending from the root; sign code, table[256] -> canonical case;
//   3. per non-trivial cell, the case triangles (src/visitorextract.cpp:95-199)
//      name leaf pairs; mesh vertices are deduplicated by the sorted leaf-id
//      pair, as Mesh::insert_vert keys them (src/global.cpp:13-32), the
//      first (lowest) slot of a key winning, through a hash table in L2;
//   4. one thread per mesh vertex bisects its leaf-to-leaf segment down to
//      r/2 with a field evaluation per step and interpolates with the 0.1/0.9
//      snap (calc_vertices, src/visitorextract.cpp:47-84);
//   5. triangles are oriented by the table's flip and deduplicated by their
//      sorted vertex triple, the first generated winning (Mesh::insert_tri,
//      src/global.cpp:34-53).
// The output order differs from the reference's traversal order; the mesh is
// the same set of vertices (by leaf-id pair) and triangles.
#include <algorithm>
#include <mutex>

#include "device.cuh"
#include "dmc.h"
#include "internal.h"

namespace pisurf {

__constant__ int c_trans[256][8];
__constant__ int c_flip[256];
__constant__ int c_code[256];
__constant__ int c_ntri[256];
__constant__ int c_tri[256][15];

void dmc_host_table(int trans[256][8], bool flip[256], int code[256]) {
  DmcTables t;
  dmc_build(&t);
  for (int i = 0; i < 256; ++i) {
    for (int k = 0; k < 8; ++k) trans[i][k] = t.trans[i][k];
    flip[i] = t.flip[i] != 0;
    code[i] = t.code[i];
  }
}

static void upload_tables(int device) {
  static std::mutex mu;
  static bool done[128] = {false};
  std::lock_guard<std::mutex> lk(mu);
  if (device >= 0 && device < 128 && done[device]) return;
  DmcTables t;
  dmc_build(&t);
  PI_CUDA(cudaMemcpyToSymbol(c_trans, t.trans, sizeof(t.trans)));
  PI_CUDA(cudaMemcpyToSymbol(c_flip, t.flip, sizeof(t.flip)));
  PI_CUDA(cudaMemcpyToSymbol(c_code, t.code, sizeof(t.code)));
  PI_CUDA(cudaMemcpyToSymbol(c_ntri, t.ntri, sizeof(t.ntri)));
  PI_CUDA(cudaMemcpyToSymbol(c_tri, t.tri, sizeof(t.tri)));
  if (device >= 0 && device < 128) done[device] = true;
}

__device__ __forceinline__ void edge_corners(int e, int* c0, int* c1) {
  const int axis = e >> 2, k = e & 3;
  const int u = axis == 0 ? 1 : 0, v = axis == 2 ? 1 : 2;
  *c0 = ((k & 1) << u) | (((k >> 1) & 1) << v);
  *c1 = *c0 | (1 << axis);
}

__global__ void k_leaf_flag(const int* __restrict__ nd_child, long long n, int* __restrict__ flag) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) flag[i] = nd_child[i] < 0 ? 1 : 0;
  if (i == n) flag[i] = 0;
}

__global__ void k_leaf_list(const int* __restrict__ nd_child, const int* __restrict__ scan, long long n,
                            int* __restrict__ leaves) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n && nd_child[i] < 0) leaves[scan[i]] = (int)i;
}

// Interior corners of each leaf, key (x << 2B) | (y << B) | z, B = D_max + 1;
// boundary corners get the all-ones key.
__global__ void k_corner_keys(const int* __restrict__ leaves, long long nl, const int4* __restrict__ nd_org,
                              int full, int B, uint64_t* __restrict__ keys, uint32_t* __restrict__ vals) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nl * 8) return;
  const int4 o = nd_org[leaves[t >> 3]];
  const int k = (int)(t & 7);
  const int x = o.x + ((k & 1) ? o.w : 0), y = o.y + ((k & 2) ? o.w : 0), z = o.z + ((k & 4) ? o.w : 0);
  uint64_t key;
  if (x > 0 && x < full && y > 0 && y < full && z > 0 && z < full)
    key = ((uint64_t)x << (2 * B)) | ((uint64_t)y << B) | (uint64_t)z;
  else
    key = (1ull << (3 * B)) - 1ull;
  keys[t] = key;
  vals[t] = (uint32_t)t;
}

// Morton code of three coordinates of up to 21 bits each (bit interleaving
// by the usual shift-and-mask steps), and its inverse.
__device__ __forceinline__ uint64_t spread3(uint64_t v) {
  v &= 0x1fffffull;
  v = (v | (v << 32)) & 0x1f00000000ffffull;
  v = (v | (v << 16)) & 0x1f0000ff0000ffull;
  v = (v | (v << 8)) & 0x100f00f00f00f00full;
  v = (v | (v << 4)) & 0x10c30c30c30c30c3ull;
  v = (v | (v << 2)) & 0x1249249249249249ull;
  return v;
}
__device__ __forceinline__ uint64_t compact3(uint64_t v) {
  v &= 0x1249249249249249ull;
  v = (v ^ (v >> 2)) & 0x10c30c30c30c30c3ull;
  v = (v ^ (v >> 4)) & 0x100f00f00f00f00full;
  v = (v ^ (v >> 8)) & 0x1f0000ff0000ffull;
  v = (v ^ (v >> 16)) & 0x1f00000000ffffull;
  v = (v ^ (v >> 32)) & 0x1fffffull;
  return v;
}

// Interior leaf corners (coordinates 1 .. 2^D_max - 1) as bits of a lattice
// bitmap indexed by the Morton code of (x - 1, y - 1, z - 1).  The Morton
// range is cut into blocks of 2^bb codes (a 2^(bb/3)-cube of lattice
// points).  Up to D_max = 10 (2^30 bits) every block is stored (slot = block,
// slot and blist null); above it only the blocks that hold a corner, with
// consecutive slots in block order, so that work and memory follow the
// surface rather than the volume of the lattice.  Either way the set bits in
// slot order are the unique corners in Z order, which keeps the later
// per-vertex work spatially coherent (as the reference's recursive
// traversal is).
__device__ __forceinline__ bool corner_code(const int* __restrict__ leaves, const int4* __restrict__ nd_org,
                                            int full, long long t, uint64_t* idx) {
  const int4 o = nd_org[leaves[t >> 3]];
  const int k = (int)(t & 7);
  const int x = o.x + ((k & 1) ? o.w : 0), y = o.y + ((k & 2) ? o.w : 0), z = o.z + ((k & 4) ? o.w : 0);
  if (!(x > 0 && x < full && y > 0 && y < full && z > 0 && z < full)) return false;
  *idx = spread3((uint64_t)(x - 1)) | (spread3((uint64_t)(y - 1)) << 1) | (spread3((uint64_t)(z - 1)) << 2);
  return true;
}

// used[block] = 1 for every block that holds a corner.
__global__ void k_block_mark(const int* __restrict__ leaves, long long nl, const int4* __restrict__ nd_org, int full,
                             int bb, int* __restrict__ used) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  uint64_t idx;
  if (t < nl * 8 && corner_code(leaves, nd_org, full, t, &idx)) used[idx >> bb] = 1;
}

// slot -> block (the inverse of the scan of used)
__global__ void k_block_list(long long nb, const int* __restrict__ used, const int* __restrict__ slot,
                             long long* __restrict__ blist) {
  const long long b = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (b < nb && used[b]) blist[slot[b]] = b;
}

__global__ void k_corner_mark(const int* __restrict__ leaves, long long nl, const int4* __restrict__ nd_org,
                              int full, int bb, const int* __restrict__ slot, unsigned* __restrict__ bits) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  // one lane per corner; corners of sibling leaves fall in a few bitmap words,
  // so the warp ORs its bits per word and issues one atomic per word
  long long word = -1;
  unsigned bit = 0u;
  uint64_t idx;
  if (t < nl * 8 && corner_code(leaves, nd_org, full, t, &idx)) {
    const uint64_t in_block = idx & ((1ull << bb) - 1ull);
    const long long blk = slot ? (long long)slot[idx >> bb] : (long long)(idx >> bb);
    word = (blk << (bb - 5)) + (long long)(in_block >> 5);
    bit = 1u << (unsigned)(in_block & 31ull);
  }
  unsigned todo = __ballot_sync(0xffffffffu, word >= 0);
  while (todo) {
    const int leader = __ffs(todo) - 1;
    const long long lw = __shfl_sync(0xffffffffu, word, leader);
    const bool mine = word == lw;
    const unsigned m = __reduce_or_sync(0xffffffffu, mine ? bit : 0u);
    if (lane == leader && (__ldg(bits + lw) & m) != m) atomicOr(bits + lw, m);
    todo &= ~__ballot_sync(0xffffffffu, mine);
  }
}

__global__ void k_bitmap_count(const unsigned* __restrict__ bits, long long nw, int* __restrict__ cnt) {
  long long w = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (w < nw) cnt[w] = __popc(bits[w]);
  if (w == nw) cnt[w] = 0;
}

__global__ void k_bitmap_keys(const unsigned* __restrict__ bits, long long nw, const int* __restrict__ off, int bb,
                              const long long* __restrict__ blist, int B, uint64_t* __restrict__ out) {
  long long w = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= nw) return;
  unsigned b = bits[w];
  int o = off[w];
  const long long sl = w >> (bb - 5);
  const uint64_t base = ((uint64_t)(blist ? blist[sl] : sl) << bb) | ((uint64_t)(w & ((1LL << (bb - 5)) - 1)) << 5);
  while (b) {
    const int i = __ffs(b) - 1;
    b &= b - 1;
    const uint64_t idx = base | (uint64_t)i;
    const uint64_t x = compact3(idx) + 1, y = compact3(idx >> 1) + 1, z = compact3(idx >> 2) + 1;
    out[o++] = (x << (2 * B)) | (y << B) | z;
  }
}

__device__ __forceinline__ uint32_t mix64to32(uint64_t k) {
  k ^= k >> 33;
  k *= 0xff51afd7ed558ccdull;
  k ^= k >> 33;
  k *= 0xc4ceb9fe1a85ec53ull;
  k ^= k >> 33;
  return (uint32_t)k;
}

// Deduplication by key with "first insertion wins" (Mesh::insert_vert /
// insert_tri, src/global.cpp:13-53): an open-addressing table of slot + 1
// per distinct key keeps the lowest slot (atomicMin), keys are compared
// through the slots' own key arrays.  The table has more entries than
// slots, so a probe always ends.
__global__ void k_vkey_insert(long long ns, const uint64_t* __restrict__ khi, const uint64_t* __restrict__ klo,
                              uint32_t mask, unsigned* __restrict__ tab, uint32_t* __restrict__ where) {
  long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= ns) return;
  const uint64_t lo = klo[s], hi = khi ? khi[s] : 0ull;
  uint32_t h = mix64to32(lo ^ (hi * 0x9E3779B97F4A7C15ull)) & mask;
  for (uint32_t t = 0; t <= mask; ++t) {
    unsigned cur = tab[h];
    if (cur == 0u) {
      cur = atomicCAS(tab + h, 0u, (unsigned)s + 1u);
      if (cur == 0u) break;
    }
    const long long o = (long long)cur - 1;
    if (klo[o] == lo && (!khi || khi[o] == hi)) {
      atomicMin(tab + h, (unsigned)s + 1u);
      break;
    }
    h = (h + 1u) & mask;
  }
  where[s] = h;
}

// Triangles: the sorted vertex triple of the oriented triangle is the key.
__device__ __forceinline__ void sorted3(const int* o, int& s0, int& s1, int& s2) {
  const int a = o[0], b = o[1], c = o[2];
  s0 = min(a, min(b, c));
  s2 = max(a, max(b, c));
  s1 = a + b + c - s0 - s2;
}

__global__ void k_tri_insert(long long nt, const int* __restrict__ otri, uint32_t mask, unsigned* __restrict__ tab,
                             uint32_t* __restrict__ where) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nt) return;
  int s0, s1, s2;
  sorted3(otri + 3 * t, s0, s1, s2);
  uint32_t h = mix64to32(((uint64_t)(uint32_t)s0 << 42) ^ ((uint64_t)(uint32_t)s1 << 21) ^ (uint64_t)(uint32_t)s2 ^
                         ((uint64_t)(uint32_t)s0 >> 22) * 0x9E3779B97F4A7C15ull) &
               mask;
  for (uint32_t i = 0; i <= mask; ++i) {
    unsigned cur = tab[h];
    if (cur == 0u) {
      cur = atomicCAS(tab + h, 0u, (unsigned)t + 1u);
      if (cur == 0u) break;
    }
    int o0, o1, o2;
    sorted3(otri + 3 * ((long long)cur - 1), o0, o1, o2);
    if (o0 == s0 && o1 == s1 && o2 == s2) {
      atomicMin(tab + h, (unsigned)t + 1u);
      break;
    }
    h = (h + 1u) & mask;
  }
  where[t] = h;
}

// flag[s] = 1 where slot s is its key's first (lowest) slot
__global__ void k_first_flag(long long n, const unsigned* __restrict__ tab, const uint32_t* __restrict__ where,
                             int* __restrict__ flag) {
  long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (s < n) flag[s] = tab[where[s]] == (unsigned)s + 1u ? 1 : 0;
  if (s == n) flag[s] = 0;
}

// slot -> vertex (numbered in order of first slots); vertex -> its first slot
__global__ void k_vertex_map(long long ns, const unsigned* __restrict__ tab, const uint32_t* __restrict__ where,
                             const int* __restrict__ rank, int* __restrict__ slot_vertex, int* __restrict__ rep) {
  long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= ns) return;
  const long long first = (long long)tab[where[s]] - 1;
  const int v = rank[first];
  slot_vertex[s] = v;
  if (first == s) rep[v] = (int)s;
}

__global__ void k_tri_write(long long nt, const int* __restrict__ rank, const int* __restrict__ otri,
                            int* __restrict__ out) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nt) return;
  const int o = rank[t];
  if (rank[t + 1] == o) return;
  out[3 * o] = otri[3 * t];
  out[3 * o + 1] = otri[3 * t + 1];
  out[3 * o + 2] = otri[3 * t + 2];
}

__global__ void k_unique_flag(const uint64_t* __restrict__ keys, long long n, uint64_t invalid,
                              int* __restrict__ flag) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i > n) return;
  if (i == n) {
    flag[i] = 0;
    return;
  }
  uint64_t k = keys[i];
  flag[i] = (k != invalid && (i == 0 || keys[i - 1] != k)) ? 1 : 0;
}

__global__ void k_unique_write(const uint64_t* __restrict__ keys, const int* __restrict__ scan, long long n,
                               uint64_t invalid, uint64_t* __restrict__ out) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint64_t k = keys[i];
  if (k != invalid && (i == 0 || keys[i - 1] != k)) out[scan[i]] = k;
}

// One thread per dual vertex (a unique interior leaf corner): the eight leaves
// around it by descent from the root, the octant of each point deciding the
// side of a mid-plane that holds it, then the DMC case.
__global__ void k_dual(const uint64_t* __restrict__ verts, long long nu, int B, const int* __restrict__ nd_child,
                       const int4* __restrict__ nd_org, const float4* __restrict__ nd_v, int* __restrict__ cells,
                       int* __restrict__ procs, int* __restrict__ tcount, unsigned long long* __restrict__ ndual) {
  long long u = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (u > nu) return;
  if (u == nu) {
    tcount[u] = 0;
    return;
  }
  const uint64_t key = verts[u];
  const uint64_t m = (1ull << B) - 1ull;
  const int x = (int)((key >> (2 * B)) & m), y = (int)((key >> B) & m), z = (int)(key & m);
  // the eight octant points share the descent until the node one of whose
  // mid-planes holds the corner; each octant continues from there
  int start = 0;
  for (int guard = 0; guard < 64; ++guard) {
    const int ch = nd_child[start];
    if (ch < 0) break;
    const int4 o = nd_org[start];
    const int mid = o.w >> 1;
    if (x == o.x + mid || y == o.y + mid || z == o.z + mid) break;
    start = ch + ((x > o.x + mid) ? 1 : 0) + ((y > o.y + mid) ? 2 : 0) + ((z > o.z + mid) ? 4 : 0);
  }
  // the eight descents below `start` advance in lockstep, so that their
  // loads are in flight together rather than one chain after another
  int n8[8];
#pragma unroll
  for (int c = 0; c < 8; ++c) n8[c] = start;
  for (int guard = 0; guard < 64; ++guard) {
    int ch[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) ch[c] = nd_child[n8[c]];
    bool more = false;
#pragma unroll
    for (int c = 0; c < 8; ++c)
      if (ch[c] >= 0) {
        const int4 o = nd_org[n8[c]];
        const int mid = o.w >> 1;
        const int bx = (x > o.x + mid || (x == o.x + mid && (c & 1))) ? 1 : 0;
        const int by = (y > o.y + mid || (y == o.y + mid && (c & 2))) ? 1 : 0;
        const int bz = (z > o.z + mid || (z == o.z + mid && (c & 4))) ? 1 : 0;
        n8[c] = ch[c] + (bx | (by << 1) | (bz << 2));
        more = true;
      }
    if (!more) break;
  }
  int index = 0;
#pragma unroll
  for (int c = 0; c < 8; ++c)
    if (nd_v[n8[c]].w > 0.f) index |= 1 << c;
  const int code = c_code[index];
  int nt = 0;
  if (code != 0 && code != 255) {
    nt = c_ntri[code];
    for (int c = 0; c < 8; ++c) cells[8 * u + c] = n8[c_trans[index][c]];
    stripe_add(ndual, C_DUAL, 1ull);
  }
  procs[u] = index;
  tcount[u] = nt;
}

__global__ void k_tri_slots(long long nu, const int* __restrict__ cells, const int* __restrict__ procs,
                            const int* __restrict__ toff, const uint64_t* __restrict__ nd_id, int id_bits,
                            int packed, int* __restrict__ slotA, int* __restrict__ slotB,
                            uint64_t* __restrict__ khi, uint64_t* __restrict__ klo, int8_t* __restrict__ tflip) {
  long long u = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (u >= nu) return;
  const int index = procs[u];
  const int code = c_code[index];
  if (code == 0 || code == 255) return;
  const int nt = c_ntri[code];
  const long long t0 = toff[u];
  for (int t = 0; t < nt; ++t) {
    tflip[t0 + t] = (int8_t)c_flip[index];
    for (int k = 0; k < 3; ++k) {
      int c0, c1;
      edge_corners(c_tri[code][3 * t + k], &c0, &c1);
      const int A = cells[8 * u + c0], Bn = cells[8 * u + c1];
      const long long s = 3 * (t0 + t) + k;
      slotA[s] = A;
      slotB[s] = Bn;
      uint64_t ia = nd_id[A], ib = nd_id[Bn];
      uint64_t lo = ia < ib ? ia : ib, hi = ia < ib ? ib : ia;
      if (packed) {
        klo[s] = (lo << id_bits) | hi;
      } else {
        khi[s] = lo;
        klo[s] = hi;
      }
    }
  }
}

struct BisectArgs {
  GridView g;  // the hash grid (constant radius); with a variable radius the grid the vertices are bucketed by
  PartView P;
  float iso;
  float rr;  // r / 2 (variable radius: the searcher's minimum radius / 2)
  const MultiGridView* mg;  // variable radius: the bins' grids, else null
};

// Vertices listed by the hash cell of their first bisection midpoint (count
// per cell, scan, place), so that neighbouring threads of k_bisect walk the
// same cells.  Order within a cell is arbitrary: each vertex's result
// depends on its own edge only.
__device__ __forceinline__ int vertex_cell(const BisectArgs& a, const float4& p, const float4& q, int ekx,
                                           int eky) {
  const float mx = __fmul_rn(__fadd_rn(p.x, q.x), 0.5f);
  const float my = __fmul_rn(__fadd_rn(p.y, q.y), 0.5f);
  const float mz = __fmul_rn(__fadd_rn(p.z, q.z), 0.5f);
  int cx, cy, cz;
  cell_of(a.g, mx, my, mz, cx, cy, cz);
  return ((cz + 2) * eky + (cy + 2)) * ekx + (cx + 2);
}

__global__ void k_vcell_count(BisectArgs a, long long nv, const int* __restrict__ rep, const int* __restrict__ slotA,
                              const int* __restrict__ slotB, const float4* __restrict__ nd_v, int ekx, int eky,
                              int* __restrict__ cnt, int* __restrict__ key) {
  const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  int k = -1;
  if (v < nv) {
    const int s = rep[v];
    k = vertex_cell(a, nd_v[slotA[s]], nd_v[slotB[s]], ekx, eky);
  }
  const unsigned peers = __match_any_sync(0xffffffffu, k);
  if (k >= 0 && lane == __ffs(peers) - 1) atomicAdd(cnt + k, __popc(peers));
  if (v < nv) key[v] = k;
}

__global__ void k_vcell_place(long long nv, const int* __restrict__ key, const int* __restrict__ off,
                              int* __restrict__ fill, int* __restrict__ list) {
  const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  const int k = v < nv ? key[v] : -1;
  const unsigned peers = __match_any_sync(0xffffffffu, k);
  if (k < 0) return;
  const int leader = __ffs(peers) - 1;
  int b = 0;
  if (lane == leader) b = atomicAdd(fill + k, __popc(peers));
  b = __shfl_sync(peers, b, leader);
  list[off[k] + b + __popc(peers & ((1u << lane) - 1u))] = (int)v;
}

template <bool VR>
__global__ void k_bisect(BisectArgs a, long long nv, const int* __restrict__ order, const int* __restrict__ rep,
                         const int* __restrict__ slotA,
                         const int* __restrict__ slotB, const float4* __restrict__ nd_v,
                         const uint64_t* __restrict__ nd_id, float* __restrict__ out,
                         uint64_t* __restrict__ vkeys, int2* __restrict__ vedge,
                         unsigned long long* __restrict__ counters) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nv) return;
  const long long v = order[t];
  const int s = rep[v];
  const int A = slotA[s], B = slotB[s];
  vedge[v] = make_int2(A, B);
  float4 p = nd_v[A], q = nd_v[B];
  const float dx = __fsub_rn(p.x, q.x), dy = __fsub_rn(p.y, q.y), dz = __fsub_rn(p.z, q.z);
  float d = __fsqrt_rn(__fadd_rn(__fmul_rn(dx, dx), __fadd_rn(__fmul_rn(dy, dy), __fmul_rn(dz, dz))));
  long long pairs = 0;
  int steps = 0;
  while (d > a.rr && steps < 64) {
    float4 m;
    m.x = __fmul_rn(__fadd_rn(p.x, q.x), 0.5f);
    m.y = __fmul_rn(__fadd_rn(p.y, q.y), 0.5f);
    m.z = __fmul_rn(__fadd_rn(p.z, q.z), 0.5f);
    m.w = a.iso - (VR ? field_sum_vr(*a.mg, a.P, m.x, m.y, m.z, &pairs) : field_sum(a.g, a.P, m.x, m.y, m.z, &pairs));
    if ((m.w > 0.f) == (p.w > 0.f))
      p = m;
    else
      q = m;
    d = __fmul_rn(d, 0.5f);
    ++steps;
  }
  const float ratio = __fdiv_rn(__fsub_rn(0.0f, p.w), __fsub_rn(q.w, p.w));
  float3 r;
  if (ratio < kAbove01) {  // (double)ratio < 0.1
    r = make_float3(p.x, p.y, p.z);
  } else if (ratio > kBelow09) {  // (double)ratio > 0.9
    r = make_float3(q.x, q.y, q.z);
  } else {
    r.x = __fadd_rn(p.x, __fmul_rn(__fsub_rn(q.x, p.x), ratio));
    r.y = __fadd_rn(p.y, __fmul_rn(__fsub_rn(q.y, p.y), ratio));
    r.z = __fadd_rn(p.z, __fmul_rn(__fsub_rn(q.z, p.z), ratio));
  }
  out[3 * v] = r.x;
  out[3 * v + 1] = r.y;
  out[3 * v + 2] = r.z;
  uint64_t ia = nd_id[A], ib = nd_id[B];
  vkeys[2 * v] = ia < ib ? ia : ib;
  vkeys[2 * v + 1] = ia < ib ? ib : ia;
  stripe_add(counters, C_BISECT_EVALS, (unsigned long long)steps);
  stripe_add(counters, C_BISECT_PAIRS, (unsigned long long)pairs);
}

// Oriented triangle in Mesh::insert_tri argument order.
__global__ void k_tri_orient(long long nt, const int* __restrict__ slot_vertex, const int8_t* __restrict__ tflip,
                             int* __restrict__ otri) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nt) return;
  const int a = slot_vertex[3 * t], b = slot_vertex[3 * t + 1], c = slot_vertex[3 * t + 2];
  otri[3 * t] = tflip[t] ? a : c;
  otri[3 * t + 1] = b;
  otri[3 * t + 2] = tflip[t] ? c : a;
}

// Mask of the smallest power-of-two table with more than n entries.
static uint32_t table_mask(long long n) {
  uint32_t m = 1;
  while ((long long)m < n + 1) m <<= 1;
  return m - 1;
}

static int read_int(pi_frame* f, const int* d) {
  int v = 0;
  PI_CUDA(cudaMemcpyAsync(&v, d, sizeof(int), cudaMemcpyDeviceToHost, f->ctx->stream));
  PI_CUDA(cudaStreamSynchronize(f->ctx->stream));
  return v;
}

// A count read in two halves: the copy to pinned memory is queued, the
// caller queues a kernel that does not need the count, then waits for the
// copy only, so the device is busy while the host takes the value.
static void read_int_start(pi_frame* f, const int* d) {
  int* const h = reinterpret_cast<int*>(f->ctx->hpin + kPinReadOffset);
  PI_CUDA(cudaMemcpyAsync(h, d, sizeof(int), cudaMemcpyDeviceToHost, f->ctx->stream));
  PI_CUDA(cudaEventRecord(f->ctx->ev_read, f->ctx->stream));
}
static int read_int_finish(pi_frame* f) {
  PI_CUDA(cudaEventSynchronize(f->ctx->ev_read));
  return *reinterpret_cast<const int*>(f->ctx->hpin + kPinReadOffset);
}

// A count read on stream st through a pinned word and an event.
struct CountReader {
  pi_frame* f;
  cudaStream_t st;
  int off;
  cudaEvent_t ev;
  int read(const int* d) const {
    start(d);
    return finish();
  }
  void start(const int* d) const {
    int* const h = reinterpret_cast<int*>(f->ctx->hpin + off);
    PI_CUDA(cudaMemcpyAsync(h, d, sizeof(int), cudaMemcpyDeviceToHost, st));
    PI_CUDA(cudaEventRecord(ev, st));
  }
  int finish() const {
    PI_CUDA(cudaEventSynchronize(ev));
    return *reinterpret_cast<const int*>(f->ctx->hpin + off);
  }
};

// Steps 1-2 of the extraction, the mesh topology: it reads only the tree
// (nd_child, nd_org of the f->nNodes nodes), not the leaves' values.  Sets
// f->nLeaves, f->tp_uverts (the unique interior leaf corners as lattice
// keys, in Z order) and f->tp_nu.
static void extract_topology(pi_frame* f, cudaStream_t s, const CountReader& rd) {
  pi_ctx* c = f->ctx;
  const long long nn = f->nNodes;
  // 1. leaves
  DBuf<int> flag, leaves, tmp;
  flag.alloc(c, s, nn + 1);
  tmp.alloc(c, s, scan_tmp_ints(nn * 8 + 1));
  PI_LAUNCH(k_leaf_flag, div_up(nn + 1, 256), 256, 0, s, f->nd_child.p, nn, flag.p);
  exclusive_scan_i32(flag.p, flag.p, nn + 1, nullptr, tmp.p, s);
  rd.start(flag.p + nn);
  leaves.alloc(c, s, nn > 0 ? nn : 1);  // room for every node
  PI_LAUNCH(k_leaf_list, div_up(nn, 256), 256, 0, s, f->nd_child.p, flag.p, nn, leaves.p);
  const long long nl = rd.finish();
  f->nLeaves = nl;
  // 2. dual vertices = unique interior leaf corners
  const int B = f->dmax + 1;
  const int full = 1 << f->dmax;
  const long long nk = nl * 8;
  DBuf<uint64_t>& uverts = f->tp_uverts;
  long long nu = 0;
  // block size: 2^bb Morton codes, bb a multiple of 3 and at least 15 (32^3
  // points, 1024 words), so that at most 2^24 blocks cover the lattice; past
  // 2^18 codes a block (D_max > 14) the blocks grow too large and the corners
  // are sorted instead (below)
  const int bb = std::max(15, ((3 * f->dmax - 24 + 2) / 3) * 3);
  if (bb <= 18) {
    const long long nb = 1LL << std::max(0, 3 * f->dmax - bb);
    // the whole bitmap costs less than finding the used blocks up to 2^30 bits
    const bool dense = f->dmax <= 10;
    long long nused = nb;
    DBuf<int> used, slot;
    DBuf<long long> blist;
    if (!dense) {
      used.alloc(c, s, nb + 1);
      if (tmp.n < scan_tmp_ints(nb + 1)) tmp.alloc(c, s, scan_tmp_ints(nb + 1));
      PI_CUDA(cudaMemsetAsync(used.p, 0, sizeof(int) * (nb + 1), s));
      PI_LAUNCH(k_block_mark, div_up(nk, 256), 256, 0, s, leaves.p, nl, f->nd_org.p, full, bb, used.p);
      slot.alloc(c, s, nb + 1);
      exclusive_scan_i32(used.p, slot.p, nb + 1, nullptr, tmp.p, s);
      nused = rd.read(slot.p + nb);
      blist.alloc(c, s, nused > 0 ? nused : 1);
      PI_LAUNCH(k_block_list, div_up(nb, 256), 256, 0, s, nb, used.p, slot.p, blist.p);
    }
    const long long nw = nused << (bb - 5);
    DBuf<unsigned> bits;
    DBuf<int> cnt;
    bits.alloc(c, s, nw > 0 ? nw : 1);
    cnt.alloc(c, s, nw + 1);
    if (tmp.n < scan_tmp_ints(nw + 1)) tmp.alloc(c, s, scan_tmp_ints(nw + 1));
    PI_CUDA(cudaMemsetAsync(bits.p, 0, sizeof(unsigned) * (nw > 0 ? nw : 1), s));
    PI_LAUNCH(k_corner_mark, div_up(nk, 256), 256, 0, s, leaves.p, nl, f->nd_org.p, full, bb,
              dense ? nullptr : slot.p, bits.p);
    PI_LAUNCH(k_bitmap_count, div_up(nw + 1, 256), 256, 0, s, bits.p, nw, cnt.p);
    exclusive_scan_i32(cnt.p, cnt.p, nw + 1, nullptr, tmp.p, s);
    nu = rd.read(cnt.p + nw);
    if (uverts.n < (size_t)(nu > 0 ? nu : 1)) uverts.alloc(c, s, nu > 0 ? nu : 1);
    PI_LAUNCH(k_bitmap_keys, div_up(nw, 256), 256, 0, s, bits.p, nw, cnt.p, bb, dense ? nullptr : blist.p, B,
              uverts.p);
  } else {
    const uint64_t invalid = (1ull << (3 * B)) - 1ull;
    DBuf<uint64_t> keys, keys2;
    DBuf<uint32_t> vals, vals2;
    keys.alloc(c, s, nk);
    keys2.alloc(c, s, nk);
    vals.alloc(c, s, nk);
    vals2.alloc(c, s, nk);
    PI_LAUNCH(k_corner_keys, div_up(nk, 256), 256, 0, s, leaves.p, nl, f->nd_org.p, full, B, keys.p, vals.p);
    DBuf<int> rtmp;
    rtmp.alloc(c, s, radix_tmp_ints(nk));
    uint64_t *kp = keys.p, *ka = keys2.p;
    uint32_t *vp = vals.p, *va = vals2.p;
    radix_sort_u64(&kp, &vp, &ka, &va, nk, 3 * B, rtmp.p, s);
    DBuf<int> uf;
    uf.alloc(c, s, nk + 1);
    PI_LAUNCH(k_unique_flag, div_up(nk + 1, 256), 256, 0, s, kp, nk, invalid, uf.p);
    exclusive_scan_i32(uf.p, uf.p, nk + 1, nullptr, tmp.p, s);
    nu = rd.read(uf.p + nk);
    if (uverts.n < (size_t)(nu > 0 ? nu : 1)) uverts.alloc(c, s, nu > 0 ? nu : 1);
    PI_LAUNCH(k_unique_write, div_up(nk, 256), 256, 0, s, kp, uf.p, nk, invalid, uverts.p);
  }
  f->tp_nu = nu;
}

void topology_start(pi_frame* f) {
  pi_ctx* c = f->ctx;
  cudaStream_t ts = c->topo_stream;
  PI_CUDA(cudaStreamWaitEvent(ts, c->ev_topo_in, 0));
  extract_topology(f, ts, CountReader{f, ts, kPinTopoReadOffset, c->ev_topo_read});
  PI_CUDA(cudaEventRecord(c->ev_topo_done, ts));
  f->tp_inflight = true;
}

void topology_join(pi_frame* f) {
  if (!f->tp_inflight) return;
  PI_CUDA(cudaStreamWaitEvent(f->ctx->stream, f->ctx->ev_topo_done, 0));
  f->tp_inflight = false;
}

void topology_fence(pi_frame* f) {
  topology_join(f);
  pi_ctx* c = f->ctx;
  PI_CUDA(cudaEventRecord(c->ev_topo_in, c->stream));
  PI_CUDA(cudaStreamWaitEvent(c->topo_stream, c->ev_topo_in, 0));
}

void stage_extract(pi_frame* f) {
  pi_ctx* c = f->ctx;
  cudaStream_t s = c->stream;
  upload_tables(c->device);
  // steps 1-2: the topology, started beside the octree's last level or run
  // here
  if (f->tp_inflight)
    topology_join(f);
  else
    extract_topology(f, s, CountReader{f, s, kPinReadOffset, c->ev_read});
  const int B = f->dmax + 1;
  const long long nu = f->tp_nu;
  const uint64_t* const uverts = f->tp_uverts.p;
  DBuf<int> tmp;
  tmp.alloc(c, s, scan_tmp_ints(nu + 1));
  // 3. dual cells
  DBuf<int> cells, procs, toff;
  cells.alloc(c, s, nu * 8 > 0 ? nu * 8 : 1);
  procs.alloc(c, s, nu > 0 ? nu : 1);
  toff.alloc(c, s, nu + 1);
  if (tmp.n < scan_tmp_ints(nu + 1)) tmp.alloc(c, s, scan_tmp_ints(nu + 1));
  // k_dual reads the leaves' values: the octree's last QEF level, if it was
  // left running, ends here, and the octree's counters are taken
  if (f->qef_inflight) {
    qef_join(f);
    counters_snapshot(f, kPinOctree);
  }
  counters_reset(f);
  PI_LAUNCH(k_dual, div_up(nu + 1, 128), 128, 0, s, uverts, nu, B, f->nd_child.p, f->nd_org.p, f->nd_v.p,
            cells.p, procs.p, toff.p, f->dcount.p);
  exclusive_scan_i32(toff.p, toff.p, nu + 1, nullptr, tmp.p, s);
  const long long nt0 = read_int(f, toff.p + nu);
  // 4. triangle slots and vertex keys (sorted leaf-id pairs)
  const int id_bits = 3 * f->dmax;
  const int packed = (2 * id_bits <= 64) ? 1 : 0;
  const long long ns = 3 * nt0;
  DBuf<int> slotA, slotB;
  DBuf<uint64_t> khi, klo;
  DBuf<int8_t> tflip;
  slotA.alloc(c, s, ns > 0 ? ns : 1);
  slotB.alloc(c, s, ns > 0 ? ns : 1);
  klo.alloc(c, s, ns > 0 ? ns : 1);
  if (!packed) khi.alloc(c, s, ns > 0 ? ns : 1);
  tflip.alloc(c, s, nt0 > 0 ? nt0 : 1);
  PI_LAUNCH(k_tri_slots, div_up(nu, 128), 128, 0, s, nu, cells.p, procs.p, toff.p, f->nd_id.p, id_bits, packed,
            slotA.p, slotB.p, khi.p, klo.p, tflip.p);
  cells.release();
  procs.release();
  toff.release();
  // 5. unique mesh vertices: first slot of each key, numbered in slot order
  DBuf<unsigned> vtab;
  DBuf<uint32_t> vwhere;
  DBuf<int> vrank, slot_vertex, rep;
  const uint32_t vmask = table_mask(ns);
  vtab.alloc(c, s, (size_t)vmask + 1);
  vwhere.alloc(c, s, ns > 0 ? ns : 1);
  vrank.alloc(c, s, ns + 1);
  if (tmp.n < scan_tmp_ints(ns + 1)) tmp.alloc(c, s, scan_tmp_ints(ns + 1));
  PI_CUDA(cudaMemsetAsync(vtab.p, 0, sizeof(unsigned) * ((size_t)vmask + 1), s));
  PI_LAUNCH(k_vkey_insert, div_up(ns, 256), 256, 0, s, ns, packed ? nullptr : khi.p, klo.p, vmask, vtab.p,
            vwhere.p);
  PI_LAUNCH(k_first_flag, div_up(ns + 1, 256), 256, 0, s, ns, vtab.p, vwhere.p, vrank.p);
  exclusive_scan_i32(vrank.p, vrank.p, ns + 1, nullptr, tmp.p, s);
  read_int_start(f, vrank.p + ns);
  slot_vertex.alloc(c, s, ns > 0 ? ns : 1);
  rep.alloc(c, s, ns > 0 ? ns : 1);  // room for a vertex per slot
  PI_LAUNCH(k_vertex_map, div_up(ns, 256), 256, 0, s, ns, vtab.p, vwhere.p, vrank.p, slot_vertex.p, rep.p);
  const long long nv = read_int_finish(f);
  vtab.release();
  vwhere.release();
  vrank.release();
  khi.release();
  klo.release();
  // 6. triangles: first of each sorted vertex triple, in generation order
  // (they need the vertex numbering, not the positions, so they come before
  // the bisection and, for a host destination, their copy overlaps it)
  DBuf<int> otri, trank;
  DBuf<unsigned> ttab;
  DBuf<uint32_t> twhere;
  otri.alloc(c, s, nt0 * 3 > 0 ? nt0 * 3 : 3);
  PI_LAUNCH(k_tri_orient, div_up(nt0, 256), 256, 0, s, nt0, slot_vertex.p, tflip.p, otri.p);
  // nearly every triangle is distinct, so the table gets twice as many
  // entries as triangles (load at most 1/2; linear probing degrades fast
  // above that)
  const uint32_t tmask = table_mask(2 * nt0);
  ttab.alloc(c, s, (size_t)tmask + 1);
  twhere.alloc(c, s, nt0 > 0 ? nt0 : 1);
  trank.alloc(c, s, nt0 + 1);
  PI_CUDA(cudaMemsetAsync(ttab.p, 0, sizeof(unsigned) * ((size_t)tmask + 1), s));
  PI_LAUNCH(k_tri_insert, div_up(nt0, 256), 256, 0, s, nt0, otri.p, tmask, ttab.p, twhere.p);
  PI_LAUNCH(k_first_flag, div_up(nt0 + 1, 256), 256, 0, s, nt0, ttab.p, twhere.p, trank.p);
  exclusive_scan_i32(trank.p, trank.p, nt0 + 1, nullptr, tmp.p, s);
  read_int_start(f, trank.p + nt0);
  // room for every generated triangle and the splash icosahedra
  const long long nsp = f->P.splash ? f->nSplash : 0;
  const long long tcap = (nt0 + 20 * nsp) * 3;
  f->mt.alloc(c, s, tcap > 0 ? tcap : 3);
  PI_LAUNCH(k_tri_write, div_up(nt0, 256), 256, 0, s, nt0, trank.p, otri.p, f->mt.p);
  f->mv.alloc(c, s, (nv + 12 * nsp) * 3 > 0 ? (nv + 12 * nsp) * 3 : 3);
  f->mk.alloc(c, s, (nv + 12 * nsp) * 2 > 0 ? (nv + 12 * nsp) * 2 : 2);
  f->vedge.alloc(c, s, nv + 12 * nsp > 0 ? nv + 12 * nsp : 1);
  if (nsp > 0) PI_CUDA(cudaMemsetAsync(f->vedge.p + nv, 0xff, sizeof(int2) * 12 * nsp, s));
  const long long nt = read_int_finish(f);
  // splash icosahedra after the surface (Mesh::AppendSplash_ConstR runs
  // after generate_mesh, src/surface_reconstructor.cpp:299-320)
  if (nsp > 0) splash_mesh(f, nv, nt);
  f->nT = nt + 20 * nsp;
  if (f->host_tris && f->nT > 0 && f->nT <= f->host_tcap) {
    PI_CUDA(cudaEventRecord(c->ev_tris_ready, s));
    PI_CUDA(cudaStreamWaitEvent(c->copy_stream, c->ev_tris_ready, 0));
    PI_CUDA(cudaMemcpyAsync(f->host_tris, f->mt.p, sizeof(int) * 3 * f->nT, cudaMemcpyDeviceToHost,
                            c->copy_stream));
    PI_CUDA(cudaEventRecord(c->ev_tris_copied, c->copy_stream));
    f->tris_sent = true;
  }
  // 7. vertex positions by bisection (the splash vertices follow them)
  f->nV = nv + 12 * nsp;
  const GridHost& gh = f->g;
  BisectArgs ba{GridView{gh.bounding[0], gh.bounding[2], gh.bounding[4], gh.cell, gh.nx, gh.ny, gh.nz, f->off.p},
                PartView{f->pos.p, f->xm.p, f->ga.p, f->gb.p, f->xlo.p}, f->iso, f->P.radius / 2, nullptr};
  if (f->varR) {
    // bucket the vertices by a grid of cells 4 * maxR over the root box;
    // bisect down to half the searcher's minimum radius
    // (src/visitorextract.cpp:54)
    const float bcell = f->vrMaxR * 4.0f;
    const int bn = std::max(1, (int)std::ceil(2.0f * f->rootH / bcell));
    ba.g = GridView{f->rootC[0] - f->rootH, f->rootC[1] - f->rootH, f->rootC[2] - f->rootH, bcell, bn, bn, bn, nullptr};
    ba.rr = f->vrMinR / 2;
    ba.mg = f->mgv.p;
  }
  {
    const int ekx = ba.g.nx + 4, eky = ba.g.ny + 4;
    const long long nc = (long long)ekx * eky * (ba.g.nz + 4);
    DBuf<int> vcnt, vfill, vkey, vorder;
    vcnt.alloc(c, s, nc + 1);
    vfill.alloc(c, s, nc);
    vkey.alloc(c, s, nv > 0 ? nv : 1);
    vorder.alloc(c, s, nv > 0 ? nv : 1);
    if (tmp.n < scan_tmp_ints(nc + 1)) tmp.alloc(c, s, scan_tmp_ints(nc + 1));
    PI_CUDA(cudaMemsetAsync(vcnt.p, 0, sizeof(int) * (nc + 1), s));
    PI_CUDA(cudaMemsetAsync(vfill.p, 0, sizeof(int) * nc, s));
    PI_LAUNCH(k_vcell_count, div_up(nv, 256), 256, 0, s, ba, nv, rep.p, slotA.p, slotB.p, f->nd_v.p, ekx, eky,
              vcnt.p, vkey.p);
    exclusive_scan_i32(vcnt.p, vcnt.p, nc + 1, nullptr, tmp.p, s);
    PI_LAUNCH(k_vcell_place, div_up(nv, 256), 256, 0, s, nv, vkey.p, vcnt.p, vfill.p, vorder.p);
    prof_begin(c, s, PG_BISECT);
    if (f->varR)
      PI_LAUNCH(k_bisect<true>, div_up(nv, 128), 128, 0, s, ba, nv, vorder.p, rep.p, slotA.p, slotB.p, f->nd_v.p,
                f->nd_id.p, f->mv.p, f->mk.p, f->vedge.p, f->dcount.p);
    else
      PI_LAUNCH(k_bisect<false>, div_up(nv, 128), 128, 0, s, ba, nv, vorder.p, rep.p, slotA.p, slotB.p, f->nd_v.p,
                f->nd_id.p, f->mv.p, f->mk.p, f->vedge.p, f->dcount.p);
    prof_end(c, s, PG_BISECT);
  }
  counters_snapshot(f, kPinExtract);
}

}  // namespace pisurf
