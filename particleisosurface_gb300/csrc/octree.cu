// K4: adaptive octree, genIsoOurs state 0 (src/surface_reconstructor.cpp:326-407).
//
// The reference keeps a LIFO of nodes but processes the whole frontier at
// once (inProcessSize = 10^7), so refinement is breadth-first: one level per
// iteration.  Here each level is three launches:
//   k_empty_curv  beforeSampleEval / checkEmptyAndCalcCurv (:152-235): one
//                 warp per node walks the hash-cell rows of the node box and
//                 tests particles against the box grown by r * smooth_factor;
//                 nodes above D_min only need existence (early exit on ballot).
//   k_sample      afterSampleEval (:237-273) with TNode::GenerateSampling /
//                 NodeSampling / GridEval (src/iso_method_ours.cpp:52-99,
//                 src/evaluator.cpp:127-252): one warp per node, lanes 0..26
//                 evaluate the 3x3x3 samples, lane 27 the centre; the sign
//                 change is a warp ballot.
//   k_spawn       8 children per INTERNAL node (TNode ctor,
//                 src/iso_method_ours.cpp:25-38) after an exclusive scan of
//                 the INTERNAL flags.
#include <algorithm>
#include <cmath>

#include "device.cuh"
#include "internal.h"

namespace pisurf {

enum : int8_t { T_EMPTY = 0, T_INTERNAL = 1, T_LEAF = 2, T_UNCERTAIN = 3 };

struct LevelArgs {
  GridView g;
  float B1, B3, B5;  // Bounding upper corners
  const float4* pos;
  const float4* nrm;
  float expand;      // r * smooth_factor
  float iso;
  long long lb, le;  // node range of the level
  int big;           // depth < D_min
};

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__global__ void k_empty_curv(LevelArgs a, const float4* __restrict__ nd_c, float4* __restrict__ nd_v,
                             int8_t* __restrict__ nd_type, float* __restrict__ nd_curv) {
  const long long node = a.lb + (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (node >= a.le) return;
  const float4 c = nd_c[node];
  const float h = c.w;
  const float b1x = __fsub_rn(c.x, h), b1y = __fsub_rn(c.y, h), b1z = __fsub_rn(c.z, h);
  const float b2x = __fadd_rn(c.x, h), b2y = __fadd_rn(c.y, h), b2z = __fadd_rn(c.z, h);
  const float lox = __fsub_rn(b1x, a.expand), loy = __fsub_rn(b1y, a.expand), loz = __fsub_rn(b1z, a.expand);
  const float hix = __fadd_rn(b2x, a.expand), hiy = __fadd_rn(b2y, a.expand), hiz = __fadd_rn(b2z, a.expand);
  // GetInBoxParticles cell block (src/hash_grid.cpp:164-194)
  int mnx, mny, mnz, mxx, mxy, mxz;
  cell_of(a.g, fmaxf(b1x, a.g.b0), fmaxf(b1y, a.g.b2), fmaxf(b1z, a.g.b4), mnx, mny, mnz);
  cell_of(a.g, fminf(b2x, a.B1), fminf(b2y, a.B3), fminf(b2z, a.B5), mxx, mxy, mxz);
  const int x0 = max(mnx - 1, 0), x1 = min(mxx + 1, a.g.nx - 1);
  const int y0 = max(mny - 1, 0), y1 = min(mxy + 1, a.g.ny - 1);
  const int z0 = max(mnz - 1, 0), z1 = min(mxz + 1, a.g.nz - 1);
  bool found = false;
  Kahan sx, sy, sz, ar;
  if (x0 <= x1) {
    for (int z = z0; z <= z1; ++z) {
      for (int y = y0; y <= y1; ++y) {
        long long base = ((long long)z * a.g.ny + y) * a.g.nx;
        int s = __ldg(a.g.off + base + x0), e = __ldg(a.g.off + base + x1 + 1);
        for (int j0 = s; j0 < e; j0 += 32) {
          int j = j0 + lane;
          bool in = false;
          if (j < e) {
            float4 p = __ldg(a.pos + j);
            in = p.x > lox && p.x < hix && p.y > loy && p.y < hiy && p.z > loz && p.z < hiz;
            if (in && !a.big) {
              float4 nv = __ldg(a.nrm + j);
              sx.add(nv.x);
              sy.add(nv.y);
              sz.add(nv.z);
              ar.add(nv.w);
            }
          }
          found |= in;
          if (a.big && __any_sync(0xffffffffu, found)) goto done;
        }
      }
    }
  }
done:
  found = __any_sync(0xffffffffu, found);
  float nx = warp_sum(sx.s + (-sx.c)), ny = warp_sum(sy.s + (-sy.c)), nz = warp_sum(sz.s + (-sz.c));
  float area = warp_sum(ar.s + (-ar.c));
  if (lane == 0) {
    float curv = (area == 0.f) ? 1.0f : sqrtf(nx * nx + ny * ny + nz * nz) / area;
    nd_curv[node] = curv;
    if (!found) {
      nd_type[node] = T_EMPTY;
      float4 v = nd_v[node];
      v.w = a.iso;
      nd_v[node] = v;
    } else {
      nd_type[node] = a.big ? T_INTERNAL : T_UNCERTAIN;
    }
  }
}

struct SampleArgs {
  GridView g;
  PartView P;
  float iso;
  float radius;
  long long lb, le;
  int qef;
};

__global__ void k_sample(SampleArgs a, const float4* __restrict__ nd_c, float4* __restrict__ nd_v,
                         int8_t* __restrict__ nd_type, int8_t* __restrict__ nd_sc,
                         const float* __restrict__ nd_curv, float* __restrict__ nd_samp,
                         unsigned long long* __restrict__ counters) {
  const long long node = a.lb + (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (node >= a.le) return;
  if (nd_type[node] != T_UNCERTAIN) return;  // warp-uniform
  const float4 c = nd_c[node];
  const float h = c.w;
  float qx, qy, qz;
  if (lane < 27) {
    const int ix = lane % 3, iy = (lane / 3) % 3, iz = lane / 9;
    const float mn[3] = {__fsub_rn(c.x, h), __fsub_rn(c.y, h), __fsub_rn(c.z, h)};
    const float mx[3] = {__fadd_rn(c.x, h), __fadd_rn(c.y, h), __fadd_rn(c.z, h)};
    const float t[3] = {ix * 0.5f, iy * 0.5f, iz * 0.5f};
    qx = __fadd_rn(__fmul_rn(1.0f - t[0], mn[0]), __fmul_rn(t[0], mx[0]));
    qy = __fadd_rn(__fmul_rn(1.0f - t[1], mn[1]), __fmul_rn(t[1], mx[1]));
    qz = __fadd_rn(__fmul_rn(1.0f - t[2], mn[2]), __fmul_rn(t[2], mx[2]));
  } else {
    const float4 v = nd_v[node];
    qx = v.x, qy = v.y, qz = v.z;
  }
  long long pairs = 0;
  float val = 0.f;
  if (lane < 28) val = a.iso - field_sum(a.g, a.P, qx, qy, qz, &pairs);
  // GridEval sign change against sample 0, ">= 0" (src/evaluator.cpp:169-172)
  unsigned pos_mask = __ballot_sync(0xffffffffu, lane < 27 && val >= 0.f);
  bool origin = pos_mask & 1u;
  bool signchange = origin ? (pos_mask != 0x07ffffffu) : (pos_mask != 0u);
  float vc = __shfl_sync(0xffffffffu, val, 27);
  if (a.qef && lane < 27) nd_samp[node * 27 + lane] = val;
  // pair count for the kernel roofline
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) pairs += __shfl_xor_sync(0xffffffffu, pairs, o);
  if (lane == 0) {
    const float cellsize = 2.0f * h;
    const float curv = nd_curv[node];
    int8_t type;
    if ((double)(cellsize - a.radius) < 1e-8) {
      type = T_LEAF;
    } else if (signchange && (double)curv < 0.99) {
      type = T_INTERNAL;
    } else {
      type = T_LEAF;
    }
    nd_type[node] = type;
    nd_sc[node] = signchange ? 1 : 0;
    if (type == T_LEAF) {
      float4 v = nd_v[node];
      v.w = vc;
      nd_v[node] = v;
    }
    atomicAdd(counters + 0, (unsigned long long)(27 + (type == T_LEAF ? 1 : 0)));
    atomicAdd(counters + 1, (unsigned long long)pairs);
  }
}

__global__ void k_internal_flag(const int8_t* __restrict__ nd_type, long long lb, long long le,
                                int* __restrict__ flag) {
  long long i = lb + (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= le) return;
  flag[i - lb] = nd_type[i] == T_INTERNAL ? 1 : 0;
}

__global__ void k_spawn(long long lb, long long le, long long cbase, const int* __restrict__ rank,
                        const int8_t* __restrict__ nd_type, int child_depth, float4* __restrict__ nd_c,
                        float4* __restrict__ nd_v, uint64_t* __restrict__ nd_id, int* __restrict__ nd_parent,
                        int* __restrict__ nd_child, int8_t* __restrict__ nd_ctype,
                        int8_t* __restrict__ nd_depth, int8_t* __restrict__ nd_sc, float* __restrict__ nd_curv,
                        int4* __restrict__ nd_org) {
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

static void ensure_nodes(pi_frame* f, long long need) {
  if ((long long)f->nd_c.n >= need) return;
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
}

void stage_octree(pi_frame* f) {
  pi_ctx* ctx = f->ctx;
  cudaStream_t s = ctx->stream;
  if (f->dmax > 20) throw std::length_error("octree depth above 20");
  f->nNodes = 0;
  f->levelBegin.clear();
  ensure_nodes(f, 1 << 16);
  PI_LAUNCH(k_root, 1, 1, 0, s, f->rootC[0], f->rootC[1], f->rootC[2], f->rootH, 1 << f->dmax, f->nd_c.p,
            f->nd_v.p, f->nd_id.p, f->nd_parent.p, f->nd_child.p, f->nd_type.p, f->nd_depth.p, f->nd_sc.p,
            f->nd_curv.p, f->nd_org.p);
  f->nNodes = 1;
  const GridHost& gh = f->g;
  GridView g{gh.bounding[0], gh.bounding[2], gh.bounding[4], gh.cell, gh.nx, gh.ny, gh.nz, f->off.p};
  PartView P{f->pos.p, f->xm.p, f->ga.p, f->gb.p};
  f->dcount.alloc(ctx, s, 8);
  PI_CUDA(cudaMemsetAsync(f->dcount.p, 0, sizeof(unsigned long long) * 8, s));
  DBuf<int> flag;
  long long lb = 0, le = 1;
  for (int depth = 0;; ++depth) {
    f->levelBegin.push_back(lb);
    const long long nl = le - lb;
    LevelArgs la{g, gh.bounding[1], gh.bounding[3], gh.bounding[5], f->pos.p, f->nrm.p,
                 f->P.radius * f->P.smooth_factor, f->iso, lb, le, depth < f->dmin ? 1 : 0};
    const int wpb = 8;  // warps per block
    PI_LAUNCH(k_empty_curv, div_up(nl, wpb), 32 * wpb, 0, s, la, f->nd_c.p, f->nd_v.p, f->nd_type.p,
              f->nd_curv.p);
    if (depth >= f->dmin) {
      SampleArgs sa{g, P, f->iso, f->P.radius, lb, le, f->P.qef};
      prof_begin(ctx, s);
      PI_LAUNCH(k_sample, div_up(nl, wpb), 32 * wpb, 0, s, sa, f->nd_c.p, f->nd_v.p, f->nd_type.p, f->nd_sc.p,
                f->nd_curv.p, f->nd_samp.p, f->dcount.p);
      prof_end(ctx, s, -1, -1);
    }
    flag.alloc(ctx, s, nl + 1);
    if (f->tmp.n < scan_tmp_ints(nl + 1)) f->tmp.alloc(ctx, s, scan_tmp_ints(nl + 1));
    PI_LAUNCH(k_internal_flag, div_up(nl, 256), 256, 0, s, f->nd_type.p, lb, le, flag.p);
    PI_CUDA(cudaMemsetAsync(flag.p + nl, 0, sizeof(int), s));
    exclusive_scan_i32(flag.p, flag.p, nl + 1, nullptr, f->tmp.p, s);
    int nint = 0;
    PI_CUDA(cudaMemcpyAsync(&nint, flag.p + nl, sizeof(int), cudaMemcpyDeviceToHost, s));
    PI_CUDA(cudaStreamSynchronize(s));
    const long long newn = 8LL * nint;
    ensure_nodes(f, le + newn);
    PI_LAUNCH(k_spawn, div_up(nl, 256), 256, 0, s, lb, le, le, flag.p, f->nd_type.p, depth + 1, f->nd_c.p,
              f->nd_v.p, f->nd_id.p, f->nd_parent.p, f->nd_child.p, f->nd_type.p, f->nd_depth.p, f->nd_sc.p,
              f->nd_curv.p, f->nd_org.p);
    f->nNodes = le + newn;
    // depth D_max nodes are leaves by size, so nothing spawns past it
    if (nint == 0 || depth >= f->dmax) break;
    lb = le;
    le = le + newn;
  }
  unsigned long long cnt[2];
  PI_CUDA(cudaMemcpyAsync(cnt, f->dcount.p, sizeof(cnt), cudaMemcpyDeviceToHost, s));
  PI_CUDA(cudaStreamSynchronize(s));
  f->fieldEvals = (long long)cnt[0];
  f->pairs = (long long)cnt[1];
}

}  // namespace pisurf
