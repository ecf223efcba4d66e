// Splash particles (pi_params.splash): the reference's GlobalSplash with its
// marking switched on (src/evaluator.cpp:675,690) and GEN_SPLASH on.
//
//   - k_xmean marks a particle with <= 2 candidates or <= 2 neighbours within
//     4r (aniso.cu); k_cov_G gives it the identity G and a negative cull
//     radius, so no field sum, normal or grid sample counts it.
//   - stage_splash_list sets pos.w = 1 for it, so that node emptiness and
//     curvature skip it (checkEmptyAndCalcCurv, src/surface_reconstructor.cpp:
//     171-214) and its normal stays zero (CalcParticlesNormal, :363-375), and
//     lists the splash particles in particle order.
//   - splash_mesh appends one icosahedron per splash particle after the
//     surface mesh (Mesh::AppendSplash_ConstR, src/global.cpp:94-115): 12
//     vertices pos + T[i] * r and 20 triangles, in particle order.
#include <cmath>

#include "device.cuh"
#include "internal.h"

namespace pisurf {

// Flag in particle order (for the scan) and pos.w = 1 for splash particles.
__global__ void k_splash_mark(const int8_t* __restrict__ spl, const uint32_t* __restrict__ sidx, long long n,
                              float4* __restrict__ pos, int* __restrict__ flag) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const int s = spl[t];
  flag[sidx[t]] = s;
  if (s) pos[t].w = 1.0f;
}

// list[rank of the particle among the splash particles] = its sorted position.
__global__ void k_splash_list(const int8_t* __restrict__ spl, const uint32_t* __restrict__ sidx, long long n,
                              const int* __restrict__ rank, int* __restrict__ list) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  if (spl[t]) list[rank[sidx[t]]] = (int)t;
}

void stage_splash_list(pi_frame* f) {
  pi_ctx* c = f->ctx;
  cudaStream_t s = c->stream;
  const long long n = f->N;
  DBuf<int> flag, tmp;
  flag.alloc(c, s, n + 1);
  tmp.alloc(c, s, scan_tmp_ints(n + 1));
  PI_CUDA(cudaMemsetAsync(flag.p + n, 0, sizeof(int), s));
  PI_LAUNCH(k_splash_mark, div_up(n, 256), 256, 0, s, f->spl.p, f->sidx.p, n, f->pos.p, flag.p);
  exclusive_scan_i32(flag.p, flag.p, n + 1, nullptr, tmp.p, s);
  int total = 0;
  PI_CUDA(cudaMemcpyAsync(&total, flag.p + n, sizeof(int), cudaMemcpyDeviceToHost, s));
  PI_CUDA(cudaStreamSynchronize(s));
  f->nSplash = total;
  f->splList.alloc(c, s, total > 0 ? total : 1);
  PI_LAUNCH(k_splash_list, div_up(n, 256), 256, 0, s, f->spl.p, f->sidx.p, n, flag.p, f->splList.p);
}

// Mesh::BuildIcosaTable (src/global.cpp:65-92): the 12 unit vertices of the
// icosahedron, computed in float as the reference computes them: the
// north pole, two rings of five at elevation +-atan(1/2) with longitudes
// from -126 and -90 degrees in steps of 72, the south pole.
struct IcosaTable {
  float v[12][3];
};

static IcosaTable icosa_table() {
  IcosaTable t{};
  const float pi = 3.1415926f;
  const float step = pi / 180 * 72;
  const float elev = std::atan(1.0f / 2);
  float lon1 = -pi / 2 - step / 2, lon2 = -pi / 2;
  t.v[0][0] = 0.f, t.v[0][1] = 0.f, t.v[0][2] = 1.f;
  for (int i = 1; i <= 5; ++i) {
    const float z = std::sin(elev), xy = std::cos(elev);
    t.v[i][0] = xy * std::cos(lon1), t.v[i][1] = xy * std::sin(lon1), t.v[i][2] = z;
    t.v[i + 5][0] = xy * std::cos(lon2), t.v[i + 5][1] = xy * std::sin(lon2), t.v[i + 5][2] = -z;
    lon1 += step;
    lon2 += step;
  }
  t.v[11][0] = 0.f, t.v[11][1] = 0.f, t.v[11][2] = -1.f;
  return t;
}

// One thread per splash particle: its 12 vertices at v0 + 12 k and 20
// triangles at t0 + 20 k (0-based), in the insert order of
// AppendSplash_ConstR; vertex keys (12 p + i, all ones) for particle p.
__global__ void k_splash_mesh(IcosaTable T, long long ns, const int* __restrict__ list,
                              const float4* __restrict__ pos, const uint32_t* __restrict__ sidx, float r,
                              long long v0, long long t0, float* __restrict__ mv, uint64_t* __restrict__ mk,
                              int* __restrict__ mt) {
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= ns) return;
  const int t = list[k];
  const float4 p = pos[t];
  const uint64_t pid = sidx[t];
  const long long vb = v0 + 12 * k;
  for (int i = 0; i < 12; ++i) {
    mv[3 * (vb + i)] = __fadd_rn(p.x, __fmul_rn(T.v[i][0], r));
    mv[3 * (vb + i) + 1] = __fadd_rn(p.y, __fmul_rn(T.v[i][1], r));
    mv[3 * (vb + i) + 2] = __fadd_rn(p.z, __fmul_rn(T.v[i][2], r));
    mk[2 * (vb + i)] = 12 * pid + i;
    mk[2 * (vb + i) + 1] = ~0ull;
  }
  int* o = mt + 3 * (t0 + 20 * k);
  const int b = (int)vb;
  for (int i = 0; i < 5; ++i) {
    const int u = 1 + i, w = (1 + i) % 5 + 1;
    const int tri[4][3] = {{0, u, w}, {u, w, 6 + i}, {w, 6 + i, (1 + i) % 5 + 6}, {6 + i, (1 + i) % 5 + 6, 11}};
    for (int q = 0; q < 4; ++q)
      for (int c = 0; c < 3; ++c) o[3 * (4 * i + q) + c] = b + tri[q][c];
  }
}

void splash_mesh(pi_frame* f, long long v0, long long t0) {
  if (f->nSplash <= 0) return;
  const IcosaTable T = icosa_table();
  PI_LAUNCH(k_splash_mesh, div_up(f->nSplash, 128), 128, 0, f->ctx->stream, T, f->nSplash, f->splList.p, f->pos.p,
            f->sidx.p, f->P.radius, v0, t0, f->mv.p, f->mk.p, f->mt.p);
}

}  // namespace pisurf
