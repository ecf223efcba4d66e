// K3: anisotropic SPH field at points and particle normals.
//   - CalcParticlesNormal (src/evaluator.cpp:363-375): per particle the
//     poly6-gradient form sum_j det_j Sigma (-6 G_j d) (h^2 - |G_j d|^2)^2,
//     d = p_i - xmean_j (AnisotropicInterpolateGrad, :455-463, :408-415).
//   - SingleEval / SingleEvalWithGrad at arbitrary points (:60-125).
//   - HashGrid::GetPIdxList / GetInBoxParticles as device queries.
// The per-point field sum itself is field_sum() in device.cuh.
#include <vector>

#include "device.cuh"
#include "internal.h"

namespace pisurf {

// Gradient-form sum at q (without the -6 h^5 factor): sum_j wdet_j u (1 - s2)^2
// with u = A_j (q - xmean_j), s2 = |u|^2 < 1.
__device__ __forceinline__ void grad_sum(const GridView& g, const PartView& P, float qx, float qy, float qz,
                                         float& gx, float& gy, float& gz) {
  int cx, cy, cz;
  cell_of(g, qx, qy, qz, cx, cy, cz);
  Kahan ax, ay, az;
  for (int dz = -1; dz <= 1; ++dz)
    for (int dy = -1; dy <= 1; ++dy) {
      int s, e;
      if (!nb_row(g, cx, cy + dy, cz + dz, &s, &e)) continue;
      // 32 candidates at a time: the |d| < R / 2 test (|A d| < 1 needs it)
      // into a bit mask, then the terms of the set bits in candidate order
      for (int j0 = s; j0 < e; j0 += 32) {
        const int cnt = min(32, e - j0);
        unsigned m = 0u;
        for (int k = 0; k < cnt; ++k) {
          const float4 x = __ldg(P.xm + j0 + k);
          const float dx = qx - x.x, dyy = qy - x.y, dzz = qz - x.z;
          const float e2 = fmaf(dx, dx, fmaf(dyy, dyy, dzz * dzz));
          m |= (e2 < 0.25f * x.w ? 1u : 0u) << k;
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
          if (s2 < 1.0f) {
            const float om = 1.0f - s2;
            const float f = b.z * om * om;
            ax.add(u0 * f);
            ay.add(u1 * f);
            az.add(u2 * f);
          }
        }
      }
    }
  gx = ax.s;
  gy = ay.s;
  gz = az.s;
}

__global__ void __launch_bounds__(128, 12) k_normals(GridView g, PartView P, long long n, float gscale, float4* __restrict__ nrm) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  float4 p = P.pos[t];
  if (p.w != 0.f) {  // a splash particle's normal stays zero
    nrm[t] = make_float4(0.f, 0.f, 0.f, 0.f);
    return;
  }
  float gx, gy, gz;
  grad_sum(g, P, p.x, p.y, p.z, gx, gy, gz);
  gx *= gscale;
  gy *= gscale;
  gz *= gscale;
  nrm[t] = make_float4(gx, gy, gz, sqrtf(gx * gx + gy * gy + gz * gz));
}

__global__ void k_eval_points(GridView g, PartView P, const float* __restrict__ pts, long long m, float iso,
                              float gscale, float* __restrict__ val, float* __restrict__ grad) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  float qx = pts[3 * i], qy = pts[3 * i + 1], qz = pts[3 * i + 2];
  val[i] = iso - field_sum(g, P, qx, qy, qz, nullptr);
  if (grad) {
    float gx, gy, gz;
    grad_sum(g, P, qx, qy, qz, gx, gy, gz);
    grad[3 * i] = gx * gscale;
    grad[3 * i + 1] = gy * gscale;
    grad[3 * i + 2] = gz * gscale;
  }
}

static GridView gview(pi_frame* f) {
  const GridHost& gh = f->g;
  return GridView{gh.bounding[0], gh.bounding[2], gh.bounding[4], gh.cell, gh.nx, gh.ny, gh.nz, f->off.p};
}
static PartView pview(pi_frame* f) { return PartView{f->pos.p, f->xm.p, f->ga.p, f->gb.p, f->xlo.p}; }

// -6 h^5 with h = 2r (see AnisotropicInterpolateGrad in A = G / h units)
static float grad_scale(pi_frame* f) {
  double h = 2.0 * (double)f->P.radius;
  return (float)(-6.0 * h * h * h * h * h);
}

// ---- variable radius: the bins' candidate lists, per-particle scales ----

// Gradient-form sum with each term scaled by its particle's -6 h_j^5 (gb.w).
__device__ __forceinline__ void grad_sum_vr(const MultiGridView& m, const PartView& P, float qx, float qy, float qz,
                                            float& gx, float& gy, float& gz) {
  Kahan ax, ay, az;
  for (int b = 0; b < m.nb; ++b) {
    const BinGrid g = m.g[b];
    const int cx = cell_coord(qx, g.b0, g.cell, g.nx), cy = cell_coord(qy, g.b2, g.cell, g.ny),
              cz = cell_coord(qz, g.b4, g.cell, g.nz);
    for (int dz = -1; dz <= 1; ++dz)
      for (int dy = -1; dy <= 1; ++dy) {
        int s, e;
        if (!bin_row(g, m.off, cx, cy + dy, cz + dz, &s, &e)) continue;
        for (int j = s; j < e; ++j) {
          const float4 x = __ldg(P.xm + j);
          const float dx = qx - x.x, dyy = qy - x.y, dzz = qz - x.z;
          if (!(fmaf(dx, dx, fmaf(dyy, dyy, dzz * dzz)) < 0.25f * x.w)) continue;
          const float4 a = __ldg(P.ga + j);
          const float4 bb = __ldg(P.gb + j);
          const float4 lo = __ldg(P.xlo + j);
          float u0, u1, u2;
          amul(a, bb, dx - lo.x, dyy - lo.y, dzz - lo.z, u0, u1, u2);
          const float s2 = fmaf(u0, u0, fmaf(u1, u1, u2 * u2));
          if (s2 < 1.0f) {
            const float om = 1.0f - s2;
            const float fct = bb.z * om * om * bb.w;
            ax.add(u0 * fct);
            ay.add(u1 * fct);
            az.add(u2 * fct);
          }
        }
      }
  }
  gx = ax.s;
  gy = ay.s;
  gz = az.s;
}

__global__ void __launch_bounds__(128) k_vr_normals(const MultiGridView* __restrict__ mg, PartView P, long long n,
                                                    float4* __restrict__ nrm) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const float4 p = P.pos[t];
  float gx, gy, gz;
  grad_sum_vr(*mg, P, p.x, p.y, p.z, gx, gy, gz);
  nrm[t] = make_float4(gx, gy, gz, sqrtf(gx * gx + gy * gy + gz * gz));
}

__global__ void k_vr_eval_points(const MultiGridView* __restrict__ mg, PartView P, const float* __restrict__ pts,
                                 long long m, float iso, float* __restrict__ val, float* __restrict__ grad) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  const float qx = pts[3 * i], qy = pts[3 * i + 1], qz = pts[3 * i + 2];
  val[i] = iso - field_sum_vr(*mg, P, qx, qy, qz, nullptr);
  if (grad) grad_sum_vr(*mg, P, qx, qy, qz, grad[3 * i], grad[3 * i + 1], grad[3 * i + 2]);
}

__global__ void k_vr_nb_count(const MultiGridView* __restrict__ mg, const float* __restrict__ pts, long long m,
                              int* __restrict__ cnt) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  const MultiGridView& v = *mg;
  int c = 0;
  for (int b = 0; b < v.nb; ++b) {
    const BinGrid g = v.g[b];
    const int cx = cell_coord(pts[3 * i], g.b0, g.cell, g.nx), cy = cell_coord(pts[3 * i + 1], g.b2, g.cell, g.ny),
              cz = cell_coord(pts[3 * i + 2], g.b4, g.cell, g.nz);
    for (int dz = -1; dz <= 1; ++dz)
      for (int dy = -1; dy <= 1; ++dy) {
        int s, e;
        if (bin_row(g, v.off, cx, cy + dy, cz + dz, &s, &e)) c += e - s;
      }
  }
  cnt[i] = c;
}

__global__ void k_vr_nb_fill(const MultiGridView* __restrict__ mg, const float* __restrict__ pts, long long m,
                             const int* __restrict__ off, const uint32_t* __restrict__ sidx, int* __restrict__ out) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  const MultiGridView& v = *mg;
  int o = off[i];
  for (int b = 0; b < v.nb; ++b) {
    const BinGrid g = v.g[b];
    const int cx = cell_coord(pts[3 * i], g.b0, g.cell, g.nx), cy = cell_coord(pts[3 * i + 1], g.b2, g.cell, g.ny),
              cz = cell_coord(pts[3 * i + 2], g.b4, g.cell, g.nz);
    for (int dz = -1; dz <= 1; ++dz)
      for (int dy = -1; dy <= 1; ++dy) {
        int s, e;
        if (!bin_row(g, v.off, cx, cy + dy, cz + dz, &s, &e)) continue;
        for (int j = s; j < e; ++j) out[o++] = (int)sidx[j];
      }
  }
}

void stage_normals(pi_frame* f) {
  cudaStream_t s = f->ctx->stream;
  if (f->varR) {
    PI_LAUNCH(k_vr_normals, div_up(f->N, 128), 128, 0, s, f->mgv.p, pview(f), f->N, f->nrm.p);
    return;
  }
  PI_LAUNCH(k_normals, div_up(f->N, 128), 128, 0, s, gview(f), pview(f), f->N, grad_scale(f), f->nrm.p);
}

void eval_points(pi_frame* f, const float* d_pts, long long m, float* d_val, float* d_grad) {
  cudaStream_t s = f->ctx->stream;
  if (f->varR) {
    PI_LAUNCH(k_vr_eval_points, div_up(m, 128), 128, 0, s, f->mgv.p, pview(f), d_pts, m, f->iso, d_val, d_grad);
    return;
  }
  PI_LAUNCH(k_eval_points, div_up(m, 128), 128, 0, s, gview(f), pview(f), d_pts, m, f->iso, grad_scale(f),
            d_val, d_grad);
}

// GetPIdxList: counts, then lists (particle indices through IndexList).
__global__ void k_nb_count(GridView g, const float* __restrict__ pts, long long m, int* __restrict__ cnt) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  int cx, cy, cz;
  cell_of(g, pts[3 * i], pts[3 * i + 1], pts[3 * i + 2], cx, cy, cz);
  int c = 0;
  for (int dz = -1; dz <= 1; ++dz)
    for (int dy = -1; dy <= 1; ++dy) {
      int s, e;
      if (nb_row(g, cx, cy + dy, cz + dz, &s, &e)) c += e - s;
    }
  cnt[i] = c;
}

__global__ void k_nb_fill(GridView g, const float* __restrict__ pts, long long m, const int* __restrict__ off,
                          const uint32_t* __restrict__ sidx, int* __restrict__ out) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  int cx, cy, cz;
  cell_of(g, pts[3 * i], pts[3 * i + 1], pts[3 * i + 2], cx, cy, cz);
  int o = off[i];
  for (int dz = -1; dz <= 1; ++dz)
    for (int dy = -1; dy <= 1; ++dy) {
      int s, e;
      if (!nb_row(g, cx, cy + dy, cz + dz, &s, &e)) continue;
      for (int j = s; j < e; ++j) out[o++] = (int)sidx[j];
    }
}

long long neighbors(pi_frame* f, const float* h_pts, long long m, long long* h_off, int* h_idx, long long cap) {
  cudaStream_t s = f->ctx->stream;
  DBuf<float> pts;
  DBuf<int> cnt, tmp;
  pts.alloc(f->ctx, s, m * 3);
  cnt.alloc(f->ctx, s, m + 1);
  tmp.alloc(f->ctx, s, scan_tmp_ints(m + 1));
  PI_CUDA(cudaMemcpyAsync(pts.p, h_pts, sizeof(float) * 3 * m, cudaMemcpyHostToDevice, s));
  GridView g = gview(f);
  PI_CUDA(cudaMemsetAsync(cnt.p, 0, sizeof(int) * (m + 1), s));
  if (f->varR)
    PI_LAUNCH(k_vr_nb_count, div_up(m, 128), 128, 0, s, f->mgv.p, pts.p, m, cnt.p);
  else
    PI_LAUNCH(k_nb_count, div_up(m, 128), 128, 0, s, g, pts.p, m, cnt.p);
  int total = 0;
  exclusive_scan_i32(cnt.p, cnt.p, m + 1, nullptr, tmp.p, s);
  PI_CUDA(cudaMemcpyAsync(&total, cnt.p + m, sizeof(int), cudaMemcpyDeviceToHost, s));
  PI_CUDA(cudaStreamSynchronize(s));
  std::vector<int> offs(m + 1);
  PI_CUDA(cudaMemcpy(offs.data(), cnt.p, sizeof(int) * (m + 1), cudaMemcpyDeviceToHost));
  for (long long i = 0; i <= m; ++i) h_off[i] = offs[i];
  if (total > cap) return total;
  DBuf<int> out;
  out.alloc(f->ctx, s, total > 0 ? total : 1);
  if (f->varR)
    PI_LAUNCH(k_vr_nb_fill, div_up(m, 128), 128, 0, s, f->mgv.p, pts.p, m, cnt.p, f->sidx.p, out.p);
  else
    PI_LAUNCH(k_nb_fill, div_up(m, 128), 128, 0, s, g, pts.p, m, cnt.p, f->sidx.p, out.p);
  PI_CUDA(cudaMemcpyAsync(h_idx, out.p, sizeof(int) * total, cudaMemcpyDeviceToHost, s));
  PI_CUDA(cudaStreamSynchronize(s));
  return total;
}

// GetInBoxParticles (src/hash_grid.cpp:164-194): x outer, z inner, one
// thread walks the cell block (a query, not a hot path).
__global__ void k_in_box(GridView g, float b1x, float b1y, float b1z, float b2x, float b2y, float b2z,
                         float B1, float B3, float B5, const uint32_t* __restrict__ sidx, int* __restrict__ out,
                         long long cap, long long* __restrict__ total) {
  b1x = fmaxf(b1x, g.b0);
  b1y = fmaxf(b1y, g.b2);
  b1z = fmaxf(b1z, g.b4);
  b2x = fminf(b2x, B1);
  b2y = fminf(b2y, B3);
  b2z = fminf(b2z, B5);
  int mnx, mny, mnz, mxx, mxy, mxz;
  cell_of(g, b1x, b1y, b1z, mnx, mny, mnz);
  cell_of(g, b2x, b2y, b2z, mxx, mxy, mxz);
  long long k = 0;
  for (int x = mnx - 1; x <= mxx + 1; ++x)
    for (int y = mny - 1; y <= mxy + 1; ++y)
      for (int z = mnz - 1; z <= mxz + 1; ++z) {
        if (x < 0 || x >= g.nx || y < 0 || y >= g.ny || z < 0 || z >= g.nz) continue;
        long long c = ((long long)z * g.ny + y) * g.nx + x;
        for (int j = g.off[c]; j < g.off[c + 1]; ++j) {
          if (k < cap) out[k] = (int)sidx[j];
          ++k;
        }
      }
  *total = k;
}

long long in_box(pi_frame* f, const float* b1, const float* b2, int* h_idx, long long cap) {
  cudaStream_t s = f->ctx->stream;
  DBuf<int> out;
  DBuf<long long> tot;
  out.alloc(f->ctx, s, cap > 0 ? cap : 1);
  tot.alloc(f->ctx, s, 1);
  const GridHost& gh = f->g;
  PI_LAUNCH(k_in_box, 1, 1, 0, s, gview(f), b1[0], b1[1], b1[2], b2[0], b2[1], b2[2], gh.bounding[1],
            gh.bounding[3], gh.bounding[5], f->sidx.p, out.p, cap, tot.p);
  long long total = 0;
  PI_CUDA(cudaMemcpyAsync(&total, tot.p, sizeof(long long), cudaMemcpyDeviceToHost, s));
  PI_CUDA(cudaStreamSynchronize(s));
  if (total <= cap && total > 0)
    PI_CUDA(cudaMemcpy(h_idx, out.p, sizeof(int) * total, cudaMemcpyDeviceToHost));
  return total;
}

}  // namespace pisurf
