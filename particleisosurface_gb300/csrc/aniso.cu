// K2: per-particle anisotropy, Evaluator::compute_Gs_xMeans
// (src/evaluator.cpp:656-749): pass 1 smoothed centres (compute_xMeans,
// :465-512), pass 2 weighted covariance of neighbour centres and its
// eigen-decomposition into the anisotropy matrix G (compute_G_Yus, :585-654).
//
// One thread per particle in cell order, so a warp's particles share most of
// their 27-cell candidates and the candidate loads hit L1.  Distances that
// decide neighbour membership (d^2 < (4r)^2) are rounded exactly as the
// reference rounds them (no fused multiply-add, x0 + (x1 + x2) order), so the
// neighbour sets match; the sums are compensated FP32.
//
// The covariance is symmetric positive definite (Influnce2 * I is added), so
// the reference's JacobiSVD has U = V and G = V diag(s / w) V^T is a spectral
// function of the covariance: any accurate symmetric eigensolver gives the same
// G.  The solver is cyclic Jacobi in FP32; when the neighbourhood is
// near-degenerate (smallest eigenvalue below a quarter of the largest, i.e.
// sheet- or filament-like, where the reference clamps) the decomposition is
// redone in FP64.
#include <cmath>

#include "device.cuh"
#include "internal.h"

namespace pisurf {

// wij (src/evaluator.cpp:751-766) in FP32; inv_h3 = 1 / h^3.
__device__ __forceinline__ float wij_f(float d, float h, float inv_h3) {
  if (d < h) {
    float hd = h - d;
    if (d < h * 0.5f) return 1.0f - 6.0f * d * d * inv_h3 * hd;
    return 2.0f * inv_h3 * hd * hd * hd;
  }
  return 0.0f;
}

// Squared distance rounded as the reference rounds it.
__device__ __forceinline__ float d2_exact(float dx, float dy, float dz) {
  return __fadd_rn(__fmul_rn(dx, dx), __fadd_rn(__fmul_rn(dy, dy), __fmul_rn(dz, dz)));
}

// The smoothed centre x = (1 - delta) p + delta m, m = sum w p_j / sum w, is
// formed as x = p + delta * sum w (p_j - p) / sum w: the offsets are small, so
// the centre is kept as a float pair hi + lo with hi = fl(x) and lo the rest.
// Coordinates of order 1 against r = 0.01 would otherwise lose ~1e-5 r to the
// float rounding of x alone.  (c_self + c_mean == 1 exactly in float.)
//
// Splash particles (spl not null): a particle with <= 2 candidates or <= 2
// neighbours within 4r (the GlobalSplash marking of src/evaluator.cpp:675,690
// switched on) gets spl = 1.
__global__ void k_xmean(GridView g, const float4* __restrict__ pos, long long n, float nI, float nI2,
                        float inv_h3, float c_mean, float4* __restrict__ xm, float4* __restrict__ xlo,
                        int8_t* __restrict__ spl) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  float4 p = pos[t];
  int cx, cy, cz;
  cell_of(g, p.x, p.y, p.z, cx, cy, cz);
  long long cand = 0;
  int nn = 0;  // neighbours within 4r (compute_xMeans' neighbors.size())
  Kahan ws, sx, sy, sz;
  for (int dz = -1; dz <= 1; ++dz)
    for (int dy = -1; dy <= 1; ++dy) {
      int s, e;
      if (!nb_row(g, cx, cy + dy, cz + dz, &s, &e)) continue;
      cand += e - s;
      // 32 candidates at a time: the distance test into a bit mask, then
      // the weights of the set bits in candidate order
      for (int j0 = s; j0 < e; j0 += 32) {
        const int cnt = min(32, e - j0);
        unsigned m = 0u;
        for (int k = 0; k < cnt; ++k) {
          const float4 q = __ldg(pos + j0 + k);
          const float dx = __fsub_rn(q.x, p.x), dy2 = __fsub_rn(q.y, p.y), dz2 = __fsub_rn(q.z, p.z);
          m |= (d2_exact(dx, dy2, dz2) < nI2 && j0 + k != t ? 1u : 0u) << k;
        }
        nn += __popc(m);
        while (m) {
          const int j = j0 + __ffs(m) - 1;
          m &= m - 1u;
          const float4 q = __ldg(pos + j);
          const float dx = __fsub_rn(q.x, p.x), dy2 = __fsub_rn(q.y, p.y), dz2 = __fsub_rn(q.z, p.z);
          const float w = wij_f(__fsqrt_rn(d2_exact(dx, dy2, dz2)), nI, inv_h3);
          ws.add(w);
          sx.add(dx * w);
          sy.add(dy2 * w);
          sz.add(dz2 * w);
        }
      }
    }
  float4 hi = make_float4(p.x, p.y, p.z, 0.f), lo = make_float4(0.f, 0.f, 0.f, 0.f);
  if (cand > 2 && ws.s > 0.f) {
    const float ox = c_mean * ((sx.s - sx.c) / ws.s), oy = c_mean * ((sy.s - sy.c) / ws.s),
                oz = c_mean * ((sz.s - sz.c) / ws.s);
    hi.x = __fadd_rn(p.x, ox);
    hi.y = __fadd_rn(p.y, oy);
    hi.z = __fadd_rn(p.z, oz);
    lo.x = __fadd_rn(__fsub_rn(p.x, hi.x), ox);
    lo.y = __fadd_rn(__fsub_rn(p.y, hi.y), oy);
    lo.z = __fadd_rn(__fsub_rn(p.z, hi.z), oz);
  }
  xm[t] = hi;
  xlo[t] = lo;
  if (spl) spl[t] = (cand <= 2 || nn <= 2) ? 1 : 0;
}

// Cyclic Jacobi on a symmetric 3x3 (a: 00 01 02 11 12 22).  On return
// w = eigenvalues, V columns = eigenvectors.
template <class T>
__device__ __forceinline__ void sym_eig3(const T a6[6], T w[3], T V[3][3]) {
  T A[3][3] = {{a6[0], a6[1], a6[2]}, {a6[1], a6[3], a6[4]}, {a6[2], a6[4], a6[5]}};
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) V[i][j] = (i == j) ? T(1) : T(0);
  const T eps = sizeof(T) == 4 ? T(1e-7) : T(1e-16);
  for (int sweep = 0; sweep < 12; ++sweep) {
    T off = fabs(A[0][1]) + fabs(A[0][2]) + fabs(A[1][2]);
    T dia = fabs(A[0][0]) + fabs(A[1][1]) + fabs(A[2][2]);
    if (off <= eps * dia) break;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const int p = k == 2 ? 1 : 0;
      const int q = k == 0 ? 1 : 2;
      T apq = A[p][q];
      if (fabs(apq) <= eps * T(1e-3) * dia) continue;
      T theta = (A[q][q] - A[p][p]) / (T(2) * apq);
      T tt = T(1) / (fabs(theta) + sqrt(theta * theta + T(1)));
      if (theta < T(0)) tt = -tt;
      T c = T(1) / sqrt(tt * tt + T(1));
      T s = tt * c;
      // A' = J^T A J on rows/cols p, q
      for (int r = 0; r < 3; ++r) {
        T arp = A[r][p], arq = A[r][q];
        A[r][p] = c * arp - s * arq;
        A[r][q] = s * arp + c * arq;
      }
      for (int r = 0; r < 3; ++r) {
        T apr = A[p][r], aqr = A[q][r];
        A[p][r] = c * apr - s * aqr;
        A[q][r] = s * apr + c * aqr;
      }
      for (int r = 0; r < 3; ++r) {
        T vrp = V[r][p], vrq = V[r][q];
        V[r][p] = c * vrp - s * vrq;
        V[r][q] = s * vrp + c * vrq;
      }
    }
  }
  w[0] = A[0][0];
  w[1] = A[1][1];
  w[2] = A[2][2];
}

// G = V diag(scale / w) V^T with the reference's clamp w >= max(w) / 4 and
// volume-preserving scale = cbrt(w0 w1 w2) (src/evaluator.cpp:627-651).
// Returns G (row-major 9) and max(w) / scale for the support radius.
template <class T>
__device__ __forceinline__ void g_from_eig(const T w_in[3], const T V[3][3], float G[9], float* stretch) {
  T w[3] = {fabs(w_in[0]), fabs(w_in[1]), fabs(w_in[2])};
  T wmax = fmax(w[0], fmax(w[1], w[2]));
  for (int k = 0; k < 3; ++k) w[k] = fmax(w[k], wmax / T(4));
  T scale = cbrt(w[0] * w[1] * w[2]);
  T d[3] = {scale / w[0], scale / w[1], scale / w[2]};
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      G[3 * i + j] = (float)(V[i][0] * d[0] * V[j][0] + V[i][1] * d[1] * V[j][1] + V[i][2] * d[2] * V[j][2]);
  *stretch = (float)(wmax / scale);
}

__global__ void __launch_bounds__(128, 8) k_cov_G(GridView g, const float4* __restrict__ pos, const float4* __restrict__ xm0,
                        const float4* __restrict__ xlo, float4* __restrict__ xm, long long n,
                        float nI, float nI2, float inv_h3, float h2, float inv_h, float sigma,
                        float4* __restrict__ ga, float4* __restrict__ gb, float* __restrict__ gfull,
                        float* __restrict__ det_out, int8_t* __restrict__ f64flag,
                        unsigned long long* __restrict__ f64count, const int8_t* __restrict__ spl) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  float4 p = pos[t];
  float4 xp = xm0[t];
  const float4 lp = xlo[t];
  if (spl && spl[t]) {
    // a splash particle keeps pass 1's identity G (pass 2 skips it,
    // src/evaluator.cpp:723-726) and takes part in no field sum: its cull
    // radius is negative, so no support test passes
    xm[t] = make_float4(xp.x, xp.y, xp.z, -1.0f);
    ga[t] = make_float4(inv_h, 0.f, 0.f, inv_h);
    gb[t] = make_float4(0.f, inv_h, sigma, 0.f);
    for (int k = 0; k < 9; ++k) gfull[9 * t + k] = (k % 4 == 0) ? 1.0f : 0.0f;
    det_out[t] = 1.0f;
    f64flag[t] = 0;
    return;
  }
  int cx, cy, cz;
  cell_of(g, p.x, p.y, p.z, cx, cy, cz);
  Kahan ws, c00, c01, c02, c11, c12, c22;
  for (int dz = -1; dz <= 1; ++dz)
    for (int dy = -1; dy <= 1; ++dy) {
      int s, e;
      if (!nb_row(g, cx, cy + dy, cz + dz, &s, &e)) continue;
      // 32 candidates at a time: the distance test into a bit mask, then
      // the weighted products of the set bits in candidate order
      for (int j0 = s; j0 < e; j0 += 32) {
        const int cnt = min(32, e - j0);
        unsigned m = 0u;
        for (int k = 0; k < cnt; ++k) {
          const float4 q = __ldg(xm0 + j0 + k);
          const float4 lq = __ldg(xlo + j0 + k);
          // centre difference from the hi parts (exact for nearby centres) plus the lo parts
          const float dx = __fadd_rn(__fsub_rn(q.x, xp.x), __fsub_rn(lq.x, lp.x));
          const float dy2 = __fadd_rn(__fsub_rn(q.y, xp.y), __fsub_rn(lq.y, lp.y));
          const float dz2 = __fadd_rn(__fsub_rn(q.z, xp.z), __fsub_rn(lq.z, lp.z));
          m |= (d2_exact(dx, dy2, dz2) < nI2 ? 1u : 0u) << k;
        }
        while (m) {
          const int j = j0 + __ffs(m) - 1;
          m &= m - 1u;
          const float4 q = __ldg(xm0 + j);
          const float4 lq = __ldg(xlo + j);
          const float dx = __fadd_rn(__fsub_rn(q.x, xp.x), __fsub_rn(lq.x, lp.x));
          const float dy2 = __fadd_rn(__fsub_rn(q.y, xp.y), __fsub_rn(lq.y, lp.y));
          const float dz2 = __fadd_rn(__fsub_rn(q.z, xp.z), __fsub_rn(lq.z, lp.z));
          const float w = wij_f(__fsqrt_rn(d2_exact(dx, dy2, dz2)), nI, inv_h3);
          ws.add(w);
          c00.add(dx * dx * w);
          c01.add(dx * dy2 * w);
          c02.add(dx * dz2 * w);
          c11.add(dy2 * dy2 * w);
          c12.add(dy2 * dz2 * w);
          c22.add(dz2 * dz2 * w);
        }
      }
    }
  float iw = 1.0f / ws.s;
  float a6[6] = {(h2 + c00.s) * iw, c01.s * iw, c02.s * iw, (h2 + c11.s) * iw, c12.s * iw, (h2 + c22.s) * iw};
  float w[3], V[3][3];
  float G[9], stretch;
  bool degenerate = false;
  if (!(ws.s > 0.f)) {
    // no candidate within 4r: the reference divides by zero here (its G is
    // NaN); the identity is used, as for particles with <= 2 candidates
    for (int k = 0; k < 9; ++k) G[k] = (k % 4 == 0) ? 1.0f : 0.0f;
    stretch = 1.0f;
  } else {
    sym_eig3<float>(a6, w, V);
    float aw0 = fabsf(w[0]), aw1 = fabsf(w[1]), aw2 = fabsf(w[2]);
    float wmx = fmaxf(aw0, fmaxf(aw1, aw2)), wmn = fminf(aw0, fminf(aw1, aw2));
    degenerate = wmn < 0.25f * wmx;
    if (degenerate) {
      double a6d[6], wd[3], Vd[3][3];
      for (int k = 0; k < 6; ++k) a6d[k] = (double)a6[k];
      sym_eig3<double>(a6d, wd, Vd);
      g_from_eig<double>(wd, Vd, G, &stretch);
      stripe_add(f64count, 0, 1ull);
    } else {
      g_from_eig<float>(w, V, G, &stretch);
    }
  }
  // Matrix3f::determinant, cofactors along the first row
  float det = G[0] * (G[4] * G[8] - G[5] * G[7]) - G[1] * (G[3] * G[8] - G[5] * G[6]) +
              G[2] * (G[3] * G[7] - G[4] * G[6]);
  // support of the B-spline: |A d| < 2 needs |d| < 2 h max(w) / scale
  float R = 2.0f * stretch / inv_h;
  xm[t] = make_float4(xp.x, xp.y, xp.z, R * R * 1.002f);
  ga[t] = make_float4(G[0] * inv_h, G[1] * inv_h, G[2] * inv_h, G[4] * inv_h);
  gb[t] = make_float4(G[5] * inv_h, G[8] * inv_h, det * sigma, 0.f);
  for (int k = 0; k < 9; ++k) gfull[9 * t + k] = G[k];
  det_out[t] = det;
  f64flag[t] = degenerate ? 1 : 0;
}

// ---------------------------------------------------------------------------
// Variable radius (compute_xMeans / compute_G_Yus with per-particle radii,
// src/evaluator.cpp:465-512, 585-654): a neighbour j counts within its own
// neighbour radius nI_j = 4 r_j with weight wij(d, nI_j); the covariance
// starts from the particle's own Influnce2 = (2 r_i)^2; A = G / (2 r_i) and
// det * Sigma_i per particle.  The radius rides in pos.w.  Candidates are the
// bins' 27-cell lists in bin order.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(128) k_vr_xmean(const MultiGridView* __restrict__ mg,
                                                  const float4* __restrict__ pos, const float4* __restrict__ vrc,
                                                  long long n, float c_mean, float4* __restrict__ xm,
                                                  float4* __restrict__ xlo) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const MultiGridView& m = *mg;
  const float4 p = pos[t];
  long long cand = 0;
  Kahan ws, sx, sy, sz;
  for (int b = 0; b < m.nb; ++b) {
    const BinGrid g = m.g[b];
    const int cx = cell_coord(p.x, g.b0, g.cell, g.nx), cy = cell_coord(p.y, g.b2, g.cell, g.ny),
              cz = cell_coord(p.z, g.b4, g.cell, g.nz);
    for (int dz = -1; dz <= 1; ++dz)
      for (int dy = -1; dy <= 1; ++dy) {
        int s, e;
        if (!bin_row(g, m.off, cx, cy + dy, cz + dz, &s, &e)) continue;
        cand += e - s;
        for (int j = s; j < e; ++j) {
          if (j == t) continue;
          const float4 q = __ldg(pos + j);
          const float4 cj = __ldg(vrc + j);  // (Influnce2, Sigma, nI, 1 / nI^3) of the neighbour
          const float dx = __fsub_rn(q.x, p.x), dy2 = __fsub_rn(q.y, p.y), dz2 = __fsub_rn(q.z, p.z);
          const float d2 = d2_exact(dx, dy2, dz2);
          if (!(d2 < __fmul_rn(cj.z, cj.z))) continue;
          const float w = wij_f(__fsqrt_rn(d2), cj.z, cj.w);
          ws.add(w);
          sx.add(dx * w);
          sy.add(dy2 * w);
          sz.add(dz2 * w);
        }
      }
  }
  float4 hi = make_float4(p.x, p.y, p.z, 0.f), lo = make_float4(0.f, 0.f, 0.f, 0.f);
  if (cand > 2 && ws.s > 0.f) {
    const float ox = c_mean * ((sx.s - sx.c) / ws.s), oy = c_mean * ((sy.s - sy.c) / ws.s),
                oz = c_mean * ((sz.s - sz.c) / ws.s);
    hi.x = __fadd_rn(p.x, ox);
    hi.y = __fadd_rn(p.y, oy);
    hi.z = __fadd_rn(p.z, oz);
    lo.x = __fadd_rn(__fsub_rn(p.x, hi.x), ox);
    lo.y = __fadd_rn(__fsub_rn(p.y, hi.y), oy);
    lo.z = __fadd_rn(__fsub_rn(p.z, hi.z), oz);
  }
  xm[t] = hi;
  xlo[t] = lo;
}

__global__ void __launch_bounds__(128) k_vr_cov_G(const MultiGridView* __restrict__ mg,
                                                  const float4* __restrict__ pos, const float4* __restrict__ vrc,
                                                  const float4* __restrict__ xm0,
                                                  const float4* __restrict__ xlo, float4* __restrict__ xm, long long n,
                                                  float4* __restrict__ ga, float4* __restrict__ gb,
                                                  float* __restrict__ gfull, float* __restrict__ det_out,
                                                  int8_t* __restrict__ f64flag, unsigned long long* __restrict__ f64count) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const MultiGridView& m = *mg;
  const float4 p = pos[t];
  const float4 xp = xm0[t];
  const float4 lp = xlo[t];
  const float4 ci = vrc[t];
  const float h = p.w * 2.0f;  // 2 r_i
  const float h2 = ci.x;       // Influnce2_i
  const float sigma = ci.y;    // Sigma_i
  const float inv_h = 1.0f / h;
  Kahan ws, c00, c01, c02, c11, c12, c22;
  for (int b = 0; b < m.nb; ++b) {
    const BinGrid g = m.g[b];
    const int cx = cell_coord(p.x, g.b0, g.cell, g.nx), cy = cell_coord(p.y, g.b2, g.cell, g.ny),
              cz = cell_coord(p.z, g.b4, g.cell, g.nz);
    for (int dz = -1; dz <= 1; ++dz)
      for (int dy = -1; dy <= 1; ++dy) {
        int s, e;
        if (!bin_row(g, m.off, cx, cy + dy, cz + dz, &s, &e)) continue;
        for (int j = s; j < e; ++j) {
          const float4 q = __ldg(xm0 + j);
          const float4 lq = __ldg(xlo + j);
          const float4 cj = __ldg(vrc + j);
          const float nI = cj.z;
          const float dx = __fadd_rn(__fsub_rn(q.x, xp.x), __fsub_rn(lq.x, lp.x));
          const float dy2 = __fadd_rn(__fsub_rn(q.y, xp.y), __fsub_rn(lq.y, lp.y));
          const float dz2 = __fadd_rn(__fsub_rn(q.z, xp.z), __fsub_rn(lq.z, lp.z));
          const float d2 = d2_exact(dx, dy2, dz2);
          if (!(d2 < __fmul_rn(nI, nI))) continue;
          const float w = wij_f(__fsqrt_rn(d2), nI, cj.w);
          ws.add(w);
          c00.add(dx * dx * w);
          c01.add(dx * dy2 * w);
          c02.add(dx * dz2 * w);
          c11.add(dy2 * dy2 * w);
          c12.add(dy2 * dz2 * w);
          c22.add(dz2 * dz2 * w);
        }
      }
  }
  const float iw = 1.0f / ws.s;
  float a6[6] = {(h2 + c00.s) * iw, c01.s * iw, c02.s * iw, (h2 + c11.s) * iw, c12.s * iw, (h2 + c22.s) * iw};
  float w[3], V[3][3];
  float G[9], stretch;
  bool degenerate = false;
  if (!(ws.s > 0.f)) {
    for (int k = 0; k < 9; ++k) G[k] = (k % 4 == 0) ? 1.0f : 0.0f;
    stretch = 1.0f;
  } else {
    sym_eig3<float>(a6, w, V);
    const float aw0 = fabsf(w[0]), aw1 = fabsf(w[1]), aw2 = fabsf(w[2]);
    const float wmx = fmaxf(aw0, fmaxf(aw1, aw2)), wmn = fminf(aw0, fminf(aw1, aw2));
    degenerate = wmn < 0.25f * wmx;
    if (degenerate) {
      double a6d[6], wd[3], Vd[3][3];
      for (int k = 0; k < 6; ++k) a6d[k] = (double)a6[k];
      sym_eig3<double>(a6d, wd, Vd);
      g_from_eig<double>(wd, Vd, G, &stretch);
      stripe_add(f64count, 0, 1ull);
    } else {
      g_from_eig<float>(w, V, G, &stretch);
    }
  }
  const float det = G[0] * (G[4] * G[8] - G[5] * G[7]) - G[1] * (G[3] * G[8] - G[5] * G[6]) +
                    G[2] * (G[3] * G[7] - G[4] * G[6]);
  const float R = 2.0f * stretch / inv_h;
  const float h5 = h * h * h * h * h;
  xm[t] = make_float4(xp.x, xp.y, xp.z, R * R * 1.002f);
  ga[t] = make_float4(G[0] * inv_h, G[1] * inv_h, G[2] * inv_h, G[4] * inv_h);
  // gb.w: -6 h_i^5, the factor of the normal's gradient form in A units
  gb[t] = make_float4(G[5] * inv_h, G[8] * inv_h, det * sigma, -6.0f * h5);
  for (int k = 0; k < 9; ++k) gfull[9 * t + k] = G[k];
  det_out[t] = det;
  f64flag[t] = degenerate ? 1 : 0;
}

void stage_aniso_vr(pi_frame* f) {
  cudaStream_t s = f->ctx->stream;
  const long long n = f->N;
  f->xm.alloc(f->ctx, s, n);
  f->nrm.alloc(f->ctx, s, n);  // holds the pass-1 centres until the normals overwrite it
  f->ga.alloc(f->ctx, s, n);
  f->gb.alloc(f->ctx, s, n);
  f->xlo.alloc(f->ctx, s, n);
  f->gfull.alloc(f->ctx, s, n * 9);
  f->det.alloc(f->ctx, s, n);
  f->f64flag.alloc(f->ctx, s, n);
  counters_reset(f);
  PI_LAUNCH(k_vr_xmean, div_up(n, 128), 128, 0, s, f->mgv.p, f->pos.p, f->vrcs.p, n, (float)0.9, f->nrm.p,
            f->xlo.p);
  PI_LAUNCH(k_vr_cov_G, div_up(n, 128), 128, 0, s, f->mgv.p, f->pos.p, f->vrcs.p, f->nrm.p, f->xlo.p, f->xm.p, n,
            f->ga.p, f->gb.p, f->gfull.p, f->det.p, f->f64flag.p, f->dcount.p);
  counters_snapshot(f, kPinAniso);
}

void stage_aniso(pi_frame* f) {
  cudaStream_t s = f->ctx->stream;
  const long long n = f->N;
  const GridHost& gh = f->g;
  GridView g{gh.bounding[0], gh.bounding[2], gh.bounding[4], gh.cell, gh.nx, gh.ny, gh.nz, f->off.p};
  // Evaluator ctor constants (src/evaluator.cpp:5-58), reference float/double semantics
  const float r = f->P.radius;
  f->influ2 = (float)std::pow(r * 2.0f, 2);
  f->sigma = (float)(1 / std::pow(r * 2.0f, 6));
  const float nI = r * 4.0f;  // nR * _NEIGHBOR_FACTOR
  const float nI2 = nI * nI;
  const float inv_h3 = (float)(1.0 / ((double)nI * nI * nI));
  const float delta = (float)0.9;
  const float c_mean = delta;
  const float h = r * 2.0f;
  f->xm.alloc(f->ctx, s, n);
  f->nrm.alloc(f->ctx, s, n);  // holds the pass-1 centres until the normals overwrite it
  f->ga.alloc(f->ctx, s, n);
  f->gb.alloc(f->ctx, s, n);
  f->xlo.alloc(f->ctx, s, n);
  f->gfull.alloc(f->ctx, s, n * 9);
  f->det.alloc(f->ctx, s, n);
  f->f64flag.alloc(f->ctx, s, n);
  const bool splash = f->P.splash != 0;
  if (splash) f->spl.alloc(f->ctx, s, n);
  counters_reset(f);
  PI_LAUNCH(k_xmean, div_up(n, 128), 128, 0, s, g, f->pos.p, n, nI, nI2, inv_h3, c_mean, f->nrm.p, f->xlo.p,
            splash ? f->spl.p : nullptr);
  PI_LAUNCH(k_cov_G, div_up(n, 128), 128, 0, s, g, f->pos.p, f->nrm.p, f->xlo.p, f->xm.p, n, nI, nI2, inv_h3, f->influ2,
            1.0f / h, f->sigma, f->ga.p, f->gb.p, f->gfull.p, f->det.p, f->f64flag.p, f->dcount.p,
            splash ? f->spl.p : nullptr);
  if (splash) stage_splash_list(f);
  counters_snapshot(f, kPinAniso);
}

}  // namespace pisurf
