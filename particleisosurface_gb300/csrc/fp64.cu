// FP64 oracle on the GPU: the reference's anisotropy and field formulas in
// double precision, written for accuracy rather than speed, as the arbiter
// of the FP32 path's error reports.
//
//   k_f64_xmean   compute_xMeans + wij (src/evaluator.cpp:465-512,751-766),
//                 pass 1 of compute_Gs_xMeans (:658-718)
//   k_f64_G       compute_G_Yus (:585-654), pass 2 (:720-749), and
//                 Matrix3f::determinant (:746)
//   k_f64_eval    SingleEval / SingleEvalWithGrad (:60-125) with
//                 AnisotropicInterpolate(Grad) and Bspline_kernel
//                 (:437-463, :383-396, :408-415)
//
// One thread per particle or point.  Each walks the reference's whole 27-cell
// candidate list (GetPIdxList, src/hash_grid.cpp:196-214) on the frame's hash
// grid, whose keys and cell order are the reference's bit for bit, and tests
// every candidate in double: no support culling, no deduplication, no
// compensated sums, no float centre pairs.  Only the reconstruction's
// inputs are shared with the FP32 path: the float particle positions and
// the hash grid.  The covariance eigen-decomposition is its own cyclic
// Jacobi, run to convergence in double.
//
// Per-particle state (sorted order): x64[3N], g64[9N], det64[N], 104 bytes
// per particle, allocated on the first call and kept with the frame.  With
// splash particles on, the oracle marks them itself (<= 2 candidates or <= 2
// neighbours within 4r, distances in double) into spl64[N], gives them the
// identity G and leaves them out of its sums.
#include <cmath>
#include <vector>

#include "device.cuh"
#include "internal.h"

namespace pisurf {

struct F64Consts {
  double radius;  // r as double (the reference's Radius)
  double nI, nI2; // neighbour radius 4r and its square
  double influ2;  // (2r)^2
  double sigma;   // 1 / (2r)^6
  double iso;     // Bspline_kernel(0.01, Sigma)
};

// wij (src/evaluator.cpp:751-766) in double.
__device__ __forceinline__ double wij_d(double d, double h) {
  if (d < h) {
    const double hmd = h - d;
    if (d < h / 2) return 1.0 - 6.0 * d * d / (h * h * h) * hmd;
    return 2.0 / (h * h * h) * hmd * hmd * hmd;
  }
  return 0.0;
}

// Bspline_kernel (src/evaluator.cpp:383-396) in double.
__device__ __forceinline__ double bspline_d(double ratio, double sigma) {
  if (ratio < 2.0) {
    if (ratio <= 1.0) return sigma * (1.0 - 1.5 * ratio * ratio + 0.75 * ratio * ratio * ratio);
    const double t = 2.0 - ratio;
    return sigma * (0.25 * t * t * t);
  }
  return 0.0;
}

// Symmetric 3x3 eigen-decomposition by cyclic Jacobi rotations (Golub and
// Van Loan, Matrix Computations, 8.5.2): sweeps over (0,1), (0,2), (1,2) until
// the off-diagonal mass is below 1e-30 of the diagonal's (a few sweeps in
// double).  A is overwritten; eigenvalues on its diagonal, eigenvectors in the
// columns of V.
__device__ void jacobi_eig3_d(double A[3][3], double V[3][3]) {
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) V[i][j] = i == j ? 1.0 : 0.0;
  for (int sweep = 0; sweep < 32; ++sweep) {
    const double off = A[0][1] * A[0][1] + A[0][2] * A[0][2] + A[1][2] * A[1][2];
    const double dia = A[0][0] * A[0][0] + A[1][1] * A[1][1] + A[2][2] * A[2][2];
    if (off <= 1e-30 * dia) break;
    for (int k = 0; k < 3; ++k) {
      const int p = k < 2 ? 0 : 1, q = k == 0 ? 1 : 2;
      const double apq = A[p][q];
      if (apq == 0.0) continue;
      // rotation angle that zeroes A[p][q]: tan of the smaller root
      const double tau = (A[q][q] - A[p][p]) / (2.0 * apq);
      const double t = (tau >= 0.0 ? 1.0 : -1.0) / (fabs(tau) + sqrt(1.0 + tau * tau));
      const double c = 1.0 / sqrt(1.0 + t * t), s = t * c;
      for (int r = 0; r < 3; ++r) {
        const double arp = A[r][p], arq = A[r][q];
        A[r][p] = c * arp - s * arq;
        A[r][q] = s * arp + c * arq;
      }
      for (int r = 0; r < 3; ++r) {
        const double apr = A[p][r], aqr = A[q][r];
        A[p][r] = c * apr - s * aqr;
        A[q][r] = s * apr + c * aqr;
      }
      for (int r = 0; r < 3; ++r) {
        const double vrp = V[r][p], vrq = V[r][q];
        V[r][p] = c * vrp - s * vrq;
        V[r][q] = s * vrp + c * vrq;
      }
    }
  }
}

__global__ void k_f64_xmean(GridView g, const float4* __restrict__ pos, long long n, F64Consts k,
                            double* __restrict__ x64, int8_t* __restrict__ spl64) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const float4 pf = pos[t];
  const double px = pf.x, py = pf.y, pz = pf.z;
  int cx, cy, cz;
  cell_of(g, pf.x, pf.y, pf.z, cx, cy, cz);
  long long cand = 0;
  int nn = 0;
  double ws = 0.0, mx = 0.0, my = 0.0, mz = 0.0;
  for (int dz = -1; dz <= 1; ++dz)
    for (int dy = -1; dy <= 1; ++dy) {
      int s, e;
      if (!nb_row(g, cx, cy + dy, cz + dz, &s, &e)) continue;
      cand += e - s;
      for (int j = s; j < e; ++j) {
        if (j == t) continue;
        const float4 q = pos[j];
        const double dx = (double)q.x - px, dyy = (double)q.y - py, dzz = (double)q.z - pz;
        const double d2 = dx * dx + dyy * dyy + dzz * dzz;
        if (d2 >= k.nI2) continue;
        ++nn;
        const double w = wij_d(sqrt(d2), k.nI);
        ws += w;
        mx += (double)q.x * w;
        my += (double)q.y * w;
        mz += (double)q.z * w;
      }
    }
  double ox = px, oy = py, oz = pz;
  // <= 2 candidates: the particle itself (src/evaluator.cpp:670-673)
  if (cand > 2 && ws > 0.0) {
    ox = px * (1.0 - 0.9) + (mx / ws) * 0.9;
    oy = py * (1.0 - 0.9) + (my / ws) * 0.9;
    oz = pz * (1.0 - 0.9) + (mz / ws) * 0.9;
  }
  x64[3 * t] = ox;
  x64[3 * t + 1] = oy;
  x64[3 * t + 2] = oz;
  if (spl64) spl64[t] = (cand <= 2 || nn <= 2) ? 1 : 0;
}

__global__ void k_f64_G(GridView g, const float4* __restrict__ pos, long long n, F64Consts k,
                        const double* __restrict__ x64, const int8_t* __restrict__ spl64, double* __restrict__ g64,
                        double* __restrict__ det64) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  if (spl64 && spl64[t]) {  // splash: pass 1's identity
    for (int a = 0; a < 9; ++a) g64[9 * t + a] = (a % 4 == 0) ? 1.0 : 0.0;
    det64[t] = 1.0;
    return;
  }
  const float4 pf = pos[t];
  const double xp[3] = {x64[3 * t], x64[3 * t + 1], x64[3 * t + 2]};
  int cx, cy, cz;
  cell_of(g, pf.x, pf.y, pf.z, cx, cy, cz);
  double ws = 0.0, c[3][3] = {{k.influ2, 0, 0}, {0, k.influ2, 0}, {0, 0, k.influ2}};
  for (int dz = -1; dz <= 1; ++dz)
    for (int dy = -1; dy <= 1; ++dy) {
      int s, e;
      if (!nb_row(g, cx, cy + dy, cz + dz, &s, &e)) continue;
      for (int j = s; j < e; ++j) {
        const double d[3] = {x64[3 * j] - xp[0], x64[3 * j + 1] - xp[1], x64[3 * j + 2] - xp[2]};
        const double d2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
        if (d2 >= k.nI2) continue;
        const double w = wij_d(sqrt(d2), k.nI);
        ws += w;
        for (int a = 0; a < 3; ++a)
          for (int b = 0; b < 3; ++b) c[a][b] += d[a] * d[b] * w;
      }
    }
  double G[3][3];
  if (!(ws > 0.0)) {
    // no candidate within 4r: identity, as for particles with <= 2 candidates
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b) G[a][b] = a == b ? 1.0 : 0.0;
  } else {
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b) c[a][b] /= ws;
    double V[3][3];
    jacobi_eig3_d(c, V);
    double w[3] = {fabs(c[0][0]), fabs(c[1][1]), fabs(c[2][2])};
    const double wmax = fmax(w[0], fmax(w[1], w[2]));
    for (int a = 0; a < 3; ++a) w[a] = fmax(w[a], wmax / 4.0);  // kr = 4 (src/evaluator.cpp:642-645)
    const double scale = cbrt(w[0] * w[1] * w[2]);
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b)
        G[a][b] = scale * (V[a][0] * V[b][0] / w[0] + V[a][1] * V[b][1] / w[1] + V[a][2] * V[b][2] / w[2]);
  }
  for (int a = 0; a < 3; ++a)
    for (int b = 0; b < 3; ++b) g64[9 * t + 3 * a + b] = G[a][b];
  det64[t] = G[0][0] * (G[1][1] * G[2][2] - G[1][2] * G[2][1]) - G[0][1] * (G[1][0] * G[2][2] - G[1][2] * G[2][0]) +
             G[0][2] * (G[1][0] * G[2][1] - G[1][1] * G[2][0]);
}

__global__ void k_f64_eval(GridView g, long long m, const float* __restrict__ pts, F64Consts k,
                           const double* __restrict__ x64, const double* __restrict__ g64,
                           const double* __restrict__ det64, const int8_t* __restrict__ spl64,
                           double* __restrict__ val, double* __restrict__ grad) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  const float qf[3] = {pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]};
  int cx, cy, cz;
  cell_of(g, qf[0], qf[1], qf[2], cx, cy, cz);
  double sum = 0.0, gs[3] = {0.0, 0.0, 0.0};
  for (int dz = -1; dz <= 1; ++dz)
    for (int dy = -1; dy <= 1; ++dy) {
      int s, e;
      if (!nb_row(g, cx, cy + dy, cz + dz, &s, &e)) continue;
      for (int j = s; j < e; ++j) {
        if (spl64 && spl64[j]) continue;  // CheckSplash (src/evaluator.cpp:73-76)
        const double d[3] = {(double)qf[0] - x64[3 * j], (double)qf[1] - x64[3 * j + 1],
                             (double)qf[2] - x64[3 * j + 2]};
        const double* G = g64 + 9 * j;
        double u[3];
        for (int a = 0; a < 3; ++a) u[a] = G[3 * a] * d[0] + G[3 * a + 1] * d[1] + G[3 * a + 2] * d[2];
        const double d2 = u[0] * u[0] + u[1] * u[1] + u[2] * u[2];
        sum += det64[j] * bspline_d(sqrt(d2 / k.influ2), k.sigma);
        if (grad && d2 <= k.influ2) {
          const double h = (k.influ2 - d2) * (k.influ2 - d2);
          for (int a = 0; a < 3; ++a) gs[a] += det64[j] * (k.sigma * (-6.0 * u[a]) * h);
        }
      }
    }
  val[i] = k.iso - sum;
  if (grad)
    for (int a = 0; a < 3; ++a) grad[3 * i + a] = gs[a];
}

// sorted order -> original particle order, `w` doubles per particle
__global__ void k_f64_unsort(const double* __restrict__ src, const uint32_t* __restrict__ sidx, long long n, int w,
                             double* __restrict__ dst) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const long long i = sidx[t];
  for (int k = 0; k < w; ++k) dst[i * w + k] = src[t * w + k];
}

static F64Consts f64_consts(const pi_frame* f) {
  // Evaluator ctor and RecommendIsoValueConstR in double (src/evaluator.cpp:
  // 5-58, 323-335): the reference's Influnce2 and Sigma from (2r) with r the
  // float radius, the iso value the kernel at ratio 0.01
  F64Consts k;
  k.radius = (double)f->P.radius;
  k.nI = k.radius * 4.0;
  k.nI2 = k.nI * k.nI;
  const double h = (double)(f->P.radius * 2.0f);
  k.influ2 = h * h;
  k.sigma = 1.0 / (h * h * h * h * h * h);
  const double q = 0.01;
  k.iso = k.sigma * (1.0 - 1.5 * q * q + 0.75 * q * q * q);
  return k;
}

static GridView f64_gview(const pi_frame* f) {
  const GridHost& gh = f->g;
  return GridView{gh.bounding[0], gh.bounding[2], gh.bounding[4], gh.cell, gh.nx, gh.ny, gh.nz, f->off.p};
}

void fp64_state(pi_frame* f) {
  if (f->x64.p && (long long)f->det64.n == f->N && f->f64_ready) return;
  cudaStream_t s = f->ctx->stream;
  const long long n = f->N;
  f->x64.alloc(f->ctx, s, 3 * n);
  f->g64.alloc(f->ctx, s, 9 * n);
  f->det64.alloc(f->ctx, s, n);
  int8_t* spl = nullptr;
  if (f->P.splash) {
    f->spl64.alloc(f->ctx, s, n);
    spl = f->spl64.p;
  }
  const F64Consts k = f64_consts(f);
  const GridView g = f64_gview(f);
  PI_LAUNCH(k_f64_xmean, div_up(n, 128), 128, 0, s, g, f->pos.p, n, k, f->x64.p, spl);
  PI_LAUNCH(k_f64_G, div_up(n, 128), 128, 0, s, g, f->pos.p, n, k, f->x64.p, spl, f->g64.p, f->det64.p);
  f->f64_ready = true;
}

void fp64_aniso_get(pi_frame* f, double* h_x3, double* h_g9, double* h_det) {
  fp64_state(f);
  cudaStream_t s = f->ctx->stream;
  const long long n = f->N;
  DBuf<double> tmp;
  tmp.alloc(f->ctx, s, 9 * n);
  struct Out {
    const double* src;
    int w;
    double* dst;
  } outs[3] = {{f->x64.p, 3, h_x3}, {f->g64.p, 9, h_g9}, {f->det64.p, 1, h_det}};
  for (const Out& o : outs) {
    if (!o.dst) continue;
    PI_LAUNCH(k_f64_unsort, div_up(n, 256), 256, 0, s, o.src, f->sidx.p, n, o.w, tmp.p);
    PI_CUDA(cudaMemcpyAsync(o.dst, tmp.p, sizeof(double) * o.w * n, cudaMemcpyDeviceToHost, s));
    PI_CUDA(cudaStreamSynchronize(s));
  }
}

void fp64_eval(pi_frame* f, const float* d_pts, long long m, double* d_val, double* d_grad) {
  fp64_state(f);
  PI_LAUNCH(k_f64_eval, div_up(m, 128), 128, 0, f->ctx->stream, f64_gview(f), m, d_pts, f64_consts(f), f->x64.p,
            f->g64.p, f->det64.p, f->P.splash ? f->spl64.p : nullptr, d_val, d_grad);
}

void fp64_scalars(const pi_frame* f, double out4[4]) {
  const F64Consts k = f64_consts(f);
  // CalculateMaxScalarConstR (src/evaluator.cpp:272-291) in double
  auto B = [&](double q) {
    if (q <= 1.0) return k.sigma * (1.0 - 1.5 * q * q + 0.75 * q * q * q);
    const double t = 2.0 - q;
    return k.sigma * 0.25 * t * t * t;
  };
  out4[0] = k.iso;
  out4[1] = B(0.0) + 6.0 * B(1.0) + 12.0 * B(std::sqrt(2.0)) + 8.0 * B(std::sqrt(3.0));
  out4[2] = k.influ2;
  out4[3] = k.sigma;
}

}  // namespace pisurf
