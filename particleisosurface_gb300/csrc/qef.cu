// K5: per-leaf QEF vertex, TNode::NodeCalcNode (src/iso_method_ours.cpp:101-174)
// with QEFNormal<float,4>::combineSelf (include/qefnorm.h:18-33) and
// calcErrorDMC (src/iso_method_ours.cpp:40-50).  In the reference both call
// sites are commented out (src/surface_reconstructor.cpp:258,270); pi_params.qef
// switches them on with the same semantics:
//   leaf by size:      node = QEF vertex if it lies in the cell, value
//                      f(node), zeroed if err / cellsize < 1e-4;
//   leaf by criteria:  node = QEF vertex if it lies in the cell, value
//                      f(node) (the later SingleEval undoes the zeroing).
// Gradients are the finite differences of GridEval (src/evaluator.cpp:293-359)
// over the 27 samples.  Accumulation and solve are FP64; the solve follows
// the pseudo-inverse rule of a Jacobi eigen-decomposition of the equilibrated
// symmetric 4x4 normal matrix (eigenvalues below 1e-12 of the largest are
// dropped), decided by LDL^T bounds where they settle it.  Where that matrix
// is singular the reference's Matrix4f::inverse yields non-finite values and
// the vertex is rejected; so is it here, and the number of singular leaves is
// counted.
#include <cmath>

#include "device.cuh"
#include "internal.h"

namespace pisurf {

enum : int8_t { Q_EMPTY = 0, Q_INTERNAL = 1, Q_LEAF = 2 };

// Symmetric 4x4 Jacobi eigen-decomposition, A = V diag(w) V^T.
__device__ void sym_eig4(double A[4][4], double w[4], double V[4][4]) {
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) V[i][j] = (i == j) ? 1.0 : 0.0;
  for (int sweep = 0; sweep < 20; ++sweep) {
    double off = 0.0, dia = 0.0;
    for (int p = 0; p < 4; ++p) {
      dia += fabs(A[p][p]);
      for (int q = p + 1; q < 4; ++q) off += fabs(A[p][q]);
    }
    if (off <= 1e-18 * dia || off == 0.0) break;
    for (int p = 0; p < 3; ++p)
      for (int q = p + 1; q < 4; ++q) {
        const double apq = A[p][q];
        if (fabs(apq) <= 1e-300) continue;
        const double theta = (A[q][q] - A[p][p]) / (2.0 * apq);
        double t = 1.0 / (fabs(theta) + sqrt(theta * theta + 1.0));
        if (theta < 0.0) t = -t;
        const double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
        for (int r = 0; r < 4; ++r) {
          const double arp = A[r][p], arq = A[r][q];
          A[r][p] = c * arp - s * arq;
          A[r][q] = s * arp + c * arq;
        }
        for (int r = 0; r < 4; ++r) {
          const double apr = A[p][r], aqr = A[q][r];
          A[p][r] = c * apr - s * aqr;
          A[q][r] = s * apr + c * aqr;
        }
        for (int r = 0; r < 4; ++r) {
          const double vrp = V[r][p], vrq = V[r][q];
          V[r][p] = c * vrp - s * vrq;
          V[r][q] = s * vrp + c * vrq;
        }
      }
  }
  for (int i = 0; i < 4; ++i) w[i] = A[i][i];
}

// d / 2 for a double d that is 0 or at least 2^-1021 in magnitude (here a
// difference of two floats, so at least 2^-149), exactly, on the integer
// pipe: the exponent field is decremented.
__device__ __forceinline__ double half_exact(double d) {
  const long long b = __double_as_longlong(d);
  return (b << 1) == 0 ? d : __longlong_as_double(b - (1LL << 52));
}

// (double)f on the integer pipe for a normal float f (the exponent rebased
// from 127 to 1023, the 23 fraction bits moved to the top of the 52), the
// hardware conversion for zero, subnormal, infinite and NaN inputs.
__device__ __forceinline__ double f2d_exact(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned e = (u >> 23) & 0xffu;
  if (e == 0u || e == 0xffu) return (double)f;
  const unsigned hi = (u & 0x80000000u) | (((u >> 3) & 0x0fffffffu) + (896u << 20));
  return __hiloint2double((int)hi, (int)(u << 29));
}

// Equilibration scale of a diagonal entry v: about v^-1/2 from the FP32
// reciprocal square root when v converts to a normal float, the FP64 value
// otherwise, 1 for v <= 0.  Any positive scale gives the same solution.
__device__ __forceinline__ double equil_scale(double v) {
  if (!(v > 0.0)) return 1.0;
  const float vf = (float)v;
  if (vf >= 1.17549435e-38f && vf <= 3.0e38f) return (double)rsqrtf(vf);
  return 1.0 / sqrt(v);
}

struct QefArgs {
  GridView g;
  PartView P;
  float iso;
  float radius;
  long long lb, le;
  // the level's finite-difference step (every node of a level has the same
  // half size), in FP64, and its reciprocal
  double step, i1;
};

constexpr int kQefThreads = 64;

// LDL^T factorisation of the symmetric 4x4 A (no pivoting): pivots d, their
// reciprocals id, and M = L^-1 (unit lower triangular), so that
// A^-1 = M^T diag(id) M.  Returns 0 if a pivot is below `floor`, 1 otherwise.
__device__ int ldlt4(const double A[4][4], double floor, double d[4], double id[4], double M[4][4]) {
  double L[4][4] = {{1, 0, 0, 0}, {0, 1, 0, 0}, {0, 0, 1, 0}, {0, 0, 0, 1}};
  for (int j = 0; j < 4; ++j) {
    double dj = A[j][j];
    for (int k = 0; k < j; ++k) dj -= L[j][k] * L[j][k] * d[k];
    if (!(dj >= floor)) return 0;
    d[j] = dj;
    id[j] = 1.0 / dj;
    for (int i = j + 1; i < 4; ++i) {
      double l = A[i][j];
      for (int k = 0; k < j; ++k) l -= L[i][k] * L[j][k] * d[k];
      L[i][j] = l * id[j];
    }
  }
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) M[i][j] = i == j ? 1.0 : 0.0;
  for (int i = 1; i < 4; ++i)
    for (int j = 0; j < i; ++j) {
      double v = -L[i][j];
      for (int k = j + 1; k < i; ++k) v -= L[i][k] * M[k][j];
      M[i][j] = v;
    }
  return 1;
}

// The leaves of the level [lb, le), as offsets node - lb, so that k_qef's
// threads are all leaves: the FP64 pipe issues per warp instruction, and a
// thread that has no leaf would leave its lane of every FP64 instruction
// idle (on a level with few leaves most of them).  One atomic per warp;
// list[0] counts the leaves and they follow from list[1] (each warp's in
// node order; each leaf's result does not depend on the order).
// With npart, only the leaves of part `part` (the leaf level in parts).
__global__ void k_qef_pick(const int8_t* __restrict__ nd_type, long long lb, long long le,
                           const int8_t* __restrict__ npart, int part, int* __restrict__ list) {
  const long long node = lb + (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  const bool leaf = node < le && (!npart || npart[node - lb] == part) && nd_type[node] == Q_LEAF;
  const unsigned m = __ballot_sync(0xffffffffu, leaf);
  if (m == 0u) return;  // warp-uniform
  int base = 0;
  if (lane == 0) base = atomicAdd(list, __popc(m));
  base = __shfl_sync(0xffffffffu, base, 0);
  if (leaf) list[1 + base + __popc(m & ((1u << lane) - 1u))] = (int)(node - lb);
}

// counters: QEF vertices accepted, singular systems, field evaluations, leaves solved
__global__ void __launch_bounds__(kQefThreads) k_qef(QefArgs a, const int* __restrict__ list,
                                                     float4* __restrict__ nd_v,
                                                     const float4* __restrict__ nd_c,
                                                     const float* __restrict__ nd_samp, float* __restrict__ qef_err,
                                                     unsigned long long* __restrict__ counters) {
  // the 27 sample values in FP64, converted once per leaf on the integer
  // pipe (the FP64 pipe bounds this kernel)
  __shared__ double s_sv[27][kQefThreads];
  const int t = blockIdx.x * kQefThreads + threadIdx.x;
  if (t >= __ldg(list)) return;
  {
    const unsigned am = __activemask();  // the warp's lanes that hold a leaf
    if ((int)(threadIdx.x & 31) == __ffs(am) - 1) stripe_add(counters, C_QEF_LEAVES, (unsigned long long)__popc(am));
  }
  const long long node = a.lb + __ldg(list + 1 + t);
  const float4 c = nd_c[node];
  const float h = c.w;
  const float cellsize = 2.0f * h;
  const float step = cellsize / 2;
  const float mn[3] = {__fsub_rn(c.x, h), __fsub_rn(c.y, h), __fsub_rn(c.z, h)};
  const float mx[3] = {__fadd_rn(c.x, h), __fadd_rn(c.y, h), __fadd_rn(c.z, h)};
  const float* sv = nd_samp + node * 27;
  double* const sd = &s_sv[0][threadIdx.x];  // sd[i * kQefThreads] = sample i
#pragma unroll
  for (int i = 0; i < 27; ++i) sd[i * kQefThreads] = f2d_exact(sv[i]);
  // sample positions (GenerateSampling): three per axis, in units of the
  // finite-difference step (times 1 / step, see below)
  const double i1 = a.i1;
  auto lattice = [&](int ax, int k) {
    return f2d_exact(__fadd_rn(__fmul_rn(1.0f - k * 0.5f, mn[ax]), __fmul_rn(k * 0.5f, mx[ax]))) * i1;
  };
  const double px0 = lattice(0, 0), px1 = lattice(0, 1), px2 = lattice(0, 2);
  const double py0 = lattice(1, 0), py1 = lattice(1, 1), py2 = lattice(1, 2);
  const double pz0 = lattice(2, 0), pz1 = lattice(2, 1), pz2 = lattice(2, 2);
  // GridEval's finite differences (src/evaluator.cpp:185-240) are g = d / step
  // (one-sided) and g = d / (2 step) (central), d a difference of samples.
  // NodeCalcNode's residual of plane i at (x, v) is g.(x - p) - v + f, which
  // with y = x / step and q = p / step reads d'.(y - q) - v + f, d' = d or
  // d / 2: the same least-squares problem in the variables (y, v), solved
  // below and mapped back by x = step y.  So no sample difference is scaled
  // by the step; the central ones are halved on the integer pipe, and only
  // the nine lattice coordinates are multiplied (FP64 instructions bound this
  // kernel).  The pseudo-inverse rule sees the same equilibrated matrix: a
  // diagonal change of variables cancels in D A D.
  //
  // The plane's -1 entry makes q[3], q[7], q[10] minus the sums of the
  // differences over the 27 samples.  Along one row of three samples
  // s0, s1, s2 those are (s0 - s1) + (s0 - s2) / 2 + (s1 - s2) = 3 times the
  // central one, so each is taken as -3 times the sum over the 9 central
  // samples of its axis.
  double q[15];
  double cx = 0.0, cy = 0.0, cz = 0.0;
#pragma unroll
  for (int k = 0; k < 15; ++k) q[k] = 0.0;
#pragma unroll
  for (int i = 0; i < 27; ++i) {
    const int x = i % 3, y = (i / 3) % 3, z = i / 9;
    const double px = x == 0 ? px0 : x == 1 ? px1 : px2;
    const double py = y == 0 ? py0 : y == 1 ? py1 : py2;
    const double pz = z == 0 ? pz0 : z == 1 ? pz1 : pz2;
    auto fd = [&](int d, int stride) {
      if (d == 0) return sd[i * kQefThreads] - sd[(i + stride) * kQefThreads];
      if (d == 2) return sd[(i - stride) * kQefThreads] - sd[i * kQefThreads];
      return half_exact(sd[(i - stride) * kQefThreads] - sd[(i + stride) * kQefThreads]);
    };
    const double gx = fd(x, 1), gy = fd(y, 3), gz = fd(z, 9);
    // plane [d', -1, f - q.d'] accumulated as QEFNormal::combineSelf
    const double w = fma(-pz, gz, fma(-py, gy, fma(-px, gx, sd[i * kQefThreads])));
    const double pl[5] = {gx, gy, gz, -1.0, w};
    if (x == 1) cx += gx;
    if (y == 1) cy += gy;
    if (z == 1) cz += gz;
    int idx = 0;
#pragma unroll
    for (int r = 0; r < 5; ++r)
#pragma unroll
      for (int s2 = r; s2 < 5; ++s2, ++idx)
        if (idx != 3 && idx != 7 && idx != 10 && idx != 12) q[idx] += pl[r] * pl[s2];
  }
  q[3] = -3.0 * cx;
  q[7] = -3.0 * cy;
  q[10] = -3.0 * cz;
  q[12] = 27.0;  // the (-1) x (-1) entry: 27 ones
  double A[4][4], B[4];
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    const int idx = ((2 * 4 + 3 - r) * r) / 2;
#pragma unroll
    for (int s2 = r; s2 < 4; ++s2) A[r][s2] = A[s2][r] = q[idx + s2 - r];
    B[r] = -q[idx + 4 - r];
  }
  // Equilibrate: the gradient rows are ~|f| / step while the w column is 1,
  // so A's condition number exceeds what FP32 or even FP64 resolves.  With
  // a positive diagonal D close to diag(A_ii)^-1/2 the solve is
  // (D A D) y = D B, x = D y: the same minimiser in exact arithmetic for any
  // such D, well conditioned unless the planes are degenerate.  D is taken
  // from the FP32 reciprocal square root (two conversions instead of an FP64
  // square root and division); the equilibrated diagonal is then 1 to about
  // 1e-7, and dmax, its largest entry, bounds the largest eigenvalue from
  // below.
  double D[4];
#pragma unroll
  for (int r = 0; r < 4; ++r) D[r] = equil_scale(A[r][r]);
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    B[r] *= D[r];
#pragma unroll
    for (int s2 = r; s2 < 4; ++s2) A[r][s2] = A[s2][r] = A[r][s2] * (D[r] * D[s2]);
  }
  const double dmax = fmax(fmax(A[0][0], A[1][1]), fmax(A[2][2], A[3][3]));
  // Pseudo-inverse rule: eigenvalues at most 1e-12 * max |eigenvalue| are
  // dropped, and a system with a dropped eigenvalue counts as singular (the
  // reference's Matrix4f::inverse gives non-finite values there and the
  // vertex is rejected).  Decided without an eigen-decomposition where the
  // bounds settle it: the smallest eigenvalue is at most every LDL^T pivot,
  // and at least min(d) / ||M||_F^2 and 1 / ||A^-1||_F (A^-1 = M^T D^-1 M,
  // so ||A^-1||_2 <= ||M||_2^2 / min(d)), while the largest lies in
  // [dmax, trace].  The first lower bound costs a few instructions and
  // settles the dam-break leaves with a margin of 1e6 or more; the second
  // needs the whole inverse and is the fallback.
  const double tr = A[0][0] + A[1][1] + A[2][2] + A[3][3];
  bool singular, solved = false;
  double xs[4] = {0.0, 0.0, 0.0, 0.0};
  double dd[4], id[4], M[4][4];
  const int ok = tr > 0.0 ? ldlt4(A, 1e-12 * dmax, dd, id, M) : 0;
  if (!(tr > 0.0) || !ok) {
    singular = true;  // a pivot below 1e-12 dmax <= 1e-12 * max eigenvalue
    solved = true;
  } else {
    singular = false;
    double m2 = 4.0;
#pragma unroll
    for (int r = 1; r < 4; ++r)
#pragma unroll
      for (int c2 = 0; c2 < r; ++c2) m2 = fma(M[r][c2], M[r][c2], m2);
    const double dmin = fmin(fmin(dd[0], dd[1]), fmin(dd[2], dd[3]));
    const double t = 1e-12 * tr;
    if (dmin > t * m2) {
      // x = M^T D^-1 M B: forward product, scaling, back product
      double z[4];
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        double v = B[r];
#pragma unroll
        for (int k = 0; k < r; ++k) v = fma(M[r][k], B[k], v);
        z[r] = v * id[r];
      }
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        double v = z[r];
#pragma unroll
        for (int k = r + 1; k < 4; ++k) v = fma(M[k][r], z[k], v);
        xs[r] = v;
      }
      solved = true;
    } else {
      double Ai[4][4];
#pragma unroll
      for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int c2 = r; c2 < 4; ++c2) {
          double v = 0.0;
#pragma unroll
          for (int k = c2; k < 4; ++k) v += M[k][r] * id[k] * M[k][c2];
          Ai[r][c2] = Ai[c2][r] = v;
        }
      double f2 = 0.0, f2o = 0.0;  // ||A^-1||_F^2: diagonal, twice the upper part
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        f2 = fma(Ai[r][r], Ai[r][r], f2);
#pragma unroll
        for (int s2 = r + 1; s2 < 4; ++s2) f2o = fma(Ai[r][s2], Ai[r][s2], f2o);
      }
      f2 = fma(2.0, f2o, f2);
      if (f2 * t * t < 1.0) {  // smallest eigenvalue > 1e-12 * trace >= tolerance
#pragma unroll
        for (int r = 0; r < 4; ++r) xs[r] = Ai[r][0] * B[0] + Ai[r][1] * B[1] + Ai[r][2] * B[2] + Ai[r][3] * B[3];
        solved = true;
      }
    }
  }
  if (!solved) {
    // borderline conditioning: the eigen-decomposition decides
    double w[4], V[4][4];
    sym_eig4(A, w, V);
    double wmax = 0.0;
    for (int k = 0; k < 4; ++k) wmax = fmax(wmax, fabs(w[k]));
    const double tol = 1e-12 * wmax;
    singular = !(wmax > 0.0);
    for (int k = 0; k < 4; ++k) {
      if (fabs(w[k]) <= tol) {
        singular = true;
        continue;
      }
      double proj = 0.0;
      for (int r = 0; r < 4; ++r) proj += V[r][k] * B[r];
      proj /= w[k];
      for (int r = 0; r < 4; ++r) xs[r] += V[r][k] * proj;
    }
  }
  float4 v = nd_v[node];
  float err = 1e30f;
  bool accepted = false;
  if (!singular) {
#pragma unroll
    for (int r = 0; r < 4; ++r) xs[r] *= D[r];
#pragma unroll
    for (int r = 0; r < 3; ++r) xs[r] *= a.step;  // x = step y
    const bool in_cell = xs[0] >= mn[0] && xs[0] <= mx[0] && xs[1] >= mn[1] && xs[1] <= mx[1] &&
                         xs[2] >= mn[2] && xs[2] <= mx[2];
    if (in_cell) {
      v = make_float4((float)xs[0], (float)xs[1], (float)xs[2], (float)xs[3]);
      // calcErrorDMC (src/iso_method_ours.cpp:40-50) with GridEval's float
      // gradients, float as in the reference
      err = 0.0f;
      for (int i = 0; i < 27; ++i) {
        const int x = i % 3, y = (i / 3) % 3, z = i / 9;
        const float px = __fadd_rn(__fmul_rn(1.0f - x * 0.5f, mn[0]), __fmul_rn(x * 0.5f, mx[0]));
        const float py = __fadd_rn(__fmul_rn(1.0f - y * 0.5f, mn[1]), __fmul_rn(y * 0.5f, mx[1]));
        const float pz = __fadd_rn(__fmul_rn(1.0f - z * 0.5f, mn[2]), __fmul_rn(z * 0.5f, mx[2]));
        auto fdf = [&](int d, int stride) {
          if (d == 0) return (sv[i] - sv[i + stride]) / step;
          if (d == 2) return (sv[i - stride] - sv[i]) / step;
          return (sv[i - stride] - sv[i + stride]) / (step * 2);
        };
        const float gx = fdf(x, 1), gy = fdf(y, 3), gz = fdf(z, 9);
        const float d = gx * (v.x - px) + gy * (v.y - py) + gz * (v.z - pz) - v.w;
        err += d * d / (1.0f + gx * gx + gy * gy + gz * gz);
      }
      accepted = true;
    }
  } else {
    stripe_add(counters, C_QEF_SINGULAR, 1ull);
  }
  if (accepted) {
    v.w = a.iso - field_sum(a.g, a.P, v.x, v.y, v.z, nullptr);
    stripe_add(counters, C_QEF_EVALS, 1ull);
    stripe_add(counters, C_QEF_ACCEPTED, 1ull);
  }
  // leaf by size keeps the zeroing (no SingleEval follows it)
  const bool leaf_by_size = cellsize - a.radius < kAbove1em8;
  if (leaf_by_size && err / cellsize < 0.0001f) v.w = 0.0f;
  nd_v[node] = v;
  if (qef_err) qef_err[node] = err;
}

// On the context's QEF stream, after the level's classification on the
// context stream: the FP64 pipe is busy with these leaves while the FP32
// pipes run the next level's sampling (or the mesh topology after the last
// level).  The leaf list is the QEF stream's own, allocated and freed in its
// order.
void qef_level(pi_frame* f, long long lb, long long le, int depth, const int8_t* npart, int part) {
  pi_ctx* c = f->ctx;
  cudaStream_t s = c->qef_stream;
  PI_CUDA(cudaEventRecord(c->ev_qef_in, c->stream));
  PI_CUDA(cudaStreamWaitEvent(s, c->ev_qef_in, 0));
  f->qef_inflight = true;
  DBuf<int> list;
  list.alloc(c, s, le - lb + 1);
  int* const scratch = list.p;
  const GridHost& gh = f->g;
  // half size of the level's nodes (the root's halved exactly per level);
  // the step of GridEval is cellsize / 2 = that half size
  const float step = std::ldexp(f->rootH, -depth);
  QefArgs qa{GridView{gh.bounding[0], gh.bounding[2], gh.bounding[4], gh.cell, gh.nx, gh.ny, gh.nz, f->off.p},
             PartView{f->pos.p, f->xm.p, f->ga.p, f->gb.p, f->xlo.p},
             f->iso,
             f->P.radius,
             lb,
             le,
             (double)step,
             1.0 / (double)step};
  PI_CUDA(cudaMemsetAsync(scratch, 0, sizeof(int), s));
  PI_LAUNCH(k_qef_pick, div_up(le - lb, 256), 256, 0, s, f->nd_type.p, lb, le, npart, part, scratch);
  prof_begin(f->ctx, s, PG_QEF);
  PI_LAUNCH(k_qef, div_up(le - lb, kQefThreads), kQefThreads, 0, s, qa, scratch, f->nd_v.p, f->nd_c.p,
            f->nd_samp.p, nullptr, f->dcount.p);
  prof_end(f->ctx, s, PG_QEF);
  list.release();
  PI_CUDA(cudaEventRecord(c->ev_qef_done, s));
}

void qef_join(pi_frame* f) {
  if (!f->qef_inflight) return;
  PI_CUDA(cudaStreamWaitEvent(f->ctx->stream, f->ctx->ev_qef_done, 0));
  f->qef_inflight = false;
}

}  // namespace pisurf
