// CPU oracle: restatement of the reference's OpenMP CPU algorithm for the
// field-evaluation + octree-meshing path.  TEST INFRASTRUCTURE ONLY: used by
// the tests as the checker and by the benchmark as the timed CPU baseline; the
// shipped CUDA library never links it.
//
// Every function cites the reference (LCM1999/ParticleIsosurface) file:line it
// follows.  Arithmetic follows the reference's C++ types: float where the
// reference stores float, double where `pow()` or a double literal promotes.
// Eigen 3.4 (absent here) is restated for the few kernels the path calls:
// fixed-size-3 sums in Eigen's unrolled-redux order x0 + (x1 + x2),
// JacobiSVD<Matrix3f> (two-sided 2x2 Jacobi sweeps), the 3x3 determinant by
// cofactors along the first row, and the 4x4 inverse by the adjugate.
//
// Build with -ffp-contract=off so no multiply-add is fused (the reference's
// x86-64 GCC build has no FMA instructions).
#include "pi_oracle.h"

#include <omp.h>

#include <algorithm>
#include <array>
#include <atomic>
#include <cfloat>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "dmc_cases.h"

namespace pio {

using F3 = std::array<float, 3>;

template <class R>
struct V3 {
  R v[3];
  R& operator[](int i) { return v[i]; }
  const R& operator[](int i) const { return v[i]; }
};

template <class R>
struct M3 {
  R m[3][3];
  R& operator()(int i, int j) { return m[i][j]; }
  const R& operator()(int i, int j) const { return m[i][j]; }
};

// Sum of three terms as Eigen 3.4's unrolled redux evaluates a fixed-size-3
// expression: x0 + (x1 + x2).
template <class R>
static inline R sum3(R a, R b, R c) {
  return a + (b + c);
}

template <class R>
static inline R sqnorm3(R a, R b, R c) {
  return sum3<R>(a * a, b * b, c * c);
}

template <class R>
static inline V3<R> matvec(const M3<R>& G, const V3<R>& d) {
  V3<R> r;
  for (int i = 0; i < 3; ++i) r[i] = sum3<R>(G(i, 0) * d[0], G(i, 1) * d[1], G(i, 2) * d[2]);
  return r;
}

static double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// ---------------------------------------------------------------------------
// HashGrid, constant radius (src/hash_grid.cpp:4-34, 71-214)
// ---------------------------------------------------------------------------
struct HashGrid {
  const std::vector<F3>* Particles = nullptr;
  unsigned int ParticlesNum = 0;
  float Radius = 0, CellSize = 0;
  float Bounding[6];
  unsigned int XYZCellNum[3];
  unsigned long long CellNum = 0;
  std::vector<long long> HashList;
  std::vector<int> IndexList;
  std::vector<long long> Keys;  // per particle, kept for dumps
  std::map<long long, int> StartList, EndList;
  // variable radius: one grid per radius bin over the bin's particles
  // (src/hash_grid.cpp:36-69); indices below are bin-local, PIndexes maps
  // them to particles
  bool var = false;
  std::vector<int> PIndexes;
  int RadiusId = -1;

  // src/hash_grid.cpp:4-34
  void init(const std::vector<F3>* particles, const float* bounding, float radius,
            float inf_factor, bool std_sort) {
    Particles = particles;
    ParticlesNum = (unsigned int)particles->size();
    Radius = radius;
    CellSize = radius * inf_factor;
    for (int i = 0; i < 3; ++i) {
      float length = (std::ceil((bounding[i * 2 + 1] - bounding[i * 2]) / CellSize)) * CellSize;
      float center = (bounding[i * 2] + bounding[i * 2 + 1]) / 2;
      Bounding[i * 2] = center - length / 2;
      Bounding[i * 2 + 1] = center + length / 2;
    }
    for (int i = 0; i < 3; ++i)
      XYZCellNum[i] =
          std::max(int(std::ceil((Bounding[i * 2 + 1] - Bounding[i * 2]) / CellSize)), 1);
    CellNum = (long long)XYZCellNum[0] * (long long)XYZCellNum[1] * (long long)XYZCellNum[2];
    HashList.assign(ParticlesNum, 0);
    IndexList.assign(ParticlesNum, 0);
    BuildTable(std_sort);
    HashList.clear();
  }

  // src/hash_grid.cpp:36-69: the grid of one radius bin; the cell size is
  // the bin's largest radius times inf_factor, over the bin's bounding box
  void init_var(const std::vector<F3>* particles, const std::vector<float>& radiuses,
                const std::vector<int>& pIndexes, const float* bounding, int radiusId, float inf_factor,
                bool std_sort) {
    var = true;
    Particles = particles;
    PIndexes = pIndexes;
    ParticlesNum = (unsigned int)PIndexes.size();
    RadiusId = radiusId;
    Radius = radiuses[radiusId];
    CellSize = Radius * inf_factor;
    for (int i = 0; i < 3; ++i) {
      float length = ((std::ceil((bounding[i * 2 + 1] - bounding[i * 2]) / CellSize)) * CellSize);
      float center = (bounding[i * 2] + bounding[i * 2 + 1]) / 2;
      Bounding[i * 2] = center - length / 2;
      Bounding[i * 2 + 1] = center + length / 2;
    }
    for (int i = 0; i < 3; ++i)
      XYZCellNum[i] =
          std::max(int(std::ceil((Bounding[i * 2 + 1] - Bounding[i * 2]) / CellSize)), 1);
    CellNum = (long long)XYZCellNum[0] * (long long)XYZCellNum[1] * (long long)XYZCellNum[2];
    HashList.assign(ParticlesNum, 0);
    IndexList.assign(ParticlesNum, 0);
    BuildTable(std_sort);
    HashList.clear();
  }

  // src/hash_grid.cpp:71-85.  The reference's std::sort leaves the order of
  // equal keys unspecified; by default the oracle keeps particle-index order
  // inside a cell (stable sort), PIO_STD_SORT uses std::sort as written.
  void BuildTable(bool std_sort) {
    CalcHashList();
    Keys = HashList;
    auto cmp = [&](const int& a, const int& b) { return HashList[a] < HashList[b]; };
    if (std_sort)
      std::sort(IndexList.begin(), IndexList.end(), cmp);
    else
      std::stable_sort(IndexList.begin(), IndexList.end(), cmp);
    std::vector<long long> temp(HashList);
    for (unsigned int i = 0; i < ParticlesNum; i++) HashList[i] = temp[IndexList[i]];
    FindStartEnd();
  }

  // src/hash_grid.cpp:87-101
  void CalcHashList() {
    int xyz[3];
    for (size_t index = 0; index < ParticlesNum; index++) {
      CalcXYZIdx((*Particles)[var ? PIndexes[index] : index].data(), xyz);
      HashList[index] = CalcCellHash(xyz);
      IndexList[index] = (int)index;
    }
  }

  // src/hash_grid.cpp:103-122.  Start/end count only non-negative keys, while
  // GetInCellList indexes IndexList, which still holds the key -1 particles at
  // its front: the reference's offsets are shifted by their number.  Kept.
  void FindStartEnd() {
    int hash, count = 0, previous = -1;
    for (size_t index = 0; index < ParticlesNum; index++) {
      hash = (int)HashList[index];
      if (hash < 0) continue;
      if (hash != previous) {
        StartList[hash] = count;
        previous = hash;
      }
      count++;
      EndList[hash] = count;
    }
  }

  // src/hash_grid.cpp:124-129 (int() truncates toward zero)
  void CalcXYZIdx(const float* pos, int* xyz) const {
    for (int i = 0; i < 3; i++) xyz[i] = int((pos[i] - Bounding[i * 2]) / CellSize);
  }

  // src/hash_grid.cpp:131-139 (int compared with unsigned, as written)
  long long CalcCellHash(const int* xyz) const {
    if (xyz[0] < 0 || (unsigned)xyz[0] >= XYZCellNum[0] || xyz[1] < 0 ||
        (unsigned)xyz[1] >= XYZCellNum[1] || xyz[2] < 0 || (unsigned)xyz[2] >= XYZCellNum[2])
      return -1;
    return (long long)xyz[2] * (long long)XYZCellNum[0] * (long long)XYZCellNum[1] +
           (long long)xyz[1] * (long long)XYZCellNum[0] + (long long)xyz[0];
  }

  // src/hash_grid.cpp:141-162
  void GetInCellList(const long long hash, std::vector<int>& out) {
    int startIndex, endIndex;
    auto s = StartList.find(hash);
    auto e = EndList.find(hash);
    if (s != StartList.end() && e != EndList.end()) {
      startIndex = s->second;
      endIndex = e->second;
    } else {
      return;
    }
    for (int c = startIndex; c < endIndex; c++) out.push_back(var ? PIndexes[IndexList[c]] : IndexList[c]);
  }

  // src/hash_grid.cpp:164-194 (x outer, z inner)
  void GetInBoxParticles(F3 box1, F3 box2, std::vector<int>& insides) {
    int mn[3], mx[3];
    for (int i = 0; i < 3; i++) {
      box1[i] = std::max(box1[i], Bounding[2 * i]);
      box2[i] = std::min(box2[i], Bounding[2 * i + 1]);
    }
    CalcXYZIdx(box1.data(), mn);
    CalcXYZIdx(box2.data(), mx);
    for (int x = mn[0] - 1; x <= mx[0] + 1; x++)
      for (int y = mn[1] - 1; y <= mx[1] + 1; y++)
        for (int z = mn[2] - 1; z <= mx[2] + 1; z++) {
          int c[3] = {x, y, z};
          long long h = CalcCellHash(c);
          if (h < 0) continue;
          GetInCellList(h, insides);
        }
  }

  // src/hash_grid.cpp:196-214 (z outer, x inner)
  void GetPIdxList(const float* pos, std::vector<int>& out) {
    int xyz[3];
    CalcXYZIdx(pos, xyz);
    for (int z = -1; z <= 1; z++)
      for (int y = -1; y <= 1; y++)
        for (int x = -1; x <= 1; x++) {
          int c[3] = {xyz[0] + x, xyz[1] + y, xyz[2] + z};
          long long h = CalcCellHash(c);
          if (h < 0) continue;
          GetInCellList(h, out);
        }
  }
};

// ---------------------------------------------------------------------------
// MultiLevelSearcher (src/multi_level_reseacher.cpp:6-117): particles binned
// by radius into bins of width about minRadius / 2, a HashGrid per non-empty
// bin.  GetNeighbors is the reference's with its query switched on.  Two
// departures where the reference's dead code is broken: it indexes its
// searcher list with the bin index, which picks the wrong grid once an
// earlier bin is empty (its GetInBoxParticles keeps a separate searcher
// counter), and its GetInBoxParticles maps the grid's answers, which are
// already particle indices (HashGrid::GetInCellList, src/hash_grid.cpp:
// 155-160), through the bin's index list a second time.  Here each non-empty
// bin's grid is queried in bin order and its particle indices are kept.
// ---------------------------------------------------------------------------
struct MultiLevelSearcher {
  float maxRadius = 0, minRadius = 0, avgRadius = 0;
  std::vector<std::vector<int>> sortedIndex;
  std::vector<HashGrid> searchers;  // one per non-empty bin, in bin order

  void init(const std::vector<F3>* particles, const std::vector<float>& radiuses, float inf_factor,
            bool std_sort) {
    maxRadius = *std::max_element(radiuses.begin(), radiuses.end()) * 1.01;
    minRadius = *std::min_element(radiuses.begin(), radiuses.end()) * 0.99;
    std::vector<std::pair<float, float>> bin_bounds;
    float bin_extent = minRadius * 0.5;
    int bins = std::max(int(std::ceil((maxRadius - minRadius) / bin_extent)), 1);
    bin_extent = (maxRadius - minRadius) / bins;
    for (int i = 0; i < bins; i++)
      bin_bounds.push_back({minRadius + (i * bin_extent), std::min(minRadius + ((i + 1) * bin_extent), maxRadius)});
    auto whichBin = [&](const float r) {
      for (size_t k = 0; k < bin_bounds.size(); ++k)
        if (r >= bin_bounds[k].first && r <= bin_bounds[k].second) return (int)k;
      return -1;
    };
    sortedIndex.assign(bins, {});
    avgRadius = 0;
    for (size_t i = 0; i < radiuses.size(); i++) {
      sortedIndex[whichBin(radiuses[i])].push_back((int)i);
      avgRadius += radiuses[i];
    }
    avgRadius /= radiuses.size();
    if (avgRadius < minRadius) avgRadius = minRadius;
    if (avgRadius > maxRadius) avgRadius = maxRadius;
    searchers.clear();
    for (int i = 0; i < bins; i++) {
      if (sortedIndex[i].empty()) continue;
      float b[6] = {FLT_MAX, -FLT_MAX, FLT_MAX, -FLT_MAX, FLT_MAX, -FLT_MAX};
      for (int pI : sortedIndex[i])
        for (int k = 0; k < 3; ++k) {
          if ((*particles)[pI][k] < b[2 * k]) b[2 * k] = (*particles)[pI][k];
          if ((*particles)[pI][k] > b[2 * k + 1]) b[2 * k + 1] = (*particles)[pI][k];
        }
      // the bin's largest radius (std::max_element: the first of equal maxima)
      int rid = *std::max_element(sortedIndex[i].begin(), sortedIndex[i].end(),
                                  [&](int a, int c) { return radiuses[a] < radiuses[c]; });
      searchers.emplace_back();
      searchers.back().init_var(particles, radiuses, sortedIndex[i], b, rid, inf_factor, std_sort);
    }
  }

  void GetNeighbors(const float* pos, std::vector<int>& out) {
    for (HashGrid& g : searchers) g.GetPIdxList(pos, out);
  }

  void GetInBoxParticles(const F3& box1, const F3& box2, std::vector<int>& insides) {
    for (HashGrid& g : searchers) g.GetInBoxParticles(box1, box2, insides);
  }
};

// ---------------------------------------------------------------------------
// Eigen::JacobiSVD<Matrix3> restated (two-sided Jacobi, Eigen 3.4
// Eigen/src/SVD/JacobiSVD.h compute() for square input, real_2x2_jacobi_svd,
// JacobiRotation::makeJacobi).  Used by compute_G_Yus
// (src/evaluator.cpp:627).
// ---------------------------------------------------------------------------
template <class R>
struct Rot {
  R c, s;
};

template <class R>
static Rot<R> make_jacobi(R x, R y, R z) {
  Rot<R> r;
  R deno = R(2) * std::abs(y);
  if (deno < std::numeric_limits<R>::min()) {
    r.c = R(1);
    r.s = R(0);
  } else {
    R tau = (x - z) / deno;
    R w = std::sqrt(tau * tau + R(1));
    R t;
    if (tau > R(0))
      t = R(1) / (tau + w);
    else
      t = R(1) / (tau - w);
    R sign_t = t > R(0) ? R(1) : R(-1);
    R n = R(1) / std::sqrt(t * t + R(1));
    r.s = -sign_t * (y / std::abs(y)) * std::abs(t) * n;
    r.c = n;
  }
  return r;
}

// rows p,q of A: x' = c x + s y, y' = -s x + c y
template <class R>
static void rot_left(M3<R>& A, int p, int q, Rot<R> j) {
  for (int i = 0; i < 3; ++i) {
    R xi = A(p, i), yi = A(q, i);
    A(p, i) = j.c * xi + j.s * yi;
    A(q, i) = -j.s * xi + j.c * yi;
  }
}

// cols p,q of A with rotation j applied as x' = c x + s y, y' = -s x + c y
template <class R>
static void rot_cols(M3<R>& A, int p, int q, Rot<R> j) {
  for (int i = 0; i < 3; ++i) {
    R xi = A(i, p), yi = A(i, q);
    A(i, p) = j.c * xi + j.s * yi;
    A(i, q) = -j.s * xi + j.c * yi;
  }
}

template <class R>
static void jacobi_svd3(const M3<R>& Ain, M3<R>& U, V3<R>& S, M3<R>& V) {
  const R precision = R(2) * std::numeric_limits<R>::epsilon();
  const R considerAsZero = std::numeric_limits<R>::min();
  R scale = R(0);
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) scale = std::max(scale, std::abs(Ain(i, j)));
  if (scale == R(0)) scale = R(1);
  M3<R> W;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      W(i, j) = Ain(i, j) / scale;
      U(i, j) = V(i, j) = (i == j) ? R(1) : R(0);
    }
  R maxDiag = std::max(std::abs(W(0, 0)), std::max(std::abs(W(1, 1)), std::abs(W(2, 2))));
  bool finished = false;
  int sweeps = 0;
  while (!finished && sweeps < 64) {
    finished = true;
    ++sweeps;
    for (int p = 1; p < 3; ++p)
      for (int q = 0; q < p; ++q) {
        R threshold = std::max(considerAsZero, precision * maxDiag);
        if (std::abs(W(p, q)) > threshold || std::abs(W(q, p)) > threshold) {
          finished = false;
          // real_2x2_jacobi_svd
          R m00 = W(p, p), m01 = W(p, q), m10 = W(q, p), m11 = W(q, q);
          Rot<R> rot1;
          R t = m00 + m11;
          R d = m10 - m01;
          if (std::abs(d) < std::numeric_limits<R>::min()) {
            rot1.s = R(0);
            rot1.c = R(1);
          } else {
            R u = t / d;
            R tmp = std::sqrt(R(1) + u * u);
            rot1.s = R(1) / tmp;
            rot1.c = u / tmp;
          }
          // m.applyOnTheLeft(0,1,rot1)
          R a00 = rot1.c * m00 + rot1.s * m10, a01 = rot1.c * m01 + rot1.s * m11;
          R a10 = -rot1.s * m00 + rot1.c * m10, a11 = -rot1.s * m01 + rot1.c * m11;
          (void)a10;
          Rot<R> jr = make_jacobi<R>(a00, a01, a11);
          // j_left = rot1 * j_right.transpose(); transpose = (c, -s)
          Rot<R> jrt{jr.c, -jr.s};
          Rot<R> jl{rot1.c * jrt.c - rot1.s * jrt.s, rot1.c * jrt.s + rot1.s * jrt.c};
          rot_left(W, p, q, jl);
          rot_cols(U, p, q, jl);
          rot_cols(W, p, q, Rot<R>{jr.c, -jr.s});
          rot_cols(V, p, q, Rot<R>{jr.c, -jr.s});
          maxDiag = std::max(maxDiag, std::max(std::abs(W(p, p)), std::abs(W(q, q))));
        }
      }
  }
  for (int i = 0; i < 3; ++i) {
    R a = W(i, i);
    S[i] = std::abs(a);
    if (a < R(0))
      for (int k = 0; k < 3; ++k) U(k, i) = -U(k, i);
  }
  for (int i = 0; i < 3; ++i) S[i] *= scale;
  for (int i = 0; i < 3; ++i) {
    int pos = i;
    R mx = S[i];
    for (int k = i + 1; k < 3; ++k)
      if (S[k] > mx) {
        mx = S[k];
        pos = k;
      }
    if (mx == R(0)) break;
    if (pos != i) {
      std::swap(S[i], S[pos]);
      for (int k = 0; k < 3; ++k) {
        std::swap(U(k, i), U(k, pos));
        std::swap(V(k, i), V(k, pos));
      }
    }
  }
}

// Matrix3::determinant: cofactors along the first row.
template <class R>
static R det3(const M3<R>& m) {
  auto h = [&](int a, int b, int c) { return m(0, a) * (m(1, b) * m(2, c) - m(1, c) * m(2, b)); };
  return h(0, 1, 2) - h(1, 0, 2) + h(2, 0, 1);
}

// Matrix4::inverse by the adjugate; singular input gives non-finite entries.
template <class R>
static void inv4(const R a[4][4], R out[4][4]) {
  R m[16], inv[16];
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) m[i * 4 + j] = a[i][j];
  inv[0] = m[5] * m[10] * m[15] - m[5] * m[11] * m[14] - m[9] * m[6] * m[15] +
           m[9] * m[7] * m[14] + m[13] * m[6] * m[11] - m[13] * m[7] * m[10];
  inv[4] = -m[4] * m[10] * m[15] + m[4] * m[11] * m[14] + m[8] * m[6] * m[15] -
           m[8] * m[7] * m[14] - m[12] * m[6] * m[11] + m[12] * m[7] * m[10];
  inv[8] = m[4] * m[9] * m[15] - m[4] * m[11] * m[13] - m[8] * m[5] * m[15] +
           m[8] * m[7] * m[13] + m[12] * m[5] * m[11] - m[12] * m[7] * m[9];
  inv[12] = -m[4] * m[9] * m[14] + m[4] * m[10] * m[13] + m[8] * m[5] * m[14] -
            m[8] * m[6] * m[13] - m[12] * m[5] * m[10] + m[12] * m[6] * m[9];
  inv[1] = -m[1] * m[10] * m[15] + m[1] * m[11] * m[14] + m[9] * m[2] * m[15] -
           m[9] * m[3] * m[14] - m[13] * m[2] * m[11] + m[13] * m[3] * m[10];
  inv[5] = m[0] * m[10] * m[15] - m[0] * m[11] * m[14] - m[8] * m[2] * m[15] +
           m[8] * m[3] * m[14] + m[12] * m[2] * m[11] - m[12] * m[3] * m[10];
  inv[9] = -m[0] * m[9] * m[15] + m[0] * m[11] * m[13] + m[8] * m[1] * m[15] -
           m[8] * m[3] * m[13] - m[12] * m[1] * m[11] + m[12] * m[3] * m[9];
  inv[13] = m[0] * m[9] * m[14] - m[0] * m[10] * m[13] - m[8] * m[1] * m[14] +
            m[8] * m[2] * m[13] + m[12] * m[1] * m[10] - m[12] * m[2] * m[9];
  inv[2] = m[1] * m[6] * m[15] - m[1] * m[7] * m[14] - m[5] * m[2] * m[15] +
           m[5] * m[3] * m[14] + m[13] * m[2] * m[7] - m[13] * m[3] * m[6];
  inv[6] = -m[0] * m[6] * m[15] + m[0] * m[7] * m[14] + m[4] * m[2] * m[15] -
           m[4] * m[3] * m[14] - m[12] * m[2] * m[7] + m[12] * m[3] * m[6];
  inv[10] = m[0] * m[5] * m[15] - m[0] * m[7] * m[13] - m[4] * m[1] * m[15] +
            m[4] * m[3] * m[13] + m[12] * m[1] * m[7] - m[12] * m[3] * m[5];
  inv[14] = -m[0] * m[5] * m[14] + m[0] * m[6] * m[13] + m[4] * m[1] * m[14] -
            m[4] * m[2] * m[13] - m[12] * m[1] * m[6] + m[12] * m[2] * m[5];
  inv[3] = -m[1] * m[6] * m[11] + m[1] * m[7] * m[10] + m[5] * m[2] * m[11] -
           m[5] * m[3] * m[10] - m[9] * m[2] * m[7] + m[9] * m[3] * m[6];
  inv[7] = m[0] * m[6] * m[11] - m[0] * m[7] * m[10] - m[4] * m[2] * m[11] +
           m[4] * m[3] * m[10] + m[8] * m[2] * m[7] - m[8] * m[3] * m[6];
  inv[11] = -m[0] * m[5] * m[11] + m[0] * m[7] * m[9] + m[4] * m[1] * m[11] -
            m[4] * m[3] * m[9] - m[8] * m[1] * m[7] + m[8] * m[3] * m[5];
  inv[15] = m[0] * m[5] * m[10] - m[0] * m[6] * m[9] - m[4] * m[1] * m[10] +
            m[4] * m[2] * m[9] + m[8] * m[1] * m[6] - m[8] * m[2] * m[5];
  R det = m[0] * inv[0] + m[1] * inv[4] + m[2] * inv[8] + m[3] * inv[12];
  R invdet = R(1) / det;
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) out[i][j] = inv[i * 4 + j] * invdet;
}

// ---------------------------------------------------------------------------
// Evaluator, constant radius, anisotropic B-spline
// (src/evaluator.cpp, globals of src/main.cpp:29-52: USE_ANI=1, USE_POLY6=0,
// CALC_P_NORMAL=1; splash particles only with PIO_SPLASH, which switches on
// the GlobalSplash marking commented out at :675,690)
// ---------------------------------------------------------------------------
template <class R>
struct Evaluator {
  HashGrid* grid = nullptr;
  MultiLevelSearcher* searcher = nullptr;  // variable radius (grid unused)
  const std::vector<float>* GlobalRadius = nullptr;
  std::vector<R> GlobalInflunce2, GlobalSigma;
  void neighbors(const float* p, std::vector<int>& out) {
    if (searcher)
      searcher->GetNeighbors(p, out);
    else
      grid->GetPIdxList(p, out);
  }
  R influ2(int j) const { return searcher ? GlobalInflunce2[j] : Influnce2; }
  R sigma(int j) const { return searcher ? GlobalSigma[j] : Sigma; }
  R rad(int j) const { return searcher ? (R)(*GlobalRadius)[j] : Radius; }
  const std::vector<F3>* P = nullptr;
  int N = 0;
  float _NEIGHBOR_FACTOR = 4.0f;
  float _SMOOTH_FACTOR = 2.0f;
  float _XMEAN_DELTA = 0.0f;
  R Radius = 0, Influnce2 = 0, Sigma = 0;
  R _MAX_SCALAR = -1, _ISO_VALUE = 0;
  std::vector<V3<R>> xMeans, Normals;
  std::vector<M3<R>> Gs;
  std::vector<R> Dets;
  bool splash_on = false;
  std::vector<char> GlobalSplash;
  // src/evaluator.cpp:254-261
  bool CheckSplash(int j) const { return splash_on && GlobalSplash[j]; }
  std::atomic<long long> nEvals{0}, nPairs{0};

  // src/evaluator.cpp:5-58 (constant-radius branch).  Influnce2 and Sigma use
  // the default smoothing factor 2: Run() sets the caller's factor only after
  // construction (src/surface_reconstructor.cpp:432-433).
  void init(HashGrid* g, const std::vector<F3>* p, float radius) {
    grid = g;
    P = p;
    N = (int)p->size();
    Radius = radius;
    if (sizeof(R) == sizeof(float)) {
      Influnce2 = (R)(float)std::pow(radius * _SMOOTH_FACTOR, 2);
      Sigma = (R)(float)(1 / std::pow(radius * _SMOOTH_FACTOR, 6));
    } else {
      Influnce2 = (R)std::pow((double)(radius * _SMOOTH_FACTOR), 2);
      Sigma = (R)(1 / std::pow((double)(radius * _SMOOTH_FACTOR), 6));
    }
    _XMEAN_DELTA = (float)0.9;
    if (searcher) {
      // src/evaluator.cpp:16-29: per particle, from that particle's radius
      GlobalInflunce2.resize(N);
      GlobalSigma.resize(N);
      for (int i = 0; i < N; ++i) {
        const float smooth = (*GlobalRadius)[i] * _SMOOTH_FACTOR;
        if (sizeof(R) == sizeof(float)) {
          GlobalInflunce2[i] = (R)(float)std::pow(smooth, 2);
          GlobalSigma[i] = (R)(float)(1 / std::pow(smooth, 6));
        } else {
          GlobalInflunce2[i] = (R)std::pow((double)smooth, 2);
          GlobalSigma[i] = (R)(1 / std::pow((double)smooth, 6));
        }
      }
    }
    Normals.assign(N, V3<R>{{0, 0, 0}});
    GlobalSplash.assign(N, 0);
    xMeans.resize(N);
    Gs.resize(N);
    Dets.resize(N);
  }

  V3<R> pos(int i) const { return V3<R>{{(R)(*P)[i][0], (R)(*P)[i][1], (R)(*P)[i][2]}}; }

  // src/evaluator.cpp:383-396.  The polynomial is evaluated in double (pow and
  // the double literals promote), then returned as R.
  static R Bspline_kernel(R ratio, R sigma) {
    if (ratio < 2) {
      if (ratio <= 1) {
        return (R)(sigma * (1 - 1.5 * std::pow((double)ratio, 2) + 0.75 * std::pow((double)ratio, 3)));
      } else {
        R tmq = 2 - ratio;
        return (R)(sigma * (0.25 * std::pow((double)tmq, 3)));
      }
    }
    return (R)0.0f;
  }

  // src/evaluator.cpp:751-766
  static R wij(R d, R h) {
    if (d < h) {
      if (d < h / 2) {
        R hmd = h - d;
        return (R)(1 - (6 * std::pow((double)d, 2) / std::pow((double)h, 3) * (double)hmd));
      } else {
        R hmd = h - d;
        return (R)(2 / std::pow((double)h, 3) * std::pow((double)hmd, 3));
      }
    }
    return (R)0.0;
  }

  // src/evaluator.cpp:437-453
  R AnisotropicInterpolate(int j, const V3<R>& diff) const {
    V3<R> gd = matvec(Gs[j], diff);
    R ratio = std::sqrt(sqnorm3<R>(gd[0], gd[1], gd[2]) / influ2(j));
    R k = Bspline_kernel(ratio, sigma(j));
    return Dets[j] * k;
  }

  // src/evaluator.cpp:455-463 with poly6_gradient_kernel (:408-415)
  V3<R> AnisotropicInterpolateGrad(int j, const V3<R>& diff) const {
    V3<R> gd = matvec(Gs[j], diff);
    R d2 = sqnorm3<R>(gd[0], gd[1], gd[2]);
    R h2 = influ2(j);
    V3<R> g;
    for (int k = 0; k < 3; ++k)
      g[k] = sigma(j) * (-6 * gd[k]) * (d2 > h2 ? (R)0.0f : ((h2 - d2) * (h2 - d2)));
    for (int k = 0; k < 3; ++k) g[k] = Dets[j] * g[k];
    return g;
  }

  // src/evaluator.cpp:60-87
  R SingleEval(const float* p) {
    R scalar = 0;
    std::vector<int> nb;
    neighbors(p, nb);
    V3<R> q{{(R)p[0], (R)p[1], (R)p[2]}};
    for (int j : nb) {
      if (CheckSplash(j)) continue;
      V3<R> diff{{q[0] - xMeans[j][0], q[1] - xMeans[j][1], q[2] - xMeans[j][2]}};
      scalar += AnisotropicInterpolate(j, diff);
    }
    nEvals.fetch_add(1, std::memory_order_relaxed);
    nPairs.fetch_add((long long)nb.size(), std::memory_order_relaxed);
    return _ISO_VALUE - scalar;
  }

  // src/evaluator.cpp:89-125
  void SingleEvalWithGrad(const float* p, R& scalar, V3<R>& grad) {
    if (_MAX_SCALAR >= 0) {
      scalar = 0;
      grad = V3<R>{{0, 0, 0}};
    }
    std::vector<int> nb;
    neighbors(p, nb);
    V3<R> q{{(R)p[0], (R)p[1], (R)p[2]}};
    for (int j : nb) {
      if (CheckSplash(j)) continue;
      V3<R> diff{{q[0] - xMeans[j][0], q[1] - xMeans[j][1], q[2] - xMeans[j][2]}};
      scalar += AnisotropicInterpolate(j, diff);
      V3<R> g = AnisotropicInterpolateGrad(j, diff);
      for (int k = 0; k < 3; ++k) grad[k] += g[k];
    }
    scalar = _ISO_VALUE - scalar;
  }

  // src/evaluator.cpp:465-512
  void compute_xMeans(int p, const std::vector<int>& temp, int& n_neighbors, V3<R>& xMean) {
    R pD2 = Influnce2;
    R wSum = 0;
    V3<R> pp = pos(p);
    for (int n : temp) {
      if (n == p) continue;
      R nR = rad(n);
      R nD = (R)(_SMOOTH_FACTOR * (double)nR * 1.6);
      R nD2 = nD * nD;
      R nI = nR * (R)_NEIGHBOR_FACTOR;
      R nI2 = nI * nI;
      V3<R> pn = pos(n);
      R d2 = sqnorm3<R>(pn[0] - pp[0], pn[1] - pp[1], pn[2] - pp[2]);
      if (d2 >= nI2) continue;
      R d = std::sqrt(d2);
      R wj = wij(d, nI);
      wSum += wj;
      for (int k = 0; k < 3; ++k) xMean[k] += pn[k] * wj;
      ++n_neighbors;
      (void)pD2;
      (void)nD2;
    }
    if (wSum > 0) {
      for (int k = 0; k < 3; ++k) xMean[k] /= wSum;
      R a = (R)(1 - _XMEAN_DELTA), b = (R)_XMEAN_DELTA;
      if (sizeof(R) == sizeof(double)) {
        a = (R)(1 - 0.9);
        b = (R)0.9;
      }
      for (int k = 0; k < 3; ++k) xMean[k] = pp[k] * a + xMean[k] * b;
    } else {
      xMean = pp;
    }
  }

  // src/evaluator.cpp:585-654
  void compute_G_Yus(int p, V3<R> xMean, const std::vector<int>& nb, M3<R>& G) {
    R wSum = 0;
    M3<R> cov;
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) cov(i, j) = (i == j) ? influ2(p) : (R)0;
    for (int n : nb) {
      R nR = rad(n);
      R nI = nR * (R)_NEIGHBOR_FACTOR;
      R nI2 = nI * nI;
      const V3<R>& xn = xMeans[n];
      const V3<R>& xp = xMeans[p];
      R d2 = sqnorm3<R>(xn[0] - xp[0], xn[1] - xp[1], xn[2] - xp[2]);
      if (d2 >= nI2) continue;
      R d = std::sqrt(sqnorm3<R>(xp[0] - xn[0], xp[1] - xn[1], xp[2] - xn[2]));
      R wj = wij(d, nI);
      wSum += wj;
      V3<R> wd{{xn[0] - xMean[0], xn[1] - xMean[1], xn[2] - xMean[2]}};
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) cov(i, j) += (wd[i] * wd[j]) * wj;
    }
    if (!(wSum > R(0))) {
      // no candidate within 4r: the reference divides by zero here (its G is
      // NaN); the identity is used, as for particles with <= 2 candidates
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) G(i, j) = (i == j) ? R(1) : R(0);
      return;
    }
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) cov(i, j) /= wSum;
    M3<R> u, v;
    V3<R> w;
    jacobi_svd3<R>(cov, u, w, v);
    for (int k = 0; k < 3; ++k) w[k] = std::abs(w[k]);
    R maxSV = std::max(w[0], std::max(w[1], w[2]));
    const R kr = 4.0;
    for (int k = 0; k < 3; ++k) w[k] = std::max(w[k], maxSV / kr);
    R invS[3];
    for (int k = 0; k < 3; ++k) invS[k] = R(1) / w[k];
    R scale = (R)std::pow((double)(w[0] * w[1] * w[2]), 1.0 / 3.0);
    // (v * invSigma) * u^T, then * scale
    M3<R> vs;
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j)
        vs(i, j) = sum3<R>(v(i, 0) * (j == 0 ? invS[0] : R(0)), v(i, 1) * (j == 1 ? invS[1] : R(0)),
                           v(i, 2) * (j == 2 ? invS[2] : R(0)));
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j)
        G(i, j) = sum3<R>(vs(i, 0) * u(j, 0), vs(i, 1) * u(j, 1), vs(i, 2) * u(j, 2)) * scale;
  }

  // the pass-1 branches for <= 2 candidates or neighbours
  // (src/evaluator.cpp:670-697): identity G; a splash particle with the
  // marking switched on, whose G pass 2 then leaves alone
  void splash_mark(int p) {
    if (!splash_on) return;
    GlobalSplash[p] = 1;
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) Gs[p](i, j) = (i == j) ? R(1) : R(0);
    Dets[p] = det3<R>(Gs[p]);
  }

  // src/evaluator.cpp:656-749
  void compute_Gs_xMeans() {
#pragma omp parallel for
    for (int p = 0; p < N; p++) {
      std::vector<int> temp;
      int nn = 0;
      V3<R> xMean{{0, 0, 0}};
      neighbors((*P)[p].data(), temp);
      if (temp.size() <= 2) {
        xMeans[p] = pos(p);
        splash_mark(p);
        continue;
      }
      compute_xMeans(p, temp, nn, xMean);
      xMeans[p] = xMean;
      if (nn <= 2) splash_mark(p);
    }
#pragma omp parallel for
    for (int p = 0; p < N; p++) {
      if (CheckSplash(p)) continue;
      std::vector<int> temp;
      M3<R> G;
      neighbors((*P)[p].data(), temp);
      compute_G_Yus(p, xMeans[p], temp, G);
      Gs[p] = G;
      Dets[p] = det3<R>(G);
    }
  }

  // src/evaluator.cpp:272-291
  void CalculateMaxScalarConstR() {
    const float sqrt2 = 1.4142135623730950488016887242097f;
    const float sqrt3 = 1.7320508075688772935274463415059f;
    R k = 0;
    k += Bspline_kernel(0.0, Sigma);
    k += Bspline_kernel(1.0, Sigma) * 6;
    k += Bspline_kernel(sizeof(R) == sizeof(float) ? (R)sqrt2 : (R)1.4142135623730950488, Sigma) * 12;
    k += Bspline_kernel(sizeof(R) == sizeof(float) ? (R)sqrt3 : (R)1.7320508075688772935, Sigma) * 8;
    _MAX_SCALAR = k;
  }

  // src/evaluator.cpp:323-335
  void RecommendIsoValueConstR() { _ISO_VALUE = Bspline_kernel((R)0.01, Sigma); }

  // src/evaluator.cpp:293-321: the largest MaxScalar over the searchers'
  // radius particles
  void CalculateMaxScalarVarR() {
    const float sqrt2 = 1.4142135623730950488016887242097f;
    const float sqrt3 = 1.7320508075688772935274463415059f;
    R mx = 0;
    for (const HashGrid& g : searcher->searchers) {
      const R sg = GlobalSigma[g.RadiusId];
      R k = 0;
      k += Bspline_kernel(0.0, sg);
      k += Bspline_kernel(1.0, sg) * 6;
      k += Bspline_kernel(sizeof(R) == sizeof(float) ? (R)sqrt2 : (R)1.4142135623730950488, sg) * 12;
      k += Bspline_kernel(sizeof(R) == sizeof(float) ? (R)sqrt3 : (R)1.7320508075688772935, sg) * 8;
      if (k > mx) mx = k;
    }
    _MAX_SCALAR = mx;
  }

  // src/evaluator.cpp:337-361: the largest Bspline_kernel(0.25) over the
  // searchers' radius particles
  void RecommendIsoValueVarR() {
    R rec = 0;
    for (const HashGrid& g : searcher->searchers) {
      const R v = Bspline_kernel((R)0.25, GlobalSigma[g.RadiusId]);
      if (v > rec) rec = v;
    }
    _ISO_VALUE = rec;
  }

  // src/evaluator.cpp:363-375
  void CalcParticlesNormal() {
#pragma omp parallel for
    for (int p = 0; p < N; p++) {
      R s = 0;
      if (!CheckSplash(p)) SingleEvalWithGrad((*P)[p].data(), s, Normals[p]);
    }
  }
};

// ---------------------------------------------------------------------------
// Octree node (include/iso_method_ours.h:30-78, src/iso_method_ours.cpp)
// ---------------------------------------------------------------------------
enum : char { EMPTY = 0, INTERNAL = 1, LEAF = 2, UNCERTAIN = 3 };

template <class R>
struct TNode {
  float center[3];
  float half_length;
  R node[4] = {0, 0, 0, 0};
  char depth = 0;
  char type = UNCERTAIN;
  unsigned long long id = 0;
  int children[8] = {-1, -1, -1, -1, -1, -1, -1, -1};
  int parent = -1;
  float curv = 0;
  bool signchange = false;
  bool is_leaf() const { return type == LEAF || type == EMPTY; }
};

template <class R>
struct DualGrid {
  DmcProc proc;
  int grid[8];
};

template <class R>
struct DualCell {
  float vertices[12][3];
  std::vector<std::array<int, 3>> faces;
};

// ---------------------------------------------------------------------------
// SurfReconstructor (src/surface_reconstructor.cpp)
// ---------------------------------------------------------------------------
struct FrameBase {
  virtual ~FrameBase() {}
  std::vector<F3> P;
  float radius = 0, smooth_factor = 2.0f, iso_factor = 1.9f;
  int flags = 0;
  int stage_done = 0;
  double seconds[6] = {0, 0, 0, 0, 0, 0};
  HashGrid grid;
  // variable radius (SurfReconstructor with per-particle radii): the radii
  // and the multi-level searcher in place of the grid
  bool varR = false;
  std::vector<float> radii;
  MultiLevelSearcher searcher;
  float BoundingBox[6];
  float RawBox[6];  // loadRootBox's box before resizeRootBoxConstR (UniformGrid reads it)
  bool single_layer = false;
  int DEPTH_MAX = 6, DEPTH_MIN = 5;
  float RootHalfLength = 0;
  float RootCenter[3] = {0, 0, 0};
  long long nDual = 0;
  std::atomic<long long> nBisect{0};
  // mesh (src/global.cpp:13-53)
  std::vector<F3> mverts;
  std::vector<std::array<unsigned long long, 2>> mvkeys;
  std::vector<std::array<int, 3>> mtris;
  virtual int stage(int s) = 0;
  virtual long long counter(int w) const = 0;
};

template <class R>
struct Frame : FrameBase {
  Evaluator<R> ev;
  std::vector<TNode<R>> nodes;
  std::vector<DualGrid<R>> dual_grids;
  std::vector<DualCell<R>> dual_cells;
  DmcProc table[256];
  const int OVERSAMPLE = 2;  // _OVERSAMPLE_QEF, include/surface_reconstructor.h:25

  long long counter(int w) const override {
    if (w == 0) return ev.nEvals.load();
    if (w == 1) return ev.nPairs.load();
    if (w == 2) return nDual;
    if (w == 3) return nBisect.load();
    return -1;
  }

  // src/surface_reconstructor.cpp:30-49
  void loadRootBox() {
    BoundingBox[0] = BoundingBox[2] = BoundingBox[4] = FLT_MAX;
    BoundingBox[1] = BoundingBox[3] = BoundingBox[5] = -FLT_MAX;
    for (const F3& p : P) {
      if (p[0] < BoundingBox[0]) BoundingBox[0] = p[0];
      if (p[0] > BoundingBox[1]) BoundingBox[1] = p[0];
      if (p[1] < BoundingBox[2]) BoundingBox[2] = p[1];
      if (p[1] > BoundingBox[3]) BoundingBox[3] = p[1];
      if (p[2] < BoundingBox[4]) BoundingBox[4] = p[2];
      if (p[2] > BoundingBox[5]) BoundingBox[5] = p[2];
    }
    single_layer = (BoundingBox[0] == BoundingBox[1] || BoundingBox[2] == BoundingBox[3] ||
                    BoundingBox[4] == BoundingBox[5]);
    for (int i = 0; i < 6; ++i) RawBox[i] = BoundingBox[i];
  }

  // src/surface_reconstructor.cpp:97-122
  void resizeRootBoxConstR() {
    float r = radius;
    float maxLen = std::max({(BoundingBox[1] - BoundingBox[0]), (BoundingBox[3] - BoundingBox[2]),
                             (BoundingBox[5] - BoundingBox[4])});
    // all particles at one point: log2(0) leaves the reference's depth
    // undefined; the search then starts at depth 0 (as the library does)
    const float cells = std::ceil(maxLen / r);
    DEPTH_MAX = cells >= 1.0f ? int(std::ceil(std::log2(cells))) : 0;
    float resizeLen = (float)(std::pow(2, DEPTH_MAX) * r);
    while (resizeLen - maxLen < (ev._NEIGHBOR_FACTOR * radius * 2)) {
      DEPTH_MAX++;
      resizeLen = (float)(std::pow(2, DEPTH_MAX) * r);
    }
    RootHalfLength = resizeLen / 2;
    for (int i = 0; i < 3; i++) {
      float center = (BoundingBox[i * 2] + BoundingBox[i * 2 + 1]) / 2;
      BoundingBox[i * 2] = center - RootHalfLength;
      BoundingBox[i * 2 + 1] = center + RootHalfLength;
      RootCenter[i] = center;
    }
    DEPTH_MIN = (DEPTH_MAX - (single_layer ? 1 : 3));
  }

  // src/surface_reconstructor.cpp:124-149
  void resizeRootBoxVarR() {
    const float minR = searcher.minRadius, maxR = searcher.maxRadius;
    float maxLen = std::max({(BoundingBox[1] - BoundingBox[0]), (BoundingBox[3] - BoundingBox[2]),
                             (BoundingBox[5] - BoundingBox[4])});
    const float cells = std::ceil(maxLen / minR);
    DEPTH_MAX = cells >= 1.0f ? int(std::ceil(std::log2(cells))) : 0;
    float resizeLen = (float)(std::pow(2, DEPTH_MAX) * minR);
    while (resizeLen - maxLen < (ev._NEIGHBOR_FACTOR * maxR * 2)) {
      DEPTH_MAX++;
      resizeLen = (float)(std::pow(2, DEPTH_MAX) * minR);
    }
    RootHalfLength = resizeLen / 2;
    for (int i = 0; i < 3; i++) {
      float center = (BoundingBox[i * 2] + BoundingBox[i * 2 + 1]) / 2;
      BoundingBox[i * 2] = center - RootHalfLength;
      BoundingBox[i * 2 + 1] = center + RootHalfLength;
      RootCenter[i] = center;
    }
    const float cmax = std::ceil(maxLen / maxR);
    const int dmaxr = cmax >= 1.0f ? int(std::ceil(std::log2(cmax))) : 0;
    DEPTH_MIN = std::min(dmaxr - 1, DEPTH_MAX - 2);
  }

  // src/surface_reconstructor.cpp:152-222.  min_radius: the smallest radius
  // of the particles inside the grown box (variable radius), else the radius
  void checkEmptyAndCalcCurv(TNode<R>& t, unsigned char& empty, R& curv, float& min_radius) {
    V3<R> norms{{0, 0, 0}};
    R area = 0;
    std::vector<int> insides;
    min_radius = varR ? FLT_MAX : radius;
    F3 box1 = {t.center[0] - t.half_length, t.center[1] - t.half_length, t.center[2] - t.half_length};
    F3 box2 = {t.center[0] + t.half_length, t.center[1] + t.half_length, t.center[2] + t.half_length};
    if (varR)
      searcher.GetInBoxParticles(box1, box2, insides);
    else
      grid.GetInBoxParticles(box1, box2, insides);
    empty = insides.empty();
    if (!empty) {
      bool all_splash = true;
      for (const int& in : insides) {
        if (ev.CheckSplash(in)) continue;
        const float e = (varR ? radii[in] : radius) * ev._SMOOTH_FACTOR;
        const F3& p = P[in];
        if (p[0] > (box1[0] - e) && p[0] < (box2[0] + e) && p[1] > (box1[1] - e) &&
            p[1] < (box2[1] + e) && p[2] > (box1[2] - e) && p[2] < (box2[2] + e)) {
          const V3<R>& n = ev.Normals[in];
          for (int k = 0; k < 3; ++k) norms[k] += n[k];
          area += std::sqrt(sqnorm3<R>(n[0], n[1], n[2]));
          if (varR && min_radius > radii[in]) min_radius = radii[in];
          all_splash = false;
        }
      }
      empty = all_splash;
    }
    curv = (area == 0) ? (R)1.0 : (std::sqrt(sqnorm3<R>(norms[0], norms[1], norms[2])) / area);
  }

  // src/iso_method_ours.cpp:52-75
  void GenerateSampling(const TNode<R>& t, float* sp) {
    float minV[3] = {t.center[0] - t.half_length, t.center[1] - t.half_length, t.center[2] - t.half_length};
    float maxV[3] = {t.center[0] + t.half_length, t.center[1] + t.half_length, t.center[2] + t.half_length};
    const int o = OVERSAMPLE;
    for (int z = 0; z <= o; z++)
      for (int y = 0; y <= o; y++)
        for (int x = 0; x <= o; x++) {
          int idx = (z * (o + 1) * (o + 1) + y * (o + 1) + x) * 4;
          sp[idx + 0] = (1 - float(x) / o) * minV[0] + (float(x) / o) * maxV[0];
          sp[idx + 1] = (1 - float(y) / o) * minV[1] + (float(y) / o) * maxV[1];
          sp[idx + 2] = (1 - float(z) / o) * minV[2] + (float(z) / o) * maxV[2];
          sp[idx + 3] = 0;
        }
  }

  // src/evaluator.cpp:127-252 (GridEval), called by NodeSampling
  // (src/iso_method_ours.cpp:77-99).  Sample values are R.
  void GridEval(const float* sp, R* vals, R* grads, float cellsize, bool& signchange) {
    const int o = OVERSAMPLE;
    float step = cellsize / o;
    for (int i = 0; i < (o + 1) * (o + 1) * (o + 1); i++) {
      vals[i] = ev.SingleEval(sp + i * 4);
      bool origin_sign = (vals[0] >= 0);
      if (!signchange) signchange = origin_sign ^ (vals[i] >= 0);
    }
    for (int z = 0; z <= o; z++)
      for (int y = 0; y <= o; y++)
        for (int x = 0; x <= o; x++) {
          int index = z * (o + 1) * (o + 1) + y * (o + 1) + x;
          R g[3];
          int nx = index + 1, lx = index - 1;
          int ny = index + (o + 1), ly = index - (o + 1);
          int nz = index + (o + 1) * (o + 1), lz = index - (o + 1) * (o + 1);
          g[0] = x == 0 ? (vals[index] - vals[nx]) / step
                        : (x == o ? (vals[lx] - vals[index]) / step : (vals[lx] - vals[nx]) / (step * 2));
          g[1] = y == 0 ? (vals[index] - vals[ny]) / step
                        : (y == o ? (vals[ly] - vals[index]) / step : (vals[ly] - vals[ny]) / (step * 2));
          g[2] = z == 0 ? (vals[index] - vals[nz]) / step
                        : (z == o ? (vals[lz] - vals[index]) / step : (vals[lz] - vals[nz]) / (step * 2));
          for (int k = 0; k < 3; ++k) grads[index * 3 + k] = g[k];
        }
  }

  // src/iso_method_ours.cpp:40-50
  R calcErrorDMC(const R p[4], const float* sp, const R* vals, const R* grads) {
    R err = 0;
    for (int i = 0; i < 27; i++) {
      R g0 = grads[i * 3 + 0], g1 = grads[i * 3 + 1], g2 = grads[i * 3 + 2];
      R dot = sum3<R>(g0 * (p[0] - (R)sp[i * 4 + 0]), g1 * (p[1] - (R)sp[i * 4 + 1]),
                      g2 * (p[2] - (R)sp[i * 4 + 2]));
      R e = dot - p[3];
      err += (e * e) / (1 + sqnorm3<R>(g0, g1, g2));
    }
    (void)vals;
    return err;
  }

  // src/iso_method_ours.cpp:101-174 (QEFNormal<float,4>, include/qefnorm.h)
  void NodeCalcNode(TNode<R>& t, const float* sp, const R* vals, const R* grads, float cellsize) {
    const float border = 0.0f * cellsize;
    float minV[3], maxV[3];
    for (int k = 0; k < 3; ++k) {
      minV[k] = t.center[k] - t.half_length + border;
      maxV[k] = t.center[k] + t.half_length - border;
    }
    R q[15];
    for (int k = 0; k < 15; ++k) q[k] = 0;
    for (int i = 0; i < 27; ++i) {
      R pl[5];
      R px = sp[i * 4 + 0], py = sp[i * 4 + 1], pz = sp[i * 4 + 2];
      pl[0] = grads[i * 3 + 0];
      pl[1] = grads[i * 3 + 1];
      pl[2] = grads[i * 3 + 2];
      pl[3] = -1;
      pl[4] = -(px * pl[0] + py * pl[1] + pz * pl[2]) + vals[i];
      int index = 0;
      for (int a = 0; a < 5; ++a)
        for (int b = a; b < 5; ++b) q[index++] += pl[a] * pl[b];
    }
    const int n = 4;
    R A[4][4] = {{0}}, B[4];
    for (int i = 0; i < n; i++) {
      int index = ((2 * n + 3 - i) * i) / 2;
      for (int j = i; j < n; j++) {
        A[i][j] = q[index + j - i];
        A[j][i] = A[i][j];
      }
      B[i] = -q[index + n - i];
    }
    R err = (R)1e30;
    R inv[4][4];
    inv4<R>(A, inv);
    R rv[4];
    for (int i = 0; i < n; i++) {
      rv[i] = 0;
      for (int j = 0; j < n; j++) rv[i] += inv[j][i] * B[j];
    }
    if (rv[0] >= minV[0] && rv[0] <= maxV[0] && rv[1] >= minV[1] && rv[1] <= maxV[1] &&
        rv[2] >= minV[2] && rv[2] <= maxV[2]) {
      err = calcErrorDMC(rv, sp, vals, grads);
      for (int k = 0; k < 4; ++k) t.node[k] = rv[k];
    }
    float np[3] = {(float)t.node[0], (float)t.node[1], (float)t.node[2]};
    t.node[3] = ev.SingleEval(np);
    if (err / cellsize < 0.0001) t.node[3] = 0.0;
  }

  // src/surface_reconstructor.cpp:237-273
  void afterSampleEval(TNode<R>& t, R curv, float min_radius, float* sp, R* vals, R* grads) {
    const bool qef = (flags & PIO_QEF) != 0;
    bool isbig = (t.depth < DEPTH_MIN);
    bool signchange = false;
    float cellsize = 2 * t.half_length;
    if (!isbig) {
      GenerateSampling(t, sp);
      GridEval(sp, vals, grads, cellsize, signchange);
    }
    t.signchange = signchange;
    float np[3];
    if ((cellsize - min_radius) < 1e-8) {
      t.type = LEAF;
      np[0] = (float)t.node[0], np[1] = (float)t.node[1], np[2] = (float)t.node[2];
      t.node[3] = ev.SingleEval(np);
      if (qef) NodeCalcNode(t, sp, vals, grads, cellsize);
      return;
    }
    if (isbig || (signchange && curv < 0.99)) {
      t.type = INTERNAL;
    } else {
      t.type = LEAF;
      if (qef) NodeCalcNode(t, sp, vals, grads, cellsize);
      np[0] = (float)t.node[0], np[1] = (float)t.node[1], np[2] = (float)t.node[2];
      t.node[3] = ev.SingleEval(np);
    }
  }

  // TNode(constructor, parent, i) (src/iso_method_ours.cpp:25-38)
  TNode<R> makeChild(int parent, int i) {
    const TNode<R>& pa = nodes[parent];
    TNode<R> c;
    c.depth = pa.depth + 1;
    c.half_length = pa.half_length / 2;
    const float sx = (i & 1) ? 1.0f : -1.0f, sy = (i & 2) ? 1.0f : -1.0f, sz = (i & 4) ? 1.0f : -1.0f;
    c.center[0] = pa.center[0] + sx * c.half_length;
    c.center[1] = pa.center[1] + sy * c.half_length;
    c.center[2] = pa.center[2] + sz * c.half_length;
    c.node[0] = c.center[0];
    c.node[1] = c.center[1];
    c.node[2] = c.center[2];
    c.node[3] = 0;
    c.type = UNCERTAIN;
    c.id = pa.id * 8 + (unsigned long long)i;
    c.parent = parent;
    return c;
  }

  // genIsoOurs state 0 (src/surface_reconstructor.cpp:283-288, 326-407)
  void buildTree() {
    nodes.clear();
    nodes.reserve(1 << 16);
    TNode<R> root;
    root.id = 0;
    root.depth = 0;
    for (int k = 0; k < 3; ++k) {
      root.center[k] = RootCenter[k];
      root.node[k] = RootCenter[k];
    }
    root.node[3] = 0;
    root.half_length = RootHalfLength;
    nodes.push_back(root);
    const size_t inProcessSize = 10000000;
    std::vector<int> waiting{0}, batch;
    std::vector<R> curvs;
    std::vector<float> minrs;
    std::vector<unsigned char> emptys;
    std::vector<float> sps;
    std::vector<R> vals, grads;
    while (!waiting.empty()) {
      batch.clear();
      while (batch.size() < inProcessSize && !waiting.empty()) {
        batch.push_back(waiting.back());
        waiting.pop_back();
      }
      const size_t nb = batch.size();
      curvs.assign(nb, 0);
      minrs.assign(nb, 0);
      emptys.assign(nb, 0);
#pragma omp parallel
      {
#pragma omp single
        {
          for (size_t i = 0; i < nb; i++) {
#pragma omp task firstprivate(i)
            {
              TNode<R>& t = nodes[batch[i]];
              checkEmptyAndCalcCurv(t, emptys[i], curvs[i], minrs[i]);
              t.curv = (float)curvs[i];
              if (emptys[i]) {
                t.node[3] = ev._ISO_VALUE;
                t.type = EMPTY;
              }
            }
          }
        }
      }
      sps.assign(nb * 27 * 4, 0.0f);
      vals.assign(nb * 27, 0);
      grads.assign(nb * 27 * 3, 0);
#pragma omp parallel
      {
#pragma omp single
        {
          for (size_t i = 0; i < nb; i++) {
            if (emptys[i]) continue;
#pragma omp task firstprivate(i)
            afterSampleEval(nodes[batch[i]], curvs[i], minrs[i], &sps[i * 108], &vals[i * 27], &grads[i * 81]);
          }
        }
      }
      for (size_t i = 0; i < nb; i++) {
        if (nodes[batch[i]].type == INTERNAL) {
          for (int t = 0; t < 8; ++t) {
            TNode<R> c = makeChild(batch[i], t);
            nodes.push_back(c);
            int ci = (int)nodes.size() - 1;
            nodes[batch[i]].children[t] = ci;
            waiting.push_back(ci);
          }
        }
      }
    }
  }

  // ---- dual traversal (include/traverse.h) + VisitorExtract ----
  struct TD {
    int n;
    char depth;
  };
  static int I3(int x, int y, int z) { return x | (y << 1) | (z << 2); }

  // TraversalData::gen_trav (src/visitorextract.cpp:22-33)
  TD gen(const TD& td, int i) const {
    if (!nodes[td.n].is_leaf()) return TD{nodes[td.n].children[i], (char)(td.depth + 1)};
    return td;
  }
  bool leaf(const TD& t) const { return nodes[t.n].is_leaf(); }

  // VisitorExtract::on_vert (src/visitorextract.cpp:229-256)
  bool on_vert(const TD* n8) {
    for (int i = 0; i < 8; ++i)
      if (!leaf(n8[i])) return true;
    int index = 0;
    for (int i = 0; i < 8; i++)
      if (nodes[n8[i].n].node[3] > 0) index += 1 << i;
    const DmcProc& proc = table[index];
    DualGrid<R> g;
    g.proc = proc;
    for (int i = 0; i < 8; i++) g.grid[i] = n8[proc.trans[i]].n;
    if (!(proc.code == 0 || proc.code == 255)) dual_grids.push_back(g);
    return false;
  }

  // traverse_vert (include/traverse.h:12-36)
  void t_vert(const TD* n8) {
    if (!on_vert(n8)) return;
    TD c[8];
    for (int i = 0; i < 8; ++i) c[i] = gen(n8[i], 7 - i);
    t_vert(c);
  }

  // traverse_edge_x / _y / _z (include/traverse.h:38-139); axis a is the edge
  // direction, (n00, n10, n01, n11) index the two other axes in order.
  void t_edge(int a, const TD& n00, const TD& n10, const TD& n01, const TD& n11) {
    if (leaf(n00) && leaf(n10) && leaf(n01) && leaf(n11)) return;
    TD c[8];
    auto idx = [&](int i, int u, int v) {
      if (a == 0) return I3(i, u, v);
      if (a == 1) return I3(u, i, v);
      return I3(u, v, i);
    };
    for (int i = 0; i < 2; i++) {
      c[idx(i, 0, 0)] = gen(n00, idx(i, 1, 1));
      c[idx(i, 1, 0)] = gen(n10, idx(i, 0, 1));
      c[idx(i, 0, 1)] = gen(n01, idx(i, 1, 0));
      c[idx(i, 1, 1)] = gen(n11, idx(i, 0, 0));
    }
    for (int i = 0; i < 2; i++) t_edge(a, c[idx(i, 0, 0)], c[idx(i, 1, 0)], c[idx(i, 0, 1)], c[idx(i, 1, 1)]);
    t_vert(c);
  }
  void edge_x(const TD* c, int i) { t_edge(0, c[I3(i, 0, 0)], c[I3(i, 1, 0)], c[I3(i, 0, 1)], c[I3(i, 1, 1)]); }
  void edge_y(const TD* c, int i) { t_edge(1, c[I3(0, i, 0)], c[I3(1, i, 0)], c[I3(0, i, 1)], c[I3(1, i, 1)]); }
  void edge_z(const TD* c, int i) { t_edge(2, c[I3(0, 0, i)], c[I3(1, 0, i)], c[I3(0, 1, i)], c[I3(1, 1, i)]); }

  // traverse_face_x / _y / _z (include/traverse.h:141-263)
  void t_face(int a, const TD& n0, const TD& n1) {
    if (leaf(n0) && leaf(n1)) return;
    TD c[8];
    auto idx = [&](int s, int u, int v) {
      if (a == 0) return I3(s, u, v);
      if (a == 1) return I3(u, s, v);
      return I3(u, v, s);
    };
    for (int i = 0; i < 4; i++) {
      int ix = i & 1, iy = (i >> 1) & 1;
      c[idx(0, ix, iy)] = gen(n0, idx(1, ix, iy));
      c[idx(1, ix, iy)] = gen(n1, idx(0, ix, iy));
    }
    for (int i = 0; i < 4; i++) {
      int ix = i & 1, iy = (i >> 1) & 1;
      t_face(a, c[idx(0, ix, iy)], c[idx(1, ix, iy)]);
    }
    for (int i = 0; i < 2; i++) {
      if (a == 0) {
        edge_y(c, i);
        edge_z(c, i);
      } else if (a == 1) {
        edge_x(c, i);
        edge_z(c, i);
      } else {
        edge_x(c, i);
        edge_y(c, i);
      }
    }
    t_vert(c);
  }

  // traverse_node (include/traverse.h:267-312)
  void t_node(const TD& td) {
    if (leaf(td)) return;
    TD c[8];
    for (int i = 0; i < 8; i++) {
      c[i] = gen(td, i);
      t_node(c[i]);
    }
    for (int i = 0; i < 4; i++) {
      int ix = i & 1, iy = (i >> 1) & 1;
      t_face(0, c[I3(0, ix, iy)], c[I3(1, ix, iy)]);
      t_face(1, c[I3(ix, 0, iy)], c[I3(ix, 1, iy)]);
      t_face(2, c[I3(ix, iy, 0)], c[I3(ix, iy, 1)]);
    }
    for (int i = 0; i < 2; i++) {
      edge_x(c, i);
      edge_y(c, i);
      edge_z(c, i);
    }
    t_vert(c);
  }

  static int nsign(R v) { return v > 0 ? 1 : -1; }  // include/utils.h:7-11

  // VisitorExtract::calc_vertices (src/visitorextract.cpp:41-201)
  void calc_vertices() {
    dual_cells.assign(dual_grids.size(), DualCell<R>());
    // src/visitorextract.cpp:54: half the (searcher's minimum) radius
    const float rr = (varR ? searcher.minRadius : radius) / 2;
#pragma omp parallel for
    for (long long i = 0; i < (long long)dual_grids.size(); i++) {
      DualCell<R>& dc = dual_cells[i];
      for (int e = 0; e < 12; ++e) {
        int c0, c1;
        dmc_edge_corners(e, &c0, &c1);
        const TNode<R>& v1 = nodes[dual_grids[i].grid[c0]];
        const TNode<R>& v2 = nodes[dual_grids[i].grid[c1]];
        if (nsign(v1.node[3]) == nsign(v2.node[3])) continue;
        R a[4], b[4], m[4] = {0, 0, 0, 0};
        for (int k = 0; k < 4; ++k) {
          a[k] = v1.node[k];
          b[k] = v2.node[k];
        }
        R d = std::sqrt(sqnorm3<R>(a[0] - b[0], a[1] - b[1], a[2] - b[2]));
        while (d > rr) {
          m[0] = (a[0] + b[0]) / 2;
          m[1] = (a[1] + b[1]) / 2;
          m[2] = (a[2] + b[2]) / 2;
          float mp[3] = {(float)m[0], (float)m[1], (float)m[2]};
          m[3] = ev.SingleEval(mp);
          nBisect.fetch_add(1, std::memory_order_relaxed);
          if (nsign(m[3]) == nsign(a[3])) {
            for (int k = 0; k < 4; ++k) a[k] = m[k], m[k] = 0;
          } else if (nsign(m[3]) == nsign(b[3])) {
            for (int k = 0; k < 4; ++k) b[k] = m[k], m[k] = 0;
          } else {
            break;
          }
          d /= 2;
        }
        R ratio = (R(0.0f) - a[3]) / (b[3] - a[3]);
        R outp[4];
        if (ratio < 0.1) {
          for (int k = 0; k < 4; ++k) outp[k] = a[k];
        } else if (ratio > 0.9) {
          for (int k = 0; k < 4; ++k) outp[k] = b[k];
        } else {
          for (int k = 0; k < 4; ++k) outp[k] = a[k] + (b[k] - a[k]) * ratio;
        }
        for (int k = 0; k < 3; ++k) dc.vertices[e][k] = (float)outp[k];
      }
      int tris[8][3];
      int nt = dmc_case_tris(dual_grids[i].proc.code, tris);
      for (int t = 0; t < nt; ++t) dc.faces.push_back({tris[t][0], tris[t][1], tris[t][2]});
    }
  }

  // VisitorExtract::generate_mesh (src/visitorextract.cpp:203-227) with
  // Mesh::insert_vert / insert_tri (src/global.cpp:13-53)
  void generate_mesh() {
    std::map<std::string, int> vmap, tmap;
    mverts.clear();
    mvkeys.clear();
    mtris.clear();
    auto key2 = [](unsigned long long a, unsigned long long b) {
      if (b < a) std::swap(a, b);
      return std::to_string(a) + "," + std::to_string(b) + ",";
    };
    auto key3 = [](int a, int b, int c) {
      int v[3] = {a, b, c};
      std::sort(v, v + 3);
      return std::to_string(v[0]) + "," + std::to_string(v[1]) + "," + std::to_string(v[2]) + ",";
    };
    for (size_t i = 0; i < dual_grids.size(); i++) {
      for (size_t j = 0; j < dual_cells[i].faces.size(); j++) {
        int ids[3];
        for (int k = 0; k < 3; k++) {
          int e = dual_cells[i].faces[j][k];
          int c0, c1;
          dmc_edge_corners(e, &c0, &c1);
          unsigned long long i1 = nodes[dual_grids[i].grid[c0]].id, i2 = nodes[dual_grids[i].grid[c1]].id;
          auto ins = vmap.try_emplace(key2(i1, i2), (int)mverts.size());
          if (ins.second) {
            const float* v = dual_cells[i].vertices[e];
            mverts.push_back({v[0], v[1], v[2]});
            mvkeys.push_back({std::min(i1, i2), std::max(i1, i2)});
          }
          ids[k] = ins.first->second + 1;
        }
        int t0, t1, t2;
        if (dual_grids[i].proc.flip) {
          t0 = ids[0], t1 = ids[1], t2 = ids[2];
        } else {
          t0 = ids[2], t1 = ids[1], t2 = ids[0];
        }
        auto ins = tmap.try_emplace(key3(t0, t1, t2), (int)mtris.size());
        if (ins.second) mtris.push_back({t0, t1, t2});
      }
    }
  }

  // Mesh::BuildIcosaTable (src/global.cpp:65-92), in float
  static void icosa_table(float T[12][3]) {
    const float PI = 3.1415926f;
    const float H_ANGLE = PI / 180 * 72;
    const float V_ANGLE = std::atan(1.0f / 2);
    float hAngle1 = -PI / 2 - H_ANGLE / 2, hAngle2 = -PI / 2;
    T[0][0] = 0, T[0][1] = 0, T[0][2] = 1;
    for (int i = 1; i <= 5; i++) {
      const float z = std::sin(V_ANGLE), xy = std::cos(V_ANGLE);
      T[i][0] = xy * std::cos(hAngle1), T[i][1] = xy * std::sin(hAngle1), T[i][2] = z;
      T[i + 5][0] = xy * std::cos(hAngle2), T[i + 5][1] = xy * std::sin(hAngle2), T[i + 5][2] = -z;
      hAngle1 += H_ANGLE;
      hAngle2 += H_ANGLE;
    }
    T[11][0] = 0, T[11][1] = 0, T[11][2] = -1;
  }

  // GEN_SPLASH (src/surface_reconstructor.cpp:299-320) with
  // Mesh::AppendSplash_ConstR / AppendSplash_VarR (src/global.cpp:94-138):
  // 12 vertices and 20 triangles per splash particle, particle order; vertex
  // keys (12 p + i, ~0)
  void append_splash() {
    float T[12][3];
    icosa_table(T);
    for (int p = 0; p < ev.N; p++) {
      if (!ev.CheckSplash(p)) continue;
      int idx[12];
      const float rr = varR ? radii[p] : radius;
      for (int i = 0; i < 12; i++) {
        const F3& q = P[p];
        mverts.push_back({q[0] + T[i][0] * rr, q[1] + T[i][1] * rr, q[2] + T[i][2] * rr});
        mvkeys.push_back({12ull * (unsigned long long)p + (unsigned long long)i, ~0ull});
        idx[i] = (int)mverts.size();
      }
      for (int i = 0; i < 5; i++) {
        mtris.push_back({idx[0], idx[1 + i], idx[(1 + i) % 5 + 1]});
        mtris.push_back({idx[1 + i], idx[(1 + i) % 5 + 1], idx[6 + i]});
        mtris.push_back({idx[(1 + i) % 5 + 1], idx[6 + i], idx[(1 + i) % 5 + 6]});
        mtris.push_back({idx[6 + i], idx[(1 + i) % 5 + 6], idx[11]});
      }
    }
  }

  int stage(int s) override {
    if (s != stage_done + 1) return -2;
    double t0 = now_s();
    switch (s) {
      case 1:  // src/surface_reconstructor.cpp:418-424
        loadRootBox();
        if (varR)
          searcher.init(&P, radii, 4.0f, (flags & PIO_STD_SORT) != 0);
        else
          grid.init(&P, BoundingBox, radius, 4.0f, (flags & PIO_STD_SORT) != 0);
        break;
      case 2:  // :432-435
        if (varR) {
          ev.searcher = &searcher;
          ev.GlobalRadius = &radii;
        }
        ev.init(&grid, &P, radius);
        ev.splash_on = (flags & PIO_SPLASH) != 0;
        ev._SMOOTH_FACTOR = smooth_factor;
        ev.compute_Gs_xMeans();
        break;
      case 3:  // :453-470
        if (varR) {
          resizeRootBoxVarR();
          ev.CalculateMaxScalarVarR();
          ev.RecommendIsoValueVarR();
        } else {
          resizeRootBoxConstR();
          ev.CalculateMaxScalarConstR();
          ev.RecommendIsoValueConstR();
        }
        ev.CalcParticlesNormal();
        break;
      case 4:
        buildTree();
        break;
      case 5: {  // genIsoOurs state 1 (:290-323)
        for (int i = 0; i < 256; ++i) table[i] = DmcProc();
        dmc_build_table(table);
        dual_grids.clear();
        t_node(TD{0, 0});
        nDual = (long long)dual_grids.size();
        calc_vertices();
        generate_mesh();
        if (ev.splash_on) append_splash();
        break;
      }
      default:
        return -1;
    }
    seconds[s] = now_s() - t0;
    stage_done = s;
    return 0;
  }
};

}  // namespace pio

using namespace pio;

struct pio_frame {
  std::unique_ptr<FrameBase> f;
  bool fp64 = false;
};

template <class F>
static auto with(pio_frame* h, F fn) {
  if (h->fp64) return fn(*static_cast<Frame<double>*>(h->f.get()));
  return fn(*static_cast<Frame<float>*>(h->f.get()));
}
template <class F>
static auto withc(const pio_frame* h, F fn) {
  if (h->fp64) return fn(*static_cast<const Frame<double>*>(h->f.get()));
  return fn(*static_cast<const Frame<float>*>(h->f.get()));
}

extern "C" {

pio_frame* pio_create(const float* xyz, int64_t n, float radius, float smooth_factor, float iso_factor,
                      int flags) {
  pio_frame* h = new pio_frame();
  h->fp64 = (flags & PIO_FP64) != 0;
  if (h->fp64)
    h->f.reset(new Frame<double>());
  else
    h->f.reset(new Frame<float>());
  FrameBase& f = *h->f;
  f.P.resize(n);
  for (int64_t i = 0; i < n; ++i) f.P[i] = {xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]};
  f.radius = radius;
  f.smooth_factor = smooth_factor;
  f.iso_factor = iso_factor;
  f.flags = flags;
  return h;
}

pio_frame* pio_create_var(const float* xyz, const float* radii, int64_t n, float smooth_factor, float iso_factor,
                          int flags) {
  pio_frame* h = pio_create(xyz, n, radii[0], smooth_factor, iso_factor, flags);
  h->f->varR = true;
  h->f->radii.assign(radii, radii + n);
  return h;
}

int pio_num_bins(const pio_frame* h) { return h->f->varR ? (int)h->f->searcher.searchers.size() : 1; }

int pio_bin_info(const pio_frame* h, int b, float* b6, int64_t* xyz3, int64_t* cn, float* cs, int64_t* count,
                 int32_t* radius_id) {
  if (h->f->stage_done < 1) return -1;
  const HashGrid& g = h->f->varR ? h->f->searcher.searchers.at(b) : h->f->grid;
  for (int i = 0; i < 6; ++i) b6[i] = g.Bounding[i];
  for (int i = 0; i < 3; ++i) xyz3[i] = g.XYZCellNum[i];
  *cn = (int64_t)g.CellNum;
  *cs = g.CellSize;
  *count = (int64_t)g.ParticlesNum;
  *radius_id = g.RadiusId;
  return 0;
}

int pio_bin_lists(const pio_frame* h, int b, int32_t* particles, int64_t* keys, int32_t* index_list) {
  if (h->f->stage_done < 1) return -1;
  const HashGrid& g = h->f->varR ? h->f->searcher.searchers.at(b) : h->f->grid;
  for (unsigned i = 0; i < g.ParticlesNum; ++i) {
    if (particles) particles[i] = g.var ? g.PIndexes[i] : (int32_t)i;
    if (keys) keys[i] = g.Keys[i];
    if (index_list) index_list[i] = g.var ? g.PIndexes[g.IndexList[i]] : g.IndexList[i];
  }
  return 0;
}

int pio_searcher_radii(const pio_frame* h, float* out3) {
  if (!h->f->varR || h->f->stage_done < 1) return -1;
  out3[0] = h->f->searcher.minRadius;
  out3[1] = h->f->searcher.maxRadius;
  out3[2] = h->f->searcher.avgRadius;
  return 0;
}

void pio_destroy(pio_frame* f) { delete f; }
void pio_set_threads(int n) {
  if (n > 0) omp_set_num_threads(n);
}

int pio_stage(pio_frame* f, int s) { return f->f->stage(s); }
int pio_run(pio_frame* f) {
  for (int s = f->f->stage_done + 1; s <= 5; ++s) {
    int rc = f->f->stage(s);
    if (rc) return rc;
  }
  return 0;
}
double pio_stage_seconds(const pio_frame* f, int s) { return (s >= 1 && s <= 5) ? f->f->seconds[s] : -1; }
int64_t pio_counter(const pio_frame* f, int w) { return f->f->counter(w); }

int pio_grid_info(const pio_frame* h, float* b6, int64_t* xyz3, int64_t* cn, float* cs) {
  const HashGrid& g = h->f->grid;
  if (h->f->stage_done < 1) return -1;
  for (int i = 0; i < 6; ++i) b6[i] = g.Bounding[i];
  for (int i = 0; i < 3; ++i) xyz3[i] = g.XYZCellNum[i];
  *cn = (int64_t)g.CellNum;
  *cs = g.CellSize;
  return 0;
}
int pio_get_keys(const pio_frame* h, int64_t* keys) {
  const HashGrid& g = h->f->grid;
  for (size_t i = 0; i < g.Keys.size(); ++i) keys[i] = g.Keys[i];
  return 0;
}
int pio_get_index_list(const pio_frame* h, int32_t* idx) {
  const HashGrid& g = h->f->grid;
  for (size_t i = 0; i < g.IndexList.size(); ++i) idx[i] = g.IndexList[i];
  return 0;
}
int64_t pio_num_cells(const pio_frame* h) { return (int64_t)h->f->grid.StartList.size(); }
int pio_get_cells(const pio_frame* h, int64_t* hash, int32_t* start, int32_t* end) {
  const HashGrid& g = h->f->grid;
  size_t k = 0;
  for (auto& kv : g.StartList) {
    hash[k] = kv.first;
    start[k] = kv.second;
    end[k] = g.EndList.at(kv.first);
    ++k;
  }
  return 0;
}
int64_t pio_neighbors(pio_frame* h, const float* pts, int64_t m, int64_t* offsets, int32_t* out, int64_t cap) {
  HashGrid& g = h->f->grid;
  int64_t tot = 0;
  offsets[0] = 0;
  std::vector<int> nb;
  for (int64_t i = 0; i < m; ++i) {
    nb.clear();
    if (h->f->varR)
      h->f->searcher.GetNeighbors(pts + 3 * i, nb);
    else
      g.GetPIdxList(pts + 3 * i, nb);
    if (tot + (int64_t)nb.size() > cap) return -1;
    for (int j : nb) out[tot++] = j;
    offsets[i + 1] = tot;
  }
  return tot;
}
int64_t pio_in_box(pio_frame* h, const float* b1, const float* b2, int32_t* out, int64_t cap) {
  HashGrid& g = h->f->grid;
  std::vector<int> nb;
  if (h->f->varR)
    h->f->searcher.GetInBoxParticles(F3{b1[0], b1[1], b1[2]}, F3{b2[0], b2[1], b2[2]}, nb);
  else
    g.GetInBoxParticles(F3{b1[0], b1[1], b1[2]}, F3{b2[0], b2[1], b2[2]}, nb);
  if ((int64_t)nb.size() > cap) return -1;
  for (size_t j = 0; j < nb.size(); ++j) out[j] = nb[j];
  return (int64_t)nb.size();
}
int pio_get_aniso(const pio_frame* h, double* xm, double* g9, double* det) {
  if (h->f->stage_done < 2) return -1;
  return withc(h, [&](const auto& f) {
    for (int i = 0; i < f.ev.N; ++i) {
      for (int k = 0; k < 3; ++k) xm[3 * i + k] = (double)f.ev.xMeans[i][k];
      for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) g9[9 * i + 3 * a + b] = (double)f.ev.Gs[i](a, b);
      det[i] = (double)f.ev.Dets[i];
    }
    return 0;
  });
}
int pio_get_splash(const pio_frame* h, int8_t* out) {
  if (h->f->stage_done < 2) return -1;
  return withc(h, [&](const auto& f) {
    for (int i = 0; i < f.ev.N; ++i) out[i] = f.ev.CheckSplash(i) ? 1 : 0;
    return 0;
  });
}
int pio_get_normals(const pio_frame* h, double* nrm) {
  if (h->f->stage_done < 3) return -1;
  return withc(h, [&](const auto& f) {
    for (int i = 0; i < f.ev.N; ++i)
      for (int k = 0; k < 3; ++k) nrm[3 * i + k] = (double)f.ev.Normals[i][k];
    return 0;
  });
}
int pio_scalars(const pio_frame* h, double* o) {
  return withc(h, [&](const auto& f) {
    o[0] = (double)f.ev._ISO_VALUE;
    o[1] = (double)f.ev._MAX_SCALAR;
    o[2] = (double)f.ev.Influnce2;
    o[3] = (double)f.ev.Sigma;
    return 0;
  });
}
int pio_depths(const pio_frame* h, int32_t* o2, float* rc3, float* rh) {
  const FrameBase& f = *h->f;
  o2[0] = f.DEPTH_MAX;
  o2[1] = f.DEPTH_MIN;
  for (int k = 0; k < 3; ++k) rc3[k] = f.RootCenter[k];
  *rh = f.RootHalfLength;
  return 0;
}
int pio_eval(pio_frame* h, const float* pts, int64_t m, double* scalar, double* grad3) {
  if (h->f->stage_done < 3) return -1;
  return with(h, [&](auto& f) {
    using R = std::remove_reference_t<decltype(f.ev._ISO_VALUE)>;
#pragma omp parallel for
    for (int64_t i = 0; i < m; ++i) {
      if (grad3) {
        R s = 0;
        V3<R> g{{0, 0, 0}};
        f.ev.SingleEvalWithGrad(pts + 3 * i, s, g);
        scalar[i] = (double)s;
        for (int k = 0; k < 3; ++k) grad3[3 * i + k] = (double)g[k];
      } else {
        scalar[i] = (double)f.ev.SingleEval(pts + 3 * i);
      }
    }
    return 0;
  });
}
// UniformGrid::resizeRootBoxConstR (src/marching.cpp:42-55) on the
// loadRootBox box: per axis resizeLen = ceil(length / r) r + 4 r around the
// centre, steps = int(resizeLen / r), dims = steps + 1.
static void uniform_grid_box(const FrameBase& f, float box[6], int steps[3], int dims[3]) {
  for (int i = 0; i < 3; i++) {
    float center = (f.RawBox[i * 2] + f.RawBox[i * 2 + 1]) / 2;
    float length = f.RawBox[i * 2 + 1] - f.RawBox[i * 2];
    float resizeLen = std::ceil(length / f.radius) * f.radius + f.radius * 4;
    box[i * 2] = center - resizeLen / 2;
    box[i * 2 + 1] = center + resizeLen / 2;
    steps[i] = int(resizeLen / (f.radius));
    dims[i] = steps[i] + 1;
  }
}

int pio_uniform_grid(const pio_frame* h, float* box6, int32_t* steps3, int32_t* dims3) {
  const FrameBase& f = *h->f;
  if (f.stage_done < 1) return -1;
  float box[6];
  int steps[3], dims[3];
  uniform_grid_box(f, box, steps, dims);
  for (int i = 0; i < 6; ++i) box6[i] = box[i];
  for (int i = 0; i < 3; ++i) {
    steps3[i] = steps[i];
    dims3[i] = dims[i];
  }
  return 0;
}

// UniformGrid::gridSampling (src/marching.cpp:72-93): SingleEval at every
// lattice point, x fastest; point = (steps - x) / steps * min + x / steps * max.
int pio_grid_sample(pio_frame* h, double* out, int64_t n) {
  if (h->f->stage_done < 3) return -1;
  float box[6];
  int steps[3], dims[3];
  uniform_grid_box(*h->f, box, steps, dims);
  const int64_t total = (int64_t)dims[0] * dims[1] * dims[2];
  if (n < total) return -2;
  return with(h, [&](auto& f) {
    const float minV[3] = {box[0], box[2], box[4]}, maxV[3] = {box[1], box[3], box[5]};
#pragma omp parallel for
    for (int64_t i = 0; i < total; i++) {
      const int z = (int)(i / (dims[0] * dims[1]));
      const int y = (int)((i % (dims[0] * dims[1])) / dims[0]);
      const int x = (int)((i % (dims[0] * dims[1])) % dims[0]);
      const float p[3] = {
          float(steps[0] - x) / float(steps[0]) * minV[0] + float(x) / float(steps[0]) * maxV[0],
          float(steps[1] - y) / float(steps[1]) * minV[1] + float(y) / float(steps[1]) * maxV[1],
          float(steps[2] - z) / float(steps[2]) * minV[2] + float(z) / float(steps[2]) * maxV[2]};
      out[i] = (double)f.ev.SingleEval(p);
    }
    return 0;
  });
}

int64_t pio_num_nodes(const pio_frame* h) {
  return withc(h, [&](const auto& f) { return (int64_t)f.nodes.size(); });
}
int pio_get_nodes(const pio_frame* h, uint64_t* id, int8_t* depth, int8_t* type, float* node4, float* center3,
                  float* half, float* curv, int8_t* sc, int32_t* parent) {
  return withc(h, [&](const auto& f) {
    for (size_t i = 0; i < f.nodes.size(); ++i) {
      const auto& t = f.nodes[i];
      id[i] = t.id;
      depth[i] = t.depth;
      type[i] = t.type;
      for (int k = 0; k < 4; ++k) node4[4 * i + k] = (float)t.node[k];
      for (int k = 0; k < 3; ++k) center3[3 * i + k] = t.center[k];
      half[i] = t.half_length;
      curv[i] = t.curv;
      sc[i] = t.signchange;
      parent[i] = t.parent;
    }
    return 0;
  });
}
int pio_mesh_counts(const pio_frame* h, int64_t* nv, int64_t* nt) {
  *nv = (int64_t)h->f->mverts.size();
  *nt = (int64_t)h->f->mtris.size();
  return 0;
}
int pio_mesh_get(const pio_frame* h, float* v3, int32_t* t3, uint64_t* vk2) {
  const FrameBase& f = *h->f;
  for (size_t i = 0; i < f.mverts.size(); ++i) {
    for (int k = 0; k < 3; ++k) v3[3 * i + k] = f.mverts[i][k];
    if (vk2) {
      vk2[2 * i] = f.mvkeys[i][0];
      vk2[2 * i + 1] = f.mvkeys[i][1];
    }
  }
  for (size_t i = 0; i < f.mtris.size(); ++i)
    for (int k = 0; k < 3; ++k) t3[3 * i + k] = f.mtris[i][k];
  return 0;
}
// writeObjFile (src/main.cpp:54-67)
int pio_write_obj(const pio_frame* h, const char* path) {
  FILE* fp = std::fopen(path, "w");
  if (!fp) return -1;
  for (auto& p : h->f->mverts) std::fprintf(fp, "v %f %f %f\n", p[0], p[1], p[2]);
  for (auto& t : h->f->mtris) std::fprintf(fp, "f %d %d %d\n", t[0], t[1], t[2]);
  std::fclose(fp);
  return 0;
}
int pio_dmc_table(int32_t* trans, int8_t* flip, int32_t* code) {
  DmcProc t[256];
  dmc_build_table(t);
  for (int i = 0; i < 256; ++i) {
    for (int k = 0; k < 8; ++k) trans[8 * i + k] = t[i].trans[k];
    flip[i] = t[i].flip;
    code[i] = t[i].code;
  }
  return 0;
}

}  // extern "C"
