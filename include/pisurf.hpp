// pisurf.hpp - C++ facade with the reference's class and method names.
//
// Host code written against LCM1999/ParticleIsosurface's in-process API
// (SurfReconstructor, Evaluator, HashGrid, TNode, Mesh, writeObjFile,
// UniformGrid) calls
// the GPU library through these header-only classes.  They hold no
// computation of their own: every call goes through the C ABI of pisurf.h,
// so the library (libpisurf.so) does the work on the GPU and errors come back
// as pisurf::Error (the reference has no error path; it exits on I/O errors).
//
// Vector types: when Eigen is included before this header, the classes take
// and return Eigen::Vector3f / Vector4f like the reference; otherwise a small
// pisurf::Vector3f / Vector4f with the same element access is used.
//
// The classes are declared in namespace pisurf and, unless
// PISURF_NO_GLOBAL_NAMES is defined, also made visible at global scope under
// the reference's names.
//
// Reference interfaces mirrored:
//   SurfReconstructor   include/surface_reconstructor.h:71-98
//   Evaluator           include/evaluator.h:76-112
//   HashGrid            include/hash_grid.h:9-45
//   TNode               include/iso_method_ours.h:30-78
//   Mesh, Vertex, Triangle  include/global.h:13-60, 86-115
//   writeObjFile        src/main.cpp:54-67
//   writePlyFile, loadParticlesFromCSV  src/main.cpp:69-114, 215-275
//   readShonDyParticleData  src/main.cpp:281-327 (HDF5, read by the library)
//   readShonDyParticleXDMF  src/hdf5Utils.cpp:7-47
//   UniformGrid         include/marching.h:18-70 (dense-grid mode)
//   MultiLevelSearcher  include/multi_level_researcher.h:8-40 (per-particle radii)
//   IS_CONST_RADIUS     include/iso_common.h:6, defined by the host program
//                       (src/main.cpp:32) unless PISURF_NO_GLOBAL_NAMES is set
#ifndef PISURF_HPP
#define PISURF_HPP

#include <array>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "pisurf.h"

#ifndef PISURF_NO_GLOBAL_NAMES
// The reference's run-mode switch: true for one radius, false for the
// per-particle radii passed to SurfReconstructor.  The host program defines
// it, as the reference's main does.
extern bool IS_CONST_RADIUS;
#endif

namespace pisurf {

#ifdef EIGEN_WORLD_VERSION
using Vector3f = Eigen::Vector3f;
using Vector4f = Eigen::Vector4f;
#else
struct Vector3f {
  float v[3] = {0.f, 0.f, 0.f};
  Vector3f() = default;
  Vector3f(float a, float b, float c) : v{a, b, c} {}
  float& operator[](int i) { return v[i]; }
  float operator[](int i) const { return v[i]; }
  float& x() { return v[0]; }
  float& y() { return v[1]; }
  float& z() { return v[2]; }
  float x() const { return v[0]; }
  float y() const { return v[1]; }
  float z() const { return v[2]; }
  float* data() { return v; }
  const float* data() const { return v; }
};
struct Vector4f {
  float v[4] = {0.f, 0.f, 0.f, 0.f};
  Vector4f() = default;
  Vector4f(float a, float b, float c, float d) : v{a, b, c, d} {}
  float& operator[](int i) { return v[i]; }
  float operator[](int i) const { return v[i]; }
  float* data() { return v; }
  const float* data() const { return v; }
};
#endif

class Error : public std::runtime_error {
 public:
  Error(int code, const std::string& msg) : std::runtime_error(msg), code_(code) {}
  int code() const { return code_; }

 private:
  int code_;
};

inline void check(int rc) {
  if (rc != PI_OK) throw Error(rc, std::string("pisurf: ") + pi_last_error());
}

// Mesh element types of include/global.h: Vertex = vect3<float>, Triangle
// holds 1-based vertex indices (Mesh::insert_vert returns index + 1).
struct Vertex {
  float v[3] = {0.f, 0.f, 0.f};
  Vertex() = default;
  Vertex(float a, float b, float c) : v{a, b, c} {}
  float& operator[](int i) { return v[i]; }
  float operator[](int i) const { return v[i]; }
};

struct Triangle {
  std::array<int, 3> v{{0, 0, 0}};
  Triangle() = default;
  Triangle(int a, int b, int c) : v{{a, b, c}} {}
};

class Mesh {
 public:
  explicit Mesh(int mesh_precision = 10000) : MESH_PRECISION(mesh_precision) {}
  int MESH_PRECISION;
  std::vector<Vertex> vertices;
  std::vector<Triangle> tris;
  unsigned int verticesNum = 0;
  unsigned int trianglesNum = 0;
  // the sorted leaf-id pair that names each vertex (Mesh::insert_vert's key)
  std::vector<std::array<unsigned long long, 2>> vertexKeys;
  void reset() {
    vertices.clear();
    tris.clear();
    vertexKeys.clear();
    verticesNum = trianglesNum = 0;
  }
};

// writeObjFile (src/main.cpp:54-67): the same text format.
inline void writeObjFile(Mesh& m, const std::string& fn) {
  FILE* f = std::fopen(fn.c_str(), "w");
  if (!f) throw Error(PI_ERR_INVALID, "pisurf: cannot open " + fn);
  for (const Vertex& p : m.vertices) std::fprintf(f, "v %f %f %f\n", p[0], p[1], p[2]);
  for (const Triangle& t : m.tris) std::fprintf(f, "f %d %d %d\n", t.v[0], t.v[1], t.v[2]);
  std::fclose(f);
}

// writePlyFile (src/main.cpp:69-114): binary PLY as RPly writes it.
inline void writePlyFile(Mesh& m, const std::string& fn) {
  std::vector<float> v(m.vertices.size() * 3);
  std::vector<int32_t> t(m.tris.size() * 3);
  for (size_t i = 0; i < m.vertices.size(); ++i)
    for (int k = 0; k < 3; ++k) v[3 * i + k] = m.vertices[i][k];
  for (size_t i = 0; i < m.tris.size(); ++i)
    for (int k = 0; k < 3; ++k) t[3 * i + k] = m.tris[i].v[k];
  check(pi_write_ply(fn.c_str(), v.data(), (int64_t)m.vertices.size(), t.data(), (int64_t)m.tris.size(), 1));
}

// loadParticlesFromCSV (src/main.cpp:215-275); radiuses are read when
// is_const_radius is false (the reference's IS_CONST_RADIUS).
inline void loadParticlesFromCSV(const std::string& csvPath, std::vector<Vector3f>& particles,
                                 std::vector<float>& radiuses, bool is_const_radius = true) {
  int64_t n = 0;
  check(pi_load_csv(csvPath.c_str(), nullptr, nullptr, 0, &n, nullptr));
  std::vector<float> xyz((size_t)n * 3);
  std::vector<float> rad(is_const_radius ? 0 : (size_t)n);
  check(pi_load_csv(csvPath.c_str(), xyz.data(), is_const_radius ? nullptr : rad.data(), n, &n, nullptr));
  particles.resize((size_t)n);
  for (int64_t i = 0; i < n; ++i) particles[i] = Vector3f(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]);
  if (!is_const_radius) radiuses = rad;
}

namespace detail {

// One GPU context per thread and device, shared by the frames made there.
struct Context {
  pi_ctx* h = nullptr;
  explicit Context(int device) { check(pi_ctx_create(device, 0, &h)); }
  ~Context() {
    if (h) pi_ctx_destroy(h);
  }
  Context(const Context&) = delete;
  Context& operator=(const Context&) = delete;
  static std::shared_ptr<Context> get(int device) {
    thread_local std::shared_ptr<Context> ctx[16];
    if (device < 0 || device >= 16) throw Error(PI_ERR_INVALID, "pisurf: device index out of range");
    if (!ctx[device]) ctx[device] = std::make_shared<Context>(device);
    return ctx[device];
  }
};

struct Frame {
  std::shared_ptr<Context> ctx;
  pi_frame* h = nullptr;
  Frame(std::shared_ptr<Context> c, const pi_params& p) : ctx(std::move(c)) {
    check(pi_frame_create(ctx->h, &p, &h));
  }
  ~Frame() {
    if (h) pi_frame_destroy(h);
  }
  Frame(const Frame&) = delete;
  Frame& operator=(const Frame&) = delete;
  pi_frame_info info() const {
    pi_frame_info fi;
    check(pi_frame_info_get(h, &fi));
    return fi;
  }
  template <class T>
  std::vector<T> dump(int what) {
    size_t bytes = 0;
    check(pi_stage_dump_size(h, what, &bytes));
    std::vector<T> out(bytes / sizeof(T));
    if (bytes) check(pi_stage_dump(h, what, out.data(), bytes));
    return out;
  }
};

inline bool const_radius_mode() {
#ifndef PISURF_NO_GLOBAL_NAMES
  return ::IS_CONST_RADIUS;
#else
  return true;
#endif
}
}  // namespace detail

// readShonDyParticleData (src/main.cpp:281-327): "position" and, unless the
// radius is constant, "particleRadius" of an HDF5 particle file.  The
// library reads the HDF5 format itself; errors throw.
inline bool readShonDyParticleData(const std::string& fileName, std::vector<Vector3f>& positions,
                                   std::vector<float>& radiuses,
                                   bool is_const_radius = detail::const_radius_mode()) {
  int64_t n = 0;
  check(pi_load_hdf5(fileName.c_str(), nullptr, nullptr, 0, &n));
  std::vector<float> xyz((size_t)n * 3);
  std::vector<float> rad(is_const_radius ? 0 : (size_t)n);
  check(pi_load_hdf5(fileName.c_str(), xyz.data(), is_const_radius ? nullptr : rad.data(), n, &n));
  positions.resize((size_t)n);
  for (int64_t i = 0; i < n; ++i) positions[i] = Vector3f(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]);
  if (!is_const_radius) radiuses = rad;
  return true;
}

// readShonDyParticleXDMF (src/hdf5Utils.cpp:7-47): the frame files listed by
// <dir_path>/<xdmf_file>, all or only frame target_frame (1-based).
inline bool readShonDyParticleXDMF(const std::string& dir_path, const std::string& xdmf_file,
                                   std::vector<std::string>& files, const int target_frame) {
  int64_t len = 0;
  int32_t frames = 0;
  check(pi_load_xdmf(dir_path.c_str(), xdmf_file.c_str(), target_frame, nullptr, 0, &len, &frames));
  std::string buf((size_t)len, '\0');
  check(pi_load_xdmf(dir_path.c_str(), xdmf_file.c_str(), target_frame, &buf[0], len, &len, &frames));
  size_t s = 0;
  for (int32_t k = 0; k < frames; ++k) {
    size_t e = buf.find('\n', s);
    if (e == std::string::npos) e = std::strlen(buf.c_str());
    files.push_back(buf.substr(s, e - s));
    s = e + 1;
  }
  return true;
}

// MultiLevelSearcher (src/multi_level_reseacher.cpp): the radius bins of a
// frame with per-particle radii, one hash grid per non-empty bin, built by
// SurfReconstructor::Run.  GetNeighbors runs on the GPU.
class MultiLevelSearcher {
 public:
  explicit MultiLevelSearcher(std::shared_ptr<detail::Frame> f) : frame_(std::move(f)) {
    const pi_frame_info fi = frame_->info();
    minRadius_ = fi.radius_min;
    maxRadius_ = fi.radius_max;
    particlesNum_ = (unsigned int)fi.num_particles;
    grids_ = fi.num_grids;
  }
  float getMaxRadius() const { return maxRadius_; }
  float getMinRadius() const { return minRadius_; }
  float getParticlesNum() const { return (float)particlesNum_; }
  // the number of hash grids (getSearchers()->size() in the reference)
  int getSearchersNum() const { return grids_; }
  // GetNeighbors (src/multi_level_reseacher.cpp:79-92): the bins' 27-cell
  // candidate lists, in bin order.
  void GetNeighbors(const Vector3f& pos, std::vector<int>& neighbors) {
    const float p[3] = {pos[0], pos[1], pos[2]};
    int64_t off[2] = {0, 0}, total = 0;
    neighbors.assign(1024, 0);
    int rc = pi_hashgrid_neighbors(frame_->h, p, 1, off, neighbors.data(), (int64_t)neighbors.size(), &total);
    if (rc == PI_ERR_LIMIT) {
      neighbors.assign((size_t)total, 0);
      rc = pi_hashgrid_neighbors(frame_->h, p, 1, off, neighbors.data(), total, &total);
    }
    check(rc);
    neighbors.resize((size_t)total);
  }

 private:
  std::shared_ptr<detail::Frame> frame_;
  float minRadius_ = 0.f, maxRadius_ = 0.f;
  unsigned int particlesNum_ = 0;
  int grids_ = 0;
};

// HashGrid, constant radius (src/hash_grid.cpp).  Built by
// SurfReconstructor::Run; the queries run on the GPU.
class HashGrid {
 public:
  explicit HashGrid(std::shared_ptr<detail::Frame> f) : frame_(std::move(f)) {
    const pi_frame_info fi = frame_->info();
    ParticlesNum = (unsigned int)fi.num_particles;
    CellSize = fi.cell_size;
    Radius = fi.cell_size / 4.0f;  // the reference's cell is 4r at inf_factor 4
    for (int i = 0; i < 6; ++i) Bounding[i] = fi.bounding[i];
    for (int i = 0; i < 3; ++i) XYZCellNum[i] = (unsigned int)fi.xyz_cell_num[i];
    CellNum = (unsigned long long)fi.cell_num;
  }
  unsigned int ParticlesNum = 0;
  float Radius = 0.f;
  float CellSize = 0.f;
  float Bounding[6] = {0, 0, 0, 0, 0, 0};
  unsigned int XYZCellNum[3] = {0, 0, 0};
  unsigned long long CellNum = 0;

  // HashList / IndexList of the reference, copied from the device on request.
  std::vector<long long> HashList() { return frame_->dump<long long>(PI_DUMP_KEYS); }
  std::vector<int> IndexList() { return frame_->dump<int>(PI_DUMP_INDEX_LIST); }

  // GetPIdxList (src/hash_grid.cpp:196-214): the 27-cell candidate list.
  void GetPIdxList(const Vector3f& pos, std::vector<int>& pIdxList) {
    const float p[3] = {pos[0], pos[1], pos[2]};
    int64_t off[2] = {0, 0}, total = 0;
    pIdxList.assign(1024, 0);
    int rc = pi_hashgrid_neighbors(frame_->h, p, 1, off, pIdxList.data(), (int64_t)pIdxList.size(), &total);
    if (rc == PI_ERR_LIMIT) {
      pIdxList.assign((size_t)total, 0);
      rc = pi_hashgrid_neighbors(frame_->h, p, 1, off, pIdxList.data(), total, &total);
    }
    check(rc);
    pIdxList.resize((size_t)total);
  }

  // GetInBoxParticles (src/hash_grid.cpp:164-194).
  void GetInBoxParticles(Vector3f box1, Vector3f box2, std::vector<int>& insides) {
    const float b1[3] = {box1[0], box1[1], box1[2]}, b2[3] = {box2[0], box2[1], box2[2]};
    int64_t total = 0;
    insides.assign(4096, 0);
    int rc = pi_hashgrid_in_box(frame_->h, b1, b2, insides.data(), (int64_t)insides.size(), &total);
    if (rc == PI_ERR_LIMIT || total > (int64_t)insides.size()) {
      insides.assign((size_t)total, 0);
      rc = pi_hashgrid_in_box(frame_->h, b1, b2, insides.data(), total, &total);
    }
    check(rc);
    insides.resize((size_t)total);
  }

  // CalcXYZIdx / CalcCellHash (src/hash_grid.cpp:124-139): host arithmetic,
  // the same float expressions as the device keys.
  void CalcXYZIdx(const Vector3f& pos, std::array<int, 3>& xyzIdx) const {
    for (int i = 0; i < 3; ++i) xyzIdx[i] = int((pos[i] - Bounding[i * 2]) / CellSize);
  }
  long long CalcCellHash(const std::array<int, 3>& xyzIdx) const {
    if (xyzIdx[0] < 0 || xyzIdx[0] >= (int)XYZCellNum[0] || xyzIdx[1] < 0 || xyzIdx[1] >= (int)XYZCellNum[1] ||
        xyzIdx[2] < 0 || xyzIdx[2] >= (int)XYZCellNum[2])
      return -1;
    return (long long)XYZCellNum[0] * (long long)XYZCellNum[1] * (long long)xyzIdx[2] +
           (long long)XYZCellNum[0] * (long long)xyzIdx[1] + (long long)xyzIdx[0];
  }

 private:
  std::shared_ptr<detail::Frame> frame_;
};

// Evaluator (src/evaluator.cpp): field, gradient and the per-particle state.
class Evaluator {
 public:
  explicit Evaluator(std::shared_ptr<detail::Frame> f, float smooth_factor, float iso_factor)
      : frame_(std::move(f)), smooth_(smooth_factor), iso_factor_(iso_factor) {
    const pi_frame_info fi = frame_->info();
    iso_ = fi.iso_value;
    max_scalar_ = fi.max_scalar;
    Influnce2 = fi.influence2;
    Sigma = fi.sigma;
    Radius = fi.cell_size / 4.0f;
  }
  float Radius = 0.f, Influnce2 = 0.f, Sigma = 0.f;

  // The reference's public per-particle arrays, filled by LoadParticleState()
  // (a device-to-host copy of about 64 bytes per particle).
  std::vector<Vector3f> GlobalxMeans;
  std::vector<std::array<float, 9>> GlobalGs;  // row-major 3x3
  std::vector<float> GlobalDeterminant;
  std::vector<Vector3f> PariclesNormals;
  void LoadParticleState() {
    auto xm = frame_->dump<float>(PI_DUMP_XMEANS);
    auto g = frame_->dump<float>(PI_DUMP_G);
    GlobalDeterminant = frame_->dump<float>(PI_DUMP_DET);
    auto nr = frame_->dump<float>(PI_DUMP_NORMALS);
    const size_t n = xm.size() / 3;
    GlobalxMeans.resize(n);
    PariclesNormals.resize(n);
    GlobalGs.resize(n);
    for (size_t i = 0; i < n; ++i) {
      GlobalxMeans[i] = Vector3f(xm[3 * i], xm[3 * i + 1], xm[3 * i + 2]);
      PariclesNormals[i] = Vector3f(nr[3 * i], nr[3 * i + 1], nr[3 * i + 2]);
      for (int k = 0; k < 9; ++k) GlobalGs[i][k] = g[9 * i + k];
    }
  }

  // SingleEval / SingleEvalWithGrad (src/evaluator.cpp:60-125).
  void SingleEval(const Vector3f& pos, float& scalar) {
    const float p[3] = {pos[0], pos[1], pos[2]};
    check(pi_eval_field(frame_->h, p, 1, &scalar, nullptr));
  }
  void SingleEvalWithGrad(const Vector3f& pos, float& scalar, Vector3f& gradient) {
    const float p[3] = {pos[0], pos[1], pos[2]};
    float g[3];
    check(pi_eval_field(frame_->h, p, 1, &scalar, g));
    gradient = Vector3f(g[0], g[1], g[2]);
  }
  // Many points in one call: pts[m*3] -> scalar[m] (grad[m*3] optional).
  void Eval(const float* pts, int64_t m, float* scalar, float* grad = nullptr) {
    check(pi_eval_field(frame_->h, pts, m, scalar, grad));
  }

  // GridEval (src/evaluator.cpp:127-252): values at the (oversample+1)^3
  // points sample_points[i*4 .. i*4+2] into sample_points[i*4+3], sign change
  // against point 0 (">= 0"), and the reference's finite-difference
  // gradients (one-sided at the ends, central inside) into field_gradients.
  void GridEval(float* sample_points, float* field_gradients, float cellsize, bool& signchange, int oversample,
                bool grad_normalize = false) {
    const int k = oversample + 1, m = k * k * k;
    std::vector<float> pts(3 * (size_t)m), val((size_t)m);
    for (int i = 0; i < m; ++i)
      for (int c = 0; c < 3; ++c) pts[3 * i + c] = sample_points[i * 4 + c];
    check(pi_eval_field(frame_->h, pts.data(), m, val.data(), nullptr));
    signchange = false;
    for (int i = 0; i < m; ++i) {
      sample_points[i * 4 + 3] = val[i];
      if (!signchange) signchange = (sample_points[3] >= 0) ^ (val[i] >= 0);
    }
    const float step = cellsize / oversample;
    auto at = [&](int x, int y, int z) { return sample_points[(z * k * k + y * k + x) * 4 + 3]; };
    for (int z = 0; z < k; ++z)
      for (int y = 0; y < k; ++y)
        for (int x = 0; x < k; ++x) {
          const int idx[3] = {x, y, z};
          float g[3];
          for (int a = 0; a < 3; ++a) {
            int lo[3] = {x, y, z}, hi[3] = {x, y, z};
            --lo[a];
            ++hi[a];
            if (idx[a] == 0)
              g[a] = (at(x, y, z) - at(hi[0], hi[1], hi[2])) / step;
            else if (idx[a] == oversample)
              g[a] = (at(lo[0], lo[1], lo[2]) - at(x, y, z)) / step;
            else
              g[a] = (at(lo[0], lo[1], lo[2]) - at(hi[0], hi[1], hi[2])) / (step * 2);
          }
          if (grad_normalize) {
            const float nn = std::sqrt(g[0] * g[0] + g[1] * g[1] + g[2] * g[2]);
            for (float& c : g) c = (nn > 0.f) ? c / nn : 0.f;
          }
          const int i = z * k * k + y * k + x;
          for (int a = 0; a < 3; ++a) field_gradients[i * 3 + a] = g[a];
        }
  }

  float getNeighborFactor() const { return 4.0f; }
  float getSmoothFactor() const { return smooth_; }
  float getIsoFactor() const { return iso_factor_; }
  float getIsoValue() const { return iso_; }
  float getMaxScalar() const { return max_scalar_; }
  float getMinScalar() const { return 0.0f; }
  bool getUseXMean() const { return true; }
  float getXMeanDelta() const { return 0.9f; }

 private:
  std::shared_ptr<detail::Frame> frame_;
  float smooth_, iso_factor_, iso_ = 0.f, max_scalar_ = -1.f;
};

// TNode (include/iso_method_ours.h:30-78), read back from the device octree.
const char EMPTY = 0;
const char INTERNAL = 1;
const char LEAF = 2;
const char UNCERTAIN = 3;

struct TNode {
  Vector3f center;
  float half_length = 0.f;
  Vector4f node;
  char depth = 0;
  char type = EMPTY;
  unsigned long long id = 0;
  float curv = 0.f;  // checkEmptyAndCalcCurv's curvature
  std::array<std::shared_ptr<TNode>, 8> children;
  bool is_leaf() const { return type == LEAF || type == EMPTY; }
};

// SurfReconstructor (src/surface_reconstructor.cpp).  Run reads
// IS_CONST_RADIUS as the reference does: when it is false the frame takes the
// per-particle radii (radiuses, one per particle) and the radius argument is
// not used.
class SurfReconstructor {
 public:
  SurfReconstructor() = default;
  SurfReconstructor(std::vector<Vector3f>& particles, std::vector<float>& radiuses, Mesh* mesh, float radius,
                    int device = 0)
      : mesh_(mesh), radius_(radius), device_(device), radii_(radiuses) {
    xyz_.resize(particles.size() * 3);
    for (size_t i = 0; i < particles.size(); ++i)
      for (int c = 0; c < 3; ++c) xyz_[3 * i + c] = particles[i][c];
  }

  // Run (src/surface_reconstructor.cpp:409-479): hash grid, anisotropy,
  // normals, octree, extraction on the GPU; the mesh is copied into *mesh.
  void Run(float iso_factor, float smooth_factor) {
    pi_params p;
    pi_params_default(&p);
    p.radius = radius_;
    p.smooth_factor = smooth_factor;
    p.iso_factor = iso_factor;
    p.qef = qef_ ? 1 : 0;
    p.splash = splash_ ? 1 : 0;
    const bool var_r = !detail::const_radius_mode();
    if (var_r && !radii_.empty()) {
      float lo = radii_[0];
      for (float r : radii_) lo = r < lo ? r : lo;
      p.radius = lo;  // not used by the variable-radius path; any valid radius
    }
    frame_ = std::make_shared<detail::Frame>(detail::Context::get(device_), p);
    check(pi_frame_upload(frame_->h, xyz_.data(), (int64_t)(xyz_.size() / 3)));
    if (var_r) check(pi_frame_upload_radii(frame_->h, radii_.data(), (int64_t)radii_.size()));
    check(pi_run(frame_->h));
    info_ = frame_->info();
    searcher_ = var_r ? std::make_shared<MultiLevelSearcher>(frame_) : nullptr;
    hashgrid_ = var_r ? nullptr : std::make_shared<HashGrid>(frame_);
    evaluator_ = std::make_shared<Evaluator>(frame_, smooth_factor, iso_factor);
    root_.reset();
    if (mesh_) {
      int64_t nv = 0, nt = 0;
      check(pi_mesh_counts(frame_->h, &nv, &nt));
      std::vector<float> v((size_t)nv * 3);
      std::vector<int32_t> t((size_t)nt * 3);
      std::vector<uint64_t> k((size_t)nv * 2);
      check(pi_mesh_get(frame_->h, v.data(), t.data(), k.data()));
      mesh_->reset();
      mesh_->vertices.resize((size_t)nv);
      mesh_->vertexKeys.resize((size_t)nv);
      for (int64_t i = 0; i < nv; ++i) {
        mesh_->vertices[i] = Vertex(v[3 * i], v[3 * i + 1], v[3 * i + 2]);
        mesh_->vertexKeys[i] = {k[2 * i], k[2 * i + 1]};
      }
      mesh_->tris.resize((size_t)nt);
      for (int64_t i = 0; i < nt; ++i) mesh_->tris[i] = Triangle(t[3 * i] + 1, t[3 * i + 1] + 1, t[3 * i + 2] + 1);
      mesh_->verticesNum = (unsigned int)nv;
      mesh_->trianglesNum = (unsigned int)nt;
    }
    state_ = 1;
  }

  // Per-leaf QEF vertices (TNode::NodeCalcNode, commented out in the
  // reference at src/surface_reconstructor.cpp:258,270); off by default.
  void setQEF(bool on) { qef_ = on; }
  // Splash particles (GlobalSplash with its marking, commented out in the
  // reference at src/evaluator.cpp:675,690, switched on; GEN_SPLASH): the
  // mesh gains an icosahedron per isolated particle; off by default.
  void setSplash(bool on) { splash_ = on; }

  int getOverSampleQEF() const { return 2; }
  float getBorder() const { return 0.0f; }
  int getDepthMax() const { return info_.depth_max; }
  int getDepthMin() const { return info_.depth_min; }
  std::shared_ptr<HashGrid> getHashGrid() const { return hashgrid_; }
  std::shared_ptr<MultiLevelSearcher> getSearcher() const { return searcher_; }
  std::shared_ptr<Evaluator> getEvaluator() const { return evaluator_; }
  int getGlobalParticlesNum() const { return (int)(xyz_.size() / 3); }
  float getConstRadius() const { return radius_; }
  int getSTATE() const { return state_; }
  const pi_frame_info& getFrameInfo() const { return info_; }

  // The octree as TNode objects (copied from the device on first call).
  std::shared_ptr<TNode> getRoot() {
    if (root_ || !frame_) return root_;
    auto nodes = frame_->dump<pi_node>(PI_DUMP_NODES);
    std::vector<std::shared_ptr<TNode>> made(nodes.size());
    for (size_t i = 0; i < nodes.size(); ++i) {
      auto t = std::make_shared<TNode>();
      const pi_node& q = nodes[i];
      t->center = Vector3f(q.center[0], q.center[1], q.center[2]);
      t->half_length = q.half;
      t->node = Vector4f(q.node[0], q.node[1], q.node[2], q.node[3]);
      t->depth = (char)q.depth;
      t->type = (char)q.type;
      t->id = q.id;
      t->curv = q.curv;
      made[i] = t;
    }
    for (size_t i = 0; i < nodes.size(); ++i)
      if (nodes[i].first_child >= 0)
        for (int c = 0; c < 8; ++c) made[i]->children[c] = made[(size_t)nodes[i].first_child + c];
    root_ = made.empty() ? nullptr : made[0];
    return root_;
  }

 private:
  std::vector<float> xyz_;
  Mesh* mesh_ = nullptr;
  float radius_ = 0.f;
  int device_ = 0;
  std::vector<float> radii_;
  bool qef_ = false;
  bool splash_ = false;
  int state_ = 0;
  pi_frame_info info_{};
  std::shared_ptr<detail::Frame> frame_;
  std::shared_ptr<HashGrid> hashgrid_;
  std::shared_ptr<MultiLevelSearcher> searcher_;
  std::shared_ptr<Evaluator> evaluator_;
  std::shared_ptr<TNode> root_;
};

// UniformGrid (include/marching.h:18-70, src/marching.cpp), constant radius:
// Run samples the field on the lattice of spacing r over the particles' box
// (resizeRootBoxConstR) into _Scalars (x fastest) and, given a file name,
// writes <filepath>/<filename>.vti as the reference does through VTK.
class UniformGrid {
 public:
  UniformGrid(const std::vector<Vector3f>& particles, float radius, int device = 0)
      : _RADIUS(radius), device_(device) {
    _GlobalParticlesNum = (int)particles.size();
    xyz_.resize(particles.size() * 3);
    for (size_t i = 0; i < particles.size(); ++i)
      for (int c = 0; c < 3; ++c) xyz_[3 * i + c] = particles[i][c];
  }
  float _RADIUS = 0.f;
  float _SMOOTH_FACTOR = 2.0f;
  int _GlobalParticlesNum = 0;
  float _BoundingBox[6] = {0, 0, 0, 0, 0, 0};
  int dims[3] = {0, 0, 0};
  int steps[3] = {0, 0, 0};
  std::vector<float> _Scalars;

  // The reference computes its own iso value and ignores iso_value.
  void Run(float iso_value, const std::string& filename = "", const std::string& filepath = ".") {
    (void)iso_value;
    pi_params p;
    pi_params_default(&p);
    p.radius = _RADIUS;
    p.smooth_factor = _SMOOTH_FACTOR;
    frame_ = std::make_shared<detail::Frame>(detail::Context::get(device_), p);
    check(pi_frame_upload(frame_->h, xyz_.data(), (int64_t)(xyz_.size() / 3)));
    check(pi_hashgrid_build(frame_->h));
    check(pi_aniso_compute(frame_->h));
    check(pi_normals_compute(frame_->h));
    int64_t n = 0;
    check(pi_grid_dims(frame_->h, dims, _BoundingBox, &n));
    for (int i = 0; i < 3; ++i) steps[i] = dims[i] - 1;
    _Scalars.assign((size_t)n, 0.f);
    check(pi_grid_sample(frame_->h, _Scalars.data(), n));
    if (!filename.empty()) check(pi_grid_write_vti(frame_->h, (filepath + "/" + filename + ".vti").c_str()));
  }
  float getIsoValue() const { return frame_ ? frame_->info().iso_value : 0.f; }
  float getMaxScalar() const { return frame_ ? frame_->info().max_scalar : 0.f; }

 private:
  std::vector<float> xyz_;
  int device_ = 0;
  std::shared_ptr<detail::Frame> frame_;
};

}  // namespace pisurf

#ifndef PISURF_NO_GLOBAL_NAMES
using pisurf::UniformGrid;
using pisurf::Evaluator;
using pisurf::HashGrid;
using pisurf::Mesh;
using pisurf::MultiLevelSearcher;
using pisurf::SurfReconstructor;
using pisurf::TNode;
using pisurf::Triangle;
using pisurf::Vertex;
using pisurf::loadParticlesFromCSV;
using pisurf::readShonDyParticleData;
using pisurf::readShonDyParticleXDMF;
using pisurf::writeObjFile;
using pisurf::writePlyFile;
#endif

#endif  // PISURF_HPP
