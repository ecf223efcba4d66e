// Host program written against the reference's C++ API (the calls of
// runOurs, src/main.cpp:330-405), compiled against include/pisurf.hpp.
//   facade_main <xyz float32 file | particles .csv | particles .h5> <n> <radius> <out.obj> [radii float32 file]
// (also writes <out.obj>.ply, and <out.obj's directory>/grid.vti through
// UniformGrid).  With a radii file the program runs as the reference does
// with IS_CONST_RADIUS false: per-particle radii and MultiLevelSearcher.
// Prints one JSON line; exits 3 when no CUDA device is usable (the library
// has no CPU fallback).
#include <cstdio>
#include <fstream>
#include <iostream>
#include <vector>

#include "pisurf.hpp"

bool IS_CONST_RADIUS = true;

// Variable-radius run: the mesh, the searcher's radii and one neighbour query.
static int run_var_radius(std::vector<pisurf::Vector3f>& particles, std::vector<float>& radiuses, float radius,
                          const char* out_obj) {
  IS_CONST_RADIUS = false;
  Mesh mesh;
  try {
    SurfReconstructor constructor(particles, radiuses, &mesh, radius);
    constructor.Run(1.9f, 2.0f);
    writeObjFile(mesh, out_obj);
    std::shared_ptr<MultiLevelSearcher> searcher = constructor.getSearcher();
    std::vector<int> nb;
    searcher->GetNeighbors(particles[0], nb);
    std::printf(
        "{\"vertices\": %u, \"triangles\": %u, \"depth_max\": %d, \"depth_min\": %d, \"min_radius\": %.9g, "
        "\"max_radius\": %.9g, \"grids\": %d, \"neighbors0\": %zu, \"has_hash_grid\": %d}\n",
        mesh.verticesNum, mesh.trianglesNum, constructor.getDepthMax(), constructor.getDepthMin(),
        searcher->getMinRadius(), searcher->getMaxRadius(), searcher->getSearchersNum(), nb.size(),
        constructor.getHashGrid() ? 1 : 0);
  } catch (const pisurf::Error& e) {
    std::printf("{\"error\": %d, \"message\": \"%s\"}\n", e.code(), e.what());
    return e.code() == PI_ERR_CUDA ? 3 : 1;
  }
  return 0;
}

int main(int argc, char** argv) {
  if (argc != 5 && argc != 6) {
    std::fprintf(stderr, "usage: %s xyz.f32 n radius out.obj [radii.f32]\n", argv[0]);
    return 2;
  }
  const long n = std::atol(argv[2]);
  const float radius = (float)std::atof(argv[3]);
  std::vector<pisurf::Vector3f> particles;
  std::vector<float> radiuses;
  const std::string src = argv[1];
  if (src.size() > 4 && src.substr(src.size() - 4) == ".csv") {
    try {
      loadParticlesFromCSV(src, particles, radiuses, true);
    } catch (const pisurf::Error& e) {
      std::printf("{\"error\": %d, \"message\": \"%s\"}\n", e.code(), e.what());
      return 1;
    }
  } else if (src.size() > 3 && src.substr(src.size() - 3) == ".h5") {
    try {
      readShonDyParticleData(src, particles, radiuses);
    } catch (const pisurf::Error& e) {
      std::printf("{\"error\": %d, \"message\": \"%s\"}\n", e.code(), e.what());
      return 1;
    }
  } else {
    std::vector<float> raw((size_t)n * 3);
    std::ifstream in(argv[1], std::ios::binary);
    in.read(reinterpret_cast<char*>(raw.data()), (std::streamsize)(raw.size() * sizeof(float)));
    if (!in) {
      std::fprintf(stderr, "cannot read %s\n", argv[1]);
      return 2;
    }
    particles.resize((size_t)n);
    for (long i = 0; i < n; ++i) particles[i] = pisurf::Vector3f(raw[3 * i], raw[3 * i + 1], raw[3 * i + 2]);
  }
  if (argc == 6) {
    radiuses.resize(particles.size());
    std::ifstream rin(argv[5], std::ios::binary);
    rin.read(reinterpret_cast<char*>(radiuses.data()), (std::streamsize)(radiuses.size() * sizeof(float)));
    if (!rin) {
      std::fprintf(stderr, "cannot read %s\n", argv[5]);
      return 2;
    }
    return run_var_radius(particles, radiuses, radius, argv[4]);
  }
  radiuses.assign(particles.size(), radius);

  Mesh mesh;
  try {
    SurfReconstructor constructor(particles, radiuses, &mesh, radius);
    constructor.Run(1.9f, 2.0f);
    writeObjFile(mesh, argv[4]);
    writePlyFile(mesh, std::string(argv[4]) + ".ply");

    std::shared_ptr<Evaluator> ev = constructor.getEvaluator();
    std::shared_ptr<HashGrid> hg = constructor.getHashGrid();
    float s0 = 0.f;
    pisurf::Vector3f g0;
    ev->SingleEvalWithGrad(particles[0], s0, g0);
    std::vector<int> nb;
    hg->GetPIdxList(particles[0], nb);
    std::array<int, 3> xyz;
    hg->CalcXYZIdx(particles[0], xyz);
    const long long key0 = hg->CalcCellHash(xyz);
    std::vector<int> inbox;
    hg->GetInBoxParticles(pisurf::Vector3f(hg->Bounding[0], hg->Bounding[2], hg->Bounding[4]),
                          pisurf::Vector3f(hg->Bounding[1], hg->Bounding[3], hg->Bounding[5]), inbox);

    // GridEval over the root node's 27-point lattice (TNode::GenerateSampling)
    std::shared_ptr<TNode> root = constructor.getRoot();
    float samples[27 * 4], grads[27 * 3];
    for (int z = 0; z <= 2; ++z)
      for (int y = 0; y <= 2; ++y)
        for (int x = 0; x <= 2; ++x) {
          const int i = z * 9 + y * 3 + x;
          const int t[3] = {x, y, z};
          for (int c = 0; c < 3; ++c) {
            const float lo = root->center[c] - root->half_length, hi = root->center[c] + root->half_length;
            samples[i * 4 + c] = (1 - float(t[c]) / 2) * lo + (float(t[c]) / 2) * hi;
          }
          samples[i * 4 + 3] = 0.f;
        }
    bool signchange = false;
    ev->GridEval(samples, grads, 2 * root->half_length, signchange, 2);

    // walk the octree
    long leaves = 0, nodes = 0;
    std::vector<std::shared_ptr<TNode>> stack{root};
    while (!stack.empty()) {
      auto t = stack.back();
      stack.pop_back();
      ++nodes;
      if (t->is_leaf()) {
        if (t->type == pisurf::LEAF) ++leaves;
        continue;
      }
      for (auto& c : t->children)
        if (c) stack.push_back(c);
    }
    // the dense-grid mode (UniformGrid::Run writes <dir>/grid.vti)
    std::string out_obj = argv[4];
    const size_t slash = out_obj.find_last_of('/');
    const std::string dir = slash == std::string::npos ? std::string(".") : out_obj.substr(0, slash);
    UniformGrid ug(particles, radius);
    ug.Run(0.0f, "grid", dir);
    double gsum = 0.0;
    for (float v : ug._Scalars) gsum += v;
    std::printf(
        "{\"vertices\": %u, \"triangles\": %u, \"depth_max\": %d, \"depth_min\": %d, \"iso\": %.9g, "
        "\"max_scalar\": %.9g, \"scalar0\": %.9g, \"neighbors0\": %zu, \"key0\": %lld, \"in_box\": %zu, "
        "\"grid_sign_change\": %d, \"nodes\": %ld, \"leaves\": %ld, \"grid_dims\": [%d, %d, %d], "
        "\"grid_points\": %zu}\n",
        mesh.verticesNum, mesh.trianglesNum, constructor.getDepthMax(), constructor.getDepthMin(), ev->getIsoValue(),
        ev->getMaxScalar(), s0, nb.size(), key0, inbox.size(), signchange ? 1 : 0, nodes, leaves, ug.dims[0],
        ug.dims[1], ug.dims[2], ug._Scalars.size());
  } catch (const pisurf::Error& e) {
    std::printf("{\"error\": %d, \"message\": \"%s\"}\n", e.code(), e.what());
    return e.code() == PI_ERR_CUDA ? 3 : 1;
  }
  return 0;
}
