// Host-side context and frame state shared by the stage implementations.
#pragma once
#include <cuda_runtime.h>

#include <atomic>
#include <string>
#include <vector>

#include "../../include/pisurf.h"
#include "common.cuh"
#include "device.cuh"

struct pi_ctx;

namespace pisurf {

void ctx_account(pi_ctx* c, long long delta);

// Stream-ordered device buffer (cudaMallocAsync from the device's pool on the
// context stream), counted against the context budget.
template <class T>
struct DBuf {
  T* p = nullptr;
  size_t n = 0;
  pi_ctx* ctx = nullptr;
  cudaStream_t s = nullptr;
  DBuf() = default;
  DBuf(const DBuf&) = delete;
  DBuf& operator=(const DBuf&) = delete;
  void alloc(pi_ctx* c, cudaStream_t st, size_t count);
  // grows to at least count elements keeping the first `keep` elements
  void grow(pi_ctx* c, cudaStream_t st, size_t count, size_t keep);
  void release();
  ~DBuf() { release(); }
  size_t bytes() const { return n * sizeof(T); }
};

// One radius bin's hash grid (variable radius): the HashGrid of the bin's
// particles (src/hash_grid.cpp:36-69).
struct BinHost {
  float bounding[6];
  float cell;
  int nx, ny, nz;
  long long cellNum;
  int offBase;         // first entry of the bin in the concatenated offsets
  long long start;     // first sorted position of the bin's particles
  long long count;
  int radius_id;       // the particle whose radius sets the cell size
  int bin;             // index of the bin among all radius bins
};

struct GridHost {
  float bounding[6];
  float cell;
  int nx, ny, nz;
  long long cellNum;
  int nInvalid;
  int bits;  // radix sort width for key+1
};

// Configurations of the chunked field evaluation at octree samples
// (octree.cu): samples per lane, warps per block, staged candidates per warp.
constexpr int kMaxQefParts = 64;  // pi_ctx_tune_qef_parts

struct EvalConfig {
  int K, W, CB, bulk;
};
constexpr int kEvalConfigs = 10;
extern const EvalConfig kEvalTable[kEvalConfigs];

}  // namespace pisurf

struct pi_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  size_t budget = 0;
  std::atomic<long long> used{0};
  bool profile = false;
  // per kernel group (ProfGroup): event pairs (start, stop) not read yet, and
  // the accumulated device time, launches, candidate pairs and work units
  // (evaluations, or leaves for the QEF) since the last read
  std::vector<cudaEvent_t> prof_events[pisurf::kProfGroups];
  double group_ms[pisurf::kProfGroups] = {};
  int64_t group_launches[pisurf::kProfGroups] = {}, group_pairs[pisurf::kProfGroups] = {},
          group_units[pisurf::kProfGroups] = {};
  int smCount = 0;
  // one reference for the owner plus one per live frame; the context is
  // released when the last reference goes
  std::atomic<int> refs{1};
  // samples per lane of the chunked field evaluation, per dense-level kind
  // (0: leaf level, cell-octant buckets; 1: the level above, cell buckets);
  // 0 = not chosen yet (timed on the first such level), forced by pi_ctx_tune
  int eval_cfg[2] = {0, 0};  // chosen configuration + 1 per dense level kind (0: not yet)
  int eval_forced = 0;
  int qef_parts = 16;  // leaf level with the QEF on: parts pipelined against the QEF stream (1: none)
  // pinned host area for reads that need no synchronisation of their own:
  // per-stage counter snapshots (kPinSlots x kCounterWords words) and one
  // word for the hash grid's valid-key count; folded into the frame at the
  // end of the API call that produced them
  unsigned long long* hpin = nullptr;
  // the frame pi_reconstruct reuses from call to call when the context has
  // no budget (its device buffers and events carry over); freed with the
  // context
  pi_frame* recon = nullptr;
  // grid of the cooperative coarse-level octree kernel (0: no cooperative
  // launch on this device)
  int coop_blocks = 0;
  // a second stream for device-to-host copies that overlap the compute
  // stream (pi_reconstruct's triangle download), and its two events
  cudaStream_t copy_stream = nullptr;
  // the FP64 QEF of a level runs on its own stream beside the FP32 work that
  // follows it (the next level's sampling, the mesh topology); ev_qef_in
  // hands it the level's classification, ev_qef_done hands back the result
  cudaStream_t qef_stream = nullptr;
  cudaEvent_t ev_qef_in = nullptr, ev_qef_done = nullptr;
  cudaEvent_t ev_tris_ready = nullptr, ev_tris_copied = nullptr;
  cudaEvent_t ev_read = nullptr;  // the extraction's split count reads
  // the extraction's mesh topology, started beside the octree's last level
  // (extract_topology): its stream, the event that hands it the final tree,
  // the one that hands back its result, and its count reads
  cudaStream_t topo_stream = nullptr;
  cudaEvent_t ev_topo_in = nullptr, ev_topo_done = nullptr, ev_topo_read = nullptr;
};

struct pi_frame {
  pi_ctx* ctx = nullptr;
  pi_params P;
  int stage = 0;  // last completed: 0 none, 1 uploaded, 2 hash, 3 aniso, 4 normals, 5 octree, 6 mesh
  long long N = 0;
  pisurf::GridHost g;

  pisurf::DBuf<float> xyz;       // N*3, original order
  pisurf::DBuf<unsigned> misc;   // small scalars: bbox encodings, counters
  pisurf::DBuf<int> key;         // N, original order, -1 outside the grid
  pisurf::DBuf<uint32_t> sidx;   // N, IndexList: sorted position -> particle
  pisurf::DBuf<uint32_t> skey;   // N, sorted key+1
  pisurf::DBuf<int> off;         // C+1 cell offsets
  pisurf::DBuf<float4> pos, xm, ga, gb, nrm;  // N, sorted order
  pisurf::DBuf<float4> xlo;      // N, sorted order: centre minus its float rounding
  pisurf::DBuf<float> gfull;     // N*9, sorted order (dumps)
  pisurf::DBuf<float> det;       // N, sorted order (dumps)
  pisurf::DBuf<int8_t> f64flag;  // N, sorted order
  // QEF work in flight on the context's QEF stream (qef_join waits for it),
  // and whether the octree stage may leave the last level's QEF running for
  // the extraction to overlap (pi_run, pi_reconstruct)
  bool qef_inflight = false;
  bool defer_qef_join = false;
  bool extract_follows = false;  // pi_run: the extraction follows the octree (its topology may start early)
  // splash particles (pi_params.splash): the flag per particle (sorted
  // order), the sorted positions of the splash particles listed in particle
  // order, and their count
  pisurf::DBuf<int8_t> spl;
  pisurf::DBuf<int> splList;
  long long nSplash = 0;
  // variable radius (pi_frame_upload_radii): host and device radii, the grid
  // index of each particle, the bins' grids (host and a device view), the
  // searcher's min / max / average radius and the per-node min radius
  bool varR = false;
  std::vector<float> hrad;
  pisurf::DBuf<float> rad;
  // per-particle kernel constants (Influnce2, Sigma, nI = 4 r, 1 / nI^3) with
  // the reference's float / double semantics, original and sorted order
  pisurf::DBuf<float4> vrc, vrcs;
  pisurf::DBuf<int> pbin;
  std::vector<pisurf::BinHost> bins;
  pisurf::DBuf<pisurf::MultiGridView> mgv;
  float vrMinR = 0, vrMaxR = 0, vrAvgR = 0;
  pisurf::DBuf<float> nd_minr;
  // FP64 oracle state (fp64.cu), sorted order: centres, G, det; computed on
  // demand and invalid once the hash grid changes
  pisurf::DBuf<double> x64, g64, det64;
  pisurf::DBuf<int8_t> spl64;   // splash flags decided in double (splash mode)
  bool f64_ready = false;
  pisurf::DBuf<int> tmp;         // scan / sort scratch
  pisurf::DBuf<uint32_t> u32a, u32b, u32c;  // sort ping-pong scratch

  // scalars (Evaluator / SurfReconstructor members)
  float iso = 0, maxScalar = -1, influ2 = 0, sigma = 0;
  int dmax = 0, dmin = 0;
  float rootC[3] = {0, 0, 0}, rootH = 0;
  float bbox6[6] = {0, 0, 0, 0, 0, 0};  // loadRootBox tight box
  bool singleLayer = false;

  // octree, all levels concatenated in creation (level) order
  long long nNodes = 0;
  std::vector<long long> levelBegin;
  pisurf::DBuf<float4> nd_c;     // center xyz, half
  pisurf::DBuf<float4> nd_v;     // node xyz, value
  pisurf::DBuf<uint64_t> nd_id;
  pisurf::DBuf<int> nd_parent, nd_child;
  pisurf::DBuf<int8_t> nd_type, nd_depth, nd_sc;
  pisurf::DBuf<float> nd_curv;
  pisurf::DBuf<int4> nd_org;     // integer origin at depth-max resolution, size
  pisurf::DBuf<float> nd_samp;   // 27 sample values per node (QEF mode)
  pisurf::DBuf<int8_t> npart;    // leaf level in QEF mode: each node's part (read by the QEF stream too)

  // mesh
  long long nV = 0, nT = 0, nDual = 0;
  pisurf::DBuf<float> mv;        // nV*3
  pisurf::DBuf<int> mt;          // nT*3
  pisurf::DBuf<uint64_t> mk;     // nV*2
  pisurf::DBuf<int2> vedge;      // nV: the two leaf nodes whose edge each vertex bisects (-1 for splash)
  // the extraction's topology: unique interior leaf corners (dual vertices)
  // as lattice keys, their count, and whether it runs on the topology stream
  pisurf::DBuf<uint64_t> tp_uverts;
  long long tp_nu = 0;
  bool tp_inflight = false;

  // counters
  long long fieldEvals = 0, pairs = 0, bisectEvals = 0, fp64Count = 0, nLeaves = 0, nEmpty = 0;
  long long doneEvals = 0;  // evaluations the kernels performed (after deduplication)
  long long qefAccepted = 0, qefSingular = 0;
  long long gridPairs = 0;  // candidate pairs of the last uniform-grid sampling
  pisurf::DBuf<unsigned long long> dcount;  // device counters
  // stage timing: ev[2k], ev[2k+1] bracket stage slot k; the times are read
  // when the frame's next synchronisation point has passed
  cudaEvent_t ev[17] = {};
  // pi_reconstruct's host triangle buffer: when set and large enough, the
  // extraction copies the triangles there on the context's copy stream while
  // the bisection runs (tris_sent then holds until the call ends)
  int32_t* host_tris = nullptr;
  long long host_tcap = 0;
  bool tris_sent = false;
  int ev_pending = 0;   // bit k: slot k's events recorded, time not read yet
  int pin_pending = 0;  // bit k: pinned slot k written by this call, not folded yet
  float stage_ms[8] = {0, 0, 0, 0, 0, 0, 0, 0};
};

namespace pisurf {

// pinned snapshot slots
constexpr int kPinAniso = 0, kPinOctree = 1, kPinExtract = 2, kPinSlots = 3;
constexpr int kPinValid = kPinSlots;  // bit of pin_pending for the valid-key count
// after the slots: word 0 the valid-key count, word 1 the octree level's
// INTERNAL count; then the coarse-level kernel's level starts and depth
constexpr int kPinTopOffset = kPinSlots * kCounterWords + 8;
constexpr int kPinTopWords = 32;
// one word for the extraction's split count reads, one for the topology's
constexpr int kPinReadOffset = kPinTopOffset + kPinTopWords;
constexpr int kPinTopoReadOffset = kPinReadOffset + 8;
constexpr int kPinWords = kPinTopoReadOffset + 8;
// event that marks the INTERNAL count's copy in the octree level loop
constexpr int kLevelEvent = 16;
// Copies the frame's device counters into pinned slot `slot` (stream-ordered,
// no synchronisation); the values reach the frame in resolve_pending.
void counters_snapshot(pi_frame* f, int slot);
// Parameter checks of pi_frame_create (throws std::invalid_argument).
void check_params(const pi_params* p);
// Back to `stage` (0: nothing uploaded, 1: particles uploaded) with every
// result and counter cleared; device buffers are kept for reuse.
void frame_clear(pi_frame* f, int stage);
// Waits for the context stream once and folds every pending stage time and
// counter snapshot into the frame.
void resolve_pending(pi_frame* f);

// Hash cells per axis of the grid over `bounding` (HashGrid::XYZCellNum,
// src/hash_grid.cpp:24-27) into nn; returns their product.  Throws
// std::length_error, before any int conversion could overflow, when an axis
// or the product exceeds max_cells.
long long grid_cell_counts(const float bounding[6], float cell, long long max_cells, int nn[3]);

// Variable radius (varr.cu): radii upload, the bins' hash grids, the root
// box and scalars (resizeRootBoxVarR, CalculateMaxScalarVarR,
// RecommendIsoValueVarR); the anisotropy pass (aniso.cu).
void stage_upload_radii(pi_frame* f, const float* radii, long long n);
void stage_hashgrid_vr(pi_frame* f);
void host_root_and_scalars_vr(pi_frame* f);
void stage_aniso_vr(pi_frame* f);

void stage_upload_host(pi_frame* f, const float* xyz, long long n);
void stage_upload_device(pi_frame* f, const float* d_xyz, long long n);
void stage_hashgrid(pi_frame* f);
void stage_aniso(pi_frame* f);
void stage_normals(pi_frame* f);
void stage_octree(pi_frame* f);
void stage_extract(pi_frame* f);
// Splash particles (splash.cu): pos.w = 1 and the list in particle order
// after the anisotropy pass; the icosahedra at vertex v0 and triangle t0.
void stage_splash_list(pi_frame* f);
void splash_mesh(pi_frame* f, long long v0, long long t0);
// Grid (blocks) of the cooperative coarse-level octree kernel on `device`,
// 0 where cooperative launches are not available.
int top_levels_grid(int device, int sm_count);
// QEF vertices of the leaves of level [lb, le); scratch holds at least
// le - lb + 1 ints (device memory the caller no longer needs).
void qef_level(pi_frame* f, long long lb, long long le, int depth, const int8_t* npart = nullptr, int part = 0);
// The context stream waits for the QEF work in flight (no host wait).
void qef_join(pi_frame* f);
// The extraction's topology on the topology stream, after the context
// stream's ev_topo_in (the caller records it where the tree is final);
// topology_join makes the context stream wait for it; topology_fence also
// orders the topology stream after the context stream's work so far (before
// frees of buffers it allocated).
void topology_start(pi_frame* f);
void topology_join(pi_frame* f);
void topology_fence(pi_frame* f);
// UniformGrid: lattice of the loadRootBox box; sampling into d_out (device,
// x fastest) when cap holds it; returns the number of lattice points.
void uniform_grid_host(const pi_frame* f, float box[6], int steps[3], int dims[3]);
long long grid_sample(pi_frame* f, float* d_out, long long cap);
// Host formats: CSV particles (returns the row count; fills xyz / radius up
// to cap rows; cols = x, y, z, radius column indices) and binary PLY meshes.
long long load_csv(const char* path, float* xyz, float* radius, long long cap, int cols[4]);
// HDF5 particle files and XDMF frame lists (h5.cu): positions (and radii)
// as float, *n_out set before a short buffer is reported; one dataset as
// double; the frame files of an XDMF list.
long long load_hdf5(const char* path, float* xyz, float* radius, long long cap, bool want_radius,
                    long long* n_out);
std::vector<double> load_hdf5_dataset(const char* path, const char* name, std::vector<uint64_t>* dims);
std::vector<std::string> load_xdmf(const char* dir, const char* file, int target_frame);
void write_ply(const char* path, const float* verts, long long nv, const int32_t* tris, long long nt,
               int one_based);
void eval_points(pi_frame* f, const float* d_pts, long long m, float* d_val, float* d_grad);
// FP64 oracle (fp64.cu): per-particle state on demand; values at device
// points; the state in original particle order into host arrays (each may be
// null); iso, MaxScalar, Influnce2, Sigma in double.
void fp64_state(pi_frame* f);
void fp64_eval(pi_frame* f, const float* d_pts, long long m, double* d_val, double* d_grad);
void fp64_aniso_get(pi_frame* f, double* h_x3, double* h_g9, double* h_det);
void fp64_scalars(const pi_frame* f, double out4[4]);
long long neighbors(pi_frame* f, const float* h_pts, long long m, long long* h_off, int* h_idx,
                    long long cap);
long long in_box(pi_frame* f, const float* b1, const float* b2, int* h_idx, long long cap);
void dmc_host_table(int trans[256][8], bool flip[256], int code[256]);
// Events around the launches of kernel group g when the context profiles.
void prof_begin(pi_ctx* c, cudaStream_t s, int g);
void prof_end(pi_ctx* c, cudaStream_t s, int g);

// Striped device counters of a frame: zero them / read and sum the stripes
// (synchronises the context stream).
void counters_reset(pi_frame* f);
void counters_read(pi_frame* f, unsigned long long out[kCounters]);

// Host scalar constants with the reference's float/double semantics.
float bspline_host(float ratio, float sigma);

}  // namespace pisurf
