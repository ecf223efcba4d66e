/* pisurf.h - C ABI of the GB300-native particle-isosurface library.
 *
 * This is the drop-in boundary for the field-evaluation + octree-meshing
 * path of LCM1999/ParticleIsosurface.  The reference exposes that path as
 * in-process C++ classes (no plugin or FFI layer); each entry point below
 * names the reference interface it replaces.  Plain pointers and sizes only.
 *
 * Conventions
 *  - Every call returns PI_OK (0) or a negative PI_ERR_* code; the message of
 *    the last error on the calling thread is returned by pi_last_error().
 *  - Host pointers are caller-owned and only read/written during the call.
 *  - A frame is used by one thread at a time; frames of one context share its
 *    CUDA stream, so their work is ordered.
 *  - All computation runs on the GPU.  There is no CPU fallback: without a
 *    usable CUDA device every call that computes returns PI_ERR_CUDA.
 *  - Constant particle radius, anisotropic cubic B-spline kernel
 *    (the reference's USE_ANI=1, USE_POLY6=0, CALC_P_NORMAL=1,
 *    src/main.cpp:29-52).
 */
#ifndef PISURF_H
#define PISURF_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PI_OK 0
#define PI_ERR_INVALID (-1) /* bad argument: null pointer, n <= 0, non-finite position, ... */
#define PI_ERR_CUDA (-2)    /* CUDA runtime error (message in pi_last_error) */
#define PI_ERR_NOMEM (-3)   /* device memory budget of the context exceeded */
#define PI_ERR_STATE (-4)   /* stage called before the stages it depends on */
#define PI_ERR_LIMIT (-5)   /* size limit: >= 2^31 hash cells, octree depth > 20, ... */

typedef struct pi_ctx pi_ctx;
typedef struct pi_frame pi_frame;

/* Reconstruction parameters: the reference's SurfReconstructor arguments and
 * Run(iso_factor, smooth_factor) (include/surface_reconstructor.h:71-79). */
typedef struct pi_params {
  float radius;        /* particle radius r (RADIUS) */
  float smooth_factor; /* SMOOTH_FACTOR, default 2 */
  float iso_factor;    /* ISO_FACTOR, default 1.9 (poly6 variant only; kept for the API) */
  int32_t qef;         /* 0: leaf value at the cell centre (reference default);
                          1: per-leaf QEF vertex (TNode::NodeCalcNode switched on) */
  int32_t max_depth;   /* 0: no cap; otherwise PI_ERR_LIMIT if D_max exceeds it */
  int32_t splash;      /* 0: no splash particle (the reference as it ships);
                          1: splash particles (GlobalSplash with the marking of
                          src/evaluator.cpp:675,690 switched on, GEN_SPLASH):
                          a particle with <= 2 candidates or <= 2 neighbours
                          within 4r is a splash particle; it keeps the identity
                          G, takes no part in field sums, normals or node
                          emptiness, has a zero normal, and is appended to the
                          mesh as an icosahedron of radius r (12 vertices, 20
                          triangles, Mesh::AppendSplash_ConstR,
                          src/global.cpp:65-115) after the surface, in particle
                          order.  Constant radius only. */
  int32_t reserved[6];
} pi_params;

/* Per-frame results of the non-mesh stages (pi_frame_info). */
typedef struct pi_frame_info {
  int64_t num_particles;
  int64_t num_invalid_keys;  /* particles outside the hash grid (key -1) */
  float bounding[6];         /* HashGrid::Bounding */
  float cell_size;           /* HashGrid::CellSize = 4r */
  int32_t xyz_cell_num[3];   /* HashGrid::XYZCellNum */
  int64_t cell_num;          /* HashGrid::CellNum */
  int32_t depth_max, depth_min;
  float root_center[3], root_half;
  float iso_value, max_scalar, influence2, sigma;
  int64_t num_nodes, num_leaves, num_empty;
  int64_t num_dual_cells, num_vertices, num_triangles;
  int64_t field_evals;      /* reference-equivalent evaluations: the SingleEval calls the
                               reference makes for this frame's octree (27 lattice samples
                               per sampled node, the leaf values, QEF vertices), plus one
                               bisection chain per mesh vertex */
  int64_t candidate_pairs;  /* particle candidates visited by the evaluations performed */
  int64_t bisection_evals;
  int64_t fp64_eigen;       /* particles whose eigen-decomposition ran in FP64 */
  float stage_ms[8];        /* device time of upload, hash, aniso, normals, octree, qef,
                               extract, download */
  int64_t qef_accepted;     /* leaves whose QEF vertex lies in the cell (qef mode) */
  int64_t qef_singular;     /* leaves whose equilibrated normal matrix is singular
                               (an eigenvalue below 1e-12 of the largest); their
                               vertex is rejected, as the reference's non-finite
                               inverse is */
  int64_t grid_pairs;       /* candidate pairs of the last uniform-grid sampling */
  int64_t field_evals_performed; /* evaluations the kernels performed: distinct sample
                                    points (shared lattice points once), leaf values,
                                    QEF vertices, bisection midpoints */
  int32_t num_grids;        /* hash grids: 1, or the non-empty radius bins (per-particle radii) */
  float radius_min, radius_max; /* the radius, or the searcher's min / max radius
                                   (smallest * 0.99, largest * 1.01) */
  int64_t num_splash;       /* splash particles (pi_params.splash) */
} pi_frame_info;

/* Parity dumps (pi_stage_dump).  Arrays are in original particle order unless
 * noted.  Sizes from pi_stage_dump_size. */
#define PI_DUMP_KEYS 1        /* int64[N]  cell key or -1 (HashGrid::CalcCellHash) */
#define PI_DUMP_INDEX_LIST 2  /* int32[N]  HashGrid::IndexList (sorted order) */
#define PI_DUMP_CELL_OFFSETS 3 /* int32[C+1] cell c -> IndexList[off[c], off[c+1]) */
#define PI_DUMP_XMEANS 4      /* float[N*3] Evaluator::GlobalxMeans */
#define PI_DUMP_G 5           /* float[N*9] Evaluator::GlobalGs (row major) */
#define PI_DUMP_DET 6         /* float[N]   Evaluator::GlobalDeterminant */
#define PI_DUMP_NORMALS 7     /* float[N*3] Evaluator::PariclesNormals */
#define PI_DUMP_NODES 8       /* pi_node[num_nodes], creation (level) order */
#define PI_DUMP_FP64_FLAGS 9  /* int8[N] 1 where the eigen step ran in FP64 */
#define PI_DUMP_QEF_SAMPLES 10 /* float[num_nodes*27] GridEval sample values (qef mode) */
#define PI_DUMP_GRID_OF 11    /* int32[N]  hash grid (radius bin) of each particle */
#define PI_DUMP_SPLASH 12     /* int8[N]   1 for a splash particle (Evaluator::GlobalSplash) */
#define PI_DUMP_VERTEX_EDGES 13 /* int32[nV*2] the two leaves (indices into PI_DUMP_NODES) whose
                                   node points bound each mesh vertex's bisection; -1 for
                                   splash vertices */

typedef struct pi_node {
  uint64_t id;      /* TNode::id */
  float center[3];  /* TNode::center */
  float half;       /* TNode::half_length */
  float node[4];    /* TNode::node (position, value) */
  float curv;       /* checkEmptyAndCalcCurv curvature */
  int32_t parent;   /* index of the parent, -1 for the root */
  int32_t first_child; /* index of child 0 (children are consecutive), -1 if none */
  int8_t depth, type, signchange, pad; /* type: 0 EMPTY, 1 INTERNAL, 2 LEAF */
} pi_node;

const char* pi_last_error(void);
const char* pi_version(void);
void pi_params_default(pi_params* p);

/* Context: one CUDA device, one stream, a stream-ordered memory pool capped at
 * budget_bytes (0 = no cap). */
int pi_ctx_create(int device, size_t budget_bytes, pi_ctx** out);
int pi_ctx_destroy(pi_ctx* ctx);
/* launches: kernels launched by the library since load; bytes: device bytes
 * held by the context's frames. */
int pi_ctx_stats(const pi_ctx* ctx, uint64_t* launches, uint64_t* bytes);
/* Device time accounting of the dominant kernel class (field evaluation at
 * octree samples), for roofline reporting: when enabled, each launch is
 * bracketed with CUDA events on the context stream.  Read and reset with
 * pi_ctx_kernel_time. */
int pi_ctx_profile(pi_ctx* ctx, int enable);
/* field evaluation at octree samples: the chunked (k_q_eval), per-sample
 * (k_q_eval_thread) and leaf-value (k_leaf_level) kernels together; evals =
 * the evaluations they performed */
int pi_ctx_kernel_time(pi_ctx* ctx, double* total_ms, int64_t* launches, int64_t* pairs,
                       int64_t* evals);
/* The same per kernel group, arrays of ngroups entries: 0 chunked sampling
 * (k_q_eval), 1 per-sample sampling (k_q_eval_thread), 2 leaf values
 * (k_leaf_level), 3 edge bisection (k_bisect), 4 FP64 QEF (k_qef; units =
 * leaves solved), 5 uniform grid (k_grid_eval).  Reads and resets. */
#define PI_PROF_GROUPS 6
int pi_ctx_kernel_groups(pi_ctx* ctx, int32_t ngroups, double* ms, int64_t* launches, int64_t* pairs,
                         int64_t* units);
/* Samples per lane of the chunked field evaluation at the two finest
 * octree levels (a warp evaluates chunks of 32 x that many samples sharing a
 * candidate list).  By default each context times 1, 2 and 4 on its first
 * frame's levels and keeps the fastest per level kind; pi_ctx_tune(ctx, k)
 * with k = 1, 2 or 4 fixes it, k = 0 returns to timing.  The choice changes
 * no result.  pi_ctx_tuning reports it (0 = not chosen yet): out2[0] for the
 * leaf level, out2[1] for the level above. */
int pi_ctx_tune(pi_ctx* ctx, int32_t samples_per_lane);
int pi_ctx_tuning(const pi_ctx* ctx, int32_t* out2);
/* The whole configuration the timing chose per level kind (leaf level, level
 * above): out8 = K, warps per block, staged candidates per warp, staging (0:
 * box test from global memory, then cp.async of the survivors; 1: TMA bulk
 * copies of whole row runs, box test from shared memory), for each.  The
 * timing runs every configuration of a fixed table (pi_eval_configs()
 * entries: K 1, 2, 4; 4, 8 or 16 warps; 48, 64 or 96 staged candidates; both
 * stagings) once on the first level of each kind; pi_ctx_tune(ctx, K) fixes
 * K with 8 warps, 96 candidates and the first staging. */
int pi_ctx_tuning_config(const pi_ctx* ctx, int32_t* out8);
int pi_eval_configs(void);
/* Fixes entry `index` (0 to pi_eval_configs() - 1) of that table for both
 * level kinds; -1 returns to timing. */
int pi_ctx_tune_config(pi_ctx* ctx, int32_t index);
/* With the QEF on, the leaf level runs in `parts` parts (1 to 64; default
 * 16): buckets of its samples cut into z-ordered ranges of about equal
 * sample count, each range evaluated and its nodes classified on the context
 * stream, then those leaves' FP64 QEF solved on the context's QEF stream
 * while the next range is evaluated (the evaluator leaves room on every SM
 * for the QEF kernel).  1 runs the level in one piece.  The number of parts
 * changes no result: every sample, node and vertex is the same bit for bit.
 * pi_ctx_qef_parts reads it. */
int pi_ctx_tune_qef_parts(pi_ctx* ctx, int32_t parts);
int pi_ctx_qef_parts(const pi_ctx* ctx, int32_t* out);
/* The context stream as a cudaStream_t cast to void*. */
void* pi_ctx_stream(pi_ctx* ctx);

/* SurfReconstructor(particles, radiuses, mesh, radius)
 * (src/surface_reconstructor.cpp:13-28): a frame owns copies of the
 * particles and all device state of one reconstruction. */
int pi_frame_create(pi_ctx* ctx, const pi_params* params, pi_frame** out);
int pi_frame_destroy(pi_frame* f);
int pi_frame_upload(pi_frame* f, const float* xyz, int64_t n);        /* host xyz[n*3] */
int pi_frame_upload_device(pi_frame* f, const float* d_xyz, int64_t n); /* device xyz[n*3] */
/* Per-particle radii (radii[n], n = the particle count): the reference's
 * variable-radius SurfReconstructor (IS_CONST_RADIUS false) with its
 * neighbour query switched on.  Particles are binned by radius into bins of
 * about half the smallest radius (MultiLevelSearcher,
 * src/multi_level_reseacher.cpp:6-77), one hash grid per non-empty bin with
 * the bin's largest radius times 4 as its cell; a point's candidates are
 * the bins' 27-cell lists in bin order; each particle's kernel uses its own
 * radius (src/evaluator.cpp:16-29); the root box and depths follow
 * resizeRootBoxVarR (src/surface_reconstructor.cpp:124-149), a node is a
 * leaf by size when it is no larger than the smallest radius reaching it,
 * and the bisection stops at half the searcher's smallest radius.  The
 * radius of pi_params is not used.  The per-particle radii stay with the
 * frame until the next upload; not available with them: the QEF
 * (PI_ERR_INVALID), the uniform grid, pi_hashgrid_in_box and the FP64 oracle
 * (PI_ERR_STATE).  pi_frame_grid describes hash grid k (the grid's cells
 * start at offset_base in PI_DUMP_CELL_OFFSETS; radius_id is the particle
 * whose radius sets its cell, -1 for a constant radius). */
int pi_frame_upload_radii(pi_frame* f, const float* radii, int64_t n);
int pi_frame_grid(const pi_frame* f, int32_t k, float* bounding6, int32_t* dims3, float* cell_size, int64_t* count,
                  int64_t* offset_base, int32_t* radius_id);
/* Keeps the uploaded particles on the device and discards every later stage,
 * so pi_run reconstructs the same frame again (a new Run on resident input). */
int pi_frame_reset(pi_frame* f);

/* The stages of SurfReconstructor::Run (src/surface_reconstructor.cpp:409-479),
 * each enqueued on the context stream and synchronised before return. */
int pi_hashgrid_build(pi_frame* f);  /* loadRootBox + HashGrid ctor (:418-424) */
int pi_aniso_compute(pi_frame* f);   /* Evaluator::compute_Gs_xMeans (:432-435) */
int pi_normals_compute(pi_frame* f); /* resizeRootBoxConstR, CalculateMaxScalarConstR,
                                        RecommendIsoValueConstR, CalcParticlesNormal (:453-470) */
int pi_octree_build(pi_frame* f);    /* genIsoOurs state 0 (:326-407), incl. QEF when enabled */
int pi_extract_mesh(pi_frame* f);    /* genIsoOurs state 1 (:290-323) */
int pi_run(pi_frame* f);             /* all remaining stages (Run) */

int pi_frame_info_get(const pi_frame* f, pi_frame_info* out);

/* Mesh (Mesh::vertices / Mesh::tris, include/global.h:86-115): vertices as
 * float xyz, triangles as 0-based int32 index triples, vkeys (optional) the
 * sorted leaf-id pair naming each vertex (Mesh::insert_vert key). */
int pi_mesh_counts(const pi_frame* f, int64_t* nverts, int64_t* ntris);
int pi_mesh_get(pi_frame* f, float* verts, int32_t* tris, uint64_t* vkeys);
/* writeObjFile (src/main.cpp:54-67): "v %f %f %f" and 1-based "f" lines */
int pi_mesh_write_obj(pi_frame* f, const char* path);

/* Evaluator::SingleEval / SingleEvalWithGrad (src/evaluator.cpp:60-125) at m
 * host points; grad may be null.  Needs pi_normals_compute. */
int pi_eval_field(pi_frame* f, const float* pts, int64_t m, float* scalar, float* grad);

/* FP64 oracle on the GPU.  No counterpart in the reference, whose arithmetic
 * is float: the reference's formulas for the smoothed centres and anisotropy
 * matrices (compute_xMeans, compute_G_Yus, src/evaluator.cpp:465-512,585-654)
 * and for SingleEval / SingleEvalWithGrad (:60-125) evaluated in double, one
 * thread per particle or point over the whole 27-cell candidate list of the
 * frame's hash grid (no support culling, no deduplication, plain sums).  It
 * is the arbiter of the FP32 path's error reports (field, G and determinant
 * errors) and takes no part in the reconstruction.  Needs pi_hashgrid_build;
 * the per-particle state (104 bytes a particle) is computed on the first
 * call after the hash grid and kept with the frame.
 * pi_fp64_aniso: centres xmeans3[N*3], G g9[N*9] (row major), det[N], original
 * particle order; any output may be null.
 * pi_fp64_eval_field: field (and, when grad is not null, the normal-form
 * gradient of SingleEvalWithGrad) at m host points.
 * pi_fp64_scalars: iso value, MaxScalar, Influnce2, Sigma in double. */
int pi_fp64_aniso(pi_frame* f, double* xmeans3, double* g9, double* det);
int pi_fp64_eval_field(pi_frame* f, const float* pts, int64_t m, double* scalar, double* grad);
int pi_fp64_scalars(const pi_frame* f, double* out4);

/* HashGrid::GetPIdxList (src/hash_grid.cpp:196-214) for m host points:
 * offsets[m+1] and the concatenated particle indices; *total receives the
 * number of indices; PI_ERR_LIMIT (with *total set) if cap is too small. */
int pi_hashgrid_neighbors(pi_frame* f, const float* pts, int64_t m, int64_t* offsets, int32_t* idx,
                          int64_t cap, int64_t* total);
/* HashGrid::GetInBoxParticles (src/hash_grid.cpp:164-194). */
int pi_hashgrid_in_box(pi_frame* f, const float* box1, const float* box2, int32_t* idx, int64_t cap,
                       int64_t* total);

int pi_stage_dump_size(const pi_frame* f, int what, size_t* bytes);
int pi_stage_dump(pi_frame* f, int what, void* host_buf, size_t bytes);

/* UniformGrid (src/marching.cpp), the reference's dense-grid mode: the field
 * on a lattice of spacing r over the particles' box grown as in
 * UniformGrid::resizeRootBoxConstR (:42-55), values as gridSampling (:72-93)
 * computes them (SingleEval, x fastest).  pi_grid_dims needs the hash grid
 * (box6 = lattice min/max per axis, origin = box6[0], box6[2], box6[4]);
 * the sampling needs pi_normals_compute (iso value).  values/d_values must
 * hold npoints floats (PI_ERR_LIMIT otherwise).  pi_grid_write_vti writes the
 * samples as a VTK XML image ("scalars", raw appended Float32), the file the
 * reference writes through VTK (:160-185). */
int pi_grid_dims(pi_frame* f, int32_t* dims3, float* box6, int64_t* npoints);
int pi_grid_sample(pi_frame* f, float* values, int64_t cap);
int pi_grid_sample_device(pi_frame* f, float* d_values, int64_t cap);
int pi_grid_write_vti(pi_frame* f, const char* path);

/* Host data formats (no GPU needed).
 * pi_load_csv: loadParticlesFromCSV (src/main.cpp:215-275).  The header's
 * quote marks are removed and it is split at ','; the x, y and z columns are
 * the first titles matching the reference's case-insensitive patterns
 * ^(.*(:|_|-)( *)(x|0)("*)|x)$ (likewise y|1, z|2), the radius column (read
 * when radius is not null) the first matching ^((.*)radius|r)$.  Rows follow
 * until the first empty line, each value parsed as std::stof.  Call with
 * xyz = radius = null to count rows (*n); cols4 (may be null) receives the
 * x, y, z, radius column indices (-1 when the radius was not asked for).
 * PI_ERR_INVALID when a column is missing or a value does not parse (the
 * reference exits or throws there); PI_ERR_LIMIT when cap < rows.
 * pi_write_ply / pi_mesh_write_ply: writePlyFile (src/main.cpp:69-114), the
 * RPly binary file in the host byte order: "float32" x y z per vertex and a
 * "uchar"-counted "int" list per face with 0-based indices (tris given
 * 0-based, or 1-based when one_based is set). */
int pi_load_csv(const char* path, float* xyz, float* radius, int64_t cap, int64_t* n, int32_t* cols4);
/* pi_load_hdf5: readShonDyParticleData (src/main.cpp:281-327): the dataset
 * "position" (3N values, flat as the reference reads it, or N x 3) and, when
 * radius is not null, "particleRadius" (N values), converted to float; call
 * with xyz = null to count (*n).  The HDF5 library is not needed: the file
 * format is read by the library (superblock versions 0-3, version 1 and 2
 * object headers, symbol-table and compact groups, compact / contiguous /
 * chunked layouts with the deflate, shuffle and Fletcher-32 filters, integer
 * and IEEE float elements of either byte order).  PI_ERR_INVALID for a
 * missing file or dataset or an unsupported structure (named in the
 * message); PI_ERR_LIMIT when cap < N (with *n set).
 * pi_hdf5_dataset: any dataset of such a file as double (count, dims, rank).
 * pi_load_xdmf: readShonDyParticleXDMF (src/hdf5Utils.cpp:7-47): the frame
 * files of <dir>/<xdmf_file> (the text of each Xdmf/Domain/Grid/Grid/
 * Geometry/DataItem up to its first ':'), all of them, or only frame
 * target_frame (1-based) when it is in range; written to out separated by
 * '\n' and NUL-terminated, *len the bytes that takes, *frames the count. */
int pi_load_hdf5(const char* path, float* xyz, float* radius, int64_t cap, int64_t* n);
int pi_hdf5_dataset(const char* path, const char* name, double* out, int64_t cap, int64_t* count,
                    int64_t* dims8, int32_t* rank);
int pi_load_xdmf(const char* dir, const char* xdmf_file, int32_t target_frame, char* out, int64_t cap,
                 int64_t* len, int32_t* frames);
int pi_write_ply(const char* path, const float* verts, int64_t nv, const int32_t* tris, int64_t nt,
                 int32_t one_based);
int pi_mesh_write_ply(pi_frame* f, const char* path);

/* One call, host in / host out: upload, Run, download (the e2e path of a
 * frame).  verts/tris must hold max_verts / max_tris entries; the actual
 * counts are returned (PI_ERR_LIMIT if the buffers are too small).  A
 * context created without a budget keeps the frame of this call for the
 * next one (its device buffers stay allocated until pi_ctx_destroy); with a
 * budget the frame's memory is returned before the call ends. */
int pi_reconstruct(pi_ctx* ctx, const pi_params* params, const float* xyz, int64_t n, float* verts,
                   int64_t max_verts, int32_t* tris, int64_t max_tris, int64_t* nverts,
                   int64_t* ntris);

/* Hash-grid build that performs no device allocation.  This entry point has
 * no counterpart in the reference.  It is for host programs that cannot let a
 * library call cudaMalloc once they run: ones that reserve the whole GPU for
 * their own memory pool at start-up, or whose real-time rules forbid
 * allocation after initialisation.  The caller passes device buffers:
 * d_xyz[n*3] particles, and outputs d_keys[n] (cell key or -1, original
 * order), d_index_list[n] (particles in cell order, HashGrid::IndexList) and
 * d_cell_offsets[cell_offsets_len] (cell c holds d_index_list[off[c] ..
 * off[c+1])); the grid parameters are returned in host memory.  The results
 * equal pi_hashgrid_build's (PI_DUMP_KEYS / _INDEX_LIST / _CELL_OFFSETS).
 * Temporaries live in a fixed 12.5 MiB array inside the library's device
 * image, held on every GPU that loads the library until exit; so at most
 * PI_NOALLOC_MAX_PARTICLES particles and PI_NOALLOC_MAX_CELLS hash cells
 * (PI_ERR_LIMIT beyond them; also PI_ERR_LIMIT, with *cell_num_out set, when
 * cell_offsets_len < cell count + 1; a radius so small that a hash-grid axis
 * would exceed the cell limit is rejected the same way, *cell_num_out = -1).
 * The first call on a device looks up the array's device address
 * (cudaGetSymbolAddress) with that device current, and with CUDA's default
 * lazy module loading it is also the call that loads the library's device
 * code and the array onto that device, which takes device memory once.  So
 * make one warm-up call per device during the caller's initialisation, before
 * it reserves its memory pool or stops allowing allocation, and before any
 * stream capture; later calls allocate nothing.  The looked-up address is
 * kept for the life of the process: cudaDeviceReset on a device while this
 * library is loaded is not supported.  All calls on a device share the
 * array: calls whose GPU work may overlap (unordered streams) race and must
 * be serialised by the caller.  Work runs on `stream` (a cudaStream_t, 0 for
 * the default stream) and is complete on return. */
#define PI_NOALLOC_MAX_PARTICLES 1048576
#define PI_NOALLOC_MAX_CELLS 16777216
int pi_hashgrid_build_noalloc(const float* d_xyz, int64_t n, float radius, int32_t* d_keys,
                              int32_t* d_index_list, int32_t* d_cell_offsets, int64_t cell_offsets_len,
                              float* bounding_out6, int32_t* xyz_cell_num_out3, int64_t* cell_num_out,
                              void* stream);

/* Request loop (continuous batching).  The reference reconstructs one frame
 * per run of its driver loop (runOurs, src/main.cpp:330-405); a server keeps
 * `slots` worker threads, each with its own stream, admits queued requests
 * while their device-memory reservation fits in budget_bytes next to the
 * frames in flight and the resident frame states (0 = no cap; a request is
 * always admitted when nothing else holds memory), runs admitted frames
 * concurrently and keeps results in host memory until fetched.  A result
 * equals pi_run's on the same input.
 *  - Reservation: bytes_per_particle * n + fixed_bytes (by default 3072 B a
 *    particle + 128 MiB; pi_server_set_estimate changes it for later
 *    submissions).  With a budget the frame's context is capped at its
 *    reservation (at most the budget): a frame that needs more fails inside
 *    the worker and is queued again at the head with twice the reservation,
 *    up to the whole budget; a frame that needs more than the whole budget
 *    fails with PI_ERR_NOMEM.
 *  - Order: arrival order; when the head does not fit, up to 16 requests
 *    behind it that fit may pass it, and no request is passed more than 8
 *    times.
 *  - Resident frame states: each worker keeps its last frame (hash grid,
 *    octree, device buffers) until its next request; the next step of a
 *    sequence (pi_server_submit_seq, sequence != 0) goes to the idle worker
 *    holding that sequence's frame and is built in its buffers.  At most
 *    `slots` states are resident; with a budget their bytes count against it
 *    and idle workers give them back, least recently used first, when an
 *    admission needs the room. */
typedef struct pi_server pi_server;
int pi_server_create(int device, int slots, size_t budget_bytes, pi_server** out);
/* copies xyz[n*3]; returns a ticket */
int pi_server_submit(pi_server* s, const pi_params* params, const float* xyz, int64_t n, uint64_t* ticket);
/* the same for one step of a sequence of frames (an advected particle set):
 * its steps share a resident frame state where they can */
int pi_server_submit_seq(pi_server* s, const pi_params* params, const float* xyz, int64_t n, uint64_t sequence,
                         uint64_t* ticket);
int pi_server_set_estimate(pi_server* s, size_t bytes_per_particle, size_t fixed_bytes);
int pi_server_poll(pi_server* s, uint64_t ticket, int* done);
/* blocks until done; latency = completion - submission, queue = start - submission */
int pi_server_wait(pi_server* s, uint64_t ticket, int64_t* nverts, int64_t* ntris, double* latency_ms,
                   double* queue_ms);
/* copies the mesh (0-based triangles) and releases the request */
int pi_server_fetch(pi_server* s, uint64_t ticket, float* verts, int32_t* tris);
int pi_server_stats(pi_server* s, int64_t* completed, int64_t* in_flight, int64_t* max_in_flight,
                    int64_t* queued, int64_t* bytes_reserved);
/* out8: completed, bytes reserved by frames in flight, resident bytes
 * (counted with a budget), resident frame states, head-of-line passes,
 * re-queued reservations, steps that reused their sequence's resident
 * frame, budget */
int pi_server_info(pi_server* s, int64_t* out8);
/* finishes queued requests, then stops the workers */
int pi_server_destroy(pi_server* s);

/* The dual-marching-cubes canonicalisation table the library uses
 * (include/visitorextract.h:35-293 in the reference). */
int pi_dmc_table(int32_t* trans8x256, int8_t* flip256, int32_t* code256);

#ifdef __cplusplus
}
#endif
#endif
