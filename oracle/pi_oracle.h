/* CPU oracle for the particle-isosurface hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a restatement of the reference's OpenMP
 * CPU algorithm (LCM1999/ParticleIsosurface: src/hash_grid.cpp,
 * src/evaluator.cpp, src/surface_reconstructor.cpp, src/iso_method_ours.cpp,
 * include/traverse.h, src/visitorextract.cpp, src/global.cpp) used to check
 * the CUDA library and to time the reference CPU path.  The shipped library
 * never links or calls it.
 *
 * The oracle keeps the reference's data structures on purpose (std::map cell
 * table, per-query std::vector candidate lists, OpenMP tasks per octree node,
 * string-keyed mesh maps) so that its run time is the reference's.
 *
 * Parity unpinned: the reference cannot be compiled in this environment (it
 * needs Eigen 3.4, HDF5, VTK and MPI, and Windows-only headers) and ships no
 * tests, golden vectors or fixtures, so no output of the reference itself
 * checks this restatement.  Pinned: the DMC case table and triangle lists
 * against digests of the reference's source tables (tests/golden), and the
 * known-answer tests of tests/test_oracle.py.  Eigen's JacobiSVD,
 * determinant and inverse are restated (Jacobi SVD of the symmetric
 * covariance, cofactor determinant, adjugate inverse).
 */
#ifndef PI_ORACLE_H
#define PI_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* flags */
#define PIO_STD_SORT 1  /* order cells with std::sort like the reference (unstable);
                           default is (key, particle index) */
#define PIO_QEF 2       /* call NodeCalcNode on leaves (the two commented-out calls
                           at src/surface_reconstructor.cpp:258,270 switched on) */
#define PIO_FP64 4      /* evaluator arithmetic in double (the FP64 oracle) */
#define PIO_SPLASH 8    /* splash particles: the GlobalSplash marking of
                           src/evaluator.cpp:675,690 switched on, GEN_SPLASH on */

typedef struct pio_frame pio_frame;

/* splash flag per particle (after stage 2; zeros without PIO_SPLASH) */
int pio_get_splash(const pio_frame* h, int8_t* out);
pio_frame* pio_create(const float* xyz, int64_t n, float radius, float smooth_factor,
                      float iso_factor, int flags);
/* Variable radius (per-particle radii, the reference's non-constant-radius
 * SurfReconstructor with its neighbour query switched on): the same stages
 * with the MultiLevelSearcher in place of the hash grid. */
pio_frame* pio_create_var(const float* xyz, const float* radii, int64_t n, float smooth_factor,
                          float iso_factor, int flags);
/* grids: 1 for a constant radius, else the searcher's non-empty bins in bin
 * order; per grid its bounding box, cell counts, cell size, particle count,
 * the particle whose radius sets the cell (-1 for a constant radius), and
 * its particles (bin-local order), their keys, and IndexList as particle
 * indices */
int pio_num_bins(const pio_frame* f);
int pio_bin_info(const pio_frame* f, int bin, float* bounding6, int64_t* xyz_cell_num3, int64_t* cell_num,
                 float* cell_size, int64_t* count, int32_t* radius_id);
int pio_bin_lists(const pio_frame* f, int bin, int32_t* particles, int64_t* keys, int32_t* index_list);
/* MultiLevelSearcher min / max / average radius */
int pio_searcher_radii(const pio_frame* f, float* out3);
void pio_destroy(pio_frame* f);
void pio_set_threads(int nthreads);

/* Stages of SurfReconstructor::Run (src/surface_reconstructor.cpp:409-479).
 * 1 box + hash grid, 2 anisotropy (compute_Gs_xMeans), 3 depth/iso/normals,
 * 4 octree (genIsoOurs state 0), 5 extraction (genIsoOurs state 1).  Stages
 * run in order; pio_run runs all of them. */
int pio_stage(pio_frame* f, int stage);
int pio_run(pio_frame* f);
double pio_stage_seconds(const pio_frame* f, int stage);
/* 0 field evals (SingleEval calls), 1 candidate pairs of those evals,
 * 2 dual cells, 3 bisection evals */
int64_t pio_counter(const pio_frame* f, int which);

/* hash grid */
int pio_grid_info(const pio_frame* f, float* bounding6, int64_t* xyz_cell_num3,
                  int64_t* cell_num, float* cell_size);
int pio_get_keys(const pio_frame* f, int64_t* keys);          /* per particle */
int pio_get_index_list(const pio_frame* f, int32_t* idx);     /* IndexList */
int64_t pio_num_cells(const pio_frame* f);                    /* StartList size */
int pio_get_cells(const pio_frame* f, int64_t* hash, int32_t* start, int32_t* end);
/* GetPIdxList for m points: offsets[m+1] (int64) then the lists; returns total
 * or -1 if cap is too small */
int64_t pio_neighbors(pio_frame* f, const float* pts, int64_t m, int64_t* offsets,
                      int32_t* out, int64_t cap);
int64_t pio_in_box(pio_frame* f, const float* box1, const float* box2, int32_t* out,
                   int64_t cap);

/* evaluator state; double outputs whatever the arithmetic */
int pio_get_aniso(const pio_frame* f, double* xmeans3, double* g9, double* det);
int pio_get_normals(const pio_frame* f, double* normals3);
int pio_scalars(const pio_frame* f, double* out4); /* iso, max scalar, Influnce2, Sigma */
int pio_depths(const pio_frame* f, int32_t* out2, float* root_center3, float* root_half);
/* SingleEval / SingleEvalWithGrad at m points */
int pio_eval(pio_frame* f, const float* pts, int64_t m, double* scalar, double* grad3);

/* octree nodes in creation order */
int64_t pio_num_nodes(const pio_frame* f);
int pio_get_nodes(const pio_frame* f, uint64_t* id, int8_t* depth, int8_t* type,
                  float* node4, float* center3, float* half, float* curv,
                  int8_t* signchange, int32_t* parent);

/* mesh (Mesh::vertices / Mesh::tris, 1-based indices as in the OBJ) */
int pio_mesh_counts(const pio_frame* f, int64_t* nverts, int64_t* ntris);
int pio_mesh_get(const pio_frame* f, float* verts3, int32_t* tris3, uint64_t* vkeys2);
int pio_write_obj(const pio_frame* f, const char* path);

/* the oracle's own dual-marching-cubes tables, for table tests */
int pio_dmc_table(int32_t* trans8x256, int8_t* flip256, int32_t* code256);

/* UniformGrid (src/marching.cpp): the sampling lattice of the loadRootBox box
 * resized by resizeRootBoxConstR, and SingleEval at every lattice point (x
 * fastest); pio_grid_sample needs stage 3. */
int pio_uniform_grid(const pio_frame* f, float* box6, int32_t* steps3, int32_t* dims3);
int pio_grid_sample(pio_frame* f, double* out, int64_t n);

#ifdef __cplusplus
}
#endif
#endif
