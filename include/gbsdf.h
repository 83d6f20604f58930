/*
 * gbsdf.h — C ABI of the GB300 mesh-to-SDF engine.
 *
 * Drop-in boundary for the reference's "Fast SDF" path (golemid/rhizome_v24.15):
 *
 *   static bool CudaRasterizer::compute_mesh_sdf(
 *       const std::vector<CudaTriangle>& triangles, float voxel_size,
 *       glm::ivec3 min_coord, glm::ivec3 max_coord,
 *       std::vector<float>& out_distances, float& out_time_ms);
 *     declared native/src/engine/sdf/cuda_rasterizer.hpp:21-28,
 *     defined  native/src/engine/sdf/cuda_rasterizer.cu:1163-1265
 *     (fast path rhi_compute_mesh_sdf_fast, cuda_rasterizer.cu:796-1159)
 *
 *   static std::shared_ptr<CudaVolumeGrid> CudaRasterizer::build_from_mesh(
 *       const TriangleMesh& mesh, float voxel_size, float& out_time_ms);
 *     declared native/src/engine/sdf/cuda_rasterizer.hpp:31-35,
 *     defined  native/src/engine/sdf/cuda_rasterizer.cu:1340-1435
 *
 * Plain pointers and sizes only. Grid contract (cuda_rasterizer.cu:117-118):
 * dims = max - min + 1 (inclusive lattice), value at (x, y, z) is for the world
 * point ((min.x+x) h, (min.y+y) h, (min.z+z) h), dense, x fastest; negative
 * inside, inside <=> |generalized winding number| >= 0.5.
 *
 * Errors: every entry point returns a gbsdf_status; 0 is success. On any
 * non-zero status the output buffer is left untouched (the reference's
 * "output untouched on failure" contract, cuda_rasterizer.cu:788-791), and a
 * one-line reason is written to err (if err != NULL and errlen > 0).
 * There is no CPU fallback: without a usable CUDA device the call fails.
 */
#ifndef GBSDF_H
#define GBSDF_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Triangle record, layout of the reference's CudaTriangle
 * (native/src/engine/sdf/cuda_types.hpp:18-21): v0, v1, v2, unit normal; 48 bytes.
 * The normal is carried but not used by the SDF. */
typedef struct gbsdf_tri {
    float v0[3];
    float v1[3];
    float v2[3];
    float n[3];
} gbsdf_tri;

typedef enum gbsdf_status {
    GBSDF_OK = 0,
    GBSDF_EINVAL = 1,   /* bad arguments, empty mesh, non-finite or out-of-range coordinates */
    GBSDF_EGUARD = 2,   /* reference int-range guard declines the fast path (cuda_rasterizer.cu:816-820) */
    GBSDF_ECSR = 3,     /* reference supercell-CSR guard declines (cuda_rasterizer.cu:867-869) */
    GBSDF_EVERIFY = 4,  /* sign verification found systematic divergence (cuda_rasterizer.cu:1124-1132):
                           the caller falls back to the legacy exact path */
    GBSDF_ENOMEM = 5,   /* device or pinned host allocation failed (cuda_rasterizer.cu:913-917) */
    GBSDF_ECUDA = 6,    /* CUDA runtime error */
    GBSDF_ENODEV = 7    /* no usable CUDA device */
} gbsdf_status;

typedef enum gbsdf_mode {
    /* The reference's algorithm: its Godunov update, its round loop (<= 8 rounds of
     * 6 sweeps, audit-gated extra rounds, clamp), parity signs, 3 x 4096 stratified
     * probes and r = 24 patch boxes, its decline conditions. Sweeps are lockstep
     * (deterministic); winding signs are decided exactly. */
    GBSDF_MODE_REFERENCE = 0,
    /* Exact signs and the corrected, monotone Godunov update run to its (unique) fixed
     * point; no int-range / CSR guards. */
    GBSDF_MODE_EXACT = 1,
    /* Exact signs with the reference's distances: signed crossings (the winding number of
     * a closed, consistently oriented mesh, overlapping shells included) along rays 1000x
     * closer to the lattice points than the reference's jitter; columns through holes
     * (nonzero signed total) and the stratified probes decided by the exact winding
     * number; voxels within 1e-3 voxel of the surface are on it (inside). Reference
     * eikonal and decline conditions. */
    GBSDF_MODE_EXACT_SIGNS = 2,
    /* Reference mode's signs plus learned proposals: a small network (32 brick features ->
     * 64 -> 64 -> 1, BF16 weights, FP32 accumulation) scores every 8^3 brick's sign-error
     * risk and the riskiest bricks are re-decided by the exact winding kernel after the
     * stratified probes; the network never supplies a sign. Where a probe finds a mismatch
     * (the plain path would patch boxes or decline), no box is patched: the signs are
     * re-decided instead -- signed crossings along near-lattice rays, the exact winding
     * number for rays through holes (stats->escalated) -- and no brick is proposed (the
     * signs are no longer the plain path's). No int-range guard. Needs opt->mlp_params (or
     * opt->brick_scores). */
    GBSDF_MODE_LEARNED = 3
} gbsdf_mode;

typedef enum gbsdf_path {
    GBSDF_PATH_AUTO = 0,   /* reference dispatch: legacy exact kernel below 32M voxels,
                              fast path at or above (cuda_rasterizer.cu:1189) */
    GBSDF_PATH_FAST = 1,   /* always the fast path */
    GBSDF_PATH_LEGACY = 2  /* always the legacy exact kernel (cuda_rasterizer.cu:97-185) */
} gbsdf_path;

typedef struct gbsdf_options {
    int32_t mode;          /* gbsdf_mode */
    int32_t path;          /* gbsdf_path */
    int32_t device;        /* CUDA device ordinal */
    int32_t tris_on_device;/* 1: `tris` is a device pointer */
    int32_t max_rounds;    /* exact mode: safety cap on sweep rounds (0 = default 4096) */
    int32_t mlp_budget;    /* learned mode: most bricks proposed (0 = 1/16 of the bricks) */
    float mlp_threshold;   /* learned mode: risk probability above which a brick is proposed */
    int32_t wait_poll_limit; /* the eikonal's bounded waits on staged tiles: 0 = the default limit
                                (2^17 polls, each suspending the thread for at most 20 us until
                                the tile lands), > 0 = that many polls, < 0 = no polling (every wait
                                gives up at once: exercises the failure path, which returns
                                GBSDF_ECUDA with the output untouched) */
    const float* mlp_params; /* learned mode: GBSDF_MLP_PARAMS FP32 parameters in device memory */
    const float* brick_scores; /* learned mode, instead of the network: caller-supplied risk
                                  logits, one per 8^3 brick (x fastest), in device memory */
    int32_t sweep_schedule; /* eikonal sweep schedules (identical results), x + 10 w: x = 1 x sweep
                               staged by cp.async, 2 by TMA tiles on a CTA-barrier ring, 3 by TMA
                               tiles on a warp-specialised mbarrier pipeline, 4 the same with two
                               lines per thread updated in packed FP32 pairs (the reference's
                               update at voxel sizes 2^-20 to 2^20; otherwise 3 runs), 5 the
                               pipeline with 16-voxel chunks staged as 20-column boxes; w = 1 y / z walks
                               staged by cp.async, 2 by TMA batches on a pipeline, 3 the same
                               with four adjacent lines per thread, 4 the same with the lines'
                               updates in packed FP32 pairs (the reference's update at voxel
                               sizes 2^-20 to 2^20; otherwise 3 runs); a 0 digit (and
                               0 overall) = autotuned (the first build of a lattice class times
                               the candidates for the rounds after the first; the first round
                               takes 3 + 10 x 4). Every lattice can take the TMA schedules: the
                               sweeps run in copies with rows padded to a multiple of 8 voxels. */
    int32_t host_output;    /* host outputs: 0 = a page-locked output is written by the sign-apply
                               kernel through its device mapping (no staging copy), others are
                               staged in device memory and copied; 1 = always stage and copy */
    int32_t winding_eval;   /* exact winding decisions: 0 = clustered (far clusters by a dipole
                               with a rigorous error bound, undecided voxels summed exactly;
                               same decisions), 1 = every voxel summed triangle by triangle */
    int32_t splat_dense_cut; /* binned triangles per 8^3 brick above which the band splat takes the
                                brick with its sub-brick kernel: 0 = autotuned per lattice class
                                (gbsdf_stats.splat_dense_cut reports it), > 0 = that cut.
                                Identical results at every cut. */
} gbsdf_options;

/* Learned sign-risk model: parameter count and brick feature count. */
#define GBSDF_MLP_PARAMS 6337
#define GBSDF_MLP_FEATURES 32

typedef struct gbsdf_stats {
    int32_t status;
    int32_t path_taken;    /* gbsdf_path actually run (FAST or LEGACY) */
    float ms_total;        /* wall time of the call */
    float ms_h2d, ms_prep, ms_splat, ms_parity, ms_fixup, ms_eikonal, ms_verify, ms_apply, ms_d2h;
    int32_t eikonal_rounds;
    int32_t extra_rounds;
    int32_t probes;
    int32_t sites;
    int32_t patch_rounds;
    int32_t splat_dense_cut; /* binned triangles per 8^3 brick above which the band splat takes the
                                brick with its sub-brick kernel (autotuned per lattice class) */
    int64_t unknown_columns;
    int64_t fixup_voxels;
    int64_t far_residual;
    int64_t safe_clamped;
    int64_t patched_voxels;
    int64_t fp64_rechecks;
    int64_t band_voxels;
    int64_t splat_evals;   /* exact point-triangle distance evaluations */
    int64_t gwn_pairs;     /* point-triangle solid-angle evaluations */
    int64_t brick_pairs;   /* (triangle, brick) pairs binned for the splat */
    int64_t csr_entries;   /* entries of the reference's supercell CSR */
    int64_t kernel_launches; /* CUDA kernels this call launched */
    int64_t proposed;      /* learned mode: bricks the network proposed for the exact winding number */
    int64_t sweep_schedule; /* schedules that ran in the rounds after the first: x schedule (1-5)
                               + 10 x walk schedule (1-4), numbered as in
                               gbsdf_options.sweep_schedule */
    int64_t winding_certified; /* exact winding decisions settled by the cluster bound */
    int64_t winding_summed;    /* ... and by the triangle-by-triangle sum */
    int64_t escalated;         /* learned mode: 1 when the stratified verify diverged and the signs
                                  were re-decided (signed crossings, exact winding number for rays
                                  through holes) instead of declining */
    double band_err_fp64;      /* largest |FP32 band distance - FP64 distance| over the sampled band
                                  voxels, in voxels (fast path; 0 when no band voxel was sampled) */
    int64_t band_err_samples;  /* band voxels sampled for band_err_fp64 */
    float ms_sweeps;           /* fast path: the directional sweeps of the eikonal stage alone (from
                                  the first sweep's launch to the last's end, round bookkeeping
                                  included; without the padded copies, audit and clamp that
                                  ms_eikonal also holds) */
    int32_t sweep_schedule_first; /* the schedules of the first round (x + 10 x walk): the default
                                     plan unless forced; the autotuner picks the later rounds'
                                     (sweep_schedule) */
} gbsdf_stats;

/* Fill `opt` with defaults: reference mode, AUTO path, device 0, host triangles. */
void gbsdf_default_options(gbsdf_options* opt);

/* Replaces CudaRasterizer::compute_mesh_sdf (cuda_rasterizer.hpp:21-28,
 * cuda_rasterizer.cu:1163-1265). `out` holds dims.x*dims.y*dims.z floats, on the
 * device when out_on_device != 0, else in host memory (pinned or pageable). */
int gbsdf_compute_mesh_sdf(const gbsdf_tri* tris, int64_t n_tris, float voxel_size, const int32_t min_coord[3],
                           const int32_t max_coord[3], float* out, int32_t out_on_device,
                           const gbsdf_options* opt, gbsdf_stats* stats, char* err, size_t errlen);

/* One mesh of a batched call. */
typedef struct gbsdf_mesh_desc {
    const gbsdf_tri* tris;   /* host or device (opt->tris_on_device) */
    int64_t n_tris;
    float voxel_size;
    int32_t min_coord[3];
    int32_t max_coord[3];
    float* out;              /* dims.x*dims.y*dims.z floats, host or device (out_on_device) */
    int32_t status;          /* written: this mesh's gbsdf_status */
    int32_t pad;
} gbsdf_mesh_desc;

/* Batched form of gbsdf_compute_mesh_sdf (the descriptor list of the reference-side
 * C ABI plan). With the fast path (opt->path == GBSDF_PATH_FAST) in reference, exact-signs
 * or learned mode (the network's parameters, not caller-supplied brick scores) the meshes
 * run as one planned batch (gbsdf_batch_create / _run / _destroy below, one CUDA graph,
 * every mesh its own branch); otherwise they run back to back through
 * gbsdf_compute_mesh_sdf. Returns GBSDF_OK when every mesh succeeded, else
 * the first failing mesh's status; per-mesh statuses are written to meshes[i].status and
 * per-mesh statistics to stats[i] (stats may be NULL). A failing mesh's output is left
 * untouched. No reference counterpart. */
int gbsdf_compute_mesh_sdf_batch(gbsdf_mesh_desc* meshes, int32_t n_meshes, int32_t out_on_device,
                                 const gbsdf_options* opt, gbsdf_stats* stats, char* err, size_t errlen);

/* A planned batch: the meshes' device buffers are sized from one counting pass, and the
 * whole build of every mesh -- upload, binning, splat, parity, exact-winding fixup,
 * eikonal rounds, verify / patch, sign apply, download -- is captured once as a CUDA
 * graph with no host round trip inside, one independent branch per mesh. A run replays
 * the graph: the descriptors' pointers and lattices are fixed at creation, their
 * triangle contents may change between runs (a run whose counts outgrow the planned
 * lists re-plans itself and runs again). Fast path only; opt->mode must be
 * GBSDF_MODE_REFERENCE, GBSDF_MODE_EXACT_SIGNS or GBSDF_MODE_LEARNED (with opt->mlp_params
 * in device memory, kept alive by the caller while the batch exists; the budget and
 * threshold apply to each mesh). No reference counterpart. */
typedef struct gbsdf_batch gbsdf_batch;
int gbsdf_batch_create(const gbsdf_mesh_desc* meshes, int32_t n_meshes, int32_t out_on_device,
                       const gbsdf_options* opt, gbsdf_batch** batch, char* err, size_t errlen);
/* statuses[i] / stats[i] receive each mesh's gbsdf_status / statistics (either may be
 * NULL); returns GBSDF_OK when every mesh succeeded, else the first failing status. */
int gbsdf_batch_run(gbsdf_batch* batch, int32_t* statuses, gbsdf_stats* stats, char* err, size_t errlen);
void gbsdf_batch_destroy(gbsdf_batch* batch);

/* Lattice of CudaRasterizer::build_from_mesh (cuda_rasterizer.cu:1354-1372): bounding box
 * of all vertices, padded by 10 voxels, floor/ceil onto the voxel lattice. */
int gbsdf_mesh_lattice(const float* verts, int64_t n_verts, float voxel_size, int32_t min_coord[3],
                       int32_t max_coord[3], char* err, size_t errlen);

/* Replaces CudaRasterizer::build_from_mesh (cuda_rasterizer.cu:1340-1435): builds the
 * triangles on the device (degenerate |cross|^2 <= 1e-12 and out-of-range faces dropped,
 * kept in index order, math_utils.cuh:484-514) and computes the SDF on the lattice given
 * by gbsdf_mesh_lattice. `indices` has n_indices entries (3 per face). */
int gbsdf_build_from_mesh(const float* verts, int64_t n_verts, const uint32_t* indices, int64_t n_indices,
                          float voxel_size, const int32_t min_coord[3], const int32_t max_coord[3], float* out,
                          int32_t out_on_device, const gbsdf_options* opt, gbsdf_stats* stats, char* err,
                          size_t errlen);

/* Brick features of the learned sign-risk model for one lattice (8^3 bricks, x fastest):
 * GBSDF_MLP_FEATURES floats per brick written to `features_dev` (device memory,
 * capacity_bricks bricks). n_bricks[3] receives the brick grid. The work runs on the device
 * that holds features_dev; device triangles (tris_on_device = 1) must be on that device too
 * (GBSDF_EINVAL otherwise). No counterpart in the reference. */
int gbsdf_brick_features(const gbsdf_tri* tris, int64_t n_tris, float voxel_size, const int32_t min_coord[3],
                         const int32_t max_coord[3], int32_t tris_on_device, float* features_dev,
                         int64_t capacity_bricks, int32_t n_bricks[3], char* err, size_t errlen);

/* The model's forward pass: logits_dev[i] for the n feature rows of features_dev (device). */
int gbsdf_mlp_forward(const float* params_dev, const float* features_dev, int64_t n, float* logits_dev,
                      int32_t device, char* err, size_t errlen);

/* Backward pass of the weighted binary cross-entropy with logits: grad_dev receives the
 * gradient summed over the n rows (deterministic order), loss_dev[0] the summed loss.
 * labels_dev: 0/1 floats; weights_dev: per-row weights or NULL. */
int gbsdf_mlp_backward(const float* params_dev, const float* features_dev, const float* labels_dev,
                       const float* weights_dev, int64_t n, float* grad_dev, float* loss_dev, int32_t device,
                       char* err, size_t errlen);

/* One Adam step on params_dev with moments m_dev, v_dev (all GBSDF_MLP_PARAMS floats on
 * the device); the gradient is multiplied by grad_scale first; step counts from 1. */
int gbsdf_mlp_adam(float* params_dev, const float* grad_dev, float* m_dev, float* v_dev, float lr, float beta1,
                   float beta2, float eps, float grad_scale, int32_t step, int32_t device, char* err, size_t errlen);

/* Mesh wire formats. Each decodes on the GPU of `device` and writes host arrays;
 * vertices are x, y, z floats, indices 3 per triangle.
 *
 * Replaces CudaRasterizer::parse_binary_stl_gpu (cuda_mesh_io.cu:592-722, record decode
 * :524-590): 80-byte header, uint32 triangle count, 50-byte records. Vertices are welded
 * on round(coordinate * 10000) keys in first-occurrence order and triangles whose welded
 * corners repeat are dropped, as the reference's host weld does -- here on the GPU.
 * out_vertices / out_indices must hold 3 x T entries (T from the header); out_normals
 * (3 x T floats, may be NULL) receives every record's normal, normalised with the
 * reference's fallbacks. An empty STL (T = 0) succeeds with no output. */
int gbsdf_parse_binary_stl(const uint8_t* bytes, size_t n_bytes, float* out_vertices, int64_t vertex_capacity,
                           uint32_t* out_indices, int64_t index_capacity, float* out_normals, int64_t* n_vertices,
                           int64_t* n_indices, int32_t device, char* err, size_t errlen);

/* Replaces CudaRasterizer::parse_obj_text_gpu (cuda_mesh_io.cu:962-1090): lines starting
 * "v " (three numbers) and "f " (up to four 1-based or negative indices; quads split
 * (0,1,2) (0,2,3)), at most n_bytes / 10 + 1024 of each in file order, triangles in file
 * order. Capacities of n_bytes / 10 + 1024 vertices and 6 times that many indices always
 * suffice. GBSDF_EINVAL when the text holds no vertex, face or triangle (the reference
 * returns false) or an output is too small (the counts needed are written). */
int gbsdf_parse_obj(const char* text, size_t n_bytes, float* out_vertices, int64_t vertex_capacity,
                    uint32_t* out_indices, int64_t index_capacity, int64_t* n_vertices, int64_t* n_indices,
                    int32_t device, char* err, size_t errlen);

/* Replaces CudaRasterizer::parse_ascii_stl_gpu (cuda_mesh_io.cu:1201-1325, token finder
 * :1094-1118, weld :1146-1186), the decoder StlParser::parse (stl_parser.cpp:43-57) runs
 * when the header's triangle count does not fit the file: "vertex" tokens (at the text
 * start or after a space, tab, CR or LF, followed by a space or tab) in file order, at
 * most gbsdf_ascii_stl_capacity(n_bytes) of them, cut to whole facets; three numbers
 * after each token (the OBJ number rule); corners welded on the reference's 64-bit hash
 * of round(coordinate * 10000) and every corner kept. Vertices are numbered in order of
 * first occurrence with the first corner's coordinates (the reference's numbering follows
 * its threads' timing). out_vertices / out_indices must hold the capacity's count.
 * GBSDF_EINVAL when the text is shorter than 15 bytes or holds no whole facet. */
int gbsdf_ascii_stl_capacity(size_t n_bytes, int64_t* vertex_capacity);
int gbsdf_parse_ascii_stl(const char* text, size_t n_bytes, float* out_vertices, int64_t vertex_capacity,
                          uint32_t* out_indices, int64_t index_capacity, int64_t* n_vertices, int64_t* n_indices,
                          int32_t device, char* err, size_t errlen);

/* Replaces CudaRasterizer::orient_mesh_gpu (cuda_mesh_topology.cu:707-842), the pre-pass
 * the reference's OBJ loader runs after decoding: makes the winding of `indices` (host,
 * 3 per triangle, rewritten in place) consistent across every edge shared by two
 * triangles -- each connected component oriented like its smallest triangle -- and
 * outward (the mesh is inverted when its signed volume is below -1e-5). Reports whether
 * the mesh is orientable, whether any winding was inconsistent, whether it was inverted,
 * and the signed volume (FP64). Runs the label propagation to convergence (the reference
 * stops after 256 steps). */
int gbsdf_orient_mesh(const float* vertices, int64_t n_vertices, uint32_t* indices, int64_t n_indices,
                      int32_t* is_orientable, int32_t* had_inconsistent_winding, int32_t* was_inverted,
                      double* signed_volume, int32_t device, char* err, size_t errlen);

/* Iso-surface of a grid (marching cubes), the consumer of a device-resident SDF.
 * Replaces CudaRasterizer::extract_iso_surface (cuda_marching_cubes.cu:829-951): the
 * reference uploads a host grid; here `grid` may also be a device pointer
 * (grid_on_device = 1, e.g. the output of gbsdf_compute_mesh_sdf) and is read in place,
 * never written. Same rules: boundary voxels read below iso + h read as iso + h; a corner
 * is inside when value - iso <= 0; one vertex per crossing grid edge at the reference's
 * clamped linear interpolation, origin + index * h; triangles outward. Vertices are numbered
 * in voxel order (x, y, z edges of a voxel in turn) and triangles in cube order (the
 * reference's atomic counters give a run-dependent order). The triangle table is generated
 * by one face rule (inside corners on an ambiguous face are cut off separately), which
 * closes the surface for any grid; on ambiguous cubes it may connect the vertices
 * differently from the reference's hand-written table. dims < 2 on any axis: an empty mesh.
 * Outputs on the host, or on the device with outputs_on_device = 1. When an output is too
 * small (capacities 0 to query) GBSDF_EINVAL is returned with *n_vertices / *n_indices set
 * to the counts needed. */
int gbsdf_extract_iso_surface(const float* grid, int32_t grid_on_device, const int32_t dims[3], float voxel_size,
                              const float origin[3], float iso_value, float* out_vertices, int64_t vertex_capacity,
                              uint32_t* out_indices, int64_t index_capacity, int32_t outputs_on_device,
                              int64_t* n_vertices, int64_t* n_indices, int32_t device, char* err, size_t errlen);
/* The same with the mesh left on the device in library-owned buffers (one call, no size
 * query): *vertices_dev / *indices_dev stay valid until the next extraction on `device` or
 * gbsdf_release_workspace(device). */
int gbsdf_extract_iso_surface_device(const float* grid, int32_t grid_on_device, const int32_t dims[3],
                                     float voxel_size, const float origin[3], float iso_value, float** vertices_dev,
                                     uint32_t** indices_dev, int64_t* n_vertices, int64_t* n_indices, int32_t device,
                                     char* err, size_t errlen);
/* Interior volume of an SDF grid: the voxels with value <= 0 times h^3. Replaces
 * CudaRasterizer::compute_sdf_interior_volume_gpu (cuda_viewport_gl.cu:702-741); `grid`
 * (n_voxels floats) on the host (uploaded, as the reference does) or on the device
 * (grid_on_device = 1, read in place). GBSDF_EINVAL for an empty grid (the reference
 * returns false). */
int gbsdf_interior_volume(const float* grid, int32_t grid_on_device, int64_t n_voxels, float voxel_size,
                          float* out_volume_mm3, int64_t* out_inside_voxels, int32_t device, char* err,
                          size_t errlen);
/* Default growth seed inside an SDF grid. Replaces CudaRasterizer::find_default_seed_gpu
 * (cuda_viewport_packers.cu:304-384): the seed starts at (centre x, centre y, min_p.z + 2h)
 * of the box (min_p, max_p); with m the grid minimum (at most 1e30), the voxels with value
 * <= (m < 0 ? max(desired_margin, 0.65 m) : m + h) compete on 10 max(0, z - min_p.z) +
 * 0.5 |xy - centre xy| (ties: the lower index), and the winner's lattice point
 * ((min_coord + i) h) is the seed. Same grid placement as gbsdf_interior_volume. */
int gbsdf_find_default_seed(const float* grid, int32_t grid_on_device, const int32_t dims[3],
                            const int32_t min_coord[3], float voxel_size, const float min_p[3], const float max_p[3],
                            float desired_margin, float out_seed[3], int32_t device, char* err, size_t errlen);
/* The generated triangle table: 256 cases x 16 edge numbers (3 per triangle, -1 ends).
 * Needs no GPU. */
int gbsdf_iso_surface_table(int8_t* out_table);

/* Releases the cached device workspaces of `device` -- the SDF builder's and the
 * iso-surface extractor's (buffers are otherwise reused across calls on the same device). */
void gbsdf_release_workspace(int32_t device);

/* The exact (legacy-kernel) SDF of gbsdf_compute_mesh_sdf with GBSDF_PATH_LEGACY, for
 * callers that cannot allocate device memory: a step running under a device-memory
 * budget fixed at start-up, a plugin whose host application owns all device allocations,
 * or a latency-critical loop that cannot afford cudaMalloc's implicit synchronisation.
 * No counterpart in the reference. It calls no cudaMalloc, cudaFree or allocating library
 * routine: `tris_dev` (n_tris CudaTriangle records) and `out_dev` (dims.x*dims.y*dims.z
 * floats) are caller-owned device buffers, and all scratch lives in one fixed array
 * inside the library (about 12.6 MB per GPU, held from module load until process exit).
 * Limits: at most 16,777,216 voxels, 1,048,576 sign words (ceil(dims.x/32)*dims.y*dims.z)
 * and 1,048,576 triangles; larger inputs return GBSDF_EINVAL before any work.
 * The first call on a device resolves the array's device address (cudaGetSymbolAddress);
 * make that first call before any stream capture. Every call shares the array, so two
 * calls whose GPU work overlapped would race; the entry point takes a process-wide lock
 * and synchronises `stream` (a cudaStream_t, NULL = legacy default stream) before it
 * returns. Unlike the other entry points it builds in place: squared distances are
 * written to `out_dev` before the sign kernels run, so a GBSDF_ECUDA returned after the
 * first launch can leave `out_dev` partly written (argument and limit errors leave it
 * untouched). */
int gbsdf_legacy_sdf_noalloc(const gbsdf_tri* tris_dev, int64_t n_tris, float voxel_size,
                             const int32_t min_coord[3], const int32_t max_coord[3], float* out_dev,
                             int32_t device, void* stream, gbsdf_stats* stats, char* err, size_t errlen);

/* Engine self-tests (no counterpart in the reference). which = 0: the correctly rounded
 * divisions by 3 used by the eikonal update are compared with the IEEE quotient -- the
 * general one for every non-NaN float input, the one for non-negative arguments for every
 * finite non-negative float -- and the packed square root of the paired updates with
 * sqrtf on zero and every float in [2^-100, 2^100]; which = 1: the x sweep's TMA tile layout (32-byte swizzle,
 * out-of-lattice fill) is checked element by element on five boxes of a test grid;
 * which = 2: the branch-free and packed-lane forms of the reference's Godunov update used
 * by the sweeps are compared bit for bit with the reference's branching form on 2^30
 * generated neighbour triples at eight voxel sizes (ties, far sentinels and the 1D / 2D
 * boundary included). *result = number of mismatches (0 expected). */
int gbsdf_selftest(int32_t which, int32_t device, uint64_t* result, char* err, size_t errlen);

/* Library version string. */
const char* gbsdf_version(void);

#ifdef __cplusplus
}
#endif

#endif /* GBSDF_H */
