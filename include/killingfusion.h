/*
 * killingfusion.h -- C ABI of the GB300 KillingFusion registration loop.
 *
 * A drop-in for the hot path of saurabheights/KillingFusion: the TSDF grid
 * (class SDF), the displacement field psi (class DisplacementField), the
 * gradient-descent psi update (KillingFusion::computeDisplacementField) and
 * the mesher (SDF::getMesh / Polygonise).  The reference has no FFI; its
 * boundary is the C++ class API, and each entry point below names the method
 * it stands in for (file:line in the reference).  The C++ classes with the
 * reference's names and call shapes (killingfusion_gb300/csrc/host/) are
 * written on top of these functions.
 *
 * Conventions
 *  - Every function returns a kf_status; kf_last_error() describes the last
 *    failure of the calling thread.
 *  - Grids are dense, x fastest: idx = z*nx*ny + y*nx + x (SDF.cpp:27).
 *    phi is float32 metres (value of voxel i at its centre i+0.5), weights
 *    int32; psi is three float32 (or float64, see kf_precision) planes in
 *    voxel units, stored at integer positions (DisplacementField.cpp:40-58).
 *  - `stream` is a cudaStream_t (NULL = legacy default stream).  All work is
 *    stream-ordered; functions that return host values synchronise `stream`
 *    (the *_async forms do not).  A grid or field keeps its scratch (meshing,
 *    integration, solver lists and statistics) with it, so calls on the same
 *    handle must not run concurrently on different streams.
 *  - Buffers documented as "host or device" may be either (the copy uses
 *    cudaMemcpyDefault); all others are device pointers.
 */
#ifndef KILLINGFUSION_GB300_H
#define KILLINGFUSION_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define KF_ABI_VERSION 2

typedef enum kf_status {
  KF_OK = 0,
  KF_ERR_INVALID = 1,  /* bad argument: null handle, size mismatch, range   */
  KF_ERR_OOM = 2,      /* device or pinned allocation failed                */
  KF_ERR_CUDA = 3,     /* CUDA runtime error                                */
  KF_ERR_DIVERGED = 4, /* psi non-finite at a voxel in the band; the
                          reference throws -1 (KillingFusion.cpp:328-332)   */
  KF_ERR_TIMEOUT = 5,  /* a bounded device-side wait gave up (the grid-wide
                          barrier of a persistent kernel, kf_set_wait_limit) */
  KF_ERR_CAPACITY = 6, /* caller buffer too small (count is still returned) */
  KF_ERR_INTERNAL = 7  /* a consistency check of the library failed         */
} kf_status;

/* Arithmetic of the psi solve. */
typedef enum kf_precision {
  KF_F32 = 0, /* float32 fields and arithmetic (production)                */
  KF_F64 = 1  /* float64 psi and arithmetic, no fused multiply-add, in the
                 reference's operation order: reproduces the reference's
                 FP64 result bit for bit given the same float32 SDFs        */
} kf_precision;

/* Form of the psi update kernel(s). */
typedef enum kf_solver {
  KF_SOLVER_FUSED = 0, /* one stencil pass per iteration, CUDA-graph loop  */
  KF_SOLVER_PLAIN = 1, /* one kernel per energy term, fields through HBM   */
  KF_SOLVER_EXACT = 2, /* float64 replay of the reference (needs KF_F64 psi) */
  KF_SOLVER_BAND = 3,  /* the fused stencil on the band only: a voxel outside
                          the band keeps psi, so its band test keeps failing
                          and the band can only shrink; after the first dense
                          pass each iteration visits the previous iteration's
                          band.  Same psi as KF_SOLVER_FUSED.               */
  KF_SOLVER_PERVOXEL = 4 /* the reference's default schedule
                          (KillingFusion.cpp:353-396): every voxel inside the
                          symmetric band steps psi in place until its step or
                          gradient is at most params.threshold or `iterations`
                          steps were taken, its neighbours fixed meanwhile.
                          Voxels go in 8 colours (parity of x, y, z) instead
                          of the reference's z, y, x order, so the result is
                          deterministic but not the reference's bit for bit
                          (nor is the reference's with more than one OpenMP
                          thread).                                          */
} kf_solver;

/* The reference's config.h globals that the hot path reads. */
typedef struct kf_params {
  double voxel_size;    /* VoxelSize (config.cpp:4)                        */
  double unknown_clip;  /* UnknownClipDistance (config.cpp:5)              */
  double max_surface;   /* MaxSurfaceVoxelDistance (config.cpp:6)          */
  double epsilon;       /* epsilon (config.cpp:57)                         */
  double delta_size;    /* deltaSize h, voxel units (config.cpp:29)        */
  double alpha;         /* gradient step (config.cpp:45)                   */
  double omega_k;       /* Killing weight (config.cpp:48)                  */
  double gamma_k;       /* Killing rigidity gamma (config.cpp:51)          */
  double omega_s;       /* level-set weight (config.cpp:54)                */
  double threshold;     /* convergence threshold on max |dpsi| (config.cpp:43),
                           used only when early_exit is set                */
  double killing_clamp; /* |g| clamp, DisplacementField.cpp:342 (0.1)     */
  int use_data;         /* EnergyTypeUsed[0..2] (config.cpp:23)            */
  int use_levelset;
  int use_killing;
  int early_exit;       /* 0: run every requested iteration, as the
                           reference's Jacobi schedule does; 1: stop once
                           max |dpsi| <= threshold, the criterion of its
                           per-voxel schedule (KillingFusion.cpp:381)      */
  int use_trust;        /* UseTrustStrategy (config.cpp:27): the trust-region
                           step of the Jacobi schedule (KillingFusion.cpp:
                           288-314), taken only with the data term alone
                           (use_data set, use_levelset and use_killing
                           clear), as the reference takes it.  Run by
                           KF_SOLVER_FUSED, _BAND and _EXACT; _PLAIN and
                           kf_batch_create reject it; _PERVOXEL ignores it,
                           as the reference's per-voxel schedule does.    */
} kf_params;

typedef struct kf_solve_stats {
  int32_t iterations_run; /* iterations executed                           */
  int32_t converged;      /* 1 if max |dpsi| fell to params.threshold      */
  int32_t diverged;       /* 1 if psi turned non-finite inside the band    */
  int32_t capped;         /* KF_SOLVER_PERVOXEL: voxels that hit the cap   */
  int64_t active_first;   /* voxels inside the band, first iteration       */
  int64_t active_last;    /* ... last executed iteration                   */
  double energy_first;    /* monitored energy (FP64 reduction)             */
  double energy_last;
  double max_delta_last;  /* max |dpsi| of the last executed iteration     */
  double device_ms;       /* device time of the solve                      */
} kf_solve_stats;

typedef struct kf_grid_s *kf_grid;   /* an SDF: phi + weights on a grid     */
typedef struct kf_field_s *kf_field; /* a displacement field psi           */
typedef struct kf_fusion_s *kf_fusion; /* the per-frame pipeline           */

/* ---- library -------------------------------------------------------- */
int kf_version(void);
const char *kf_last_error(void);
/* The reference's compiled-in values (config.cpp:4-57). */
void kf_params_reference(kf_params *p);
/* Paper weights (alpha 0.1, omega_k 0.5, gamma 0.1, omega_s 0.2) with the
 * truncation band set to trunc_voxels voxels (config.cpp:32-41 comment). */
void kf_params_paper(kf_params *p, double voxel_size, double trunc_voxels);
/* Limit, in seconds, of one device-side wait: the grid-wide barrier between
 * the iterations of the persistent kernels (KF_SOLVER_BAND and the batched
 * solver run every iteration in one cooperative launch).  A wait that lasts
 * longer gives up, the kernel ends and the call returns KF_ERR_TIMEOUT, with
 * psi undefined.  No counterpart in the reference, which runs on the CPU.
 * Default 1 s, process-wide; 0 makes every wait give up at once (for testing
 * the error path).  Returns the previous limit, or -1 for a value outside
 * [0, 60] (ignored). */
double kf_set_wait_limit(double seconds);
/* Bounds-check build (the library compiled with -DKF_BOUNDS_CHECK,
 * libkillingfusion_bc.so): the kernels of the hot path check every index
 * they take from data (band lists and their append positions, the dense
 * passes' queues and run tables, the in-place write-back, side lists, the
 * marching-cubes block list) and skip an access outside its bound instead
 * of making it.  kf_bounds_status reports whether this build checks
 * (enabled), how many checks failed since the last kf_bounds_reset, and the
 * first failure's site (KfBoundsSite in kf_bounds.cuh), index and bound; the
 * normal build reports enabled = 0 and no failures.  kf_bounds_reset clears
 * the records; a positive limit also lowers every bound to `limit` (the
 * checked build only), so that a test can make the checks fire on a small
 * grid while every access stays inside its buffer.  No counterpart in the
 * reference, which has no sanitizer mode. */
int kf_bounds_status(int *enabled, int64_t *violations, int *site, int64_t *index, int64_t *bound);
int kf_bounds_reset(int64_t limit);
/* Introspection of the marching-cubes table (MarchingCubes.h:26-318): edge
 * mask of a cube configuration and its triangle list (edge ids, -1 padded). */
int kf_mc_case(int cubeindex, int *edge_mask, int tri_edges[16]);

/* ---- SDF grid (SDF.h:16-200) ------------------------------------------ */
/* SDF::SDF(voxelSize, min, max, unknownClip) with the grid size given
 * directly (SDF.cpp:14-30, 117-135); phi = max_surface+epsilon, w = 0. */
int kf_grid_create(const int dims[3], double voxel_size, const double min3d[3],
                   double unknown_clip, const kf_params *p, kf_grid *out);
int kf_grid_destroy(kf_grid g);
int kf_grid_info(kf_grid g, int dims[3], double *voxel_size, double min3d[3],
                 double *unknown_clip);
/* Refill with phi = max_surface+epsilon, w = 0 (SDF.cpp:126-135). */
int kf_grid_reset(kf_grid g, const kf_params *p, void *stream);
/* Copy N phi values / weights in or out (host or device; NULL skips). */
int kf_grid_upload(kf_grid g, const float *phi, const int32_t *weight, void *stream);
int kf_grid_download(kf_grid g, float *phi, int32_t *weight, void *stream);
/* Raw device pointers (owned by the grid). */
int kf_grid_device(kf_grid g, float **phi, int32_t **weight);

/* ---- displacement field (DisplacementField.h:9-66) -------------------- */
/* DisplacementField(gridSize, voxelSize): zero-initialised
 * (DisplacementField.cpp:8-16). */
int kf_field_create(const int dims[3], kf_precision prec, kf_field *out);
int kf_field_destroy(kf_field f);
int kf_field_zero(kf_field f, void *stream);
/* Copy psi in or out as [N][3] (array of structs, the reference's layout),
 * float for KF_F32 fields and double for KF_F64 (host or device). */
int kf_field_upload(kf_field f, const void *xyz, void *stream);
int kf_field_download(kf_field f, void *xyz, void *stream);
/* Raw device planes (valid until the next solve, which may exchange them
 * with its second buffer).  From then on the library no longer relies on
 * knowing where psi is zero (after kf_field_zero, the band-only solver
 * otherwise tests the band on phi_live alone and zeroes only the voxels it
 * changed). */
int kf_field_device(kf_field f, void **px, void **py, void **pz);

/* psi += other (DisplacementField::operator+, DisplacementField.cpp:73-80). */
int kf_field_add(kf_field f, kf_field other, void *stream);
/* psi = v everywhere (DisplacementField::initializeAllVoxels,
 * DisplacementField.cpp:82-88). */
int kf_field_fill(kf_field f, const double v[3], void *stream);
/* psi at n voxels (host int32 xyz triples) into host double[n][3]
 * (DisplacementField::getDisplacementAt, DisplacementField.cpp:22-38: a
 * linear index outside the grid reads 0). */
int kf_field_get_voxels(kf_field f, const int32_t *xyz, int n, double *out, void *stream);
/* psi(i) += delta at n voxels (DisplacementField::update,
 * DisplacementField.cpp:65-71); KF_ERR_INVALID for an index outside the
 * grid (the reference's vector::at throws). */
int kf_field_add_voxels(kf_field f, const int32_t *xyz, int n, const double *delta, void *stream);
/* Trilinear samples of psi at n grid points (host double[n][3]) into host
 * double[n][3] (DisplacementField::getDisplacementAtf, :40-58). */
int kf_field_sample(kf_field f, const double *pts, int n, double *out, void *stream);

/* Trilinear samples of phi and of the weights at n grid points (host
 * double[n][3], grid units with the reference's half-voxel convention) into
 * host double[n] (SDF::getDistance / SDF::getWeight, SDF.cpp:503-604;
 * either output may be NULL). */
int kf_grid_sample(kf_grid g, const kf_params *p, const double *pts, int n, double *phi,
                   double *weight, void *stream);
/* phi and weight at n voxels (host int32 xyz) into host arrays
 * (SDF::getDistanceAtIndex / getWeightAtIndex, SDF.cpp:475-501: outside the
 * grid phi = max_surface+epsilon, w = 0). */
int kf_grid_get_voxels(kf_grid g, const kf_params *p, const int32_t *xyz, int n, double *phi,
                       int64_t *weight, void *stream);

/* ---- hot path --------------------------------------------------------- */
/* SDF::integrateDepthFrame (SDF.cpp:137-197).  depth: float32 metres,
 * row-major [height][width] (host or device); c2w: row-major camera->world
 * pose; K: row-major intrinsics. */
int kf_integrate_depth(kf_grid g, const float *depth, int width, int height,
                       const double c2w[16], const double K[9], double min_depth,
                       double max_depth, void *stream);
/* The same with 16-bit depth (the reference's PNG frames, millimetres for
 * the Kinect datasets): each value becomes (double)v * scale, as
 * cv::Mat::convertTo(CV_64FC1, 1.0 / 1000) produces it in the reference
 * (DatasetReader.cpp:131-132), so integration matches the reference's
 * double depth exactly.  Masked-out pixels are 0 (below any minimum depth). */
int kf_integrate_depth_u16(kf_grid g, const uint16_t *depth, int width, int height, double scale,
                           const double c2w[16], const double K[9], double min_depth,
                           double max_depth, void *stream);
/* KillingFusion::computeSDF (KillingFusion.cpp:209-230): a new SDF of one
 * frame, i.e. kf_grid_reset (phi = max_surface + epsilon, w = 0) followed by
 * kf_integrate_depth, with the same result, in one pass that writes every
 * voxel once instead of a fill and an integration that reads the grid back. */
int kf_compute_sdf(kf_grid g, const kf_params *p, const float *depth, int width, int height,
                   const double c2w[16], const double K[9], double min_depth, double max_depth,
                   void *stream);
/* The same on 16-bit depth (kf_grid_reset + kf_integrate_depth_u16). */
int kf_compute_sdf_u16(kf_grid g, const kf_params *p, const uint16_t *depth, int width, int height,
                       double scale, const double c2w[16], const double K[9], double min_depth,
                       double max_depth, void *stream);

/* KillingFusion::computeDisplacementField, Jacobi schedule
 * (KillingFusion.cpp:240-352): `iterations` gradient-descent steps of psi
 * registering `live` onto `canonical`.  Returns KF_ERR_DIVERGED when psi
 * turned non-finite inside the band.  stats may be NULL.  With
 * KF_SOLVER_PERVOXEL `iterations` caps each voxel's steps and the statistics
 * read: iterations_run = most steps a voxel took, converged = no voxel hit
 * the cap, active_first = active_last = voxels visited, energy_last = their
 * monitored energy at their last step, max_delta_last = largest last step. */
int kf_psi_solve(kf_grid live, kf_grid canonical, kf_field psi, const kf_params *p,
                 int iterations, kf_solver solver, kf_solve_stats *stats, void *stream);

/* kf_psi_solve without waiting (no counterpart in the reference, whose
 * solve returns when done): queues the solve on `stream` and returns, so
 * that a frame's later work (meshes, warp + fuse) queues behind it without
 * the host waiting in between.  psi's planes hold the result for everything
 * queued after this call.  kf_psi_solve_wait then waits for the solve and
 * returns its statistics and status (KF_ERR_DIVERGED as kf_psi_solve).
 * With params.early_exit only KF_SOLVER_FUSED and _PERVOXEL are accepted
 * (the others alternate two buffers, and which holds psi would depend on the
 * iterations run).  Only the last solve queued on a field can be waited on. */
int kf_psi_solve_async(kf_grid live, kf_grid canonical, kf_field psi, const kf_params *p,
                       int iterations, kf_solver solver, void *stream);
int kf_psi_solve_wait(kf_field psi, kf_solve_stats *stats);

/* Per-iteration statistics of the last solve on psi, once it has been waited
 * for (no counterpart in the reference, which prints only timings): for
 * each executed iteration k < max_iterations, the monitored energy (FP64
 * sum), max |dpsi| and the number of band voxels, into the arrays given
 * (any may be NULL); *count receives the number of iterations written.
 * KF_ERR_INVALID for the per-voxel schedule, which keeps none. */
int kf_psi_solve_history(kf_field psi, int32_t max_iterations, double *energy, double *max_delta,
                         int64_t *active, int32_t *count);

/* KillingFusion::computeEnergyGradient (KillingFusion.cpp:399-442) at
 * `count` voxels (device int32 xyz triples), in the field's precision;
 * out: device double[count][3].  Also the band test (KillingFusion.cpp:272)
 * into active (device uint8[count], may be NULL). */
int kf_psi_gradient_ref(kf_grid live, kf_grid canonical, kf_field psi,
                        const kf_params *p, const int32_t *voxels, int count,
                        double *out, uint8_t *active, void *stream);

/* ---- project energy and its adjoint ----------------------------------- */
/* No counterpart in the reference, whose solver descends the Euler-Lagrange
 * gradients of KillingFusion::computeEnergyGradient (KillingFusion.cpp:399-476)
 * without ever evaluating an energy.  This is a discrete energy with the same
 * three terms, differentiable exactly:
 *   E = sum over active i of 1/2((phi_w(i) - phi_can(i))/v)^2
 *       + omega_s 1/2(sqrt(g.g + (v eps)^2)/v - 1)^2
 *       + omega_k(|J|^2 + gamma <J, J^T>)
 * with phi_w(j) = live sampled at j + psi(j) (grid units), g and J clamped
 * central differences of phi_w and psi.  active: device uint8[N] mask, NULL =
 * every voxel. */
/* Energy terms {data, level set, Killing} of the active voxels inside box
 * (x0, y0, z0, x1, y1, z1, half-open; NULL = whole grid), evaluated in
 * `arith` precision and summed in float64 in a fixed order (deterministic);
 * terms is a host double[3]; the call waits for the result. */
int kf_energy(kf_grid live, kf_grid canonical, kf_field psi, const kf_params *p,
              const uint8_t *active, const int box[6], kf_precision arith, double terms[3],
              void *stream);
/* dE/dpsi, float64, into device double[N][3] (deterministic gather). */
int kf_energy_adjoint(kf_grid live, kf_grid canonical, kf_field psi, const kf_params *p,
                      const uint8_t *active, double *grad, void *stream);
/* Float64 central differences (E(psi + h e) - E(psi - h e)) / 2h for each of
 * `count` voxels (device int32 xyz) and each psi component, into device
 * double[count][3]; only the 3x3x3 window whose energy depends on psi(j) is
 * evaluated. */
int kf_energy_fd(kf_grid live, kf_grid canonical, kf_field psi, const kf_params *p,
                 const uint8_t *active, const int32_t *voxels, int count, double h, double *out,
                 void *stream);

/* SDF::update(psi) (SDF.cpp:300-328): resample g at i+0.5+psi(i), weights
 * truncated to integers. */
int kf_warp(kf_grid g, kf_field psi, const kf_params *p, void *stream);
/* SDF::fuse(other) with FUSE_BY_MERGE (SDF.cpp:199-241). */
int kf_fuse(kf_grid canonical, kf_grid other, void *stream);
/* SDF::update(psi) on `live` followed by canonical->fuse(live)
 * (KillingFusion.cpp:158-159) in one pass; live is left warped. */
int kf_warp_fuse(kf_grid canonical, kf_grid live, kf_field psi, const kf_params *p,
                 void *stream);
/* SDF::fuse(other, psi) (SDF.cpp:244-297). */
int kf_fuse_warped(kf_grid dst, kf_grid other, kf_field psi, const kf_params *p,
                   void *stream);

/* SDF::getMesh (SDF.cpp:396-414) + Polygonise (MarchingCubes.h:366-422):
 * triangle soup in the reference's order (cells z, y, x; triangles in table
 * order), 9 floats per triangle (3 vertices, y negated as
 * SimpleMesh::AddVertex does).  *ntri receives the count; verts (device, may
 * be NULL) receives min(count, capacity) triangles; KF_ERR_CAPACITY when
 * capacity < count. */
int kf_marching_cubes(kf_grid g, const kf_params *p, float *verts, int64_t capacity,
                      int64_t *ntri, void *stream);

/* kf_marching_cubes without waiting: queues the count, the scan and the
 * emit pass and returns.  The triangle count is written to *ntri on the
 * stream (device, pinned host or managed memory; read it after the stream
 * has passed this call); verts receives the first min(count, capacity)
 * triangles, and a count above capacity is the caller's to check. */
int kf_marching_cubes_async(kf_grid g, const kf_params *p, float *verts, int64_t capacity,
                            int64_t *ntri, void *stream);

/* kf_marching_cubes into host memory (SDF::getMesh for callers without a
 * CUDA runtime of their own): verts is a host buffer of `capacity`
 * triangles (may be NULL to count). */
int kf_mesh_host(kf_grid g, const kf_params *p, float *verts, int64_t capacity, int64_t *ntri,
                 void *stream);

/* ---- batched solves ---------------------------------------------------- */
/* Many independent registration problems -- each a live SDF, a canonical SDF
 * and psi of its own size and parameters -- advanced together (no
 * counterpart in the reference, which registers one frame at a time): one
 * dense first pass over every problem, then every band pass of every
 * iteration in one persistent cooperative launch, the iterations separated
 * by a grid-wide barrier with a bounded wait (kf_set_wait_limit).  Each
 * problem gets the Jacobi schedule of kf_psi_solve with KF_SOLVER_BAND and
 * the same psi bit for bit; with params.early_exit a problem stops on its
 * own once an iteration moved psi by at most params.threshold (the criterion
 * of KillingFusion.cpp:381, 392), while the others go on.  Fields must be
 * KF_F32 and distinct; at most 256 problems.  The batch keeps the handles:
 * keep them alive until kf_batch_destroy. */
typedef struct kf_batch_s *kf_batch;
typedef struct kf_batch_item {
  kf_grid live;
  kf_grid canonical;
  kf_field psi;
  kf_params params;
} kf_batch_item;

/* Launch shape of a batch.  The band work of an iteration is cut into chunks
 * of band_chunk voxels that never cross a problem; a CTA of band_threads
 * threads takes one chunk at a time (band_chunk / band_threads voxels per
 * thread), band_blocks_per_sm CTAs per SM with at most band_registers
 * registers per thread.  The dense first pass takes tiles of 32 x 8 columns
 * and `slab` z-planes.  The times are those the autotuner measured for the
 * chosen shape (0 when the shape was set by kf_batch_set_shape). */
typedef struct kf_batch_shape {
  int band_threads;       /* 256 or 512                                       */
  int band_chunk;         /* band_threads or 2 * band_threads                 */
  int band_blocks_per_sm; /* 1, 2 or 3 (as the register budget allows)        */
  int band_registers;     /* 128, or 80 for 3 CTAs of 256 threads per SM      */
  int slab;               /* 4, 8 or 16                                       */
  int reserved;
  double band_ms;         /* one band pass (the first iteration)              */
  double stream_ms;       /* the dense first pass                             */
} kf_batch_shape;

int kf_batch_create(const kf_batch_item *items, int count, int iterations, kf_batch *out);
int kf_batch_destroy(kf_batch b);
/* Times, on this batch's data, the dense first pass at each slab depth and
 * the band pass of the first iteration at each band shape (CTA size x chunk
 * size x resident CTAs), and keeps the fastest of each for kf_batch_run
 * (psi is not changed).  shape (may be NULL) receives the choice. */
int kf_batch_autotune(kf_batch b, kf_batch_shape *shape, void *stream);
/* Sets the launch shape (one of the shapes the autotuner tries); the
 * default before any autotuning is 256 threads, chunks of 256, 2 CTAs per SM,
 * slabs of 8.  KF_ERR_INVALID for a shape outside that set. */
int kf_batch_set_shape(kf_batch b, const kf_batch_shape *shape);
/* Runs the batch's iterations on every problem from its current psi.  stats:
 * one record per problem (may be NULL).  KF_ERR_DIVERGED when any problem
 * diverged (its record says which); the others are still solved.
 * KF_ERR_TIMEOUT when a barrier wait gave up (psi undefined). */
int kf_batch_run(kf_batch b, kf_solve_stats *stats, void *stream);

/* ---- per-frame pipeline (KillingFusion::processNextFrame) -------------- */

/* Meshes a frame can return (bit mask). */
enum { KF_MESH_LIVE = 1, KF_MESH_REGISTERED = 2, KF_MESH_CANONICAL = 4 };

typedef struct kf_fusion_config {
  int dims[3];          /* grid size of the canonical and live SDFs          */
  double voxel_size;    /* SDF voxel size (m)                                */
  double min3d[3];      /* world position of the grid's min corner (m)       */
  double K[9];          /* depth intrinsics, row-major                       */
  int width, height;    /* depth frame size                                  */
  double min_depth;     /* valid depth range (DatasetReader thresholds)      */
  double max_depth;
  kf_params params;     /* solver parameters                                 */
  int iterations;       /* psi iterations per frame (KILLING_MAX_ITERATIONS) */
  kf_solver solver;     /* KF_SOLVER_FUSED, _BAND, _PLAIN, _EXACT, _PERVOXEL */
} kf_fusion_config;

typedef struct kf_frame_result {
  int32_t frame;              /* frames processed so far, this one included  */
  int32_t reserved;
  kf_solve_stats solve;       /* zero for the first frame                    */
  int64_t ntri[3];            /* live, registered, canonical triangle counts */
  const float *mesh[3];       /* host (pinned) triangle soups, 9 floats per
                                 triangle, valid until the next call; NULL
                                 when not requested                          */
  double device_ms;           /* device time of the whole frame              */
} kf_frame_result;

/* The state of KillingFusion (KillingFusion.h:13-100): canonical SDF, the
 * live frame's SDF and psi, on the device. */
int kf_fusion_create(const kf_fusion_config *cfg, kf_fusion *out);
int kf_fusion_destroy(kf_fusion f);
/* KillingFusion::processNextFrame (KillingFusion.cpp:109-175).  The first
 * frame becomes the canonical SDF; every later frame is integrated into a
 * fresh live SDF, registered onto the canonical SDF from a zero psi
 * (UseZeroDisplacementFieldForNextFrame), meshed, warped by psi and fused.
 * depth: float32 metres (host or device); c2w may be NULL (identity, as
 * KillingFusion::computeSDF uses).  meshes: KF_MESH_* bits. */
int kf_fusion_process_frame(kf_fusion f, const float *depth, const double c2w[16], int meshes,
                            kf_frame_result *res, void *stream);
/* Handles of the pipeline's state (owned by the pipeline). */
int kf_fusion_state(kf_fusion f, kf_grid *canonical, kf_grid *live, kf_field *psi);
/* Checkpoint and resume of the pipeline: its canonical SDF, psi and frame
 * count go to a state file (kf_state_save); a pipeline created with the same
 * configuration and loaded from that file continues the sequence with the
 * same results, bit for bit, as the pipeline that wrote it.  No counterpart
 * in the reference, whose dumps (SDF.cpp:432-446, DisplacementField.cpp:
 * 349-366) keep no weights and have no reader. */
int kf_fusion_save(kf_fusion f, const char *path, void *stream);
int kf_fusion_load(kf_fusion f, const char *path, void *stream);

/* ---- files ------------------------------------------------------------ */
/* State file (version 2) of a registration sequence: the canonical SDF's
 * float32 values and int32 weights, psi if given (float32 or float64 planes)
 * and a frame counter, with the grid's dims, placement, voxel size and
 * unknown-clip distance in the header.  No counterpart in the reference. */
int kf_state_save(const char *path, kf_grid canonical, kf_field psi, int32_t frame, void *stream);
/* Header of a state file; psi_precision receives KF_F32, KF_F64 or -1 (no
 * psi).  Any output may be NULL. */
int kf_state_info(const char *path, int dims[3], double *voxel, double min3d[3], double *unknown_clip,
                  int32_t *frame, int *psi_precision);
/* Reads a state file into existing handles of the file's size, placement
 * and psi precision (psi may be NULL to skip it); KF_ERR_INVALID when they
 * differ or the file is not a state file. */
int kf_state_load(const char *path, kf_grid canonical, kf_field psi, int32_t *frame, void *stream);
/* A grid from the reference's SDF dump (SDF::dumpToBinFile, SDF.cpp:432-446:
 * int32 dims[3], double min[3], double voxel, double truncation, double
 * phi[N]).  Values are stored as float32.  The file keeps no weights: a
 * voxel whose value is not the initial MaxSurfaceVoxelDistance + epsilon of
 * params gets weight 1, the others 0.  truncation (may be NULL) receives the
 * file's truncation distance in voxels. */
int kf_grid_load_ref_bin(const char *path, const kf_params *params, double unknown_clip, kf_grid *out,
                         double *truncation, void *stream);

/* Marching cubes that allocates nothing.  No counterpart in the reference:
 * it exists for callers that cannot allocate device memory on their own --
 * a frame loop where a cudaMalloc/cudaFree would block on the device and
 * break the frame budget, or a host whose device memory is handed out by
 * another allocator (a framework's caching pool, a fixed arena reserved at
 * start-up).  Same output as kf_marching_cubes, but it takes the SDF as a
 * plain device array (phi, float32, dims[0]*dims[1]*dims[2] values, x
 * fastest) and keeps its scratch in a fixed device array inside the library
 * (786,440 bytes: a triangle count per block of 2048 cells and the blocks'
 * 64-bit offsets for up to KF_MC_NOALLOC_MAX_CELLS cells; held on every GPU
 * that loads the library until the process exits); it calls no cudaMalloc,
 * cudaFree or allocating library routine.  Grids above
 * KF_MC_NOALLOC_MAX_CELLS cells are rejected with KF_ERR_INVALID.  The
 * first call on a device looks up the array's address on that device (make
 * that first call outside any CUDA stream capture).  The call returns the
 * triangle count, so it waits on `stream` until the count is known (copied
 * into a host variable of the call); the emit pass runs over every block of
 * cells, not only those with triangles.  All calls share the one array:
 * calls that overlap on the GPU (from two streams or two host threads at
 * once) race and must be serialised. */
#define KF_MC_NOALLOC_MAX_CELLS (512LL * 512LL * 512LL)
int kf_marching_cubes_noalloc(const float *phi, const int dims[3], const kf_params *p,
                              float *verts, int64_t capacity, int64_t *ntri, void *stream);

#ifdef __cplusplus
}
#endif
#endif
