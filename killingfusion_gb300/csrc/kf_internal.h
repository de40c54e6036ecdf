// Internal declarations shared by the CUDA translation units of the library.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "killingfusion.h"

// ---------------------------------------------------------------------------
// handles
// ---------------------------------------------------------------------------
struct kf_grid_s {
  int n[3];
  int64_t count;
  double voxel;
  double min3d[3];
  double unknown_clip;
  float *phi;      // device, count
  int32_t *w;      // device, count
  float *phi_alt;  // second buffers for out-of-place resampling (lazy)
  int32_t *w_alt;
  float *depth;    // device staging for host depth frames (lazily sized)
  size_t depth_cap;
  void *integ;     // integration scratch: counter, coordinate tables, list
  size_t integ_bytes;
  unsigned *ctr;   // device counter of the warp's moved-voxel list
  void *mc;        // marching-cubes scratch: offsets, per-block totals and masks
  size_t mc_bytes;
};

struct IterStats;
struct FusedGraph;

struct kf_field_s {
  int n[3];
  int64_t count;
  kf_precision prec;
  void *p[3];      // device planes x, y, z (float or double)
  void *q[3];      // second buffer of the Jacobi ping-pong (lazily allocated)
  // solver workspace (lazily allocated, kept until the field is destroyed)
  IterStats *stats;       // device, per iteration
  IterStats *stats_host;  // pinned mirror
  int stats_cap;
  void *plain_scratch;    // intermediate fields of the per-term solver
  size_t plain_bytes;
  FusedGraph *graph;      // captured fused iteration loop
  int *band;              // band-voxel lists (two, of one int per voxel each)
  int2 *runs;             // per run of the dense pass: its entries of the list
  int64_t runs_cap;
  int *rows;              // trust-region step: the first x of each row (y, z)
                          // whose step failed, two arrays of ny*nz
  void *sync;             // barrier state of the persistent band pass
                          // (GridSync, kf_grid_sync.cuh)
  // the last solve launched on this field: its events (start, end, end of
  // the statistics copy), iteration count, solver and whether its statistics
  // are still to be read (kf_psi_solve_wait)
  cudaEvent_t ev[3];
  int last_iterations;
  kf_solver last_solver;
  int pending;
  // What is known of each buffer's contents once the work queued so far has
  // run (the states follow the order calls are made in, which is the order
  // a caller must give the streams they use; KfPsiState).  kf_field_zero
  // makes p zero, and q too once the band-only solver has used the field
  // (q_zero_wanted); a band-only solve that starts from a zero p changes
  // psi only at the voxels of its first list, which it records in
  // `touched`, and leaves both buffers zero elsewhere; warp + fuse then
  // records how many entries of q its moved-voxel list takes
  // (side_recorded).  Every other write makes a buffer unknown
  // (kf_field_written), and nothing is known once kf_field_device has handed
  // the planes out.  With both buffers zero, the band-only solver's first
  // pass reads phi_live alone; zero outside the records, kf_field_zero
  // clears the records alone.
  int p_state, q_state;
  bool q_zero_wanted, exposed, side_recorded;
  int *touched;  // device: the records (KfRecords, kf_field_records)
};

enum KfPsiState { kPsiUnknown = 0, kPsiZero = 1, kPsiRecorded = 2 };

// A call is about to write psi's planes.
inline void kf_field_written(kf_field f) { f->p_state = f->q_state = kPsiUnknown; }
// The records of a field, in one allocation (made on first use; the bitmap
// is cleared on stream s then).
struct KfRecords {
  int *touched;         // count entries: the voxels a band-only solve from zero listed
  unsigned *touched_n;  // how many
  unsigned *side_n;     // the entries of each q plane warp + fuse's moved-voxel list took
  unsigned *moved;      // a bit per voxel (32 a word): warp + fuse's moved voxels,
                        // all clear between its calls
};
int kf_field_records(kf_field f, cudaStream_t s, KfRecords *r);

// ---------------------------------------------------------------------------
// error state
// ---------------------------------------------------------------------------
int kf_fail(int status, const std::string &msg);
int kf_cuda_fail(cudaError_t e, const char *what);

#define KF_CHECK_CUDA(expr)                                    \
  do {                                                         \
    cudaError_t e_ = (expr);                                   \
    if (e_ != cudaSuccess) return kf_cuda_fail(e_, #expr);     \
  } while (0)

#define KF_REQUIRE(cond, msg)                                  \
  do {                                                         \
    if (!(cond)) return kf_fail(KF_ERR_INVALID, (msg));        \
  } while (0)

inline cudaStream_t kf_stream(void *s) { return reinterpret_cast<cudaStream_t>(s); }

// Launch-error check right after a kernel launch.
#define KF_CHECK_LAUNCH(what)                                  \
  do {                                                         \
    cudaError_t e_ = cudaGetLastError();                       \
    if (e_ != cudaSuccess) return kf_cuda_fail(e_, what);      \
  } while (0)

// ---------------------------------------------------------------------------
// device-side parameter block (all thresholds precomputed on the host)
// ---------------------------------------------------------------------------
struct DevParams {
  int nx, ny, nz;
  int64_t count;
  double voxel_size, unknown_clip, max_surface, epsilon, delta_size, alpha, omega_k,
      gamma_k, omega_s, killing_clamp;
  double oob_phi;        // max_surface + epsilon (value outside the grid)
  double band_hi;        // max_surface - epsilon (upper band edge, exclusive)
  float band_hi_f;       // largest float <= band_hi  (s > band_hi <=> s > band_hi_f)
  float band_lo_f;       // smallest float >= -unknown_clip (s < lo <=> s < band_lo_f)
  float mc_hi_f;         // largest float <= max_surface
  float oob_phi_f;       // (float)(max_surface + epsilon)
  float pv_lo_f;         // smallest float >= -(max_surface - epsilon), the lower
                         // band edge of the per-voxel schedule
  int use_data, use_levelset, use_killing;
  int early_exit;
  double threshold;
  int trust;             // the trust-region step applies: use_trust with the
                         // data term alone (KillingFusion.cpp:289)
  int pad_;
};

DevParams kf_make_dev_params(const int n[3], const kf_params *p);
int kf_check_params(const kf_params *p);

// Per-iteration device statistics of a psi solve.
struct IterStats {
  double energy;          // FP64 reduction of the monitored energy
  unsigned int active;    // voxels inside the band
  unsigned int max_delta; // bits of max |dpsi| (non-negative float)
  int diverged;           // psi non-finite inside the band
  int skipped;            // iteration skipped after convergence
  unsigned int list;      // entries of this iteration's band-voxel list
  unsigned int cold;      // band voxels the split dense schedule found in a
                          // run without band voxels at the first iteration
                          // (never expected: such voxels keep psi)
  int timeout;            // record 0: a grid-wide wait of a persistent kernel
                          // gave up (KF_ERR_TIMEOUT)
  int pad_;
};

// The bounds-check build's record of one translation unit (kf_bounds.cuh).
struct KfBoundsRecord {
  unsigned count;  // checks that failed
  int site;        // the first one's site, index and bound
  long long index;
  long long bound;
};
int kf_bounds_tu_read_fused(KfBoundsRecord *r);
int kf_bounds_tu_reset_fused(long long limit);
int kf_bounds_tu_read_batch(KfBoundsRecord *r);
int kf_bounds_tu_reset_batch(long long limit);
int kf_bounds_tu_read_exact(KfBoundsRecord *r);
int kf_bounds_tu_reset_exact(long long limit);
int kf_bounds_tu_read_mc(KfBoundsRecord *r);
int kf_bounds_tu_reset_mc(long long limit);

// Limit of one device-side wait (kf_set_wait_limit), in nanoseconds.
unsigned long long kf_wait_limit_ns();
// Barrier state of the persistent kernels (GridSync, 32 bytes) of a field,
// lazily allocated.
int kf_field_sync(kf_field f, void **out);

// solver entry points implemented in the solver translation units
// p_zero, q_zero: psi's buffers are all zero when the solve starts
// (kf_field_s::p_state, q_state); the band-only solver then sets the
// states it leaves.
int kf_solve_fused(kf_grid live, kf_grid can, kf_field psi, const DevParams &dp,
                   int iterations, IterStats *stats_dev, bool band_only, bool p_zero, bool q_zero,
                   cudaStream_t s);
int kf_solve_plain(kf_grid live, kf_grid can, kf_field psi, const DevParams &dp,
                   int iterations, IterStats *stats_dev, cudaStream_t s);
int kf_solve_exact(kf_grid live, kf_grid can, kf_field psi, const DevParams &dp,
                   int iterations, IterStats *stats_dev, cudaStream_t s);
// Per-voxel schedule (KF_SOLVER_PERVOXEL); stats_dev[0] and [1] as
// documented at kf_psi_solve.
int kf_solve_pervoxel(kf_grid live, kf_grid can, kf_field psi, const DevParams &dp,
                      int max_iters, IterStats *stats_dev, cudaStream_t s);
int kf_gradient_ref_launch(kf_grid live, kf_grid can, kf_field psi, const DevParams &dp,
                           const int32_t *voxels, int count, double *out, uint8_t *active,
                           cudaStream_t s);

// ensure the ping-pong buffer of a field exists
int kf_field_ensure_pair(kf_field f);
// per-iteration statistics buffers of a field (device + pinned host)
int kf_field_stats(kf_field f, int iterations, IterStats **dev);
// two band-voxel lists (one int per voxel of the grid each)
int kf_field_band_list(kf_field f, int **out);
// Row table of the trust-region step: two arrays of ny*nz ints.
int kf_field_trust_rows(kf_field f, int **out);
// "No step failed in this row": larger than any x; also the value of every
// byte, so that one memset initialises a table.
constexpr int kRowClear = 0x7f7f7f7f;
// free the solver workspace of a field (graph, scratch, statistics)
void kf_field_release_solver(kf_field f);
void kf_fused_graph_destroy(FusedGraph *g);
size_t kf_prec_size(kf_precision p);

// Number of SMs of the current device (cached).
int kf_num_sms();

// Asks once per device (`done`: a flag per device) that `func` get
// `percent` % of the largest shared-memory share
// (cudaFuncAttributePreferredSharedMemoryCarveout); a preference only.
//
// The kernels that run beside the band-only solver's persistent kernel (the
// frame's integration and meshes, the zeroing of psi) and the solver itself
// all ask for kBesideSolveCarveout, the largest shared share, which the
// marching-cubes count pass wants for its cp.async rings.  The solve holds
// every SM for its whole length, an SM keeps its L1 / shared split while any
// block is resident, and a kernel that asked for another split than the
// one an SM was in was seen to wait for the solve to end (one mesh or one
// integration per frame took 1.2-1.3 ms instead of 60-90 us).
constexpr int kBesideSolveCarveout = (int)cudaSharedmemCarveoutMaxShared;
inline void kf_prefer_carveout(const void *func, int percent, bool (&done)[64]) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
    cudaGetLastError();
    return;
  }
  if (done[dev]) return;
  if (cudaFuncSetAttribute(func, cudaFuncAttributePreferredSharedMemoryCarveout, percent) != cudaSuccess)
    cudaGetLastError();
  done[dev] = true;
}

// launches implemented in kf_exact.cu (float64 arithmetic without fused
// multiply-add where the reference's rounding decides a discrete outcome)
int kf_grid_ensure_alt(kf_grid g);
// fresh_phi == NULL: integrate into the grid as it is; otherwise the grid is
// taken as reset to (*fresh_phi, 0) and every voxel is written
int kf_launch_integrate_u16(kf_grid g, const uint16_t *depth_dev, double scale, int width, int height,
                            const double w2c[16], const double K[9], double min_depth, double max_depth,
                            const float *fresh_phi, cudaStream_t s);
int kf_launch_integrate(kf_grid g, const float *depth_dev, int width, int height,
                        const double w2c[16], const double K[9], double min_depth,
                        double max_depth, const float *fresh_phi, cudaStream_t s);
int kf_launch_warp(kf_grid g, kf_field psi, const DevParams &dp, cudaStream_t s);
int kf_launch_fuse(kf_grid can, kf_grid other, cudaStream_t s);
int kf_launch_warp_fuse(kf_grid can, kf_grid live, kf_field psi, const DevParams &dp,
                        cudaStream_t s);
int kf_launch_fuse_warped(kf_grid dst, kf_grid other, kf_field psi, const DevParams &dp,
                          cudaStream_t s);
// marching cubes (kf_mc.cu)
int kf_mc_run(kf_grid g, const DevParams &dp, float *verts, int64_t capacity, int64_t *ntri,
              cudaStream_t s, int64_t *ntri_async = nullptr);
