/*
 * kf_oracle.h -- FP64 CPU oracle for the KillingFusion registration loop.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker that the CUDA path is
 * compared against.  It is linked only by tests/, by __graft_entry__.smoke()
 * and by the cpu_baseline / --impl reference legs of bench.py.  The product
 * library (killingfusion_gb300) never calls it.
 *
 * Every function restates, in plain C and in double precision, one method of
 * the reference (saurabheights/KillingFusion) with the same operation order,
 * so that on the same inputs it reproduces the reference bit for bit when
 * both are compiled with -ffp-contract=off.  The pin against the reference's
 * own translation units (compiled against project shims into oracle/_ref) is
 * in tests/test_oracle_ref.py.
 *
 * Layouts (as in the reference):
 *   grid index   idx = z*nx*ny + y*nx + x                  (SDF.cpp:27,189)
 *   phi          double[N], metres, value of voxel i at centre i+0.5
 *   weights      int64[N]                                  (SDF.h:25)
 *   psi          double[N][3] (array of structs), voxel units, at i (DF.cpp:14)
 */
#ifndef KF_ORACLE_H
#define KF_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* The reference's config.h globals that the hot path reads. */
typedef struct orc_params {
  double voxel_size;      /* VoxelSize (config.cpp:4)                    */
  double unknown_clip;    /* UnknownClipDistance (config.cpp:5)          */
  double max_surface;     /* MaxSurfaceVoxelDistance (config.cpp:6)      */
  double epsilon;         /* epsilon (config.cpp:57)                     */
  double delta_size;      /* deltaSize, h (config.cpp:29)                */
  double alpha;           /* alpha (config.cpp:45)                       */
  double omega_k;         /* omegaKilling (config.cpp:48)                */
  double gamma_k;         /* gammaKilling (config.cpp:51)                */
  double omega_s;         /* omegaLevelSet (config.cpp:54)               */
  double threshold;       /* threshold (config.cpp:43)                   */
  double killing_clamp;   /* killingThreshold, DisplacementField.cpp:342 */
  int use_data;           /* EnergyTypeUsed[0] (config.cpp:23)           */
  int use_levelset;       /* EnergyTypeUsed[1]                           */
  int use_killing;        /* EnergyTypeUsed[2]                           */
  int use_trust;          /* UseTrustStrategy (config.cpp:27)            */
} orc_params;

/* ---- samplers (SDF.cpp:475-524, 570-604; DisplacementField.cpp:22-58) ---- */
double orc_phi_at(const double *phi, const int n[3], const orc_params *P,
                  int x, int y, int z);
double orc_phi_sample(const double *phi, const int n[3], const orc_params *P,
                      const double p[3]);
double orc_weight_sample(const int64_t *w, const int n[3], const double p[3]);
void orc_psi_at(const double *psi, const int n[3], int x, int y, int z,
                double out[3]);
void orc_psi_sample(const double *psi, const int n[3], const double p[3],
                    double out[3]);

/* ---- finite differences without psi (SDF.cpp:657-679, 746-795) ---- */
void orc_distance_gradient_at(const double *phi, const int n[3],
                              const orc_params *P, const double p[3],
                              double out[3]);
void orc_distance_hessian_at(const double *phi, const int n[3],
                             const orc_params *P, const double p[3],
                             double out[9]);

/* ---- Jacobian / Killing energy (DisplacementField.cpp:90-193, 274-347) ---- */
void orc_jacobian(const double *psi, const int n[3], const orc_params *P,
                  double x, double y, double z, double out[9]);
double orc_killing_energy(const double *psi, const int n[3],
                          const orc_params *P, double x, double y, double z);
void orc_killing_energy_gradient_fd(const double *psi, const int n[3],
                                    const orc_params *P, int x, int y, int z,
                                    double out[3]);

/* ---- per-voxel energy gradient (KillingFusion.cpp:399-476, SDF.cpp:726-886) ---- */
void orc_distance_gradient(const double *live, const double *psi,
                           const int n[3], const orc_params *P, int x, int y,
                           int z, double out[3]);
void orc_distance_hessian(const double *live, const double *psi,
                          const int n[3], const orc_params *P, int x, int y,
                          int z, double out[9]);
void orc_killing_gradient(const double *psi, const int n[3],
                          const orc_params *P, int x, int y, int z,
                          double out[3]);
void orc_energy_gradient(const double *live, const double *can,
                         const double *psi, const int n[3],
                         const orc_params *P, int x, int y, int z,
                         double out[3]);
/* Warped value getDistance(i, psi) (SDF.cpp:570-575). */
double orc_warped_distance(const double *live, const double *psi,
                           const int n[3], const orc_params *P, int x, int y,
                           int z);
/* Band test of computeDisplacementField (KillingFusion.cpp:272-274). */
int orc_is_active(const double *live, const double *psi, const int n[3],
                  const orc_params *P, int x, int y, int z);

/* ---- psi solve, Jacobi schedule (KillingFusion.cpp:248-352) ----
 * Returns 0, or -1 when psi turned non-finite at an active voxel (the
 * reference's `throw -1`).  active_counts (may be NULL) receives the number of
 * voxels inside the band for each iteration.  nthreads<=0 uses OpenMP's
 * default. */
int orc_solve_pervoxel(const double *live, const double *can, double *psi,
                       const int n[3], const orc_params *P, int max_iters,
                       int colored, int64_t counts[3]);
/* 1 when the trust-region strategy applies: use_trust with the data term
 * alone (KillingFusion.cpp:289). */
int orc_trust_active(const orc_params *P);
int orc_solve_jacobi(const double *live, const double *can, double *psi,
                     const int n[3], const orc_params *P, int iters,
                     int nthreads, int64_t *active_counts);

/* ---- TSDF integration (SDF.cpp:137-197) ----
 * w2c is the row-major world->camera matrix (the reference inverts the C2W
 * pose first), K the row-major 3x3 intrinsics, depth row-major [h][w]. */
void orc_integrate(double *phi, int64_t *w, const int n[3], double voxel,
                   const double min3[3], double unknown_clip,
                   const double *depth, int width, int height,
                   const double w2c[16], const double K[9], double min_depth,
                   double max_depth);

/* 4x4 inverse by Gauss-Jordan elimination with partial pivoting (the
 * algorithm of the project's Eigen stand-in, so that the pose the reference's
 * integrateDepthFrame inverts (SDF.cpp:147) is inverted identically).
 * Row-major; returns 0 on success, -1 if singular. */
int orc_invert4(const double m[16], double out[16]);

/* ---- warp / fuse (SDF.cpp:199-328) ---- */
void orc_update(double *phi, int64_t *w, const double *psi, const int n[3],
                const orc_params *P);
void orc_fuse(double *phi1, int64_t *w1, const double *phi2,
              const int64_t *w2, int64_t count);
void orc_fuse_psi(double *phi1, int64_t *w1, const double *phi2,
                  const int64_t *w2, const double *psi, const int n[3],
                  const orc_params *P);

/* ---- marching cubes (SDF.cpp:330-414, MarchingCubes.h:326-422) ----
 * orc_mc_extract writes 9 doubles per triangle (3 vertices, y already
 * negated as SimpleMesh::AddVertex does) and returns the triangle count; it
 * writes at most `cap` triangles. */
int64_t orc_mc_extract(const double *phi, const int n[3], const orc_params *P,
                       double *verts, int64_t cap);
/* The 256-case tables the mesher uses (edge mask, and up to 5 triangles as
 * edge indices, -1 terminated) -- exported so tests can pin them. */
int orc_mc_edge_mask(int cubeindex);
int orc_mc_tri_row(int cubeindex, int out[16]);

/* ---- project energy and its exact gradient (FP64) ----
 * E = sum over the active set A of
 *   0.5*((phi_w(i) - phi_can(i))/v)^2
 * + omega_s * 0.5*(|grad phi_w(i)|/v - 1)^2
 * + omega_k * (|J_i|_F^2 + gamma * <J_i, J_i^T>)
 * with phi_w(i) = warped live value at i (getDistance(i, psi)),
 * grad phi_w(i)_k = (phi_w(i+e_k) - phi_w(i-e_k))/2 and
 * J_i[:,k] = (psi(i+e_k) - psi(i-e_k))/2, neighbours outside the grid
 * clamped to the edge.  `active` is a byte mask over the grid. */
double orc_project_energy(const double *live, const double *can,
                          const double *psi, const uint8_t *active,
                          const int n[3], const orc_params *P);
double orc_project_energy_local(const double *live, const double *can,
                                const double *psi, const uint8_t *active,
                                const int n[3], const orc_params *P, int x,
                                int y, int z, int radius);
void orc_project_energy_grad(const double *live, const double *can,
                             const double *psi, const uint8_t *active,
                             const int n[3], const orc_params *P,
                             double *grad);

#ifdef __cplusplus
}
#endif
#endif
