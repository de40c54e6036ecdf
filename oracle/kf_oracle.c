/*
 * kf_oracle.c -- FP64 CPU restatement of the KillingFusion registration loop.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the CUDA path (see kf_oracle.h).
 *
 * Each function names the reference method it restates (file:line within
 * saurabheights/KillingFusion).  The arithmetic is written in the same order
 * as the reference evaluates it, so that with -ffp-contract=off the results
 * agree bit for bit with the reference's own code built against the project
 * shims (oracle/ref/).  Build: oracle/Makefile.
 */
#include "kf_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------------ */
/* helpers                                                                  */
/* ------------------------------------------------------------------------ */

static inline int64_t lin(const int n[3], int x, int y, int z) {
  return (int64_t)z * n[0] * n[1] + (int64_t)y * n[0] + x;
}

static inline int in_grid(const int n[3], int x, int y, int z) {
  return x >= 0 && x < n[0] && y >= 0 && y < n[1] && z >= 0 && z < n[2];
}

/* utils.h:6-25 -- lerp order x, then y, then z. */
static inline double lerp1(double a, double b, double t) {
  return a * (1 - t) + b * t;
}
static inline double lerp2(double v00, double v01, double v10, double v11,
                           double x, double y) {
  double s = lerp1(v00, v01, x);
  double t = lerp1(v10, v11, x);
  return lerp1(s, t, y);
}
static inline double lerp3(const double v[8], double x, double y, double z) {
  /* v[] ordered (dx,dy,dz) = 000,100,010,110,001,101,011,111, i.e. the
   * reference's vertex_000, vertex_001, vertex_010, vertex_011, vertex_100 ... */
  double s = lerp2(v[0], v[1], v[2], v[3], x, y);
  double t = lerp2(v[4], v[5], v[6], v[7], x, y);
  return lerp1(s, t, z);
}

static const int kCorner[8][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {1, 1, 0},
                                  {0, 0, 1}, {1, 0, 1}, {0, 1, 1}, {1, 1, 1}};

/* ------------------------------------------------------------------------ */
/* samplers                                                                 */
/* ------------------------------------------------------------------------ */

/* SDF::getDistanceAtIndex (SDF.cpp:475-487): outside the grid reads
 * MaxSurfaceVoxelDistance + epsilon. */
double orc_phi_at(const double *phi, const int n[3], const orc_params *P,
                  int x, int y, int z) {
  if (!in_grid(n, x, y, z)) return P->max_surface + P->epsilon;
  return phi[lin(n, x, y, z)];
}

static inline double w_at(const int64_t *w, const int n[3], int x, int y,
                          int z) {
  if (!in_grid(n, x, y, z)) return 0;
  return (double)w[lin(n, x, y, z)];
}

/* SDF::getDistance(gridLocation) (SDF.cpp:503-524): sample at p-0.5, base
 * index by truncation toward zero (Eigen cast<int>). */
double orc_phi_sample(const double *phi, const int n[3], const orc_params *P,
                      const double p[3]) {
  double t0 = p[0] - 0.5, t1 = p[1] - 0.5, t2 = p[2] - 0.5;
  int b0 = (int)t0, b1 = (int)t1, b2 = (int)t2;
  double v[8];
  for (int c = 0; c < 8; ++c)
    v[c] = orc_phi_at(phi, n, P, b0 + kCorner[c][0], b1 + kCorner[c][1],
                      b2 + kCorner[c][2]);
  return lerp3(v, t0 - (double)b0, t1 - (double)b1, t2 - (double)b2);
}

/* SDF::getWeight(gridLocation) (SDF.cpp:584-604). */
double orc_weight_sample(const int64_t *w, const int n[3], const double p[3]) {
  double t0 = p[0] - 0.5, t1 = p[1] - 0.5, t2 = p[2] - 0.5;
  int b0 = (int)t0, b1 = (int)t1, b2 = (int)t2;
  double v[8];
  for (int c = 0; c < 8; ++c)
    v[c] = w_at(w, n, b0 + kCorner[c][0], b1 + kCorner[c][1],
                b2 + kCorner[c][2]);
  return lerp3(v, t0 - (double)b0, t1 - (double)b1, t2 - (double)b2);
}

/* DisplacementField::getDisplacementAt (DisplacementField.cpp:22-38): only
 * the linear index is range-checked, so x/y overflow wraps into the next
 * row/plane. */
void orc_psi_at(const double *psi, const int n[3], int x, int y, int z,
                double out[3]) {
  int index = z * (n[0] * n[1]) + y * n[0] + x;
  int total = n[0] * n[1] * n[2];
  if (index < 0 || index >= total) {
    out[0] = out[1] = out[2] = 0.0;
    return;
  }
  out[0] = psi[3 * (int64_t)index + 0];
  out[1] = psi[3 * (int64_t)index + 1];
  out[2] = psi[3 * (int64_t)index + 2];
}

/* DisplacementField::getDisplacementAtf (DisplacementField.cpp:40-58): no
 * half-voxel shift. */
void orc_psi_sample(const double *psi, const int n[3], const double p[3],
                    double out[3]) {
  int b0 = (int)p[0], b1 = (int)p[1], b2 = (int)p[2];
  double v[8][3];
  for (int c = 0; c < 8; ++c)
    orc_psi_at(psi, n, b0 + kCorner[c][0], b1 + kCorner[c][1],
               b2 + kCorner[c][2], v[c]);
  double f0 = p[0] - (double)b0, f1 = p[1] - (double)b1, f2 = p[2] - (double)b2;
  for (int k = 0; k < 3; ++k) {
    double s[8];
    for (int c = 0; c < 8; ++c) s[c] = v[c][k];
    out[k] = lerp3(s, f0, f1, f2);
  }
}

/* SDF::getDistance(spatialIndex, psi) (SDF.cpp:570-575). */
double orc_warped_distance(const double *live, const double *psi,
                           const int n[3], const orc_params *P, int x, int y,
                           int z) {
  double d[3], loc[3];
  orc_psi_at(psi, n, x, y, z, d);
  loc[0] = ((double)x + d[0]) + 0.5;
  loc[1] = ((double)y + d[1]) + 0.5;
  loc[2] = ((double)z + d[2]) + 0.5;
  return orc_phi_sample(live, n, P, loc);
}

/* SDF::getDistancef(gridLocation, psi) (SDF.cpp:577-582). */
static double warped_distance_f(const double *live, const double *psi,
                                const int n[3], const orc_params *P,
                                const double p[3]) {
  double d[3], loc[3];
  orc_psi_sample(psi, n, p, d);
  loc[0] = (p[0] + d[0]) + 0.5;
  loc[1] = (p[1] + d[1]) + 0.5;
  loc[2] = (p[2] + d[2]) + 0.5;
  return orc_phi_sample(live, n, P, loc);
}

/* ------------------------------------------------------------------------ */
/* finite differences without psi (known-answer tests of the reference)     */
/* ------------------------------------------------------------------------ */

/* SDF::computeDistanceGradient(gridLocation) (SDF.cpp:657-679). */
void orc_distance_gradient_at(const double *phi, const int n[3],
                              const orc_params *P, const double p[3],
                              double out[3]) {
  for (int k = 0; k < 3; ++k)
    if (p[k] < 0.0 || p[k] >= (double)n[k]) {
      out[0] = out[1] = out[2] = 0.0;
      return;
    }
  for (int k = 0; k < 3; ++k) {
    double a[3] = {p[0], p[1], p[2]}, b[3] = {p[0], p[1], p[2]};
    for (int j = 0; j < 3; ++j) {
      double e = (j == k) ? 1.0 : 0.0;
      a[j] = p[j] + e;
      b[j] = p[j] - e;
    }
    out[k] = orc_phi_sample(phi, n, P, a) - orc_phi_sample(phi, n, P, b);
  }
  for (int k = 0; k < 3; ++k) out[k] = out[k] / 2;
}

/* The 19 offsets (in units of h) of the second-derivative stencils, in the
 * order the reference evaluates them (SDF.cpp:847-865,
 * DisplacementField.cpp:305-323). */
static const int kHessOff[19][3] = {
    {0, 0, 0},   {2, 0, 0},   {-2, 0, 0},  {0, 2, 0},   {0, -2, 0},
    {0, 0, 2},   {0, 0, -2},  {1, 0, 1},   {-1, 0, 1},  {0, 1, 1},
    {0, -1, 1},  {1, 1, 0},   {-1, 1, 0},  {-1, 0, -1}, {1, 0, -1},
    {0, -1, -1}, {0, 1, -1},  {-1, -1, 0}, {1, -1, 0}};
enum {
  H0 = 0, HXP2, HXM2, HYP2, HYM2, HZP2, HZM2, HXPZP, HXMZP, HYPZP, HYMZP,
  HXPYP, HXMYP, HXMZM, HXPZM, HYMZM, HYPZM, HXMYM, HXPYM
};

/* Assemble the 3x3 (row-major) second-difference matrix from the 19 samples
 * (SDF.cpp:867-881) -- not yet divided by 4h^2. */
static void hess_assemble(const double f[19], double H[9]) {
  double fxx = (f[HXP2] - 2 * f[H0] + f[HXM2]);
  double fyy = (f[HYP2] - 2 * f[H0] + f[HYM2]);
  double fzz = (f[HZP2] - 2 * f[H0] + f[HZM2]);
  double fxz = (f[HXPZP] + f[HXMZM] - f[HXPZM] - f[HXMZP]);
  double fyz = (f[HYPZP] + f[HYMZM] - f[HYPZM] - f[HYMZP]);
  double fxy = (f[HXPYP] + f[HXMYM] - f[HXPYM] - f[HXMYP]);
  H[0] = fxx; H[4] = fyy; H[8] = fzz;
  H[1] = H[3] = fxy;
  H[2] = H[6] = fxz;
  H[5] = H[7] = fyz;
}

/* SDF::computeDistanceHessian(gridLocation) (SDF.cpp:746-795). */
void orc_distance_hessian_at(const double *phi, const int n[3],
                             const orc_params *P, const double p[3],
                             double out[9]) {
  const double h = P->delta_size;
  for (int k = 0; k < 3; ++k) {
    double t = p[k] - 0.5;
    if (t < 0.0 || t >= (double)n[k]) {
      for (int j = 0; j < 9; ++j) out[j] = 0.0;
      return;
    }
  }
  double f[19];
  for (int s = 0; s < 19; ++s) {
    double q[3];
    for (int k = 0; k < 3; ++k) q[k] = p[k] + h * (double)kHessOff[s][k];
    f[s] = orc_phi_sample(phi, n, P, q);
  }
  hess_assemble(f, out);
  double den = (4 * h * h);
  for (int j = 0; j < 9; ++j) out[j] = out[j] / den;
}

/* DisplacementField::computeJacobian (DisplacementField.cpp:90-140); out is
 * row-major, column k = d psi / d x_k. */
void orc_jacobian(const double *psi, const int n[3], const orc_params *P,
                  double x, double y, double z, double out[9]) {
  const double h = P->delta_size;
  for (int k = 0; k < 3; ++k) {
    double a[3] = {x + (k == 0) * h, y + (k == 1) * h, z + (k == 2) * h};
    double b[3] = {x - (k == 0) * h, y - (k == 1) * h, z - (k == 2) * h};
    double u[3], w[3];
    orc_psi_sample(psi, n, a, u);
    orc_psi_sample(psi, n, b, w);
    for (int r = 0; r < 3; ++r) out[3 * r + k] = u[r] - w[r];
  }
  double den = 2 * h;
  for (int j = 0; j < 9; ++j) out[j] = out[j] / den;
}

/* DisplacementField::computeKillingEnergy (DisplacementField.cpp:171-193). */
double orc_killing_energy(const double *psi, const int n[3],
                          const orc_params *P, double x, double y, double z) {
  double J[9];
  orc_jacobian(psi, n, P, x, y, z, J);
  for (int j = 0; j < 9; ++j)
    if (!isfinite(J[j])) return 0.0;
  /* column-major flattening of J and of J^T, then dot products. */
  double jv[9], jt[9];
  for (int c = 0; c < 3; ++c)
    for (int r = 0; r < 3; ++r) {
      jv[3 * c + r] = J[3 * r + c];
      jt[3 * c + r] = J[3 * c + r];
    }
  double d1 = 0.0, d2 = 0.0;
  d1 = jv[0] * jv[0];
  for (int j = 1; j < 9; ++j) d1 = d1 + jv[j] * jv[j];
  d2 = jt[0] * jv[0];
  for (int j = 1; j < 9; ++j) d2 = d2 + jt[j] * jv[j];
  return d1 + P->gamma_k * d2;
}

/* DisplacementField::computeKillingEnergyGradient (DisplacementField.cpp:274-299),
 * the finite difference of the energy (not used by the solver). */
void orc_killing_energy_gradient_fd(const double *psi, const int n[3],
                                    const orc_params *P, int x, int y, int z,
                                    double out[3]) {
  const double h = P->delta_size;
  int s[3] = {x, y, z};
  for (int k = 0; k < 3; ++k)
    if ((double)s[k] < 2 * h || (double)s[k] >= ((double)n[k] - 2 * h)) {
      out[0] = out[1] = out[2] = 0.0;
      return;
    }
  for (int k = 0; k < 3; ++k) {
    double ep = orc_killing_energy(psi, n, P, x + (k == 0) * h,
                                   y + (k == 1) * h, z + (k == 2) * h);
    double em = orc_killing_energy(psi, n, P, x - (k == 0) * h,
                                   y - (k == 1) * h, z - (k == 2) * h);
    out[k] = ep - em;
  }
  double den = 2 * h;
  for (int k = 0; k < 3; ++k) out[k] = out[k] / den;
}

/* ------------------------------------------------------------------------ */
/* per-voxel energy gradient                                                */
/* ------------------------------------------------------------------------ */

/* SDF::computeDistanceGradient(spatialIndex, psi) (SDF.cpp:726-744): central
 * differences of the warped live SDF at i+0.5 (half a voxel off the value
 * sample of getDistance(i, psi)). */
void orc_distance_gradient(const double *live, const double *psi,
                           const int n[3], const orc_params *P, int x, int y,
                           int z, double out[3]) {
  const double h = P->delta_size;
  double g[3] = {(double)x + 0.5, (double)y + 0.5, (double)z + 0.5};
  for (int k = 0; k < 3; ++k) {
    double a[3], b[3];
    for (int j = 0; j < 3; ++j) {
      double d = h * (double)(j == k);
      a[j] = g[j] + d;
      b[j] = g[j] - d;
    }
    out[k] = warped_distance_f(live, psi, n, P, a) -
             warped_distance_f(live, psi, n, P, b);
  }
  double den = (2 * h);
  for (int k = 0; k < 3; ++k) out[k] = out[k] / den;
}

/* SDF::computeDistanceHessian(spatialIndex, psi) (SDF.cpp:842-886). */
void orc_distance_hessian(const double *live, const double *psi,
                          const int n[3], const orc_params *P, int x, int y,
                          int z, double out[9]) {
  const double h = P->delta_size;
  double g[3] = {(double)x + 0.5, (double)y + 0.5, (double)z + 0.5};
  double f[19];
  for (int s = 0; s < 19; ++s) {
    double q[3];
    for (int k = 0; k < 3; ++k) q[k] = g[k] + h * (double)kHessOff[s][k];
    f[s] = warped_distance_f(live, psi, n, P, q);
  }
  hess_assemble(f, out);
  double den = (4 * h * h);
  for (int j = 0; j < 9; ++j) out[j] = out[j] / den;
}

static inline double norm3(const double v[3]) {
  return sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
}

/* DisplacementField::computeKillingEnergyGradient2 (DisplacementField.cpp:301-347):
 * second differences of psi~ sampled at the integer point, the damped
 * divergence term, the clamp of |g| to killingThreshold, then /4h^2. */
void orc_killing_gradient(const double *psi, const int n[3],
                          const orc_params *P, int x, int y, int z,
                          double out[3]) {
  const double h = P->delta_size;
  double g[3] = {(double)x, (double)y, (double)z};
  double d[19][3];
  for (int s = 0; s < 19; ++s) {
    double q[3];
    for (int k = 0; k < 3; ++k) q[k] = g[k] + h * (double)kHessOff[s][k];
    orc_psi_sample(psi, n, q, d[s]);
  }
  double xx[3], yy[3], zz[3], xy[3], xz[3], yz[3];
  for (int c = 0; c < 3; ++c) {
    xx[c] = (d[HXP2][c] - 2 * d[H0][c] + d[HXM2][c]);
    yy[c] = (d[HYP2][c] - 2 * d[H0][c] + d[HYM2][c]);
    zz[c] = (d[HZP2][c] - 2 * d[H0][c] + d[HZM2][c]);
    xz[c] = (d[HXPZP][c] + d[HXMZM][c] - d[HXPZM][c] - d[HXMZP][c]);
    yz[c] = (d[HYPZP][c] + d[HYMZM][c] - d[HYPZM][c] - d[HYMZP][c]);
    xy[c] = (d[HXPYP][c] + d[HXMYM][c] - d[HXPYM][c] - d[HXMYP][c]);
  }
  double div[3] = {xx[0] + xy[1] + xz[2], xy[0] + yy[1] + yz[2],
                   xz[0] + yz[1] + zz[2]};
  double gk = -2 * P->gamma_k;
  double kg[3];
  for (int c = 0; c < 3; ++c)
    kg[c] = -2.0 * (xx[c] + yy[c] + zz[c]) + gk * div[c];
  double den = (4 * h * h);
  double clamp = P->killing_clamp;
  double nrm = norm3(kg);
  if (nrm > clamp) {
    double s = sqrt(kg[0] * kg[0] + kg[1] * kg[1] + kg[2] * kg[2]);
    for (int c = 0; c < 3; ++c) kg[c] = (kg[c] / s) * clamp;
  }
  for (int c = 0; c < 3; ++c) out[c] = kg[c] / den;
}

/* KillingFusion::computeEnergyGradient and its three terms
 * (KillingFusion.cpp:399-476). */
void orc_energy_gradient(const double *live, const double *can,
                         const double *psi, const int n[3],
                         const orc_params *P, int x, int y, int z,
                         double out[3]) {
  double dg[3] = {0, 0, 0}, lg[3] = {0, 0, 0}, kg[3] = {0, 0, 0};
  if (P->use_data) {
    double g[3];
    orc_distance_gradient(live, psi, n, P, x, y, z, g);
    double s = orc_warped_distance(live, psi, n, P, x, y, z);
    double dd = orc_phi_at(can, n, P, x, y, z);
    double c = (s - dd) / P->voxel_size;
    for (int k = 0; k < 3; ++k) dg[k] = c * g[k];
  }
  if (P->use_levelset) {
    double g[3], H[9];
    orc_distance_gradient(live, psi, n, P, x, y, z, g);
    orc_distance_hessian(live, psi, n, P, x, y, z, H);
    double hg[3];
    for (int r = 0; r < 3; ++r)
      hg[r] = H[3 * r + 0] * g[0] + H[3 * r + 1] * g[1] + H[3 * r + 2] * g[2];
    double nm1 = norm3(g) - 1;
    double np = norm3(g) + P->epsilon;
    for (int r = 0; r < 3; ++r) lg[r] = ((hg[r] * nm1) / np) * P->omega_s;
  }
  if (P->use_killing) {
    double k3[3];
    orc_killing_gradient(psi, n, P, x, y, z, k3);
    for (int r = 0; r < 3; ++r) kg[r] = k3[r] * P->omega_k;
  }
  for (int r = 0; r < 3; ++r) out[r] = (dg[r] + kg[r]) + lg[r];
}

/* Band test of the Jacobi sweep (KillingFusion.cpp:272-274). */
int orc_is_active(const double *live, const double *psi, const int n[3],
                  const orc_params *P, int x, int y, int z) {
  double s = orc_warped_distance(live, psi, n, P, x, y, z);
  if (s > P->max_surface - P->epsilon || s < -P->unknown_clip) return 0;
  return 1;
}

/* The trust-region strategy of the Jacobi sweep (KillingFusion.cpp:288-314),
 * taken only with the data term alone: while the step d = -a * g does not
 * bring phi_live at ((i + psi(i)) + d) + 0.5 closer to phi_can(i) than
 * phi_live at the voxel's own warped position, a /= 1.5.  Returns 1 with the
 * accepted step in d, or 0 when a fell below 1e-7 (the reference then breaks
 * out of the voxel's x loop: this voxel and the rest of its row keep their
 * psi for this iteration). */
static int trust_step(const double *live, const double *can, const double *psi,
                      const int n[3], const orc_params *P, int x, int y, int z,
                      const double g[3], double d[3]) {
  double a = P->alpha;
  int decreased = 0;
  const double dest = orc_phi_at(can, n, P, x, y, z);
  const double prev = orc_warped_distance(live, psi, n, P, x, y, z);
  double cur[3];
  orc_psi_at(psi, n, x, y, z, cur);
  do {
    double loc[3];
    loc[0] = (((double)x + cur[0]) + d[0]) + 0.5;
    loc[1] = (((double)y + cur[1]) + d[1]) + 0.5;
    loc[2] = (((double)z + cur[2]) + d[2]) + 0.5;
    double s = orc_phi_sample(live, n, P, loc);
    double worse = fabs(s - dest) - fabs(prev - dest);
    if (worse > 0) {
      a /= 1.5;
      for (int k = 0; k < 3; ++k) d[k] = -a * g[k];
    } else {
      decreased = 1;
    }
  } while (!decreased && a > 1e-7);
  return !(a < 1e-7);
}

int orc_trust_active(const orc_params *P) {
  return P->use_trust && P->use_data && !P->use_levelset && !P->use_killing;
}

/* KillingFusion::computeDisplacementField, Jacobi schedule
 * (UpdateAllVoxelsInEachIter && UsePreviousIterationDeformationField,
 * KillingFusion.cpp:248-352): every iteration allocates a zero update field,
 * fills it with -alpha*gradient at the voxels inside the band, then adds it
 * to psi.  With P->use_trust and the data term alone, each step goes through
 * the trust-region strategy (trust_step).  active_counts counts the voxels
 * inside the band, including those a row break leaves unvisited. */
int orc_solve_jacobi(const double *live, const double *can, double *psi,
                     const int n[3], const orc_params *P, int iters,
                     int nthreads, int64_t *active_counts) {
  const int64_t N = (int64_t)n[0] * n[1] * n[2];
  const int trust = orc_trust_active(P);
  int diverged = 0;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#else
  (void)nthreads;
#endif
  for (int it = 0; it < iters; ++it) {
    double *delta = (double *)calloc((size_t)N * 3, sizeof(double));
    if (!delta) return -2;
    int64_t act = 0;
#pragma omp parallel for schedule(dynamic) reduction(+ : act) reduction(| : diverged)
    for (int z = 0; z < n[2]; ++z) {
      for (int y = 0; y < n[1]; ++y) {
        int broken = 0;
        for (int x = 0; x < n[0]; ++x) {
          if (!orc_is_active(live, psi, n, P, x, y, z)) continue;
          ++act;
          if (broken) continue;
          double g[3], d[3];
          orc_energy_gradient(live, can, psi, n, P, x, y, z, g);
          int64_t i = lin(n, x, y, z);
          for (int k = 0; k < 3; ++k) d[k] = -P->alpha * g[k];
          if (trust && !trust_step(live, can, psi, n, P, x, y, z, g, d)) {
            broken = 1;
            continue;
          }
          for (int k = 0; k < 3; ++k) delta[3 * i + k] += d[k];
          double cur[3];
          orc_psi_at(psi, n, x, y, z, cur);
          if (!isfinite(cur[0]) || !isfinite(cur[1]) || !isfinite(cur[2]))
            diverged = 1;
        }
      }
    }
    if (active_counts) active_counts[it] = act;
    if (diverged) {
      free(delta);
      return -1;
    }
    for (int64_t i = 0; i < 3 * N; ++i) psi[i] += delta[i];
    free(delta);
  }
  return 0;
}

/* KillingFusion::computeDisplacementField, default per-voxel schedule
 * (KillingFusion.cpp:353-396) on one thread: a voxel whose warped value lies
 * inside the symmetric band +-(MaxSurface - epsilon) (:369) steps psi in
 * place, -alpha * gradient at a time, until the step or the gradient is at
 * most threshold or max_iters steps were taken (:374-394).  Order: cells in
 * z, y, x order (the reference's, colored == 0), or colour by colour
 * ((x&1) | (y&1)<<1 | (z&1)<<2 = 0..7, z, y, x within a colour; colored != 0)
 * as the GPU solver runs them.  Returns 0, or -1 when psi turned non-finite
 * (the reference throws -1).  counts (may be NULL): voxels visited, steps
 * taken, voxels that hit max_iters. */
int orc_solve_pervoxel(const double *live, const double *can, double *psi,
                       const int n[3], const orc_params *P, int max_iters,
                       int colored, int64_t counts[3]) {
  int64_t visited = 0, steps = 0, capped = 0;
  for (int color = 0; color < (colored ? 8 : 1); ++color)
  for (int z = 0; z < n[2]; ++z)
    for (int y = 0; y < n[1]; ++y)
      for (int x = 0; x < n[0]; ++x) {
        if (colored && ((x & 1) | (y & 1) << 1 | (z & 1) << 2) != color) continue;
        double s = orc_warped_distance(live, psi, n, P, x, y, z);
        if (s > P->max_surface - P->epsilon || s < -P->max_surface + P->epsilon)
          continue;
        ++visited;
        const int64_t i = lin(n, x, y, z);
        double g[3];
        int iter = 0;
        do {
          orc_energy_gradient(live, can, psi, n, P, x, y, z, g);
          double d[3];
          for (int k = 0; k < 3; ++k) d[k] = -P->alpha * g[k];
          for (int k = 0; k < 3; ++k) psi[3 * i + k] = psi[3 * i + k] + d[k];
          ++steps;
          if (norm3(d) <= P->threshold) break;
          if (!isfinite(psi[3 * i]) || !isfinite(psi[3 * i + 1]) || !isfinite(psi[3 * i + 2]))
            return -1;
          iter += 1;
        } while (norm3(g) > P->threshold && iter < max_iters);
        if (iter >= max_iters) ++capped;
      }
  if (counts) {
    counts[0] = visited;
    counts[1] = steps;
    counts[2] = capped;
  }
  return 0;
}

/* ------------------------------------------------------------------------ */
/* TSDF integration (SDF.cpp:137-197)                                       */
/* ------------------------------------------------------------------------ */

void orc_integrate(double *phi, int64_t *w, const int n[3], double voxel,
                   const double min3[3], double unknown_clip,
                   const double *depth, int width, int height,
                   const double W[16], const double K[9], double min_depth,
                   double max_depth) {
  for (int z = 0; z < n[2]; ++z) {
    double Z = voxel * ((double)z + 0.5) + min3[2];
    for (int y = 0; y < n[1]; ++y) {
      double Y = voxel * ((double)y + 0.5) + min3[1];
      for (int x = 0; x < n[0]; ++x) {
        double X = voxel * ((double)x + 0.5) + min3[0];
        double c[4];
        for (int r = 0; r < 4; ++r)
          c[r] = W[4 * r + 0] * X + W[4 * r + 1] * Y + W[4 * r + 2] * Z +
                 W[4 * r + 3] * 1.0;
        double a = c[0] / c[2], b = c[1] / c[2];
        double u = K[0] * a + K[1] * b + K[2] * 1.0;
        double v = K[3] * a + K[4] * b + K[5] * 1.0;
        /* A non-finite pixel coordinate never lands in the image: x86-64
         * converts it to INT_MIN (stated explicitly so aarch64 agrees). */
        float fu = (float)(u + 0.5);
        if (!isfinite(fu)) continue;
        int col = (int)roundf(fu);
        if (col < 0 || col >= width) continue;
        float fv = (float)(v + 0.5);
        if (!isfinite(fv)) continue;
        int row = (int)roundf(fv);
        if (row < 0 || row >= height) continue;
        double zc = c[2];
        double d = depth[(int64_t)row * width + col];
        if (d < min_depth || d > max_depth) continue;
        double dist = d - zc;
        if (dist < -unknown_clip) continue;
        int64_t i = lin(n, x, y, z);
        phi[i] = (phi[i] * (double)w[i] + dist) / (double)(w[i] + 1);
        w[i] += 1;
      }
    }
  }
}

int orc_invert4(const double m[16], double out[16]) {
  double a[4][4], inv[4][4];
  for (int r = 0; r < 4; ++r)
    for (int c = 0; c < 4; ++c) {
      a[r][c] = m[4 * r + c];
      inv[r][c] = (r == c) ? 1.0 : 0.0;
    }
  for (int c = 0; c < 4; ++c) {
    int p = c;
    for (int r = c + 1; r < 4; ++r)
      if (fabs(a[r][c]) > fabs(a[p][c])) p = r;
    if (a[p][c] == 0.0) return -1;
    if (p != c)
      for (int k = 0; k < 4; ++k) {
        double t = a[c][k]; a[c][k] = a[p][k]; a[p][k] = t;
        t = inv[c][k]; inv[c][k] = inv[p][k]; inv[p][k] = t;
      }
    double piv = a[c][c];
    for (int k = 0; k < 4; ++k) {
      a[c][k] = a[c][k] / piv;
      inv[c][k] = inv[c][k] / piv;
    }
    for (int r = 0; r < 4; ++r) {
      if (r == c) continue;
      double f = a[r][c];
      if (f == 0.0) continue;
      for (int k = 0; k < 4; ++k) {
        a[r][k] = a[r][k] - f * a[c][k];
        inv[r][k] = inv[r][k] - f * inv[c][k];
      }
    }
  }
  for (int r = 0; r < 4; ++r)
    for (int c = 0; c < 4; ++c) out[4 * r + c] = inv[r][c];
  return 0;
}

/* ------------------------------------------------------------------------ */
/* warp and fuse                                                            */
/* ------------------------------------------------------------------------ */

/* SDF::update (SDF.cpp:300-328): resample the SDF at i+0.5+psi(i); the
 * interpolated weight is truncated into an integer. */
void orc_update(double *phi, int64_t *w, const double *psi, const int n[3],
                const orc_params *P) {
  const int64_t N = (int64_t)n[0] * n[1] * n[2];
  double *nphi = (double *)malloc((size_t)N * sizeof(double));
  int64_t *nw = (int64_t *)malloc((size_t)N * sizeof(int64_t));
  for (int z = 0; z < n[2]; ++z)
    for (int y = 0; y < n[1]; ++y)
      for (int x = 0; x < n[0]; ++x) {
        double d[3];
        orc_psi_at(psi, n, x, y, z, d);
        double loc[3] = {((double)x + 0.5) + d[0], ((double)y + 0.5) + d[1],
                         ((double)z + 0.5) + d[2]};
        double ww = orc_weight_sample(w, n, loc);
        double dist = orc_phi_sample(phi, n, P, loc);
        int64_t i = lin(n, x, y, z);
        nphi[i] = dist;
        nw[i] = (int64_t)ww;
      }
  memcpy(phi, nphi, (size_t)N * sizeof(double));
  memcpy(w, nw, (size_t)N * sizeof(int64_t));
  free(nphi);
  free(nw);
}

/* SDF::fuse(otherSdf) with FUSE_BY_MERGE (SDF.cpp:199-241). */
void orc_fuse(double *phi1, int64_t *w1, const double *phi2,
              const int64_t *w2, int64_t count) {
#pragma omp parallel for
  for (int64_t i = 0; i < count; ++i) {
    int64_t b = w2[i];
    if (b == 0) continue;
    int64_t a = w1[i];
    double d2 = phi2[i];
    if (a == 0) {
      phi1[i] = d2;
      w1[i] = b;
    } else {
      double d1 = phi1[i];
      phi1[i] = ((double)a * d1 + (double)b * d2) / (double)(a + b);
      w1[i] = a + b;
    }
  }
}

/* SDF::fuse(otherSdf, psi) with FUSE_BY_MERGE (SDF.cpp:244-297): the other
 * SDF is sampled at i+0.5+psi(i); its interpolated weight stays a double
 * until it is stored into the integer weight. */
void orc_fuse_psi(double *phi1, int64_t *w1, const double *phi2,
                  const int64_t *w2, const double *psi, const int n[3],
                  const orc_params *P) {
#pragma omp parallel for
  for (int z = 0; z < n[2]; ++z)
    for (int y = 0; y < n[1]; ++y)
      for (int x = 0; x < n[0]; ++x) {
        double d[3];
        orc_psi_at(psi, n, x, y, z, d);
        double loc[3] = {((double)x + 0.5) + d[0], ((double)y + 0.5) + d[1],
                         ((double)z + 0.5) + d[2]};
        double b = orc_weight_sample(w2, n, loc);
        if (fabs(b) < (double)1e-5f) continue;
        int64_t i = lin(n, x, y, z);
        int64_t a = w1[i];
        double d2 = orc_phi_sample(phi2, n, P, loc);
        if (a == 0) {
          phi1[i] = d2;
          w1[i] = (int64_t)b;
        } else {
          double d1 = phi1[i];
          phi1[i] = ((double)a * d1 + b * d2) / ((double)a + b);
          w1[i] = (int64_t)((double)a + b);
        }
      }
}

/* ------------------------------------------------------------------------ */
/* marching cubes                                                           */
/* ------------------------------------------------------------------------ */

/* The classic 256-case triangulation table (P. Bourke, "Polygonising a
 * scalar field", 1994, public domain), the one the reference uses
 * (MarchingCubes.h:61-318).  Row c lists, as hex digits, the cube edges of
 * each triangle of case c. */
static const char *const kTriRows[256] = {
  "", "083", "019", "183981", "12a", "08312a", "92a029", "2832a8a98",
  "3b2", "0b28b0", "19023b", "1b219b98b", "3a1ba3", "0a108a8ba", "3903b9ba9", "98aa8b",
  "478", "430734", "019847", "419471731", "12a847", "34730412a", "92a902847", "2a9297273794",
  "8473b2", "b47b24204", "90184723b", "47b94b9b2921", "3a13ba784", "1ba14b1047b4", "47890b9bab03", "47b4b99ba",
  "954", "954083", "054150", "854835315", "12a954", "30812a495", "52a542402", "2a5325354348",
  "95423b", "0b208b495", "05401523b", "21525828b485", "a3ba13954", "4950818a18ba", "54050b5bab03", "54858aa8b",
  "978579", "930953573", "078017157", "153357", "978957a12", "a12950530573", "802825857a52", "2a5253357",
  "7957893b2", "95797292027b", "23b018178157", "b21b17715", "958857a13a3b", "5705097b010aba0", "ba0b03a50807570", "ba57b5",
  "a65", "0835a6", "9015a6", "1831985a6", "165261", "165126308", "965906026", "598582526328",
  "23ba65", "b08b20a65", "01923b5a6", "5a61929b298b", "63b653513", "08b0b50515b6", "3b6036065059", "65969bb98",
  "5a6478", "43047365a", "1905a6847", "a65197173794", "612651478", "125526304347", "847905065026", "739794329596269",
  "3b2784a65", "5a647242027b", "01947823b5a6", "9219b294b7b45a6", "8473b53515b6", "51b5b610b7b404b", "059065036b63847", "65969b4797b9",
  "a4964a", "4a649a083", "a01a60640", "83181686461a", "149124264", "308129249264", "024426", "832824426",
  "a49a64b23", "08228b49a4a6", "3b201606461a", "64161a48121b8b1", "964936913b63", "8b1810b61914641", "3b6360064", "648b68",
  "7a678a89a", "0730a709a67a", "a671a7178180", "a67a71173", "126168189867", "269291679093739", "780706602", "732672",
  "23ba68a89867", "20727b09767a9a7", "1801781a767a23b", "b21b17a61671", "896867916b63136", "091b67", "7807063b0b60", "7b6",
  "76b", "308b76", "019b76", "819831b76", "a126b7", "12a3086b7", "2902a96b7", "6b72a3a83a98",
  "723627", "708760620", "276237019", "162186198876", "a76a17137", "a7617a187108", "03707a0a96a7", "76a7a88a9",
  "684b86", "36b306046", "86b846901", "946963931b36", "6846b82a1", "12a30b06b046", "4b846b0292a9", "a93a32943b36463",
  "823842462", "042462", "190234246438", "194142246", "8138618466a1", "a10a06604", "4634386a3039a93", "a946a4",
  "49576b", "083495b76", "50154076b", "b76834354315", "954a1276b", "6b712a083495", "76b54a42a402", "348354325a52b76",
  "723762549", "954086062687", "362376150540", "628687218485158", "954a16176137", "16a176107870954", "40a4a503a6a737a", "76a7a854a48a",
  "6956b9b89", "36b063056095", "0b805b01556b", "6b3635531", "12a95b9b8b56", "0b306b09656912a", "b85b56805a52025", "6b36352a3a53",
  "589528562382", "956960062", "158180568382628", "156216", "13616a386569896", "a10a06950560", "03856a", "a56",
  "b5a75b", "b5ab75830", "5b75ab190", "a75ab7981831", "b12b71751", "08312717572b", "9759279022b7", "75272b592328982",
  "25a235375", "820852875a25", "9015a35373a2", "982921872a25752", "135375", "087071175", "903935537", "987597",
  "5845a8ab8", "5045b05abb30", "01984a8aba45", "ab4a45b34941314", "2512852b8458", "04b0b345b2b151b", "0250592b5458b85", "9452b3",
  "25a352345384", "5a2524420", "3a235a385458019", "5a2524192942", "845853351", "045105", "845853905035", "945",
  "4b749b9ab", "0834979b79ab", "1ab1b414074b", "3143481a474bab4", "4b79b492b912", "9749b791b2b1083", "b74b42240", "b74b42834324",
  "29a279237749", "9a7974a27870207", "37a3a274a1a040a", "1a2874", "491417713", "491417081871", "403743", "487",
  "9a8ab8", "30939bb9a", "01a0a88ab", "31ab3a", "12b1b99b8", "30939b1292b9", "02b80b", "32b",
  "23828aa89", "9a2092", "23828a0181a8", "1a2", "138918", "091", "038", "",
};

/* Edge k joins cube corners kEdge[k][0] and kEdge[k][1] (the corner and edge
 * numbering of MarchingCubes.h:392-415 and SDF.cpp:338-355). */
static const int kEdge[12][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0},
                                 {4, 5}, {5, 6}, {6, 7}, {7, 4},
                                 {0, 4}, {1, 5}, {2, 6}, {3, 7}};

/* The edge table (MarchingCubes.h:26-59) is derived: an edge is cut when its
 * two corners fall on different sides of the iso level. */
int orc_mc_edge_mask(int cube) {
  int m = 0;
  for (int e = 0; e < 12; ++e) {
    int a = (cube >> kEdge[e][0]) & 1, b = (cube >> kEdge[e][1]) & 1;
    if (a != b) m |= 1 << e;
  }
  return m;
}

static int hexval(char c) { return c <= '9' ? c - '0' : c - 'a' + 10; }

int orc_mc_tri_row(int cube, int out[16]) {
  const char *s = kTriRows[cube & 255];
  int k = 0;
  for (; s[k]; ++k) out[k] = hexval(s[k]);
  int len = k;
  for (; k < 16; ++k) out[k] = -1;
  return len;
}

/* Corner k of the cell at (x,y,z) (SDF.cpp:338-355). */
static const int kCellCorner[8][3] = {{1, 0, 0}, {0, 0, 0}, {0, 1, 0},
                                      {1, 1, 0}, {1, 0, 1}, {0, 0, 1},
                                      {0, 1, 1}, {1, 1, 1}};

/* VertexInterp (MarchingCubes.h:326-356): p1 + (iso-v1)/(v1-v2)*(p1-p2). */
static void vinterp(double iso, const double p1[3], const double p2[3],
                    double v1, double v2, double out[3]) {
  double t = (iso - v1) / (v1 - v2);
  for (int k = 0; k < 3; ++k) out[k] = p1[k] + t * (p1[k] - p2[k]);
}

/* SDF::getMesh + ProcessVolumeCell + Polygonise (SDF.cpp:330-414,
 * MarchingCubes.h:366-422). */
int64_t orc_mc_extract(const double *phi, const int n[3], const orc_params *P,
                       double *verts, int64_t cap) {
  int64_t ntri = 0;
  double half[3] = {(double)n[0] / 2, (double)n[1] / 2, (double)n[2] / 2};
  for (int z = 0; z < n[2]; ++z)
    for (int y = 0; y < n[1]; ++y)
      for (int x = 0; x < n[0]; ++x) {
        double dist = orc_phi_at(phi, n, P, x, y, z);
        if (dist > P->max_surface || dist < -P->unknown_clip) continue;
        double p[8][3], val[8];
        int cube = 0;
        for (int k = 0; k < 8; ++k) {
          int cx = x + kCellCorner[k][0], cy = y + kCellCorner[k][1],
              cz = z + kCellCorner[k][2];
          p[k][0] = ((double)cx / half[0]) - 1;
          p[k][1] = ((double)cy / half[1]) - 1;
          p[k][2] = ((double)cz / half[2]) - 1;
          val[k] = orc_phi_at(phi, n, P, cx, cy, cz);
          if (val[k] < 0.0) cube |= 1 << k;
        }
        int em = orc_mc_edge_mask(cube);
        if (em == 0) continue;
        double vl[12][3];
        for (int e = 0; e < 12; ++e)
          if (em & (1 << e))
            vinterp(0.0, p[kEdge[e][0]], p[kEdge[e][1]], val[kEdge[e][0]],
                    val[kEdge[e][1]], vl[e]);
        int row[16];
        int len = orc_mc_tri_row(cube, row);
        for (int t = 0; t + 2 < len; t += 3) {
          if (verts && ntri < cap) {
            double *o = verts + 9 * ntri;
            for (int j = 0; j < 3; ++j) {
              const double *v = vl[row[t + j]];
              o[3 * j + 0] = v[0];
              o[3 * j + 1] = -v[1];
              o[3 * j + 2] = v[2];
            }
          }
          ++ntri;
        }
      }
  return ntri;
}

/* ------------------------------------------------------------------------ */
/* project energy and its exact gradient                                    */
/* ------------------------------------------------------------------------ */

static inline int clampi(int v, int lo, int hi) {
  return v < lo ? lo : (v > hi ? hi : v);
}

/* Trilinear sample at t (grid coordinates, i.e. getDistance(t+0.5)) and its
 * derivative with respect to t inside the cell chosen by truncation. */
static double phi_sample_grad(const double *phi, const int n[3],
                              const orc_params *P, const double t[3],
                              double dv[3]) {
  int b[3] = {(int)t[0], (int)t[1], (int)t[2]};
  double v[8];
  for (int c = 0; c < 8; ++c)
    v[c] = orc_phi_at(phi, n, P, b[0] + kCorner[c][0], b[1] + kCorner[c][1],
                      b[2] + kCorner[c][2]);
  double fx = t[0] - b[0], fy = t[1] - b[1], fz = t[2] - b[2];
  double gx = (1 - fz) * ((1 - fy) * (v[1] - v[0]) + fy * (v[3] - v[2])) +
              fz * ((1 - fy) * (v[5] - v[4]) + fy * (v[7] - v[6]));
  double gy = (1 - fz) * ((1 - fx) * (v[2] - v[0]) + fx * (v[3] - v[1])) +
              fz * ((1 - fx) * (v[6] - v[4]) + fx * (v[7] - v[5]));
  double gz = lerp2(v[4], v[5], v[6], v[7], fx, fy) -
              lerp2(v[0], v[1], v[2], v[3], fx, fy);
  dv[0] = gx; dv[1] = gy; dv[2] = gz;
  return lerp3(v, fx, fy, fz);
}

/* Warped value phi_w(j) = live at j + psi_j (grid coordinates). */
static double warped_value(const double *live, const double *psi,
                           const int n[3], const orc_params *P, int x, int y,
                           int z, double dv[3]) {
  int64_t j = lin(n, x, y, z);
  double t[3] = {(double)x + psi[3 * j], (double)y + psi[3 * j + 1],
                 (double)z + psi[3 * j + 2]};
  double tmp[3];
  return phi_sample_grad(live, n, P, t, dv ? dv : tmp);
}

/* Energy of voxel i (assumed active). */
static double voxel_energy(const double *live, const double *can,
                           const double *psi, const int n[3],
                           const orc_params *P, int x, int y, int z) {
  const double v = P->voxel_size;
  int64_t i = lin(n, x, y, z);
  double e = 0.0;
  if (P->use_data) {
    double r = (warped_value(live, psi, n, P, x, y, z, NULL) - can[i]) / v;
    e += 0.5 * r * r;
  }
  int c[3] = {x, y, z};
  if (P->use_levelset) {
    double g[3];
    for (int k = 0; k < 3; ++k) {
      int p[3] = {c[0], c[1], c[2]}, m[3] = {c[0], c[1], c[2]};
      p[k] = clampi(c[k] + 1, 0, n[k] - 1);
      m[k] = clampi(c[k] - 1, 0, n[k] - 1);
      g[k] = 0.5 * (warped_value(live, psi, n, P, p[0], p[1], p[2], NULL) -
                    warped_value(live, psi, n, P, m[0], m[1], m[2], NULL));
    }
    double ve = v * P->epsilon;
    double nr = sqrt(g[0] * g[0] + g[1] * g[1] + g[2] * g[2] + ve * ve);
    double r = nr / v - 1.0;
    e += P->omega_s * 0.5 * r * r;
  }
  if (P->use_killing) {
    double J[3][3];
    for (int k = 0; k < 3; ++k) {
      int p[3] = {c[0], c[1], c[2]}, m[3] = {c[0], c[1], c[2]};
      p[k] = clampi(c[k] + 1, 0, n[k] - 1);
      m[k] = clampi(c[k] - 1, 0, n[k] - 1);
      int64_t ip = lin(n, p[0], p[1], p[2]), im = lin(n, m[0], m[1], m[2]);
      for (int a = 0; a < 3; ++a)
        J[a][k] = 0.5 * (psi[3 * ip + a] - psi[3 * im + a]);
    }
    double f = 0.0, s = 0.0;
    for (int a = 0; a < 3; ++a)
      for (int k = 0; k < 3; ++k) {
        f += J[a][k] * J[a][k];
        s += J[a][k] * J[k][a];
      }
    e += P->omega_k * (f + P->gamma_k * s);
  }
  return e;
}

double orc_project_energy(const double *live, const double *can,
                          const double *psi, const uint8_t *active,
                          const int n[3], const orc_params *P) {
  double e = 0.0;
#pragma omp parallel for reduction(+ : e) schedule(static)
  for (int z = 0; z < n[2]; ++z)
    for (int y = 0; y < n[1]; ++y)
      for (int x = 0; x < n[0]; ++x)
        if (active[lin(n, x, y, z)])
          e += voxel_energy(live, can, psi, n, P, x, y, z);
  return e;
}

double orc_project_energy_local(const double *live, const double *can,
                                const double *psi, const uint8_t *active,
                                const int n[3], const orc_params *P, int x,
                                int y, int z, int radius) {
  double e = 0.0;
  for (int k = z - radius; k <= z + radius; ++k)
    for (int j = y - radius; j <= y + radius; ++j)
      for (int i = x - radius; i <= x + radius; ++i)
        if (in_grid(n, i, j, k) && active[lin(n, i, j, k)])
          e += voxel_energy(live, can, psi, n, P, i, j, k);
  return e;
}

/* Exact gradient of orc_project_energy, by scattering each active voxel's
 * partial derivatives onto the psi entries it reads. */
void orc_project_energy_grad(const double *live, const double *can,
                             const double *psi, const uint8_t *active,
                             const int n[3], const orc_params *P,
                             double *grad) {
  const double v = P->voxel_size;
  const int64_t N = (int64_t)n[0] * n[1] * n[2];
  memset(grad, 0, (size_t)N * 3 * sizeof(double));
  for (int z = 0; z < n[2]; ++z)
    for (int y = 0; y < n[1]; ++y)
      for (int x = 0; x < n[0]; ++x) {
        int64_t i = lin(n, x, y, z);
        if (!active[i]) continue;
        int c[3] = {x, y, z};
        if (P->use_data) {
          double dv[3];
          double r = (warped_value(live, psi, n, P, x, y, z, dv) - can[i]) / v;
          for (int a = 0; a < 3; ++a) grad[3 * i + a] += r / v * dv[a];
        }
        if (P->use_levelset) {
          double g[3], dp[3][3], dm[3][3];
          int64_t ip[3], im[3];
          for (int k = 0; k < 3; ++k) {
            int p[3] = {c[0], c[1], c[2]}, m[3] = {c[0], c[1], c[2]};
            p[k] = clampi(c[k] + 1, 0, n[k] - 1);
            m[k] = clampi(c[k] - 1, 0, n[k] - 1);
            ip[k] = lin(n, p[0], p[1], p[2]);
            im[k] = lin(n, m[0], m[1], m[2]);
            g[k] = 0.5 * (warped_value(live, psi, n, P, p[0], p[1], p[2], dp[k]) -
                          warped_value(live, psi, n, P, m[0], m[1], m[2], dm[k]));
          }
          double ve = v * P->epsilon;
          double nr = sqrt(g[0] * g[0] + g[1] * g[1] + g[2] * g[2] + ve * ve);
          double coef = P->omega_s * (nr / v - 1.0) / (v * nr);
          for (int k = 0; k < 3; ++k) {
            double s = coef * g[k] * 0.5;
            for (int a = 0; a < 3; ++a) {
              grad[3 * ip[k] + a] += s * dp[k][a];
              grad[3 * im[k] + a] -= s * dm[k][a];
            }
          }
        }
        if (P->use_killing) {
          double J[3][3];
          int64_t ip[3], im[3];
          for (int k = 0; k < 3; ++k) {
            int p[3] = {c[0], c[1], c[2]}, m[3] = {c[0], c[1], c[2]};
            p[k] = clampi(c[k] + 1, 0, n[k] - 1);
            m[k] = clampi(c[k] - 1, 0, n[k] - 1);
            ip[k] = lin(n, p[0], p[1], p[2]);
            im[k] = lin(n, m[0], m[1], m[2]);
            for (int a = 0; a < 3; ++a)
              J[a][k] = 0.5 * (psi[3 * ip[k] + a] - psi[3 * im[k] + a]);
          }
          for (int k = 0; k < 3; ++k)
            for (int a = 0; a < 3; ++a) {
              double dJ = P->omega_k * (2 * J[a][k] + 2 * P->gamma_k * J[k][a]);
              grad[3 * ip[k] + a] += 0.5 * dJ;
              grad[3 * im[k] + a] -= 0.5 * dJ;
            }
        }
      }
}
