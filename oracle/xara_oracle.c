/*
 * xara_oracle.c -- TEST INFRASTRUCTURE ONLY (the oracle).
 *
 * A plain-C, single-threaded restatement of the reference's CPU algorithm for
 * the Newton-iteration hot path.  It is the checker for libxara_gpu.so and
 * the timed CPU baseline; the product never links, loads or calls it.
 * Every function cites the reference file:line it restates (paths relative
 * to the reference's SRC/ directory).  Its outputs are pinned against the
 * reference's own classes compiled from source (ref_harness.cpp) through the
 * fixtures in tests/golden/.
 *
 * Scope: J2 plasticity (plane strain and 3D), FourNodeQuad, Brick, the
 * Plain/Transformation (SP-only) handlers, RCM DOF numbering, the
 * SparseGenColLinSOE pattern, the ProfileSPD skyline LDL^T solver, and the
 * Newton-Raphson loop with LoadControl and CTestNormDispIncr /
 * CTestNormUnbalance.
 */
#define _POSIX_C_SOURCE 200809L
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "../include/xara_gpu.h"

#define XO_MAX_NEN 8

static double now_s(void) {
  struct timespec t;
  clock_gettime(CLOCK_MONOTONIC, &t);
  return (double)t.tv_sec + 1e-9 * (double)t.tv_nsec;
}

/* ------------------------------------------------------------------------ */
/* J2 plasticity                                                            */
/* ------------------------------------------------------------------------ */

/* Deviatoric projector entries (matrix/identity.h IIdev table). */
static double iidev(int i, int j, int k, int l) {
  if (i == j && k == l) return (i == k) ? 2. / 3. : -1. / 3.;
  if ((i == k && j == l) || (i == l && j == k)) return 0.5;
  return 0.0;
}
static double ibuni(int i, int j, int k, int l) { return (i == j && k == l) ? 1.0 : 0.0; }

/* J2Plasticity::index_map (material/plastic/J2Plasticity.cpp:445-490) */
static const int XO_IMAP[6][2] = {{0, 0}, {1, 1}, {2, 2}, {0, 1}, {1, 2}, {2, 0}};

/* Hardening q(xi) and q'(xi) (J2Plasticity.cpp:426-438). */
static double j2_q(const double *p, double xi) {
  return p[5] * xi + p[3] + (p[2] - p[3]) * exp(-p[4] * xi);
}
static double j2_qprime(const double *p, double xi) {
  return (p[2] - p[3]) * (-p[4]) * exp(-p[4] * xi) + p[5];
}

/*
 * J2Plasticity::plastic_integrator (material/plastic/J2Plasticity.cpp:228-395).
 * p = K G sigma0 sigma_inf delta H eta rho.  strain, epn (3x3 row major) are
 * the trial strain tensor and the committed plastic strain; outputs the
 * stress tensor, the rank-4 tangent (81), the trial plastic strain and xi.
 * Returns -1 after more than 25 local iterations (:309-314), else 0.
 * eta > 0 uses dt (ops_Dt); the workloads here are rate independent.
 */
static int xo_j2_integrate(const double *p, double dt, const double strain[9],
                           const double epn[9], double xin, double stress[9],
                           double tangent[81], double epnp1[9], double *xinp1) {
  const double bulk = p[0], shear = p[1], sigma0 = p[2], eta = p[6];
  const double tolerance = 1.0e-10 * sigma0;
  const double root23 = sqrt(2.0 / 3.0);
  double dev_strain[9], dev_stress[9], normal[9];
  double trace = strain[0] + strain[4] + strain[8];
  for (int i = 0; i < 9; i++) dev_strain[i] = strain[i];
  for (int i = 0; i < 3; i++) dev_strain[4 * i] -= 1. / 3. * trace;
  for (int i = 0; i < 9; i++) dev_stress[i] = (dev_strain[i] - epn[i]) * (2.0 * shear);
  double norm_tau = 0.0;
  for (int i = 0; i < 9; i++) norm_tau += dev_stress[i] * dev_stress[i];
  norm_tau = sqrt(norm_tau);
  double inv_norm_tau = 0.0;
  if (norm_tau > tolerance) {
    inv_norm_tau = 1.0 / norm_tau;
    for (int i = 0; i < 9; i++) normal[i] = inv_norm_tau * dev_stress[i];
  } else {
    for (int i = 0; i < 9; i++) normal[i] = 0.0;
  }
  double phi = norm_tau - root23 * j2_q(p, xin);
  double gamma = 0.0, theta_inv = 0.0;
  int status = 0;
  if (phi > 0.0) {
    double resid = 1.0;
    int it = 0;
    while (fabs(resid) > tolerance) {
      resid = norm_tau - (2.0 * shear) * gamma - root23 * j2_q(p, xin + root23 * gamma);
      if (eta > 0.0 && dt > 0.0) resid -= (eta / dt) * gamma;
      double tang = -(2.0 * shear) - 2. / 3. * j2_qprime(p, xin + root23 * gamma);
      if (eta > 0.0 && dt > 0.0) tang -= (eta / dt);
      gamma -= (resid / tang);
      it++;
      if (it > 25) { status = -1; break; }
    }
    gamma *= 1.0 - 1e-08;
    for (int i = 0; i < 9; i++) epnp1[i] = epn[i] + gamma * normal[i];
    *xinp1 = xin + root23 * gamma;
    for (int i = 0; i < 9; i++) dev_stress[i] = (2.0 * shear) * (dev_strain[i] - epnp1[i]);
    double theta = (2.0 * shear) + 2. / 3. * j2_qprime(p, *xinp1);
    if (eta > 0.0 && dt > 0.0) theta += (eta / dt);
    theta_inv = 1.0 / theta;
  } else {
    for (int i = 0; i < 9; i++) epnp1[i] = epn[i];
    *xinp1 = xin;
  }
  for (int i = 0; i < 9; i++) stress[i] = dev_stress[i];
  for (int i = 0; i < 3; i++) stress[4 * i] += bulk * trace;
  double c1 = -4.0 * shear * shear;
  double c2 = c1 * theta_inv;
  double c3 = c1 * gamma * inv_norm_tau;
  for (int ii = 0; ii < 6; ii++) {
    for (int jj = 0; jj < 6; jj++) {
      int i = XO_IMAP[ii][0], j = XO_IMAP[ii][1], k = XO_IMAP[jj][0], l = XO_IMAP[jj][1];
      double NbunN = normal[3 * i + j] * normal[3 * k + l];
      double t = bulk * ibuni(i, j, k, l);
      t += (2.0 * shear) * iidev(i, j, k, l);
      t += c2 * NbunN;
      t += c3 * (iidev(i, j, k, l) - NbunN);
      tangent[27 * i + 9 * j + 3 * k + l] = t;
      tangent[27 * j + 9 * i + 3 * k + l] = t;
      tangent[27 * i + 9 * j + 3 * l + k] = t;
      tangent[27 * j + 9 * i + 3 * l + k] = t;
    }
  }
  return status;
}
#define T4(t, i, j, k, l) (t)[27 * (i) + 9 * (j) + 3 * (k) + (l)]

/*
 * J2PlaneStrain::setTrialStrain/getStress/getTangent
 * (material/Plane/J2PlaneStrain.cpp:124-213): eps = [exx, eyy, gxy];
 * the integrator status is discarded (:133).
 * ep/xi: committed state in, trial state out (ep as 3x3 tensor).
 */
static void xo_j2_plane_strain(const double *p, const double eps[3], const double epn[9],
                               double xin, double sig[3], double D[9], double epnp1[9],
                               double *xinp1) {
  double strain[9] = {0}, stress[9], t[81];
  strain[0] = eps[0];
  strain[4] = eps[1];
  strain[1] = 0.50 * eps[2];
  strain[3] = strain[1];
  xo_j2_integrate(p, 0.0, strain, epn, xin, stress, t, epnp1, xinp1);
  sig[0] = stress[0]; sig[1] = stress[4]; sig[2] = stress[1];
  D[0] = T4(t, 0, 0, 0, 0); D[4] = T4(t, 1, 1, 1, 1); D[8] = T4(t, 0, 1, 0, 1);
  D[1] = T4(t, 0, 0, 1, 1); D[3] = T4(t, 1, 1, 0, 0);
  D[2] = T4(t, 0, 0, 0, 1); D[6] = T4(t, 0, 1, 0, 0);
  D[5] = T4(t, 1, 1, 0, 1); D[7] = T4(t, 0, 1, 1, 1);
}

/* J2ThreeDimensional (material/plastic/J2ThreeDimensional.cpp:123-226):
   eps = [e11 e22 e33 g12 g23 g31]; returns the integrator status (:140). */
static int xo_j2_3d(const double *p, const double eps[6], const double epn[9], double xin,
                    double sig[6], double D[36], double epnp1[9], double *xinp1) {
  double strain[9] = {0}, stress[9], t[81];
  strain[0] = eps[0]; strain[4] = eps[1]; strain[8] = eps[2];
  strain[1] = 0.50 * eps[3]; strain[3] = strain[1];
  strain[5] = 0.50 * eps[4]; strain[7] = strain[5];
  strain[6] = 0.50 * eps[5]; strain[2] = strain[6];
  int st = xo_j2_integrate(p, 0.0, strain, epn, xin, stress, t, epnp1, xinp1);
  sig[0] = stress[0]; sig[1] = stress[4]; sig[2] = stress[8];
  sig[3] = stress[1]; sig[4] = stress[5]; sig[5] = stress[6];
  for (int ii = 0; ii < 6; ii++)
    for (int jj = 0; jj < 6; jj++)
      D[6 * ii + jj] = T4(t, XO_IMAP[ii][0], XO_IMAP[ii][1], XO_IMAP[jj][0], XO_IMAP[jj][1]);
  return st;
}

/* Material-point path driver (tests): dim 2 or 3. */
int xo_j2_path(int dim, const double *p, int npts, const double *strain, const int *commit,
               double *stress, double *tangent) {
  double ep[9] = {0}, xi = 0.0, ep1[9], xi1;
  int ns = dim == 2 ? 3 : 6;
  for (int k = 0; k < npts; k++) {
    if (dim == 2)
      xo_j2_plane_strain(p, strain + 3 * k, ep, xi, stress + 3 * k, tangent + 9 * k, ep1, &xi1);
    else
      xo_j2_3d(p, strain + 6 * k, ep, xi, stress + 6 * k, tangent + 36 * k, ep1, &xi1);
    if (commit[k]) { memcpy(ep, ep1, sizeof ep); xi = xi1; }
  }
  (void)ns;
  return 0;
}

/* ------------------------------------------------------------------------ */
/* FourNodeQuad (element/Plane/FourNodeQuad.cpp)                            */
/* ------------------------------------------------------------------------ */

/* Gauss points in GaussLegendre<2,4> order (quadrature/GaussLegendre2D.hpp:27-32) */
static const double XO_QPTS[4][2] = {{-0.57735026918962573, -0.57735026918962573},
                                     {-0.57735026918962573, 0.57735026918962573},
                                     {0.57735026918962573, -0.57735026918962573},
                                     {0.57735026918962573, 0.57735026918962573}};

/* FourNodeQuad::shapeFunction (FourNodeQuad.cpp:1128-1196); xy[4][2]. */
static double xo_quad_shape(const double xy[4][2], double xi, double eta, double shp[3][4]) {
  double oneMinuseta = 1.0 - eta, onePluseta = 1.0 + eta;
  double oneMinusxi = 1.0 - xi, onePlusxi = 1.0 + xi;
  shp[2][0] = 0.25 * oneMinusxi * oneMinuseta;
  shp[2][1] = 0.25 * onePlusxi * oneMinuseta;
  shp[2][2] = 0.25 * onePlusxi * onePluseta;
  shp[2][3] = 0.25 * oneMinusxi * onePluseta;
  double J00 = 0.25 * (-xy[0][0] * oneMinuseta + xy[1][0] * oneMinuseta + xy[2][0] * onePluseta -
                       xy[3][0] * onePluseta);
  double J01 = 0.25 * (-xy[0][0] * oneMinusxi - xy[1][0] * onePlusxi + xy[2][0] * onePlusxi +
                       xy[3][0] * oneMinusxi);
  double J10 = 0.25 * (-xy[0][1] * oneMinuseta + xy[1][1] * oneMinuseta + xy[2][1] * onePluseta -
                       xy[3][1] * onePluseta);
  double J11 = 0.25 * (-xy[0][1] * oneMinusxi - xy[1][1] * onePlusxi + xy[2][1] * onePlusxi +
                       xy[3][1] * oneMinusxi);
  double detJ = J00 * J11 - J01 * J10;
  double r = 1.0 / detJ;
  double L00 = 0.25 * (J11 * r), L10 = 0.25 * (-J01 * r);
  double L01 = 0.25 * (-J10 * r), L11 = 0.25 * (J00 * r);
  shp[0][0] = -L00 * oneMinuseta - L01 * oneMinusxi;
  shp[0][1] = L00 * oneMinuseta - L01 * onePlusxi;
  shp[0][2] = L00 * onePluseta + L01 * onePlusxi;
  shp[0][3] = -L00 * onePluseta + L01 * oneMinusxi;
  shp[1][0] = -L10 * oneMinuseta - L11 * oneMinusxi;
  shp[1][1] = L10 * oneMinuseta - L11 * onePlusxi;
  shp[1][2] = L10 * onePluseta + L11 * onePlusxi;
  shp[1][3] = -L10 * onePluseta + L11 * oneMinusxi;
  return detJ;
}

/*
 * FourNodeQuad::update (FourNodeQuad.cpp:190-224) when `compute` is set:
 * the trial state of each point from its committed history and u[8], kept in
 * sig[4][6] / D[4][36] like the material objects keep their trial state; then
 * getTangentStiff + getResistingForce (:226-282, :507-552) from the stored
 * trial state, with zero body force, pressure and element load.
 * K[64] row major, P[8].
 */
static void xo_quad_state(int compute, const double *p, double t, const double xy[4][2],
                          const double u[8], const double epn[4][9], const double xin[4],
                          double epnp1[4][9], double xinp1[4], double sig[4][6],
                          double Dm[4][36], double K[64], double P[8]) {
  memset(K, 0, 64 * sizeof(double));
  memset(P, 0, 8 * sizeof(double));
  for (int ip = 0; ip < 4; ip++) {
    double shp[3][4];
    double detJ = xo_quad_shape(xy, XO_QPTS[ip][0], XO_QPTS[ip][1], shp);
    if (compute) {
      double eps[3] = {0, 0, 0};
      for (int b = 0; b < 4; b++) {
        eps[0] += shp[0][b] * u[2 * b];
        eps[1] += shp[1][b] * u[2 * b + 1];
        eps[2] += shp[0][b] * u[2 * b + 1] + shp[1][b] * u[2 * b];
      }
      xo_j2_plane_strain(p, eps, epn[ip], xin[ip], sig[ip], Dm[ip], epnp1[ip], &xinp1[ip]);
    }
    const double *D = Dm[ip], *sg = sig[ip];
    double dvol = detJ * (t * 1.0);
    for (int a = 0, ia = 0; a < 4; a++, ia += 2) {
      for (int b = 0, ib = 0; b < 4; b++, ib += 2) {
        double DB00 = dvol * (D[0] * shp[0][b] + D[2] * shp[1][b]);
        double DB10 = dvol * (D[3] * shp[0][b] + D[5] * shp[1][b]);
        double DB20 = dvol * (D[6] * shp[0][b] + D[8] * shp[1][b]);
        double DB01 = dvol * (D[1] * shp[1][b] + D[2] * shp[0][b]);
        double DB11 = dvol * (D[4] * shp[1][b] + D[5] * shp[0][b]);
        double DB21 = dvol * (D[7] * shp[1][b] + D[8] * shp[0][b]);
        K[8 * ia + ib] += shp[0][a] * DB00 + shp[1][a] * DB20;
        K[8 * ia + ib + 1] += shp[0][a] * DB01 + shp[1][a] * DB21;
        K[8 * (ia + 1) + ib] += shp[1][a] * DB10 + shp[0][a] * DB20;
        K[8 * (ia + 1) + ib + 1] += shp[1][a] * DB11 + shp[0][a] * DB21;
      }
      P[ia] += dvol * (shp[0][a] * sg[0] + shp[1][a] * sg[2]);
      P[ia + 1] += dvol * (shp[1][a] * sg[1] + shp[0][a] * sg[2]);
    }
  }
}

/* ------------------------------------------------------------------------ */
/* Brick (element/Brick/Brick.cpp) and shp3d (interpolate/shp3d.cpp)         */
/* ------------------------------------------------------------------------ */

/* shp3d (interpolate/shp3d.cpp:31-180): shp[4][8] (d/dx, d/dy, d/dz, N). */
static void xo_shp3d(const double xn[3], double *xsj, double shp[4][8], const double xl[3][8]) {
  double ap1 = 1.0 + xn[0], am1 = 1.0 - xn[0];
  double ap2 = 1.0 + xn[1], am2 = 1.0 - xn[1];
  double ap3 = 1.0 + xn[2], am3 = 1.0 - xn[2];
  double c1, c2, c3;
  c1 = 0.125 * am1 * am2; c2 = 0.125 * am2 * am3; c3 = 0.125 * am1 * am3;
  shp[0][0] = -c2; shp[0][1] = c2; shp[1][0] = -c3; shp[1][3] = c3;
  shp[2][0] = -c1; shp[2][4] = c1; shp[3][0] = c1 * am3; shp[3][4] = c1 * ap3;
  c1 = 0.125 * ap1 * ap2; c2 = 0.125 * ap2 * ap3; c3 = 0.125 * ap1 * ap3;
  shp[0][7] = -c2; shp[0][6] = c2; shp[1][5] = -c3; shp[1][6] = c3;
  shp[2][2] = -c1; shp[2][6] = c1; shp[3][2] = c1 * am3; shp[3][6] = c1 * ap3;
  c1 = 0.125 * am1 * ap2; c2 = 0.125 * am2 * ap3; c3 = 0.125 * am1 * ap3;
  shp[0][4] = -c2; shp[0][5] = c2; shp[1][4] = -c3; shp[1][7] = c3;
  shp[2][3] = -c1; shp[2][7] = c1; shp[3][3] = c1 * am3; shp[3][7] = c1 * ap3;
  c1 = 0.125 * ap1 * am2; c2 = 0.125 * ap2 * am3; c3 = 0.125 * ap1 * am3;
  shp[0][3] = -c2; shp[0][2] = c2; shp[1][1] = -c3; shp[1][2] = c3;
  shp[2][1] = -c1; shp[2][5] = c1; shp[3][1] = c1 * am3; shp[3][5] = c1 * ap3;
  double xs[3][3];
  for (int j = 0; j < 3; j++) {
    xs[j][0] = (xl[j][1] - xl[j][0]) * shp[0][1] + (xl[j][2] - xl[j][3]) * shp[0][2] +
               (xl[j][5] - xl[j][4]) * shp[0][5] + (xl[j][6] - xl[j][7]) * shp[0][6];
    xs[j][1] = (xl[j][2] - xl[j][1]) * shp[1][2] + (xl[j][3] - xl[j][0]) * shp[1][3] +
               (xl[j][6] - xl[j][5]) * shp[1][6] + (xl[j][7] - xl[j][4]) * shp[1][7];
    xs[j][2] = (xl[j][4] - xl[j][0]) * shp[2][4] + (xl[j][5] - xl[j][1]) * shp[2][5] +
               (xl[j][6] - xl[j][2]) * shp[2][6] + (xl[j][7] - xl[j][3]) * shp[2][7];
  }
  double ad[3][3];
  ad[0][0] = xs[1][1] * xs[2][2] - xs[1][2] * xs[2][1];
  ad[0][1] = xs[2][1] * xs[0][2] - xs[2][2] * xs[0][1];
  ad[0][2] = xs[0][1] * xs[1][2] - xs[0][2] * xs[1][1];
  ad[1][0] = xs[1][2] * xs[2][0] - xs[1][0] * xs[2][2];
  ad[1][1] = xs[2][2] * xs[0][0] - xs[2][0] * xs[0][2];
  ad[1][2] = xs[0][2] * xs[1][0] - xs[0][0] * xs[1][2];
  ad[2][0] = xs[1][0] * xs[2][1] - xs[1][1] * xs[2][0];
  ad[2][1] = xs[2][0] * xs[0][1] - xs[2][1] * xs[0][0];
  ad[2][2] = xs[0][0] * xs[1][1] - xs[0][1] * xs[1][0];
  *xsj = xs[0][0] * ad[0][0] + xs[0][1] * ad[1][0] + xs[0][2] * ad[2][0];
  double rxsj = 1.0 / *xsj;
  for (int j = 0; j < 3; j++)
    for (int i = 0; i < 3; i++) xs[i][j] = ad[i][j] * rxsj;
  for (int k = 0; k < 8; k++) {
    double d1 = shp[0][k] * xs[0][0] + shp[1][k] * xs[1][0] + shp[2][k] * xs[2][0];
    double d2 = shp[0][k] * xs[0][1] + shp[1][k] * xs[1][1] + shp[2][k] * xs[2][1];
    double d3 = shp[0][k] * xs[0][2] + shp[1][k] * xs[1][2] + shp[2][k] * xs[2][2];
    shp[0][k] = d1; shp[1][k] = d2; shp[2][k] = d3;
  }
}

/*
 * Brick::update (Brick.cpp:719-840) when `compute` is set, then
 * formResidAndTangent (:844-1021) from the stored trial state, zero body
 * force: 2x2x2 Gauss in (i,j,k) nested order with sg = -+1/sqrt(3), wg = 1.
 * K[24*24] row major, R[24].  Returns -1 if a point's return map failed.
 */
static int xo_brick_state(int compute, const double *p, const double xl[3][8],
                          const double u[24], const double epn[8][9], const double xin[8],
                          double epnp1[8][9], double xinp1[8], double sigm[8][6],
                          double Dm[8][36], double *K, double *R) {
  const double one_over_root3 = 1.0 / sqrt(3.0);   /* Brick.cpp:56-59 */
  const double sg[2] = {-one_over_root3, one_over_root3};
  memset(K, 0, 576 * sizeof(double));
  memset(R, 0, 24 * sizeof(double));
  int count = 0, status = 0;
  for (int i = 0; i < 2; i++)
    for (int j = 0; j < 2; j++)
      for (int k = 0; k < 2; k++, count++) {
        double xi[3] = {sg[i], sg[j], sg[k]}, xsj, shp[4][8];
        xo_shp3d(xi, &xsj, shp, xl);
        double dvol = 1.0 * xsj;
        if (compute) {
          double eps[6] = {0, 0, 0, 0, 0, 0};
          for (int a = 0; a < 8; a++) {
            const double *ul = u + 3 * a;
            eps[0] += shp[0][a] * ul[0];
            eps[1] += shp[1][a] * ul[1];
            eps[2] += shp[2][a] * ul[2];
            eps[3] += shp[1][a] * ul[0] + shp[0][a] * ul[1];
            eps[4] += shp[2][a] * ul[1] + shp[1][a] * ul[2];
            eps[5] += shp[2][a] * ul[0] + shp[0][a] * ul[2];
          }
          if (xo_j2_3d(p, eps, epn[count], xin[count], sigm[count], Dm[count], epnp1[count],
                       &xinp1[count]) < 0)
            status = -1;
        }
        double s[6], D[36];
        for (int q = 0; q < 6; q++) s[q] = sigm[count][q] * dvol;
        for (int q = 0; q < 36; q++) D[q] = Dm[count][q] * dvol;
        for (int a = 0; a < 8; a++) {
          double b0 = shp[0][a], b1 = shp[1][a], b2 = shp[2][a];
          R[3 * a + 0] += b0 * s[0] + b1 * s[3] + b2 * s[5];
          R[3 * a + 1] += b1 * s[1] + b0 * s[3] + b2 * s[4];
          R[3 * a + 2] += b2 * s[2] + b1 * s[4] + b0 * s[5];
          /* BJ^T D (3x6), with BJ from Brick::computeB (:1047-1081) */
          double BtD[3][6];
          for (int q = 0; q < 6; q++) {
            BtD[0][q] = b0 * D[0 * 6 + q] + b1 * D[3 * 6 + q] + b2 * D[5 * 6 + q];
            BtD[1][q] = b1 * D[1 * 6 + q] + b0 * D[3 * 6 + q] + b2 * D[4 * 6 + q];
            BtD[2][q] = b2 * D[2 * 6 + q] + b1 * D[4 * 6 + q] + b0 * D[5 * 6 + q];
          }
          for (int c = 0; c < 8; c++) {
            double g0 = shp[0][c], g1 = shp[1][c], g2 = shp[2][c];
            for (int r = 0; r < 3; r++) {
              double *row = K + (size_t)(3 * a + r) * 24 + 3 * c;
              row[0] += BtD[r][0] * g0 + BtD[r][3] * g1 + BtD[r][5] * g2;
              row[1] += BtD[r][1] * g1 + BtD[r][3] * g0 + BtD[r][4] * g2;
              row[2] += BtD[r][2] * g2 + BtD[r][4] * g1 + BtD[r][5] * g0;
            }
          }
        }
      }
  return status;
}

/* ------------------------------------------------------------------------ */
/* Model: handler, numbering, pattern                                       */
/* ------------------------------------------------------------------------ */

typedef struct xo_model {
  xg_model_desc d;
  int nen, nip, neq, nnz, nu;
  int *conn;         /* [ne*nen] node indices                                */
  int *eqn;          /* [nn*ndf]                                             */
  int *rowptr, *colidx;
  int *rowtop;       /* skyline: first row of each column                    */
  long *diag;        /* skyline: offset of column i's first stored entry     */
  double *sky;       /* skyline storage                                      */
  double *invD;
  double *U, *Uc;    /* trial / committed displacements [nu]                 */
  double *ep_c, *xi_c, *ep_t, *xi_t;   /* history [ne*nip*9], [ne*nip]       */
  double *sig_t, *D_t;                 /* trial stress / tangent [ne*nip*6|36] */
  double *vals, *resid, *fext, *dU, *B;
  double lambda_const[8];            /* frozen load factor per pattern       */
  int pattern_const[8], added[8];
  double time, time_c;
  double elem_s, solve_s;
  /* force-based frames (xara_oracle_frame.inc) */
  int fr_nb, fr_order, fr_nip;
  double *ybar, *zbar;               /* section centroids                   */
  double *fr_L, *fr_R;               /* length, local axes [ne*9]           */
  long *fr_foff;                     /* fiber record offset per element     */
  double *fr_fh_c, *fr_fh_t;         /* fiber records                       */
  double *fr_Se, *fr_kv, *fr_Se_c, *fr_kv_c, *fr_vs, *fr_vs_c, *fr_fs, *fr_Ssr, *fr_vlast;
  int *fr_init;
  long long work_pts, work_fib, work_sec;   /* work counters (benchmarks) */
  double *V, *A, *Vc, *Ac;           /* Newmark trial / committed vel, accel [nu] */
  double *K0vals;                    /* assembled initial stiffness (CSR)    */
  double *keepK, *keepP;             /* caller buffers for every element's K, P, or NULL */
} xo_model;

/* Every element's K [ned*ned] and P [ned] also go to these buffers (element
   order, dof order node by node) at each element phase, as
   Element::getTangentStiff / getResistingForce return them; NULL stops it. */
static void xo_keep(xo_model *m, int e, int ned, const double *K, const double *P) {
  if (m->keepK) memcpy(m->keepK + (size_t)e * ned * ned, K, sizeof(double) * ned * ned);
  if (m->keepP) memcpy(m->keepP + (size_t)e * ned, P, sizeof(double) * ned);
}

static int csr_find(const struct xo_model *m, int row, int col);
#include "xara_oracle_frame.inc"

static int node_index(const xg_model_desc *d, int tag) {
  int lo = 0, hi = d->num_nodes - 1;
  while (lo <= hi) {
    int mid = (lo + hi) / 2;
    if (d->node_tag[mid] == tag) return mid;
    if (d->node_tag[mid] < tag) lo = mid + 1; else hi = mid - 1;
  }
  return -1;
}

static int cmp_int(const void *a, const void *b) {
  int x = *(const int *)a, y = *(const int *)b;
  return (x > y) - (x < y);
}

typedef struct { int *v; int n, cap; } ivec;
static void iv_insert_sorted(ivec *a, int x) {
  /* ID::insert (matrix/ID.cpp:512-560): sorted, no duplicates */
  int lo = 0, hi = a->n - 1;
  while (lo <= hi) {
    int mid = (lo + hi) / 2;
    if (a->v[mid] == x) return;
    if (x > a->v[mid]) lo = mid + 1; else hi = mid - 1;
  }
  if (a->n == a->cap) {
    a->cap = a->cap ? 2 * a->cap : 8;
    a->v = (int *)realloc(a->v, sizeof(int) * a->cap);
  }
  memmove(a->v + lo + 1, a->v + lo, sizeof(int) * (a->n - lo));
  a->v[lo] = x;
  a->n++;
}

/*
 * DOF numbering: PlainHandler::handle (analysis/handler/PlainHandler.cpp:60-
 * 200) or TransformationConstraintHandler::handle with SP constraints only
 * (TransformationConstraintHandler.cpp:80-250): every dof -2, SP dofs -1;
 * AnalysisModel::getDOFGroupGraph (analysis/model/AnalysisModel.cpp:356-
 * 392): vertex per node (tag order), edges between all nodes of an element,
 * adjacency sorted (graph/graph/Vertex.cpp:97-105); RCM::number without GPS
 * from the first vertex (graph/numberer/RCM.cpp:67-277);
 * DOF_Numberer::numberDOF (analysis/numberer/DOF_Numberer.cpp:93-140):
 * equations in RCM order over each node's -2 dofs.
 */
static int xo_number(xo_model *m) {
  const xg_model_desc *d = &m->d;
  int nn = d->num_nodes, ndf = d->ndf;
  for (int i = 0; i < nn * ndf; i++) m->eqn[i] = -2;
  for (int s = 0; s < d->num_sp; s++) {
    int n = node_index(d, d->sp_node[s]);
    if (n < 0) return -1;
    m->eqn[n * ndf + d->sp_dof[s]] = -1;
  }
  /* PlainHandler MP constraints with identity matrix: constrained dof -4
     if still -2 (PlainHandler.cpp:128-180) */
  for (int q = 0; q < d->num_mp; q++) {
    int n = node_index(d, d->mp_constrained[q]);
    if (n < 0 || node_index(d, d->mp_retained[q]) < 0) return -1;
    if (m->eqn[n * ndf + d->mp_dof[q]] == -2) m->eqn[n * ndf + d->mp_dof[q]] = -4;
  }
  ivec *adj = (ivec *)calloc(nn, sizeof(ivec));
  for (int e = 0; e < d->num_elems; e++) {
    const int *c = m->conn + (size_t)e * m->nen;
    for (int i = 0; i < m->nen; i++)
      for (int j = 0; j < m->nen; j++)
        if (i != j && c[i] != c[j]) iv_insert_sorted(&adj[c[i]], c[j]);
  }
  /* RCM (non-GPS) */
  int *tmp = (int *)malloc(sizeof(int) * nn), *res = (int *)malloc(sizeof(int) * nn);
  for (int i = 0; i < nn; i++) tmp[i] = -1;
  int currentMark = nn - 1, nextMark = currentMark - 1, iter4 = 0;
  res[currentMark] = 0;
  tmp[0] = currentMark;
  while (nextMark >= 0) {
    int v = res[currentMark];
    for (int i = 0; i < adj[v].n; i++) {
      int w = adj[v].v[i];
      if (tmp[w] == -1) { tmp[w] = nextMark; res[nextMark--] = w; }
    }
    currentMark--;
    if (currentMark == nextMark && currentMark >= 0) {
      /* disconnected: next vertex of the iterator not yet visited */
      while (iter4 < nn && tmp[iter4] != -1) iter4++;
      if (iter4 >= nn) break;
      int w = iter4++;
      nextMark--;
      tmp[w] = currentMark;
      res[currentMark] = w;
    }
  }
  int eq = 0;
  for (int i = 0; i < nn; i++) {
    int n = res[i];
    for (int j = 0; j < ndf; j++)
      if (m->eqn[n * ndf + j] == -2) m->eqn[n * ndf + j] = eq++;
  }
  m->neq = eq;
  /* -4 dofs take the retained node's equation (DOF_Numberer.cpp:155-185) */
  for (int q = 0; q < d->num_mp; q++) {
    int c = node_index(d, d->mp_constrained[q]), r = node_index(d, d->mp_retained[q]);
    if (m->eqn[c * ndf + d->mp_dof[q]] == -4)
      m->eqn[c * ndf + d->mp_dof[q]] = m->eqn[r * ndf + d->mp_dof[q]];
  }
  /* pattern: SparseGenColLinSOE::setSize (sparseGEN/SparseGenColLinSOE.cpp:
     161-261) over AnalysisModel::getDOFGraph (:286-349): row r holds the
     diagonal and every equation that shares an element with r */
  int *cnt = (int *)calloc(m->neq + 1, sizeof(int));
  for (int n = 0; n < nn; n++) {
    int others = 0;
    for (int j = 0; j < ndf; j++) others += m->eqn[n * ndf + j] >= 0;
    for (int k = 0; k < adj[n].n; k++) {
      int o = adj[n].v[k];
      for (int j = 0; j < ndf; j++) others += m->eqn[o * ndf + j] >= 0;
    }
    for (int j = 0; j < ndf; j++) {
      int e = m->eqn[n * ndf + j];
      if (e >= 0) cnt[e + 1] += others;
    }
  }
  int *start = (int *)malloc(sizeof(int) * (m->neq + 1));
  start[0] = 0;
  for (int i = 0; i < m->neq; i++) start[i + 1] = start[i] + cnt[i + 1];
  int *raw = (int *)malloc(sizeof(int) * (size_t)(start[m->neq] + 1));
  int *fill = (int *)calloc(m->neq, sizeof(int));
  for (int n = 0; n < nn; n++) {
    for (int j = 0; j < ndf; j++) {
      int e = m->eqn[n * ndf + j];
      if (e < 0) continue;
      int *dst = raw + start[e] + fill[e];
      int k = 0;
      for (int jj = 0; jj < ndf; jj++) if (m->eqn[n * ndf + jj] >= 0) dst[k++] = m->eqn[n * ndf + jj];
      for (int a = 0; a < adj[n].n; a++) {
        int o = adj[n].v[a];
        for (int jj = 0; jj < ndf; jj++) if (m->eqn[o * ndf + jj] >= 0) dst[k++] = m->eqn[o * ndf + jj];
      }
      fill[e] += k;
    }
  }
  m->rowptr = (int *)malloc(sizeof(int) * (m->neq + 1));
  m->rowptr[0] = 0;
  for (int i = 0; i < m->neq; i++) {      /* sort + unique in place */
    int *row = raw + start[i], k = start[i + 1] - start[i];
    qsort(row, k, sizeof(int), cmp_int);
    int u = 0;
    for (int t = 0; t < k; t++) if (u == 0 || row[t] != row[u - 1]) row[u++] = row[t];
    m->rowptr[i + 1] = m->rowptr[i] + u;
  }
  m->nnz = m->rowptr[m->neq];
  m->colidx = (int *)malloc(sizeof(int) * (size_t)m->nnz);
  for (int i = 0; i < m->neq; i++)
    memcpy(m->colidx + m->rowptr[i], raw + start[i], sizeof(int) * (m->rowptr[i + 1] - m->rowptr[i]));
  free(raw); free(start); free(fill);
  /* skyline profile: ProfileSPDLinSOE::setSize (profileSPD/ProfileSPDLinSOE.cpp:115-190) */
  m->rowtop = (int *)malloc(sizeof(int) * (m->neq + 1));
  m->diag = (long *)malloc(sizeof(long) * (m->neq + 1));
  long off = 0;
  for (int i = 0; i < m->neq; i++) {
    int top = m->colidx[m->rowptr[i]];
    if (top > i) top = i;
    m->rowtop[i] = top;
    m->diag[i] = off;
    off += i - top + 1;
  }
  m->diag[m->neq] = off;
  for (int i = 0; i < nn; i++) free(adj[i].v);
  free(adj); free(tmp); free(res); free(cnt);
  return 0;
}

int xo_elem_update_flag(xo_model *m, int compute);
void xo_destroy(xo_model *m);

xo_model *xo_create(const xg_model_desc *desc) {
  xo_model *m = (xo_model *)calloc(1, sizeof(xo_model));
  m->d = *desc;
  const xg_model_desc *d = &m->d;
  int frames = d->elem_type == XG_ELE_FBC2D || d->elem_type == XG_ELE_FBC3D;
  if (d->elem_type == XG_ELE_QUAD) { m->nen = 4; m->nip = 4; }
  else if (d->elem_type == XG_ELE_BRICK) { m->nen = 8; m->nip = 8; }
  else if (frames) { m->nen = 2; m->nip = 0; }
  else { free(m); return NULL; }
  m->nu = d->num_nodes * d->ndf;
  m->conn = (int *)malloc(sizeof(int) * (size_t)d->num_elems * m->nen);
  for (long i = 0; i < (long)d->num_elems * m->nen; i++) {
    m->conn[i] = node_index(d, d->elem_conn[i]);
    if (m->conn[i] < 0) { free(m->conn); free(m); return NULL; }
  }
  m->eqn = (int *)malloc(sizeof(int) * m->nu);
  if (xo_number(m) < 0) { free(m); return NULL; }
  size_t nh = (size_t)d->num_elems * m->nip;
  m->U = (double *)calloc(m->nu, sizeof(double));
  m->Uc = (double *)calloc(m->nu, sizeof(double));
  m->ep_c = (double *)calloc(nh * 9, sizeof(double));
  m->ep_t = (double *)calloc(nh * 9, sizeof(double));
  m->xi_c = (double *)calloc(nh, sizeof(double));
  m->xi_t = (double *)calloc(nh, sizeof(double));
  m->sig_t = (double *)calloc(nh * 6, sizeof(double));
  m->D_t = (double *)calloc(nh * 36, sizeof(double));
  m->vals = (double *)calloc(m->nnz, sizeof(double));
  m->resid = (double *)calloc(m->neq, sizeof(double));
  m->fext = (double *)calloc(m->neq, sizeof(double));
  m->dU = (double *)calloc(m->neq, sizeof(double));
  m->B = (double *)calloc(m->neq, sizeof(double));
  m->invD = (double *)calloc(m->neq, sizeof(double));
  m->sky = (double *)calloc(m->diag[m->neq], sizeof(double));
  m->V = (double *)calloc(m->nu, sizeof(double));
  m->A = (double *)calloc(m->nu, sizeof(double));
  m->Vc = (double *)calloc(m->nu, sizeof(double));
  m->Ac = (double *)calloc(m->nu, sizeof(double));
  if (frames && xo_frame_setup(m) < 0) { xo_destroy(m); return NULL; }
  /* Domain::addElement calls Element::update once (domain/domain/Domain.cpp:
     390-392); the J2 constructors also evaluate the zero-strain state
     (J2Plasticity.cpp:84-111) */
  xo_elem_update_flag(m, 1);
  return m;
}

void xo_destroy(xo_model *m) {
  if (!m) return;
  if (m->d.elem_type == XG_ELE_FBC2D || m->d.elem_type == XG_ELE_FBC3D) xo_frame_free(m);
  free(m->conn); free(m->eqn); free(m->rowptr); free(m->colidx); free(m->rowtop);
  free(m->diag); free(m->sky); free(m->invD); free(m->U); free(m->Uc); free(m->ep_c);
  free(m->ep_t); free(m->xi_c); free(m->xi_t); free(m->sig_t); free(m->D_t); free(m->vals); free(m->resid);
  free(m->fext); free(m->dU); free(m->B);
  free(m->V); free(m->A); free(m->Vc); free(m->Ac); free(m->K0vals);
  free(m);
}

void xo_sizes(const xo_model *m, int *neq, int *nnz) { *neq = m->neq; *nnz = m->nnz; }
void xo_numbering(const xo_model *m, int *eqn) { memcpy(eqn, m->eqn, sizeof(int) * m->nu); }
void xo_pattern(const xo_model *m, int *rowptr, int *colidx) {
  memcpy(rowptr, m->rowptr, sizeof(int) * (m->neq + 1));
  memcpy(colidx, m->colidx, sizeof(int) * (size_t)m->nnz);
}

static int csr_find(const struct xo_model *m, int row, int col) {
  int lo = m->rowptr[row], hi = m->rowptr[row + 1] - 1;
  while (lo <= hi) {
    int mid = (lo + hi) / 2;
    if (m->colidx[mid] == col) return mid;
    if (m->colidx[mid] < col) lo = mid + 1; else hi = mid - 1;
  }
  return -1;
}

/*
 * Domain::update (domain/domain/Domain.cpp:1988-2006) when `compute` is set,
 * followed by IncrementalIntegrator::formTangent / formElementResidual
 * (analysis/integrator/IncrementalIntegrator.cpp:74-101, 202-237): every
 * element's K and P from its stored trial state, assembled in element tag
 * order into the CSR values and the resisting force (equations only).
 */
int xo_elem_update_flag(xo_model *m, int compute) {
  const xg_model_desc *d = &m->d;
  if (d->elem_type == XG_ELE_FBC2D || d->elem_type == XG_ELE_FBC3D)
    return xo_frame_elem_phase(m, compute);
  int ndf = d->ndf, nen = m->nen, nip = m->nip, ned = nen * ndf;
  memset(m->vals, 0, sizeof(double) * (size_t)m->nnz);
  memset(m->resid, 0, sizeof(double) * m->neq);
  double K[576], P[24], u[24];
  int ids[24], bad = 0;
  for (int e = 0; e < d->num_elems; e++) {
    const int *c = m->conn + (size_t)e * nen;
    const double *p = d->j2_param + (size_t)d->elem_mat[e] * XG_J2_NPARAM;
    for (int a = 0; a < nen; a++)
      for (int j = 0; j < ndf; j++) {
        u[a * ndf + j] = m->U[c[a] * ndf + j];
        ids[a * ndf + j] = m->eqn[c[a] * ndf + j];
      }
    size_t h0 = (size_t)e * nip;
    if (d->elem_type == XG_ELE_QUAD) {
      double xy[4][2];
      for (int a = 0; a < 4; a++) { xy[a][0] = d->node_crd[2 * c[a]]; xy[a][1] = d->node_crd[2 * c[a] + 1]; }
      xo_quad_state(compute, p, d->thickness, xy, u, (const double(*)[9])(m->ep_c + 9 * h0),
                    m->xi_c + h0, (double(*)[9])(m->ep_t + 9 * h0), m->xi_t + h0,
                    (double(*)[6])(m->sig_t + 6 * h0), (double(*)[36])(m->D_t + 36 * h0), K, P);
    } else {
      double xl[3][8];
      for (int a = 0; a < 8; a++)
        for (int j = 0; j < 3; j++) xl[j][a] = d->node_crd[3 * c[a] + j];
      bad += xo_brick_state(compute, p, xl, u, (const double(*)[9])(m->ep_c + 9 * h0),
                            m->xi_c + h0, (double(*)[9])(m->ep_t + 9 * h0), m->xi_t + h0,
                            (double(*)[6])(m->sig_t + 6 * h0), (double(*)[36])(m->D_t + 36 * h0),
                            K, P) < 0;
    }
    xo_keep(m, e, ned, K, P);
    for (int i = 0; i < ned; i++) {
      int r = ids[i];
      if (r < 0) continue;
      m->resid[r] += P[i];
      for (int j = 0; j < ned; j++) {
        int cc = ids[j];
        if (cc < 0) continue;
        m->vals[csr_find(m, r, cc)] += K[i * ned + j];
      }
    }
  }
  return -bad;
}

void xo_keep_element_matrices(xo_model *m, double *K, double *P) {
  m->keepK = K;
  m->keepP = P;
}

int xo_elem_update(xo_model *m) {
  if (m->d.elem_type == XG_ELE_QUAD || m->d.elem_type == XG_ELE_BRICK)
    m->work_pts += (long long)m->d.num_elems * m->nip;
  return xo_elem_update_flag(m, 1);
}

/* Work counters: material-point updates (J2 points, or fibers per
   compatibility iteration) and section updates. */
void xo_work(const xo_model *m, long long *points, long long *sections) {
  *points = m->work_pts + m->work_fib;
  *sections = m->work_sec;
}

/* Replay entry for tests: state from committed history + U, no commit. */
int xo_elem_state(xo_model *m, const double *U, double *vals, double *resid) {
  memcpy(m->U, U, sizeof(double) * m->nu);
  int r = xo_elem_update(m);
  if (vals) memcpy(vals, m->vals, sizeof(double) * (size_t)m->nnz);
  if (resid) memcpy(resid, m->resid, sizeof(double) * m->neq);
  return r;
}

void xo_commit(xo_model *m) {
  size_t nh = (size_t)m->d.num_elems * m->nip;
  if (m->d.elem_type == XG_ELE_FBC2D || m->d.elem_type == XG_ELE_FBC3D) xo_frame_commit(m);
  memcpy(m->ep_c, m->ep_t, sizeof(double) * nh * 9);
  memcpy(m->xi_c, m->xi_t, sizeof(double) * nh);
  memcpy(m->Uc, m->U, sizeof(double) * m->nu);
  memcpy(m->Vc, m->V, sizeof(double) * m->nu);
  memcpy(m->Ac, m->A, sizeof(double) * m->nu);
  m->time_c = m->time;
}

/* Domain::revertToLastCommit (domain/domain/Domain.cpp:1925-1949): nodes
   and elements back to the last commit, then Domain::update. */
void xo_revert(xo_model *m) {
  size_t nh = (size_t)m->d.num_elems * m->nip;
  memcpy(m->U, m->Uc, sizeof(double) * m->nu);
  memcpy(m->ep_t, m->ep_c, sizeof(double) * nh * 9);
  memcpy(m->xi_t, m->xi_c, sizeof(double) * nh);
  m->time = m->time_c;
  if (m->d.elem_type == XG_ELE_FBC2D || m->d.elem_type == XG_ELE_FBC3D) xo_frame_revert(m);
  xo_elem_update(m);   /* Domain::revertToLastCommit ends with update() */
}

/*
 * ProfileSPDLinDirectSolver::solve (profileSPD/ProfileSPDLinDirectSolver.cpp:
 * 100-250): skyline LDL^T of the assembled tangent, then forward and back
 * substitution.  The skyline is filled from the CSR values.
 */
static int xo_skyline_solve(xo_model *m, const double *b, double *x) {
  int n = m->neq;
  memset(m->sky, 0, sizeof(double) * m->diag[n]);
  for (int i = 0; i < n; i++) {            /* column i: rows rowtop[i]..i */
    for (int k = m->rowptr[i]; k < m->rowptr[i + 1]; k++) {
      int r = m->colidx[k];
      if (r <= i) m->sky[m->diag[i] + (r - m->rowtop[i])] = m->vals[k];
    }
  }
  for (int i = 0; i < n; i++) x[i] = b[i];
  if (m->sky[0] <= 0.0) return -2;
  m->invD[0] = 1.0 / m->sky[0];
  for (int i = 1; i < n; i++) {
    int ti = m->rowtop[i];
    double *ci = m->sky + m->diag[i];       /* ci[r - ti] = a(r, i) */
    for (int j = ti; j < i; j++) {
      int tj = m->rowtop[j];
      double *cj = m->sky + m->diag[j];
      int k0 = ti > tj ? ti : tj;
      double t = ci[j - ti];
      for (int k = k0; k < j; k++) t -= cj[k - tj] * ci[k - ti];
      ci[j - ti] = t;
    }
    double aii = ci[i - ti], t = 0.0;
    for (int j = ti; j < i; j++) {
      double aji = ci[j - ti];
      double lij = aji * m->invD[j];
      t -= lij * x[j];
      ci[j - ti] = lij;
      aii = aii - lij * aji;
    }
    if (aii == 0.0 || fabs(aii) <= 1.0e-12) return -2;   /* minDiagTol, ProfileSPDLinDirectSolver.h:49 */
    m->invD[i] = 1.0 / aii;
    x[i] += t;
  }
  for (int j = 0; j < n; j++) x[j] = m->invD[j] * x[j];
  for (int k = n - 1; k > 0; k--) {
    int tk = m->rowtop[k];
    double bk = x[k], *ck = m->sky + m->diag[k];
    for (int j = tk; j < k; j++) x[j] -= ck[j - tk] * bk;
  }
  return 0;
}

/* ProfileSPD factor + solve of the tangent assembled by the last element
   update (benchmarks and tests). */
int xo_soe_solve(xo_model *m, const double *b, double *x) { return xo_skyline_solve(m, b, x); }

/* Load factor of pattern p: a LinearSeries pattern follows the domain time
   until `loadConst` freezes it (domain/pattern/LoadPattern.cpp:setLoadConstant). */
static double xo_lambda(const xo_model *m, int p, double time) {
  if (p < 0 || p >= 8 || !m->added[p]) return 0.0;
  return m->pattern_const[p] ? m->lambda_const[p] : time;
}

/* External load vector on the equations at domain time `time`
   (LoadPattern::applyLoad, domain/pattern/LoadPattern.cpp). */
static void xo_form_fext(xo_model *m, double time) {
  const xg_model_desc *d = &m->d;
  memset(m->fext, 0, sizeof(double) * m->neq);
  for (int i = 0; i < d->num_loads; i++) {
    int n = node_index(d, d->load_node[i]);
    double lam = xo_lambda(m, d->load_pattern[i], time);
    for (int j = 0; j < d->ndf; j++) {
      int e = m->eqn[n * d->ndf + j];
      if (e >= 0) m->fext[e] += lam * d->load_value[(size_t)i * d->ndf + j];
    }
  }
}

/* AnalysisModel::incrDisp (analysis/model/AnalysisModel.cpp:452-470): every
   (node, dof) with an equation takes the equation's increment, so dofs
   sharing an equation through equalDOF move together. */
static void xo_incr_disp(xo_model *m, const double *dU, double f) {
  for (int a = 0; a < m->nu; a++) {
    int e = m->eqn[a];
    if (e >= 0) m->U[a] += f * dU[e];
  }
}

/* Forward/back substitution with the factors of the last xo_skyline_solve
   (ProfileSPDLinDirectSolver::solve, isAfactored branch, :203-225). */
static int xo_skyline_resolve(xo_model *m, const double *b, double *x) {
  int n = m->neq;
  for (int i = 0; i < n; i++) x[i] = b[i];
  for (int i = 1; i < n; i++) {
    int ti = m->rowtop[i];
    double *ci = m->sky + m->diag[i], t = 0.0;
    for (int j = ti; j < i; j++) t -= ci[j - ti] * x[j];
    x[i] += t;
  }
  for (int j = 0; j < n; j++) x[j] = m->invD[j] * x[j];
  for (int k = n - 1; k > 0; k--) {
    int tk = m->rowtop[k];
    double bk = x[k], *ck = m->sky + m->diag[k];
    for (int j = tk; j < k; j++) x[j] -= ck[j - tk] * bk;
  }
  return 0;
}

/* TransformationDOF_Group::enforceSPs (analysis/dof_grp/
   TransformationDOF_Group.cpp:1029-1050): imposed values lambda_p * value;
   under PlainHandler every SP is homogeneous (PlainHandler.cpp:78-82). */
static void xo_enforce_sps(xo_model *m) {
  const xg_model_desc *d = &m->d;
  for (int s = 0; s < d->num_sp; s++) {
    int n = node_index(d, d->sp_node[s]);
    double v = 0.0;
    if (d->sp_pattern[s] >= 0 && d->handler == XG_HANDLER_TRANSFORMATION)
      v = xo_lambda(m, d->sp_pattern[s], m->time) * d->sp_value[s];
    m->U[n * d->ndf + d->sp_dof[s]] = v;
  }
}

static int xo_solve_timed(xo_model *m, const double *b, double *x, int refactor, double *acc) {
  double ts = now_s();
  int r = refactor ? xo_skyline_solve(m, b, x) : xo_skyline_resolve(m, b, x);
  *acc += now_s() - ts;
  return r;
}

/*
 * One analysis phase, each step as BasicAnalysisBuilder::analyzeStatic
 * (runtime/runtime/BasicAnalysisBuilder.cpp:337-420): integrator newStep,
 * NewtonRaphson::solveCurrentStep (analysis/algorithm/equiSolnAlgo/
 * NewtonRaphson.cpp:125-222) and commit.
 *   LoadControl: newStep (analysis/integrator/Static/LoadControl.cpp:70-100),
 *     update (:102-121).
 *   DisplacementControl: phat at domainChanged (Static/DisplacementControl.cpp:
 *     372-392), newStep (:121-200) and update (:202-250); the second solve of
 *     every iteration reuses the factorisation as ProfileSPD does.
 */
/* PathSeries::getFactor (domain/pattern/series/PathSeries.cpp:334-356) with
   startTime 0, factor 1 and useLast false: linear between samples, 0 past
   the next-to-last sample. */
static double xo_path(const double *a, int npts, double dt, double t) {
  if (t < 0.0) return 0.0;
  const double incr = t / dt;
  const int i1 = (int)floor(incr), i2 = i1 + 1;
  if (i2 >= npts) return 0.0;
  const double v1 = a[i1], v2 = a[i2];
  return v1 + (v2 - v1) * (incr - i1);
}

/* Initial stiffness of every frame element assembled into CSR values
   (Element::getInitialStiff, the K0 of Rayleigh's betaK0 term). */
static int xo_assemble_k0(xo_model *m, double bk0, const double *bk0_elem) {
  const xg_model_desc *d = &m->d;
  if (d->elem_type != XG_ELE_FBC2D && d->elem_type != XG_ELE_FBC3D) return -1;
  const int ndf = d->ndf, ned = 2 * ndf;
  free(m->K0vals);
  m->K0vals = (double *)calloc(m->nnz > 0 ? m->nnz : 1, sizeof(double));
  double K[144];
  for (int e = 0; e < d->num_elems; e++) {
    xo_frame_initial_stiff(m, e, K);
    const double f = bk0_elem ? bk0_elem[e] : bk0;
    for (int k = 0; k < ned * ned; k++) K[k] *= f;
    int ids[12];
    for (int a = 0; a < 2; a++)
      for (int j = 0; j < ndf; j++) ids[a * ndf + j] = m->eqn[m->conn[2 * e + a] * ndf + j];
    for (int i = 0; i < ned; i++) {
      if (ids[i] < 0) continue;
      for (int j = 0; j < ned; j++)
        if (ids[j] >= 0) m->K0vals[csr_find(m, ids[i], ids[j])] += K[i * ned + j];
    }
  }
  return 0;
}

/*
 * Transient phase: Newmark (displacement formulation, Dynamic/Newmark.cpp:
 * 105-245 newStep, :262-300 tangents, :410-455 update) under NewtonRaphson.
 * Effective tangent c1 Kt + c2 (betaK0 K0) + nodal c2 alphaM M + c3 M;
 * unbalance = nodal loads (patterns, and UniformExcitation's -M r ag(t),
 * EarthquakePattern.cpp:68-99, Node.cpp:668-689) - M a - alphaM M v
 * (Node::getUnbalancedLoadIncInertia, Node.cpp:743-764) - (P_int + betaK0
 * K0 v) (Element::getRayleighDampingForces, element/Element.cpp:284-330).
 * Lumped nodal masses; betaK and betaKc must be 0.
 */
static int xo_run_newmark(xo_model *m, const xg_phase_desc *ph, double *step_u,
                          double *step_lambda, int *step_iters) {
  const xg_model_desc *d = &m->d;
  const int n = m->neq, nu = m->nu, ndf = d->ndf;
  if (ph->dt <= 0.0 || ph->beta == 0.0 || ph->beta_k != 0.0 || ph->beta_k_comm != 0.0)
    return XG_EINVAL;
  const int has_k0 = ph->beta_k_init != 0.0 || ph->beta_k_init_elem != NULL;
  if (has_k0 && xo_assemble_k0(m, ph->beta_k_init, ph->beta_k_init_elem) < 0) return XG_EINVAL;
  const double dt = ph->dt, gam = ph->gamma, bet = ph->beta;
  const double c1 = 1.0, c2 = gam / (bet * dt), c3 = 1.0 / (bet * dt * dt);
  const double a1 = 1.0 - gam / bet, a2 = dt * (1.0 - 0.5 * gam / bet);
  const double a3 = -1.0 / (bet * dt), a4 = 1.0 - 0.5 / bet;
  const double bk0 = has_k0 ? 1.0 : 0.0;   /* K0vals carry betaK0 */
  double *Vt = (double *)calloc(nu, sizeof(double)), *At = (double *)calloc(nu, sizeof(double));
  double *K0v = (double *)calloc(n > 0 ? n : 1, sizeof(double));
  double *Veq = (double *)calloc(n > 0 ? n : 1, sizeof(double));
  int rc = 0;
  for (int s = 0; s < ph->num_steps; s++) {
    double t0 = now_s(), solve_t = 0.0;
    /* newStep */
    memcpy(Vt, m->V, sizeof(double) * nu);
    memcpy(At, m->A, sizeof(double) * nu);
    for (int i = 0; i < nu; i++) {
      if (m->eqn[i] < 0) continue;
      m->V[i] = m->V[i] * a1 + At[i] * a2;
      m->A[i] = m->A[i] * a4 + Vt[i] * a3;
    }
    m->time += dt;
    xo_elem_update(m);
    int it = 0, ok = 0;
    while (1) {
      /* formUnbalance */
      xo_form_fext(m, m->time);
      for (int i = 0; i < n; i++) m->B[i] = m->fext[i];
      for (int a = 0; a < nu; a++) {
        const int e = m->eqn[a];
        if (e < 0) continue;
        const double mass = d->node_mass ? d->node_mass[a] : 0.0;
        if (mass == 0.0) continue;
        if (ph->gm_npts > 0 && a % ndf == ph->gm_dof) {
          const int rec = ph->gm_node_record ? ph->gm_node_record[a / ndf] : 0;
          const double ag = xo_path(ph->gm_accel + (size_t)rec * ph->gm_npts, ph->gm_npts,
                                    ph->gm_dt, m->time);
          m->B[e] -= mass * ag;
        }
        const double am = ph->alpha_m_node ? ph->alpha_m_node[a / ndf] : ph->alpha_m;
        m->B[e] -= mass * m->A[a];
        if (am != 0.0) m->B[e] -= am * mass * m->V[a];
      }
      for (int i = 0; i < n; i++) m->B[i] -= m->resid[i];
      if (bk0 != 0.0) {
        for (int a = 0; a < nu; a++) if (m->eqn[a] >= 0) Veq[m->eqn[a]] = m->V[a];
        for (int r = 0; r < n; r++) {
          double t = 0.0;
          for (int k = m->rowptr[r]; k < m->rowptr[r + 1]; k++) t += m->K0vals[k] * Veq[m->colidx[k]];
          K0v[r] = t;
        }
        for (int i = 0; i < n; i++) m->B[i] -= bk0 * K0v[i];
      }
      if (it > 0) {
        double norm = 0.0;
        if (ph->test == XG_TEST_NORM_DISP_INCR)
          for (int i = 0; i < n; i++) norm += m->dU[i] * m->dU[i];
        else
          for (int i = 0; i < n; i++) norm += m->B[i] * m->B[i];
        if (sqrt(norm) <= ph->tol) { ok = 1; break; }
        if (it >= ph->max_iter) break;
      }
      /* formTangent: c1 Kt + c2 betaK0 K0 + nodal (c2 alphaM + c3) M */
      for (int k = 0; k < m->nnz; k++) {
        m->vals[k] *= c1;
        if (bk0 != 0.0) m->vals[k] += c2 * bk0 * m->K0vals[k];
      }
      for (int a = 0; a < nu; a++) {
        const int e = m->eqn[a];
        const double mass = d->node_mass ? d->node_mass[a] : 0.0;
        if (e < 0 || mass == 0.0) continue;
        const double am = ph->alpha_m_node ? ph->alpha_m_node[a / ndf] : ph->alpha_m;
        m->vals[csr_find(m, e, e)] += c2 * am * mass + c3 * mass;
      }
      if (xo_solve_timed(m, m->B, m->dU, 1, &solve_t) < 0) { rc = XG_ESOLVE; break; }
      /* update */
      xo_incr_disp(m, m->dU, 1.0);
      for (int a = 0; a < nu; a++) {
        const int e = m->eqn[a];
        if (e < 0) continue;
        m->V[a] += m->dU[e] * c2;
        m->A[a] += m->dU[e] * c3;
      }
      xo_elem_update(m);
      it++;
    }
    if (rc) break;
    if (!ok) { rc = XG_ENOCONV; break; }
    xo_commit(m);
    double tt = now_s() - t0;
    m->solve_s += solve_t;
    m->elem_s += tt - solve_t;
    if (step_u) memcpy(step_u + (size_t)s * nu, m->Uc, sizeof(double) * nu);
    if (step_lambda) step_lambda[s] = m->time;
    if (step_iters) step_iters[s] = it;
  }
  free(Vt); free(At); free(K0v); free(Veq);
  return rc;
}

int xo_run_phase(xo_model *m, const xg_phase_desc *ph, double *step_u, double *step_lambda,
                 int *step_iters) {
  const xg_model_desc *d = &m->d;
  int n = m->neq;
  if (ph->integrator == XG_INT_NEWMARK) {
    if (ph->pattern >= 0 && ph->pattern < 8) m->added[ph->pattern] = 1;
    return xo_run_newmark(m, ph, step_u, step_lambda, step_iters);
  }
  if (ph->integrator != XG_INT_LOAD_CONTROL && ph->integrator != XG_INT_DISP_CONTROL)
    return XG_EINVAL;
  if (ph->pattern >= 0 && ph->pattern < 8) m->added[ph->pattern] = 1;
  double *phat = (double *)calloc(n > 0 ? n : 1, sizeof(double));
  double *dUhat = (double *)calloc(n > 0 ? n : 1, sizeof(double));
  int dcEq = -1;
  if (ph->integrator == XG_INT_DISP_CONTROL) {
    int nd = node_index(d, ph->dc_node);
    if (nd < 0) { free(phat); free(dUhat); return XG_EINVAL; }
    dcEq = m->eqn[nd * d->ndf + ph->dc_dof];
    if (dcEq < 0) { free(phat); free(dUhat); return XG_EINVAL; }
    xo_form_fext(m, m->time + 1.0);
    xo_elem_update_flag(m, 0);
    for (int i = 0; i < n; i++) phat[i] = m->fext[i] - m->resid[i];
  }
  int rc = 0;
  for (int s = 0; s < ph->num_steps; s++) {
    double t0 = now_s(), solve_t = 0.0;
    if (ph->integrator == XG_INT_LOAD_CONTROL) {
      m->time += ph->d_lambda;
      xo_enforce_sps(m);
      /* Transformation handler: enforceSPs updates the elements (all of them
         here, which only matters for elements on constrained nodes);
         PlainHandler: no element update before formUnbalance */
      xo_elem_update_flag(m, d->handler == XG_HANDLER_TRANSFORMATION);
    } else {
      xo_elem_update_flag(m, 0);                     /* formTangent: last trial state */
      if (xo_solve_timed(m, phat, dUhat, 1, &solve_t) < 0) { rc = XG_ESOLVE; break; }
      double dUahat = dUhat[dcEq];
      if (dUahat == 0.0) { rc = XG_ESOLVE; break; }
      double dlambda = ph->dc_incr / dUahat;
      m->time += dlambda;
      xo_incr_disp(m, dUhat, dlambda);
      /* applyLoadDomain(currentLambda): the Transformation handler enforces
         the sp values (DisplacementControl.cpp:213) */
      if (d->handler == XG_HANDLER_TRANSFORMATION) xo_enforce_sps(m);
      xo_elem_update(m);
    }
    xo_form_fext(m, m->time);
    for (int i = 0; i < n; i++) m->B[i] = m->fext[i] - m->resid[i];
    int it = 0, ok = 0;
    while (1) {
      if (xo_solve_timed(m, m->B, m->dU, 1, &solve_t) < 0) { rc = XG_ESOLVE; break; }
      if (ph->integrator == XG_INT_DISP_CONTROL) {
        if (xo_solve_timed(m, phat, dUhat, 0, &solve_t) < 0) { rc = XG_ESOLVE; break; }
        double dUahat = dUhat[dcEq];
        if (dUahat == 0.0) { rc = XG_ESOLVE; break; }
        double dLambda = -m->dU[dcEq] / dUahat;
        for (int i = 0; i < n; i++) m->dU[i] = m->dU[i] + dLambda * dUhat[i];
        m->time += dLambda;
      }
      xo_incr_disp(m, m->dU, 1.0);
      if (ph->integrator == XG_INT_DISP_CONTROL && d->handler == XG_HANDLER_TRANSFORMATION)
        xo_enforce_sps(m);   /* DisplacementControl::update's applyLoadDomain (:269) */
      xo_elem_update(m);
      xo_form_fext(m, m->time);
      for (int i = 0; i < n; i++) m->B[i] = m->fext[i] - m->resid[i];
      it++;
      double norm = 0.0;
      if (ph->test == XG_TEST_NORM_DISP_INCR)
        for (int i = 0; i < n; i++) norm += m->dU[i] * m->dU[i];
      else
        for (int i = 0; i < n; i++) norm += m->B[i] * m->B[i];
      norm = sqrt(norm);
      if (getenv("XO_DEBUG")) fprintf(stderr, "step %d iter %d norm %.6e\n", s, it, norm);
      if (norm <= ph->tol) { ok = 1; break; }
      if (it >= ph->max_iter) break;
    }
    if (rc) break;
    if (!ok) { rc = XG_ENOCONV; break; }
    xo_commit(m);
    double dt = now_s() - t0;
    m->solve_s += solve_t;
    m->elem_s += dt - solve_t;
    if (step_u) memcpy(step_u + (size_t)s * m->nu, m->Uc, sizeof(double) * m->nu);
    if (step_lambda) step_lambda[s] = m->time;
    if (step_iters) step_iters[s] = it;
  }
  free(phat);
  free(dUhat);
  if (rc) return rc;
  if (ph->load_const) {
    for (int p = 0; p < 8; p++)
      if (m->added[p] && !m->pattern_const[p]) {
        m->pattern_const[p] = 1;
        m->lambda_const[p] = m->time;
      }
    m->time = m->time_c = 0.0;
  }
  return 0;
}

void xo_times(const xo_model *m, double *elem_s, double *solve_s) {
  *elem_s = m->elem_s;
  *solve_s = m->solve_s;
}

/* Committed history: J2 plastic strain tensor per point [ne*nip*9] and xi. */
void xo_history(const xo_model *m, double *ep, double *xi) {
  size_t nh = (size_t)m->d.num_elems * m->nip;
  if (ep) memcpy(ep, m->ep_c, sizeof(double) * nh * 9);
  if (xi) memcpy(xi, m->xi_c, sizeof(double) * nh);
}
void xo_set_history(xo_model *m, const double *ep, const double *xi) {
  size_t nh = (size_t)m->d.num_elems * m->nip;
  memcpy(m->ep_c, ep, sizeof(double) * nh * 9);
  memcpy(m->xi_c, xi, sizeof(double) * nh);
}
