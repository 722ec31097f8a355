// xg_kernels.cu -- element state determination and deterministic assembly.
//
// FP64 throughout.  Per-point work (the J2 return map) runs one thread per
// integration point over structure-of-arrays history; per-element stiffness
// is formed from the stored trial state of the points, as the reference's
// Element::getTangentStiff reads NDMaterial::getTangent; assembly is a gather
// through a precomputed slot -> contribution map, so the summation order is
// fixed (element tag order) and the result is bit-identical run to run.
#include <cuda_runtime.h>

#include <algorithm>

#include <cstdint>

#include "xg_ff.h"
#include "xg_internal.h"
#include "xg_rcp.h"

namespace xg {

namespace {

constexpr int kThreads = 256;

inline int nblocks(long n, int t = kThreads) { return (int)((n + t - 1) / t); }

// ---------------------------------------------------------------------------
// J2 plasticity: J2Plasticity::plastic_integrator
// (material/plastic/J2Plasticity.cpp:228-395), rate independent.
// Symmetric tensors are held as [xx yy zz xy yz zx] (tensor components).
// ---------------------------------------------------------------------------
struct J2Out {
  double sig[6];        // stress tensor components
  double ep[6];         // trial plastic strain
  double xi;
  double c2, c3;        // plastic tangent coefficients (0 when elastic)
  double n[6];          // unit normal (0 when |s| <= tol)
  int status;
};

__device__ __forceinline__ double j2_q(const double *p, double xi) {
  return p[5] * xi + p[3] + (p[2] - p[3]) * exp(-p[4] * xi);
}
__device__ __forceinline__ double j2_qprime(const double *p, double xi) {
  return (p[2] - p[3]) * (-p[4]) * exp(-p[4] * xi) + p[5];
}

__device__ void j2_return_map(const double *p, const double eps[6], const double epn[6],
                              double xin, J2Out &o) {
  const double bulk = p[0], shear = p[1], sigma0 = p[2];
  const double tolerance = 1.0e-10 * sigma0;
  const double root23 = sqrt(2.0 / 3.0);
  const double trace = eps[0] + eps[1] + eps[2];
  double dev[6], s[6];
#pragma unroll
  for (int i = 0; i < 6; i++) dev[i] = eps[i];
#pragma unroll
  for (int i = 0; i < 3; i++) dev[i] -= 1. / 3. * trace;
#pragma unroll
  for (int i = 0; i < 6; i++) s[i] = (dev[i] - epn[i]) * (2.0 * shear);
  double norm_tau = s[0] * s[0] + s[1] * s[1] + s[2] * s[2] +
                    2.0 * (s[3] * s[3] + s[4] * s[4] + s[5] * s[5]);
  norm_tau = sqrt(norm_tau);
  double inv_norm_tau = 0.0;
  if (norm_tau > tolerance) {
    inv_norm_tau = 1.0 / norm_tau;
#pragma unroll
    for (int i = 0; i < 6; i++) o.n[i] = inv_norm_tau * s[i];
  } else {
#pragma unroll
    for (int i = 0; i < 6; i++) o.n[i] = 0.0;
  }
  const double phi = norm_tau - root23 * j2_q(p, xin);
  double gamma = 0.0, theta_inv = 0.0;
  o.status = 0;
  if (phi > 0.0) {
    double resid = 1.0;
    int it = 0;
    while (fabs(resid) > tolerance) {
      resid = norm_tau - (2.0 * shear) * gamma - root23 * j2_q(p, xin + root23 * gamma);
      const double tang = -(2.0 * shear) - 2. / 3. * j2_qprime(p, xin + root23 * gamma);
      gamma -= (resid / tang);
      if (++it > 25) { o.status = 1; break; }
    }
    gamma *= 1.0 - 1e-08;
#pragma unroll
    for (int i = 0; i < 6; i++) o.ep[i] = epn[i] + gamma * o.n[i];
    o.xi = xin + root23 * gamma;
#pragma unroll
    for (int i = 0; i < 6; i++) s[i] = (2.0 * shear) * (dev[i] - o.ep[i]);
    theta_inv = 1.0 / ((2.0 * shear) + 2. / 3. * j2_qprime(p, o.xi));
  } else {
#pragma unroll
    for (int i = 0; i < 6; i++) o.ep[i] = epn[i];
    o.xi = xin;
  }
#pragma unroll
  for (int i = 0; i < 6; i++) o.sig[i] = s[i];
#pragma unroll
  for (int i = 0; i < 3; i++) o.sig[i] += bulk * trace;
  const double c1 = -4.0 * shear * shear;
  o.c2 = c1 * theta_inv;
  o.c3 = c1 * gamma * inv_norm_tau;
}

// One tangent entry as the reference forms it (J2Plasticity.cpp:362-388):
// K*IbunI + 2G*IIdev + c2*NbunN + c3*(IIdev - NbunN).
__device__ __forceinline__ double j2_tangent_entry(double bulk, double shear, double c2,
                                                   double c3, double ibuni, double iidev,
                                                   double nn) {
  double t = bulk * ibuni;
  t += (2.0 * shear) * iidev;
  t += c2 * nn;
  t += c3 * (iidev - nn);
  return t;
}

// ---------------------------------------------------------------------------
// FourNodeQuad + J2PlaneStrain
// ---------------------------------------------------------------------------
__device__ __constant__ double kQuadPts[4][2] = {
    {-0.57735026918962573, -0.57735026918962573},
    {-0.57735026918962573, 0.57735026918962573},
    {0.57735026918962573, -0.57735026918962573},
    {0.57735026918962573, 0.57735026918962573}};

// FourNodeQuad::shapeFunction (element/Plane/FourNodeQuad.cpp:1128-1196)
__device__ double quad_shape(const double x[4], const double y[4], double xi, double eta,
                             double dN[2][4]) {
  const double oneMinuseta = 1.0 - eta, onePluseta = 1.0 + eta;
  const double oneMinusxi = 1.0 - xi, onePlusxi = 1.0 + xi;
  const double J00 = 0.25 * (-x[0] * oneMinuseta + x[1] * oneMinuseta + x[2] * onePluseta -
                             x[3] * onePluseta);
  const double J01 = 0.25 * (-x[0] * oneMinusxi - x[1] * onePlusxi + x[2] * onePlusxi +
                             x[3] * oneMinusxi);
  const double J10 = 0.25 * (-y[0] * oneMinuseta + y[1] * oneMinuseta + y[2] * onePluseta -
                             y[3] * onePluseta);
  const double J11 = 0.25 * (-y[0] * oneMinusxi - y[1] * onePlusxi + y[2] * onePlusxi +
                             y[3] * oneMinusxi);
  const double detJ = J00 * J11 - J01 * J10;
  const double r = 1.0 / detJ;
  const double L00 = 0.25 * (J11 * r), L10 = 0.25 * (-J01 * r);
  const double L01 = 0.25 * (-J10 * r), L11 = 0.25 * (J00 * r);
  dN[0][0] = -L00 * oneMinuseta - L01 * oneMinusxi;
  dN[0][1] = L00 * oneMinuseta - L01 * onePlusxi;
  dN[0][2] = L00 * onePluseta + L01 * onePlusxi;
  dN[0][3] = -L00 * onePluseta + L01 * oneMinusxi;
  dN[1][0] = -L10 * oneMinuseta - L11 * oneMinusxi;
  dN[1][1] = L10 * oneMinuseta - L11 * onePlusxi;
  dN[1][2] = L10 * onePluseta + L11 * onePlusxi;
  dN[1][3] = -L10 * onePluseta + L11 * oneMinusxi;
  return detJ;
}

__device__ __forceinline__ void quad_nodes(const ContinuumView &v, int e, double x[4],
                                           double y[4]) {
#pragma unroll
  for (int a = 0; a < 4; a++) {
    const int nd = v.conn[a * v.ne + e];
    x[a] = v.crd[nd];
    y[a] = v.crd[v.nn + nd];
  }
}

// One thread per integration point: FourNodeQuad::update (FourNodeQuad.cpp:
// 190-224) + J2PlaneStrain::setTrialStrain/getStress/getTangent
// (material/Plane/J2PlaneStrain.cpp:124-213).  Plane-strain history holds
// ep xx yy zz xy; the stored tangent holds D00 D01 D02 D11 D12 D22 and the
// stress sxx syy sxy.
__global__ void k_quad_update(ContinuumView v) {
  const long npts = (long)v.ne * 4;
  const long pt = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (pt >= npts) return;
  const int e = (int)(pt >> 2), ip = (int)(pt & 3);
  double x[4], y[4], ux[4], uy[4];
#pragma unroll
  for (int a = 0; a < 4; a++) {
    const int nd = v.conn[a * v.ne + e];
    x[a] = v.crd[nd];
    y[a] = v.crd[v.nn + nd];
    ux[a] = v.U[2 * (long)nd];
    uy[a] = v.U[2 * (long)nd + 1];
  }
  double dN[2][4];
  quad_shape(x, y, kQuadPts[ip][0], kQuadPts[ip][1], dN);
  double e0 = 0.0, e1 = 0.0, e2 = 0.0;
#pragma unroll
  for (int b = 0; b < 4; b++) {
    e0 += dN[0][b] * ux[b];
    e1 += dN[1][b] * uy[b];
    e2 += dN[0][b] * uy[b] + dN[1][b] * ux[b];
  }
  const double *p = v.j2 + (long)v.mat[e] * XG_J2_NPARAM;
  const double eps[6] = {e0, e1, 0.0, 0.50 * e2, 0.0, 0.0};
  double epn[6];
  epn[0] = v.ep_c[pt];
  epn[1] = v.ep_c[npts + pt];
  epn[2] = v.ep_c[2 * npts + pt];
  epn[3] = v.ep_c[3 * npts + pt];
  epn[4] = 0.0;
  epn[5] = 0.0;
  J2Out o;
  j2_return_map(p, eps, epn, v.xi_c[pt], o);
  v.ep_t[pt] = o.ep[0];
  v.ep_t[npts + pt] = o.ep[1];
  v.ep_t[2 * npts + pt] = o.ep[2];
  v.ep_t[3 * npts + pt] = o.ep[3];
  v.xi_t[pt] = o.xi;
  v.sig[pt] = o.sig[0];
  v.sig[npts + pt] = o.sig[1];
  v.sig[2 * npts + pt] = o.sig[3];
  const double K = p[0], G = p[1];
  const double n00 = o.n[0], n11 = o.n[1], n01 = o.n[3];
  v.tan[pt] = j2_tangent_entry(K, G, o.c2, o.c3, 1.0, 2. / 3., n00 * n00);
  v.tan[npts + pt] = j2_tangent_entry(K, G, o.c2, o.c3, 1.0, -1. / 3., n00 * n11);
  v.tan[2 * npts + pt] = j2_tangent_entry(K, G, o.c2, o.c3, 0.0, 0.0, n00 * n01);
  v.tan[3 * npts + pt] = j2_tangent_entry(K, G, o.c2, o.c3, 1.0, 2. / 3., n11 * n11);
  v.tan[4 * npts + pt] = j2_tangent_entry(K, G, o.c2, o.c3, 0.0, 0.0, n11 * n01);
  v.tan[5 * npts + pt] = j2_tangent_entry(K, G, o.c2, o.c3, 0.0, 0.5, n01 * n01);
}

// One thread per element: FourNodeQuad::getTangentStiff / getResistingForce
// (FourNodeQuad.cpp:226-282, 507-552) from the stored point state.
// Ke[e*64 + 8*i + j], Re[e*8 + i].
__global__ void k_quad_assemble(ContinuumView v) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= v.ne) return;
  const long npts = (long)v.ne * 4;
  double x[4], y[4];
  quad_nodes(v, e, x, y);
  double K[64], P[8];
#pragma unroll
  for (int i = 0; i < 64; i++) K[i] = 0.0;
#pragma unroll
  for (int i = 0; i < 8; i++) P[i] = 0.0;
  for (int ip = 0; ip < 4; ip++) {
    double dN[2][4];
    const double detJ = quad_shape(x, y, kQuadPts[ip][0], kQuadPts[ip][1], dN);
    const double dvol = detJ * (v.thickness * 1.0);
    const long pt = (long)e * 4 + ip;
    const double D00 = v.tan[pt], D01 = v.tan[npts + pt], D02 = v.tan[2 * npts + pt];
    const double D11 = v.tan[3 * npts + pt], D12 = v.tan[4 * npts + pt];
    const double D22 = v.tan[5 * npts + pt];
    const double D10 = D01, D20 = D02, D21 = D12;
    const double s0 = v.sig[pt], s1 = v.sig[npts + pt], s2 = v.sig[2 * npts + pt];
#pragma unroll
    for (int a = 0; a < 4; a++) {
      const int ia = 2 * a;
#pragma unroll
      for (int b = 0; b < 4; b++) {
        const int ib = 2 * b;
        const double DB00 = dvol * (D00 * dN[0][b] + D02 * dN[1][b]);
        const double DB10 = dvol * (D10 * dN[0][b] + D12 * dN[1][b]);
        const double DB20 = dvol * (D20 * dN[0][b] + D22 * dN[1][b]);
        const double DB01 = dvol * (D01 * dN[1][b] + D02 * dN[0][b]);
        const double DB11 = dvol * (D11 * dN[1][b] + D12 * dN[0][b]);
        const double DB21 = dvol * (D21 * dN[1][b] + D22 * dN[0][b]);
        K[8 * ia + ib] += dN[0][a] * DB00 + dN[1][a] * DB20;
        K[8 * ia + ib + 1] += dN[0][a] * DB01 + dN[1][a] * DB21;
        K[8 * (ia + 1) + ib] += dN[1][a] * DB10 + dN[0][a] * DB20;
        K[8 * (ia + 1) + ib + 1] += dN[1][a] * DB11 + dN[0][a] * DB21;
      }
      P[ia] += dvol * (dN[0][a] * s0 + dN[1][a] * s2);
      P[ia + 1] += dvol * (dN[1][a] * s1 + dN[0][a] * s2);
    }
  }
  double *Ke = v.Ke + (long)e * 64;
#pragma unroll
  for (int i = 0; i < 64; i++) Ke[i] = K[i];
  double *Re = v.Re + (long)e * 8;
#pragma unroll
  for (int i = 0; i < 8; i++) Re[i] = P[i];
}

// ---------------------------------------------------------------------------
// Brick + J2ThreeDimensional
// ---------------------------------------------------------------------------

// shp3d (interpolate/shp3d.cpp:31-180): natural derivatives, Jacobian,
// global derivatives.  xl[3][8] nodal coordinates; g[3][8] out; returns xsj.
__device__ double shp3d_grad(const double xn[3], const double xl[3][8], double g[3][8]) {
  const double ap1 = 1.0 + xn[0], am1 = 1.0 - xn[0];
  const double ap2 = 1.0 + xn[1], am2 = 1.0 - xn[1];
  const double ap3 = 1.0 + xn[2], am3 = 1.0 - xn[2];
  double s[3][8];
  double c1, c2, c3;
  c1 = 0.125 * am1 * am2; c2 = 0.125 * am2 * am3; c3 = 0.125 * am1 * am3;
  s[0][0] = -c2; s[0][1] = c2; s[1][0] = -c3; s[1][3] = c3; s[2][0] = -c1; s[2][4] = c1;
  c1 = 0.125 * ap1 * ap2; c2 = 0.125 * ap2 * ap3; c3 = 0.125 * ap1 * ap3;
  s[0][7] = -c2; s[0][6] = c2; s[1][5] = -c3; s[1][6] = c3; s[2][2] = -c1; s[2][6] = c1;
  c1 = 0.125 * am1 * ap2; c2 = 0.125 * am2 * ap3; c3 = 0.125 * am1 * ap3;
  s[0][4] = -c2; s[0][5] = c2; s[1][4] = -c3; s[1][7] = c3; s[2][3] = -c1; s[2][7] = c1;
  c1 = 0.125 * ap1 * am2; c2 = 0.125 * ap2 * am3; c3 = 0.125 * ap1 * am3;
  s[0][3] = -c2; s[0][2] = c2; s[1][1] = -c3; s[1][2] = c3; s[2][1] = -c1; s[2][5] = c1;
  double xs[3][3];
#pragma unroll
  for (int j = 0; j < 3; j++) {
    xs[j][0] = (xl[j][1] - xl[j][0]) * s[0][1] + (xl[j][2] - xl[j][3]) * s[0][2] +
               (xl[j][5] - xl[j][4]) * s[0][5] + (xl[j][6] - xl[j][7]) * s[0][6];
    xs[j][1] = (xl[j][2] - xl[j][1]) * s[1][2] + (xl[j][3] - xl[j][0]) * s[1][3] +
               (xl[j][6] - xl[j][5]) * s[1][6] + (xl[j][7] - xl[j][4]) * s[1][7];
    xs[j][2] = (xl[j][4] - xl[j][0]) * s[2][4] + (xl[j][5] - xl[j][1]) * s[2][5] +
               (xl[j][6] - xl[j][2]) * s[2][6] + (xl[j][7] - xl[j][3]) * s[2][7];
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
  const double xsj = xs[0][0] * ad[0][0] + xs[0][1] * ad[1][0] + xs[0][2] * ad[2][0];
  const double rxsj = 1.0 / xsj;
  double inv[3][3];
#pragma unroll
  for (int j = 0; j < 3; j++)
#pragma unroll
    for (int i = 0; i < 3; i++) inv[i][j] = ad[i][j] * rxsj;
#pragma unroll
  for (int k = 0; k < 8; k++) {
    g[0][k] = s[0][k] * inv[0][0] + s[1][k] * inv[1][0] + s[2][k] * inv[2][0];
    g[1][k] = s[0][k] * inv[0][1] + s[1][k] * inv[1][1] + s[2][k] * inv[2][1];
    g[2][k] = s[0][k] * inv[0][2] + s[1][k] * inv[1][2] + s[2][k] * inv[2][2];
  }
  return xsj;
}

__device__ __forceinline__ void brick_gauss(int ip, double xn[3]) {
  // Brick.cpp:56-59 and the (i,j,k) nested point order of Brick::update (:754-773)
  const double r = 1.0 / sqrt(3.0);
  xn[0] = (ip & 4) ? r : -r;
  xn[1] = (ip & 2) ? r : -r;
  xn[2] = (ip & 1) ? r : -r;
}

// One thread per point: Brick::update (Brick.cpp:719-840) +
// J2ThreeDimensional::setTrialStrain (J2ThreeDimensional.cpp:123-141).
// History ep xx yy zz xy yz zx; stored tangent a b c n(6) with
// D_ijkl = a d_ij d_kl + b I^sym_ijkl + c n_ij n_kl, which equals the
// reference's K IbunI + 2G IIdev + c2 NbunN + c3 (IIdev - NbunN) for
// a = K - b/3, b = 2G + c3, c = c2 - c3.
// dN/dx and the Jacobian determinant of brick point pt = 8e + ip, from the
// stored geometry when there is one
__device__ __forceinline__ double brick_point_grad(const ContinuumView &v, long npts, long pt,
                                                   double g[3][8]) {
  if (v.geo) {
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int a = 0; a < 8; a++) g[i][a] = v.geo[(8 * i + a) * npts + pt];
    return v.geo[24 * npts + pt];
  }
  const int e = (int)(pt >> 3), ip = (int)(pt & 7);
  double xl[3][8];
#pragma unroll
  for (int a = 0; a < 8; a++) {
    const int nd = v.conn[a * v.ne + e];
    xl[0][a] = v.crd[nd];
    xl[1][a] = v.crd[v.nn + nd];
    xl[2][a] = v.crd[2 * (long)v.nn + nd];
  }
  double xn[3];
  brick_gauss(ip, xn);
  return shp3d_grad(xn, xl, g);
}

// Whether a geometric value splits into a float pair without leaving the
// normal single-precision range: zero, or 2^-100 <= |v| < 2^100.
__device__ __forceinline__ bool geo_splits(double v) {
  const double a = fabs(v);
  return a == 0.0 || (a >= 0x1p-100 && a < 0x1p100);
}

// Stored geometry of every point; geo2 (when given) receives dN/dx split
// into float pairs for the float-float tangent, element-major
// ([point][i][node], so the lanes of one point's nodes read it contiguously),
// *bad counts the points with a value outside the split's range.
__global__ void k_brick_geometry(ContinuumView v, double *geo, float2 *geo2, int *bad) {
  const long npts = (long)v.ne * 8;
  const long pt = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (pt >= npts) return;
  ContinuumView u = v;
  u.geo = nullptr;
  double g[3][8];
  const double dvol = brick_point_grad(u, npts, pt, g);
  bool ok = true;
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int a = 0; a < 8; a++) {
      geo[(8 * i + a) * npts + pt] = g[i][a];
      if (geo2) {
        geo2[(pt * 3 + i) * 8 + a] = split2(g[i][a]);
        ok = ok && geo_splits(g[i][a]);
      }
    }
  geo[24 * npts + pt] = dvol;
  if (!ok) atomicAdd(bad, 1);
}

__global__ void k_brick_update(ContinuumView v) {
  const long npts = (long)v.ne * 8;
  const long pt = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (pt >= npts) return;
  const int e = (int)(pt >> 3);
  double g[3][8], eps[6] = {0, 0, 0, 0, 0, 0};
  int nd[8];
#pragma unroll
  for (int a = 0; a < 8; a++) nd[a] = v.conn[a * v.ne + e];
  brick_point_grad(v, npts, pt, g);
#pragma unroll
  for (int a = 0; a < 8; a++) {
    const double u0 = v.U[3 * (long)nd[a]], u1 = v.U[3 * (long)nd[a] + 1];
    const double u2 = v.U[3 * (long)nd[a] + 2];
    eps[0] += g[0][a] * u0;
    eps[1] += g[1][a] * u1;
    eps[2] += g[2][a] * u2;
    eps[3] += g[1][a] * u0 + g[0][a] * u1;
    eps[4] += g[2][a] * u1 + g[1][a] * u2;
    eps[5] += g[2][a] * u0 + g[0][a] * u2;
  }
  const double strain[6] = {eps[0], eps[1], eps[2], 0.50 * eps[3], 0.50 * eps[4], 0.50 * eps[5]};
  double epn[6];
#pragma unroll
  for (int c = 0; c < 6; c++) epn[c] = v.ep_c[c * npts + pt];
  const double *p = v.j2 + (long)v.mat[e] * XG_J2_NPARAM;
  J2Out o;
  j2_return_map(p, strain, epn, v.xi_c[pt], o);
#pragma unroll
  for (int c = 0; c < 6; c++) v.ep_t[c * npts + pt] = o.ep[c];
  v.xi_t[pt] = o.xi;
#pragma unroll
  for (int c = 0; c < 6; c++) v.sig[c * npts + pt] = o.sig[c];
  const double b = 2.0 * p[1] + o.c3;
  v.tan[pt] = p[0] - b / 3.0;
  v.tan[npts + pt] = b;
  v.tan[2 * npts + pt] = o.c2 - o.c3;
#pragma unroll
  for (int c = 0; c < 6; c++) v.tan[(3 + c) * npts + pt] = o.n[c];
  if (o.status) atomicAdd(v.nfail, 1);
}

__device__ __constant__ unsigned char kPairA[36] = {
    0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 1, 1, 1, 2, 2, 2,
    2, 2, 2, 3, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 6, 6, 7};
__device__ __constant__ unsigned char kPairB[36] = {
    0, 1, 2, 3, 4, 5, 6, 7, 1, 2, 3, 4, 5, 6, 7, 2, 3, 4,
    5, 6, 7, 3, 4, 5, 6, 7, 4, 5, 6, 7, 5, 6, 7, 6, 7, 7};

constexpr int kBrickWarps = 1;
constexpr int kBrickEPW = 4;   // elements per warp

// Four elements per warp: Brick::formResidAndTangent (Brick.cpp:844-1021)
// from the stored point state, formed per node-pair block a <= b and written
// with its transpose: Ke[e*576 + (3a+i)*24 + 3b+k] = K(3a+i, 3b+k), row-major
// like every element's scratch, so each assembled slot's contributions lie
// consecutive for consecutive columns.  Re[e*24 + 3a + i].  The lanes take (element, point) to stage the point
// terms of every node -- dN/dx, its product with the tangent's deviatoric
// direction and the three scalings of the node-pair sum -- then the
// elements' 96 residual entries and 144 node pairs three and five at a
// time: on an FP64 pipe that issues a warp instruction whatever its active
// lanes, one element per warp left 3/4 of the lanes idle in the first phase
// and 7/16 of the pair slots empty.
struct BrickSmem {
  double g[kBrickEPW][8][8][3];    // dN/dx per point, node
  double h[kBrickEPW][8][8][3];    // n . dN/dx
  double u[kBrickEPW][8][8][3];    // dvol*a dN/dx
  double vv[kBrickEPW][8][8][3];   // dvol*b/2 dN/dx
  double w[kBrickEPW][8][8][3];    // dvol*c n . dN/dx
  double sb[kBrickEPW][8];         // dvol*b/2
  double ss[kBrickEPW][8][6];      // dvol*stress
};

__global__ void __launch_bounds__(32 * kBrickWarps) k_brick_assemble(ContinuumView v) {
  __shared__ BrickSmem sm_all[kBrickWarps];
  const int wi = threadIdx.x >> 5, lane = threadIdx.x & 31;
  BrickSmem &S = sm_all[wi];
  const int e0 = (blockIdx.x * kBrickWarps + wi) * kBrickEPW;
  if (e0 >= v.ne) return;
  const long npts = (long)v.ne * 8;
  {
    const int el = lane >> 3, ip = lane & 7, e = e0 + el;
    if (e < v.ne) {
      const long pt = (long)e * 8 + ip;
      double g[3][8];
      const double dvol = brick_point_grad(v, npts, pt, g);
      const double ca = v.tan[pt], cb = v.tan[npts + pt], cc = v.tan[2 * npts + pt];
      double n[6];
#pragma unroll
      for (int c = 0; c < 6; c++) n[c] = v.tan[(3 + c) * npts + pt];
      const double da = dvol * ca, dbh = dvol * (0.5 * cb), dc = dvol * cc;
      S.sb[el][ip] = dbh;
#pragma unroll
      for (int c = 0; c < 6; c++) S.ss[el][ip][c] = dvol * v.sig[c * npts + pt];
#pragma unroll
      for (int a = 0; a < 8; a++) {
        const double gi[3] = {g[0][a], g[1][a], g[2][a]};
        const double hi[3] = {n[0] * gi[0] + n[3] * gi[1] + n[5] * gi[2],
                              n[3] * gi[0] + n[1] * gi[1] + n[4] * gi[2],
                              n[5] * gi[0] + n[4] * gi[1] + n[2] * gi[2]};
#pragma unroll
        for (int i = 0; i < 3; i++) {
          S.g[el][ip][a][i] = gi[i];
          S.h[el][ip][a][i] = hi[i];
          S.u[el][ip][a][i] = da * gi[i];
          S.vv[el][ip][a][i] = dbh * gi[i];
          S.w[el][ip][a][i] = dc * hi[i];
        }
      }
    }
  }
  __syncwarp();
  for (int t = lane; t < kBrickEPW * 24; t += 32) {
    const int el = t / 24, q = t % 24, e = e0 + el;
    if (e >= v.ne) continue;
    const int a = q / 3, i = q % 3;
    // stress tensor row i in [xx yy zz xy yz zx] storage
    const int r0 = (i == 0) ? 0 : (i == 1) ? 3 : 5;
    const int r1 = (i == 0) ? 3 : (i == 1) ? 1 : 4;
    const int r2 = (i == 0) ? 5 : (i == 1) ? 4 : 2;
    double r = 0.0;
#pragma unroll
    for (int ip = 0; ip < 8; ip++)
      r += S.g[el][ip][a][0] * S.ss[el][ip][r0] + S.g[el][ip][a][1] * S.ss[el][ip][r1] +
           S.g[el][ip][a][2] * S.ss[el][ip][r2];
    v.Re[(long)e * 24 + q] = r;
  }
  for (int t = lane; t < kBrickEPW * 36; t += 32) {
    const int el = t / 36, pp = t % 36, e = e0 + el;
    if (e >= v.ne) continue;
    const int a = kPairA[pp], b = kPairB[pp];
    double acc[3][3];
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int k = 0; k < 3; k++) acc[i][k] = 0.0;
#pragma unroll 2
    for (int ip = 0; ip < 8; ip++) {
      const double *Ga = S.g[el][ip][a], *Gb = S.g[el][ip][b], *Hb = S.h[el][ip][b];
      const double *Ua = S.u[el][ip][a], *Va = S.vv[el][ip][a], *Wa = S.w[el][ip][a];
      const double gb[3] = {Gb[0], Gb[1], Gb[2]}, hb[3] = {Hb[0], Hb[1], Hb[2]};
      const double ua[3] = {Ua[0], Ua[1], Ua[2]}, va[3] = {Va[0], Va[1], Va[2]};
      const double wa[3] = {Wa[0], Wa[1], Wa[2]};
      const double dot = S.sb[el][ip] * (Ga[0] * gb[0] + Ga[1] * gb[1] + Ga[2] * gb[2]);
#pragma unroll
      for (int i = 0; i < 3; i++) {
#pragma unroll
        for (int k = 0; k < 3; k++)
          acc[i][k] += ua[i] * gb[k] + va[k] * gb[i] + wa[i] * hb[k];
        acc[i][i] += dot;
      }
    }
    double *Ke = v.Ke + (long)e * 576;
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int k = 0; k < 3; k++) {
        Ke[(3 * a + i) * 24 + 3 * b + k] = acc[i][k];
        if (a != b) Ke[(3 * b + k) * 24 + 3 * a + i] = acc[i][k];
      }
  }
}

// Unbiased exponent of a nonzero double from its bits (-1023 for zero).
__device__ __forceinline__ int f64_exponent(double d) {
  return (int)(((unsigned)__double2hiint(d) >> 20) & 0x7ff) - 1023;
}

// (h, l) = a * b rounded to a float pair
__device__ __forceinline__ float2 ff_mul(float2 a, float2 b) {
  const float p = __fmul_rn(a.x, b.x);
  float e = __fmaf_rn(a.x, b.x, -p);
  e = __fmaf_rn(a.x, b.y, e);
  e = __fmaf_rn(a.y, b.x, e);
  const float hi = __fadd_rn(p, e);
  return make_float2(hi, __fsub_rn(e, __fsub_rn(hi, p)));
}

// (sh, sl) += (dh, dl)
__device__ __forceinline__ void ff_add(float dh, float dl, float &sh, float &sl) {
  const float t = __fadd_rn(sh, dh);
  const float bp = __fsub_rn(t, sh);
  const float err = __fadd_rn(__fsub_rn(sh, __fsub_rn(t, bp)), __fsub_rn(dh, bp));
  sh = t;
  sl = __fadd_rn(sl, __fadd_rn(err, dl));
}

// f * 2^s as a double, from the bits (no FP64 instruction); a subnormal f
// (below 2^-126 of the element's unit scale) is taken as zero.
__device__ __forceinline__ double f32_to_f64_scaled(float f, int s) {
  const unsigned u = __float_as_uint(f);
  const unsigned sign = u & 0x80000000u, m = u & 0x7fffffu;
  const int e8 = (int)((u >> 23) & 0xff);
  if (e8 == 0) return 0.0;
  if (e8 == 255) return __hiloint2double((int)(sign | 0x7ff00000u | (m >> 3)), (int)(m << 29));
  const int de = e8 + (1023 - 127) + s;
  if (de <= 0) return 0.0;
  if (de >= 2047) return __hiloint2double((int)(sign | 0x7ff00000u), 0);
  return __hiloint2double((int)(sign | ((unsigned)de << 20) | (m >> 3)), (int)(m << 29));
}

// The float-float form of k_brick_assemble, four elements per warp.  An
// FP64 FMA holds GB300's FP64 pipe for many cycles; a float-float product
// (xg_ff.h) costs about twelve single-precision instructions and keeps 46
// bits of each product, so the tangent carries the reference's values to a
// few units of 2^-46 of the row's largest entry.  The resisting force stays
// in FP64 (it sets the converged state).  Each element's staged values are
// scaled by powers of two -- the dN/dx by 2^-eg, the tangent scalings
// dvol*{a, b/2, c} by 2^-ed, the element's largest magnitudes -- so every
// product lies near 1 whatever the model's units; the scale comes back
// exactly in the exponent when a pair is written as a double.
//
// Per point first (lane = element, point): the scale exponents, the split
// tangent scalings and deviatoric direction, dvol * stress.  Then over the
// eight points (lane = element, node): the node's resisting-force terms in
// FP64, its split gradient at that point (element-major geo2), the
// projection h = n . dN/dx and the three scalings, staged in a 3.8 KB
// slice; then every lane adds the point's terms to the node-pair blocks it
// owns (144 per warp, 4.5 per lane), whose float-float sums sit in shared
// memory, transposed so that neighbouring lanes use neighbouring banks.  The
// task loop is a real loop: with the accumulators in registers its five
// unrolled copies made a 32 KB loop body that the warps' instruction
// fetches thrashed.
struct BrickSmemFF {
  float2 pt[kBrickEPW][8][9];         // per point: dvol*{a, b/2, c}*2^-ed, n[6] (split)
  double ss[kBrickEPW][8][6];         // per point: dvol * stress
  float2 nd[5][kBrickEPW][8][3];      // the point being summed: g h u v w per node
  float2 acc[9][kBrickEPW * 36];      // node-pair block sums (hi, lo), [entry][task]
  int eg[kBrickEPW], scale[kBrickEPW];
};

// f * 2^s in single precision from the bits: exact where the result is a
// normal number; below that range zero (under 2^-126 of the model's units,
// negligible against any stiffness term), above it infinity.
__device__ __forceinline__ float f32_ldexp(float f, int s) {
  const unsigned u = __float_as_uint(f);
  const int e8 = (int)((u >> 23) & 0xff);
  if (e8 == 0) return 0.0f;
  if (e8 == 255) return f;
  const int ne = e8 + s;
  if (ne <= 0) return 0.0f;
  if (ne >= 255) return __uint_as_float((u & 0x80000000u) | 0x7f800000u);
  return __uint_as_float((u & 0x807fffffu) | ((unsigned)ne << 23));
}

__global__ void __launch_bounds__(32 * kBrickWarps) k_brick_assemble_ff(ContinuumView v) {
  __shared__ BrickSmemFF sm_all[kBrickWarps];
  const int wi = threadIdx.x >> 5, lane = threadIdx.x & 31;
  BrickSmemFF &S = sm_all[wi];
  const int e0 = (blockIdx.x * kBrickWarps + wi) * kBrickEPW;
  if (e0 >= v.ne) return;
  const long npts = (long)v.ne * 8;
  constexpr int kTasks = kBrickEPW * 36;
  {
    const int el = lane >> 3, ip = lane & 7, e = e0 + el;
    const long pt = (long)(e < v.ne ? e : e0) * 8 + ip;
    int eg = -1000;
#pragma unroll
    for (int q = 0; q < 24; q++) eg = max(eg, f64_exponent(v.geo[q * npts + pt]));
    const double dvol = v.geo[24 * npts + pt];
#pragma unroll
    for (int c = 0; c < 6; c++) S.ss[el][ip][c] = dvol * v.sig[c * npts + pt];
    const double ca = v.tan[pt], cb = v.tan[npts + pt], cc = v.tan[2 * npts + pt];
    const double da = dvol * ca, dbh = dvol * (0.5 * cb), dc = dvol * cc;
    int ed = max(max(f64_exponent(da), f64_exponent(dbh)), f64_exponent(dc));
#pragma unroll
    for (int o = 1; o < 8; o <<= 1) {
      eg = max(eg, __shfl_xor_sync(0xffffffffu, eg, o));
      ed = max(ed, __shfl_xor_sync(0xffffffffu, ed, o));
    }
    if (eg < -126) eg = 0;      // all of dN/dx zero: a degenerate element
    if (ed < -1000) ed = 0;
    ed = min(ed, 1022);         // a non-finite scaling stays non-finite below
    if (ip == 0) {
      S.eg[el] = eg;
      S.scale[el] = 2 * eg + ed;
    }
    const double pd = __hiloint2double((int)((unsigned)(1023 - ed) << 20), 0);
    S.pt[el][ip][0] = split2(da * pd);
    S.pt[el][ip][1] = split2(dbh * pd);
    S.pt[el][ip][2] = split2(dc * pd);
#pragma unroll
    for (int c = 0; c < 6; c++) S.pt[el][ip][3 + c] = split2(v.tan[(3 + c) * npts + pt]);
    for (int t = lane; t < 9 * kTasks; t += 32) (&S.acc[0][0])[t] = make_float2(0.f, 0.f);
  }
  __syncwarp();
  const int el = lane >> 3, a = lane & 7, e = e0 + el;
  const bool live = e < v.ne;
  const long ebase = (long)(live ? e : e0) * 8;
  const float fg = __uint_as_float((unsigned)(127 - S.eg[el]) << 23);
  double r0 = 0.0, r1 = 0.0, r2 = 0.0;     // resisting force of node a
#pragma unroll 1
  for (int ip = 0; ip < 8; ip++) {
    {
      // node a of element el at point ip: resisting-force terms (FP64, the
      // points in order) and the staged float-float terms
      const double *Sg = S.ss[el][ip];
      const double g0 = v.geo[a * npts + ebase + ip];
      const double g1 = v.geo[(8 + a) * npts + ebase + ip];
      const double g2 = v.geo[(16 + a) * npts + ebase + ip];
      r0 += g0 * Sg[0] + g1 * Sg[3] + g2 * Sg[5];
      r1 += g0 * Sg[3] + g1 * Sg[1] + g2 * Sg[4];
      r2 += g0 * Sg[5] + g1 * Sg[4] + g2 * Sg[2];
      const float2 *gp = v.geo2 + (ebase + ip) * 24 + a;
      float2 gi[3];
#pragma unroll
      for (int i = 0; i < 3; i++) {
        const float2 q = gp[8 * i];
        gi[i] = make_float2(__fmul_rn(q.x, fg), __fmul_rn(q.y, fg));
      }
      const float2 *P = S.pt[el][ip];
      const int row[3][3] = {{0, 3, 5}, {3, 1, 4}, {5, 4, 2}};
#pragma unroll
      for (int i = 0; i < 3; i++) {
        float hh = 0.f, hl = 0.f;
#pragma unroll
        for (int j = 0; j < 3; j++) ff_madd(P[3 + row[i][j]], gi[j], hh, hl);
        const float hs = __fadd_rn(hh, hl);
        const float2 hi = make_float2(hs, __fsub_rn(hl, __fsub_rn(hs, hh)));
        S.nd[0][el][a][i] = gi[i];
        S.nd[1][el][a][i] = hi;
        S.nd[2][el][a][i] = ff_mul(P[0], gi[i]);
        S.nd[3][el][a][i] = ff_mul(P[1], gi[i]);
        S.nd[4][el][a][i] = ff_mul(P[2], hi);
      }
    }
    __syncwarp();
#pragma unroll 1
    for (int t = lane; t < kTasks; t += 32) {
      const int te = t / 36, pp = t % 36;
      if (e0 + te >= v.ne) continue;
      const int ta = kPairA[pp], tb = kPairB[pp];
      float2 gb[3], hb[3], ua[3], va[3], wa[3];
#pragma unroll
      for (int q = 0; q < 3; q++) {
        gb[q] = S.nd[0][te][tb][q];
        hb[q] = S.nd[1][te][tb][q];
        ua[q] = S.nd[2][te][ta][q];
        va[q] = S.nd[3][te][ta][q];
        wa[q] = S.nd[4][te][ta][q];
      }
      float ah[9], al[9];
#pragma unroll
      for (int q = 0; q < 9; q++) {
        const float2 c = S.acc[q][t];
        ah[q] = c.x;
        al[q] = c.y;
      }
      // (b/2) dvol dNa . dNb on the diagonal
      float dh = 0.f, dl = 0.f;
#pragma unroll
      for (int q = 0; q < 3; q++) ff_madd(va[q], gb[q], dh, dl);
#pragma unroll
      for (int i = 0; i < 3; i++) {
#pragma unroll
        for (int k = 0; k < 3; k++) {
          ff_madd(ua[i], gb[k], ah[3 * i + k], al[3 * i + k]);
          ff_madd(va[k], gb[i], ah[3 * i + k], al[3 * i + k]);
          ff_madd(wa[i], hb[k], ah[3 * i + k], al[3 * i + k]);
        }
        ff_add(dh, dl, ah[4 * i], al[4 * i]);
      }
#pragma unroll
      for (int q = 0; q < 9; q++) S.acc[q][t] = make_float2(ah[q], al[q]);
    }
    __syncwarp();   // the slice is restaged for the next point
  }
  if (live) {
    v.Re[(long)e * 24 + 3 * a] = r0;
    v.Re[(long)e * 24 + 3 * a + 1] = r1;
    v.Re[(long)e * 24 + 3 * a + 2] = r2;
  }
  for (int t = lane; t < kTasks; t += 32) {
    const int te = t / 36, pp = t % 36;
    if (e0 + te >= v.ne) continue;
    const int sc = S.scale[te];
    const int ta = kPairA[pp], tb = kPairB[pp];
    // the element matrix as float pairs in the model's units (the scale put
    // back into the exponents); the gather sums them in float-float
    float2 *Ke = reinterpret_cast<float2 *>(v.Ke) + (long)(e0 + te) * 576;
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int k = 0; k < 3; k++) {
        const float2 c = S.acc[3 * i + k][t];
        const float2 kv = make_float2(f32_ldexp(c.x, sc), f32_ldexp(c.y, sc));
        Ke[(3 * ta + i) * 24 + 3 * tb + k] = kv;
        if (ta != tb) Ke[(3 * tb + k) * 24 + 3 * ta + i] = kv;
      }
  }
}

// Zero-strain trial state (the material constructors call the integrator at
// zero strain, J2Plasticity.cpp:84-111): history zero, elastic tangent.
__global__ void k_j2_zero(ContinuumView v) {
  const long npts = (long)v.ne * v.nip;
  const long pt = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (pt >= npts) return;
  const int e = (int)(pt / v.nip);
  const double *p = v.j2 + (long)v.mat[e] * XG_J2_NPARAM;
  const int nh = v.nip == 4 ? 4 : 6;
  for (int c = 0; c < nh; c++) {
    const_cast<double *>(v.ep_c)[c * npts + pt] = 0.0;
    v.ep_t[c * npts + pt] = 0.0;
  }
  const_cast<double *>(v.xi_c)[pt] = 0.0;
  v.xi_t[pt] = 0.0;
  const double K = p[0], G = p[1];
  if (v.nip == 4) {
    for (int c = 0; c < 3; c++) v.sig[c * npts + pt] = 0.0;
    v.tan[pt] = j2_tangent_entry(K, G, 0.0, 0.0, 1.0, 2. / 3., 0.0);
    v.tan[npts + pt] = j2_tangent_entry(K, G, 0.0, 0.0, 1.0, -1. / 3., 0.0);
    v.tan[2 * npts + pt] = 0.0;
    v.tan[3 * npts + pt] = j2_tangent_entry(K, G, 0.0, 0.0, 1.0, 2. / 3., 0.0);
    v.tan[4 * npts + pt] = 0.0;
    v.tan[5 * npts + pt] = j2_tangent_entry(K, G, 0.0, 0.0, 0.0, 0.5, 0.0);
  } else {
    for (int c = 0; c < 6; c++) v.sig[c * npts + pt] = 0.0;
    const double b = 2.0 * G;
    v.tan[pt] = K - b / 3.0;
    v.tan[npts + pt] = b;
    v.tan[2 * npts + pt] = 0.0;
    for (int c = 0; c < 6; c++) v.tan[(3 + c) * npts + pt] = 0.0;
  }

}

// ---------------------------------------------------------------------------
// deterministic gather assembly
// ---------------------------------------------------------------------------
// Chunk sums in list order; a slot made of one chunk (every slot of a mesh
// whose nodes have few elements) is written to its output directly, the
// others leave partial sums for k_gather_slots.  The same additions in the
// same order either way.
template <typename Idx>
__global__ void k_gather_chunks(GatherMap g, const Idx *__restrict__ src,
                                const double *__restrict__ scratch, double *__restrict__ partial,
                                double *__restrict__ out) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= g.nchunks) return;
  double s = 0.0;
  const int64_t b = g.chunk_begin[c], end = g.chunk_begin[c + 1];
  for (int64_t k = b; k < end; k++) s += scratch[src[k]];
  const int slot = g.chunk_slot[c];
  if (g.slot_chunk[slot + 1] - g.slot_chunk[slot] == 1) out[slot] = s;
  else partial[c] = s;
}

// One run of L slots: its slots summed in contribution order (the element
// order, as the chunks sum), each contribution's values read as one
// contiguous piece.
// The same over float pairs (the float-float brick tangent), summed in
// float-float; one double per slot.
template <int L>
__device__ __forceinline__ void gather_run_pairs(const int *src, int n, const float2 *scratch,
                                                 double *out) {
  float ah[L], al[L];
#pragma unroll
  for (int t = 0; t < L; t++) ah[t] = al[t] = 0.f;
  int q = 0;
  for (; q + 4 <= n; q += 4) {
    const unsigned a0 = (unsigned)src[q], a1 = (unsigned)src[q + 1];
    const unsigned a2 = (unsigned)src[q + 2], a3 = (unsigned)src[q + 3];
    float2 v[4][L];
#pragma unroll
    for (int t = 0; t < L; t++) {
      v[0][t] = scratch[a0 + t];
      v[1][t] = scratch[a1 + t];
      v[2][t] = scratch[a2 + t];
      v[3][t] = scratch[a3 + t];
    }
#pragma unroll
    for (int u = 0; u < 4; u++)
#pragma unroll
      for (int t = 0; t < L; t++) ff_add(v[u][t].x, v[u][t].y, ah[t], al[t]);
  }
  for (; q < n; q++) {
    const float2 *p = scratch + (unsigned)src[q];
#pragma unroll
    for (int t = 0; t < L; t++) ff_add(p[t].x, p[t].y, ah[t], al[t]);
  }
#pragma unroll
  for (int t = 0; t < L; t++) out[t] = f32_to_f64_scaled(ah[t], 0) + f32_to_f64_scaled(al[t], 0);
}

template <int L>
__device__ __forceinline__ void gather_run(const int *src, int n, const double *scratch,
                                           double *out) {
  double acc[L];
#pragma unroll
  for (int t = 0; t < L; t++) acc[t] = 0.0;
  int q = 0;
  // four contributions' loads in flight, added in their order
  for (; q + 4 <= n; q += 4) {
    const unsigned a0 = (unsigned)src[q], a1 = (unsigned)src[q + 1];
    const unsigned a2 = (unsigned)src[q + 2], a3 = (unsigned)src[q + 3];
    double v[4][L];
#pragma unroll
    for (int t = 0; t < L; t++) {
      v[0][t] = scratch[a0 + t];
      v[1][t] = scratch[a1 + t];
      v[2][t] = scratch[a2 + t];
      v[3][t] = scratch[a3 + t];
    }
#pragma unroll
    for (int u = 0; u < 4; u++)
#pragma unroll
      for (int t = 0; t < L; t++) acc[t] += v[u][t];
  }
  for (; q < n; q++) {
    const double *p = scratch + (unsigned)src[q];
#pragma unroll
    for (int t = 0; t < L; t++) acc[t] += p[t];
  }
#pragma unroll
  for (int t = 0; t < L; t++) out[t] = acc[t];
}

// Thread per run.  The runs are ordered by length and contribution count, so
// a warp's threads take the same branch and loop as often: the FP64 adds,
// which hold the FP64 pipe per warp instruction whatever its active lanes,
// are then issued once per useful add.
template <bool kPairs>
__global__ void k_gather_runs(GatherMap g, const double *__restrict__ scratch,
                              double *__restrict__ out) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= g.nruns) return;
  const int s0 = g.run_slot[r], meta = g.run_meta[r];
  const int len = meta & 15, n = meta >> 4;
  const int *src = g.run_src + g.run_begin[r];
  if (kPairs) {
    const float2 *sp = reinterpret_cast<const float2 *>(scratch);
    switch (len) {
      case 1: gather_run_pairs<1>(src, n, sp, out + s0); break;
      case 2: gather_run_pairs<2>(src, n, sp, out + s0); break;
      case 3: gather_run_pairs<3>(src, n, sp, out + s0); break;
      case 4: gather_run_pairs<4>(src, n, sp, out + s0); break;
      case 5: gather_run_pairs<5>(src, n, sp, out + s0); break;
      default: gather_run_pairs<6>(src, n, sp, out + s0); break;
    }
    return;
  }
  switch (len) {
    case 1: gather_run<1>(src, n, scratch, out + s0); break;
    case 2: gather_run<2>(src, n, scratch, out + s0); break;
    case 3: gather_run<3>(src, n, scratch, out + s0); break;
    case 4: gather_run<4>(src, n, scratch, out + s0); break;
    case 5: gather_run<5>(src, n, scratch, out + s0); break;
    default: gather_run<6>(src, n, scratch, out + s0); break;
  }
}

// The chunk and slot kernels over a list of chunks / slots (the long slots
// of a map with runs), or over all of them when the list is null.
template <typename Idx, bool kPairs>
__global__ void k_gather_chunk_list(GatherMap g, const Idx *__restrict__ src,
                                    const double *__restrict__ scratch,
                                    double *__restrict__ partial, double *__restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= g.nlong_chunks) return;
  const int c = g.long_chunks[i];
  double s = 0.0;
  const int64_t b = g.chunk_begin[c], end = g.chunk_begin[c + 1];
  if (kPairs) {
    const float2 *sp = reinterpret_cast<const float2 *>(scratch);
    for (int64_t k = b; k < end; k++) {
      const float2 v = sp[src[k]];
      s += (double)v.x + (double)v.y;
    }
  } else {
    for (int64_t k = b; k < end; k++) s += scratch[src[k]];
  }
  const int slot = g.chunk_slot[c];
  if (g.slot_chunk[slot + 1] - g.slot_chunk[slot] == 1) out[slot] = s;
  else partial[c] = s;
}

// Warp per long slot: its chunk partials lane-strided in chunk order, then a
// fixed butterfly (the multi-point constraint's retained slots have
// thousands of chunks).
__global__ void k_gather_slot_list(GatherMap g, const double *__restrict__ partial,
                                   double *__restrict__ out) {
  const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (w >= g.nlong_slots) return;
  const int s = g.long_slots[w];
  const int c0 = g.slot_chunk[s], c1 = g.slot_chunk[s + 1];
  if (c1 - c0 == 1) return;               // written by its chunk
  double v = 0.0;
  for (int c = c0 + lane; c < c1; c += 32) v += partial[c];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if (lane == 0) out[s] = v;
}

__global__ void k_gather_slots(GatherMap g, const double *__restrict__ partial,
                               double *__restrict__ out) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= g.nslots) return;
  const int c0 = g.slot_chunk[s], c1 = g.slot_chunk[s + 1];
  if (c1 - c0 == 1) return;               // written by its chunk
  double v = 0.0;
  for (int c = c0; c < c1; c++) v += partial[c];
  out[s] = v;
}

// ---------------------------------------------------------------------------
// recorders (recorder/NodeRecorder.cpp:180-476, EnvelopeNodeRecorder.cpp:
// 191-470): one committed step's selected nodal values, gathered on the
// device
// ---------------------------------------------------------------------------
// row = [time] v_0 .. v_n-1, v_i = src[idx[i]] (0 where the dof does not exist)
__global__ void k_record_row(int n, const int *idx, const double *src, double t, int echo,
                             double *row) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (echo && i == 0) row[0] = t;
  if (i < n) row[echo + i] = idx[i] >= 0 ? src[idx[i]] : 0.0;
}

// Envelope [3][ncol]: rows min, max, max |.|; with echo every value has its
// time in the column before it.  The first record sets all three, later
// records update the minimum, else the maximum, and then the absolute value
// (EnvelopeNodeRecorder.cpp:401-468).
__global__ void k_record_envelope(int n, const int *idx, const double *src, double t, int echo,
                                  int first, double *env) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double v = idx[i] >= 0 ? src[idx[i]] : 0.0;
  const int w = echo ? 2 : 1, ncol = n * w, c = i * w + (echo ? 1 : 0);
  double *mn = env, *mx = env + ncol, *ab = env + 2 * ncol;
  if (first) {
    mn[c] = v;
    mx[c] = v;
    ab[c] = fabs(v);
    if (echo) mn[c - 1] = mx[c - 1] = ab[c - 1] = t;
    return;
  }
  bool moved = false;
  if (mn[c] > v) {
    mn[c] = v;
    if (echo) mn[c - 1] = t;
    moved = true;
  } else if (mx[c] < v) {
    mx[c] = v;
    if (echo) mx[c - 1] = t;
    moved = true;
  }
  if (moved && ab[c] < fabs(v)) {
    ab[c] = fabs(v);
    if (echo) ab[c - 1] = t;
  }
}

// ---------------------------------------------------------------------------
// vector helpers
// ---------------------------------------------------------------------------
__global__ void k_axpy(int n, double a, const double *x, double *y) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] += a * x[i];
}

__global__ void k_scatter_incr(int nu, const int *eqn, const double *dU, double f, double *U) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nu) return;
  const int e = eqn[i];
  if (e >= 0) U[i] += f * dU[e];
}

// TransformationDOF_Group::enforceSPs: U[idx[k]] = lam[pat[k]] * val[k]
__global__ void k_enforce_sps(int n, const int *idx, const int *pat, const double *val,
                              SpFactors lam, double *U) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) U[idx[k]] = lam.f[pat[k]] * val[k];
}

__global__ void k_sub(int n, const double *a, const double *b, double *out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = a[i] - b[i];
}

__device__ double block_sum(double v) {
  __shared__ double wsum[32];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) wsum[w] = v;
  __syncthreads();
  double t = 0.0;
  if (w == 0) {
    t = (lane < (int)(blockDim.x >> 5)) ? wsum[lane] : 0.0;
    for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
  }
  return t;  // valid in thread 0
}

__global__ void k_norm2_partial(int n, const double *x, double *partials) {
  double s = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    s += x[i] * x[i];
  s = block_sum(s);
  if (threadIdx.x == 0) partials[blockIdx.x] = s;
}

__global__ void k_norm2_final(int nb, const double *partials, double *out) {
  double s = 0.0;
  for (int i = threadIdx.x; i < nb; i += blockDim.x) s += partials[i];
  s = block_sum(s);
  if (threadIdx.x == 0) *out = s;
}

inline int check_launch() {
  return cudaGetLastError() == cudaSuccess ? 0 : XG_ECUDA;
}

}  // namespace

int launch_quad_update(const ContinuumView &v, cudaStream_t s) {
  if (v.ne == 0) return 0;
  k_quad_update<<<nblocks((long)v.ne * 4), kThreads, 0, s>>>(v);
  return check_launch();
}
int launch_quad_assemble(const ContinuumView &v, cudaStream_t s) {
  if (v.ne == 0) return 0;
  k_quad_assemble<<<nblocks(v.ne, 128), 128, 0, s>>>(v);
  return check_launch();
}
int launch_brick_update(const ContinuumView &v, cudaStream_t s) {
  if (v.ne == 0) return 0;
  k_brick_update<<<nblocks((long)v.ne * 8), kThreads, 0, s>>>(v);
  return check_launch();
}
int launch_brick_geometry(const ContinuumView &v, double *geo, float2 *geo2, int *bad,
                          cudaStream_t s) {
  if (v.ne == 0) return 0;
  k_brick_geometry<<<nblocks((long)v.ne * 8), kThreads, 0, s>>>(v, geo, geo2, bad);
  return check_launch();
}
int launch_brick_assemble(const ContinuumView &v, cudaStream_t s) {
  if (v.ne == 0) return 0;
  constexpr int per_block = kBrickWarps * kBrickEPW;
  if (v.geo && v.geo2)
    k_brick_assemble_ff<<<(v.ne + per_block - 1) / per_block, 32 * kBrickWarps, 0, s>>>(v);
  else
    k_brick_assemble<<<(v.ne + per_block - 1) / per_block, 32 * kBrickWarps, 0, s>>>(v);
  return check_launch();
}
int launch_j2_zero_state(const ContinuumView &v, cudaStream_t s) {
  if (v.ne == 0) return 0;
  k_j2_zero<<<nblocks((long)v.ne * v.nip), kThreads, 0, s>>>(v);
  return check_launch();
}
int gather_launch_count(const GatherMap &g, bool pairs) {
  if (pairs && !(g.run_slot && g.src32)) return 0;
  if (g.nslots == 0) return 0;
  if (g.run_slot && g.src32) return (g.nruns > 0) + (g.nlong_chunks > 0) + (g.nlong_slots > 0);
  return 2;
}
int launch_gather(const GatherMap &g, const double *scratch, double *partial, double *out,
                  cudaStream_t s, bool pairs) {
  if (g.nslots == 0) return 0;
  if (pairs && !(g.run_slot && g.src32)) return XG_EINVAL;   // pairs need the run map
  if (g.run_slot && g.src32) {
    if (g.nruns) {
      if (pairs) k_gather_runs<true><<<nblocks(g.nruns), kThreads, 0, s>>>(g, scratch, out);
      else k_gather_runs<false><<<nblocks(g.nruns), kThreads, 0, s>>>(g, scratch, out);
    }
    if (g.nlong_chunks) {
      if (pairs)
        k_gather_chunk_list<int, true><<<nblocks(g.nlong_chunks), kThreads, 0, s>>>(
            g, g.src32, scratch, partial, out);
      else
        k_gather_chunk_list<int, false><<<nblocks(g.nlong_chunks), kThreads, 0, s>>>(
            g, g.src32, scratch, partial, out);
    }
    if (g.nlong_slots)
      k_gather_slot_list<<<nblocks(32L * g.nlong_slots), kThreads, 0, s>>>(g, partial, out);
    return check_launch();
  }
  if (g.src32)
    k_gather_chunks<int><<<nblocks(g.nchunks), kThreads, 0, s>>>(g, g.src32, scratch, partial, out);
  else
    k_gather_chunks<int64_t><<<nblocks(g.nchunks), kThreads, 0, s>>>(g, g.src, scratch, partial,
                                                                      out);
  k_gather_slots<<<nblocks(g.nslots), kThreads, 0, s>>>(g, partial, out);
  return check_launch();
}
int launch_record(int kind, int n, const int *idx, const double *src, double t, int echo,
                  int first, double *out, cudaStream_t s) {
  if (n == 0 && !echo) return 0;
  const int nb = (std::max(n, 1) + kThreads - 1) / kThreads;
  if (kind == 0) k_record_row<<<nb, kThreads, 0, s>>>(n, idx, src, t, echo, out);
  else k_record_envelope<<<nb, kThreads, 0, s>>>(n, idx, src, t, echo, first, out);
  return check_launch();
}
int launch_axpy(int n, double a, const double *x, double *y, cudaStream_t s) {
  if (n == 0) return 0;
  k_axpy<<<nblocks(n), kThreads, 0, s>>>(n, a, x, y);
  return check_launch();
}
int launch_scatter_incr(int nu, const int *eqn, const double *dU, double f, double *U,
                        cudaStream_t s) {
  if (nu == 0) return 0;
  k_scatter_incr<<<nblocks(nu), kThreads, 0, s>>>(nu, eqn, dU, f, U);
  return check_launch();
}
int launch_enforce_sps(int n, const int *idx, const int *pat, const double *val,
                       const SpFactors &lam, double *U, cudaStream_t s) {
  if (n == 0) return 0;
  k_enforce_sps<<<nblocks(n), kThreads, 0, s>>>(n, idx, pat, val, lam, U);
  return check_launch();
}
int launch_sub(int n, const double *a, const double *b, double *out, cudaStream_t s) {
  if (n == 0) return 0;
  k_sub<<<nblocks(n), kThreads, 0, s>>>(n, a, b, out);
  return check_launch();
}
int launch_norm2(int n, const double *x, double *partials, double *out, cudaStream_t s) {
  int nb = nblocks(n);
  if (nb > 1024) nb = 1024;
  if (nb < 1) nb = 1;
  k_norm2_partial<<<nb, kThreads, 0, s>>>(n, x, partials);
  k_norm2_final<<<1, 1024, 0, s>>>(nb, partials, out);
  return check_launch();
}

}  // namespace xg

// ---------------------------------------------------------------------------
// FP64 peak probe: independent FMA chains, no memory traffic.  Used to put
// the element kernels' FP64 rate next to what this GPU delivers.
// ---------------------------------------------------------------------------
namespace xg {
namespace {
__global__ void k_fp64_fma(double *out, int iters) {
  double a0 = threadIdx.x * 1e-9, a1 = a0 + 1e-9, a2 = a0 + 2e-9, a3 = a0 + 3e-9;
  double a4 = a0 + 4e-9, a5 = a0 + 5e-9, a6 = a0 + 6e-9, a7 = a0 + 7e-9;
  const double m = 0.999999999, c = 1e-12;
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int k = 0; k < 8; k++) {
      a0 = fma(a0, m, c); a1 = fma(a1, m, c); a2 = fma(a2, m, c); a3 = fma(a3, m, c);
      a4 = fma(a4, m, c); a5 = fma(a5, m, c); a6 = fma(a6, m, c); a7 = fma(a7, m, c);
    }
  }
  const double s = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
  if (s == 12345.678) out[blockIdx.x] = s;  // keeps the chains live
}
}  // namespace
}  // namespace xg

extern "C" int xg_measure_fp64_peak(double *tflops) {
  if (!tflops) return XG_EINVAL;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  double *out = nullptr;
  if (cudaMalloc(&out, sizeof(double) * 4096) != cudaSuccess) return XG_ENOMEM;
  const int blocks = sms * 8, threads = 256, iters = 4096;
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  xg::k_fp64_fma<<<blocks, threads>>>(out, 64);  // warm up
  cudaEventRecord(a);
  xg::k_fp64_fma<<<blocks, threads>>>(out, iters);
  cudaEventRecord(b);
  cudaEventSynchronize(b);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaFree(out);
  if (cudaGetLastError() != cudaSuccess || ms <= 0.f) return XG_ECUDA;
  const double flops = 2.0 * 64.0 * (double)iters * blocks * threads;
  *tflops = flops / (ms * 1e-3) / 1e12;
  return 0;
}

// ---------------------------------------------------------------------------
// The LDL' kernels' pivot-chain reciprocal next to the correctly rounded one,
// for its error bound test.
// ---------------------------------------------------------------------------
namespace xg {
namespace {
__global__ void k_reciprocal_pair(int n, const double *d, double *y, double *y_rn) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  y[i] = chain_reciprocal(d[i]);
  y_rn[i] = __drcp_rn(d[i]);
}
}  // namespace
}  // namespace xg

extern "C" int xg_chain_reciprocal_check(int n, const double *d, double *y, double *y_rn) {
  if (n < 0 || (n > 0 && (!d || !y || !y_rn))) return XG_EINVAL;
  if (n == 0) return 0;
  double *buf = nullptr;
  const size_t bytes = sizeof(double) * (size_t)n;
  if (cudaMalloc(&buf, 3 * bytes) != cudaSuccess) return XG_ENOMEM;
  int rc = 0;
  if (cudaMemcpy(buf, d, bytes, cudaMemcpyHostToDevice) != cudaSuccess) rc = XG_ECUDA;
  if (!rc) {
    xg::k_reciprocal_pair<<<(n + 255) / 256, 256>>>(n, buf, buf + n, buf + 2 * (size_t)n);
    if (cudaGetLastError() != cudaSuccess ||
        cudaMemcpy(y, buf + n, bytes, cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(y_rn, buf + 2 * (size_t)n, bytes, cudaMemcpyDeviceToHost) != cudaSuccess)
      rc = XG_ECUDA;
  }
  cudaFree(buf);
  return rc;
}
