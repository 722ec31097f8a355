// xg_adjoint.cu -- reverse sweep of a Newmark run of force-based frames:
// the discrete adjoint of the converged step sequence with respect to the
// uniaxial materials' first three parameters (Steel02: Fy, E0, b).
//
// A converged step n satisfies R(U_n; U', V', A', h', theta) = 0 (the
// dynamic unbalance of Newmark.cpp:262-302 with the resisting force of
// ForceBeamColumn2d/3d::update at the committed fiber records h'), and
// commits the fiber records h_n = H(eps(U_n), h', theta).  Its adjoint, with
// J the exact effective tangent -dR/dU_n:
//   J' mu = Ubar_n + c2 Vbar_n + c3 Abar_n + (dh_n/dU_n)' hbar_n
// Under linear transformations J is the symmetric tangent the forward step
// factors; the 2D P-Delta transformation's tangent leaves out one
// non-symmetric term per element (k_adj_pdelta), which the host carries by a
// fixed-point iteration on the factored tangent.
//   hbar' = (dh_n/dh')' hbar_n - (dP/dh')' mu,   thetabar += the same in theta
// plus the Newmark predictor's terms for (U', V', A').  Inside an element the
// converged compatibility state (basic forces Se, section deformations e_s)
// is an implicit function of the basic deformations v, h' and theta:
//   dSe  = kv (dv + sum_s w_s b_s' fs_s q_s),   de_s = fs_s (b_s dSe - q_s),
//   q_s  = sum_f A_f a_f dsigma_f (strain fixed),  a_f = (1, -y [, z])
// so one reverse pass over an element needs the section flexibilities fs_s,
// kv and e_s of the converged state and two vector-Jacobian products of the
// fiber law: one with the records' adjoint (giving the strain adjoint that
// flows into e_s) and one with the stress adjoint the section equations
// pass down.
#include <cuda_runtime.h>

#include "xg_internal.h"
#include "xg_uniaxial_adj.h"

namespace xg {

namespace {

constexpr int kAdjWarps = 4;

__device__ __forceinline__ double warp_sum_adj(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ int stride_of(int nip) { return 6 + 36 + nip * 24 + 6 + 1; }

// kv0 = f0^-1: Gauss-Jordan with partial pivoting; in 3D the torsion row and
// column are uncoupled, so the 5x5 block is inverted and kv0(5,5) = 1/f0(5,5)
template <int NB>
__device__ void small_inverse(const double *f, double *kv) {
  constexpr int N = NB == 3 ? 3 : 5;
  double M[N][2 * N];
  for (int i = 0; i < N; i++)
    for (int j = 0; j < 2 * N; j++) M[i][j] = j < N ? f[i * NB + j] : (j - N == i ? 1.0 : 0.0);
  for (int c = 0; c < N; c++) {
    int piv = c;
    for (int i = c + 1; i < N; i++)
      if (fabs(M[i][c]) > fabs(M[piv][c])) piv = i;
    if (piv != c)
      for (int j = 0; j < 2 * N; j++) { const double t = M[c][j]; M[c][j] = M[piv][j]; M[piv][j] = t; }
    const double inv = 1.0 / M[c][c];
    for (int j = 0; j < 2 * N; j++) M[c][j] *= inv;
    for (int i = 0; i < N; i++) {
      if (i == c) continue;
      const double m = M[i][c];
      for (int j = 0; j < 2 * N; j++) M[i][j] -= m * M[c][j];
    }
  }
  for (int i = 0; i < NB * NB; i++) kv[i] = 0.0;
  for (int i = 0; i < N; i++)
    for (int j = 0; j < N; j++) kv[i * NB + j] = M[i][N + j];
  if (NB == 6) kv[35] = 1.0 / f[35];
}

// basic <- global transformation of a linear frame transformation
// (LinearCrdTransf2d.cpp:248-299, BasicFrameTransf.cpp:90-104)
template <int NB>
__device__ void basic_T(const FrameView &v, int e, double (*T)[NB == 3 ? 6 : 12]) {
  constexpr int NU = NB == 3 ? 6 : 12;
  const double L = v.L[e];
  const double *R = v.R + 9 * (long)e;
#pragma unroll
  for (int i = 0; i < NB; i++)
#pragma unroll
    for (int j = 0; j < NU; j++) T[i][j] = 0.0;
  if (NB == 3) {
    const double cs = R[0], sn = R[1], sl = sn / L, cl = cs / L;
    T[0][0] = -cs; T[0][1] = -sn; T[0][3] = cs; T[0][4] = sn;
    T[1][0] = -sl; T[1][1] = cl; T[1][2] = 1.0; T[1][3] = sl; T[1][4] = -cl;
    T[2][0] = -sl; T[2][1] = cl; T[2][3] = sl; T[2][4] = -cl; T[2][5] = 1.0;
  } else {
#pragma unroll
    for (int j = 0; j < 3; j++) {
      const double e1 = R[3 * j + 0], e2 = R[3 * j + 1], e3 = R[3 * j + 2];
      T[0][0 + j] = -e1; T[0][6 + j] = e1;
      T[1][3 + j] = e3; T[1][0 + j] = e2 / L; T[1][6 + j] = -e2 / L;
      T[2][9 + j] = e3; T[2][0 + j] = e2 / L; T[2][6 + j] = -e2 / L;
      T[3][3 + j] = e2; T[3][0 + j] = -e3 / L; T[3][6 + j] = e3 / L;
      T[4][9 + j] = e2; T[4][0 + j] = -e3 / L; T[4][6 + j] = e3 / L;
      T[5][3 + j] = -e1; T[5][9 + j] = e1;
    }
  }
}

// PDeltaCrdTransf2d (coordTransformation/PDeltaCrdTransf2d.cpp:508-560) adds
// (Se_0 / L) ul14 g to the global force, g = [-s c 0 s -c 0] and ul14 = g . u
// the chord's transverse offset at the trial displacements
__device__ __forceinline__ double pdelta_ul14(const FrameView &v, int e) {
  const double cs = v.R[9 * (long)e], sn = v.R[9 * (long)e + 1];
  const double *uI = v.U + (long)v.conn[2 * e] * v.ndf, *uJ = v.U + (long)v.conn[2 * e + 1] * v.ndf;
  return (-sn * uI[0] + cs * uI[1]) - (-sn * uJ[0] + cs * uJ[1]);
}
__device__ __forceinline__ double pdelta_g_dot(const FrameView &v, int e, const double *x) {
  const double cs = v.R[9 * (long)e], sn = v.R[9 * (long)e + 1];
  return -sn * x[0] + cs * x[1] + sn * x[3] - cs * x[4];
}

// Sum over the G lanes of a section's lane group (lanes ip*G .. ip*G+G-1; a
// fixed tree: rank r adds rank r+o, o = P2/2 .. 1), broadcast from the
// group's first lane.
__device__ __forceinline__ double group_sum_adj(double v, int rank, int G, int P2) {
  for (int o = P2 >> 1; o > 0; o >>= 1) {
    const double t = __shfl_down_sync(0xffffffffu, v, o);
    if (rank + o < G) v += t;
  }
  return __shfl_sync(0xffffffffu, v, (int)(threadIdx.x & 31) - rank);
}

constexpr int kAdjMaxIp = 10;

// tq[slot] += qb, slot known only at run time (no dynamic register indexing)
__device__ __forceinline__ void add_slot(double (&tq)[kAdjSlots][3], int slot, const double *qb) {
#pragma unroll
  for (int m = 0; m < kAdjSlots; m++)
    if (slot == m) {
      tq[m][0] += qb[0];
      tq[m][1] += qb[1];
      tq[m][2] += qb[2];
    }
}

// warp sums of tq, added to the element's slots by lane 0
__device__ __forceinline__ void theta_add(const AdjView &a, int e, int lane,
                                          double (&tq)[kAdjSlots][3]) {
#pragma unroll
  for (int m = 0; m < kAdjSlots; m++)
#pragma unroll
    for (int k = 0; k < 3; k++) {
      const double t = warp_sum_adj(tq[m][k]);
      if (lane == 0) a.theta[(3L * kAdjSlots) * e + 3 * m + k] += t;
    }
}

__device__ __forceinline__ void fiber_vjp(int type, const double *q, const double *hc,
                                          double strain, const double *yb, double *hb,
                                          double *sb, double *qb) {
  if (type == XG_UNI_STEEL02) steel02_vjp(q, hc, strain, yb, hb, sb, qb);
  else if (type == XG_UNI_CONCRETE02) concrete02_vjp(q, hc, strain, yb, hb, sb, qb);
  else if (type == XG_UNI_STEEL01) steel01_vjp(q, hc, strain, yb, hb, sb, qb);
  else if (type == XG_UNI_CONCRETE01) concrete01_vjp(q, hc, strain, yb, hb, sb, qb);
  else elastic_vjp(q, strain, yb, hb, sb, qb);
}

// Pass A (warp per element): every fiber's record adjoint through the law
// gives the adjoint of the committed record (in place), of the parameters,
// and of the fiber strain; the strain adjoints reduce to ebar_s per section,
// which the element equations turn into the adjoint of the basic
// deformations z = kv sum_s b_s' fs_s ebar_s and, through T', of the
// element's global displacements (written to the element force scratch).
template <int NB, int ORD>
__global__ void __launch_bounds__(32 * kAdjWarps) k_adj_elem_a(FrameView v, AdjView a) {
  constexpr int NU = NB == 3 ? 6 : 12;
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int e = blockIdx.x * kAdjWarps + w;
  if (e >= v.ne) return;
  const int nip = v.nip;
  const double *st = a.st + (long)e * stride_of(nip);
  const int sec = v.sec[e];
  const int f0 = v.sec_fstart[sec], nf = v.sec_fstart[sec + 1] - f0;
  const double ybar = v.ybar[sec], zbar = ORD == 4 ? v.zbar[sec] : 0.0;
  const long fbase = v.foff[e];
  double *scr = a.scr + (long)e * (6 + nip * 4);
  double tq[kAdjSlots][3] = {};
  __shared__ double tsec_all[kAdjWarps][kAdjMaxIp][4];
  double(*tsec)[4] = tsec_all[w];
  constexpr int kRow[6] = {0, 1, 1, 2, 2, 3};
  // every section at once, a group of G lanes each (the forward kernel's
  // layout); lanes past the last group take no fiber
  const int G = 32 / nip;
  int P2 = 1;
  while (P2 < G) P2 <<= 1;
  const int gip = lane / G, rank = lane % G;
  const bool on = gip < nip;
  {
    const int ip = on ? gip : nip - 1;
    double vsec[ORD];
#pragma unroll
    for (int r = 0; r < ORD; r++) vsec[r] = st[42 + ip * 4 + r];
    double eb0 = 0.0, eb1 = 0.0, eb2 = 0.0;
    const long rec0 = (fbase + (long)ip * nf) * 12;
    for (int fi = rank; on && fi < nf; fi += G) {
      const int kf = f0 + fi;
      const double y = v.fy[kf] - ybar;
      double strain = vsec[0] - y * vsec[1];
      double z = 0.0;
      if (ORD == 4) {
        z = v.fz[kf] - zbar;
        strain += z * vsec[2];
      }
      const int u = v.fmat[kf];
      const double *q = v.uparam + (long)u * XG_UNI_NPARAM;
      const double *hcp = a.fh_prev + rec0 + 12L * fi;
      double *hbr = a.hbar + rec0 + 12L * fi;
      double hc[12], yb[12], hb[12], sb, qb[3];
#pragma unroll
      for (int k = 0; k < 12; k++) { hc[k] = hcp[k]; yb[k] = hbr[k]; }
      fiber_vjp(v.utype[u], q, hc, strain, yb, hb, &sb, qb);
#pragma unroll
      for (int k = 0; k < 12; k++) hbr[k] = hb[k];
      add_slot(tq, a.fslot[kf], qb);
      eb0 += sb;
      eb1 += -y * sb;
      if (ORD == 4) eb2 += z * sb;
    }
    double eb[ORD];
    eb[0] = group_sum_adj(eb0, rank, G, P2);
    eb[1] = group_sum_adj(eb1, rank, G, P2);
    if (ORD == 4) { eb[2] = group_sum_adj(eb2, rank, G, P2); eb[3] = 0.0; }
    if (on && rank == 0) {
#pragma unroll
      for (int r = 0; r < ORD; r++) scr[6 + ip * 4 + r] = eb[r];
      const double *fs = st + 42 + nip * 4 + ip * 16;
#pragma unroll
      for (int r = 0; r < ORD; r++) {
        double t = 0.0;
#pragma unroll
        for (int k = 0; k < ORD; k++) t += fs[r * ORD + k] * eb[k];
        tsec[ip][r] = t;
      }
    }
  }
  __syncwarp();
  // Sb = sum over the sections, in section order, of b_s' t_s
  double Sb[NB];
#pragma unroll
  for (int i = 0; i < NB; i++) Sb[i] = 0.0;
  for (int ip = 0; ip < nip; ip++) {
    const double xL = v.xi[ip], xL1 = xL - 1.0;
    const double ca[6] = {1.0, xL1, xL, xL1, xL, 1.0};
#pragma unroll
    for (int c = 0; c < NB; c++) Sb[c] += ca[c] * tsec[ip][kRow[c]];
  }
  const double *kv = st + 6;
  double zA[NB];
#pragma unroll
  for (int i = 0; i < NB; i++) {
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < NB; k++) s += kv[i * NB + k] * Sb[k];
    zA[i] = s;
  }
  theta_add(a, e, lane, tq);
  if (lane == 0) {
    double T[NB][NU];
    basic_T<NB>(v, e, T);
    double *ue = v.Re + (long)e * NU;
#pragma unroll
    for (int j = 0; j < NU; j++) {
      double s = 0.0;
#pragma unroll
      for (int k = 0; k < NB; k++) s += T[k][j] * zA[k];
      ue[j] = s;
    }
#pragma unroll
    for (int i = 0; i < NB; i++) scr[i] = zA[i];
  }
}

// Pass B (warp per element), after the adjoint solve: the basic-force
// adjoint -(dP/dSe)' mu_e (-T mu_e, and under the 2D P-Delta
// transformation -(ul14 / L)(g . mu_e) more in the axial force) and pass A's
// terms give the section adjoints
// qbar_s = w_s fs_s b_s z - fs_s ebar_s; each fiber's stress adjoint
// A_f a_f . qbar_s goes through the law into the committed record's and the
// parameters' adjoints.  The betaK0 K0 damping adds -betaK0/E (T mu)' kv0
// (T V_n) to the element material's modulus (K0 is linear in it).
template <int NB, int ORD>
__global__ void __launch_bounds__(32 * kAdjWarps) k_adj_elem_b(FrameView v, AdjView a) {
  constexpr int NU = NB == 3 ? 6 : 12;
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int e = blockIdx.x * kAdjWarps + w;
  if (e >= v.ne) return;
  const int nip = v.nip, ndf = v.ndf;
  const double *st = a.st + (long)e * stride_of(nip);
  const int sec = v.sec[e];
  const int f0 = v.sec_fstart[sec], nf = v.sec_fstart[sec + 1] - f0;
  const double ybar = v.ybar[sec], zbar = ORD == 4 ? v.zbar[sec] : 0.0;
  const double L = v.L[e];
  const long fbase = v.foff[e];
  const double *scr = a.scr + (long)e * (6 + nip * 4);
  double T[NB][NU];
  basic_T<NB>(v, e, T);
  double mue[NU], ve[NU];
  const int nd = NU / 2;
#pragma unroll
  for (int j = 0; j < NU; j++) {
    const int node = v.conn[2 * e + j / nd];
    const long dof = (long)node * ndf + (j % nd);
    const int eq = a.eqn[dof];
    mue[j] = eq >= 0 ? a.mu[eq] : 0.0;
    ve[j] = a.Vn ? a.Vn[dof] : 0.0;
  }
  const double *kv = st + 6;
  double pb[NB], pq[NB], z[NB];
#pragma unroll
  for (int i = 0; i < NB; i++) {
    double s = 0.0;
#pragma unroll
    for (int j = 0; j < NU; j++) s += T[i][j] * mue[j];
    pb[i] = s;                         // T mu_e
    pq[i] = s;                         // (dP/dSe)' mu_e; the basic-force adjoint is -pq
  }
  if (NB == 3 && v.pdelta2d) pq[0] += pdelta_ul14(v, e) / L * pdelta_g_dot(v, e, mue);
#pragma unroll
  for (int i = 0; i < NB; i++) {
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < NB; k++) s -= kv[i * NB + k] * pq[k];
    z[i] = scr[i] + s;
  }
  double tq[kAdjSlots][3] = {};
  constexpr int kRow[6] = {0, 1, 1, 2, 2, 3};
  // every section at once, a group of G lanes each
  const int G = 32 / nip;
  const int gip = lane / G, rank = lane % G;
  const bool on = gip < nip;
  if (on) {
    const int ip = gip;
    const double xL = v.xi[ip], xL1 = xL - 1.0, wtL = v.wt[ip] * L;
    const double ca[6] = {1.0, xL1, xL, xL1, xL, 1.0};
    double bz[ORD];
#pragma unroll
    for (int r = 0; r < ORD; r++) bz[r] = 0.0;
#pragma unroll
    for (int c = 0; c < NB; c++) bz[kRow[c]] += ca[c] * z[c];
    double g[ORD];
#pragma unroll
    for (int r = 0; r < ORD; r++) g[r] = wtL * bz[r] - scr[6 + ip * 4 + r];
    const double *fs = st + 42 + nip * 4 + ip * 16;
    double qs[ORD];
#pragma unroll
    for (int r = 0; r < ORD; r++) {
      double t = 0.0;
#pragma unroll
      for (int k = 0; k < ORD; k++) t += fs[r * ORD + k] * g[k];
      qs[r] = t;
    }
    double vsec[ORD];
#pragma unroll
    for (int r = 0; r < ORD; r++) vsec[r] = st[42 + ip * 4 + r];
    const long rec0 = (fbase + (long)ip * nf) * 12;
    for (int fi = rank; fi < nf; fi += G) {
      const int kf = f0 + fi;
      const double y = v.fy[kf] - ybar, A = v.fA[kf];
      double strain = vsec[0] - y * vsec[1];
      double rf = qs[0] - y * qs[1];
      if (ORD == 4) {
        const double zz = v.fz[kf] - zbar;
        strain += zz * vsec[2];
        rf += zz * qs[2];
      }
      rf *= A;
      const int u = v.fmat[kf];
      const double *q = v.uparam + (long)u * XG_UNI_NPARAM;
      const double *hcp = a.fh_prev + rec0 + 12L * fi;
      double *hbr = a.hbar + rec0 + 12L * fi;
      double hc[12], yb[12], hb[12], sb, qb[3];
#pragma unroll
      for (int k = 0; k < 12; k++) { hc[k] = hcp[k]; yb[k] = 0.0; }
      yb[9] = rf;
      fiber_vjp(v.utype[u], q, hc, strain, yb, hb, &sb, qb);
#pragma unroll
      for (int k = 0; k < 12; k++) hbr[k] += hb[k];
      add_slot(tq, a.fslot[kf], qb);
    }
  }
  theta_add(a, e, lane, tq);
  if (lane == 0) {
    if (a.use_k0) {
      // elements under betaK0 damping have one Steel02 or elastic material
      // (slot 0), in which K0 is linear
      // kv0 = (sum_s w_s b_s' fs0 b_s)^-1 (ForceBeamColumn2d/3d::getInitialStiff)
      const double *fs0 = v.fs0 + 16 * (long)sec;
      double f[NB * NB];
#pragma unroll
      for (int i = 0; i < NB * NB; i++) f[i] = 0.0;
      for (int ip = 0; ip < nip; ip++) {
        const double xL = v.xi[ip], xL1 = xL - 1.0, wtL = v.wt[ip] * L;
        const double ca[6] = {1.0, xL1, xL, xL1, xL, 1.0};
#pragma unroll
        for (int c = 0; c < NB; c++) {
          const double wa = ca[c] * wtL;
#pragma unroll
          for (int d = 0; d < NB; d++) f[c * NB + d] += wa * (fs0[kRow[c] * ORD + kRow[d]] * ca[d]);
        }
      }
      double kv0[NB * NB];
      small_inverse<NB>(f, kv0);
      double rv[NB];
#pragma unroll
      for (int i = 0; i < NB; i++) {
        double s = 0.0;
#pragma unroll
        for (int j = 0; j < NU; j++) s += T[i][j] * ve[j];
        rv[i] = s;
      }
      double val = 0.0;
#pragma unroll
      for (int i = 0; i < NB; i++)
#pragma unroll
        for (int k = 0; k < NB; k++) val += pb[i] * kv0[i * NB + k] * rv[k];
      const int u = a.elem_uni[e];
      const int ie = (v.utype[u] == XG_UNI_STEEL02 || v.utype[u] == XG_UNI_STEEL01) ? 1 : 0;
      const double E = v.uparam[(long)u * XG_UNI_NPARAM + ie];
      const double bk = a.bk0 ? a.bk0[e] : a.bk0_all;
      const double d = -bk / E * val;
      a.theta[(3L * kAdjSlots) * e + ie] += d;
    }
  }
}

// The part of the transposed tangent that the 2D P-Delta transformation's
// symmetric tangent leaves out.  With P = T' Se + (Se_0 / L) ul14 g,
//   dP/du = T' kv T + (Se_0 / L) g g' + (ul14 / L) g (T' kv e_0)'
// and getGlobalStiffMatrix (PDeltaCrdTransf2d.cpp:567-700) keeps the first
// two terms; the third's transpose applied to mu_e is
// (ul14 / L)(g . mu_e) T' kv e_0 (kv symmetric), written to the element
// force scratch for the residual's gather.  Thread per element.
__global__ void k_adj_pdelta(FrameView v, AdjView a) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= v.ne) return;
  const double *kv = a.st + (long)e * stride_of(v.nip) + 6;
  double T[3][6];
  basic_T<3>(v, e, T);
  double mue[6];
#pragma unroll
  for (int j = 0; j < 6; j++) {
    const int eq = a.eqn[(long)v.conn[2 * e + j / 3] * v.ndf + j % 3];
    mue[j] = eq >= 0 ? a.mu[eq] : 0.0;
  }
  const double f = pdelta_ul14(v, e) / v.L[e] * pdelta_g_dot(v, e, mue);
  double *re = v.Re + 6L * e;
#pragma unroll
  for (int j = 0; j < 6; j++) re[j] = f * (T[0][j] * kv[0] + T[1][j] * kv[3] + T[2][j] * kv[6]);
}

// The fresh records' dependence on the parameters (Steel02 revertToStart,
// Steel02.cpp:70-95: epsmax = Fy/E0, epsmin = -Fy/E0; Concrete01
// revertToStart, Concrete01.cpp:435-457: unloading slope 2 fpc / epsc0).
__global__ void k_adj_init_records(FrameView v, AdjView a) {
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int e = blockIdx.x * kAdjWarps + w;
  if (e >= v.ne) return;
  const int sec = v.sec[e];
  const int f0 = v.sec_fstart[sec], nf = v.sec_fstart[sec + 1] - f0;
  double tq[kAdjSlots][3] = {};
  for (int k = lane; k < v.nip * nf; k += 32) {
    const int kf = f0 + k % nf;
    const int u = v.fmat[kf];
    const double *q = v.uparam + (long)u * XG_UNI_NPARAM;
    const double *hb = a.hbar + (v.foff[e] + k) * 12;
    if (v.utype[u] == XG_UNI_STEEL02) {
      const double d = hb[1] - hb[0];
      const double qb[3] = {d / q[1], -d * q[0] / (q[1] * q[1]), 0.0};
      add_slot(tq, a.fslot[kf], qb);
    } else if (v.utype[u] == XG_UNI_CONCRETE01) {
      // Concrete01::revertToStart: unloading slope Ec0 = 2 fpc / epsc0
      const C01d c = c01d_params(q);
      const double g = hb[2];
      const double qb[3] = {c.sg0 * 2.0 * g / c.epsc0,
                            -c.sg1 * 2.0 * g * c.fpc / (c.epsc0 * c.epsc0), 0.0};
      add_slot(tq, a.fslot[kf], qb);
    }
  }
  theta_add(a, e, lane, tq);
}

// J_k += w_k U[dof_k]^2, one accumulator per term
__global__ void k_adj_objective(int nterm, const int *dof, const double *w, const double *U,
                                double *J) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < nterm) J[k] += w[k] * U[dof[k]] * U[dof[k]];
}

// Ubar[eqn[dof_k]] += 2 w_k U[dof_k] (one thread, term order)
__global__ void k_adj_objective_grad(int nterm, const int *dof, const double *w, const int *eqn,
                                     const double *U, double *Ubar) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  for (int k = 0; k < nterm; k++) {
    const int eq = eqn[dof[k]];
    if (eq >= 0) Ubar[eq] += 2.0 * w[k] * U[dof[k]];
  }
}

__global__ void k_adj_rhs(int neq, const double *Ub, const double *Vb, const double *Ab,
                          const double *uA, double c2, double c3, double *rhs) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < neq) rhs[i] = Ub[i] + c2 * Vb[i] + c3 * Ab[i] + uA[i];
}

__global__ void k_adj_prev(int neq, const double *mu, const double *kmu, const double *meq,
                           const double *meq_am, NewmarkCoef c, double *Ub, double *Vb,
                           double *Ab) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= neq) return;
  const double m = meq[i] * mu[i], ma = meq_am[i] * mu[i], km = kmu ? kmu[i] : 0.0;
  const double vb = Vb[i], ab = Ab[i];
  Ub[i] = c.c3 * m + c.c2 * (ma + km) - c.c2 * vb - c.c3 * ab;
  Vb[i] = -(c.a3 * m + c.a1 * (ma + km)) + c.a1 * vb + c.a3 * ab;
  Ab[i] = -(c.a4 * m + c.a2 * (ma + km)) + c.a2 * vb + c.a4 * ab;
}

// ---------------------------------------------------------------------------
// Direct differentiation (DDM), forward mode along one parameter direction:
// the reference's Newmark::computeSensitivities (Newmark.cpp:904-959), with
// ForceBeamColumn2d's basic-force sensitivity at fixed deformation and its
// commitSensitivity (ForceBeamColumn2d.cpp:2890-3007) restated on the
// element equations of the adjoint above:
//   dSe = kv (dv + z),   z = sum_s w_s L b_s' fs_s q_s,
//   de_s = fs_s (b_s dSe - q_s),   q_s = sum_f A_f a_f dsigma_f (strain fixed)
// ---------------------------------------------------------------------------
__device__ __forceinline__ void fiber_jvp(int type, const double *q, const double *hc,
                                          double strain, double dstrain, const double *dhc,
                                          const double *dq, double *dht) {
  if (type == XG_UNI_STEEL02) steel02_jvp(q, hc, strain, dstrain, dhc, dq, dht);
  else if (type == XG_UNI_CONCRETE02) concrete02_jvp(q, hc, strain, dstrain, dhc, dq, dht);
  else if (type == XG_UNI_STEEL01) steel01_jvp(q, hc, strain, dstrain, dhc, dq, dht);
  else if (type == XG_UNI_CONCRETE01) concrete01_jvp(q, hc, strain, dstrain, dhc, dq, dht);
  else elastic_jvp(q, strain, dstrain, dq, dht);
}

// Pass 1 (warp per element, a lane group per section): every fiber's stress
// tangent at fixed strain gives q_s; z and the conditional force tangent
// T' kv z (written to the element force scratch for the residual's gather).
template <int NB, int ORD>
__global__ void __launch_bounds__(32 * kAdjWarps) k_ddm_cond(FrameView v, DdmView d) {
  constexpr int NU = NB == 3 ? 6 : 12;
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int e = blockIdx.x * kAdjWarps + w;
  if (e >= v.ne) return;
  const int nip = v.nip;
  const double *st = v.st + (long)e * stride_of(nip);
  const int sec = v.sec[e];
  const int f0 = v.sec_fstart[sec], nf = v.sec_fstart[sec + 1] - f0;
  const double ybar = v.ybar[sec], zbar = ORD == 4 ? v.zbar[sec] : 0.0;
  const double L = v.L[e];
  const long fbase = v.foff[e];
  __shared__ double tsec_all[kAdjWarps][kAdjMaxIp][4];
  double(*tsec)[4] = tsec_all[w];
  constexpr int kRow[6] = {0, 1, 1, 2, 2, 3};
  const int G = 32 / nip;
  int P2 = 1;
  while (P2 < G) P2 <<= 1;
  const int gip = lane / G, rank = lane % G;
  const bool on = gip < nip;
  {
    const int ip = on ? gip : nip - 1;
    double vsec[ORD];
#pragma unroll
    for (int r = 0; r < ORD; r++) vsec[r] = st[42 + ip * 4 + r];
    double q0 = 0.0, q1 = 0.0, q2 = 0.0;
    const long rec0 = (fbase + (long)ip * nf) * 12;
    for (int fi = rank; on && fi < nf; fi += G) {
      const int kf = f0 + fi;
      const double y = v.fy[kf] - ybar, A = v.fA[kf];
      double strain = vsec[0] - y * vsec[1];
      double zz = 0.0;
      if (ORD == 4) {
        zz = v.fz[kf] - zbar;
        strain += zz * vsec[2];
      }
      const int u = v.fmat[kf];
      double dht[12];
      fiber_jvp(v.utype[u], v.uparam + (long)u * XG_UNI_NPARAM, d.fh_prev + rec0 + 12L * fi,
                strain, 0.0, d.dh + rec0 + 12L * fi, d.dth + 3L * u, dht);
      const double ds = A * dht[9];
      q0 += ds;
      q1 -= y * ds;
      if (ORD == 4) q2 += zz * ds;
    }
    double qs[ORD];
    qs[0] = group_sum_adj(q0, rank, G, P2);
    qs[1] = group_sum_adj(q1, rank, G, P2);
    if (ORD == 4) { qs[2] = group_sum_adj(q2, rank, G, P2); qs[3] = 0.0; }
    if (on && rank == 0) {
      const double *fs = st + 42 + nip * 4 + ip * 16;
#pragma unroll
      for (int r = 0; r < ORD; r++) {
        d.q[((long)e * nip + ip) * 4 + r] = qs[r];
        double t = 0.0;
#pragma unroll
        for (int k = 0; k < ORD; k++) t += fs[r * ORD + k] * qs[k];
        tsec[ip][r] = t;
      }
    }
  }
  __syncwarp();
  if (lane != 0) return;
  double z[NB];
#pragma unroll
  for (int c = 0; c < NB; c++) z[c] = 0.0;
  for (int ip = 0; ip < nip; ip++) {
    const double xL = v.xi[ip], xL1 = xL - 1.0, wtL = v.wt[ip] * L;
    const double ca[6] = {1.0, xL1, xL, xL1, xL, 1.0};
#pragma unroll
    for (int c = 0; c < NB; c++) z[c] += wtL * ca[c] * tsec[ip][kRow[c]];
  }
  const double *kv = st + 6;
  double dS[NB];
#pragma unroll
  for (int i = 0; i < NB; i++) {
    double t = 0.0;
#pragma unroll
    for (int k = 0; k < NB; k++) t += kv[i * NB + k] * z[k];
    dS[i] = t;
    d.z[6L * e + i] = z[i];
  }
  double T[NB][NU];
  basic_T<NB>(v, e, T);
  double *re = v.Re + (long)e * NU;
#pragma unroll
  for (int j = 0; j < NU; j++) {
    double t = 0.0;
#pragma unroll
    for (int k = 0; k < NB; k++) t += T[k][j] * dS[k];
    re[j] = t;
  }
  if (NB == 3 && v.pdelta2d) {
    // the 2D P-Delta force (Se_0 / L) ul14 g at fixed displacements
    const double cs = v.R[9 * (long)e], sn = v.R[9 * (long)e + 1];
    const double f = dS[0] / L * pdelta_ul14(v, e);
    re[0] -= f * sn; re[1] += f * cs; re[3] += f * sn; re[4] -= f * cs;
  }
}

// The 2D P-Delta tangent's term that the factored symmetric tangent leaves
// out, applied to a displacement tangent x: per element (ul14 / L)
// (kv T x_e)_0 g (the forward counterpart of k_adj_pdelta).  Thread per
// element, into the element force scratch.
__global__ void k_ddm_pdelta(FrameView v, const int *eqn, const double *x) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= v.ne) return;
  const double *kv = v.st + (long)e * stride_of(v.nip) + 6;
  double T[3][6];
  basic_T<3>(v, e, T);
  double xe[6];
#pragma unroll
  for (int j = 0; j < 6; j++) {
    const int eq = eqn[(long)v.conn[2 * e + j / 3] * v.ndf + j % 3];
    xe[j] = eq >= 0 ? x[eq] : 0.0;
  }
  double t = 0.0;
#pragma unroll
  for (int k = 0; k < 3; k++) {
    double tv = 0.0;
#pragma unroll
    for (int j = 0; j < 6; j++) tv += T[k][j] * xe[j];
    t += kv[k] * tv;
  }
  const double cs = v.R[9 * (long)e], sn = v.R[9 * (long)e + 1];
  const double f = pdelta_ul14(v, e) / v.L[e] * t;
  double *re = v.Re + 6L * e;
  re[0] = -f * sn; re[1] = f * cs; re[2] = 0.0; re[3] = f * sn; re[4] = -f * cs; re[5] = 0.0;
}

// Pass 2 (warp per element), after the step's tangent solve: dv = T dU_e
// gives dSe, each section's de_s and each fiber's strain tangent, and the
// law in forward mode the record tangents after the step (in place).
template <int NB, int ORD>
__global__ void __launch_bounds__(32 * kAdjWarps) k_ddm_commit(FrameView v, DdmView d) {
  constexpr int NU = NB == 3 ? 6 : 12;
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int e = blockIdx.x * kAdjWarps + w;
  if (e >= v.ne) return;
  const int nip = v.nip, ndf = v.ndf;
  const double *st = v.st + (long)e * stride_of(nip);
  const int sec = v.sec[e];
  const int f0 = v.sec_fstart[sec], nf = v.sec_fstart[sec + 1] - f0;
  const double ybar = v.ybar[sec], zbar = ORD == 4 ? v.zbar[sec] : 0.0;
  const long fbase = v.foff[e];
  double T[NB][NU];
  basic_T<NB>(v, e, T);
  double due[NU];
  const int nd = NU / 2;
#pragma unroll
  for (int j = 0; j < NU; j++) {
    const int eq = d.eqn[(long)v.conn[2 * e + j / nd] * ndf + (j % nd)];
    due[j] = eq >= 0 ? d.dU[eq] : 0.0;
  }
  const double *kv = st + 6;
  double dvz[NB], dS[NB];
#pragma unroll
  for (int i = 0; i < NB; i++) {
    double t = d.z[6L * e + i];
#pragma unroll
    for (int j = 0; j < NU; j++) t += T[i][j] * due[j];
    dvz[i] = t;
  }
#pragma unroll
  for (int i = 0; i < NB; i++) {
    double t = 0.0;
#pragma unroll
    for (int k = 0; k < NB; k++) t += kv[i * NB + k] * dvz[k];
    dS[i] = t;
  }
  constexpr int kRow[6] = {0, 1, 1, 2, 2, 3};
  const int G = 32 / nip;
  const int gip = lane / G, rank = lane % G;
  if (gip >= nip) return;
  const int ip = gip;
  const double xL = v.xi[ip], xL1 = xL - 1.0;
  const double ca[6] = {1.0, xL1, xL, xL1, xL, 1.0};
  double g[ORD];
#pragma unroll
  for (int r = 0; r < ORD; r++) g[r] = -d.q[((long)e * nip + ip) * 4 + r];
#pragma unroll
  for (int c = 0; c < NB; c++) g[kRow[c]] += ca[c] * dS[c];
  const double *fs = st + 42 + nip * 4 + ip * 16;
  double de[ORD], vsec[ORD];
#pragma unroll
  for (int r = 0; r < ORD; r++) {
    double t = 0.0;
#pragma unroll
    for (int k = 0; k < ORD; k++) t += fs[r * ORD + k] * g[k];
    de[r] = t;
    vsec[r] = st[42 + ip * 4 + r];
  }
  const long rec0 = (fbase + (long)ip * nf) * 12;
  for (int fi = rank; fi < nf; fi += G) {
    const int kf = f0 + fi;
    const double y = v.fy[kf] - ybar;
    double strain = vsec[0] - y * vsec[1], dstrain = de[0] - y * de[1];
    if (ORD == 4) {
      const double zz = v.fz[kf] - zbar;
      strain += zz * vsec[2];
      dstrain += zz * de[2];
    }
    const int u = v.fmat[kf];
    double *dhr = d.dh + rec0 + 12L * fi;
    double dhc[12], dht[12];
#pragma unroll
    for (int k = 0; k < 12; k++) dhc[k] = dhr[k];
    fiber_jvp(v.utype[u], v.uparam + (long)u * XG_UNI_NPARAM, d.fh_prev + rec0 + 12L * fi,
              strain, dstrain, dhc, d.dth + 3L * u, dht);
#pragma unroll
    for (int k = 0; k < 12; k++) dhr[k] = dht[k];
  }
}

// Record tangents of the fresh materials: Steel02's epsmax = Fy/E0 and
// epsmin = -Fy/E0 (Steel02::revertToStart), Concrete01's unloading slope
// Ec0 = 2 fpc / epsc0 (Concrete01::revertToStart); Steel01 and elastic
// records do not depend on the parameters.  Block per element, a thread
// per fiber record.
__global__ void k_ddm_init_records(FrameView v, DdmView d) {
  const int e = blockIdx.x;
  if (e >= v.ne) return;
  const int sec = v.sec[e];
  const int f0 = v.sec_fstart[sec], nf = v.sec_fstart[sec + 1] - f0;
  for (int k = threadIdx.x; k < v.nip * nf; k += blockDim.x) {
    const int kf = f0 + k % nf;
    const int u = v.fmat[kf];
    double *dh = d.dh + (v.foff[e] + k) * 12;
    for (int j = 0; j < 12; j++) dh[j] = 0.0;
    const double *q = v.uparam + (long)u * XG_UNI_NPARAM;
    const double *dq = d.dth + 3L * u;
    if (v.utype[u] == XG_UNI_STEEL02) {
      dh[1] = dq[0] / q[1] - q[0] * dq[1] / (q[1] * q[1]);
      dh[0] = -dh[1];
    } else if (v.utype[u] == XG_UNI_CONCRETE01) {
      const C01d c = c01d_params(q);
      dh[2] = 2.0 * c.sg0 * dq[0] / c.epsc0 - 2.0 * c.fpc * c.sg1 * dq[1] / (c.epsc0 * c.epsc0);
    }
  }
}

// The betaK0 damping force's tangent at fixed velocity, added to the
// conditional force tangent: an element under betaK0 has one Steel02,
// Steel01 or elastic material, in which its initial stiffness K0 = T' kv0 T
// (ForceBeamColumn2d/3d::getInitialStiff) is linear in E, so d(betaK0 K0 V)
// = betaK0 (dE / E) K0 V.  Thread per element.
template <int NB, int ORD>
__global__ void k_ddm_k0(FrameView v, DdmView d) {
  constexpr int NU = NB == 3 ? 6 : 12;
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= v.ne) return;
  const double bk = d.bk0 ? d.bk0[e] : d.bk0_all;
  if (bk == 0.0) return;
  const int u = d.elem_uni[e];
  const int ie = (v.utype[u] == XG_UNI_STEEL02 || v.utype[u] == XG_UNI_STEEL01) ? 1 : 0;
  const double E = v.uparam[(long)u * XG_UNI_NPARAM + ie], dE = d.dth[3L * u + ie];
  if (dE == 0.0) return;
  constexpr int kRow[6] = {0, 1, 1, 2, 2, 3};
  const double L = v.L[e];
  const double *fs0 = v.fs0 + 16 * (long)v.sec[e];
  double f[NB * NB];
#pragma unroll
  for (int i = 0; i < NB * NB; i++) f[i] = 0.0;
  for (int ip = 0; ip < v.nip; ip++) {
    const double xL = v.xi[ip], xL1 = xL - 1.0, wtL = v.wt[ip] * L;
    const double ca[6] = {1.0, xL1, xL, xL1, xL, 1.0};
#pragma unroll
    for (int c = 0; c < NB; c++)
#pragma unroll
      for (int k = 0; k < NB; k++) f[c * NB + k] += ca[c] * wtL * (fs0[kRow[c] * ORD + kRow[k]] * ca[k]);
  }
  double kv0[NB * NB];
  small_inverse<NB>(f, kv0);
  double T[NB][NU];
  basic_T<NB>(v, e, T);
  const int nd = NU / 2;
  double rv[NB];
#pragma unroll
  for (int i = 0; i < NB; i++) {
    double t = 0.0;
#pragma unroll
    for (int j = 0; j < NU; j++) t += T[i][j] * d.Vn[(long)v.conn[2 * e + j / nd] * v.ndf + j % nd];
    rv[i] = t;
  }
  double kr[NB];
#pragma unroll
  for (int i = 0; i < NB; i++) {
    double t = 0.0;
#pragma unroll
    for (int k = 0; k < NB; k++) t += kv0[i * NB + k] * rv[k];
    kr[i] = bk * dE / E * t;
  }
  double *re = v.Re + (long)e * NU;
#pragma unroll
  for (int j = 0; j < NU; j++) {
    double t = 0.0;
#pragma unroll
    for (int k = 0; k < NB; k++) t += T[k][j] * kr[k];
    re[j] += t;
  }
}

// c2 dU' - a1 dV' - a2 dA': the previous step's tangents as the damping
// term K0 (c2 (U - U') - a1 V' - a2 A') sees them
__global__ void k_ddm_k0_vec(int neq, const double *dU, const double *dV, const double *dA,
                             NewmarkCoef c, double *out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < neq) out[i] = c.c2 * dU[i] - c.a1 * dV[i] - c.a2 * dA[i];
}

// rhs = -dP_cond + M (c3 dU' - a3 dV' - a4 dA') + alphaM M (c2 dU' - a1 dV' - a2 dA'):
// the derivative of the step's unbalance at fixed displacement, with the
// Newmark relations A = c3 (U - U') + a3 V' + a4 A', V = c2 (U - U') + a1 V' + a2 A'
__global__ void k_ddm_rhs(int neq, const double *dPc, const double *dU, const double *dV,
                          const double *dA, const double *meq, const double *meq_am,
                          NewmarkCoef c, double *rhs) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= neq) return;
  double r = -dPc[i];
  if (meq) r += meq[i] * (c.c3 * dU[i] - c.a3 * dV[i] - c.a4 * dA[i]);   // null: no inertia
  if (meq_am) r += meq_am[i] * (c.c2 * dU[i] - c.a1 * dV[i] - c.a2 * dA[i]);
  rhs[i] = r;
}

// the step's displacement tangent x and the Newmark relations give dA, dV
__global__ void k_ddm_update(int neq, const double *x, NewmarkCoef c, double *dU, double *dV,
                             double *dA) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= neq) return;
  const double du = x[i] - dU[i], v = dV[i], a = dA[i];
  dA[i] = c.c3 * du + c.a3 * v + c.a4 * a;
  dV[i] = c.c2 * du + c.a1 * v + c.a2 * a;
  dU[i] = x[i];
}

// dJ[k] += 2 w_k U[dof_k] dU[eqn[dof_k]], one accumulator per term
__global__ void k_ddm_objective(int nterm, const int *dof, const double *w, const int *eqn,
                                const double *U, const double *dU, double *dJ) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nterm) return;
  const int eq = eqn[dof[k]];
  if (eq >= 0) dJ[k] += 2.0 * w[k] * U[dof[k]] * dU[eq];
}

inline int grid_of(long n, int b) { return (int)((n + b - 1) / b); }

}  // namespace

int launch_adj_elem_a(const FrameView &v, const AdjView &a, cudaStream_t s) {
  if (v.ne == 0) return 0;
  const int grid = grid_of(v.ne, kAdjWarps);
  if (v.nb == 3) k_adj_elem_a<3, 2><<<grid, 32 * kAdjWarps, 0, s>>>(v, a);
  else k_adj_elem_a<6, 4><<<grid, 32 * kAdjWarps, 0, s>>>(v, a);
  return cudaGetLastError() == cudaSuccess ? 0 : XG_ECUDA;
}

int launch_adj_elem_b(const FrameView &v, const AdjView &a, cudaStream_t s) {
  if (v.ne == 0) return 0;
  const int grid = grid_of(v.ne, kAdjWarps);
  if (v.nb == 3) k_adj_elem_b<3, 2><<<grid, 32 * kAdjWarps, 0, s>>>(v, a);
  else k_adj_elem_b<6, 4><<<grid, 32 * kAdjWarps, 0, s>>>(v, a);
  return cudaGetLastError() == cudaSuccess ? 0 : XG_ECUDA;
}

int launch_adj_pdelta(const FrameView &v, const AdjView &a, cudaStream_t s) {
  if (v.ne == 0) return 0;
  if (v.nb != 3) return XG_EINVAL;
  k_adj_pdelta<<<grid_of(v.ne, 128), 128, 0, s>>>(v, a);
  return cudaGetLastError() == cudaSuccess ? 0 : XG_ECUDA;
}

int launch_ddm_cond(const FrameView &v, const DdmView &d, cudaStream_t s) {
  if (v.ne == 0) return 0;
  const int grid = grid_of(v.ne, kAdjWarps);
  if (v.nb == 3) k_ddm_cond<3, 2><<<grid, 32 * kAdjWarps, 0, s>>>(v, d);
  else k_ddm_cond<6, 4><<<grid, 32 * kAdjWarps, 0, s>>>(v, d);
  return cudaGetLastError() == cudaSuccess ? 0 : XG_ECUDA;
}

int launch_ddm_commit(const FrameView &v, const DdmView &d, cudaStream_t s) {
  if (v.ne == 0) return 0;
  const int grid = grid_of(v.ne, kAdjWarps);
  if (v.nb == 3) k_ddm_commit<3, 2><<<grid, 32 * kAdjWarps, 0, s>>>(v, d);
  else k_ddm_commit<6, 4><<<grid, 32 * kAdjWarps, 0, s>>>(v, d);
  return cudaGetLastError() == cudaSuccess ? 0 : XG_ECUDA;
}

int launch_ddm_pdelta(const FrameView &v, const int *eqn, const double *x, cudaStream_t s) {
  if (v.ne == 0) return 0;
  if (v.nb != 3) return XG_EINVAL;
  k_ddm_pdelta<<<grid_of(v.ne, 128), 128, 0, s>>>(v, eqn, x);
  return cudaGetLastError() == cudaSuccess ? 0 : XG_ECUDA;
}

int launch_ddm_init_records(const FrameView &v, const DdmView &d, cudaStream_t s) {
  if (v.ne == 0) return 0;
  k_ddm_init_records<<<v.ne, 128, 0, s>>>(v, d);
  return cudaGetLastError() == cudaSuccess ? 0 : XG_ECUDA;
}

int launch_ddm_k0(const FrameView &v, const DdmView &d, cudaStream_t s) {
  if (v.ne == 0) return 0;
  if (v.nb == 3) k_ddm_k0<3, 2><<<grid_of(v.ne, 128), 128, 0, s>>>(v, d);
  else k_ddm_k0<6, 4><<<grid_of(v.ne, 128), 128, 0, s>>>(v, d);
  return cudaGetLastError() == cudaSuccess ? 0 : XG_ECUDA;
}

int launch_ddm_k0_vec(int neq, const double *dU, const double *dV, const double *dA,
                      const NewmarkCoef &c, double *out, cudaStream_t s) {
  if (neq == 0) return 0;
  k_ddm_k0_vec<<<grid_of(neq, 256), 256, 0, s>>>(neq, dU, dV, dA, c, out);
  return cudaGetLastError() == cudaSuccess ? 0 : XG_ECUDA;
}

int launch_ddm_rhs(int neq, const double *dPc, const double *dU, const double *dV,
                   const double *dA, const double *meq, const double *meq_am,
                   const NewmarkCoef &c, double *rhs, cudaStream_t s) {
  if (neq == 0) return 0;
  k_ddm_rhs<<<grid_of(neq, 256), 256, 0, s>>>(neq, dPc, dU, dV, dA, meq, meq_am, c, rhs);
  return cudaGetLastError() == cudaSuccess ? 0 : XG_ECUDA;
}

int launch_ddm_update(int neq, const double *x, const NewmarkCoef &c, double *dU, double *dV,
                      double *dA, cudaStream_t s) {
  if (neq == 0) return 0;
  k_ddm_update<<<grid_of(neq, 256), 256, 0, s>>>(neq, x, c, dU, dV, dA);
  return cudaGetLastError() == cudaSuccess ? 0 : XG_ECUDA;
}

int launch_ddm_objective(int nterm, const int *dof, const double *w, const int *eqn,
                         const double *U, const double *dU, double *dJ, cudaStream_t s) {
  if (nterm == 0) return 0;
  k_ddm_objective<<<grid_of(nterm, 128), 128, 0, s>>>(nterm, dof, w, eqn, U, dU, dJ);
  return cudaGetLastError() == cudaSuccess ? 0 : XG_ECUDA;
}

int launch_adj_init_records(const FrameView &v, const AdjView &a, cudaStream_t s) {
  if (v.ne == 0) return 0;
  k_adj_init_records<<<grid_of(v.ne, kAdjWarps), 32 * kAdjWarps, 0, s>>>(v, a);
  return cudaGetLastError() == cudaSuccess ? 0 : XG_ECUDA;
}

int launch_adj_objective(int nterm, const int *dof, const double *w, const double *U, double *J,
                         cudaStream_t s) {
  if (nterm == 0) return 0;
  k_adj_objective<<<grid_of(nterm, 128), 128, 0, s>>>(nterm, dof, w, U, J);
  return cudaGetLastError() == cudaSuccess ? 0 : XG_ECUDA;
}

int launch_adj_objective_grad(int nterm, const int *dof, const double *w, const int *eqn,
                              const double *U, double *Ubar, cudaStream_t s) {
  if (nterm == 0) return 0;
  k_adj_objective_grad<<<1, 32, 0, s>>>(nterm, dof, w, eqn, U, Ubar);
  return cudaGetLastError() == cudaSuccess ? 0 : XG_ECUDA;
}

int launch_adj_rhs(int neq, const double *Ub, const double *Vb, const double *Ab,
                   const double *uA, double c2, double c3, double *rhs, cudaStream_t s) {
  if (neq == 0) return 0;
  k_adj_rhs<<<grid_of(neq, 256), 256, 0, s>>>(neq, Ub, Vb, Ab, uA, c2, c3, rhs);
  return cudaGetLastError() == cudaSuccess ? 0 : XG_ECUDA;
}

int launch_adj_prev(int neq, const double *mu, const double *kmu, const double *meq,
                    const double *meq_am, const NewmarkCoef &c, double *Ub, double *Vb,
                    double *Ab, cudaStream_t s) {
  if (neq == 0) return 0;
  k_adj_prev<<<grid_of(neq, 256), 256, 0, s>>>(neq, mu, kmu, meq, meq_am, c, Ub, Vb, Ab);
  return cudaGetLastError() == cudaSuccess ? 0 : XG_ECUDA;
}

}  // namespace xg

// Host entry for the derivative tests: the Jacobian-vector product of one
// material point (no device work).
extern "C" int xg_uniaxial_jvp(int type, const double *q, const double *hc, double strain,
                               double dstrain, const double *dhc, const double *dq,
                               double *dht) {
  if (!q || !hc || !dhc || !dq || !dht) return XG_EINVAL;
  if (type == XG_UNI_STEEL02) {
    if (q[10] != 0.0) return XG_EINVAL;
    xg::steel02_jvp(q, hc, strain, dstrain, dhc, dq, dht);
  } else if (type == XG_UNI_CONCRETE02) xg::concrete02_jvp(q, hc, strain, dstrain, dhc, dq, dht);
  else if (type == XG_UNI_STEEL01) xg::steel01_jvp(q, hc, strain, dstrain, dhc, dq, dht);
  else if (type == XG_UNI_CONCRETE01) xg::concrete01_jvp(q, hc, strain, dstrain, dhc, dq, dht);
  else if (type == XG_UNI_ELASTIC) xg::elastic_jvp(q, strain, dstrain, dq, dht);
  else return XG_EINVAL;
  return 0;
}

// Host entry for the derivative tests: the vector-Jacobian product of one
// material point (no device work).
extern "C" int xg_uniaxial_vjp(int type, const double *q, const double *hc, double strain,
                               const double *yb, double *hb, double *sb, double *qb) {
  if (!q || !hc || !yb || !hb || !sb || !qb) return XG_EINVAL;
  if (type == XG_UNI_STEEL02) {
    if (q[10] != 0.0) return XG_EINVAL;
    xg::steel02_vjp(q, hc, strain, yb, hb, sb, qb);
  } else if (type == XG_UNI_CONCRETE02) {
    xg::concrete02_vjp(q, hc, strain, yb, hb, sb, qb);
  } else if (type == XG_UNI_STEEL01) {
    xg::steel01_vjp(q, hc, strain, yb, hb, sb, qb);
  } else if (type == XG_UNI_CONCRETE01) {
    xg::concrete01_vjp(q, hc, strain, yb, hb, sb, qb);
  } else if (type == XG_UNI_ELASTIC) {
    xg::elastic_vjp(q, strain, yb, hb, sb, qb);
  } else {
    return XG_EINVAL;
  }
  return 0;
}
