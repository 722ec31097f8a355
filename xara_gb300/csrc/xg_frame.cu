// xg_frame.cu -- force-based frame elements with fiber sections, FP64.
//
// k_fbc_update: one warp per ForceBeamColumn2d/3d element.  The element's
// compatibility iteration (strategy cascade and subdivision) runs in lock
// step in all 32 lanes; the element's small matrices live in the warp's
// slice of shared memory; the fibers of a section are spread across the
// lanes and their stiffness and force resultants are reduced with a fixed
// xor butterfly, so every run gives the same bits.  Fiber history is one
// 12-double record per (element, integration point, fiber): committed and
// trial copies.  k_fbc_assemble forms the global tangent and resisting
// force of each element from its basic stiffness and forces.
#include <cuda_runtime.h>

#include <cstdint>

#include "xg_internal.h"
#include "xg_rcp.h"

namespace xg {

namespace {

constexpr double kDblEps = 2.220446049250313e-16;

// ---------------------------------------------------------------------------
// uniaxial laws on a 12-double record:
//   Steel02: 0 epsmin 1 epsmax 2 epspl 3 epss0 4 sigs0 5 epsr 6 sigr 7 kon
//            11 R of the current branch
//   Concrete02: 0 ecmin 1 dept
//   Steel01: 0 minStrain 1 maxStrain 2 shiftP 3 shiftN 4 loading
//   all: 8 e 9 sig 10 eps
// ---------------------------------------------------------------------------

// Steel01::setTrialStrain / determineTrialState
// (material/uniaxial/steel/Steel01.cpp:68-92, 124-198): bilinear kinematic
// hardening with the isotropic shifts a1..a4 applied at load reversals;
// q = fy E0 b a1 a2 a3 a4.  A strain within DBL_EPSILON of the committed one
// leaves the committed state (strain included) as the trial state.
__device__ __forceinline__ void steel01_trial(const double *q, const double *hc,
                                              double trialStrain, double *ht) {
  const double fy = q[0], E0 = q[1], b = q[2], a1 = q[3], a2 = q[4], a3 = q[5], a4 = q[6];
  const double Cstrain = hc[10], Cstress = hc[9];
  double TminStrain = hc[0], TmaxStrain = hc[1], TshiftP = hc[2], TshiftN = hc[3];
  int Tloading = (int)hc[4];
  const double dStrain = trialStrain - Cstrain;
  if (!(fabs(dStrain) > kDblEps)) {
    for (int c = 0; c < 12; c++) ht[c] = hc[c];
    return;
  }
  const double fyOneMinusB = fy * (1.0 - b);
  const double Esh = b * E0;
  const double epsy = fy / E0;
  const double c1 = Esh * trialStrain;
  const double c2 = TshiftN * fyOneMinusB;
  const double c3 = TshiftP * fyOneMinusB;
  const double c = Cstress + E0 * dStrain;
  const double c1c3 = c1 + c3;
  double Tstress = c1c3 < c ? c1c3 : c;
  const double c1c2 = c1 - c2;
  if (c1c2 > Tstress) Tstress = c1c2;
  const double Ttangent = fabs(Tstress - c) < kDblEps ? E0 : Esh;
  if (Tloading == 0 && dStrain != 0.0) Tloading = dStrain > 0.0 ? 1 : -1;
  if (Tloading == 1 && dStrain < 0.0) {
    Tloading = -1;
    if (Cstrain > TmaxStrain) TmaxStrain = Cstrain;
    TshiftN = 1 + a1 * pow((TmaxStrain - TminStrain) / (2.0 * a2 * epsy), 0.8);
  }
  if (Tloading == -1 && dStrain > 0.0) {
    Tloading = 1;
    if (Cstrain < TminStrain) TminStrain = Cstrain;
    TshiftP = 1 + a3 * pow((TmaxStrain - TminStrain) / (2.0 * a4 * epsy), 0.8);
  }
  ht[0] = TminStrain; ht[1] = TmaxStrain; ht[2] = TshiftP; ht[3] = TshiftN;
  ht[4] = (double)Tloading;
  ht[5] = hc[5]; ht[6] = hc[6]; ht[7] = hc[7]; ht[11] = hc[11];
  ht[8] = Ttangent; ht[9] = Tstress; ht[10] = trialStrain;
}

// Concrete01::setTrial (material/uniaxial/concrete/Concrete01.cpp:209-278)
// with reload, envelope and unload (:313-385): Kent-Scott-Park envelope
// (parabola to epsc0, linear to the crushing strain, flat beyond), no
// tension, unloading toward the end strain of the Karsan-Jirsa ratio.
// q = fpc epsc0 fpcu epscu, made negative as the constructor does
// (:89-112).  Record: 0 minStrain 1 endStrain 2 unloadSlope.  A strain
// within DBL_EPSILON of the committed one leaves the committed state.
__device__ __forceinline__ void concrete01_trial(const double *q, const double *hc, double strain,
                                                 double *ht) {
  const double fpc = -fabs(q[0]), epsc0 = -fabs(q[1]), fpcu = -fabs(q[2]), epscu = -fabs(q[3]);
  for (int c = 0; c < 12; c++) ht[c] = hc[c];
  const double Cstrain = hc[10], Cstress = hc[9];
  if (fabs(strain - Cstrain) < kDblEps) return;
  double minS = hc[0], endS = hc[1], slope = hc[2];
  double stress = Cstress, tangent = hc[8];
  ht[10] = strain;
  if (strain > 0.0) {
    ht[8] = 0.0;
    ht[9] = 0.0;
    return;
  }
  const double tempStress = Cstress + slope * strain - slope * Cstrain;
  if (strain <= Cstrain) {
    if (strain <= minS) {
      minS = strain;
      const double Ec0 = 2.0 * fpc / epsc0;
      if (strain > epsc0) {
        const double eta = strain / epsc0;
        stress = fpc * (2 * eta - eta * eta);
        tangent = Ec0 * (1.0 - eta);
      } else if (strain > epscu) {
        tangent = (fpc - fpcu) / (epsc0 - epscu);
        stress = fpc + tangent * (strain - epsc0);
      } else {
        stress = fpcu;
        tangent = 0.0;
      }
      const double ts = minS < epscu ? epscu : minS;
      const double eta = ts / epsc0;
      const double ratio = eta < 2.0 ? 0.145 * eta * eta + 0.13 * eta : 0.707 * (eta - 2.0) + 0.834;
      endS = ratio * epsc0;
      const double temp1 = minS - endS, temp2 = stress / Ec0;
      if (temp1 > -kDblEps) {
        slope = Ec0;
      } else if (temp1 <= temp2) {
        endS = minS - temp1;
        slope = stress / temp1;
      } else {
        endS = minS - temp2;
        slope = Ec0;
      }
    } else if (strain <= endS) {
      tangent = slope;
      stress = tangent * (strain - endS);
    } else {
      stress = 0.0;
      tangent = 0.0;
    }
    if (tempStress > stress) {
      stress = tempStress;
      tangent = slope;
    }
  } else if (tempStress <= 0.0) {
    stress = tempStress;
    tangent = slope;
  } else {
    stress = 0.0;
    tangent = 0.0;
  }
  ht[0] = minS; ht[1] = endS; ht[2] = slope;
  ht[8] = tangent; ht[9] = stress;
}

// Steel02::setTrialStrain (material/uniaxial/steel/Steel02.cpp:113-227).
// Record slot 11 keeps R, which changes only where the branch does (the
// reference recomputes the same value every call); q[11] holds Fy/E0 (the
// model's device parameter table).  The Menegotto-Pinto powers go through
// log/exp and 1/(epss0 - epsr), 1/dum2 are formed once, by the three-FMA
// reciprocal of xg_rcp.h (within an ulp of the correctly rounded one): the
// stress and tangent differ from the reference's expression order by a few
// ulps.
// Tests and conversions on the bits of a double (integer instructions): the
// FP64 pipe, this law's bottleneck, then takes only arithmetic.  Exact for
// every non-NaN value.
__device__ __forceinline__ bool d_nonzero(double x) {
  return ((unsigned long long)__double_as_longlong(x) << 1) != 0ull;
}
__device__ __forceinline__ bool d_pos(double x) {    // x > 0
  const long long b = __double_as_longlong(x);
  return b > 0;
}
__device__ __forceinline__ bool d_neg(double x) {    // x < 0
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  return (b >> 63) != 0ull && (b << 1) != 0ull;
}
// kon (0..3) as the record keeps it (a double) and back
__device__ __forceinline__ int kon_of(double k) {
  const unsigned hi = (unsigned)__double2hiint(k);
  return hi == 0x3FF00000u ? 1 : hi == 0x40000000u ? 2 : hi == 0x40080000u ? 3 : 0;
}
__device__ __forceinline__ double kon_value(int k) {
  return k == 1 ? 1.0 : k == 2 ? 2.0 : k == 3 ? 3.0 : 0.0;
}
// |x| in single precision, truncated, clamped to the normal range (for
// estimates with a margin)
__device__ __forceinline__ float f32_abs_trunc(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x) & 0x7fffffffffffffffull;
  const int e = (int)(b >> 52) - 1023;
  if (e < -126) return 1.17549435e-38f;
  if (e > 127) return 3.40282347e+38f;
  return __uint_as_float((unsigned)((e + 127) << 23) | (unsigned)((b >> 29) & 0x7fffffu));
}

__device__ void steel02_trial(const double *q, const double *hc, double trialStrain,
                              double *ht) {
  const double Fy = q[0], E0 = q[1], b = q[2], R0 = q[3], cR1 = q[4], cR2 = q[5];
  const double a1 = q[6], a2 = q[7], a3 = q[8], a4 = q[9], sigini = q[10];
  const double Esh = b * E0, epsy = q[11];
  double eps = trialStrain;
  if (d_nonzero(sigini)) eps = trialStrain + sigini / E0;
  const double epsP = hc[10], sigP = hc[9];
  const double deps = eps - epsP;
  double epsmax = hc[1], epsmin = hc[0], epspl = hc[2], epss0 = hc[3], sigs0 = hc[4];
  double epsr = hc[5], sigr = hc[6], R = hc[11];
  int kon = kon_of(hc[7]);
  bool newR = false;
  ht[10] = eps;
  if (kon == 0 || kon == 3) {
    if (fabs(deps) < 10.0 * kDblEps) {
      ht[0] = epsmin; ht[1] = epsmax; ht[2] = epspl; ht[3] = epss0; ht[4] = sigs0;
      ht[5] = epsr; ht[6] = sigr; ht[7] = 3.0; ht[8] = E0; ht[9] = sigini; ht[11] = R;
      return;
    }
    epsmax = epsy;
    epsmin = -epsy;
    if (d_neg(deps)) { kon = 2; epss0 = epsmin; sigs0 = -Fy; epspl = epsmin; }
    else { kon = 1; epss0 = epsmax; sigs0 = Fy; epspl = epsmax; }
    newR = true;
  }
  if (kon == 2 && d_pos(deps)) {
    kon = 1;
    epsr = epsP;
    sigr = sigP;
    if (epsP < epsmin) epsmin = epsP;
    const double d1 = (epsmax - epsmin) / (2.0 * (a4 * epsy));
    const double shft = 1.0 + a3 * pow(d1, 0.8);
    epss0 = (Fy * shft - Esh * epsy * shft - sigr + E0 * epsr) / (E0 - Esh);
    sigs0 = Fy * shft + Esh * (epss0 - epsy * shft);
    epspl = epsmax;
    newR = true;
  } else if (kon == 1 && d_neg(deps)) {
    kon = 2;
    epsr = epsP;
    sigr = sigP;
    if (epsP > epsmax) epsmax = epsP;
    const double d1 = (epsmax - epsmin) / (2.0 * (a2 * epsy));
    const double shft = 1.0 + a1 * pow(d1, 0.8);
    epss0 = (-Fy * shft + Esh * epsy * shft - sigr + E0 * epsr) / (E0 - Esh);
    sigs0 = -Fy * shft + Esh * (epss0 + epsy * shft);
    epspl = epsmin;
    newR = true;
  }
  if (newR) {
    const double xi = fabs((epspl - epss0) / epsy);
    R = R0 * (1.0 - (cR1 * xi) / (cR2 + xi));
  }
  const double rden = chain_reciprocal(epss0 - epsr);
  const double epsrat = (eps - epsr) * rden;
  // |e*|^R and 1 / (1 + |e*|^R)^(1/R) through logs and exps.  Where a
  // single-precision estimate puts |e*|^R below 2^-60 (R log2|e*| < -60 with
  // a margin of several units over the estimate's error), 1 + |e*|^R rounds
  // to 1 and both values are exactly 1: the logs and exps, half of a fiber
  // update's FP64 work, are skipped, and so is the tangent's division in
  // sig = b e* + (1-b) e* rdum2, e = b + (1-b) rdum2 / dum1.
  const double ae = fabs(epsrat);
  double se = (1.0 - b) * epsrat, te = 1.0 - b;
  const float Rf = d_neg(R) ? -f32_abs_trunc(R) : f32_abs_trunc(R);
  if (!(Rf * __log2f(f32_abs_trunc(ae)) < -60.0f)) {
    const double pr = ae > 0.0 ? exp(R * log(ae)) : 0.0;
    const double dum1 = 1.0 + pr;
    const double rdum2 = exp(-log(dum1) * chain_reciprocal(R));
    se *= rdum2;
    te = te * rdum2 * chain_reciprocal(dum1);
  }
  const double dsig = sigs0 - sigr;
  double sig = b * epsrat + se;
  sig = sig * dsig + sigr;
  double e = b + te;
  e = e * dsig * rden;
  ht[0] = epsmin; ht[1] = epsmax; ht[2] = epspl; ht[3] = epss0; ht[4] = sigs0;
  ht[5] = epsr; ht[6] = sigr; ht[7] = kon_value(kon); ht[8] = e; ht[9] = sig; ht[11] = R;
}

// Concrete02 parameters after the constructor's sign normalisation
// (Concrete02.cpp:97-111) and the constants setTrialStrain and the
// envelopes form on every call: Ec0 = 2 fc / epsc0, the unloading reference
// point epsr = (fcu - rat Ec0 epscu) / (Ec0 (1 - rat)), sigmr = Ec0 epsr,
// and the tension envelope's eps0 = ft / Ec0 and epsu = ft (1/Ets + 1/Ec0).
// The device parameter table keeps the constants in slots 7-11 of every
// Concrete02 row (k_c02_constants, the same expressions).
struct C02 {
  double fc, epsc0, fcu, epscu, rat, ft, Ets;
  double ec0, epsr, sigmr, eps0, epsu;
};

__device__ __forceinline__ C02 c02_base(const double *q) {
  C02 c;
  c.fc = q[0] > 0 ? -q[0] : q[0];
  c.epsc0 = q[1] > 0 ? -q[1] : q[1];
  c.fcu = q[2] > 0 ? -q[2] : q[2];
  c.epscu = q[3] > 0 ? -q[3] : q[3];
  c.rat = q[4];
  c.ft = q[5];
  c.Ets = q[6];
  return c;
}

__device__ __forceinline__ C02 c02_params(const double *q) {
  C02 c = c02_base(q);
  c.ec0 = q[7];
  c.epsr = q[8];
  c.sigmr = q[9];
  c.eps0 = q[10];
  c.epsu = q[11];
  return c;
}

// Concrete02::Tens_Envlp / Compr_Envlp (Concrete02.cpp:421-497)
__device__ __forceinline__ void c02_tens(const C02 &c, double epsc, double &sigc, double &Ect) {
  const double Ec0 = c.ec0;
  const double eps0 = c.eps0;
  const double epsu = c.epsu;
  if (epsc <= eps0) { sigc = epsc * Ec0; Ect = Ec0; }
  else if (epsc <= epsu) { Ect = -c.Ets; sigc = c.ft - c.Ets * (epsc - eps0); }
  else { Ect = 1.0e-10; sigc = 0.0; }
}
__device__ __forceinline__ void c02_compr(const C02 &c, double epsc, double &sigc, double &Ect) {
  const double Ec0 = c.ec0;
  const double ratLocal = epsc / c.epsc0;
  if (epsc >= c.epsc0) {
    sigc = c.fc * ratLocal * (2.0 - ratLocal);
    Ect = Ec0 * (1.0 - ratLocal);
  } else if (epsc > c.epscu) {
    sigc = (c.fcu - c.fc) * (epsc - c.epsc0) / (c.epscu - c.epsc0) + c.fc;
    Ect = (c.fcu - c.fc) / (c.epscu - c.epsc0);
  } else {
    sigc = c.fcu;
    Ect = 1.0e-10;
  }
}

// Concrete02::setTrialStrain (Concrete02.cpp:167-271); the early return
// keeps the record's previous trial stress and tangent.
__device__ void concrete02_trial(const double *q, const double *hc, double eps, double *ht) {
  const C02 c = c02_params(q);
  const double ec0 = c.ec0;
  double ecmin = hc[0], dept = hc[1];
  ht[0] = ecmin;
  ht[1] = dept;
  ht[10] = eps;
  const double epsP = hc[10], sigP = hc[9];
  const double deps = eps - epsP;
  if (fabs(deps) < kDblEps) return;
  double sig, e;
  if (eps < ecmin) {
    c02_compr(c, eps, sig, e);
    ecmin = eps;
  } else {
    const double epsr = c.epsr;
    const double sigmr = c.sigmr;
    double sigmm, dumy;
    c02_compr(c, ecmin, sigmm, dumy);
    const double er = (sigmm - sigmr) / (ecmin - epsr);
    const double ept = ecmin - sigmm / er;
    if (eps <= ept) {
      const double sigmin = sigmm + er * (eps - ecmin);
      const double sigmax = er * .5 * (eps - ept);
      sig = sigP + ec0 * deps;
      e = ec0;
      if (sig <= sigmin) { sig = sigmin; e = er; }
      if (sig >= sigmax) { sig = sigmax; e = 0.5 * er; }
    } else {
      const double epn = ept + dept;
      double sicn;
      if (eps <= epn) {
        c02_tens(c, dept, sicn, e);
        if (dept != 0.0) e = sicn / dept;
        else e = ec0;
        sig = e * (eps - ept);
      } else {
        const double epstmp = eps - ept;
        c02_tens(c, epstmp, sig, e);
        dept = eps - ept;
      }
    }
  }
  ht[0] = ecmin;
  ht[1] = dept;
  ht[8] = e;
  ht[9] = sig;
}


// ---------------------------------------------------------------------------
// small dense helpers (every lane of a warp runs them on the same data)
// ---------------------------------------------------------------------------
// Gauss-Jordan inverse with partial pivoting; the reference uses explicit
// cofactor formulas (matrix/routines/invGL*.c) -- agreement to rounding.
template <int N>
__device__ void inv_gj(const double *A, double *Ainv) {
  double M[N][2 * N];
#pragma unroll
  for (int i = 0; i < N; i++)
#pragma unroll
    for (int j = 0; j < 2 * N; j++) M[i][j] = j < N ? A[i * N + j] : (j - N == i ? 1.0 : 0.0);
#pragma unroll
  for (int c = 0; c < N; c++) {
    int piv = c;
    double best = fabs(M[c][c]);
#pragma unroll
    for (int i = c + 1; i < N; i++)
      if (fabs(M[i][c]) > best) { best = fabs(M[i][c]); piv = i; }
    if (piv != c) {
#pragma unroll
      for (int j = 0; j < 2 * N; j++) {
        // swap rows c and piv without dynamic register indexing
#pragma unroll
        for (int r = c + 1; r < N; r++)
          if (r == piv) { const double t = M[c][j]; M[c][j] = M[r][j]; M[r][j] = t; }
      }
    }
    const double inv = 1.0 / M[c][c];
#pragma unroll
    for (int j = 0; j < 2 * N; j++) M[c][j] *= inv;
#pragma unroll
    for (int i = 0; i < N; i++) {
      if (i == c) continue;
      const double f = M[i][c];
#pragma unroll
      for (int j = 0; j < 2 * N; j++) M[i][j] -= f * M[c][j];
    }
  }
#pragma unroll
  for (int i = 0; i < N; i++)
#pragma unroll
    for (int j = 0; j < N; j++) Ainv[i * N + j] = M[i][N + j];
}

// 3x3 inverse by cofactors (the reference's cmx_inv3, matrix/routines/
// invGL3.c, is the same closed form); A and Ai row major with leading
// dimension lda.
__device__ __forceinline__ void inv3_cof(const double *A, int lda, double *Ai, int ldi) {
  const double a00 = A[0], a01 = A[1], a02 = A[2];
  const double a10 = A[lda], a11 = A[lda + 1], a12 = A[lda + 2];
  const double a20 = A[2 * lda], a21 = A[2 * lda + 1], a22 = A[2 * lda + 2];
  const double c00 = a11 * a22 - a12 * a21, c01 = a12 * a20 - a10 * a22;
  const double c02 = a10 * a21 - a11 * a20;
  const double det = a00 * c00 + a01 * c01 + a02 * c02;
  const double id = 1.0 / det;
  Ai[0] = c00 * id;
  Ai[1] = (a02 * a21 - a01 * a22) * id;
  Ai[2] = (a01 * a12 - a02 * a11) * id;
  Ai[ldi] = c01 * id;
  Ai[ldi + 1] = (a00 * a22 - a02 * a20) * id;
  Ai[ldi + 2] = (a02 * a10 - a00 * a12) * id;
  Ai[2 * ldi] = c02 * id;
  Ai[2 * ldi + 1] = (a01 * a20 - a00 * a21) * id;
  Ai[2 * ldi + 2] = (a00 * a11 - a01 * a10) * id;
}

// Section flexibility: 2x2 closed form, or (3D) the 3x3 axial-bending block
// by cofactors with the uncoupled elastic torsion 1/GJ.
template <int ORD>
__device__ __forceinline__ void sec_inverse(const double *ks, double *fs) {
  if (ORD == 2) {
    const double id = 1.0 / (ks[0] * ks[3] - ks[1] * ks[2]);
    fs[0] = ks[3] * id;
    fs[1] = -ks[1] * id;
    fs[2] = -ks[2] * id;
    fs[3] = ks[0] * id;
  } else {
    inv3_cof(ks, 4, fs, 4);
    fs[3] = fs[7] = fs[11] = fs[12] = fs[13] = fs[14] = 0.0;
    fs[15] = 1.0 / ks[15];
  }
}

// Element stiffness kv = f^-1: 3x3 cofactors (2D); in 3D the torsion row
// and column of f are uncoupled (every section's T is), so the 5x5
// axial-bending block is inverted by Gauss-Jordan and kv(5,5) = 1/f(5,5).
template <int NB>
__device__ __forceinline__ void elem_inverse(const double *f, double *kv) {
  if (NB == 3) {
    inv3_cof(f, 3, kv, 3);
  } else {
    double a[25], ai[25];
#pragma unroll
    for (int i = 0; i < 5; i++)
#pragma unroll
      for (int j = 0; j < 5; j++) a[i * 5 + j] = f[i * 6 + j];
    inv_gj<5>(a, ai);
#pragma unroll
    for (int i = 0; i < 5; i++) {
#pragma unroll
      for (int j = 0; j < 5; j++) kv[i * 6 + j] = ai[i * 5 + j];
      kv[i * 6 + 5] = 0.0;
      kv[30 + i] = 0.0;
    }
    kv[35] = 1.0 / f[35];
  }
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// element-major state record: Se[6] kv[36] vs[nip*4] fs[nip*16] Ssr[nip*4]
// vlast[6] init[1]
__device__ __forceinline__ int st_stride(int nip) { return 6 + 36 + nip * 24 + 6 + 1; }

// Basic deformations: LinearCrdTransf2d::getBasicTrialDisp
// (coordTransformation/LinearCrdTransf2d.cpp:248-299) and
// BasicFrameTransf3d::getBasicTrialDisp (Frame/BasicFrameTransf.cpp:90-104)
// over LinearFrameTransf<2,6> (Frame/LinearFrameTransf.tpp:258-386).
template <int NB>
__device__ void frame_basic(const FrameView &v, int e, double *ub) {
  const int ndf = v.ndf;
  const int a = v.conn[2 * e], b = v.conn[2 * e + 1];
  const double *uI = v.U + (long)a * ndf, *uJ = v.U + (long)b * ndf;
  const double L = v.L[e];
  const double *R = v.R + 9 * (long)e;
  if (NB == 3) {
    const double cs = R[0], sn = R[1];
    const double oneOverL = 1.0 / L, sl = sn * oneOverL, cl = cs * oneOverL;
    ub[0] = -cs * uI[0] - sn * uI[1] + cs * uJ[0] + sn * uJ[1];
    ub[1] = -sl * uI[0] + cl * uI[1] + uI[2] + sl * uJ[0] - cl * uJ[1];
    ub[2] = ub[1] + uJ[2] - uI[2];
  } else {
    double du[3], tI[3], tJ[3], Du[3];
#pragma unroll
    for (int i = 0; i < 3; i++) du[i] = uJ[i] - uI[i];
#pragma unroll
    for (int j = 0; j < 3; j++) {
      Du[j] = R[0 * 3 + j] * du[0] + R[1 * 3 + j] * du[1] + R[2 * 3 + j] * du[2];
      tI[j] = R[0 * 3 + j] * uI[3] + R[1 * 3 + j] * uI[4] + R[2 * 3 + j] * uI[5];
      tJ[j] = R[0 * 3 + j] * uJ[3] + R[1 * 3 + j] * uJ[4] + R[2 * 3 + j] * uJ[5];
    }
    ub[0] = Du[0];
    ub[1] = tI[2] - Du[1] / L;
    ub[2] = tJ[2] - Du[1] / L;
    ub[3] = tI[1] + Du[2] / L;
    ub[4] = tJ[1] + Du[2] / L;
    ub[5] = tJ[0] - tI[0];
  }
}

// Fiber section state determination: FiberSection2d / FiberSection3d
// setTrialSectionDeformation (material/section/FiberSection2d.cpp:225-262,
// FiberSection3d.cpp:423-478; order P MZ [MY T]).  Fibers across the warp's
// lanes, trial records written, tangent ks[ORD*ORD] and resultant Ssr[ORD]
// reduced with a fixed butterfly so every lane holds the same values.
template <int ORD>
__device__ __forceinline__ void fbc_section(const FrameView &v, int f0, int nf, double ybar,
                                            double zbar, double GJ, long rec0, int lane,
                                            const double *vsec, double *ks, double *Ssr) {
  double k0 = 0, k1 = 0, k2 = 0, k5 = 0, k6 = 0, k10 = 0, s0 = 0, s1 = 0, s2 = 0;
  for (int fi = lane; fi < nf; fi += 32) {
    const int kf = f0 + fi;
    const double y = v.fyc[kf];
    const int u = v.fmat[kf];
    double strain = vsec[0] - y * vsec[1];
    if (ORD == 4) strain += v.fzc[kf] * vsec[2];
    // material state from the committed record and the trial strain; only
    // the fields a law reads are loaded and only those it sets are stored
    const double *hc = v.fh_c + rec0 + 12L * fi;
    double *ht = v.fh_t + rec0 + 12L * fi;
    const double *q = v.uparam + (long)u * XG_UNI_NPARAM;
    const int type = v.utype[u];
    double stress, tangent;
    if (type == XG_UNI_STEEL02) {
      double hcl[12], htl[12];
#pragma unroll
      for (int c = 0; c < 12; c++) hcl[c] = c == 8 ? 0.0 : hc[c];
      steel02_trial(q, hcl, strain, htl);
#pragma unroll
      for (int c = 0; c < 12; c++) ht[c] = htl[c];
      stress = htl[9];
      tangent = htl[8];
    } else if (type == XG_UNI_STEEL01) {
      double hcl[12], htl[12];
#pragma unroll
      for (int c = 0; c < 12; c++) hcl[c] = hc[c];
      steel01_trial(q, hcl, strain, htl);
#pragma unroll
      for (int c = 0; c < 12; c++) ht[c] = htl[c];
      stress = htl[9];
      tangent = htl[8];
    } else if (type == XG_UNI_CONCRETE01) {
      double hcl[12], htl[12];
#pragma unroll
      for (int c = 0; c < 12; c++) hcl[c] = hc[c];
      concrete01_trial(q, hcl, strain, htl);
#pragma unroll
      for (int c = 0; c < 12; c++) ht[c] = htl[c];
      stress = htl[9];
      tangent = htl[8];
    } else if (type == XG_UNI_CONCRETE02) {
      double hcl[11], htl[11];
      hcl[0] = hc[0]; hcl[1] = hc[1]; hcl[9] = hc[9]; hcl[10] = hc[10];
      if (fabs(strain - hcl[10]) < kDblEps) {
        // Concrete02.cpp:182-183: the previous trial stress and tangent stay
        ht[0] = hcl[0]; ht[1] = hcl[1]; ht[10] = strain;
        stress = ht[9];
        tangent = ht[8];
      } else {
        concrete02_trial(q, hcl, strain, htl);
        ht[0] = htl[0]; ht[1] = htl[1]; ht[8] = htl[8]; ht[9] = htl[9]; ht[10] = htl[10];
        stress = htl[9];
        tangent = htl[8];
      }
    } else {
      stress = q[0] * strain;
      tangent = q[0];
      ht[8] = tangent; ht[9] = stress; ht[10] = strain;
    }
    // sums of E A (1, -y, z, y^2, z^2, -y z) and of s A (1, -y, z) with
    // the products per fiber formed once (FrameView::fk): one FMA a term
    const long nfk = v.nfib;
    const double fA = v.fk[kf], fmy = v.fk[nfk + kf], fy2 = v.fk[3 * nfk + kf];
    k0 = fma(tangent, fA, k0);
    k1 = fma(tangent, fmy, k1);
    k5 = fma(tangent, fy2, k5);
    s0 = fma(stress, fA, s0);
    s1 = fma(stress, fmy, s1);
    if (ORD == 4) {
      const double fz1 = v.fk[2 * nfk + kf], fz2 = v.fk[4 * nfk + kf];
      const double fyz = v.fk[5 * nfk + kf];
      k2 = fma(tangent, fz1, k2);
      k10 = fma(tangent, fz2, k10);
      k6 = fma(tangent, fyz, k6);
      s2 = fma(stress, fz1, s2);
    }
  }
  k0 = warp_sum(k0); k1 = warp_sum(k1); k5 = warp_sum(k5);
  s0 = warp_sum(s0); s1 = warp_sum(s1);
  if (ORD == 2) {
    ks[0] = k0; ks[1] = k1; ks[2] = k1; ks[3] = k5;
    Ssr[0] = s0; Ssr[1] = s1;
  } else {
    k2 = warp_sum(k2); k6 = warp_sum(k6); k10 = warp_sum(k10); s2 = warp_sum(s2);
    ks[0] = k0; ks[1] = k1; ks[2] = k2; ks[3] = 0.0;
    ks[4] = k1; ks[5] = k5; ks[6] = k6; ks[7] = 0.0;
    ks[8] = k2; ks[9] = k6; ks[10] = k10; ks[11] = 0.0;
    ks[12] = 0.0; ks[13] = 0.0; ks[14] = 0.0; ks[15] = GJ;
    Ssr[0] = s0; Ssr[1] = s1; Ssr[2] = s2; Ssr[3] = GJ * vsec[3];
  }
}

// Sum over the G lanes of a section's lane group (a fixed tree: the lane of
// rank r adds the rank r+o of its group, o = P2/2 .. 1, P2 the power of two
// at or above G), the result broadcast from the group's first lane.
__device__ __forceinline__ double group_sum(double v, int rank, int G, int P2) {
  for (int o = P2 >> 1; o > 0; o >>= 1) {
    const double t = __shfl_down_sync(0xffffffffu, v, o);
    if (rank + o < G) v += t;
  }
  return __shfl_sync(0xffffffffu, v, (int)(threadIdx.x & 31) - rank);
}

// fbc_section for one section per lane group: the lane of rank r takes the
// section's fibers r, r+G, ...; lanes outside every group (on = false) take
// none and write nothing.
template <int ORD>
__device__ __forceinline__ void fbc_section_group(const FrameView &v, int f0, int nf, double ybar,
                                                  double zbar, double GJ, long rec0, int rank,
                                                  int G, int P2, bool on, const double *vsec,
                                                  double *ks, double *Ssr) {
  double k0 = 0, k1 = 0, k2 = 0, k5 = 0, k6 = 0, k10 = 0, s0 = 0, s1 = 0, s2 = 0;
  for (int fi = rank; on && fi < nf; fi += G) {
    const int kf = f0 + fi;
    const double y = v.fyc[kf];
    const int u = v.fmat[kf];
    double strain = vsec[0] - y * vsec[1];
    if (ORD == 4) strain += v.fzc[kf] * vsec[2];
    const double *hc = v.fh_c + rec0 + 12L * fi;
    double *ht = v.fh_t + rec0 + 12L * fi;
    const double *q = v.uparam + (long)u * XG_UNI_NPARAM;
    const int type = v.utype[u];
    double stress, tangent;
    if (type == XG_UNI_STEEL02) {
      double hcl[12], htl[12];
#pragma unroll
      for (int c = 0; c < 12; c++) hcl[c] = c == 8 ? 0.0 : hc[c];
      steel02_trial(q, hcl, strain, htl);
#pragma unroll
      for (int c = 0; c < 12; c++) ht[c] = htl[c];
      stress = htl[9];
      tangent = htl[8];
    } else if (type == XG_UNI_STEEL01) {
      double hcl[12], htl[12];
#pragma unroll
      for (int c = 0; c < 12; c++) hcl[c] = hc[c];
      steel01_trial(q, hcl, strain, htl);
#pragma unroll
      for (int c = 0; c < 12; c++) ht[c] = htl[c];
      stress = htl[9];
      tangent = htl[8];
    } else if (type == XG_UNI_CONCRETE01) {
      double hcl[12], htl[12];
#pragma unroll
      for (int c = 0; c < 12; c++) hcl[c] = hc[c];
      concrete01_trial(q, hcl, strain, htl);
#pragma unroll
      for (int c = 0; c < 12; c++) ht[c] = htl[c];
      stress = htl[9];
      tangent = htl[8];
    } else if (type == XG_UNI_CONCRETE02) {
      double hcl[11], htl[11];
      hcl[0] = hc[0]; hcl[1] = hc[1]; hcl[9] = hc[9]; hcl[10] = hc[10];
      if (fabs(strain - hcl[10]) < kDblEps) {
        // Concrete02.cpp:182-183: the previous trial stress and tangent stay
        ht[0] = hcl[0]; ht[1] = hcl[1]; ht[10] = strain;
        stress = ht[9];
        tangent = ht[8];
      } else {
        concrete02_trial(q, hcl, strain, htl);
        ht[0] = htl[0]; ht[1] = htl[1]; ht[8] = htl[8]; ht[9] = htl[9]; ht[10] = htl[10];
        stress = htl[9];
        tangent = htl[8];
      }
    } else {
      stress = q[0] * strain;
      tangent = q[0];
      ht[8] = tangent; ht[9] = stress; ht[10] = strain;
    }
    // sums of E A (1, -y, z, y^2, z^2, -y z) and of s A (1, -y, z) with
    // the products per fiber formed once (FrameView::fk): one FMA a term
    const long nfk = v.nfib;
    const double fA = v.fk[kf], fmy = v.fk[nfk + kf], fy2 = v.fk[3 * nfk + kf];
    k0 = fma(tangent, fA, k0);
    k1 = fma(tangent, fmy, k1);
    k5 = fma(tangent, fy2, k5);
    s0 = fma(stress, fA, s0);
    s1 = fma(stress, fmy, s1);
    if (ORD == 4) {
      const double fz1 = v.fk[2 * nfk + kf], fz2 = v.fk[4 * nfk + kf];
      const double fyz = v.fk[5 * nfk + kf];
      k2 = fma(tangent, fz1, k2);
      k10 = fma(tangent, fz2, k10);
      k6 = fma(tangent, fyz, k6);
      s2 = fma(stress, fz1, s2);
    }
  }
  k0 = group_sum(k0, rank, G, P2); k1 = group_sum(k1, rank, G, P2);
  k5 = group_sum(k5, rank, G, P2);
  s0 = group_sum(s0, rank, G, P2); s1 = group_sum(s1, rank, G, P2);
  if (ORD == 2) {
    ks[0] = k0; ks[1] = k1; ks[2] = k1; ks[3] = k5;
    Ssr[0] = s0; Ssr[1] = s1;
  } else {
    k2 = group_sum(k2, rank, G, P2); k6 = group_sum(k6, rank, G, P2);
    k10 = group_sum(k10, rank, G, P2); s2 = group_sum(s2, rank, G, P2);
    ks[0] = k0; ks[1] = k1; ks[2] = k2; ks[3] = 0.0;
    ks[4] = k1; ks[5] = k5; ks[6] = k6; ks[7] = 0.0;
    ks[8] = k2; ks[9] = k6; ks[10] = k10; ks[11] = 0.0;
    ks[12] = 0.0; ks[13] = 0.0; ks[14] = 0.0; ks[15] = GJ;
    Ssr[0] = s0; Ssr[1] = s1; Ssr[2] = s2; Ssr[3] = GJ * vsec[3];
  }
}

constexpr int kFbcWarps = 4;
constexpr int kMaxIp = 10;
constexpr int kFbcMaxRounds = 4096;

template <int NB, int ORD>
struct FbcSmem {
  double Se[6], kv[36], SeT[6], kvT[36], f[36], vr[6];
  double vs[kMaxIp][4], fs[kMaxIp][16], Ssr[kMaxIp][4];
  double vsS[kMaxIp][4], fsS[kMaxIp][16], SsrS[kMaxIp][4];
  double dvsS[kMaxIp][4];
};

// ForceBeamColumn2d::update (element/Frame/Other/Force/ForceBeamColumn2d.cpp:
// 559-935) and ForceBeamColumn3d::update (ForceBeamColumn3d.cpp:588-1066).
template <int NB, int ORD, int WARPS>
__global__ void __launch_bounds__(32 * WARPS) k_fbc_update(FrameView v) {
  __shared__ FbcSmem<NB, ORD> sm_all[WARPS];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int e = blockIdx.x * WARPS + w;
  if (e >= v.ne) return;
  FbcSmem<NB, ORD> &S = sm_all[w];
  const int nip = v.nip;
  double *st = v.st + (long)e * st_stride(nip);
  const int sec = v.sec[e];
  const int f0 = v.sec_fstart[sec], nf = v.sec_fstart[sec + 1] - f0;
  const double ybar = v.ybar[sec], zbar = ORD == 4 ? v.zbar[sec] : 0.0;
  const double GJ = ORD == 4 ? v.GJ[sec] : 0.0;
  const double *fs0 = v.fs0 + 16 * (long)sec;
  const double L = v.L[e];
  const long fbase = v.foff[e];

  double ub[6], dv[6], vin[6], dvTrial[6], dvToDo[6];
  frame_basic<NB>(v, e, ub);
  double *vlast = st + 6 + 36 + nip * 24;
  const int init = (int)st[6 + 36 + nip * 24 + 6];
  double nrm = 0.0;
#pragma unroll
  for (int i = 0; i < NB; i++) { dv[i] = ub[i] - vlast[i]; nrm += dv[i] * dv[i]; }
  if (init != 0 && sqrt(nrm) <= kDblEps) return;
#pragma unroll
  for (int i = 0; i < NB; i++) { vin[i] = ub[i] - dv[i]; dvTrial[i] = dvToDo[i] = dv[i]; }
  // load the trial element state
  for (int i = lane; i < NB; i += 32) S.Se[i] = st[i];
  for (int i = lane; i < NB * NB; i += 32) S.kv[i] = st[6 + i];
  for (int k = lane; k < nip * ORD; k += 32) {
    const int ip = k / ORD, r = k % ORD;
    S.vs[ip][r] = st[42 + ip * 4 + r];
    S.Ssr[ip][r] = st[42 + nip * 20 + ip * 4 + r];
  }
  for (int k = lane; k < nip * ORD * ORD; k += 32) {
    const int ip = k / (ORD * ORD), r = k % (ORD * ORD);
    S.fs[ip][r] = st[42 + nip * 4 + ip * 16 + r];
  }
  __syncwarp();

  // lane groups: sec_G lanes per section, section sec_ip, rank sec_rank
  const int sec_G = 32 / nip;
  int sec_P2 = 1;
  while (sec_P2 < sec_G) sec_P2 <<= 1;
  const int sec_ip = lane / sec_G, sec_rank = lane % sec_G;
  const bool sec_on = sec_ip < nip;
  const int maxSub = NB == 3 ? 4 : 10;
  int numSub = 1;
  bool converged = false;
  // The reference loop has no bound of its own (partial convergence resets
  // the subdivision count); a kernel must end, so an element that needs more
  // than kFbcMaxRounds rounds reports a failed state determination.
  int rounds = 0;
  unsigned long long nj = 0;   // compatibility iterations (each visits every section)
  while (!converged && numSub <= maxSub && ++rounds <= kFbcMaxRounds) {
    bool partial = false;
    for (int l = 0; l < 3 && !partial && !converged; l++) {
      // SeTrial = Se + kv dvTrial; section state copies
#pragma unroll
      for (int i = 0; i < NB; i++) {
        double t = S.Se[i];
        double acc = 0.0;
#pragma unroll
        for (int k = 0; k < NB; k++) acc += S.kv[i * NB + k] * dvTrial[k];
        S.SeT[i] = t + acc;
      }
#pragma unroll
      for (int i = 0; i < NB * NB; i++) S.kvT[i] = S.kv[i];
      for (int ip = 0; ip < nip; ip++) {
#pragma unroll
        for (int r = 0; r < ORD; r++) { S.vsS[ip][r] = S.vs[ip][r]; S.SsrS[ip][r] = S.Ssr[ip][r]; }
#pragma unroll
        for (int r = 0; r < ORD * ORD; r++) S.fsS[ip][r] = S.fs[ip][r];
      }
      __syncwarp();
      const int numIters = (l == 1) ? 10 * v.max_iters : v.max_iters;
      for (int j = 0; j < numIters; j++) {
        nj++;
        double f[NB * NB], vr[NB];
#pragma unroll
        for (int i = 0; i < NB * NB; i++) f[i] = 0.0;
#pragma unroll
        for (int i = 0; i < NB; i++) vr[i] = 0.0;
        {
          // every section at once, one lane group each (lanes past the
          // last group mirror the last section and write nothing)
          const int ip = sec_on ? sec_ip : nip - 1;
          const double xL = v.xi[ip], xL1 = xL - 1.0, wtL = v.wt[ip] * L;
          // Ss = b SeT (codes P MZ [MY T])
          double Ss[ORD], dSs[ORD], dvs[ORD];
          Ss[0] = S.SeT[0];
          Ss[1] = xL1 * S.SeT[1] + xL * S.SeT[2];
          if (ORD == 4) {
            Ss[2] = xL1 * S.SeT[3] + xL * S.SeT[4];
            Ss[3] = S.SeT[5];
          }
#pragma unroll
          for (int r = 0; r < ORD; r++) dSs[r] = Ss[r] - S.SsrS[ip][r];
          const bool use_fs = (l == 0) || (l == 2 && j > 0);
#pragma unroll
          for (int r = 0; r < ORD; r++) {
            double t = 0.0;
#pragma unroll
            for (int k = 0; k < ORD; k++) t += (use_fs ? S.fsS[ip][r * ORD + k] : fs0[r * ORD + k]) * dSs[k];
            dvs[r] = t;
          }
          double vsec[ORD];
#pragma unroll
          for (int r = 0; r < ORD; r++) vsec[r] = S.vsS[ip][r] + (init != 0 ? dvs[r] : 0.0);
          double ks[ORD * ORD], Ssr[ORD];
          fbc_section_group<ORD>(v, f0, nf, ybar, zbar, GJ, (fbase + (long)ip * nf) * 12,
                                 sec_rank, sec_G, sec_P2, sec_on, vsec, ks, Ssr);
          double fsec[ORD * ORD];
          sec_inverse<ORD>(ks, fsec);
          __syncwarp();
          if (sec_on && sec_rank == 0) {
#pragma unroll
            for (int r = 0; r < ORD; r++) {
              S.vsS[ip][r] = vsec[r];
              S.SsrS[ip][r] = Ssr[r];
            }
#pragma unroll
            for (int r = 0; r < ORD * ORD; r++) S.fsS[ip][r] = fsec[r];
          }
#pragma unroll
          for (int r = 0; r < ORD; r++) dSs[r] = Ss[r] - Ssr[r];
#pragma unroll
          for (int r = 0; r < ORD; r++) {
            double t = 0.0;
#pragma unroll
            for (int k = 0; k < ORD; k++) t += fsec[r * ORD + k] * dSs[k];
            dvs[r] = t + vsec[r];
          }
          // f += b' fs b wL ; vr += b' (vs + dvs) wL.  Each column a of the
          // force interpolation b has one entry: row kRow[a], value ca[a]
          // (ForceBeamColumn3d::getForceInterpolatMatrix, :1068-1110).
          if (sec_on && sec_rank == 0) {
#pragma unroll
            for (int r = 0; r < ORD; r++) S.dvsS[ip][r] = dvs[r];
          }
          (void)wtL;
        }
        // f += b' fs b wL and vr += b' (vs + dvs) wL over the sections, in
        // section order: one entry per lane from the sections' flexibilities
        // and deformations in shared memory.  Each column a of the force
        // interpolation b has one entry: row kRow[a], value ca[a]
        // (ForceBeamColumn3d::getForceInterpolatMatrix, :1068-1110).
        __syncwarp();
        {
          // kRow = {0, 1, 1, 2, 2, 3} = (a + 1) / 2; ca = {1, xL-1, xL, xL-1, xL, 1}
          for (int i = lane; i < NB * NB + NB; i += 32) {
            const bool isf = i < NB * NB;
            const int a = isf ? i / NB : i - NB * NB, c = isf ? i % NB : 0;
            const int ra = (a + 1) >> 1, rc = (c + 1) >> 1;
            double acc = 0.0;
            for (int ip = 0; ip < nip; ip++) {
              const double xL = v.xi[ip], xL1 = xL - 1.0, wtL = v.wt[ip] * L;
              const double caa = (a == 0 || a == 5) ? 1.0 : ((a & 1) ? xL1 : xL);
              const double cac = (c == 0 || c == 5) ? 1.0 : ((c & 1) ? xL1 : xL);
              const double wa = caa * wtL;
              acc += isf ? wa * (S.fsS[ip][ra * ORD + rc] * cac) : wa * S.dvsS[ip][ra];
            }
            if (isf) S.f[i] = acc;
            else S.vr[a] = acc;
          }
        }
        __syncwarp();
#pragma unroll
        for (int i = 0; i < NB * NB; i++) f[i] = S.f[i];
#pragma unroll
        for (int i = 0; i < NB; i++) vr[i] = S.vr[i];
        double kvT[NB * NB];
        elem_inverse<NB>(f, kvT);
        double dvv[NB], dW = 0.0;
#pragma unroll
        for (int i = 0; i < NB; i++) dvv[i] = vin[i] + dvTrial[i] - vr[i];
#pragma unroll
        for (int i = 0; i < NB; i++) {
          double t = 0.0;
#pragma unroll
          for (int k = 0; k < NB; k++) t += kvT[i * NB + k] * dvv[k];
          S.SeT[i] += t;
          dW += dvv[i] * t;
        }
#pragma unroll
        for (int i = 0; i < NB * NB; i++) S.kvT[i] = kvT[i];
        __syncwarp();
        if (fabs(dW) < v.tol) {
          double n2 = 0.0;
#pragma unroll
          for (int i = 0; i < NB; i++) {
            dvToDo[i] -= dvTrial[i];
            vin[i] += dvTrial[i];
            n2 += dvToDo[i] * dvToDo[i];
          }
          if (sqrt(n2) <= kDblEps) converged = true;
          else {
#pragma unroll
            for (int i = 0; i < NB; i++) dvTrial[i] = dvToDo[i];
            numSub = 1;
            partial = true;
          }
#pragma unroll
          for (int i = 0; i < NB * NB; i++) S.kv[i] = S.kvT[i];
#pragma unroll
          for (int i = 0; i < NB; i++) S.Se[i] = S.SeT[i];
          for (int ip = 0; ip < nip; ip++) {
#pragma unroll
            for (int r = 0; r < ORD; r++) { S.vs[ip][r] = S.vsS[ip][r]; S.Ssr[ip][r] = S.SsrS[ip][r]; }
#pragma unroll
            for (int r = 0; r < ORD * ORD; r++) S.fs[ip][r] = S.fsS[ip][r];
          }
          __syncwarp();
          break;
        } else if (j == numIters - 1 && l == 2) {
#pragma unroll
          for (int i = 0; i < NB; i++) dvTrial[i] /= 10.0;
          numSub++;
        }
      }
    }
  }
  if (lane == 0 && v.work) {
    atomicAdd(v.work, nj * (unsigned long long)(nip * nf));
    atomicAdd(v.work + 1, nj * (unsigned long long)nip);
  }
  if (!converged) {
    if (lane == 0) atomicAdd(v.nfail, 1);
    return;
  }
  // store the trial element state
  for (int i = lane; i < NB; i += 32) st[i] = S.Se[i];
  for (int i = lane; i < NB * NB; i += 32) st[6 + i] = S.kv[i];
  for (int k = lane; k < nip * ORD; k += 32) {
    const int ip = k / ORD, r = k % ORD;
    st[42 + ip * 4 + r] = S.vs[ip][r];
    st[42 + nip * 20 + ip * 4 + r] = S.Ssr[ip][r];
  }
  for (int k = lane; k < nip * ORD * ORD; k += 32) {
    const int ip = k / (ORD * ORD), r = k % (ORD * ORD);
    st[42 + nip * 4 + ip * 16 + r] = S.fs[ip][r];
  }
  for (int i = lane; i < NB; i += 32) vlast[i] = ub[i];
  if (lane == 0) st[6 + 36 + nip * 24 + 6] = 1.0;
}

// Global tangent and resisting force of each element: K = T' kv T, P = T' Se
// (LinearCrdTransf2d::getGlobalStiffMatrix / getGlobalResistingForce,
// coordTransformation/LinearCrdTransf2d.cpp:473-735; BasicFrameTransf3d,
// Frame/BasicFrameTransf.cpp:150-290).  The reference's 3D P-Delta
// transformation (Frame/PDeltaFrameTransf3d.tpp:95-140) adds its geometric
// terms before LinearFrameTransf<2,6>::pushResponse maps the transverse
// translations onto the chord rotation, which cancels them; its tangent and
// force equal these.
template <int NB>
__global__ void k_fbc_assemble(FrameView v) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= v.ne) return;
  constexpr int NU = NB == 3 ? 6 : 12;
  const double *st = v.st + (long)e * st_stride(v.nip);
  const double L = v.L[e];
  const double *R = v.R + 9 * (long)e;
  double T[NB][NU];
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
  const double *Se = st, *kv = st + 6;
  double kT[NB][NU];
#pragma unroll
  for (int i = 0; i < NB; i++)
#pragma unroll
    for (int j = 0; j < NU; j++) {
      double s = 0.0;
#pragma unroll
      for (int k = 0; k < NB; k++) s += kv[i * NB + k] * T[k][j];
      kT[i][j] = s;
    }
  double *Ke = v.Ke + (long)e * NU * NU;
  double *Re = v.Re + (long)e * NU;
#pragma unroll
  for (int i = 0; i < NU; i++) {
#pragma unroll
    for (int j = 0; j < NU; j++) {
      double s = 0.0;
#pragma unroll
      for (int k = 0; k < NB; k++) s += T[k][i] * kT[k][j];
      Ke[i * NU + j] = s;
    }
    double p = 0.0;
#pragma unroll
    for (int k = 0; k < NB; k++) p += T[k][i] * Se[k];
    Re[i] = p;
  }
  if (NB == 3 && v.pdelta2d) {
    // PDeltaCrdTransf2d (coordTransformation/PDeltaCrdTransf2d.cpp:508-700):
    // K += (N/L) g g', P += (N/L)(g . u) g with g = [-s c 0 s -c 0]
    const double cs = R[0], sn = R[1];
    const int a = v.conn[2 * e], b = v.conn[2 * e + 1];
    const double *uI = v.U + (long)a * v.ndf, *uJ = v.U + (long)b * v.ndf;
    const double ul14 = (-sn * uI[0] + cs * uI[1]) - (-sn * uJ[0] + cs * uJ[1]);
    const double NoverL = Se[0] / L;
    const double g[6] = {-sn, cs, 0.0, sn, -cs, 0.0};
#pragma unroll
    for (int i = 0; i < 6; i++) {
      Re[i] += NoverL * ul14 * g[i];
#pragma unroll
      for (int j = 0; j < 6; j++) Ke[i * 6 + j] += NoverL * g[i] * g[j];
    }
  }
}

// ForceBeamColumn*::commitState (ForceBeamColumn2d.cpp:277-306): committed
// element state and fiber records take the trial ones.
__global__ void k_fbc_commit(FrameView v, double *st_c, double *fh_c_mut, long nrec) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const long nst = (long)v.ne * st_stride(v.nip);
  if (i < nst) st_c[i] = v.st[i];
  if (i < nrec) fh_c_mut[i] = v.fh_t[i];
}

// revertToLastCommit: trial state and fiber records back to the committed
// ones (ForceBeamColumn2d.cpp:310-336)
__global__ void k_fbc_revert(FrameView v, const double *st_c, long nrec) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const long nst = (long)v.ne * st_stride(v.nip);
  if (i < nst) v.st[i] = st_c[i];
  if (i < nrec) v.fh_t[i] = v.fh_c[i];
}

// The rest of revertToLastCommit (ForceBeamColumn2d.cpp:315-338): each
// section set to its committed deformation gives Ssr and fs again, and
// initialFlag returns to 0.  Warp per element, after k_fbc_revert.
template <int ORD>
__global__ void __launch_bounds__(32 * kFbcWarps) k_fbc_revert_sections(FrameView v) {
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int e = blockIdx.x * kFbcWarps + w;
  if (e >= v.ne) return;
  const int nip = v.nip;
  double *st = v.st + (long)e * st_stride(nip);
  const int sec = v.sec[e];
  const int f0 = v.sec_fstart[sec], nf = v.sec_fstart[sec + 1] - f0;
  const double ybar = v.ybar[sec], zbar = ORD == 4 ? v.zbar[sec] : 0.0;
  const double GJ = ORD == 4 ? v.GJ[sec] : 0.0;
  for (int ip = 0; ip < nip; ip++) {
    double vsec[ORD], ks[ORD * ORD], Ssr[ORD], fsec[ORD * ORD];
#pragma unroll
    for (int r = 0; r < ORD; r++) vsec[r] = st[42 + ip * 4 + r];
    fbc_section<ORD>(v, f0, nf, ybar, zbar, GJ, (v.foff[e] + (long)ip * nf) * 12, lane, vsec, ks,
                     Ssr);
    inv_gj<ORD>(ks, fsec);
    __syncwarp();
    if (lane == 0) {
#pragma unroll
      for (int r = 0; r < ORD; r++) st[42 + nip * 20 + ip * 4 + r] = Ssr[r];
#pragma unroll
      for (int r = 0; r < ORD * ORD; r++) st[42 + nip * 4 + ip * 16 + r] = fsec[r];
    }
  }
  if (lane == 0) st[6 + 36 + nip * 24 + 6] = 0.0;
}

// The per-material Concrete02 constants into slots 7-11 of the device
// parameter table, with the expressions setTrialStrain and the envelopes
// use (Concrete02.cpp:190-191, 421-446).
__global__ void k_c02_constants(double *up, const int *ut, int n) {
  const int u = blockIdx.x * blockDim.x + threadIdx.x;
  if (u >= n || ut[u] != XG_UNI_CONCRETE02) return;
  double *q = up + (long)u * XG_UNI_NPARAM;
  const C02 c = c02_base(q);
  const double ec0 = c.fc * 2. / c.epsc0;
  const double epsr = (c.fcu - c.rat * ec0 * c.epscu) / (ec0 * (1.0 - c.rat));
  const double Ec0 = 2.0 * c.fc / c.epsc0;
  q[7] = ec0;
  q[8] = epsr;
  q[9] = ec0 * epsr;
  q[10] = c.ft / Ec0;
  q[11] = c.ft * (1.0 / c.Ets + 1.0 / Ec0);
}

}  // namespace

int launch_c02_constants(double *uparam, const int *utype, int n, cudaStream_t s) {
  if (n <= 0) return 0;
  k_c02_constants<<<(n + 127) / 128, 128, 0, s>>>(uparam, utype, n);
  return cudaGetLastError() == cudaSuccess ? 0 : XG_ECUDA;
}

int frame_state_stride(int nip) { return 6 + 36 + nip * 24 + 6 + 1; }

template <int WARPS>
static void fbc_update_as(const FrameView &v, cudaStream_t s) {
  const int grid = (v.ne + WARPS - 1) / WARPS;
  if (v.nb == 3) k_fbc_update<3, 2, WARPS><<<grid, 32 * WARPS, 0, s>>>(v);
  else k_fbc_update<6, 4, WARPS><<<grid, 32 * WARPS, 0, s>>>(v);
}

// warps: elements (warps) per block, one of 1, 2, 4, 8 (the autotuner's
// choice; 4 otherwise)
int launch_fbc_update(const FrameView &v, cudaStream_t s, int warps) {
  if (v.ne == 0) return 0;
  if (v.nip > kMaxIp) return XG_EINVAL;
  switch (warps) {
    case 1: fbc_update_as<1>(v, s); break;
    case 2: fbc_update_as<2>(v, s); break;
    case 8: fbc_update_as<8>(v, s); break;
    default: fbc_update_as<4>(v, s); break;
  }
  return cudaGetLastError() == cudaSuccess ? 0 : XG_ECUDA;
}

int launch_fbc_assemble(const FrameView &v, cudaStream_t s) {
  if (v.ne == 0) return 0;
  const int grid = (v.ne + 127) / 128;
  if (v.nb == 3) k_fbc_assemble<3><<<grid, 128, 0, s>>>(v);
  else k_fbc_assemble<6><<<grid, 128, 0, s>>>(v);
  return cudaGetLastError() == cudaSuccess ? 0 : XG_ECUDA;
}

namespace {
// ForceBeamColumn2d/3d::getInitialStiff (ForceBeamColumn2d.cpp:379-397,
// getInitialFlexibility :1777-1830): f0 = sum of b' fs0 b wL, kv0 = f0^-1.
template <int NB, int ORD>
__global__ void k_fbc_kv0(FrameView v, double *st) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= v.ne) return;
  const int sec = v.sec[e];
  const double *fs0 = v.fs0 + 16 * (long)sec;
  const double L = v.L[e];
  double f[NB * NB];
#pragma unroll
  for (int i = 0; i < NB * NB; i++) f[i] = 0.0;
  constexpr int kRow[6] = {0, 1, 1, 2, 2, 3};
  for (int ip = 0; ip < v.nip; ip++) {
    const double xL = v.xi[ip], xL1 = xL - 1.0, wtL = v.wt[ip] * L;
    const double ca[6] = {1.0, xL1, xL, xL1, xL, 1.0};
#pragma unroll
    for (int a = 0; a < NB; a++) {
      const double wa = ca[a] * wtL;
#pragma unroll
      for (int c = 0; c < NB; c++) f[a * NB + c] += wa * (fs0[kRow[a] * ORD + kRow[c]] * ca[c]);
    }
  }
  double kv[NB * NB];
  elem_inverse<NB>(f, kv);
  double *rec = st + (long)e * st_stride(v.nip);
#pragma unroll
  for (int i = 0; i < 6; i++) rec[i] = 0.0;
#pragma unroll
  for (int i = 0; i < NB * NB; i++) rec[6 + i] = kv[i];
}
}  // namespace

int launch_fbc_kv0(const FrameView &v, double *st_scratch, cudaStream_t s) {
  if (v.ne == 0) return 0;
  const int grid = (v.ne + 127) / 128;
  if (v.nb == 3) k_fbc_kv0<3, 2><<<grid, 128, 0, s>>>(v, st_scratch);
  else k_fbc_kv0<6, 4><<<grid, 128, 0, s>>>(v, st_scratch);
  return cudaGetLastError() == cudaSuccess ? 0 : XG_ECUDA;
}

int launch_fbc_commit(const FrameView &v, double *st_c, double *fh_c, long nrec, cudaStream_t s) {
  const long nst = (long)v.ne * frame_state_stride(v.nip);
  const long n = nst > nrec ? nst : nrec;
  if (n == 0) return 0;
  k_fbc_commit<<<(int)((n + 255) / 256), 256, 0, s>>>(v, st_c, fh_c, nrec);
  return cudaGetLastError() == cudaSuccess ? 0 : XG_ECUDA;
}

int launch_fbc_revert(const FrameView &v, const double *st_c, long nrec, cudaStream_t s) {
  const long nst = (long)v.ne * frame_state_stride(v.nip);
  const long n = nst > nrec ? nst : nrec;
  if (n == 0) return 0;
  k_fbc_revert<<<(int)((n + 255) / 256), 256, 0, s>>>(v, st_c, nrec);
  if (v.ne > 0) {
    const int grid = (v.ne + kFbcWarps - 1) / kFbcWarps;
    if (v.nb == 3) k_fbc_revert_sections<2><<<grid, 32 * kFbcWarps, 0, s>>>(v);
    else k_fbc_revert_sections<4><<<grid, 32 * kFbcWarps, 0, s>>>(v);
  }
  return cudaGetLastError() == cudaSuccess ? 0 : XG_ECUDA;
}

}  // namespace xg
