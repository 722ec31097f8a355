// xg_uniaxial_adj.h -- derivatives of the uniaxial laws, for host and
// device: reverse mode for the adjoint, forward mode for the direct
// differentiation (DDM).
//
// A law maps (trial strain, committed record, parameters) to the trial
// record.  The vector-Jacobian product takes the adjoint of the trial
// record's continuous fields and returns the adjoints of the strain, of the
// committed record's fields and of the first three parameters.  The
// Jacobian-vector product takes the tangents of the strain, of the committed
// record's continuous fields and of the first three parameters and returns
// the tangent of the trial record's continuous fields.
//
// Record layout (12 doubles): Steel02 0 epsmin 1 epsmax 2 epspl 3 epss0
// 4 sigs0 5 epsr 6 sigr 7 kon; Concrete02 0 ecmin 1 dept; Steel01
// 0 minStrain 1 maxStrain 2 shiftP 3 shiftN 4 loading; all 8 e 9 sig
// 10 eps.  The loading fields (Steel02 7, Steel01 4) are discrete and field
// 8 (the tangent) is read by no later step, so their adjoints are not
// formed.
#pragma once

#include <float.h>
#include <math.h>

#ifdef __CUDACC__
#define XG_HD __host__ __device__
#else
#define XG_HD
#endif

namespace xg {

// True where a single-precision estimate puts |rho|^R below 2^-60 (R
// log2|rho| < -60, several units inside the estimate's error): there
// 1 + |rho|^R rounds to 1.
XG_HD inline bool mp_power_negligible(double R, double ae) {
#ifdef __CUDA_ARCH__
  return (float)R * __log2f(fmaxf((float)ae, 1.17549435e-38f)) < -60.0f;
#else
  return (float)R * log2f(fmaxf((float)ae, 1.17549435e-38f)) < -60.0f;
#endif
}

// Steel02::setTrialStrain (material/uniaxial/steel/Steel02.cpp:113-227),
// primal recomputed with the same operations as the forward kernel (the
// Menegotto-Pinto powers through log/exp, the isotropic shift through pow),
// then swept backwards branch by branch.  Parameters q: Fy E0 b R0 cR1 cR2
// a1 a2 a3 a4 sigini; qb receives d/d(Fy, E0, b).  sigini must be 0 (the
// adjoint refuses models with an initial stress).
XG_HD inline void steel02_vjp(const double *q, const double *hc, double strain, const double *yb,
                              double *hb, double *sb, double *qb) {
  const double Fy = q[0], E0 = q[1], b = q[2], R0 = q[3], cR1 = q[4], cR2 = q[5];
  const double a1 = q[6], a2 = q[7], a3 = q[8], a4 = q[9];
  const double Esh = b * E0, epsy = Fy / E0;
  const double eps = strain;
  const double epsP = hc[10], sigP = hc[9];
  const double deps = eps - epsP;
  double epsmax = hc[1], epsmin = hc[0], epspl = hc[2], epss0 = hc[3], sigs0 = hc[4];
  double epsr = hc[5], sigr = hc[6];
  int kon = (int)hc[7];
  for (int k = 0; k < 12; k++) hb[k] = 0.0;
  qb[0] = qb[1] = qb[2] = 0.0;
  if ((kon == 0 || kon == 3) && fabs(deps) < 10.0 * DBL_EPSILON) {
    // zero increment: the record passes through, the stress is sigini
    for (int k = 0; k < 7; k++) hb[k] = yb[k];
    *sb = yb[10];
    return;
  }
  // ---- primal ----
  int br = 0;            // 0 same branch, 1 first loading, 2 reversal 2->1, 3 reversal 1->2
  bool first_neg = false, moved = false;
  double d1 = 0.0, shft = 1.0;
  if (kon == 0 || kon == 3) {
    br = 1;
    epsmax = epsy;
    epsmin = -epsy;
    if (deps < 0.0) { kon = 2; epss0 = epsmin; sigs0 = -Fy; epspl = epsmin; first_neg = true; }
    else { kon = 1; epss0 = epsmax; sigs0 = Fy; epspl = epsmax; }
  }
  if (kon == 2 && deps > 0.0) {
    br = 2;
    kon = 1;
    epsr = epsP;
    sigr = sigP;
    if (epsP < epsmin) { epsmin = epsP; moved = true; }
    d1 = (epsmax - epsmin) / (2.0 * (a4 * epsy));
    shft = 1.0 + a3 * pow(d1, 0.8);
    epss0 = (Fy * shft - Esh * epsy * shft - sigr + E0 * epsr) / (E0 - Esh);
    sigs0 = Fy * shft + Esh * (epss0 - epsy * shft);
    epspl = epsmax;
  } else if (kon == 1 && deps < 0.0) {
    br = 3;
    kon = 2;
    epsr = epsP;
    sigr = sigP;
    if (epsP > epsmax) { epsmax = epsP; moved = true; }
    d1 = (epsmax - epsmin) / (2.0 * (a2 * epsy));
    shft = 1.0 + a1 * pow(d1, 0.8);
    epss0 = (-Fy * shft + Esh * epsy * shft - sigr + E0 * epsr) / (E0 - Esh);
    sigs0 = -Fy * shft + Esh * (epss0 + epsy * shft);
    epspl = epsmin;
  }
  const double w = (epspl - epss0) / epsy;
  const double xi = fabs(w);
  const double R = R0 * (1.0 - (cR1 * xi) / (cR2 + xi));
  const double den = epss0 - epsr;
  const double rho = (eps - epsr) / den;
  const double ae = fabs(rho);
  // as in the forward kernel: where |rho|^R < 2^-60 the powers are exactly
  // 1 and every term through |rho|^R is below 2^-60 of the others
  double lae = 0.0, pr = 0.0, dum1 = 1.0, ld1 = 0.0, dum2 = 1.0;
  if (!mp_power_negligible(R, ae)) {
    lae = ae > 0.0 ? log(ae) : 0.0;
    pr = ae > 0.0 ? exp(R * lae) : 0.0;
    dum1 = 1.0 + pr;
    ld1 = log(dum1);
    dum2 = exp(ld1 / R);
  }
  const double sst = b * rho + (1.0 - b) * rho / dum2;
  // ---- reverse ----
  double b_epsmin = yb[0], b_epsmax = yb[1], b_epspl = yb[2], b_epss0 = yb[3];
  double b_sigs0 = yb[4], b_epsr = yb[5], b_sigr = yb[6];
  const double b_sig = yb[9];
  double b_eps = yb[10];
  double b_Fy = 0.0, b_E0 = 0.0, b_b = 0.0, b_epsy = 0.0, b_Esh = 0.0;
  double b_epsP = 0.0, b_sigP = 0.0;
  // sig = sst (sigs0 - sigr) + sigr
  const double b_sst = b_sig * (sigs0 - sigr);
  b_sigs0 += b_sig * sst;
  b_sigr += b_sig * (1.0 - sst);
  // sst = b rho + (1 - b) rho / dum2
  double b_rho = b_sst * (b + (1.0 - b) / dum2);
  b_b += b_sst * (rho - rho / dum2);
  const double b_dum2 = -b_sst * (1.0 - b) * rho / (dum2 * dum2);
  // dum2 = dum1^(1/R), dum1 = 1 + |rho|^R
  const double b_dum1 = b_dum2 * dum2 / (R * dum1);
  double b_R = -b_dum2 * dum2 * ld1 / (R * R);
  if (ae > 0.0) {
    b_rho += b_dum1 * R * pr / rho;
    b_R += b_dum1 * pr * lae;
  }
  // rho = (eps - epsr) / (epss0 - epsr)
  b_eps += b_rho / den;
  b_epsr += b_rho * (rho - 1.0) / den;
  b_epss0 -= b_rho * rho / den;
  // R = R0 (1 - cR1 xi / (cR2 + xi)), xi = |epspl - epss0| / epsy
  const double b_xi = -b_R * R0 * cR1 * cR2 / ((cR2 + xi) * (cR2 + xi));
  const double b_w = w >= 0.0 ? b_xi : -b_xi;
  b_epspl += b_w / epsy;
  b_epss0 -= b_w / epsy;
  b_epsy -= b_w * w / epsy;
  if (br == 2 || br == 3) {
    const double sg = br == 2 ? 1.0 : -1.0;       // +Fy branch (2->1) or -Fy (1->2)
    const double aa = br == 2 ? a3 : a1, ad = br == 2 ? a4 : a2;
    const double D = E0 - Esh;
    // epspl = epsmax (2->1) or epsmin (1->2)
    if (br == 2) b_epsmax += b_epspl; else b_epsmin += b_epspl;
    // sigs0 = sg Fy shft + Esh (epss0 - sg epsy shft)
    b_Fy += sg * b_sigs0 * shft;
    double b_shft = b_sigs0 * (sg * Fy - sg * Esh * epsy);
    b_Esh += b_sigs0 * (epss0 - sg * epsy * shft);
    b_epss0 += b_sigs0 * Esh;
    b_epsy -= sg * b_sigs0 * Esh * shft;
    // epss0 = (sg Fy shft - sg Esh epsy shft - sigr + E0 epsr) / (E0 - Esh)
    const double b_num = b_epss0 / D, b_D = -b_epss0 * epss0 / D;
    b_Fy += sg * b_num * shft;
    b_shft += b_num * (sg * Fy - sg * Esh * epsy);
    b_Esh -= sg * b_num * epsy * shft;
    b_epsy -= sg * b_num * Esh * shft;
    b_sigr -= b_num;
    b_E0 += b_num * epsr;
    b_epsr += b_num * E0;
    b_E0 += b_D;
    b_Esh -= b_D;
    // shft = 1 + aa d1^0.8, d1 = (epsmax - epsmin) / (2 ad epsy)
    if (aa != 0.0 && d1 > 0.0) {
      const double b_d1 = b_shft * aa * 0.8 * pow(d1, -0.2);
      b_epsmax += b_d1 / (2.0 * ad * epsy);
      b_epsmin -= b_d1 / (2.0 * ad * epsy);
      b_epsy -= b_d1 * d1 / epsy;
    }
    // the extreme strain reached before the reversal
    if (moved) {
      if (br == 2) { b_epsP += b_epsmin; b_epsmin = 0.0; }
      else { b_epsP += b_epsmax; b_epsmax = 0.0; }
    }
    // the reversal point is the last committed state
    b_epsP += b_epsr;
    b_sigP += b_sigr;
    hb[0] = b_epsmin;
    hb[1] = b_epsmax;
  } else if (br == 1) {
    // epsmax = epsy, epsmin = -epsy, epss0 = epspl = +-epsy, sigs0 = +-Fy
    const double sg = first_neg ? -1.0 : 1.0;
    b_epsy += b_epsmax - b_epsmin + sg * (b_epss0 + b_epspl);
    b_Fy += sg * b_sigs0;
    hb[5] = b_epsr;
    hb[6] = b_sigr;
  } else {
    hb[0] = b_epsmin; hb[1] = b_epsmax; hb[2] = b_epspl; hb[3] = b_epss0;
    hb[4] = b_sigs0; hb[5] = b_epsr; hb[6] = b_sigr;
  }
  hb[9] = b_sigP;
  hb[10] = b_epsP;
  *sb = b_eps;
  // epsy = Fy / E0, Esh = b E0
  b_Fy += b_epsy / E0;
  b_E0 -= b_epsy * epsy / E0;
  b_b += b_Esh * E0;
  b_E0 += b_Esh * b;
  qb[0] = b_Fy;
  qb[1] = b_E0;
  qb[2] = b_b;
}

// Steel02::setTrialStrain in forward mode: the same primal steps as the
// vector-Jacobian product above (first loading, a reversal with the
// Filippou shift and the new asymptote's origin, the Menegotto-Pinto curve
// with R from the plastic excursion), differentiated step by step.  dq =
// d(Fy, E0, b); dht receives fields 0-6, 9 and 10.  sigini must be 0.
XG_HD inline void steel02_jvp(const double *q, const double *hc, double strain, double dstrain,
                              const double *dhc, const double *dq, double *dht) {
  const double Fy = q[0], E0 = q[1], b = q[2], R0 = q[3], cR1 = q[4], cR2 = q[5];
  const double a1 = q[6], a2 = q[7], a3 = q[8], a4 = q[9];
  const double dFy = dq[0], dE0 = dq[1], db = dq[2];
  const double Esh = b * E0, epsy = Fy / E0;
  const double dEsh = db * E0 + b * dE0, depsy = dFy / E0 - Fy * dE0 / (E0 * E0);
  const double eps = strain;
  const double epsP = hc[10], sigP = hc[9];
  const double deps = eps - epsP;
  double epsmax = hc[1], epsmin = hc[0], epspl = hc[2], epss0 = hc[3], sigs0 = hc[4];
  double epsr = hc[5], sigr = hc[6];
  double t_epsmin = dhc[0], t_epsmax = dhc[1], t_epspl = dhc[2], t_epss0 = dhc[3];
  double t_sigs0 = dhc[4], t_epsr = dhc[5], t_sigr = dhc[6];
  const double t_epsP = dhc[10], t_sigP = dhc[9];
  int kon = (int)hc[7];
  for (int k = 0; k < 12; k++) dht[k] = 0.0;
  if ((kon == 0 || kon == 3) && fabs(deps) < 10.0 * DBL_EPSILON) {
    for (int k = 0; k < 7; k++) dht[k] = dhc[k];
    dht[10] = dstrain;
    return;
  }
  if (kon == 0 || kon == 3) {
    epsmax = epsy;
    epsmin = -epsy;
    t_epsmax = depsy;
    t_epsmin = -depsy;
    if (deps < 0.0) {
      kon = 2;
      epss0 = epsmin; sigs0 = -Fy; epspl = epsmin;
      t_epss0 = -depsy; t_sigs0 = -dFy; t_epspl = -depsy;
    } else {
      kon = 1;
      epss0 = epsmax; sigs0 = Fy; epspl = epsmax;
      t_epss0 = depsy; t_sigs0 = dFy; t_epspl = depsy;
    }
  }
  const bool rev21 = kon == 2 && deps > 0.0, rev12 = !rev21 && kon == 1 && deps < 0.0;
  if (rev21 || rev12) {
    const double sg = rev21 ? 1.0 : -1.0;
    const double aa = rev21 ? a3 : a1, ad = rev21 ? a4 : a2;
    epsr = epsP; sigr = sigP;
    t_epsr = t_epsP; t_sigr = t_sigP;
    if (rev21 && epsP < epsmin) { epsmin = epsP; t_epsmin = t_epsP; }
    if (rev12 && epsP > epsmax) { epsmax = epsP; t_epsmax = t_epsP; }
    const double d1 = (epsmax - epsmin) / (2.0 * (ad * epsy));
    const double t_d1 = (t_epsmax - t_epsmin) / (2.0 * (ad * epsy)) - d1 * depsy / epsy;
    const double shft = 1.0 + aa * pow(d1, 0.8);
    const double t_shft = (aa != 0.0 && d1 > 0.0) ? aa * 0.8 * pow(d1, -0.2) * t_d1 : 0.0;
    const double D = E0 - Esh, t_D = dE0 - dEsh;
    const double num = sg * Fy * shft - sg * Esh * epsy * shft - sigr + E0 * epsr;
    const double t_num = sg * (dFy * shft + Fy * t_shft) -
                         sg * (dEsh * epsy * shft + Esh * depsy * shft + Esh * epsy * t_shft) -
                         t_sigr + dE0 * epsr + E0 * t_epsr;
    epss0 = num / D;
    t_epss0 = t_num / D - epss0 * t_D / D;
    sigs0 = sg * Fy * shft + Esh * (epss0 - sg * epsy * shft);
    t_sigs0 = sg * (dFy * shft + Fy * t_shft) + dEsh * (epss0 - sg * epsy * shft) +
              Esh * (t_epss0 - sg * (depsy * shft + epsy * t_shft));
    epspl = rev21 ? epsmax : epsmin;
    t_epspl = rev21 ? t_epsmax : t_epsmin;
  }
  const double w = (epspl - epss0) / epsy;
  const double t_w = (t_epspl - t_epss0) / epsy - w * depsy / epsy;
  const double xi = fabs(w), t_xi = w >= 0.0 ? t_w : -t_w;
  const double R = R0 * (1.0 - (cR1 * xi) / (cR2 + xi));
  const double t_R = -R0 * cR1 * cR2 / ((cR2 + xi) * (cR2 + xi)) * t_xi;
  const double den = epss0 - epsr;
  const double rho = (eps - epsr) / den;
  const double t_rho = (dstrain - t_epsr) / den - rho * (t_epss0 - t_epsr) / den;
  const double ae = fabs(rho);
  double lae = 0.0, pr = 0.0, dum1 = 1.0, ld1 = 0.0, dum2 = 1.0;
  if (!mp_power_negligible(R, ae)) {
    lae = ae > 0.0 ? log(ae) : 0.0;
    pr = ae > 0.0 ? exp(R * lae) : 0.0;
    dum1 = 1.0 + pr;
    ld1 = log(dum1);
    dum2 = exp(ld1 / R);
  }
  const double t_pr = ae > 0.0 ? pr * (t_R * lae + R * t_rho / rho) : 0.0;
  const double t_dum2 = dum2 * (t_pr / (R * dum1) - ld1 * t_R / (R * R));
  const double sst = b * rho + (1.0 - b) * rho / dum2;
  const double t_sst = db * rho + b * t_rho - db * rho / dum2 +
                       (1.0 - b) * (t_rho / dum2 - rho * t_dum2 / (dum2 * dum2));
  const double t_sig = t_sst * (sigs0 - sigr) + sst * (t_sigs0 - t_sigr) + t_sigr;
  dht[0] = t_epsmin; dht[1] = t_epsmax; dht[2] = t_epspl; dht[3] = t_epss0;
  dht[4] = t_sigs0; dht[5] = t_epsr; dht[6] = t_sigr;
  dht[9] = t_sig;
  dht[10] = dstrain;
}

// Concrete02 compression envelope (Concrete02.cpp:448-497) and its partial
// derivatives in the strain and in fc, epsc0, fcu (signs already negative).
XG_HD inline double c02_compr_d(double fc, double epsc0, double fcu, double epscu, double x,
                                double *d_x, double *d_fc, double *d_e0, double *d_fcu) {
  if (x >= epsc0) {
    const double r = x / epsc0;
    *d_x = fc * (2.0 - 2.0 * r) / epsc0;
    *d_fc = r * (2.0 - r);
    *d_e0 = -fc * (2.0 - 2.0 * r) * r / epsc0;
    *d_fcu = 0.0;
    return fc * r * (2.0 - r);
  }
  if (x > epscu) {
    const double D = epscu - epsc0, t = (x - epsc0) / D;
    *d_x = (fcu - fc) / D;
    *d_fc = 1.0 - t;
    *d_e0 = (fcu - fc) * (x - epscu) / (D * D);
    *d_fcu = t;
    return (fcu - fc) * t + fc;
  }
  *d_x = *d_fc = *d_e0 = 0.0;
  *d_fcu = 1.0;
  return fcu;
}

// Concrete02 tension envelope (Concrete02.cpp:421-446) and its partial
// derivatives in the strain and in the initial modulus Ec0 = 2 fc / epsc0
// (ft and Ets are held fixed).
XG_HD inline double c02_tens_d(double Ec0, double ft, double Ets, double x, double *d_x,
                               double *d_Ec0) {
  const double eps0 = ft / Ec0;
  const double epsu = ft * (1.0 / Ets + 1.0 / Ec0);
  if (x <= eps0) {
    *d_x = Ec0;
    *d_Ec0 = x;
    return x * Ec0;
  }
  if (x <= epsu) {
    *d_x = -Ets;
    *d_Ec0 = -Ets * ft / (Ec0 * Ec0);
    return ft - Ets * (x - eps0);
  }
  *d_x = *d_Ec0 = 0.0;
  return 0.0;
}

// Concrete02::setTrialStrain (Concrete02.cpp:167-271), swept backwards
// branch by branch: the compression envelope (three regions), unloading
// from it (the elastic step, the lower and the upper bound of the
// unloading fan), and reloading in tension towards and along the tension
// envelope.  Record fields: 0 ecmin, 1 dept, 9 sig, 10 eps.  Parameters q:
// fc epsc0 fcu epscu rat ft Ets (the constructor's sign normalisation,
// Concrete02.cpp:97-111, applies); qb receives d/d(fc, epsc0, fcu) of the
// unnormalised parameters.  A strain within DBL_EPSILON of the committed one
// keeps the previous trial stress, which after a commit is the committed
// stress.
XG_HD inline void concrete02_vjp(const double *q, const double *hc, double strain,
                                 const double *yb, double *hb, double *sb, double *qb) {
  const double s_fc = q[0] > 0 ? -1.0 : 1.0, s_e0 = q[1] > 0 ? -1.0 : 1.0;
  const double s_fcu = q[2] > 0 ? -1.0 : 1.0;
  const double fc = s_fc * q[0], epsc0 = s_e0 * q[1], fcu = s_fcu * q[2];
  const double epscu = q[3] > 0 ? -q[3] : q[3], rat = q[4], ft = q[5], Ets = q[6];
  const double eps = strain;
  const double ecmin_c = hc[0], dept_c = hc[1], sigP = hc[9], epsP = hc[10];
  const double deps = eps - epsP;
  for (int k = 0; k < 12; k++) hb[k] = 0.0;
  qb[0] = qb[1] = qb[2] = 0.0;
  if (fabs(deps) < DBL_EPSILON) {
    hb[0] = yb[0];
    hb[1] = yb[1];
    hb[9] = yb[9];
    *sb = yb[10];
    return;
  }
  const double ec0 = fc * 2. / epsc0;
  const double b_sig = yb[9];
  double b_eps = yb[10], b_fc = 0.0, b_e0 = 0.0, b_fcu = 0.0, b_ec0 = 0.0;
  double hb0 = 0.0, hb1 = 0.0, b_sigP = 0.0, b_epsP = 0.0;
  if (eps < ecmin_c) {
    // on the compression envelope; ecmin = eps
    double dx, dfc, de0, dfcu;
    c02_compr_d(fc, epsc0, fcu, epscu, eps, &dx, &dfc, &de0, &dfcu);
    b_eps += yb[0] + b_sig * dx;
    b_fc += b_sig * dfc;
    b_e0 += b_sig * de0;
    b_fcu += b_sig * dfcu;
    hb1 = yb[1];
  } else {
    hb0 = yb[0];
    const double Dn = ec0 * (1.0 - rat);
    const double epsr = (fcu - rat * ec0 * epscu) / Dn;
    const double sigmr = ec0 * epsr;
    double mdx, mdfc, mde0, mdfcu;
    const double sigmm = c02_compr_d(fc, epsc0, fcu, epscu, ecmin_c, &mdx, &mdfc, &mde0, &mdfcu);
    const double den = ecmin_c - epsr;
    const double er = (sigmm - sigmr) / den;
    const double ept = ecmin_c - sigmm / er;
    double b_er = 0.0, b_ept = 0.0, b_sigmm = 0.0;
    if (eps <= ept) {
      hb1 = yb[1];
      const double sigmin = sigmm + er * (eps - ecmin_c);
      const double sigmax = er * .5 * (eps - ept);
      double sig = sigP + ec0 * deps;
      int which = 0;
      if (sig <= sigmin) { sig = sigmin; which = 1; }
      if (sig >= sigmax) { sig = sigmax; which = 2; }
      if (which == 0) {
        b_sigP += b_sig;
        b_ec0 += b_sig * deps;
        b_eps += b_sig * ec0;
        b_epsP -= b_sig * ec0;
      } else if (which == 1) {
        b_sigmm += b_sig;
        b_er += b_sig * (eps - ecmin_c);
        b_eps += b_sig * er;
        hb0 -= b_sig * er;
      } else {
        b_er += b_sig * .5 * (eps - ept);
        b_eps += b_sig * .5 * er;
        b_ept -= b_sig * .5 * er;
      }
    } else if (eps <= ept + dept_c) {
      // towards the tension envelope's last point: sig = e (eps - ept),
      // e = sicn / dept (ec0 when dept is zero)
      hb1 = yb[1];
      double e, de_dept = 0.0, de_dEc0 = 0.0;
      if (dept_c != 0.0) {
        double tdx, tdE;
        const double sicn = c02_tens_d(ec0, ft, Ets, dept_c, &tdx, &tdE);
        e = sicn / dept_c;
        de_dept = (tdx * dept_c - sicn) / (dept_c * dept_c);
        de_dEc0 = tdE / dept_c;
      } else {
        e = ec0;
        de_dEc0 = 1.0;
      }
      const double b_e = b_sig * (eps - ept);
      b_eps += b_sig * e;
      b_ept -= b_sig * e;
      hb1 += b_e * de_dept;
      b_ec0 += b_e * de_dEc0;
    } else {
      // on the tension envelope; dept = eps - ept
      double tdx, tdE;
      c02_tens_d(ec0, ft, Ets, eps - ept, &tdx, &tdE);
      b_eps += yb[1] + b_sig * tdx;
      b_ept -= yb[1] + b_sig * tdx;
      b_ec0 += b_sig * tdE;
    }
    // ept = ecmin - sigmm / er
    hb0 += b_ept;
    b_sigmm -= b_ept / er;
    b_er += b_ept * sigmm / (er * er);
    // er = (sigmm - sigmr) / (ecmin - epsr)
    b_sigmm += b_er / den;
    const double b_sigmr = -b_er / den;
    const double b_den = -b_er * er / den;
    hb0 += b_den;
    double b_epsr = -b_den;
    // sigmm = Compr_Envlp(ecmin)
    hb0 += b_sigmm * mdx;
    b_fc += b_sigmm * mdfc;
    b_e0 += b_sigmm * mde0;
    b_fcu += b_sigmm * mdfcu;
    // sigmr = ec0 epsr, epsr = (fcu - rat ec0 epscu) / (ec0 (1 - rat))
    b_ec0 += b_sigmr * epsr;
    b_epsr += b_sigmr * ec0;
    b_fcu += b_epsr / Dn;
    b_ec0 += b_epsr * (-rat * epscu - epsr * (1.0 - rat)) / Dn;
  }
  // ec0 = 2 fc / epsc0
  b_fc += b_ec0 * 2.0 / epsc0;
  b_e0 -= b_ec0 * ec0 / epsc0;
  hb[0] = hb0;
  hb[1] = hb1;
  hb[9] = b_sigP;
  hb[10] = b_epsP;
  *sb = b_eps;
  qb[0] = s_fc * b_fc;
  qb[1] = s_e0 * b_e0;
  qb[2] = s_fcu * b_fcu;
}

// Concrete02::setTrialStrain in forward mode: the branches of the
// vector-Jacobian product above (the compression envelope, unloading from
// it between the lower and upper bounds of the unloading fan, reloading
// toward the tension envelope's last point and along the tension envelope)
// differentiated forward.  dq = d(fc, epsc0, fcu) of the unnormalised
// parameters; dht receives fields 0, 1, 9 and 10.
XG_HD inline void concrete02_jvp(const double *q, const double *hc, double strain, double dstrain,
                                 const double *dhc, const double *dq, double *dht) {
  const double s_fc = q[0] > 0 ? -1.0 : 1.0, s_e0 = q[1] > 0 ? -1.0 : 1.0;
  const double s_fcu = q[2] > 0 ? -1.0 : 1.0;
  const double fc = s_fc * q[0], epsc0 = s_e0 * q[1], fcu = s_fcu * q[2];
  const double dfc = s_fc * dq[0], de0 = s_e0 * dq[1], dfcu = s_fcu * dq[2];
  const double epscu = q[3] > 0 ? -q[3] : q[3], rat = q[4], ft = q[5], Ets = q[6];
  const double eps = strain;
  const double ecmin_c = hc[0], dept_c = hc[1], sigP = hc[9], epsP = hc[10];
  const double deps = eps - epsP;
  for (int k = 0; k < 12; k++) dht[k] = 0.0;
  if (fabs(deps) < DBL_EPSILON) {
    dht[0] = dhc[0]; dht[1] = dhc[1]; dht[9] = dhc[9]; dht[10] = dstrain;
    return;
  }
  const double ec0 = fc * 2. / epsc0;
  const double dec0 = 2.0 * dfc / epsc0 - ec0 * de0 / epsc0;
  double dsig = 0.0, t_ecmin = dhc[0], t_dept = dhc[1];
  if (eps < ecmin_c) {
    double dx, dfc_, de0_, dfcu_;
    c02_compr_d(fc, epsc0, fcu, epscu, eps, &dx, &dfc_, &de0_, &dfcu_);
    dsig = dx * dstrain + dfc_ * dfc + de0_ * de0 + dfcu_ * dfcu;
    t_ecmin = dstrain;
  } else {
    const double Dn = ec0 * (1.0 - rat);
    const double epsr = (fcu - rat * ec0 * epscu) / Dn;
    const double t_epsr = dfcu / Dn + dec0 * (-rat * epscu - epsr * (1.0 - rat)) / Dn;
    const double sigmr = ec0 * epsr, t_sigmr = dec0 * epsr + ec0 * t_epsr;
    double mdx, mdfc, mde0, mdfcu;
    const double sigmm = c02_compr_d(fc, epsc0, fcu, epscu, ecmin_c, &mdx, &mdfc, &mde0, &mdfcu);
    const double t_sigmm = mdx * dhc[0] + mdfc * dfc + mde0 * de0 + mdfcu * dfcu;
    const double den = ecmin_c - epsr, t_den = dhc[0] - t_epsr;
    const double er = (sigmm - sigmr) / den;
    const double t_er = (t_sigmm - t_sigmr) / den - er * t_den / den;
    const double ept = ecmin_c - sigmm / er;
    const double t_ept = dhc[0] - t_sigmm / er + sigmm * t_er / (er * er);
    if (eps <= ept) {
      const double sigmin = sigmm + er * (eps - ecmin_c);
      const double sigmax = er * .5 * (eps - ept);
      double sig = sigP + ec0 * deps;
      int which = 0;
      if (sig <= sigmin) { sig = sigmin; which = 1; }
      if (sig >= sigmax) { sig = sigmax; which = 2; }
      if (which == 0) dsig = dhc[9] + dec0 * deps + ec0 * (dstrain - dhc[10]);
      else if (which == 1) dsig = t_sigmm + t_er * (eps - ecmin_c) + er * (dstrain - dhc[0]);
      else dsig = .5 * t_er * (eps - ept) + .5 * er * (dstrain - t_ept);
    } else if (eps <= ept + dept_c) {
      double e, t_e;
      if (dept_c != 0.0) {
        double tdx, tdE;
        const double sicn = c02_tens_d(ec0, ft, Ets, dept_c, &tdx, &tdE);
        e = sicn / dept_c;
        t_e = (tdx * dept_c - sicn) / (dept_c * dept_c) * dhc[1] + tdE / dept_c * dec0;
      } else {
        e = ec0;
        t_e = dec0;
      }
      dsig = t_e * (eps - ept) + e * (dstrain - t_ept);
    } else {
      double tdx, tdE;
      c02_tens_d(ec0, ft, Ets, eps - ept, &tdx, &tdE);
      t_dept = dstrain - t_ept;
      dsig = tdx * t_dept + tdE * dec0;
    }
  }
  dht[0] = t_ecmin;
  dht[1] = t_dept;
  dht[9] = dsig;
  dht[10] = dstrain;
}

// Elastic fiber: sig = E eps (parameter 0).
// Steel01::setTrialStrain / determineTrialState (material/uniaxial/steel/
// Steel01.cpp:68-92, 124-198), swept backwards: the stress is one of the
// elastic predictor Cstress + E0 dStrain, the upper bound b E0 eps +
// shiftP fy (1 - b) or the lower bound b E0 eps - shiftN fy (1 - b) (the
// primal is recomputed to find which); at a load reversal the new shift is
// 1 + a (dmax / (2 a' epsy))^0.8 with epsy = fy / E0 and the extreme strain
// taken from the committed strain when it goes further.  Parameters q: fy
// E0 b a1 a2 a3 a4; qb receives d/d(fy, E0, b).
XG_HD inline void steel01_vjp(const double *q, const double *hc, double strain, const double *yb,
                              double *hb, double *sb, double *qb) {
  const double fy = q[0], E0 = q[1], b = q[2], a1 = q[3], a2 = q[4], a3 = q[5], a4 = q[6];
  for (int k = 0; k < 12; k++) hb[k] = 0.0;
  qb[0] = qb[1] = qb[2] = 0.0;
  *sb = 0.0;
  const double Cstrain = hc[10], Cstress = hc[9];
  const double dStrain = strain - Cstrain;
  if (!(fabs(dStrain) > DBL_EPSILON)) {
    // the committed state passes through unchanged
    hb[0] = yb[0]; hb[1] = yb[1]; hb[2] = yb[2]; hb[3] = yb[3];
    hb[9] = yb[9]; hb[10] = yb[10];
    return;
  }
  const double fyomb = fy * (1.0 - b), epsy = fy / E0;
  const double c1 = b * E0 * strain, c2 = hc[3] * fyomb, c3 = hc[2] * fyomb;
  const double c = Cstress + E0 * dStrain;
  int branch = 0;                       // 0 predictor, 1 upper bound, 2 lower bound
  double t = c;
  if (c1 + c3 < c) { t = c1 + c3; branch = 1; }
  if (c1 - c2 > t) branch = 2;
  int loading = (int)hc[4];
  if (loading == 0) loading = dStrain > 0.0 ? 1 : -1;
  const bool revN = loading == 1 && dStrain < 0.0;
  const bool revP = !revN && loading == -1 && dStrain > 0.0;
  double gTmin = yb[0], gTmax = yb[1], gEps = yb[10], gEpsy = 0.0;
  double gFy = 0.0, gE0 = 0.0, gB = 0.0, gCstrain = 0.0, gCstress = 0.0;
  double gShiftP = 0.0, gShiftN = 0.0;
  if (revN || revP) {
    const double Tmin = revP && Cstrain < hc[0] ? Cstrain : hc[0];
    const double Tmax = revN && Cstrain > hc[1] ? Cstrain : hc[1];
    const double a = revN ? a1 : a3, den = 2.0 * (revN ? a2 : a4) * epsy;
    const double X = (Tmax - Tmin) / den;
    const double gShift = revN ? yb[3] : yb[2];
    const double gX = (a != 0.0 && X > 0.0) ? gShift * a * 0.8 * pow(X, -0.2) : 0.0;
    gTmax += gX / den;
    gTmin -= gX / den;
    gEpsy -= gX * X / epsy;
    if (revN) {
      gShiftP += yb[2];                 // the other shift passes through
      if (Cstrain > hc[1]) { gCstrain += gTmax; gTmax = 0.0; }
    } else {
      gShiftN += yb[3];
      if (Cstrain < hc[0]) { gCstrain += gTmin; gTmin = 0.0; }
    }
  } else {
    gShiftP += yb[2];
    gShiftN += yb[3];
  }
  const double gs = yb[9];
  if (branch == 0) {
    gCstress += gs;
    gE0 += gs * dStrain;
    gEps += gs * E0;
    gCstrain -= gs * E0;
  } else if (branch == 1) {
    gB += gs * (E0 * strain - hc[2] * fy);
    gE0 += gs * b * strain;
    gEps += gs * b * E0;
    gShiftP += gs * fyomb;
    gFy += gs * hc[2] * (1.0 - b);
  } else {
    gB += gs * (E0 * strain + hc[3] * fy);
    gE0 += gs * b * strain;
    gEps += gs * b * E0;
    gShiftN -= gs * fyomb;
    gFy -= gs * hc[3] * (1.0 - b);
  }
  gFy += gEpsy / E0;
  gE0 -= gEpsy * fy / (E0 * E0);
  hb[0] = gTmin; hb[1] = gTmax; hb[2] = gShiftP; hb[3] = gShiftN;
  hb[9] = gCstress; hb[10] = gCstrain;
  *sb = gEps;
  qb[0] = gFy; qb[1] = gE0; qb[2] = gB;
}

// Steel01::setTrialStrain / determineTrialState (Steel01.cpp:68-92,
// 124-198) in forward mode, written from the law itself (the reference's own
// DDM, Steel01::getStressSensitivity / commitSensitivity, Steel01.cpp:
// 552-660, is the quantity it is checked against).  The branch (elastic
// predictor, upper or lower bound, a load reversal) is the primal's; the
// bounds use the committed shifts; a reversal sets the new shift from the
// extreme strains.  dq = d(fy, E0, b); dht receives fields 0-3, 9, 10.
XG_HD inline void steel01_jvp(const double *q, const double *hc, double strain, double dstrain,
                              const double *dhc, const double *dq, double *dht) {
  const double fy = q[0], E0 = q[1], b = q[2], a1 = q[3], a2 = q[4], a3 = q[5], a4 = q[6];
  const double dfy = dq[0], dE0 = dq[1], db = dq[2];
  for (int k = 0; k < 12; k++) dht[k] = 0.0;
  const double Cstrain = hc[10], Cstress = hc[9];
  const double dStrain = strain - Cstrain;
  if (!(fabs(dStrain) > DBL_EPSILON)) {
    // the committed state is the trial state, strain included
    dht[0] = dhc[0]; dht[1] = dhc[1]; dht[2] = dhc[2]; dht[3] = dhc[3];
    dht[9] = dhc[9]; dht[10] = dhc[10];
    return;
  }
  const double fyomb = fy * (1.0 - b), dfyomb = dfy * (1.0 - b) - fy * db;
  const double epsy = fy / E0, depsy = dfy / E0 - fy * dE0 / (E0 * E0);
  const double c1 = b * E0 * strain, c2 = hc[3] * fyomb, c3 = hc[2] * fyomb;
  const double c = Cstress + E0 * dStrain;
  int branch = 0;                       // 0 predictor, 1 upper bound, 2 lower bound
  double t = c;
  if (c1 + c3 < c) { t = c1 + c3; branch = 1; }
  if (c1 - c2 > t) branch = 2;
  int loading = (int)hc[4];
  if (loading == 0) loading = dStrain > 0.0 ? 1 : -1;
  const bool revN = loading == 1 && dStrain < 0.0;
  const bool revP = !revN && loading == -1 && dStrain > 0.0;
  double dTmin = dhc[0], dTmax = dhc[1], dShiftP = dhc[2], dShiftN = dhc[3];
  if (revN || revP) {
    double Tmin = hc[0], Tmax = hc[1];
    if (revP && Cstrain < hc[0]) { Tmin = Cstrain; dTmin = dhc[10]; }
    if (revN && Cstrain > hc[1]) { Tmax = Cstrain; dTmax = dhc[10]; }
    const double a = revN ? a1 : a3, den = 2.0 * (revN ? a2 : a4) * epsy;
    const double X = (Tmax - Tmin) / den;
    const double dX = (dTmax - dTmin) / den - X * depsy / epsy;
    const double dShift = (a != 0.0 && X > 0.0) ? a * 0.8 * pow(X, -0.2) * dX : 0.0;
    if (revN) dShiftN = dShift;
    else dShiftP = dShift;
  }
  const double dEsh = db * E0 + b * dE0;
  double ds;
  if (branch == 0) ds = dhc[9] + dE0 * dStrain + E0 * (dstrain - dhc[10]);
  else if (branch == 1) ds = dEsh * strain + b * E0 * dstrain + dhc[2] * fyomb + hc[2] * dfyomb;
  else ds = dEsh * strain + b * E0 * dstrain - dhc[3] * fyomb - hc[3] * dfyomb;
  dht[0] = dTmin; dht[1] = dTmax; dht[2] = dShiftP; dht[3] = dShiftN;
  dht[9] = ds; dht[10] = dstrain;
}

// Concrete01 (material/uniaxial/concrete/Concrete01.cpp:209-385) in both
// modes.  Parameters q = fpc epsc0 fpcu epscu, made negative as the
// constructor does (:89-112); the derivatives are taken with respect to
// q[0..2] as given (sg = d internal / d q = -1 for a positive entry).
// Record: 0 minStrain 1 endStrain 2 unloadSlope, 9 stress, 10 strain.  The
// branches are the primal's: the committed state kept (a strain within
// DBL_EPSILON), tension (no stress), a new extreme compression strain (the
// Kent-Scott-Park envelope, then the unloading slope and end strain from the
// Karsan-Jirsa ratio), reloading on the committed unloading line, or the
// elastic return line Cstress + slope (eps - Cstrain) where it governs.
struct C01d {
  double fpc, epsc0, fpcu, epscu, sg0, sg1, sg2;
};
XG_HD inline C01d c01d_params(const double *q) {
  C01d c;
  c.fpc = q[0] > 0.0 ? -q[0] : q[0];
  c.sg0 = q[0] > 0.0 ? -1.0 : 1.0;
  c.epsc0 = q[1] > 0.0 ? -q[1] : q[1];
  c.sg1 = q[1] > 0.0 ? -1.0 : 1.0;
  c.fpcu = q[2] > 0.0 ? -q[2] : q[2];
  c.sg2 = q[2] > 0.0 ? -1.0 : 1.0;
  c.epscu = q[3] > 0.0 ? -q[3] : q[3];
  return c;
}

// the new extreme strain's primal quantities (envelope and unloading)
struct C01Env {
  int env;                  // 0 parabola, 1 linear descent, 2 crushed
  int unl;                  // 0 slope Ec0 (no room), 1 secant to the end strain, 2 Ec0 line
  bool clamp;               // the unloading ratio reads epscu
  double Ec0, eta, t, den, sig, ts, etau, ratio, rprime, endS0, temp1, temp2;
};
XG_HD inline C01Env c01_envelope(const C01d &c, double strain) {
  C01Env v;
  v.Ec0 = 2.0 * c.fpc / c.epsc0;
  v.eta = v.t = v.den = 0.0;
  if (strain > c.epsc0) {
    v.env = 0;
    v.eta = strain / c.epsc0;
    v.sig = c.fpc * (2 * v.eta - v.eta * v.eta);
  } else if (strain > c.epscu) {
    v.env = 1;
    v.den = c.epsc0 - c.epscu;
    v.t = (c.fpc - c.fpcu) / v.den;
    v.sig = c.fpc + v.t * (strain - c.epsc0);
  } else {
    v.env = 2;
    v.sig = c.fpcu;
  }
  v.clamp = strain < c.epscu;
  v.ts = v.clamp ? c.epscu : strain;
  v.etau = v.ts / c.epsc0;
  if (v.etau < 2.0) {
    v.ratio = 0.145 * v.etau * v.etau + 0.13 * v.etau;
    v.rprime = 0.29 * v.etau + 0.13;
  } else {
    v.ratio = 0.707 * (v.etau - 2.0) + 0.834;
    v.rprime = 0.707;
  }
  v.endS0 = v.ratio * c.epsc0;
  v.temp1 = strain - v.endS0;
  v.temp2 = v.sig / v.Ec0;
  v.unl = v.temp1 > -DBL_EPSILON ? 0 : (v.temp1 <= v.temp2 ? 1 : 2);
  return v;
}

XG_HD inline void concrete01_jvp(const double *q, const double *hc, double strain, double dstrain,
                                 const double *dhc, const double *dq, double *dht) {
  const C01d c = c01d_params(q);
  const double dfpc = c.sg0 * dq[0], de0 = c.sg1 * dq[1], dfpcu = c.sg2 * dq[2];
  for (int k = 0; k < 12; k++) dht[k] = 0.0;
  const double Cstrain = hc[10], Cstress = hc[9];
  if (fabs(strain - Cstrain) < DBL_EPSILON) {
    dht[0] = dhc[0]; dht[1] = dhc[1]; dht[2] = dhc[2]; dht[9] = dhc[9]; dht[10] = dhc[10];
    return;
  }
  double dmin = dhc[0], dend = dhc[1], dslope = dhc[2], ds = 0.0;
  dht[10] = dstrain;
  if (!(strain > 0.0)) {
    const double slope = hc[2];
    const double temp = Cstress + slope * strain - slope * Cstrain;
    const double dtemp = dhc[9] + dhc[2] * (strain - Cstrain) + slope * (dstrain - dhc[10]);
    if (strain <= Cstrain) {
      double stress;
      if (strain <= hc[0]) {
        const C01Env v = c01_envelope(c, strain);
        const double e02 = c.epsc0 * c.epsc0;
        const double dEc0 = 2.0 * dfpc / c.epsc0 - 2.0 * c.fpc * de0 / e02;
        double dsig;
        if (v.env == 0) {
          const double deta = dstrain / c.epsc0 - strain * de0 / e02;
          dsig = dfpc * (2 * v.eta - v.eta * v.eta) + c.fpc * (2.0 - 2.0 * v.eta) * deta;
        } else if (v.env == 1) {
          const double dt = (dfpc - dfpcu) / v.den - v.t * de0 / v.den;
          dsig = dfpc + dt * (strain - c.epsc0) + v.t * (dstrain - de0);
        } else {
          dsig = dfpcu;
        }
        dmin = dstrain;
        const double dts = v.clamp ? 0.0 : dmin;
        const double detau = dts / c.epsc0 - v.ts * de0 / e02;
        const double dend0 = v.rprime * detau * c.epsc0 + v.ratio * de0;
        const double dtemp1 = dmin - dend0;
        const double dtemp2 = dsig / v.Ec0 - v.sig * dEc0 / (v.Ec0 * v.Ec0);
        if (v.unl == 0) {
          dslope = dEc0;
          dend = dend0;
        } else if (v.unl == 1) {
          dend = dmin - dtemp1;
          dslope = dsig / v.temp1 - v.sig * dtemp1 / (v.temp1 * v.temp1);
        } else {
          dend = dmin - dtemp2;
          dslope = dEc0;
        }
        stress = v.sig;
        ds = dsig;
      } else if (strain <= hc[1]) {
        stress = slope * (strain - hc[1]);
        ds = dhc[2] * (strain - hc[1]) + slope * (dstrain - dhc[1]);
      } else {
        stress = 0.0;
      }
      if (temp > stress) ds = dtemp;
    } else if (temp <= 0.0) {
      ds = dtemp;
    }
  }
  dht[0] = dmin; dht[1] = dend; dht[2] = dslope; dht[9] = ds;
}

XG_HD inline void concrete01_vjp(const double *q, const double *hc, double strain, const double *yb,
                                 double *hb, double *sb, double *qb) {
  const C01d c = c01d_params(q);
  for (int k = 0; k < 12; k++) hb[k] = 0.0;
  qb[0] = qb[1] = qb[2] = 0.0;
  *sb = 0.0;
  const double Cstrain = hc[10], Cstress = hc[9];
  if (fabs(strain - Cstrain) < DBL_EPSILON) {
    hb[0] = yb[0]; hb[1] = yb[1]; hb[2] = yb[2]; hb[9] = yb[9]; hb[10] = yb[10];
    return;
  }
  double g_eps = yb[10];
  if (strain > 0.0) {
    hb[0] = yb[0]; hb[1] = yb[1]; hb[2] = yb[2];
    *sb = g_eps;
    return;
  }
  const double gs = yb[9];
  const double slope = hc[2];
  const double temp = Cstress + slope * strain - slope * Cstrain;
  double g_temp = 0.0, g_fpc = 0.0, g_e0 = 0.0, g_fpcu = 0.0;
  if (strain <= Cstrain) {
    if (strain <= hc[0]) {
      const C01Env v = c01_envelope(c, strain);
      const bool use_temp = temp > v.sig;
      const double e02 = c.epsc0 * c.epsc0;
      double g_sig = use_temp ? 0.0 : gs;
      if (use_temp) g_temp = gs;
      double g_min = yb[0], g_Ec0 = 0.0, g_end0 = 0.0, g_temp1 = 0.0, g_temp2 = 0.0;
      const double gend = yb[1], gslope = yb[2];
      if (v.unl == 0) {
        g_Ec0 += gslope;
        g_end0 += gend;
      } else if (v.unl == 1) {
        g_min += gend;
        g_temp1 -= gend;
        g_sig += gslope / v.temp1;
        g_temp1 -= gslope * v.sig / (v.temp1 * v.temp1);
      } else {
        g_min += gend;
        g_temp2 -= gend;
        g_Ec0 += gslope;
      }
      g_sig += g_temp2 / v.Ec0;
      g_Ec0 -= g_temp2 * v.sig / (v.Ec0 * v.Ec0);
      g_min += g_temp1;
      g_end0 -= g_temp1;
      const double g_etau = g_end0 * c.epsc0 * v.rprime;
      g_e0 += g_end0 * v.ratio;
      if (!v.clamp) g_min += g_etau / c.epsc0;
      g_e0 -= g_etau * v.ts / e02;
      if (v.env == 0) {
        g_fpc += g_sig * (2 * v.eta - v.eta * v.eta);
        const double g_eta = g_sig * c.fpc * (2.0 - 2.0 * v.eta);
        g_eps += g_eta / c.epsc0;
        g_e0 -= g_eta * strain / e02;
      } else if (v.env == 1) {
        g_fpc += g_sig;
        const double g_t = g_sig * (strain - c.epsc0);
        g_eps += g_sig * v.t;
        g_e0 -= g_sig * v.t;
        g_fpc += g_t / v.den;
        g_fpcu -= g_t / v.den;
        g_e0 -= g_t * v.t / v.den;
      } else {
        g_fpcu += g_sig;
      }
      g_fpc += 2.0 * g_Ec0 / c.epsc0;
      g_e0 -= 2.0 * g_Ec0 * c.fpc / e02;
      g_eps += g_min;
    } else {
      hb[0] = yb[0]; hb[1] = yb[1]; hb[2] = yb[2];
      if (strain <= hc[1]) {
        const double stress = slope * (strain - hc[1]);
        if (temp > stress) {
          g_temp = gs;
        } else {
          hb[2] += gs * (strain - hc[1]);
          g_eps += gs * slope;
          hb[1] -= gs * slope;
        }
      } else if (temp > 0.0) {
        g_temp = gs;
      }
    }
  } else {
    hb[0] = yb[0]; hb[1] = yb[1]; hb[2] = yb[2];
    if (temp <= 0.0) g_temp = gs;
  }
  hb[9] += g_temp;
  hb[2] += g_temp * (strain - Cstrain);
  g_eps += g_temp * slope;
  hb[10] -= g_temp * slope;
  *sb = g_eps;
  qb[0] = c.sg0 * g_fpc;
  qb[1] = c.sg1 * g_e0;
  qb[2] = c.sg2 * g_fpcu;
}

// the elastic law sigma = E eps in forward mode (dq[0] = dE)
XG_HD inline void elastic_jvp(const double *q, double strain, double dstrain, const double *dq,
                              double *dht) {
  for (int k = 0; k < 12; k++) dht[k] = 0.0;
  dht[9] = dq[0] * strain + q[0] * dstrain;
  dht[10] = dstrain;
}

XG_HD inline void elastic_vjp(const double *q, double strain, const double *yb, double *hb,
                              double *sb, double *qb) {
  for (int k = 0; k < 12; k++) hb[k] = 0.0;
  *sb = q[0] * yb[9] + yb[10];
  qb[0] = strain * yb[9];
  qb[1] = qb[2] = 0.0;
}

}  // namespace xg
