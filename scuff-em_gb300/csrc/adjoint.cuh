// adjoint.cuh -- reverse-mode derivatives of the far-field panel-pair
// integrals with respect to the panels' vertices (host and device).
//
// For two panels a, b (vertices V_0..V_2 in mesh order, x = V_0 + u A + v B)
// and complex coefficients C0[ja][jb], C1[ja][jb] over the nine (Qa, Qb)
// choices (Q = a vertex of its panel), the far-field value
//   S = sum_{ja,jb} C0 H0(ja,jb) + C1 H1(ja,jb),
//   H0 = int int (F_a . F_b - 4/k^2) G,   H1 = int int (F_a x F_b) . grad_x G,
//   F = x - Q,  G = e^{ikr}/(4 pi r),  grad_x G = Psi R,  R = x - x'
// (PanelPanelInteractions.cc:108-201 with the 6x6 rule of the far field) is
// differentiated by hand in reverse mode: the sums over (ja, jb) collapse
// into a few coefficient vectors, so each cubature sample costs one
// evaluation of G, Psi and Zeta = Psi'(r)/r plus ~200 flops for both
// positions' gradients, and the Q-dependence follows from nine moments
// accumulated over the samples.  Only Re S is wanted (the vertices are
// real), so the sample gradients are folded into 18 real accumulators.
//
//   dS/dx  = G (c0 xi' - qb0) + Psi (T0 R + (c1 xi' - qb1) x R + V1) + Zeta T1 R
//   dS/dx' = G (c0 xi - qa0) + Psi (-T0 R + R x (c1 xi - qa1) - V1) - Zeta T1 R
// with xi = x - V0a, xi' = x' - V0b, alpha_j = V_j(a) - V0a, beta_j likewise,
//   T0 = c0 xi.xi' - xi.qb0 - xi'.qa0 + qq0 + m c0        (m = -4/k^2)
//   V1 = c1 xi x xi' - xi x qb1 - qa1 x xi' + X1,  T1 = V1 . R
//   c = sum C,  qa = sum C alpha_ja,  qb = sum C beta_jb,  qq0 = sum C0 alpha.beta,
//   X1 = sum C1 alpha x beta.
// x = (1-u-v) V0 + u V1 + v V2 distributes dS/dx over the three vertices.
#pragma once
#include "bem_math.cuh"

namespace gbem {

GB_HD cx<double> operator*(cx<double> a, double s) { return mk(s * a.re, s * a.im); }

GB_HD cx<double> rcdot(const double* a, const cx<double>* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
GB_HD void cvcross(const cx<double>* a, const double* b, cx<double>* c) {  // complex x real
  c[0] = a[1] * b[2] - a[2] * b[1];
  c[1] = a[2] * b[0] - a[0] * b[2];
  c[2] = a[0] * b[1] - a[1] * b[0];
}
GB_HD void rcvcross(const double* a, const cx<double>* b, cx<double>* c) {  // real x complex
  c[0] = a[1] * b[2] - a[2] * b[1];
  c[1] = a[2] * b[0] - a[0] * b[2];
  c[2] = a[0] * b[1] - a[1] * b[0];
}
GB_HD void ccross(const cx<double>* a, const cx<double>* b, cx<double>* c) {  // complex x complex
  c[0] = a[1] * b[2] - a[2] * b[1];
  c[1] = a[2] * b[0] - a[0] * b[2];
  c[2] = a[0] * b[1] - a[1] * b[0];
}

// Accumulates into gA[9], gB[9] the gradient of Re S with respect to the
// vertices of panels a and b at fixed coefficients, and writes the real
// parts of the per-slot partial sums Er[ja] = sum_jb (C0 H0 + C1 H1),
// Ec[jb] = sum_ja (...), which carry the dependence on the edge lengths when
// the coefficients hold La Lb.  rule: npts (u, v, w) triples.
GB_HD void far_pair_vjp(const double* Va, const double* Vb, cx<double> k, const cx<double>* C0, const cx<double>* C1,
                        const double* rule, int npts, double* gA, double* gB, double* Er, double* Ec) {
  double Aa[3], Ba[3], Ab[3], Bb[3], D0[3], al[3][3], be[3][3];
  for (int c = 0; c < 3; c++) {
    Aa[c] = Va[3 + c] - Va[c]; Ba[c] = Va[6 + c] - Va[c];
    Ab[c] = Vb[3 + c] - Vb[c]; Bb[c] = Vb[6 + c] - Vb[c];
    D0[c] = Va[c] - Vb[c];
    al[0][c] = 0.0; al[1][c] = Aa[c]; al[2][c] = Ba[c];
    be[0][c] = 0.0; be[1][c] = Ab[c]; be[2][c] = Bb[c];
  }
  const cx<double> zero = mk(0.0, 0.0);
  // coefficient reductions
  cx<double> c0 = zero, c1 = zero, rs0[3], rs1[3], cs0[3], cs1[3];
  cx<double> B0[3][3], B1[3][3], A0[3][3], A1[3][3];  // B0[ja] = sum_jb C0 beta_jb, A0[jb] = sum_ja C0 alpha_ja
  cx<double> qq0 = zero, X1[3] = {zero, zero, zero};
  for (int j = 0; j < 3; j++) {
    rs0[j] = rs1[j] = cs0[j] = cs1[j] = zero;
    for (int c = 0; c < 3; c++) B0[j][c] = B1[j][c] = A0[j][c] = A1[j][c] = zero;
  }
  for (int ja = 0; ja < 3; ja++)
    for (int jb = 0; jb < 3; jb++) {
      const cx<double> p = C0[3 * ja + jb], q = C1[3 * ja + jb];
      c0 = c0 + p; c1 = c1 + q;
      rs0[ja] = rs0[ja] + p; rs1[ja] = rs1[ja] + q;
      cs0[jb] = cs0[jb] + p; cs1[jb] = cs1[jb] + q;
      double axb[3];
      vcross(al[ja], be[jb], axb);
      qq0 = qq0 + vdot(al[ja], be[jb]) * p;
      for (int c = 0; c < 3; c++) {
        B0[ja][c] = B0[ja][c] + be[jb][c] * p; B1[ja][c] = B1[ja][c] + be[jb][c] * q;
        A0[jb][c] = A0[jb][c] + al[ja][c] * p; A1[jb][c] = A1[jb][c] + al[ja][c] * q;
        X1[c] = X1[c] + axb[c] * q;
      }
    }
  cx<double> qa0[3], qb0[3], qa1[3], qb1[3];
  for (int c = 0; c < 3; c++) {
    qa0[c] = A0[0][c] + A0[1][c] + A0[2][c];
    qa1[c] = A1[0][c] + A1[1][c] + A1[2][c];
    qb0[c] = B0[0][c] + B0[1][c] + B0[2][c];
    qb1[c] = B1[0][c] + B1[1][c] + B1[2][c];
  }
  const cx<double> ik = mk(-k.im, k.re);
  const cx<double> mk2 = ik * ik;  // -k^2
  const cx<double> m = cdiv(mk(-4.0, 0.0), k * k);
  const cx<double> T0c = qq0 + m * c0;
  // moments: G, G xi, G xi', G xi.xi', Psi R, Psi xi x R, Psi xi' x R, Psi (xi x xi').R
  cx<double> Mg = zero, Mgx[3], Mgy[3], Mgxy = zero, MpR[3], MpxR[3], MpyR[3], MpT = zero;
  for (int c = 0; c < 3; c++) Mgx[c] = Mgy[c] = MpR[c] = MpxR[c] = MpyR[c] = zero;
  const double inv4pi = 0.079577471545947667884;
  for (int i = 0; i < npts; i++) {
    const double u = rule[3 * i], v = rule[3 * i + 1], wi = rule[3 * i + 2];
    double xi[3];
    for (int c = 0; c < 3; c++) xi[c] = u * Aa[c] + v * Ba[c];
    // xi-dependent coefficient vectors: Pa = c1 xi - qa1, Ga = c0 xi - qa0
    cx<double> Pa[3], Ga[3];
    for (int c = 0; c < 3; c++) { Pa[c] = xi[c] * c1 - qa1[c]; Ga[c] = xi[c] * c0 - qa0[c]; }
    double gx[3] = {0.0, 0.0, 0.0};
    for (int j = 0; j < npts; j++) {
      const double up = rule[3 * j], vp = rule[3 * j + 1], wj = rule[3 * j + 2];
      double yp[3], R[3];
      for (int c = 0; c < 3; c++) {
        yp[c] = up * Ab[c] + vp * Bb[c];
        R[c] = D0[c] + xi[c] - yp[c];
      }
      const double r2 = vdot(R, R), r = sqrt(r2), ri = 1.0 / r;
      double sn, cs;
      sincos_t(k.re * r, &sn, &cs);
      double amp = wi * wj * inv4pi * ri;
      if (k.im != 0.0) amp *= exp(-k.im * r);
      const cx<double> G = mk(amp * cs, amp * sn);
      const cx<double> Psi = G * mk((-k.im - ri) * ri, k.re * ri);
      // Zeta = G (3 - 3ikr - k^2 r^2) / r^4
      const cx<double> Zeta = G * ((mk(3.0, 0.0) - (3.0 * r) * ik + r2 * mk2) * (ri * ri * ri * ri));
      // T0, V1, T1
      cx<double> T0 = c0 * vdot(xi, yp) + T0c;
      double xy[3];
      vcross(xi, yp, xy);
      cx<double> xq[3], qy[3];  // xi x qb1, qa1 x xi'
      rcvcross(xi, qb1, xq);
      cvcross(qa1, yp, qy);
      cx<double> V1[3];
      for (int c = 0; c < 3; c++) {
        T0 = T0 - xi[c] * qb0[c] - yp[c] * qa0[c];
        V1[c] = xy[c] * c1 - xq[c] - qy[c] + X1[c];
      }
      const cx<double> T1 = V1[0] * R[0] + V1[1] * R[1] + V1[2] * R[2];
      // Pb = c1 xi' - qb1, Gb = c0 xi' - qb0
      cx<double> Pb[3], Gb[3], PbxR[3], RxPa[3];
      for (int c = 0; c < 3; c++) { Pb[c] = yp[c] * c1 - qb1[c]; Gb[c] = yp[c] * c0 - qb0[c]; }
      cvcross(Pb, R, PbxR);
      rcvcross(R, Pa, RxPa);
      const cx<double> PT = Psi * T0, ZT = Zeta * T1;
      const double bu = 1.0 - up - vp;
      for (int c = 0; c < 3; c++) {
        const cx<double> rad = PT * R[c] + ZT * R[c];
        const double gxc = (G * Gb[c] + Psi * (PbxR[c] + V1[c]) + rad).re;
        const double gyc = (G * Ga[c] + Psi * (RxPa[c] - V1[c]) - rad).re;
        gx[c] += gxc;
        gB[c] += bu * gyc; gB[3 + c] += up * gyc; gB[6 + c] += vp * gyc;
      }
      // moments
      double xR[3], yR[3];
      vcross(xi, R, xR);
      vcross(yp, R, yR);
      Mg = Mg + G;
      Mgxy = Mgxy + vdot(xi, yp) * G;
      MpT = MpT + vdot(xy, R) * Psi;
      for (int c = 0; c < 3; c++) {
        Mgx[c] = Mgx[c] + xi[c] * G; Mgy[c] = Mgy[c] + yp[c] * G;
        MpR[c] = MpR[c] + R[c] * Psi; MpxR[c] = MpxR[c] + xR[c] * Psi; MpyR[c] = MpyR[c] + yR[c] * Psi;
      }
    }
    const double bu = 1.0 - u - v;
    for (int c = 0; c < 3; c++) { gA[c] += bu * gx[c]; gA[3 + c] += u * gx[c]; gA[6 + c] += v * gx[c]; }
  }
  // Q_ja = vertex ja of panel a, Q_jb = vertex jb of panel b:
  //   dS/dQ_ja = -[rs0 Mgy - B0 Mg + rs1 MpyR - B1 x MpR]
  //   dS/dQ_jb = -[cs0 Mgx - A0 Mg - cs1 MpxR - MpR x A1]
  // per-slot sums (the C0 part, then the C1 part):
  //   Er = rs0 Mgxy - B0.Mgx - rs0 al.Mgy + (al.B0 + m rs0) Mg
  //        + rs1 MpT + B1.MpxR - rs1 al.MpyR + (al x B1).MpR
  //   Ec = cs0 Mgxy - cs0 be.Mgx - A0.Mgy + (A0.be + m cs0) Mg
  //        + cs1 MpT + cs1 be.MpxR - A1.MpyR + (A1 x be).MpR
  for (int j = 0; j < 3; j++) {
    cx<double> b1xR[3], Rxa1[3], axb1[3], a1xb[3];
    ccross(B1[j], MpR, b1xR);
    ccross(MpR, A1[j], Rxa1);
    rcvcross(al[j], B1[j], axb1);
    cvcross(A1[j], be[j], a1xb);
    cx<double> er = rs0[j] * Mgxy + (rcdot(al[j], B0[j]) + m * rs0[j]) * Mg + rs1[j] * MpT;
    cx<double> ec = cs0[j] * Mgxy + (rcdot(be[j], A0[j]) + m * cs0[j]) * Mg + cs1[j] * MpT;
    for (int c = 0; c < 3; c++) {
      gA[3 * j + c] -= (rs0[j] * Mgy[c] - B0[j][c] * Mg + rs1[j] * MpyR[c] - b1xR[c]).re;
      gB[3 * j + c] -= (cs0[j] * Mgx[c] - A0[j][c] * Mg - cs1[j] * MpxR[c] - Rxa1[c]).re;
      er = er - B0[j][c] * Mgx[c] - (rs0[j] * al[j][c]) * Mgy[c] + B1[j][c] * MpxR[c] -
           (rs1[j] * al[j][c]) * MpyR[c] + axb1[c] * MpR[c];
      ec = ec - (cs0[j] * be[j][c]) * Mgx[c] - A0[j][c] * Mgy[c] + (cs1[j] * be[j][c]) * MpxR[c] -
           A1[j][c] * MpyR[c] + a1xb[c] * MpR[c];
    }
    Er[j] = er.re;
    Ec[j] = ec.re;
  }
}

}  // namespace gbem
