// Host-side check of the float-float far-field arithmetic (ffmath.cuh): the
// same header the mixed-precision tile kernel uses, compiled for the host.
// Prints the largest errors against FP64 evaluations of the same sums.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include "../scuff-em_gb300/csrc/ffmath.cuh"
using namespace gbem;

// the 6-point rule of the far field (libs/libTriInt/TCR.cc:83-91)
static const double RULE6[18] = {
    0.0915762135098, 0.0915762135098, 0.0549758718276, 0.8168475729805, 0.0915762135098, 0.0549758718276,
    0.0915762135098, 0.8168475729805, 0.0549758718276, 0.1081030181681, 0.4459484909160, 0.1116907948390,
    0.4459484909160, 0.1081030181681, 0.1116907948390, 0.4459484909160, 0.4459484909160, 0.1116907948390};

static double urand(unsigned* s) {
  *s = *s * 1664525u + 1013904223u;
  return (*s >> 8) * (1.0 / 16777216.0);
}

int main() {
  SinCosTab T;
  fill_sincos_tab(&T);
  FFRule R;
  fill_ff_rule(RULE6, &R);
  unsigned seed = 12345;
  // e^{ix}
  double e_expi = 0;
  for (int t = 0; t < 100000; t++) {
    const double x = 200.0 * urand(&seed);
    const ff xf = ff_of(x);
    const cff e = expi_ff(xf, &T);
    const double xx = ff_d(xf);
    e_expi = fmax(e_expi, fabs(ff_d(e.re) - cos(xx)) + fabs(ff_d(e.im) - sin(xx)));
  }
  // moments and H0/H1 of random far panel pairs against FP64
  double e_mg = 0, e_mp = 0, e_h0 = 0, e_h1 = 0;
  for (int t = 0; t < 400; t++) {
    double Va[9], Vb[9], ca[3], cb[3], dir[3];
    for (int c = 0; c < 3; c++) { ca[c] = urand(&seed) - 0.5; dir[c] = urand(&seed) - 0.5; }
    const double dn = sqrt(dir[0] * dir[0] + dir[1] * dir[1] + dir[2] * dir[2]);
    const double dist = 0.3 + 1.7 * urand(&seed);
    for (int c = 0; c < 3; c++) cb[c] = ca[c] + dist * dir[c] / dn;
    for (int v = 0; v < 3; v++)
      for (int c = 0; c < 3; c++) {
        Va[3 * v + c] = ca[c] + 0.05 * (urand(&seed) - 0.5);
        Vb[3 * v + c] = cb[c] + 0.05 * (urand(&seed) - 0.5);
      }
    const cx<double> k = mk(1.0 + 3.0 * urand(&seed), (t % 2) ? 0.0 : 0.02 * urand(&seed));
    PairGeom<double> gd;
    for (int c = 0; c < 3; c++) {
      gd.D0[c] = Va[c] - Vb[c];
      gd.Aa[c] = Va[3 + c] - Va[c]; gd.Ba[c] = Va[6 + c] - Va[c];
      gd.Ab[c] = Vb[3 + c] - Vb[c]; gd.Bb[c] = Vb[6 + c] - Vb[c];
    }
    cx<double> MGd[9], MPd[9];
    pair_moments<double, 0>(gd, k, RULE6, 6, MGd, MPd);
    // nodes relative to the origin Va[0], float-float
    float Xa[36], Xb[36];
    for (int i = 0; i < 6; i++)
      for (int c = 0; c < 3; c++) {
        const double u = RULE6[3 * i], v = RULE6[3 * i + 1];
        const ff a = ff_of(u * gd.Aa[c] + v * gd.Ba[c]);
        const ff b = ff_of(-gd.D0[c] + u * gd.Ab[c] + v * gd.Bb[c]);
        Xa[6 * i + c] = a.hi; Xa[6 * i + 3 + c] = a.lo;
        Xb[6 * i + c] = b.hi; Xb[6 * i + 3 + c] = b.lo;
      }
    cff MG[9], MP[9];
    pair_moments_ff<6>(Xa, Xb, ff_of(k.re), ff_of(k.im), &R, &T, MG, MP);
    const double sg = sqrt(cnorm2(MGd[0])), sp = sqrt(cnorm2(MPd[0]));
    for (int m = 0; m < 9; m++) {
      const cx<double> g = cff_d(MG[m]), p = cff_d(MP[m]);
      e_mg = fmax(e_mg, sqrt(cnorm2(g - MGd[m])) / sg);
      e_mp = fmax(e_mp, sqrt(cnorm2(p - MPd[m])) / sp);
    }
    FFGeom g;
    for (int c = 0; c < 3; c++) {
      g.Aa[c] = ff_of(gd.Aa[c]); g.Ba[c] = ff_of(gd.Ba[c]);
      g.Ab[c] = ff_of(gd.Ab[c]); g.Bb[c] = ff_of(gd.Bb[c]); g.D0[c] = ff_of(gd.D0[c]);
    }
    ff D[2][2];
    h0_dots(g, D);
    H0Pre p0;
    h0_prepare(D, MG, &p0);
    H1Pre p1;
    h1_prepare(g, &p1);
    const cx<double> m4 = cdiv(mk(-4.0, 0.0), k * k);
    for (int ja = 0; ja < 3; ja++)
      for (int jb = 0; jb < 3; jb++) {
        double c[9], d[9];
        combo_coeffs(Va, Vb, ja, jb, c, d);
        cx<double> H0d, H1d;
        combine(MGd, MPd, c, d, m4, &H0d, &H1d);
        const cx<double> h0 = cff_d(h0_combo(p0, ja, jb, cff_of(m4))), h1 = cff_d(h1_combo(p1, ja, jb, MP));
        // relative to the size of the terms the sums are made of
        e_h0 = fmax(e_h0, sqrt(cnorm2(h0 - H0d)) / (sqrt(cnorm2(m4)) * sg));
        double sc = 0;
        for (int m = 0; m < 9; m++) sc += fabs(d[m]) * sqrt(cnorm2(MPd[m]));
        e_h1 = fmax(e_h1, sqrt(cnorm2(h1 - H1d)) / sc);
      }
  }
  printf("expi %.3e mg %.3e mp %.3e h0 %.3e h1 %.3e\n", e_expi, e_mg, e_mp, e_h0, e_h1);
  return 0;
}
