// ffmath.cuh -- float-float ("double-float") arithmetic for the mixed-
// precision far field.
//
// Why: the far-field entries of the RWG matrix are second differences of
// panel-pair integrals -- each edge pair sums the four (P/M, P/M) panel
// pairs with alternating signs, and the charge term -4/k^2 int int G
// cancels by a factor (panel size / distance)^2.  Rounded to FP32 per panel
// pair, that cancellation lifts the rounding into errors of ~1e-5 of the
// far entries, which move the absorbed power of a weakly lossy scatterer
// (Im eps / Re eps ~ 1e-3) by ~1e-5 relative.  Carrying every panel-pair
// quantity as an unevaluated sum hi + lo of two floats (~44 significant
// bits, on the FP32 pipes, which run ~70x the FP64 rate on this part)
// keeps the cancellation harmless; the entry is rounded to complex64 only
// after the four panel pairs are combined.
//
// Error-free transformations: two_sum (Knuth), quick_two_sum (Dekker,
// |a| >= |b|), two_prod via fma.  two_sum/quick_two_sum contain no
// products, so FMA contraction cannot change them.
#pragma once
#include "bem_math.cuh"

namespace gbem {

struct ff {
  float hi, lo;
};
GB_HD ff ffv(float h, float l) { ff r; r.hi = h; r.lo = l; return r; }
GB_HD ff ff_of(double x) { const float h = (float)x; return ffv(h, (float)(x - (double)h)); }
GB_HD double ff_d(ff a) { return (double)a.hi + (double)a.lo; }
GB_HD ff two_sum(float a, float b) {
  const float s = a + b, bb = s - a;
  return ffv(s, (a - (s - bb)) + (b - bb));
}
GB_HD ff quick_two_sum(float a, float b) {
  const float s = a + b;
  return ffv(s, b - (s - a));
}
GB_HD ff two_prod(float a, float b) {
  const float p = a * b;
  return ffv(p, fmaf(a, b, -p));
}
GB_HD ff ff_norm(ff a) { return quick_two_sum(a.hi, a.lo); }
GB_HD ff ff_neg(ff a) { return ffv(-a.hi, -a.lo); }
GB_HD ff ff_add(ff a, ff b) {
  const ff s = two_sum(a.hi, b.hi);
  return quick_two_sum(s.hi, s.lo + (a.lo + b.lo));
}
GB_HD ff ff_sub(ff a, ff b) { return ff_add(a, ff_neg(b)); }
GB_HD ff ff_add_f(ff a, float b) {
  const ff s = two_sum(a.hi, b);
  return quick_two_sum(s.hi, s.lo + a.lo);
}
// product, not renormalised (|lo| may reach a few ulp(hi))
GB_HD ff ff_mul_u(ff a, ff b) {
  const float p = a.hi * b.hi;
  return ffv(p, fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, fmaf(a.hi, b.hi, -p))));
}
GB_HD ff ff_mul(ff a, ff b) { return ff_norm(ff_mul_u(a, b)); }
GB_HD ff ff_mul_f(ff a, float b) {
  const float p = a.hi * b;
  return quick_two_sum(p, fmaf(a.lo, b, fmaf(a.hi, b, -p)));
}

// complex float-float
struct cff {
  ff re, im;
};
GB_HD cff cffv(ff r, ff i) { cff z; z.re = r; z.im = i; return z; }
GB_HD cff cff_zero() { return cffv(ffv(0.f, 0.f), ffv(0.f, 0.f)); }
GB_HD cff cff_of(cx<double> z) { return cffv(ff_of(z.re), ff_of(z.im)); }
GB_HD cx<double> cff_d(cff z) { return mk(ff_d(z.re), ff_d(z.im)); }
GB_HD cx<float> cff_hi(cff z) { return mk(z.re.hi, z.im.hi); }
GB_HD cx<float> cff_lo(cff z) { return mk(z.re.lo, z.im.lo); }
GB_HD cff cff_add(cff a, cff b) { return cffv(ff_add(a.re, b.re), ff_add(a.im, b.im)); }
GB_HD cff cff_sub(cff a, cff b) { return cffv(ff_sub(a.re, b.re), ff_sub(a.im, b.im)); }
GB_HD cff cff_mul(cff a, cff b) {
  return cffv(ff_add(ff_mul_u(a.re, b.re), ff_neg(ff_mul_u(a.im, b.im))),
              ff_add(ff_mul_u(a.re, b.im), ff_mul_u(a.im, b.re)));
}
GB_HD cff cff_mul_ff(cff a, ff s) { return cffv(ff_mul(a.re, s), ff_mul(a.im, s)); }
GB_HD cff cff_mul_f(cff a, float s) { return cffv(ff_mul_f(a.re, s), ff_mul_f(a.im, s)); }
// a + s b for a float s (the combination coefficients of the moments)
GB_HD cff cff_fma_f(cff a, float s, cff b) { return cff_add(a, cff_mul_f(b, s)); }

// Lazy accumulator: hi by two_sum, the rounding errors and lo parts summed
// in lo; renormalised once at the end (accurate to ~n ulp(lo) for n terms).
struct ffacc {
  float hi, lo;
};
GB_HD void acc_add(ffacc& a, ff x) {
  const ff s = two_sum(a.hi, x.hi);
  a.hi = s.hi;
  a.lo += s.lo + x.lo;
}
GB_HD ff acc_get(const ffacc& a) { return quick_two_sum(a.hi, a.lo); }

// ---------------------------------------------------------------------------
// e^{ix} for a float-float argument: x = j pi/64 + t with |t| <= pi/128, the
// table holding cos(j pi/64), sin(j pi/64) (j = 0..127) as float-float
// values computed in FP64 on the host; cos t, sin t by their Taylor series
// (|t|^7/5040 < 4e-15).  Cody-Waite reduction with pi/64 = P1 + P2 + P3
// (P1 of 8 and P2 of 10 significant bits, so j P1 and j P2 are exact for
// |j| < 2^14): absolute error ~1e-12 for |x| < 800 (|j| < 2^14).
// ---------------------------------------------------------------------------
struct SinCosTab {
  float c_hi[128], c_lo[128], s_hi[128], s_lo[128];
};
constexpr float PI64_1 = 0.049072265625f;                // pi/64, leading 8 bits
constexpr float PI64_2 = 1.5124678611755371e-05f;        // next 10 bits
constexpr float PI64_3 = -5.091271404467079e-09f;        // remainder to float
constexpr float INV_PI64 = 20.371832715762604f;          // 64/pi

GB_HD cff expi_ff(ff x, const SinCosTab* T) {
  const float jf = rintf(x.hi * INV_PI64);
  // t = x - j pi/64: x.hi - j P1 is exact (Sterbenz), the rest by two_sum
  const float t1 = fmaf(-jf, PI64_1, x.hi);
  const ff t2 = two_sum(t1, -jf * PI64_2);
  const ff t = quick_two_sum(t2.hi, t2.lo + fmaf(-jf, PI64_3, x.lo));
  const int j = ((int)jf) & 127;
  const ff c0 = ffv(T->c_hi[j], T->c_lo[j]), s0 = ffv(T->s_hi[j], T->s_lo[j]);
  // sin t = t + t^3 (-1/6 + t^2/120): the cubic term is < 2.5e-6, float-exact enough
  const float t2f = t.hi * t.hi;
  const float st = t.hi * t2f * fmaf(t2f, 1.0f / 120.0f, -1.0f / 6.0f);
  const ff sn = quick_two_sum(t.hi, t.lo + st);
  // cos t = 1 + dc, dc = -t^2/2 + t^4/24 (< 3.1e-4) as an unnormalised
  // float-float: t^2 exactly (two_prod), the quartic term in the lo part
  const ff p2 = two_prod(t.hi, t.hi);
  const ff dc = ffv(-0.5f * p2.hi, fmaf(p2.hi * p2.hi, 1.0f / 24.0f, -(0.5f * p2.lo + t.hi * t.lo)));
  // (c0 + i s0)(1 + dc + i sn)
  const ff re = ff_add(ff_add(c0, ff_mul_u(c0, dc)), ff_neg(ff_mul_u(s0, sn)));
  const ff im = ff_add(ff_add(s0, ff_mul_u(s0, dc)), ff_mul_u(c0, sn));
  return cffv(re, im);
}

// host-side table (FP64 libm values split to float-float)
inline void fill_sincos_tab(SinCosTab* T) {
  for (int j = 0; j < 128; j++) {
    const double a = j * (3.14159265358979323846 / 64.0);
    const ff c = ff_of(cos(a)), s = ff_of(sin(a));
    T->c_hi[j] = c.hi; T->c_lo[j] = c.lo; T->s_hi[j] = s.hi; T->s_lo[j] = s.lo;
  }
}

// ---------------------------------------------------------------------------
// Far-field bilinear moments of one panel pair in float-float (same
// definition as pair_moments: MG[m] = sum_i sum_j w_i w_j mono_m G(r_ij),
// MP likewise with Psi = G (ik - 1/r)/r).  Node positions are float-float
// offsets from one origin shared by the whole tile (formed in FP64 with
// the rule's FP64 coordinates), node stride NS floats: Xa[i*NS + c] (hi),
// Xa[i*NS + 3 + c] (lo).  r from |Xa_i - Xb_j|^2 in float-float,
// G = e^{ikr}/(4 pi r), k as float-float (kre + kre_lo, kim + kim_lo).
// The rule's coordinates and weights are float-float as well (FFRule):
// rounding them to FP32 would perturb the rule by ~3e-8, which already
// moves the absorbed power of a weakly lossy scatterer by ~1e-7.
// ---------------------------------------------------------------------------
struct FFRule {
  float u[12], v[12], w[12], w4[12];  // [j] hi, [6 + j] lo; w4 = w/(4 pi)
};

GB_HD ff rule_u(const FFRule* R, int j) { return ffv(R->u[j], R->u[6 + j]); }
GB_HD ff rule_v(const FFRule* R, int j) { return ffv(R->v[j], R->v[6 + j]); }

template <int NS>
GB_HD void pair_moments_ff(const float* Xa, const float* Xb, ff kre, ff kim, const FFRule* R, const SinCosTab* T,
                           cff* MG, cff* MP) {
  ffacc G[9][2], P[9][2];
  for (int m = 0; m < 9; m++)
    for (int c = 0; c < 2; c++) G[m][c].hi = G[m][c].lo = P[m][c].hi = P[m][c].lo = 0.f;
  for (int i = 0; i < 6; i++) {
    ff xa[3];
    for (int c = 0; c < 3; c++) xa[c] = ffv(Xa[i * NS + c], Xa[i * NS + 3 + c]);
    ffacc S[3][2], SP[3][2];
    for (int b = 0; b < 3; b++)
      for (int c = 0; c < 2; c++) S[b][c].hi = S[b][c].lo = SP[b][c].hi = SP[b][c].lo = 0.f;
    for (int j = 0; j < 6; j++) {
      // R = Xa_i - Xb_j and |R|^2, float-float
      float r2h = 0.f, r2l = 0.f;
      for (int c = 0; c < 3; c++) {
        const ff d = two_sum(xa[c].hi, -Xb[j * NS + c]);
        const float dl = d.lo + (xa[c].lo - Xb[j * NS + 3 + c]);
        const ff p = two_prod(d.hi, d.hi);
        const ff s = two_sum(r2h, p.hi);
        r2h = s.hi;
        r2l += s.lo + fmaf(2.0f * d.hi, dl, p.lo);
      }
      const ff r2 = quick_two_sum(r2h, r2l);
      // r and y = 1/r
      const float rh = sqrtf(r2.hi);
      const float yh = 1.0f / rh;
      const float rl = (fmaf(-rh, rh, r2.hi) + r2.lo) * (0.5f * yh);
      const ff y = quick_two_sum(yh, yh * (fmaf(-rh, yh, 1.0f) - rl * yh));
      // phase k r
      const float krh = kre.hi * rh;
      const ff kr = quick_two_sum(krh, fmaf(kre.hi, rh, -krh) + fmaf(kre.hi, rl, kre.lo * rh));
      const cff e = expi_ff(kr, T);
      // amplitude w_j/(4 pi r) e^{-Im k r}
      ff amp = ff_mul(y, ffv(R->w4[j], R->w4[6 + j]));
      if (kim.hi != 0.f) {
        // e^{-a}, a = Im k r: halve a (exactly) to |a| < 1/32, take
        // e^{-a} = 1 + dm with dm = -a + a^2 (1/2 - a/6 + a^2/24 - a^3/120)
        // (the quadratic part < 5e-4, FP32-accurate), square back
        const float ah = kim.hi * rh;
        ff a = quick_two_sum(ah, fmaf(kim.hi, rh, -ah) + fmaf(kim.hi, rl, kim.lo * rh));
        int m = 0;
        while (fabsf(a.hi) >= 0.03125f && m < 16) { a = ffv(0.5f * a.hi, 0.5f * a.lo); m++; }
        const float q = a.hi * a.hi * fmaf(a.hi, fmaf(a.hi, fmaf(a.hi, -1.0f / 120.0f, 1.0f / 24.0f), -1.0f / 6.0f), 0.5f);
        const ff dm0 = two_sum(-a.hi, q);
        const ff dm = ffv(dm0.hi, dm0.lo - a.lo);
        if (m == 0) {
          amp = ff_add(amp, ff_mul_u(amp, dm));
        } else {
          ff ex = ff_add_f(dm, 1.0f);
          for (int it = 0; it < m; it++) ex = ff_mul(ex, ex);
          amp = ff_mul(amp, ex);
        }
      }
      const cff g = cffv(ff_mul(amp, e.re), ff_mul(amp, e.im));
      // Psi = G f, f = (ik - 1/r)/r = (-(Im k + y) y, Re k y)
      const cff f = cffv(ff_neg(ff_mul(ff_add(kim, y), y)), ff_mul(kre, y));
      const cff ps = cff_mul(g, f);
      const ff up = rule_u(R, j), vp = rule_v(R, j);
      acc_add(S[0][0], g.re); acc_add(S[0][1], g.im);
      acc_add(S[1][0], ff_mul_u(g.re, up)); acc_add(S[1][1], ff_mul_u(g.im, up));
      acc_add(S[2][0], ff_mul_u(g.re, vp)); acc_add(S[2][1], ff_mul_u(g.im, vp));
      acc_add(SP[0][0], ps.re); acc_add(SP[0][1], ps.im);
      acc_add(SP[1][0], ff_mul_u(ps.re, up)); acc_add(SP[1][1], ff_mul_u(ps.im, up));
      acc_add(SP[2][0], ff_mul_u(ps.re, vp)); acc_add(SP[2][1], ff_mul_u(ps.im, vp));
    }
    const ff w = ffv(R->w[i], R->w[6 + i]);
    const ff a[3] = {w, ff_mul(w, rule_u(R, i)), ff_mul(w, rule_v(R, i))};
    for (int b = 0; b < 3; b++)
      for (int c = 0; c < 2; c++) {
        const ff sg = acc_get(S[b][c]), sp = acc_get(SP[b][c]);
        for (int al = 0; al < 3; al++) {
          acc_add(G[3 * al + b][c], ff_mul_u(sg, a[al]));
          acc_add(P[3 * al + b][c], ff_mul_u(sp, a[al]));
        }
      }
  }
  for (int m = 0; m < 9; m++) {
    MG[m] = cffv(acc_get(G[m][0]), acc_get(G[m][1]));
    MP[m] = cffv(acc_get(P[m][0]), acc_get(P[m][1]));
  }
}

// host-side rule table from the FP64 rule (u, v, w per point)
inline void fill_ff_rule(const double* rule6, FFRule* R) {
  for (int j = 0; j < 6; j++) {
    const ff u = ff_of(rule6[3 * j]), v = ff_of(rule6[3 * j + 1]), w = ff_of(rule6[3 * j + 2]);
    const ff w4 = ff_of(rule6[3 * j + 2] / (4.0 * 3.14159265358979323846));
    R->u[j] = u.hi; R->u[6 + j] = u.lo; R->v[j] = v.hi; R->v[6 + j] = v.lo;
    R->w[j] = w.hi; R->w[6 + j] = w.lo; R->w4[j] = w4.hi; R->w4[6 + j] = w4.lo;
  }
}

// ---------------------------------------------------------------------------
// Geometry of a far panel pair in float-float (split from FP64): edge
// vectors A = V1 - V0, B = V2 - V0 of both panels and D0 = V0a - V0b.
// ---------------------------------------------------------------------------
struct FFGeom {
  ff Aa[3], Ba[3], Ab[3], Bb[3], D0[3];
};

GB_HD ff dot_ff(const ff* x, const ff* y) {
  ffacc a;
  a.hi = a.lo = 0.f;
  for (int c = 0; c < 3; c++) acc_add(a, ff_mul_u(x[c], y[c]));
  return acc_get(a);
}
GB_HD void cross_ff(const ff* x, const ff* y, ff* z) {
  z[0] = ff_add(ff_mul_u(x[1], y[2]), ff_neg(ff_mul_u(x[2], y[1])));
  z[1] = ff_add(ff_mul_u(x[2], y[0]), ff_neg(ff_mul_u(x[0], y[2])));
  z[2] = ff_add(ff_mul_u(x[0], y[1]), ff_neg(ff_mul_u(x[1], y[0])));
}
GB_HD cff cff_mac(cff h, cff m, ff c) { return cff_add(h, cffv(ff_mul_u(m.re, c), ff_mul_u(m.im, c))); }

// ---------------------------------------------------------------------------
// H0 for the (Qa, Qb) at local vertices ja, jb from the moments.  With
// F = x - Qa = a0 + u Aa + v Ba, where the vertex offset a0 = V0a - Qa is
// 0, -Aa or -Ba (ja = 0, 1, 2), every geometric coefficient is one of the
// four dot products D[x][y] of {Aa, Ba} with {Ab, Bb}, so
//   H0 = T - Ua[ja] - Ub[jb] + (D[ja][jb] + m4) MG[0],
//   T = sum_{x,y} D[x][y] MG[3x+3+y+1], Ua[x] = sum_y D[x][y] MG[y+1],
//   Ub[y] = sum_x D[x][y] MG[3x+3]        (x, y = 0 for A, 1 for B)
// with Ua, Ub, D taken as zero for a vertex index 0; m4 = -4/k^2.
// ---------------------------------------------------------------------------
struct H0Pre {
  ff D[2][2];
  cff T, Ua[2], Ub[2], W0;
};

GB_HD void h0_dots(const FFGeom& g, ff D[2][2]) {
  const ff* va[2] = {g.Aa, g.Ba};
  const ff* vb[2] = {g.Ab, g.Bb};
  for (int x = 0; x < 2; x++)
    for (int y = 0; y < 2; y++) D[x][y] = dot_ff(va[x], vb[y]);
}

GB_HD void h0_prepare(const ff D[2][2], const cff* MG, H0Pre* p) {
  p->T = cff_zero();
  for (int x = 0; x < 2; x++) { p->Ua[x] = cff_zero(); p->Ub[x] = cff_zero(); }
  for (int x = 0; x < 2; x++)
    for (int y = 0; y < 2; y++) {
      p->D[x][y] = D[x][y];
      p->T = cff_mac(p->T, MG[3 * x + 3 + y + 1], D[x][y]);
      p->Ua[x] = cff_mac(p->Ua[x], MG[y + 1], D[x][y]);
      p->Ub[y] = cff_mac(p->Ub[y], MG[3 * x + 3], D[x][y]);
    }
  p->W0 = MG[0];
}

// (selects rather than indexing by ja, jb keep the tables in registers)
template <typename V> GB_HD V sel2(int j, const V& a, const V& b) { return j == 1 ? a : b; }

GB_HD cff h0_combo(const H0Pre& p, int ja, int jb, cff m4) {
  cff h = p.T;
  if (ja) h = cff_sub(h, sel2(ja, p.Ua[0], p.Ua[1]));
  if (jb) h = cff_sub(h, sel2(jb, p.Ub[0], p.Ub[1]));
  const ff d = (ja && jb) ? sel2(ja, sel2(jb, p.D[0][0], p.D[0][1]), sel2(jb, p.D[1][0], p.D[1][1])) : ffv(0.f, 0.f);
  return cff_add(h, cff_mul(p.W0, cffv(ff_add(d, m4.re), m4.im)));
}

// ---------------------------------------------------------------------------
// H1 = sum_m d_m MP[m], d_m = (a_al x b_be).(Qa - Qb) (combo_coeffs), from
// the cross products C[x][y] = va_x x vb_y (va = {Aa, Ba}, vb = {Ab, Bb})
// and q = Qa - Qb = D0 + va(ja) - vb(jb):
//   e[x][y] = C[x][y].q = c[x][y] + a[x][y][ja] - b[x][y][jb],
//   H1 = sum e[x][y] MP[3x+3+y+1] - sum_y e[ja][y] MP[y+1]
//        - sum_x e[x][jb] MP[3x+3] + e[ja][jb] MP[0]
// (terms of a vertex index 0 absent).  For nearly coplanar panels the
// d_m are small differences of large products, so they are formed exactly
// from the float-float geometry and the sum is taken in float-float.
// ---------------------------------------------------------------------------
struct H1Pre {
  ff c[2][2], a[2][2][2], b[2][2][2];  // a[x][y][j], b[x][y][j]: vertex index j + 1
};

GB_HD void h1_prepare(const FFGeom& g, H1Pre* p) {
  const ff* va[2] = {g.Aa, g.Ba};
  const ff* vb[2] = {g.Ab, g.Bb};
  for (int x = 0; x < 2; x++)
    for (int y = 0; y < 2; y++) {
      ff C[3];
      cross_ff(va[x], vb[y], C);
      p->c[x][y] = dot_ff(C, g.D0);
      for (int j = 0; j < 2; j++) {
        p->a[x][y][j] = (j == x) ? ffv(0.f, 0.f) : dot_ff(C, va[j]);
        p->b[x][y][j] = (j == y) ? ffv(0.f, 0.f) : dot_ff(C, vb[j]);
      }
    }
}

GB_HD cff h1_combo(const H1Pre& p, int ja, int jb, const cff* MP) {
  ff e[2][2];
  for (int x = 0; x < 2; x++)
    for (int y = 0; y < 2; y++) {
      ff v = p.c[x][y];
      if (ja) v = ff_add(v, sel2(ja, p.a[x][y][0], p.a[x][y][1]));
      if (jb) v = ff_sub(v, sel2(jb, p.b[x][y][0], p.b[x][y][1]));
      e[x][y] = v;
    }
  cff h = cff_zero();
  for (int x = 0; x < 2; x++)
    for (int y = 0; y < 2; y++) h = cff_mac(h, MP[3 * x + 3 + y + 1], e[x][y]);
  if (ja)
    for (int y = 0; y < 2; y++) h = cff_mac(h, MP[y + 1], ff_neg(sel2(ja, e[0][y], e[1][y])));
  if (jb)
    for (int x = 0; x < 2; x++) h = cff_mac(h, MP[3 * x + 3], ff_neg(sel2(jb, e[x][0], e[x][1])));
  if (ja && jb) h = cff_mac(h, MP[0], sel2(ja, sel2(jb, e[0][0], e[0][1]), sel2(jb, e[1][0], e[1][1])));
  return h;
}

}  // namespace gbem
