// bem_math.cuh -- panel-pair integration math shared by the assembly kernels.
//
// All functions are __host__ __device__ so the same code runs in the CUDA
// kernels and (for debugging only) on the host.
//
// Conventions
//  * A panel with vertices (V0, V1, V2) in mesh order is parametrised as
//    x = V0 + u A + v B, A = V1 - V0, B = V2 - V0, u, v >= 0, u + v <= 1
//    (the triangle-cubature convention of libs/libTriInt/TCR.cc); integrals
//    are over parameter space (area 1/2 per panel), so the RWG normalisation
//    leaves the factor La*Lb (EdgeEdgeInteractions.cc:183-188).
//  * For a panel pair the library keeps 9+9 "bilinear moments"
//       MG[m] = int int mono_m G(r),  MP[m] = int int mono_m Psi(r),
//    mono_m over {1, u', v', u, uu', uv', v, vu', vv'} (primes: second panel),
//    G = e^{ikr}/(4 pi r), Psi = G (ik - 1/r)/r.  The reference's per-edge
//    integrands (PanelPanelInteractions.cc:108-201)
//       H0 = int int ((x-Qa).(x'-Qb) - 4/k^2) G,
//       H1 = int int ((x-Qa) x (x'-Qb)).(x-x') Psi
//    are bilinear in (x-Qa, x'-Qb); since ((x-Qa)x(x'-Qb)).(x-x') equals
//    ((x-Qa)x(x'-Qb)).(Qa-Qb) pointwise, both follow from the moments for all
//    9 choices of (Qa, Qb) without re-integrating (the reference integrates
//    each of the up-to-9 edge pairs sharing a panel pair separately).
#pragma once
#include <cuda_runtime.h>
#include <math.h>

#define GB_HD __host__ __device__ __forceinline__
#define GB_HD_NOINLINE static __host__ __device__ __noinline__

namespace gbem {

template <typename T> struct cx { T re, im; };
template <typename T> GB_HD cx<T> mk(T a, T b) { cx<T> z; z.re = a; z.im = b; return z; }
template <typename T> GB_HD cx<T> operator+(cx<T> a, cx<T> b) { return mk(a.re + b.re, a.im + b.im); }
template <typename T> GB_HD cx<T> operator-(cx<T> a, cx<T> b) { return mk(a.re - b.re, a.im - b.im); }
template <typename T> GB_HD cx<T> operator*(cx<T> a, cx<T> b) { return mk(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re); }
template <typename T> GB_HD cx<T> operator*(T s, cx<T> a) { return mk(s * a.re, s * a.im); }
template <typename T> GB_HD cx<T> cdiv(cx<T> a, cx<T> b) {
  T d = b.re * b.re + b.im * b.im;
  return mk((a.re * b.re + a.im * b.im) / d, (a.im * b.re - a.re * b.im) / d);
}
template <typename T> GB_HD T cnorm2(cx<T> a) { return a.re * a.re + a.im * a.im; }
template <typename T> GB_HD cx<T> cexpo(cx<T> z) {
  T e = exp(z.re), s, c;
#ifdef __CUDA_ARCH__
  sincos(z.im, &s, &c);
#else
  s = sin(z.im); c = cos(z.im);
#endif
  return mk(e * c, e * s);
}

GB_HD double vdot(const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
GB_HD void vcross(const double* a, const double* b, double* c) {
  c[0] = a[1] * b[2] - a[2] * b[1];
  c[1] = a[2] * b[0] - a[0] * b[2];
  c[2] = a[0] * b[1] - a[1] * b[0];
}
GB_HD double vdet(const double* a, const double* b, const double* c) {
  double t[3];
  vcross(a, b, t);
  return vdot(t, c);
}

// 1/m for m = 1..100 (index m-1), so the series below multiplies instead of
// dividing (the same correctly rounded values as 1.0 / m)
#define GB_RECIP_VALUES 1.0 / 1, 1.0 / 2, 1.0 / 3, 1.0 / 4, 1.0 / 5, 1.0 / 6, 1.0 / 7, 1.0 / 8, 1.0 / 9, 1.0 / 10, 1.0 / 11, 1.0 / 12, 1.0 / 13, 1.0 / 14, 1.0 / 15, 1.0 / 16, 1.0 / 17, 1.0 / 18, 1.0 / 19, 1.0 / 20, 1.0 / 21, 1.0 / 22, 1.0 / 23, 1.0 / 24, 1.0 / 25, 1.0 / 26, 1.0 / 27, 1.0 / 28, 1.0 / 29, 1.0 / 30, 1.0 / 31, 1.0 / 32, 1.0 / 33, 1.0 / 34, 1.0 / 35, 1.0 / 36, 1.0 / 37, 1.0 / 38, 1.0 / 39, 1.0 / 40, 1.0 / 41, 1.0 / 42, 1.0 / 43, 1.0 / 44, 1.0 / 45, 1.0 / 46, 1.0 / 47, 1.0 / 48, 1.0 / 49, 1.0 / 50, 1.0 / 51, 1.0 / 52, 1.0 / 53, 1.0 / 54, 1.0 / 55, 1.0 / 56, 1.0 / 57, 1.0 / 58, 1.0 / 59, 1.0 / 60, 1.0 / 61, 1.0 / 62, 1.0 / 63, 1.0 / 64, 1.0 / 65, 1.0 / 66, 1.0 / 67, 1.0 / 68, 1.0 / 69, 1.0 / 70, 1.0 / 71, 1.0 / 72, 1.0 / 73, 1.0 / 74, 1.0 / 75, 1.0 / 76, 1.0 / 77, 1.0 / 78, 1.0 / 79, 1.0 / 80, 1.0 / 81, 1.0 / 82, 1.0 / 83, 1.0 / 84, 1.0 / 85, 1.0 / 86, 1.0 / 87, 1.0 / 88, 1.0 / 89, 1.0 / 90, 1.0 / 91, 1.0 / 92, 1.0 / 93, 1.0 / 94, 1.0 / 95, 1.0 / 96, 1.0 / 97, 1.0 / 98, 1.0 / 99, 1.0 / 100
static __constant__ double c_recip_dev[100] = {GB_RECIP_VALUES};
static const double c_recip_host[100] = {GB_RECIP_VALUES};
#undef GB_RECIP_VALUES
GB_HD double recip_int(int m) {
#ifdef __CUDA_ARCH__
  return c_recip_dev[m - 1];
#else
  return c_recip_host[m - 1];
#endif
}

// ExpRel(x, 4) = sum_{m>=4} x^m/m!, summed until a term falls below 1e-8 of
// the running sum (PanelPanelInteractions.cc:86-103; same truncation so the
// desingularised remainder matches the reference term for term).
GB_HD cx<double> exprel4(cx<double> x) {
  cx<double> term = mk(1.0, 0.0);
  for (int m = 1; m < 4; m++) term = recip_int(m) * (term * x);
  cx<double> sum = mk(0.0, 0.0);
  for (int m = 4; m < 100; m++) {
    term = recip_int(m) * (term * x);
    sum = sum + term;
    if (cnorm2(term) < 1.0e-16 * cnorm2(sum)) break;
  }
  return sum;
}

// ---------------------------------------------------------------------------
// Bilinear moments by a fixed product rule (LO 6x6 far field, desingularised
// remainder, HO).  Geometry is given relative to each panel's V0:
//   D0 = V0a - V0b; (Aa, Ba), (Ab, Bb) edge vectors in TCR convention.
// Kernel selector: 0 = full Helmholtz, 1 = desingularised (ExpRel(ikr,4)).
// ---------------------------------------------------------------------------
template <typename T> struct PairGeom {
  T D0[3], Aa[3], Ba[3], Ab[3], Bb[3];
};

GB_HD void sincos_t(float x, float* s, float* c) {
#ifdef __CUDA_ARCH__
  sincosf(x, s, c);
#else
  *s = sinf(x); *c = cosf(x);
#endif
}
GB_HD void sincos_t(double x, double* s, double* c) {
#ifdef __CUDA_ARCH__
  sincos(x, s, c);
#else
  *s = sin(x); *c = cos(x);
#endif
}
GB_HD float exp_t(float x) { return expf(x); }
GB_HD double exp_t(double x) { return exp(x); }
GB_HD float rsqrt_t(float x) {
#ifdef __CUDA_ARCH__
  return rsqrtf(x);
#else
  return 1.0f / sqrtf(x);
#endif
}
GB_HD double rsqrt_t(double x) { return 1.0 / sqrt(x); }

// Phi = e^{ikr}/(4 pi r), Psi = Phi (ik - 1/r)/r, both times the weight w.
template <typename T>
GB_HD void helmholtz_pp(T r2, cx<T> k, T w, cx<T>* phi, cx<T>* psi) {
  const T inv4pi = (T)0.079577471545947667884;  // 1/(4 pi)
  T rinv = rsqrt_t(r2);
  T r = r2 * rinv;
  T s, c;
  sincos_t(k.re * r, &s, &c);
  T amp = w * inv4pi * rinv;
  if (k.im != (T)0) amp *= exp_t(-k.im * r);
  cx<T> p = mk(amp * c, amp * s);
  // (ik - 1/r)/r = (-k.im - 1/r + i k.re)/r
  cx<T> f = mk((-k.im - rinv) * rinv, k.re * rinv);
  *phi = p;
  *psi = p * f;
}

GB_HD void desing_pp(double r2, cx<double> k, double w, cx<double>* phi, cx<double>* psi) {
  const double inv4pi = 0.079577471545947667884;
  double r = sqrt(r2), rinv = 1.0 / r;
  cx<double> ikr = mk(-k.im * r, k.re * r);
  cx<double> p = (w * inv4pi * rinv) * exprel4(ikr);
  cx<double> f = mk((-k.im - rinv) * rinv, k.re * rinv);
  *phi = p;
  *psi = p * f;
}

// rule: npts triples (u, v, w)
template <typename T, int DESING>
GB_HD void pair_moments(const PairGeom<T>& g, cx<T> k, const T* rule, int npts, cx<T>* MG, cx<T>* MP) {
  for (int m = 0; m < 9; m++) { MG[m] = mk((T)0, (T)0); MP[m] = mk((T)0, (T)0); }
  for (int i = 0; i < npts; i++) {
    T u = rule[3 * i], v = rule[3 * i + 1], wi = rule[3 * i + 2];
    T pa[3];
    for (int c = 0; c < 3; c++) pa[c] = g.D0[c] + u * g.Aa[c] + v * g.Ba[c];
    cx<T> SG[3], SP[3];
    for (int b = 0; b < 3; b++) { SG[b] = mk((T)0, (T)0); SP[b] = mk((T)0, (T)0); }
    for (int j = 0; j < npts; j++) {
      T up = rule[3 * j], vp = rule[3 * j + 1], wj = rule[3 * j + 2];
      T R0 = pa[0] - up * g.Ab[0] - vp * g.Bb[0];
      T R1 = pa[1] - up * g.Ab[1] - vp * g.Bb[1];
      T R2 = pa[2] - up * g.Ab[2] - vp * g.Bb[2];
      T r2 = R0 * R0 + R1 * R1 + R2 * R2;
      cx<T> phi, psi;
      if constexpr (DESING) desing_pp(r2, k, wj, &phi, &psi);
      else helmholtz_pp(r2, k, wj, &phi, &psi);
      SG[0] = SG[0] + phi; SP[0] = SP[0] + psi;
      SG[1] = SG[1] + up * phi; SP[1] = SP[1] + up * psi;
      SG[2] = SG[2] + vp * phi; SP[2] = SP[2] + vp * psi;
    }
    T a[3] = {wi, wi * u, wi * v};
    for (int al = 0; al < 3; al++)
      for (int b = 0; b < 3; b++) {
        MG[3 * al + b] = MG[3 * al + b] + a[al] * SG[b];
        MP[3 * al + b] = MP[3 * al + b] + a[al] * SP[b];
      }
  }
}

// pair_moments with the npts x npts samples dealt out: this call adds the
// samples q = p0, p0 + pstride, ... (q = i npts + j); the caller sums the
// partial moments of all p0 (one lane each).
template <typename T, bool DESING>
GB_HD void pair_moments_part(const PairGeom<T>& g, cx<T> k, const T* rule, int npts, int p0, int pstride, cx<T>* MG,
                             cx<T>* MP) {
  for (int m = 0; m < 9; m++) { MG[m] = mk((T)0, (T)0); MP[m] = mk((T)0, (T)0); }
  for (int q = p0; q < npts * npts; q += pstride) {
    const int i = q / npts, j = q - i * npts;
    const T u = rule[3 * i], v = rule[3 * i + 1], wi = rule[3 * i + 2];
    const T up = rule[3 * j], vp = rule[3 * j + 1], wj = rule[3 * j + 2];
    T R[3];
    for (int c = 0; c < 3; c++) R[c] = g.D0[c] + u * g.Aa[c] + v * g.Ba[c] - up * g.Ab[c] - vp * g.Bb[c];
    const T r2 = R[0] * R[0] + R[1] * R[1] + R[2] * R[2];
    cx<T> phi, psi;
    if constexpr (DESING) desing_pp(r2, k, wj, &phi, &psi);
    else helmholtz_pp(r2, k, wj, &phi, &psi);
    const T a[3] = {wi, wi * u, wi * v}, b[3] = {(T)1, up, vp};
    for (int al = 0; al < 3; al++)
      for (int be = 0; be < 3; be++) {
        MG[3 * al + be] = MG[3 * al + be] + (a[al] * b[be]) * phi;
        MP[3 * al + be] = MP[3 * al + be] + (a[al] * b[be]) * psi;
      }
  }
}

// ---------------------------------------------------------------------------
// Combination coefficients for one (Qa, Qb) choice.  ja, jb = local vertex
// index of Q in each panel (mesh order).  Computed in double from the
// panels' double geometry.
//   c[m] = a_al . b_be,   d[m] = (a_al x b_be) . (Qa - Qb)
// with a_1 = V0a - Qa, a_u = Aa, a_v = Ba (likewise b), m = 3 al + be.
// ---------------------------------------------------------------------------
GB_HD void combo_coeffs(const double* Va, const double* Vb, int ja, int jb, double* c, double* d) {
  double A[3], B[3], Ap[3], Bp[3], a0[3], b0[3], QmQ[3];
  for (int i = 0; i < 3; i++) {
    A[i] = Va[3 + i] - Va[i]; B[i] = Va[6 + i] - Va[i];
    Ap[i] = Vb[3 + i] - Vb[i]; Bp[i] = Vb[6 + i] - Vb[i];
    a0[i] = Va[i] - Va[3 * ja + i];
    b0[i] = Vb[i] - Vb[3 * jb + i];
    QmQ[i] = Va[3 * ja + i] - Vb[3 * jb + i];
  }
  const double* av[3] = {a0, A, B};
  const double* bv[3] = {b0, Ap, Bp};
  for (int al = 0; al < 3; al++)
    for (int be = 0; be < 3; be++) {
      c[3 * al + be] = vdot(av[al], bv[be]);
      d[3 * al + be] = vdet(av[al], bv[be], QmQ);
    }
}

// Vector form of a pair's moments.  With u = x - V0a = u Aa + v Ba and
// v = x' - V0b = u' Ab + v' Bb:
//   W0 = int G,  Wx = int u G,  Wy = int v G,  Wxy = int u.v G,
//   P0 = int Psi, Pu = int u Psi, Pv = int v Psi, Puv = int u x v Psi,
// all linear combinations of the 9+9 monomial moments.  For Q's with
// alpha = V0a - Qa, beta = V0b - Qb and q = Qa - Qb = D0 - alpha + beta:
//   H0 = Wxy + beta.Wx + alpha.Wy + (alpha.beta - 4/k^2) W0
//   H1 = q.Puv + Pu.(beta x q) + Pv.(q x alpha) + (q.(alpha x beta)) P0
// which is the monomial combination above, regrouped (about a third of its
// arithmetic per (Qa, Qb)).
template <typename T> struct VecMoments {
  cx<T> W0, Wx[3], Wy[3], Wxy, P0, Pu[3], Pv[3], Puv[3];
};

template <typename T>
GB_HD void vec_moments(const PairGeom<T>& g, const cx<T>* MG, const cx<T>* MP, VecMoments<T>* vm) {
  const T* ea[2] = {g.Aa, g.Ba};
  const T* eb[2] = {g.Ab, g.Bb};
  vm->W0 = MG[0];
  vm->P0 = MP[0];
  for (int c = 0; c < 3; c++) {
    vm->Wx[c] = g.Aa[c] * MG[3] + g.Ba[c] * MG[6];
    vm->Wy[c] = g.Ab[c] * MG[1] + g.Bb[c] * MG[2];
    vm->Pu[c] = g.Aa[c] * MP[3] + g.Ba[c] * MP[6];
    vm->Pv[c] = g.Ab[c] * MP[1] + g.Bb[c] * MP[2];
    vm->Puv[c] = mk((T)0, (T)0);
  }
  vm->Wxy = mk((T)0, (T)0);
  for (int al = 0; al < 2; al++)
    for (int be = 0; be < 2; be++) {
      const T* x = ea[al];
      const T* y = eb[be];
      const int m = 3 * (al + 1) + (be + 1);
      const T dot = x[0] * y[0] + x[1] * y[1] + x[2] * y[2];
      const T cr[3] = {x[1] * y[2] - x[2] * y[1], x[2] * y[0] - x[0] * y[2], x[0] * y[1] - x[1] * y[0]};
      vm->Wxy = vm->Wxy + dot * MG[m];
      for (int c = 0; c < 3; c++) vm->Puv[c] = vm->Puv[c] + cr[c] * MP[m];
    }
}

// H0, H1 for the Q's at local vertices ja, jb (0, 1, 2) of the two panels
template <typename T>
GB_HD void vec_combine(const PairGeom<T>& g, const VecMoments<T>& vm, int ja, int jb, cx<T> m4ok2, cx<T>* H0,
                       cx<T>* H1) {
  T al[3], be[3], q[3];
  for (int c = 0; c < 3; c++) {
    al[c] = ja == 0 ? (T)0 : (ja == 1 ? -g.Aa[c] : -g.Ba[c]);
    be[c] = jb == 0 ? (T)0 : (jb == 1 ? -g.Ab[c] : -g.Bb[c]);
    q[c] = g.D0[c] - al[c] + be[c];
  }
  const T ab = al[0] * be[0] + al[1] * be[1] + al[2] * be[2];
  const T bxq[3] = {be[1] * q[2] - be[2] * q[1], be[2] * q[0] - be[0] * q[2], be[0] * q[1] - be[1] * q[0]};
  const T qxa[3] = {q[1] * al[2] - q[2] * al[1], q[2] * al[0] - q[0] * al[2], q[0] * al[1] - q[1] * al[0]};
  // q.(alpha x beta) = alpha.(beta x q)
  const T tq = al[0] * bxq[0] + al[1] * bxq[1] + al[2] * bxq[2];
  cx<T> h0 = vm.Wxy + ab * vm.W0 + m4ok2 * vm.W0;
  cx<T> h1 = tq * vm.P0;
  for (int c = 0; c < 3; c++) {
    h0 = h0 + be[c] * vm.Wx[c] + al[c] * vm.Wy[c];
    h1 = h1 + q[c] * vm.Puv[c] + bxq[c] * vm.Pu[c] + qxa[c] * vm.Pv[c];
  }
  *H0 = h0;
  *H1 = h1;
}

// H0 = sum c MG - (4/k^2) MG[0];  H1 = sum d MP.
template <typename T>
GB_HD void combine(const cx<T>* MG, const cx<T>* MP, const T* c, const T* d, cx<T> m4ok2, cx<T>* H0, cx<T>* H1) {
  cx<T> h0 = m4ok2 * MG[0], h1 = mk((T)0, (T)0);
  for (int m = 0; m < 9; m++) {
    h0 = h0 + c[m] * MG[m];
    h1 = h1 + d[m] * MP[m];
  }
  *H0 = h0;
  *H1 = h1;
}

// ---------------------------------------------------------------------------
// Radial moments E_n(z) = int_0^1 w^n e^{zw} dw, n = 0..NMAX.
// ---------------------------------------------------------------------------
template <int NMAX>
GB_HD void expint_moments(cx<double> z, cx<double>* E) {
  double az2 = cnorm2(z);
  if (az2 < 4.0) {
    // E_n = sum_m z^m/m! / (n+m+1): one pass over m serves every n
    cx<double> term = mk(1.0, 0.0);
    for (int n = 0; n <= NMAX; n++) E[n] = mk(recip_int(n + 1), 0.0);
    for (int m = 1; m < 60; m++) {
      term = recip_int(m) * (term * z);
      double worst = 0.0;
      for (int n = 0; n <= NMAX; n++) {
        const cx<double> t = recip_int(n + m + 1) * term;
        E[n] = E[n] + t;
        worst = fmax(worst, cnorm2(t) / cnorm2(E[n]));
      }
      if (worst < 1e-36) break;
    }
  } else {
    const cx<double> ez = cexpo(z), zi = cdiv(mk(1.0, 0.0), z);
    E[0] = (ez - mk(1.0, 0.0)) * zi;
    for (int n = 1; n <= NMAX; n++) E[n] = (ez - (double)n * E[n - 1]) * zi;
  }
}

// small real polynomials in the radial variable w (degree < 8)
struct rpoly {
  double c[8];
};
GB_HD rpoly rp_aff(double a0, double a1) {
  rpoly p;
  for (int i = 0; i < 8; i++) p.c[i] = 0.0;
  p.c[0] = a0; p.c[1] = a1;
  return p;
}
GB_HD rpoly rp_add(const rpoly& a, const rpoly& b) {
  rpoly p;
  for (int i = 0; i < 8; i++) p.c[i] = a.c[i] + b.c[i];
  return p;
}
GB_HD rpoly rp_scale(const rpoly& a, double s) {
  rpoly p;
  for (int i = 0; i < 8; i++) p.c[i] = a.c[i] * s;
  return p;
}
GB_HD rpoly rp_shift(const rpoly& a) {  // times w
  rpoly p;
  p.c[0] = 0.0;
  for (int i = 0; i + 1 < 8; i++) p.c[i + 1] = a.c[i];
  return p;
}
GB_HD rpoly rp_mul(const rpoly& a, const rpoly& b) {
  rpoly p;
  for (int i = 0; i < 8; i++) p.c[i] = 0.0;
  for (int i = 0; i < 8; i++)
    for (int j = 0; i + j < 8; j++) p.c[i + j] += a.c[i] * b.c[j];
  return p;
}

// ---------------------------------------------------------------------------
// Self-panel (common-triangle) Helmholtz moments MG[9] (H1 vanishes for a
// flat panel).  The 4-D integral over the pair is split as s = s' + z:
// z runs over the 6 sectors of the hexagon T - T in polar form z = w zh(t),
// s' over T ∩ (T - z), a copy of T scaled by lambda(w) = 1 - w sig(zh)
// (integrated exactly by a degree-2 rule), and w analytically against
// e^{ikwX}: the generalized Taylor-Duffy reduction of a common-triangle
// integral to a 1-D smooth integral (TaylorDuffy.cc:152-258 does the same
// reduction with symbolic polynomial tables).  Panel parameters here are the
// edge-ordered ones, s = (s1, s2), x = V0 + s1 (V1-V0) + s2 (V2-V1),
// 0 <= s2 <= s1 <= 1, i.e. TCR (u, v) = (s1 - s2, s2).
//   gx, gw: Gauss-Legendre rule on [0,1] with nt points.
// ---------------------------------------------------------------------------
// Outer points (sector, t) with linear index p = sector*nt + t are visited
// for p = p0, p0 + pstride, ... (a warp can split them over its lanes).
GB_HD void self_moments(const double* V, cx<double> k, const double* gx, const double* gw, int nt, cx<double>* MG,
                        int p0 = 0, int pstride = 1) {
  const double inv4pi = 0.079577471545947667884;
  double E1[3], E2[3];
  for (int i = 0; i < 3; i++) { E1[i] = V[3 + i] - V[i]; E2[i] = V[6 + i] - V[3 + i]; }
  const double H[7][2] = {{1, 0}, {1, 1}, {0, 1}, {-1, 0}, {-1, -1}, {0, -1}, {1, 0}};
  const double TP[3][2] = {{0.5, 0.0}, {1.0, 0.5}, {0.5, 0.5}};
  for (int m = 0; m < 9; m++) MG[m] = mk(0.0, 0.0);
  for (int pp = p0; pp < 6 * nt; pp += pstride) {
      const int sct = pp / nt, it = pp - sct * nt;
      {
      double t = gx[it];
      double z0 = H[sct][0] + t * (H[sct + 1][0] - H[sct][0]);
      double z1 = H[sct][1] + t * (H[sct + 1][1] - H[sct][1]);
      double am = z1 < 0 ? -z1 : 0.0, bm = z0 > 0 ? z0 : 0.0, cm = (z0 - z1) < 0 ? (z0 - z1) : 0.0;
      double sig = bm + am - cm;
      double D[3];
      for (int i = 0; i < 3; i++) D[i] = z0 * E1[i] + z1 * E2[i];
      double X = sqrt(vdot(D, D));
      cx<double> E[5];
      expint_moments<4>(mk(-k.im * X, k.re * X), E);
      // om = lambda^2 = (1 - sig w)^2 (the w lambda^2 of the Jacobian over the 1/w of G)
      const double om0 = 1.0, om1 = -2.0 * sig, om2 = sig * sig;
      const double W = gw[it] * (1.0 / 6.0) * inv4pi / X;
      // sum over the three s' points of the degree-4 polynomials om * ma * mb, then
      // one combination with E_0..E_4 per monomial pair
      double Q[9][5];
      for (int m = 0; m < 9; m++)
        for (int n = 0; n < 5; n++) Q[m][n] = 0.0;
      for (int ip = 0; ip < 3; ip++) {
        double p1 = TP[ip][0], p2 = TP[ip][1];
        // s' = (p1, p2) + w ((am - cm) - sig p1, am - sig p2);  s = s' + w z
        double sb0 = p1, sb1 = (am - cm) - sig * p1, tb0 = p2, tb1 = am - sig * p2;
        double sa0 = sb0, sa1 = sb1 + z0, ta0 = tb0, ta1 = tb1 + z1;
        // TCR coordinates u = s1 - s2, v = s2, affine in w: (c0, c1)
        const double ma[3][2] = {{1.0, 0.0}, {sa0 - ta0, sa1 - ta1}, {ta0, ta1}};
        const double mb[3][2] = {{1.0, 0.0}, {sb0 - tb0, sb1 - tb1}, {tb0, tb1}};
        for (int al = 0; al < 3; al++) {
          const double P0 = om0 * ma[al][0], P1 = om0 * ma[al][1] + om1 * ma[al][0],
                       P2 = om1 * ma[al][1] + om2 * ma[al][0], P3 = om2 * ma[al][1];
          for (int be = 0; be < 3; be++) {
            const double n0 = mb[be][0], n1 = mb[be][1];
            double* q = Q[3 * al + be];
            q[0] += P0 * n0;
            q[1] += P0 * n1 + P1 * n0;
            q[2] += P1 * n1 + P2 * n0;
            q[3] += P2 * n1 + P3 * n0;
            q[4] += P3 * n1;
          }
        }
      }
      for (int m = 0; m < 9; m++) {
        cx<double> sm = mk(0.0, 0.0);
        for (int n = 0; n < 5; n++) sm = sm + Q[m][n] * E[n];
        MG[m] = MG[m] + W * sm;
      }
    }
  }
}


// ---------------------------------------------------------------------------
// Frequency-independent near-pair table (the data the reference caches as
// QIFIPPIData, libscuffInternals.h:282-292), in the TCR mesh-order basis:
//   RM1[9], R1[9], R2[9] = int int mono_m r^p  (p = -1, 1, 2)
//   XM[3] = int int (x - x')/r^3,  XX[3] = int int (xi x xi')/r^3,
// xi = x - V0a (panel a's first mesh vertex).  33 doubles per pair.
// ---------------------------------------------------------------------------
struct Fippi {
  double RM1[9], R1[9], R2[9], XM[3], XX[3];
};

// Segment integrals along the second panel's v' direction (closed forms of
// int (t^2+b2)^{p/2} t^j dt), p = -3, -1, 1, 2; j = 0, 1
// (QIFIPPICubature.cc:240-300 evaluates the same integrals).
GB_HD void seg_integrals(double a2, double v0, double b2, double up, double J[4][2]) {
  double a = sqrt(a2);
  double t1 = -v0, t2 = up - v0;
  double S1 = sqrt(t1 * t1 + b2), S2 = sqrt(t2 * t2 + b2);
  double L;
  if (t1 >= 0) L = log((t2 + S2) / (t1 + S1));
  else if (t2 <= 0) L = log((S1 - t1) / (S2 - t2));
  else L = log((t2 + S2) * (S1 - t1) / b2);
  double Im3_0;
  if (t1 * t2 > 0) Im3_0 = (t2 * t2 - t1 * t1) / (S1 * S2 * (t2 * S1 + t1 * S2));
  else Im3_0 = (t2 / S2 - t1 / S1) / b2;
  double Im3_1 = 1.0 / S1 - 1.0 / S2;
  double Im1_0 = L, Im1_1 = S2 - S1;
  double I1_0 = 0.5 * (t2 * S2 - t1 * S1 + b2 * L), I1_1 = (S2 * S2 * S2 - S1 * S1 * S1) / 3.0;
  double I2_0 = (t2 * t2 * t2 - t1 * t1 * t1) / 3.0 + b2 * (t2 - t1);
  double q1 = t1 * t1 + b2, q2 = t2 * t2 + b2;
  double I2_1 = (q2 * q2 - q1 * q1) / 4.0;
  J[0][0] = Im3_0 / (a2 * a); J[0][1] = (Im3_1 + v0 * Im3_0) / (a2 * a);
  J[1][0] = Im1_0 / a;        J[1][1] = (Im1_1 + v0 * Im1_0) / a;
  J[2][0] = I1_0 * a;         J[2][1] = (I1_1 + v0 * I1_0) * a;
  J[3][0] = I2_0 * a2;        J[3][1] = (I2_1 + v0 * I2_0) * a2;
}

GB_HD void fippi_zero(Fippi* F) {
  for (int m = 0; m < 9; m++) { F->RM1[m] = 0; F->R1[m] = 0; F->R2[m] = 0; }
  for (int i = 0; i < 3; i++) { F->XM[i] = 0; F->XX[i] = 0; }
}

// Non-touching near pair: v' integrated in closed form, (u, v/u, u') by a
// tensor Gauss-Legendre rule (the 3-D scheme of QIFIPPICubature.cc:187-325).
// Va, Vb: 9 doubles each, mesh vertex order.  fippi_far_acc adds one point
// (u, v = u t, u') of weight W; A, B, Ap, Bp are the panels' edge vectors,
// dV = V0b - V0a, a2 = |Bp|^2.
GB_HD void fippi_far_acc(const double* A, const double* B, const double* Ap, const double* Bp, const double* dV,
                         double a2, double u, double v, double up, double W, Fippi& F) {
  double Y[3], Xo[3], Zo[3];
#pragma unroll
  for (int m = 0; m < 3; m++) {
    Xo[m] = u * A[m] + v * B[m];   // x - V0a
    Zo[m] = dV[m] + up * Ap[m];    // z - V0a
    Y[m] = Xo[m] - Zo[m];
  }
  double v0 = vdot(Bp, Y) / a2;
  double b2 = vdot(Y, Y) / a2 - v0 * v0;
  if (b2 < 0) b2 = 0;
  double J[4][2];
  seg_integrals(a2, v0, b2, up, J);
#pragma unroll
  for (int m = 0; m < 3; m++) F.XM[m] += W * (Y[m] * J[0][0] - Bp[m] * J[0][1]);
  double XZ[3], XB[3];
  vcross(Xo, Zo, XZ); vcross(Xo, Bp, XB);
#pragma unroll
  for (int m = 0; m < 3; m++) F.XX[m] += W * (XZ[m] * J[0][0] + XB[m] * J[0][1]);
  // TCR a-side monomials {1, u - v, v}; b-side {1, u' - v', v'}
  const double ma[3] = {1.0, u - v, v};
#pragma unroll
  for (int al = 0; al < 3; al++) {
    double f = W * ma[al];
    F.RM1[3 * al + 0] += f * J[1][0]; F.RM1[3 * al + 1] += f * (up * J[1][0] - J[1][1]); F.RM1[3 * al + 2] += f * J[1][1];
    F.R1[3 * al + 0] += f * J[2][0];  F.R1[3 * al + 1] += f * (up * J[2][0] - J[2][1]);  F.R1[3 * al + 2] += f * J[2][1];
    F.R2[3 * al + 0] += f * J[3][0];  F.R2[3 * al + 1] += f * (up * J[3][0] - J[3][1]);  F.R2[3 * al + 2] += f * J[3][1];
  }
}

GB_HD void fippi_far_setup(const double* Va, const double* Vb, double* A, double* B, double* Ap, double* Bp, double* dV,
                           double* a2) {
  for (int i = 0; i < 3; i++) {
    A[i] = Va[3 + i] - Va[i]; B[i] = Va[6 + i] - Va[3 + i];
    Ap[i] = Vb[3 + i] - Vb[i]; Bp[i] = Vb[6 + i] - Vb[3 + i];
    dV[i] = Vb[i] - Va[i];
  }
  *a2 = vdot(Bp, Bp);
}

GB_HD void fippi_far(const double* Va, const double* Vb, const double* gx, const double* gw, int n, Fippi* F) {
  double A[3], B[3], Ap[3], Bp[3], dV[3], a2;
  fippi_far_setup(Va, Vb, A, B, Ap, Bp, dV, &a2);
  fippi_zero(F);
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++)
      for (int l = 0; l < n; l++) {
        double u = gx[i];
        fippi_far_acc(A, B, Ap, Bp, dV, a2, u, u * gx[j], gx[l], gw[i] * gw[j] * gw[l] * u, *F);
      }
}

// Touching pair (ncv = 1 common vertex, 2 common edge).  pa/pb map the
// common-vertices-first order to mesh order (E_i = V[p[i]]).  Duffy splits:
//  ncv=1: s1 = w, s2 = w al, s1' = w be, s2' = w be ga (and mirror), w^3 be;
//  ncv=2: (u-u', v, v') = w zhat over 4 polyhedral pieces, u' on its
//         interval of length 1-w (exact 2-point rule), w^2 (1-w).
// Edge-ordered parameters s: x = E0 + s1 (E1-E0) + s2 (E2-E1).
struct DuffyPt {
  double W;       // constant weight
  rpoly om;       // Jacobian polynomial in w
  double sa0[2], sa1[2], sb0[2], sb1[2];
};

GB_HD void tcr_from_edge(const int* perm, const double* s0, const double* s1, rpoly* u, rpoly* v) {
  // barycentrics on (E0,E1,E2): (1 - s1, s1 - s2, s2), affine in w; mesh
  // vertex perm[i] carries barycentric i (selected without data-dependent
  // array indexing)
  double m0[3] = {1.0 - s0[0], s0[0] - s0[1], s0[1]};
  double m1[3] = {-s1[0], s1[0] - s1[1], s1[1]};
  int i1 = perm[0] == 1 ? 0 : (perm[1] == 1 ? 1 : 2);
  int i2 = perm[0] == 2 ? 0 : (perm[1] == 2 ? 1 : 2);
  double u0 = i1 == 0 ? m0[0] : (i1 == 1 ? m0[1] : m0[2]);
  double u1 = i1 == 0 ? m1[0] : (i1 == 1 ? m1[1] : m1[2]);
  double v0 = i2 == 0 ? m0[0] : (i2 == 1 ? m0[1] : m0[2]);
  double v1 = i2 == 0 ? m1[0] : (i2 == 1 ? m1[1] : m1[2]);
  *u = rp_aff(u0, u1);
  *v = rp_aff(v0, v1);
}

// Duffy point q of a touching pair's cells (ncv = 1: 2 n^3 points, ncv = 2:
// 8 n^2 points), in the order fippi_touch and td_touch walk them.
GB_HD int duffy_npts(int ncv, int n) { return ncv == 1 ? 2 * n * n * n : 8 * n * n; }

GB_HD void duffy_pt(int ncv, int q, const double* gx, const double* gw, int n, DuffyPt& pt) {
  if (ncv == 1) {
    const int reg = q / (n * n * n), rem = q % (n * n * n);
    const int i1 = rem / (n * n), i2 = (rem / n) % n, i3 = rem % n;
    const double al = gx[i1], be = gx[i2], ga = gx[i3];
    pt.sa0[0] = pt.sa0[1] = pt.sb0[0] = pt.sb0[1] = 0.0;
    if (reg == 0) { pt.sa1[0] = 1.0; pt.sa1[1] = al; pt.sb1[0] = be; pt.sb1[1] = be * ga; }
    else { pt.sb1[0] = 1.0; pt.sb1[1] = al; pt.sa1[0] = be; pt.sa1[1] = be * ga; }
    pt.om = rp_aff(0.0, 0.0); pt.om.c[3] = be;
    pt.W = gw[i1] * gw[i2] * gw[i3];
  } else {
    const double tx[2] = {0.21132486540518711775, 0.78867513459481288225};
    const int reg = q / (2 * n * n), rem = q % (2 * n * n);
    const int ia = rem / (2 * n), ib = (rem / 2) % n, it = rem % 2;
    const double al = gx[ia], be = gx[ib];
    double z[3], J, lo;
    if (reg == 0) { z[0] = 1.0 - al; z[1] = be; z[2] = al; J = 1.0; lo = al; }
    else if (reg == 1) { z[0] = al; z[1] = 1.0; z[2] = (1.0 - al) * be; J = 1.0 - al; lo = 1.0 - al; }
    else if (reg == 2) { z[0] = -al; z[1] = (1.0 - al) * be; z[2] = 1.0; J = 1.0 - al; lo = 1.0; }
    else { z[0] = -al; z[1] = 1.0 - al; z[2] = be; J = 1.0; lo = 1.0; }
    const double tau = tx[it];
    pt.sb0[0] = tau; pt.sb1[0] = lo - tau;
    pt.sb0[1] = 0.0; pt.sb1[1] = z[2];
    pt.sa0[0] = tau; pt.sa1[0] = lo - tau + z[0];
    pt.sa0[1] = 0.0; pt.sa1[1] = z[1];
    pt.om = rp_aff(0.0, 0.0); pt.om.c[2] = 1.0; pt.om.c[3] = -1.0;
    pt.W = gw[ia] * gw[ib] * 0.5 * J;
  }
}

// One Duffy point of a touching pair's static integrals.  The cells'
// Jacobian is om(w) = o2 w^2 + o3 w^3 (o2 = 0, o3 = beta for one common
// vertex; o2 = 1, o3 = -1 for a common edge) and the monomials are affine in
// w, so every radial integral int_0^1 om(w) w^e dw is the short closed sum
// h(e) = o2 / (e+3) + o3 / (e+4) over the powers of the monomial product.
GB_HD void fippi_touch_acc(const double* Ea, const double* Eb, const int* pa, const int* pb, const double* V0a,
                           const DuffyPt& pt, Fippi& F) {
  double A[3], B[3], Ap[3], Bp[3], D[3];
#pragma unroll
  for (int i = 0; i < 3; i++) {
    A[i] = Ea[3 + i] - Ea[i]; B[i] = Ea[6 + i] - Ea[3 + i];
    Ap[i] = Eb[3 + i] - Eb[i]; Bp[i] = Eb[6 + i] - Eb[3 + i];
    D[i] = pt.sa1[0] * A[i] + pt.sa1[1] * B[i] - pt.sb1[0] * Ap[i] - pt.sb1[1] * Bp[i];
  }
  const double X = sqrt(vdot(D, D));
  const double o2 = pt.om.c[2], o3 = pt.om.c[3];
  rpoly ua, va, ub, vb;
  tcr_from_edge(pa, pt.sa0, pt.sa1, &ua, &va);
  tcr_from_edge(pb, pt.sb0, pt.sb1, &ub, &vb);
  const double a0[3] = {1.0, ua.c[0], va.c[0]}, a1[3] = {0.0, ua.c[1], va.c[1]};
  const double b0[3] = {1.0, ub.c[0], vb.c[0]}, b1[3] = {0.0, ub.c[1], vb.c[1]};
  // the monomial product m0 + m1 w + m2 w^2 meets w^-1 (r^-1), w (r), w^2 (r^2)
  constexpr double inv[9] = {0.0, 1.0, 1.0 / 2, 1.0 / 3, 1.0 / 4, 1.0 / 5, 1.0 / 6, 1.0 / 7, 1.0 / 8};
  auto h = [&](int e) { return o2 * inv[e + 2] + o3 * inv[e + 3]; };
  const double hm1[3] = {h(0), h(1), h(2)};   // r^-1
  const double h1[3] = {h(2), h(3), h(4)};    // r
  const double h2[3] = {h(3), h(4), h(5)};    // r^2
  const double iX = 1.0 / X;
  const double WX = pt.W * X, WXX = pt.W * X * X, WoX = pt.W * iX;
#pragma unroll
  for (int al = 0; al < 3; al++)
#pragma unroll
    for (int be = 0; be < 3; be++) {
      const double m0 = a0[al] * b0[be], m1 = a0[al] * b1[be] + a1[al] * b0[be], m2 = a1[al] * b1[be];
      F.RM1[3 * al + be] += WoX * (m0 * hm1[0] + m1 * hm1[1] + m2 * hm1[2]);
      F.R1[3 * al + be] += WX * (m0 * h1[0] + m1 * h1[1] + m2 * h1[2]);
      F.R2[3 * al + be] += WXX * (m0 * h2[0] + m1 * h2[1] + m2 * h2[2]);
    }
  // (x - x')/r^3 = D / (w^2 X^3): int om w^-2 = o2 + o3 / 2
  const double iX3 = iX * iX * iX;
  const double om2 = o2 + 0.5 * o3;
#pragma unroll
  for (int m = 0; m < 3; m++) F.XM[m] += pt.W * om2 * D[m] * iX3;
  // xi(w) = x(w) - V0a = c0 + c1 w; (xi x xi')/r^3 -> -(xi(w) x D) w / (w^3 X^3):
  // int om (c0 + c1 w) w^-2 dw = c0 (o2 + o3/2) + c1 (o2/2 + o3/3)
  const double g0 = om2, g1 = 0.5 * o2 + o3 / 3.0;
  double c0[3], c1[3];
#pragma unroll
  for (int m = 0; m < 3; m++) {
    c0[m] = Ea[m] - V0a[m] + pt.sa0[0] * A[m] + pt.sa0[1] * B[m];
    c1[m] = pt.sa1[0] * A[m] + pt.sa1[1] * B[m];
  }
#pragma unroll
  for (int m = 0; m < 3; m++) {
    const int m1 = (m + 1) % 3, m2 = (m + 2) % 3;
    const double x0 = c0[m1] * D[m2] - c0[m2] * D[m1], x1 = c1[m1] * D[m2] - c1[m2] * D[m1];
    F.XX[m] += -pt.W * (x0 * g0 + x1 * g1) * iX3;
  }
}

GB_HD void touch_edges(const double* Va, const double* Vb, const int* pa, const int* pb, double* Ea, double* Eb) {
  for (int i = 0; i < 3; i++)
    for (int c = 0; c < 3; c++) {
      Ea[3 * i + c] = pa[i] == 0 ? Va[c] : (pa[i] == 1 ? Va[3 + c] : Va[6 + c]);
      Eb[3 * i + c] = pb[i] == 0 ? Vb[c] : (pb[i] == 1 ? Vb[3 + c] : Vb[6 + c]);
    }
}

GB_HD void fippi_touch(int ncv, const double* Va, const double* Vb, const int* pa, const int* pb, const double* gx,
                       const double* gw, int n, Fippi* F) {
  double Ea[9], Eb[9];
  touch_edges(Va, Vb, pa, pb, Ea, Eb);
  fippi_zero(F);
  DuffyPt pt;
  const int np = duffy_npts(ncv, n);
  for (int q = 0; q < np; q++) {
    duffy_pt(ncv, q, gx, gw, n, pt);
    fippi_touch_acc(Ea, Eb, pa, pb, Va, pt, *F);
  }
}

// ---------------------------------------------------------------------------
// Touching pairs with the full Helmholtz kernel (the short-wavelength branch
// of PanelPanelInteractions.cc:449-491, which the reference evaluates by
// Taylor-Duffy with KIndex HELMHOLTZ / GRADHELMHOLTZ).  Same Duffy cells as
// fippi_touch; along each ray x - x' = w D (r = w X) the radial integrals are
// the E_n(ikX) of expint_moments.  Outputs, per (pair, region):
//   MG[9]  = int int mono_m G                     (H0 as for far pairs)
//   T[10]  = { int int (u x v).(x-x') Psi,  int int (x-x') x u Psi [3],
//              int int v x (x-x') Psi [3],  int int (x-x') Psi [3] }
// with u = x - V0a, v = x' - V0b (mesh order).  For Q's with alpha = V0a - Qa,
// beta = V0b - Qb:  H1 = T0 + beta.Tu + alpha.Tv + (alpha x beta).Tr, since
// ((u+alpha) x (v+beta)).(x-x') splits that way; every integrand keeps the
// factor (x - x') that makes the r^-3 of Psi integrable.
// ---------------------------------------------------------------------------
GB_HD_NOINLINE void td_touch_point(const double* Ea, const double* Eb, const int* pa, const int* pb,
                                   const double* Va, const double* Vb, cx<double> k, const DuffyPt& pt,
                                   cx<double>* MG, cx<double>* T) {
  const double inv4pi = 0.079577471545947667884;
  double A[3], B[3], Ap[3], Bp[3], D[3];
  for (int i = 0; i < 3; i++) {
    A[i] = Ea[3 + i] - Ea[i]; B[i] = Ea[6 + i] - Ea[3 + i];
    Ap[i] = Eb[3 + i] - Eb[i]; Bp[i] = Eb[6 + i] - Eb[3 + i];
    D[i] = pt.sa1[0] * A[i] + pt.sa1[1] * B[i] - pt.sb1[0] * Ap[i] - pt.sb1[1] * Bp[i];
  }
  const double X = sqrt(vdot(D, D));
  rpoly ua, va, ub, vb;
  tcr_from_edge(pa, pt.sa0, pt.sa1, &ua, &va);
  tcr_from_edge(pb, pt.sb0, pt.sb1, &ub, &vb);
  cx<double> E[5];
  expint_moments<4>(mk(-k.im * X, k.re * X), E);
  // G: sum_n p_n E_{n-1} / (4 pi X), p = om ma mb
  const rpoly one = rp_aff(1.0, 0.0);
  const rpoly ma[3] = {one, ua, va}, mb[3] = {one, ub, vb};
  const double gfac = pt.W * inv4pi / X;
  for (int al = 0; al < 3; al++)
    for (int be = 0; be < 3; be++) {
      const rpoly q = rp_mul(pt.om, rp_mul(ma[al], mb[be]));
      cx<double> sm = mk(0.0, 0.0);
      for (int n = 1; n <= 5; n++) sm = sm + q.c[n] * E[n - 1];
      MG[3 * al + be] = MG[3 * al + be] + gfac * sm;
    }
  // Psi: p = om w S(w); L[p] = sum_n p_n (ik/(4 pi X^2) E_{n-2} - 1/(4 pi X^3) E_{n-3})
  const cx<double> c2 = (pt.W * inv4pi / (X * X)) * mk(-k.im, k.re);
  const double c3 = -pt.W * inv4pi / (X * X * X);
  auto Lpsi = [&](const rpoly& Sw) {
    const rpoly p = rp_mul(pt.om, rp_shift(Sw));
    cx<double> acc = mk(0.0, 0.0);
    for (int n = 2; n <= 6; n++) acc = acc + p.c[n] * (c2 * E[n - 2]);
    for (int n = 3; n <= 7; n++) acc = acc + (c3 * p.c[n]) * E[n - 3];
    return acc;
  };
  double Aa[3], Ba[3], Ab[3], Bb[3];
  for (int i = 0; i < 3; i++) {
    Aa[i] = Va[3 + i] - Va[i]; Ba[i] = Va[6 + i] - Va[i];
    Ab[i] = Vb[3 + i] - Vb[i]; Bb[i] = Vb[6 + i] - Vb[i];
  }
  double x1[3], x2[3], x3[3], x4[3];
  vcross(Aa, Ab, x1); vcross(Aa, Bb, x2); vcross(Ba, Ab, x3); vcross(Ba, Bb, x4);
  // (u x v).D with u = ua Aa + va Ba, v = ub Ab + vb Bb
  const rpoly S0 = rp_add(rp_add(rp_scale(rp_mul(ua, ub), vdot(x1, D)), rp_scale(rp_mul(ua, vb), vdot(x2, D))),
                          rp_add(rp_scale(rp_mul(va, ub), vdot(x3, D)), rp_scale(rp_mul(va, vb), vdot(x4, D))));
  T[0] = T[0] + Lpsi(S0);
  double dA[3], dB[3], aD[3], bD[3];
  vcross(D, Aa, dA); vcross(D, Ba, dB); vcross(Ab, D, aD); vcross(Bb, D, bD);
  const cx<double> L1 = Lpsi(one);
  for (int c = 0; c < 3; c++) {
    T[1 + c] = T[1 + c] + Lpsi(rp_add(rp_scale(ua, dA[c]), rp_scale(va, dB[c])));   // (x-x') x u
    T[4 + c] = T[4 + c] + Lpsi(rp_add(rp_scale(ub, aD[c]), rp_scale(vb, bD[c])));   // v x (x-x')
    T[7 + c] = T[7 + c] + D[c] * L1;                                                  // (x-x')
  }
}

// Duffy cells of fippi_touch with the full kernel (ncv = 1 or 2); pt index
// range [p0, npts) in steps of pstride lets a warp split the points.
GB_HD int td_touch_npts(int ncv, int n) { return duffy_npts(ncv, n); }

GB_HD void td_touch(int ncv, const double* Va, const double* Vb, const int* pa, const int* pb, cx<double> k,
                    const double* gx, const double* gw, int n, int p0, int pstride, cx<double>* MG, cx<double>* T) {
  double Ea[9], Eb[9];
  touch_edges(Va, Vb, pa, pb, Ea, Eb);
  for (int m = 0; m < 9; m++) MG[m] = mk(0.0, 0.0);
  for (int m = 0; m < 10; m++) T[m] = mk(0.0, 0.0);
  const int np = td_touch_npts(ncv, n);
  DuffyPt pt;
  for (int q = p0; q < np; q += pstride) {
    duffy_pt(ncv, q, gx, gw, n, pt);
    td_touch_point(Ea, Eb, pa, pb, Va, Vb, k, pt, MG, T);
  }
}

// H1 of touching pairs from the T moments
GB_HD cx<double> td_h1(const double* Va, const double* Vb, const cx<double>* T, int ja, int jb) {
  double al[3], be[3], ab[3];
  for (int c = 0; c < 3; c++) {
    al[c] = Va[c] - Va[3 * ja + c];
    be[c] = Vb[c] - Vb[3 * jb + c];
  }
  vcross(al, be, ab);
  cx<double> h = T[0];
  for (int c = 0; c < 3; c++) h = h + be[c] * T[1 + c] + al[c] * T[4 + c] + ab[c] * T[7 + c];
  return h;
}

// ---------------------------------------------------------------------------
// Desingularised near pair (PanelPanelInteractions.cc:504-559): the fixed-rule
// moments of the ExpRel(ikr,4) remainder plus the Taylor terms rebuilt from
// the static table.  Adds to MG/MP; returns the extra r^-3 term of H1 per
// (Qa,Qb) through hTimesRM3 = (Qa-Qb).XX + (Qa x Qb).XM (origin V0a), which
// enters H1 with the factor -1/(4 pi).
//   PF[n] = (ik)^n/(4 pi):
//   MG += PF0 RM1 + PF1 R0 + PF2/2 R1 + PF3/6 R2
//   MP += PF2/2 RM1 + PF3/3 R0 + PF4/6 R1
// ---------------------------------------------------------------------------
GB_HD void add_taylor_terms(const Fippi& F, cx<double> k, cx<double>* MG, cx<double>* MP) {
  const double R0[9] = {1.0 / 4, 1.0 / 12, 1.0 / 12, 1.0 / 12, 1.0 / 36, 1.0 / 36, 1.0 / 12, 1.0 / 36, 1.0 / 36};
  const double inv4pi = 0.079577471545947667884;
  cx<double> ik = mk(-k.im, k.re);
  cx<double> PF[5];
  PF[0] = mk(inv4pi, 0.0);
  for (int i = 1; i < 5; i++) PF[i] = PF[i - 1] * ik;
  for (int m = 0; m < 9; m++) {
    MG[m] = MG[m] + F.RM1[m] * PF[0] + R0[m] * PF[1] + (0.5 * F.R1[m]) * PF[2] + (F.R2[m] / 6.0) * PF[3];
    MP[m] = MP[m] + (0.5 * F.RM1[m]) * PF[2] + (R0[m] / 3.0) * PF[3] + (F.R1[m] / 6.0) * PF[4];
  }
}

GB_HD double htimes_rm3(const Fippi& F, const double* Va, const double* Vb, int ja, int jb) {
  double qa[3], qb[3], d[3], x[3];
  for (int i = 0; i < 3; i++) { qa[i] = Va[3 * ja + i] - Va[i]; qb[i] = Vb[3 * jb + i] - Va[i]; d[i] = qa[i] - qb[i]; }
  vcross(qa, qb, x);
  return vdot(d, F.XX) + vdot(x, F.XM);
}

}  // namespace gbem
