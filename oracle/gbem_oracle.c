/*
 * gbem_oracle.c -- CPU oracle for the BEM hot path (TEST INFRASTRUCTURE ONLY).
 *
 * A plain-C restatement of the reference's (HomerReid/scuff-em) algorithm for
 * BEM matrix assembly, used by tests/ as the checker for the CUDA library, by
 * __graft_entry__.smoke(), and by bench.py's CPU-baseline leg.  Nothing in the
 * product links or calls this file.
 *
 * Every function cites the reference file:line it restates.  Parity of this
 * oracle is pinned against (a) the panel-panel golden values embedded in the
 * reference's own unit test (unitTests/unit-test-PPIs.cc:70-134) and (b)
 * outputs of the reference itself, built from its sources by oracle/ref/.
 *
 * Singular integrals: the reference evaluates common-triangle / -edge / -vertex
 * panel pairs with its generalized Taylor-Duffy method (TaylorDuffy.cc) and
 * Q-independent static integrals (FIPPIs) with adaptive cubature
 * (QIFIPPICubature.cc, QIFIPPITaylorDuffyV2P0.cc).  This oracle evaluates the
 * same integrals by Duffy-type splittings of the 4-D domain into cells with a
 * radial variable w, integrating w analytically and the remaining variables
 * with high-order Gauss-Legendre rules (the published Taylor-Duffy / Duffy
 * idea, derived independently here), so its values agree with the reference's
 * to the reference's own quadrature tolerance.
 */
#include <math.h>
#include <complex.h>
#include <stdlib.h>
#include <string.h>
#include <stdio.h>

typedef double complex cplx;

#define PI 3.14159265358979323846

/* ------------------------------------------------------------------ */
/* small vector helpers                                                */
/* ------------------------------------------------------------------ */
static inline void vsub(const double *a, const double *b, double *c) { c[0]=a[0]-b[0]; c[1]=a[1]-b[1]; c[2]=a[2]-b[2]; }
static inline double vdot(const double *a, const double *b) { return a[0]*b[0]+a[1]*b[1]+a[2]*b[2]; }
static inline void vcross(const double *a, const double *b, double *c)
{ c[0]=a[1]*b[2]-a[2]*b[1]; c[1]=a[2]*b[0]-a[0]*b[2]; c[2]=a[0]*b[1]-a[1]*b[0]; }
static inline double vnorm(const double *a) { return sqrt(vdot(a,a)); }
static inline double vdist(const double *a, const double *b) { double d[3]; vsub(a,b,d); return vnorm(d); }

/* ------------------------------------------------------------------ */
/* Gauss-Legendre rule on [0,1] (Golub-Welsch free: Newton on P_n)     */
/* ------------------------------------------------------------------ */
static void gauss_legendre01(int n, double *x, double *w)
{
  for (int i = 0; i < n; i++) {
    double z = cos(PI * (i + 0.75) / (n + 0.5)), pp = 0.0;
    for (int it = 0; it < 100; it++) {
      double p1 = 1.0, p2 = 0.0;
      for (int j = 1; j <= n; j++) { double p3 = p2; p2 = p1; p1 = ((2.0*j-1.0)*z*p2 - (j-1.0)*p3)/j; }
      pp = n * (z*p1 - p2) / (z*z - 1.0);
      double z1 = z; z = z1 - p1/pp;
      if (fabs(z - z1) < 1e-16) break;
    }
    x[i] = 0.5 * (1.0 - z);
    w[i] = 1.0 / ((1.0 - z*z) * pp * pp);
  }
}

/* ------------------------------------------------------------------ */
/* Triangle cubature rules.                                            */
/* LO rule: the 6-point degree-4 rule with the exact 13-digit values   */
/* the reference tabulates (libs/libTriInt/TCR.cc:83-91).  The same   */
/* values are required for entry-level parity of far-field pairs.      */
/* HO rule: a collapsed Gauss-Legendre product rule of degree 20       */
/* (the reference's 78-point order-20 table, TCR.cc:346, is replaced;  */
/* high-order pairs agree to cubature accuracy, not bitwise).          */
/* Layout: (u, v, w) triples over {u,v>=0, u+v<=1}, weights sum 1/2.   */
/* ------------------------------------------------------------------ */
static const double TCR_LO[18] = {
  0.0915762135098, 0.0915762135098, 0.0549758718276,
  0.8168475729805, 0.0915762135098, 0.0549758718276,
  0.0915762135098, 0.8168475729805, 0.0549758718276,
  0.1081030181681, 0.4459484909160, 0.1116907948390,
  0.4459484909160, 0.1081030181681, 0.1116907948390,
  0.4459484909160, 0.4459484909160, 0.1116907948390 };

#define HO_N 11
static double TCR_HO[3*HO_N*HO_N];
static int tcr_ho_ready = 0;
static void init_tcr_ho(void)
{
  if (tcr_ho_ready) return;
  double x[HO_N], w[HO_N];
  gauss_legendre01(HO_N, x, w);
  int k = 0;
  for (int i = 0; i < HO_N; i++)
    for (int j = 0; j < HO_N; j++) {
      double xi = x[i], eta = x[j];
      TCR_HO[k++] = xi * (1.0 - eta);
      TCR_HO[k++] = xi * eta;
      TCR_HO[k++] = w[i] * w[j] * xi;
    }
  tcr_ho_ready = 1;
}

/* ------------------------------------------------------------------ */
/* ExpRel(x,n): sum_{m>=n} x^m/m!, truncated at relative 1e-8          */
/* (PanelPanelInteractions.cc:86-103).                                 */
/* ------------------------------------------------------------------ */
static cplx exprel_ppi(cplx x, int n)
{
  cplx term = 1.0, sum = 0.0;
  int m;
  for (m = 1; m < n; m++) term *= x / (double)m;
  for (sum = 0.0; m < 100; m++) {
    term *= x / (double)m;
    sum += term;
    double t2 = creal(term)*creal(term) + cimag(term)*cimag(term);
    double s2 = creal(sum)*creal(sum) + cimag(sum)*cimag(sum);
    if (t2 < 1e-16 * s2) break;
  }
  return sum;
}

/* ------------------------------------------------------------------ */
/* geometry                                                            */
/* ------------------------------------------------------------------ */
typedef struct {
  int nv, np, ne;
  const double *V;     /* 3*nv */
  const int *PV;       /* 3*np */
  double *centroid;    /* 3*np */
  double *radius;      /* np */
  double *area;        /* np */
  /* edges: iV1 iV2 iQP iQM iPPanel iMPanel PIndex MIndex */
  int *E;              /* 8*ne */
  double *elen;        /* ne */
  /* memo of Q-independent FIPPI data per ordered same-surface panel pair
     (the role of FIPPICache, FIPPICache.cc:135-187) */
  long long *fkey;
  void *fval;
  int fcap;
} ora_surface;

/* Panel data (RWGSurface.cc:55-100). */
static void init_panels(ora_surface *S)
{
  for (int p = 0; p < S->np; p++) {
    const double *v0 = S->V + 3*S->PV[3*p], *v1 = S->V + 3*S->PV[3*p+1], *v2 = S->V + 3*S->PV[3*p+2];
    double *c = S->centroid + 3*p;
    for (int i = 0; i < 3; i++) c[i] = (v0[i] + v1[i] + v2[i]) / 3.0;
    double r = vdist(c, v0);
    r = fmax(r, vdist(c, v1));
    r = fmax(r, vdist(c, v2));
    S->radius[p] = r;
    double a[3], b[3], z[3];
    vsub(v1, v0, a); vsub(v2, v0, b); vcross(a, b, z);
    S->area[p] = 0.5 * vnorm(z);
  }
}

/* Interior-edge list (InitEdgeList.cc:127-205): edges are visited panel by  */
/* panel, local edge ne = (VI[ne], VI[ne+1]); the first visiting panel is    */
/* the positive panel (Q = VI[ne+2]); an edge gets its index when the second */
/* panel visits it.  Returns the number of interior edges, or -1 on a       */
/* non-manifold mesh.                                                       */
int ora_build_edges(int nv, int np, const int *PV, int *Eout, int maxe)
{
  /* open-addressing table keyed by (lesser, greater) vertex */
  int cap = 1; while (cap < 6*np + 16) cap <<= 1;
  long long *key = malloc(sizeof(long long) * cap);
  int *slot = malloc(sizeof(int) * cap);
  for (int i = 0; i < cap; i++) key[i] = -1;
  size_t ntot = 6 * (size_t)(np > 0 ? np : 1);
  int *tmp = malloc(sizeof(int) * 8 * ntot);
  int *tidx = malloc(sizeof(int) * ntot);
  int nt = 0, ne = 0, bad = 0;
  for (int p = 0; p < np && !bad; p++)
    for (int j = 0; j < 3; j++) {
      int a = PV[3*p + j], b = PV[3*p + (j+1)%3];
      int lo = a < b ? a : b, hi = a < b ? b : a;
      long long k = (long long)lo * (long long)(nv + 1) + hi;
      unsigned long long h = (unsigned long long)k * 0x9E3779B97F4A7C15ULL;
      int s = (int)(h >> 40) & (cap - 1);
      while (key[s] != -1 && key[s] != k) s = (s + 1) & (cap - 1);
      if (key[s] == -1) {
        key[s] = k; slot[s] = nt;
        int *t = tmp + 8*nt;
        t[0] = lo; t[1] = hi; t[2] = PV[3*p + (j+2)%3]; t[3] = -1;
        t[4] = p; t[5] = -1; t[6] = (j+2)%3; t[7] = (j+2)%3;
        tidx[nt] = -1;
        nt++;
      } else {
        int *t = tmp + 8*slot[s];
        if (t[5] != -1) { bad = 1; break; }
        t[3] = PV[3*p + (j+2)%3]; t[5] = p; t[7] = (j+2)%3;
        tidx[slot[s]] = ne++;
      }
    }
  if (!bad && ne <= maxe)
    for (int i = 0; i < nt; i++)
      if (tidx[i] >= 0) memcpy(Eout + 8*tidx[i], tmp + 8*i, 8*sizeof(int));
  free(key); free(slot); free(tmp); free(tidx);
  return bad ? -1 : ne;
}

/* ------------------------------------------------------------------ */
/* AssessPanelPair (AssessPanelPair.cc:52-103, 147-172)                */
/* ------------------------------------------------------------------ */
static int vclose(const double *a, const double *b, double tol)
{ return fabs(a[0]-b[0]) + fabs(a[1]-b[1]) + fabs(a[2]-b[2]) <= 3*tol; }

static int assess_order(const double *Va[3], const double *Vb[3], double rmax)
{
  int ncv = 0, ca[3], cb[3];
  double tol = fabs(1.0e-6 * rmax);
  for (int ia = 0; ia < 3; ia++)
    for (int ib = 0; ib < 3; ib++)
      if (vclose(Va[ia], Vb[ib], tol)) { ca[ncv] = ia; cb[ncv] = ib; ncv++; }
  if (ncv == 0) return 0;
  const double *oa[3] = {Va[0], Va[1], Va[2]}, *ob[3] = {Vb[0], Vb[1], Vb[2]};
  if (ncv == 1) {
    for (int i = 0; i < 3; i++) { Va[i] = oa[(ca[0]+i)%3]; Vb[i] = ob[(cb[0]+i)%3]; }
  } else if (ncv == 2) {
    Va[0] = oa[ca[0]]; Va[1] = oa[ca[1]]; Va[2] = oa[3-ca[0]-ca[1]];
    Vb[0] = ob[cb[0]]; Vb[1] = ob[cb[1]]; Vb[2] = ob[3-cb[0]-cb[1]];
  } else {
    for (int i = 0; i < 3; i++) { Va[i] = oa[ca[i]]; Vb[i] = ob[cb[i]]; }
  }
  return ncv;
}

static int assess_pair(const ora_surface *Sa, int pa, const ora_surface *Sb, int pb,
                       double *rrel, const double *Va[3], const double *Vb[3])
{
  for (int i = 0; i < 3; i++) { Va[i] = Sa->V + 3*Sa->PV[3*pa+i]; Vb[i] = Sb->V + 3*Sb->PV[3*pb+i]; }
  double rmax = fmax(Sa->radius[pa], Sb->radius[pb]);
  double d[3]; vsub(Sa->centroid + 3*pa, Sb->centroid + 3*pb, d);
  *rrel = sqrt(vdot(d,d)) / rmax;
  if (*rrel > 2.0) return 0;
  return assess_order(Va, Vb, rmax);
}

/* ------------------------------------------------------------------ */
/* Fixed-rule panel-pair cubature (PanelPanelInteractions.cc:108-201,  */
/* 211-350): H[0] = int int (F.F' - 4/k^2) Phi, H[1] = int int         */
/* ((F x F').R) Psi, Phi = e^{ikr}/(4 pi r) (or ExpRel(ikr,4)/(4 pi r) */
/* when desingularised), Psi = Phi (ik - 1/r)/r.                       */
/* ------------------------------------------------------------------ */
static void ppi_cubature(cplx k, int desing, int high, const double *Va[3], const double *Qa,
                         const double *Vb[3], const double *Qb, cplx H[2])
{
  const double *tcr; int npts;
  if (high) { init_tcr_ho(); tcr = TCR_HO; npts = HO_N*HO_N; } else { tcr = TCR_LO; npts = 6; }
  double A[3], B[3], AP[3], BP[3];
  vsub(Va[1], Va[0], A); vsub(Va[2], Va[0], B);
  vsub(Vb[1], Vb[0], AP); vsub(Vb[2], Vb[0], BP);
  cplx ik = I*k, ik2 = ik*ik;
  H[0] = H[1] = 0.0;
  for (int i = 0; i < npts; i++) {
    double u = tcr[3*i], v = tcr[3*i+1], w = tcr[3*i+2];
    double X[3], F[3];
    for (int m = 0; m < 3; m++) { X[m] = Va[0][m] + u*A[m] + v*B[m]; F[m] = X[m] - Qa[m]; }
    cplx hi0 = 0.0, hi1 = 0.0;
    for (int j = 0; j < npts; j++) {
      double up = tcr[3*j], vp = tcr[3*j+1], wp = tcr[3*j+2];
      double XP[3], FP[3], R[3], FxFP[3];
      for (int m = 0; m < 3; m++) { XP[m] = Vb[0][m] + up*AP[m] + vp*BP[m]; FP[m] = XP[m] - Qb[m]; R[m] = X[m] - XP[m]; }
      cplx hplus = vdot(F, FP) + 4.0/ik2;
      vcross(F, FP, FxFP);
      double r2 = vdot(R,R), r = sqrt(r2);
      cplx phi = desing ? exprel_ppi(ik*r, 4) / (4.0*PI*r) : cexp(ik*r) / (4.0*PI*r);
      if (!isfinite(creal(phi))) phi = 0.0;
      phi *= wp;
      cplx psi = phi * (ik - 1.0/r) / r;
      hi0 += hplus * phi;
      hi1 += vdot(FxFP, R) * psi;
    }
    H[0] += w * hi0;
    H[1] += w * hi1;
  }
}

/* ------------------------------------------------------------------ */
/* real polynomials in the radial Duffy variable w                     */
/* ------------------------------------------------------------------ */
#define PD 10
typedef struct { double c[PD]; } rpoly;
static inline rpoly rp_aff(double a0, double a1) { rpoly p; memset(&p,0,sizeof p); p.c[0]=a0; p.c[1]=a1; return p; }
static inline rpoly rp_mul(rpoly a, rpoly b)
{ rpoly p; memset(&p,0,sizeof p);
  for (int i = 0; i < PD; i++) if (a.c[i] != 0.0) for (int j = 0; i+j < PD; j++) p.c[i+j] += a.c[i]*b.c[j];
  return p; }
static inline rpoly rp_add(rpoly a, rpoly b) { for (int i = 0; i < PD; i++) a.c[i] += b.c[i]; return a; }
static inline rpoly rp_scale(rpoly a, double s) { for (int i = 0; i < PD; i++) a.c[i] *= s; return a; }
static inline rpoly rp_shift(rpoly a) /* multiply by w */ { rpoly p; memset(&p,0,sizeof p); for (int i = 0; i+1 < PD; i++) p.c[i+1] = a.c[i]; return p; }

/* E_n(z) = int_0^1 w^n e^{z w} dw for n = 0..nmax */
static void expint_moments(cplx z, int nmax, cplx *E)
{
  double az = cabs(z);
  if (az < 2.0) {
    for (int n = 0; n <= nmax; n++) {
      cplx term = 1.0, sum = 1.0 / (n + 1.0);
      for (int m = 1; m < 200; m++) {
        term *= z / (double)m;
        cplx t = term / (double)(n + m + 1);
        sum += t;
        if (cabs(t) < 1e-18 * cabs(sum)) break;
      }
      E[n] = sum;
    }
  } else {
    cplx ez = cexp(z);
    E[0] = (ez - 1.0) / z;
    for (int n = 1; n <= nmax; n++) E[n] = (ez - n * E[n-1]) / z;
  }
}

/* ------------------------------------------------------------------ */
/* Duffy-cell generator for touching panel pairs.                      */
/* Panels are in AssessPanelPair order (common vertices first) and     */
/* parametrised as x = V0 + s1 (V1-V0) + s2 (V2-V1), 0<=s2<=s1<=1,     */
/* the parametrisation of the reference's FIPPI integrals              */
/* (QIFIPPICubature.cc:187-240).  Each emitted point carries:          */
/*  - s(w) = s0 + w s1 for both panels (affine in the radial w),       */
/*  - a weight polynomial omega(w) (all Jacobians) times W,            */
/*  - D with x(w) - x'(w) = w D, X = |D|.                              */
/* Cells:                                                              */
/*  ncv=3: z = s - s' on 6 hexagon sectors, s' over the homothetic     */
/*         triangle T ∩ (T - z) (3-point degree-2 rule), 1-D rule in t.*/
/*  ncv=2: (u-u', v, v') radial over 4 polyhedral pieces, 2-D rule,    */
/*         u' over its interval with an exact 2-point rule.            */
/*  ncv=1: classical Duffy split at the common vertex, 3-D rule.       */
/* ------------------------------------------------------------------ */
typedef struct {
  double W;
  rpoly omega;
  double sa0[2], sa1[2], sb0[2], sb1[2];
  double D[3], X;
} dpoint;

typedef void (*dpoint_cb)(void *ctx, const dpoint *pt);

static void emit(const double *Va[3], const double *Vb[3], dpoint *pt, dpoint_cb cb, void *ctx)
{
  double A[3], B[3], AP[3], BP[3];
  vsub(Va[1], Va[0], A); vsub(Va[2], Va[1], B);
  vsub(Vb[1], Vb[0], AP); vsub(Vb[2], Vb[1], BP);
  /* x - x' at w: (Va0 - Vb0) + (sa0 + w sa1).(A,B) - (sb0 + w sb1).(AP,BP); constant part must vanish */
  for (int m = 0; m < 3; m++)
    pt->D[m] = pt->sa1[0]*A[m] + pt->sa1[1]*B[m] - pt->sb1[0]*AP[m] - pt->sb1[1]*BP[m];
  pt->X = vnorm(pt->D);
  cb(ctx, pt);
}

static void duffy_cells(int ncv, const double *Va[3], const double *Vb[3], int n, dpoint_cb cb, void *ctx)
{
  double gx[64], gw[64];
  gauss_legendre01(n, gx, gw);
  dpoint pt;
  if (ncv == 3) {
    static const double H[7][2] = {{1,0},{1,1},{0,1},{-1,0},{-1,-1},{0,-1},{1,0}};
    static const double TP[3][2] = {{0.5,0.0},{1.0,0.5},{0.5,0.5}}; /* degree-2 rule on 0<=p2<=p1<=1 */
    for (int k = 0; k < 6; k++)
      for (int it = 0; it < n; it++) {
        double t = gx[it];
        double zh[2] = { H[k][0] + t*(H[k+1][0]-H[k][0]), H[k][1] + t*(H[k+1][1]-H[k][1]) };
        /* a = w*max(0,-z2), b = 1 - w*max(0,z1), c = w*min(0,z1-z2), lambda = b - a + c */
        double am = fmax(0.0, -zh[1]), bm = fmax(0.0, zh[0]), cm = fmin(0.0, zh[0]-zh[1]);
        double sig = bm + am - cm;
        for (int ip = 0; ip < 3; ip++) {
          double p1 = TP[ip][0], p2 = TP[ip][1];
          /* s' = (a - c, a) + lambda (p1, p2); lambda = 1 - w sig */
          pt.sb0[0] = p1;          pt.sb1[0] = (am - cm) - sig*p1;
          pt.sb0[1] = p2;          pt.sb1[1] = am - sig*p2;
          pt.sa0[0] = pt.sb0[0];   pt.sa1[0] = pt.sb1[0] + zh[0];
          pt.sa0[1] = pt.sb0[1];   pt.sa1[1] = pt.sb1[1] + zh[1];
          rpoly lam = rp_aff(1.0, -sig);
          pt.omega = rp_shift(rp_mul(lam, lam));    /* w lambda^2 */
          pt.W = gw[it] * (1.0/6.0);
          emit(Va, Vb, &pt, cb, ctx);
        }
      }
  } else if (ncv == 2) {
    const double tx[2] = {0.5 - 0.5/sqrt(3.0), 0.5 + 0.5/sqrt(3.0)};
    for (int reg = 0; reg < 4; reg++)
      for (int ia = 0; ia < n; ia++)
        for (int ib = 0; ib < n; ib++) {
          double al = gx[ia], be = gx[ib], z[3], J, lo;
          switch (reg) {
            case 0: z[0] = 1.0 - al; z[1] = be; z[2] = al; J = 1.0; lo = al; break;
            case 1: z[0] = al; z[1] = 1.0; z[2] = (1.0-al)*be; J = 1.0 - al; lo = 1.0 - al; break;
            case 2: z[0] = -al; z[1] = (1.0-al)*be; z[2] = 1.0; J = 1.0 - al; lo = 1.0; break;
            default: z[0] = -al; z[1] = 1.0 - al; z[2] = be; J = 1.0; lo = 1.0; break;
          }
          for (int itau = 0; itau < 2; itau++) {
            double tau = tx[itau];
            /* u' = w lo + (1 - w) tau ; u = u' + w z0 ; v = w z1 ; v' = w z2 */
            pt.sb0[0] = tau; pt.sb1[0] = lo - tau;
            pt.sb0[1] = 0.0; pt.sb1[1] = z[2];
            pt.sa0[0] = tau; pt.sa1[0] = lo - tau + z[0];
            pt.sa0[1] = 0.0; pt.sa1[1] = z[1];
            rpoly om = rp_aff(0.0, 0.0); om.c[2] = 1.0; om.c[3] = -1.0;  /* w^2 (1-w) */
            pt.omega = om;
            pt.W = gw[ia] * gw[ib] * 0.5 * J;
            emit(Va, Vb, &pt, cb, ctx);
          }
        }
  } else if (ncv == 1) {
    for (int reg = 0; reg < 2; reg++)
      for (int i1 = 0; i1 < n; i1++)
        for (int i2 = 0; i2 < n; i2++)
          for (int i3 = 0; i3 < n; i3++) {
            double al = gx[i1], be = gx[i2], ga = gx[i3];
            double *s0 = reg == 0 ? pt.sa1 : pt.sb1, *s1 = reg == 0 ? pt.sb1 : pt.sa1;
            pt.sa0[0] = pt.sa0[1] = pt.sb0[0] = pt.sb0[1] = 0.0;
            s0[0] = 1.0; s0[1] = al; s1[0] = be; s1[1] = be*ga;
            rpoly om; memset(&om, 0, sizeof om); om.c[3] = be;   /* w^3 beta */
            pt.omega = om;
            pt.W = gw[i1] * gw[i2] * gw[i3];
            emit(Va, Vb, &pt, cb, ctx);
          }
  }
}

/* physical point x(w) = V0 + s1 A + s2 B as three affine polynomials */
static void xpoly(const double *V[3], const double s0[2], const double s1[2], rpoly x[3])
{
  double A[3], B[3];
  vsub(V[1], V[0], A); vsub(V[2], V[1], B);
  for (int m = 0; m < 3; m++)
    x[m] = rp_aff(V[0][m] + s0[0]*A[m] + s0[1]*B[m], s1[0]*A[m] + s1[1]*B[m]);
}

/* ------------------------------------------------------------------ */
/* Helmholtz integrals over touching pairs (the quantities TaylorDuffy */
/* returns for PIndex {UNITY, PMCHWG1, PMCHWC} and KIndex {HELMHOLTZ,   */
/* HELMHOLTZ, GRADHELMHOLTZ}, PanelPanelInteractions.cc:449-491):      */
/* H0 = int int ((x-Q).(x'-Q') - 4/k^2) G, H1 = int int                */
/* ((x-Q)x(x'-Q')).(x-x') Psi.                                         */
/* ------------------------------------------------------------------ */
typedef struct { const double **Va, **Vb; const double *Qa, *Qb; cplx k; int want_h1; cplx H0, H1; } td_ctx;

static void td_cb(void *vctx, const dpoint *pt)
{
  td_ctx *c = (td_ctx *)vctx;
  rpoly x[3], xp[3];
  xpoly(c->Va, pt->sa0, pt->sa1, x);
  xpoly(c->Vb, pt->sb0, pt->sb1, xp);
  rpoly F[3], FP[3];
  for (int m = 0; m < 3; m++) { F[m] = rp_add(x[m], rp_aff(-c->Qa[m], 0)); FP[m] = rp_add(xp[m], rp_aff(-c->Qb[m], 0)); }
  rpoly dot = rp_add(rp_add(rp_mul(F[0],FP[0]), rp_mul(F[1],FP[1])), rp_mul(F[2],FP[2]));
  rpoly q = rp_mul(pt->omega, dot);
  rpoly q1 = pt->omega;
  cplx z = I * c->k * pt->X, E[PD+2];
  expint_moments(z, PD, E);
  double X = pt->X;
  cplx s = 0.0, s1 = 0.0;
  for (int nn = 1; nn < PD; nn++) { s += q.c[nn] * E[nn-1]; s1 += q1.c[nn] * E[nn-1]; }
  c->H0 += pt->W * (s - 4.0/(c->k*c->k) * s1) / (4.0*PI*X);
  if (c->want_h1) {
    /* hTimes = w ((F x F').D) */
    rpoly cr[3];
    cr[0] = rp_add(rp_mul(F[1],FP[2]), rp_scale(rp_mul(F[2],FP[1]), -1));
    cr[1] = rp_add(rp_mul(F[2],FP[0]), rp_scale(rp_mul(F[0],FP[2]), -1));
    cr[2] = rp_add(rp_mul(F[0],FP[1]), rp_scale(rp_mul(F[1],FP[0]), -1));
    rpoly ht = rp_add(rp_add(rp_scale(cr[0], pt->D[0]), rp_scale(cr[1], pt->D[1])), rp_scale(cr[2], pt->D[2]));
    rpoly qq = rp_mul(pt->omega, rp_shift(ht));   /* omega * w * hT */
    /* Psi(wX) = (ik - 1/(wX)) e^{ikwX}/(4 pi w^2 X^2) */
    cplx ik = I * c->k, acc = 0.0;
    for (int nn = 0; nn < PD; nn++) {
      if (qq.c[nn] == 0.0) continue;
      cplx t = 0.0;
      if (nn >= 2) t += ik/(4.0*PI*X*X) * E[nn-2];
      if (nn >= 3) t -= 1.0/(4.0*PI*X*X*X) * E[nn-3];
      acc += qq.c[nn] * t;
    }
    c->H1 += pt->W * acc;
  }
}

/* ------------------------------------------------------------------ */
/* Q-independent FIPPI data (libscuffInternals.h:282-292):             */
/*  xMxpRM3 = int int (x-x')/r^3, xXxpRM3 = int int (x x x')/r^3,      */
/*  uvupvp{RM1,R1,R2}[9] = int int {1,u',v',u,uu',uv',v,vu',vv'} r^p,  */
/* in the FIPPI parametrisation (V0 + u A + v B, A=V1-V0, B=V2-V1).    */
/* ------------------------------------------------------------------ */
typedef struct {
  double xMxpRM3[3], xXxpRM3[3];
  double RM1[9], R1[9], R2[9];
  double x0[3];
} ora_qifippi;

typedef struct { const double **Va, **Vb; ora_qifippi *Q; } fip_ctx;

static void fip_cb(void *vctx, const dpoint *pt)
{
  fip_ctx *c = (fip_ctx *)vctx;
  double X = pt->X, W = pt->W;
  /* monomials {1,u',v',u,uu',uv',v,vu',vv'} as polynomials in w */
  rpoly ua = rp_aff(pt->sa0[0], pt->sa1[0]), va = rp_aff(pt->sa0[1], pt->sa1[1]);
  rpoly ub = rp_aff(pt->sb0[0], pt->sb1[0]), vb = rp_aff(pt->sb0[1], pt->sb1[1]);
  rpoly one = rp_aff(1.0, 0.0);
  rpoly ma[3] = {one, ua, va}, mb[3] = {one, ub, vb};
  for (int ia = 0; ia < 3; ia++)
    for (int ib = 0; ib < 3; ib++) {
      int m = 3*ia + ib;
      rpoly q = rp_mul(pt->omega, rp_mul(ma[ia], mb[ib]));
      double sm1 = 0, s1 = 0, s2 = 0;
      for (int nn = 0; nn < PD; nn++) {
        if (q.c[nn] == 0.0) continue;
        sm1 += q.c[nn] / (nn + 0.0);      /* w^{nn} (wX)^{-1}: int w^{nn-1} = 1/nn */
        s1  += q.c[nn] / (nn + 2.0);
        s2  += q.c[nn] / (nn + 3.0);
      }
      c->Q->RM1[m] += W * sm1 / X;
      c->Q->R1[m]  += W * s1 * X;
      c->Q->R2[m]  += W * s2 * X * X;
    }
  /* (x-x')/r^3 = w D/(w^3 X^3); (x x x')/r^3 = -(x(w) x wD)/(w^3 X^3) */
  double om_m2 = 0;
  for (int nn = 2; nn < PD; nn++) om_m2 += pt->omega.c[nn] / (nn - 1.0);
  for (int m = 0; m < 3; m++) c->Q->xMxpRM3[m] += W * om_m2 * pt->D[m] / (X*X*X);
  rpoly x[3];
  xpoly(c->Va, pt->sa0, pt->sa1, x);
  rpoly cx[3];
  cx[0] = rp_add(rp_scale(x[1], pt->D[2]), rp_scale(x[2], -pt->D[1]));
  cx[1] = rp_add(rp_scale(x[2], pt->D[0]), rp_scale(x[0], -pt->D[2]));
  cx[2] = rp_add(rp_scale(x[0], pt->D[1]), rp_scale(x[1], -pt->D[0]));
  for (int m = 0; m < 3; m++) {
    rpoly q = rp_mul(pt->omega, cx[m]);
    double s = 0;
    for (int nn = 2; nn < PD; nn++) s += q.c[nn] / (nn - 1.0);
    c->Q->xXxpRM3[m] += -W * s / (X*X*X);
  }
}

/* ncv = 0: the 3-D scheme of QIFIPPICubature.cc:187-325 -- the v'      */
/* integral along the source segment is done in closed form, (u, v/u,  */
/* u') by a tensor Gauss-Legendre rule.                                */
static void seg_integrals(double a2, double v0, double b2, double up, double J[4][2])
{
  /* r^2 = a2 ((v'-v0)^2 + b2), v' in [0, up]; J[p][j] = int v'^j r^p dv' for p=-3,-1,1,2 */
  double a = sqrt(a2);
  double t1 = -v0, t2 = up - v0;
  double S1 = sqrt(t1*t1 + b2), S2 = sqrt(t2*t2 + b2);
  /* ln(t + S) differences, evaluated without cancellation */
  double L;
  if (t1 >= 0) L = log((t2 + S2) / (t1 + S1));
  else if (t2 <= 0) L = log((S1 - t1) / (S2 - t2));
  else L = log((t2 + S2) * (S1 - t1) / b2);
  double Im3_0, Im3_1;
  if (t1 * t2 > 0) Im3_0 = (t2*t2 - t1*t1) / (S1*S2*(t2*S1 + t1*S2));
  else Im3_0 = (t2/S2 - t1/S1) / b2;
  Im3_1 = 1.0/S1 - 1.0/S2;
  double Im1_0 = L, Im1_1 = S2 - S1;
  double I1_0 = 0.5*(t2*S2 - t1*S1 + b2*L), I1_1 = (S2*S2*S2 - S1*S1*S1)/3.0;
  double I2_0 = (t2*t2*t2 - t1*t1*t1)/3.0 + b2*(t2 - t1);
  double I2_1 = ((t2*t2+b2)*(t2*t2+b2) - (t1*t1+b2)*(t1*t1+b2))/4.0;
  /* v' = t + v0 */
  J[0][0] = Im3_0 / (a2*a); J[0][1] = (Im3_1 + v0*Im3_0) / (a2*a);
  J[1][0] = Im1_0 / a;      J[1][1] = (Im1_1 + v0*Im1_0) / a;
  J[2][0] = I1_0 * a;       J[2][1] = (I1_1 + v0*I1_0) * a;
  J[3][0] = I2_0 * a2;      J[3][1] = (I2_1 + v0*I2_0) * a2;
}

static void qifippi_nc(const double *Va[3], const double *Vb[3], int n, ora_qifippi *Q)
{
  double gx[64], gw[64];
  gauss_legendre01(n, gx, gw);
  double A[3], B[3], AP[3], BP[3];
  vsub(Va[1], Va[0], A); vsub(Va[2], Va[1], B);
  vsub(Vb[1], Vb[0], AP); vsub(Vb[2], Vb[1], BP);
  double a2 = vdot(BP, BP);
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++)
      for (int l = 0; l < n; l++) {
        double u = gx[i], v = u*gx[j], up = gx[l];
        double W = gw[i]*gw[j]*gw[l]*u;
        double X[3], Z[3], Y[3];
        for (int m = 0; m < 3; m++) { X[m] = Va[0][m] + u*A[m] + v*B[m]; Z[m] = Vb[0][m] + up*AP[m]; Y[m] = X[m] - Z[m]; }
        /* |x - x'|^2 = |Y - v' BP|^2 = a2 ((v' - v0)^2 + b2) */
        double v0 = vdot(BP, Y) / a2;
        double b2 = vdot(Y, Y)/a2 - v0*v0;
        if (b2 < 0) b2 = 0;
        double J[4][2];
        seg_integrals(a2, v0, b2, up, J);
        for (int m = 0; m < 3; m++) Q->xMxpRM3[m] += W * (Y[m]*J[0][0] - BP[m]*J[0][1]);
        double XZ[3], XB[3];
        vcross(X, Z, XZ); vcross(X, BP, XB);
        for (int m = 0; m < 3; m++) Q->xXxpRM3[m] += W * (XZ[m]*J[0][0] + XB[m]*J[0][1]);
        double ma[3] = {1.0, u, v};
        for (int ia = 0; ia < 3; ia++) {
          /* b-side monomials {1, u', v'}: v' handled by J[.][1] */
          double f = W * ma[ia];
          Q->RM1[3*ia+0] += f * J[1][0]; Q->RM1[3*ia+1] += f * up * J[1][0]; Q->RM1[3*ia+2] += f * J[1][1];
          Q->R1 [3*ia+0] += f * J[2][0]; Q->R1 [3*ia+1] += f * up * J[2][0]; Q->R1 [3*ia+2] += f * J[2][1];
          Q->R2 [3*ia+0] += f * J[3][0]; Q->R2 [3*ia+1] += f * up * J[3][0]; Q->R2 [3*ia+2] += f * J[3][1];
        }
      }
}

/* ComputeQIFIPPIData (QIFIPPICubature.cc:465-487) */
void ora_qifippi_compute(const double *Va[3], const double *Vb[3], int ncv, int n, ora_qifippi *Q)
{
  memset(Q, 0, sizeof *Q);
  if (ncv == 0) qifippi_nc(Va, Vb, n, Q);
  else { fip_ctx c = {Va, Vb, Q}; duffy_cells(ncv, Va, Vb, n, fip_cb, &c); }
  for (int m = 0; m < 3; m++) Q->x0[m] = (Va[0][m] + Va[1][m] + Va[2][m]) / 3.0;
}

/* ------------------------------------------------------------------ */
/* Q-dependent FIPPI data (QDFIPPI.cc:67-260), uncached variant         */
/* (no canonical reordering, so no flip and no x0 correction).          */
/* ------------------------------------------------------------------ */
typedef struct { double hTimesRM3, hDotRM1, hNablaRM1, hTimesRM1, hDotR0, hNablaR0, hTimesR0,
                 hDotR1, hNablaR1, hTimesR1, hDotR2, hNablaR2; } ora_qdfippi;

static void qdfippi(const double *Va[3], const double *Qa, const double *Vb[3], const double *Qb,
                    const ora_qifippi *Q, ora_qdfippi *D)
{
  static const double R0[9] = {1.0/4, 1.0/6, 1.0/12, 1.0/6, 1.0/9, 1.0/18, 1.0/12, 1.0/18, 1.0/36};
  double A[3], B[3], V0mQ[3], AP[3], BP[3], V0PmQP[3];
  vsub(Va[1], Va[0], A); vsub(Va[2], Va[1], B); vsub(Va[0], Qa, V0mQ);
  vsub(Vb[1], Vb[0], AP); vsub(Vb[2], Vb[1], BP); vsub(Vb[0], Qb, V0PmQP);
  double dots[9] = { vdot(V0mQ,V0PmQP), vdot(V0mQ,AP), vdot(V0mQ,BP),
                     vdot(A,V0PmQP), vdot(A,AP), vdot(A,BP),
                     vdot(B,V0PmQP), vdot(B,AP), vdot(B,BP) };
  double QamQb[3], QaxQb[3], V0mV0P[3], S[3];
  vsub(Va[0], Vb[0], V0mV0P); vsub(Qa, Qb, QamQb); vcross(Qa, Qb, QaxQb);
  double ht[9];
  vcross(Va[0], Vb[0], S); ht[0] = vdot(QaxQb, V0mV0P) + vdot(QamQb, S);
  vcross(A, Vb[0], S);     ht[3] = vdot(QaxQb, A) + vdot(QamQb, S);
  vcross(B, Vb[0], S);     ht[6] = vdot(QaxQb, B) + vdot(QamQb, S);
  vcross(Va[0], AP, S);    ht[1] = -vdot(QaxQb, AP) + vdot(QamQb, S);
  vcross(Va[0], BP, S);    ht[2] = -vdot(QaxQb, BP) + vdot(QamQb, S);
  vcross(A, AP, S);        ht[4] = vdot(QamQb, S);
  vcross(A, BP, S);        ht[5] = vdot(QamQb, S);
  vcross(B, AP, S);        ht[7] = vdot(QamQb, S);
  vcross(B, BP, S);        ht[8] = vdot(QamQb, S);
  D->hTimesRM3 = vdot(QaxQb, Q->xMxpRM3) + vdot(QamQb, Q->xXxpRM3);
  D->hDotRM1 = D->hTimesRM1 = D->hDotR0 = D->hTimesR0 = D->hDotR1 = D->hTimesR1 = D->hDotR2 = 0;
  for (int m = 0; m < 9; m++) {
    D->hDotRM1 += Q->RM1[m]*dots[m]; D->hTimesRM1 += Q->RM1[m]*ht[m];
    D->hDotR0  += R0[m]*dots[m];     D->hTimesR0  += R0[m]*ht[m];
    D->hDotR1  += Q->R1[m]*dots[m];  D->hTimesR1  += Q->R1[m]*ht[m];
    D->hDotR2  += Q->R2[m]*dots[m];
  }
  D->hNablaRM1 = 4.0*Q->RM1[0]; D->hNablaR0 = 1.0; D->hNablaR1 = 4.0*Q->R1[0]; D->hNablaR2 = 4.0*Q->R2[0];
}

/* ------------------------------------------------------------------ */
/* Panel-panel interactions dispatcher (PanelPanelInteractions.cc:357-561) */
/* ------------------------------------------------------------------ */
enum { ALG_LO = 0, ALG_HO = 1, ALG_TD = 2, ALG_HKTD = 3, ALG_DESING = 4 };

/* quadrature orders used by the oracle (high: the oracle is the checker) */
static int ORA_N_TD3 = 32, ORA_N_TD2 = 20, ORA_N_TD1 = 14, ORA_N_FIP0 = 16, ORA_N_FIP12 = 16;

void ora_set_orders(int td3, int td2, int td1, int fip0, int fip12)
{ ORA_N_TD3 = td3; ORA_N_TD2 = td2; ORA_N_TD1 = td1; ORA_N_FIP0 = fip0; ORA_N_FIP12 = fip12; }

int ora_ppi(const ora_surface *Sa, int pa, int iQa, const ora_surface *Sb, int pb, int iQb,
            cplx k, cplx H[2], int *ncv_out)
{
  const double *Va[3], *Vb[3];
  double rrel;
  int ncv = assess_pair(Sa, pa, Sb, pb, &rrel, Va, Vb);
  if (ncv_out) *ncv_out = ncv;
  const double *Qa = Sa->V + 3*Sa->PV[3*pa + iQa], *Qb = Sb->V + 3*Sb->PV[3*pb + iQb];
  if (rrel > 4.0) { ppi_cubature(k, 0, 0, Va, Qa, Vb, Qb, H); return ALG_LO; }
  double kR = cabs(k * fmax(Sa->radius[pa], Sb->radius[pb]));
  int sw = kR > PI;
  if (sw && ncv == 0) { ppi_cubature(k, 0, 1, Va, Qa, Vb, Qb, H); return ALG_HO; }
  if (ncv == 3 || (ncv > 0 && sw)) {
    int n = ncv == 3 ? ORA_N_TD3 : (ncv == 2 ? ORA_N_TD2 : ORA_N_TD1);
    td_ctx c = {Va, Vb, Qa, Qb, k, ncv < 3, 0.0, 0.0};
    duffy_cells(ncv, Va, Vb, n, td_cb, &c);
    H[0] = c.H0;
    H[1] = (ncv == 3) ? 0.0 : c.H1;
    return ALG_TD;
  }
  /* desingularisation */
  ppi_cubature(k, 1, 0, Va, Qa, Vb, Qb, H);
  ora_qifippi Q;
  int cached = 0;
  long long key = (long long)pa * Sa->np + pb;
  ora_qifippi *tab = (ora_qifippi *)Sa->fval;
  int slot = -1;
  if (Sa == Sb && Sa->fcap) {
    slot = (int)(((unsigned long long)key * 0x9E3779B97F4A7C15ULL) >> 33) & (Sa->fcap - 1);
    #pragma omp critical(ora_fippi_cache)
    {
      while (Sa->fkey[slot] != -1 && Sa->fkey[slot] != key) slot = (slot + 1) & (Sa->fcap - 1);
      if (Sa->fkey[slot] == key) { Q = tab[slot]; cached = 1; }
    }
  }
  if (!cached) {
    ora_qifippi_compute(Va, Vb, ncv, ncv == 0 ? ORA_N_FIP0 : ORA_N_FIP12, &Q);
    if (slot >= 0) {
      #pragma omp critical(ora_fippi_cache)
      {
        while (Sa->fkey[slot] != -1 && Sa->fkey[slot] != key) slot = (slot + 1) & (Sa->fcap - 1);
        if (Sa->fkey[slot] == -1) { Sa->fkey[slot] = key; tab[slot] = Q; }
      }
    }
  }
  ora_qdfippi D;
  qdfippi(Va, Qa, Vb, Qb, &Q, &D);
  cplx ik = I*k, ooik2 = 1.0/(ik*ik), PF[5];
  PF[0] = 1.0/(4.0*PI);
  for (int i = 1; i < 5; i++) PF[i] = ik*PF[i-1];
  H[0] += PF[0]*(D.hDotRM1 + ooik2*D.hNablaRM1) + PF[1]*(D.hDotR0 + ooik2*D.hNablaR0)
        + PF[2]*0.5*(D.hDotR1 + ooik2*D.hNablaR1) + PF[3]*(1.0/6.0)*(D.hDotR2 + ooik2*D.hNablaR2);
  H[1] += PF[0]*(-1.0)*D.hTimesRM3 + PF[2]*0.5*D.hTimesRM1 + PF[3]*(1.0/3.0)*D.hTimesR0
        + PF[4]*(1.0/6.0)*D.hTimesR1;
  return ALG_DESING;
}

/* ------------------------------------------------------------------ */
/* public surface handle for ctypes                                    */
/* ------------------------------------------------------------------ */
ora_surface *ora_surface_new(int nv, const double *V, int np, const int *PV)
{
  ora_surface *S = calloc(1, sizeof *S);
  S->nv = nv; S->np = np;
  double *Vc = malloc(sizeof(double)*3*nv); memcpy(Vc, V, sizeof(double)*3*nv); S->V = Vc;
  int *Pc = malloc(sizeof(int)*3*np); memcpy(Pc, PV, sizeof(int)*3*np); S->PV = Pc;
  S->centroid = malloc(sizeof(double)*3*np);
  S->radius = malloc(sizeof(double)*np);
  S->area = malloc(sizeof(double)*np);
  init_panels(S);
  S->E = malloc(sizeof(int)*8*3*np);
  S->ne = ora_build_edges(nv, np, PV, S->E, 3*np);
  if (S->ne < 0) S->ne = 0;
  S->elen = malloc(sizeof(double)*(S->ne > 0 ? S->ne : 1));
  for (int e = 0; e < S->ne; e++) S->elen[e] = vdist(S->V + 3*S->E[8*e], S->V + 3*S->E[8*e+1]);
  S->fcap = 1; while (S->fcap < 256*np) S->fcap <<= 1;
  S->fkey = malloc(sizeof(long long)*S->fcap);
  for (int i = 0; i < S->fcap; i++) S->fkey[i] = -1;
  S->fval = malloc(sizeof(ora_qifippi)*S->fcap);
  return S;
}

void ora_surface_free(ora_surface *S)
{
  if (!S) return;
  free((void*)S->V); free((void*)S->PV); free(S->centroid); free(S->radius); free(S->area);
  free(S->E); free(S->elen); free(S->fkey); free(S->fval); free(S);
}

int ora_surface_num_edges(const ora_surface *S) { return S->ne; }
void ora_surface_edges(const ora_surface *S, int *E, double *len)
{ memcpy(E, S->E, sizeof(int)*8*S->ne); memcpy(len, S->elen, sizeof(double)*S->ne); }

int ora_ppi_c(const ora_surface *S, int pa, int iQa, int pb, int iQb, double kr, double ki, double *H4, int *ncv)
{
  cplx H[2];
  int alg = ora_ppi(S, pa, iQa, S, pb, iQb, kr + I*ki, H, ncv);
  H4[0] = creal(H[0]); H4[1] = cimag(H[0]); H4[2] = creal(H[1]); H4[3] = cimag(H[1]);
  return alg;
}

/* FIPPI data for a panel pair in the reference's conventions (for parity  */
/* against the reference's own ComputeQIFIPPIData); out = 33 doubles.      */
int ora_qifippi_c(const ora_surface *S, int pa, int pb, int n, double *out, int *order6)
{
  const double *Va[3], *Vb[3];
  double rrel;
  int ncv = assess_pair(S, pa, S, pb, &rrel, Va, Vb);
  ora_qifippi Q;
  ora_qifippi_compute(Va, Vb, ncv, n, &Q);
  memcpy(out, Q.xMxpRM3, 3*sizeof(double)); memcpy(out+3, Q.xXxpRM3, 3*sizeof(double));
  memcpy(out+6, Q.RM1, 9*sizeof(double)); memcpy(out+15, Q.R1, 9*sizeof(double)); memcpy(out+24, Q.R2, 9*sizeof(double));
  if (order6) for (int i = 0; i < 3; i++) { order6[i] = (int)((Va[i]-S->V)/3); order6[3+i] = (int)((Vb[i]-S->V)/3); }
  return ncv;
}

/* ------------------------------------------------------------------ */
/* Edge-edge interactions (EdgeEdgeInteractions.cc:50-217):            */
/* GC[0] = La Lb (HPP - HPM - HMP + HMM)[0]; GC[1] = La Lb/(ik) (...)[1] */
/* ------------------------------------------------------------------ */
static void ora_eei(const ora_surface *Sa, int ea, const ora_surface *Sb, int eb, cplx k, cplx GC[2])
{
  if (creal(k) == 0.0 && cimag(k) == 0.0) { GC[0] = GC[1] = 0.0; return; }
  const int *A = Sa->E + 8*ea, *B = Sb->E + 8*eb;
  cplx HPP[2] = {0,0}, HPM[2] = {0,0}, HMP[2] = {0,0}, HMM[2] = {0,0};
  ora_ppi(Sa, A[4], A[6], Sb, B[4], B[6], k, HPP, 0);
  if (B[5] != -1) ora_ppi(Sa, A[4], A[6], Sb, B[5], B[7], k, HPM, 0);
  if (A[5] != -1) ora_ppi(Sa, A[5], A[7], Sb, B[4], B[6], k, HMP, 0);
  if (A[5] != -1 && B[5] != -1) ora_ppi(Sa, A[5], A[7], Sb, B[5], B[7], k, HMM, 0);
  double G = Sa->elen[ea] * Sb->elen[eb];
  cplx C = G / (I*k);
  GC[0] = G * (HPP[0] - HPM[0] - HMP[0] + HMM[0]);
  GC[1] = C * (HPP[1] - HPM[1] - HMP[1] + HMM[1]);
}

/* GC[0], GC[1] (EdgeEdgeInteractions.cc:183-188) of every edge pair of one
   surface at wavenumber k: the ingredients of the EMT power integrals
   (EMTPFT.cc:333-352 with GetGCMatrixElements). */
void ora_gc_matrix(const ora_surface *S, double kr, double ki, double *GC0, double *GC1)
{
  const int ne = S->ne;
  const cplx k = kr + I*ki;
#pragma omp parallel for schedule(dynamic, 4)
  for (int ea = 0; ea < ne; ea++)
    for (int eb = 0; eb < ne; eb++) {
      cplx GC[2];
      ora_eei(S, ea, S, eb, k, GC);
      GC0[2*(ea + (size_t)eb*ne)] = creal(GC[0]); GC0[2*(ea + (size_t)eb*ne) + 1] = cimag(GC[0]);
      GC1[2*(ea + (size_t)eb*ne)] = creal(GC[1]); GC1[2*(ea + (size_t)eb*ne) + 1] = cimag(GC[1]);
    }
}

static cplx csqrt2(cplx z) { cplx r = csqrt(z); return cimag(r) < 0 ? -r : r; }

/* ------------------------------------------------------------------ */
/* Full BEM matrix of a compact geometry (AssembleBEMMatrix.cc:684-765, */
/* SurfaceSurfaceInteractions.cc:62-90, 106-334, 426-585).              */
/* surfaces: ns handles; reg[2*s] = exterior region, reg[2*s+1] =       */
/* interior region (-1 for PEC); pec[s]; eps/mu: complex per region.    */
/* M: N x N column-major complex128, N = sum of NumBFs.                */
/* ------------------------------------------------------------------ */
void ora_assemble(int ns, ora_surface **S, const int *reg, const int *pec,
                  double wr, double wi, const double *eps, const double *mu, double *Mout, int N)
{
  cplx omega = wr + I*wi;
  cplx *M = (cplx *)Mout;
  memset(M, 0, sizeof(cplx)*(size_t)N*N);
  int off[64], o = 0;
  for (int s = 0; s < ns; s++) { off[s] = o; o += pec[s] ? S[s]->ne : 2*S[s]->ne; }
  for (int sa = 0; sa < ns; sa++)
    for (int sb = sa; sb < ns; sb++) {
      /* CountCommonRegions */
      int cr[2], nc = 0; double sg[2];
      const int *Ra = reg + 2*sa, *Rb = reg + 2*sb;
      if (Ra[0] == Rb[0]) { cr[nc] = Ra[0]; sg[nc] = 1.0; nc++; }
      else if (Ra[0] == Rb[1]) { cr[nc] = Ra[0]; sg[nc] = -1.0; nc++; }
      if (Ra[1] == Rb[0] && Ra[1] >= 0) { cr[nc] = Ra[1]; sg[nc] = -1.0; nc++; }
      else if (!pec[sa] && !pec[sb] && Ra[1] == Rb[1]) { cr[nc] = Ra[1]; sg[nc] = 1.0; nc++; }
      if (nc == 0) continue;
      int sym = (sa == sb);
      cplx PF1[2], PF2[2], PF3[2], kk[2];
      for (int r = 0; r < nc; r++) {
        cplx e = eps[2*cr[r]] + I*eps[2*cr[r]+1], m = mu[2*cr[r]] + I*mu[2*cr[r]+1];
        kk[r] = csqrt2(e*m) * omega;
        PF1[r] = sg[r]*I*m*omega; PF2[r] = -sg[r]*I*kk[r]; PF3[r] = -sg[r]*I*e*omega;
      }
      int NEa = S[sa]->ne, NEb = S[sb]->ne;
      #pragma omp parallel for schedule(dynamic, 4)
      for (int ea = 0; ea < NEa; ea++)
        for (int eb = sym ? ea : 0; eb < NEb; eb++) {
          for (int r = 0; r < nc; r++) {
            cplx GC[2];
            ora_eei(S[sa], ea, S[sb], eb, kk[r], GC);
            if (pec[sa] && pec[sb]) {
              size_t X = off[sa] + ea, Y = off[sb] + eb;
              M[X + Y*N] += PF1[r]*GC[0];
            } else if (pec[sa] && !pec[sb]) {
              size_t X = off[sa] + ea, Y = off[sb] + 2*eb;
              M[X + Y*N] += PF1[r]*GC[0]; M[X + (Y+1)*N] += PF2[r]*GC[1];
            } else if (!pec[sa] && pec[sb]) {
              size_t X = off[sa] + 2*ea, Y = off[sb] + eb;
              M[X + Y*N] += PF1[r]*GC[0]; M[X+1 + Y*N] += PF2[r]*GC[1];
            } else {
              size_t X = off[sa] + 2*ea, Y = off[sb] + 2*eb;
              M[X + Y*N] += PF1[r]*GC[0];
              M[X + (Y+1)*N] += PF2[r]*GC[1];
              if (!sym || ea != eb) M[X+1 + Y*N] += PF2[r]*GC[1];
              M[X+1 + (Y+1)*N] += PF3[r]*GC[0];
            }
          }
        }
      /* lower-triangle mirror of diagonal blocks; off-diagonal blocks */
      /* are mirrored by the symmetric fill (AssembleBEMMatrix.cc:753-758) */
    }
  for (int c = 0; c < N; c++)
    for (int r = c + 1; r < N; r++) {
      /* only entries not produced by the block loop (the block loop fills
         rows <= cols inside diagonal blocks and whole upper blocks) */
      M[r + (size_t)c*N] = M[c + (size_t)r*N];
    }
}

/* ------------------------------------------------------------------ */
/* Selected whole columns of the same matrix (every row), for parity  */
/* checks of matrices too large for the full oracle.  Entry (R, C) is */
/* the one ora_assemble produces: computed in the upper triangle      */
/* (R <= C) with the same calls and summation order, mirrored below   */
/* it (AssembleBEMMatrix.cc:753-758).  cols: ncols column indices;    */
/* Mout: N x ncols column-major complex128 with leading dimension ldm. */
/* ------------------------------------------------------------------ */
typedef struct { int s, e, c; } ora_bf;

static ora_bf bf_of(int ns, const int *pec, const int *off, int X)
{
  ora_bf b = {0, 0, 0};
  for (int s = ns - 1; s >= 0; s--)
    if (X >= off[s]) {
      b.s = s;
      if (pec[s]) { b.e = X - off[s]; b.c = 0; }
      else { b.e = (X - off[s]) / 2; b.c = (X - off[s]) % 2; }
      return b;
    }
  return b;
}

/* entry (R, C), R <= C, of the full matrix */
static cplx entry_upper(int ns, ora_surface **S, const int *reg, const int *pec, const int *off, cplx omega,
                        const double *eps, const double *mu, int R, int C)
{
  ora_bf a = bf_of(ns, pec, off, R), b = bf_of(ns, pec, off, C);
  int sa = a.s, sb = b.s;
  int cr[2], nc = 0; double sg[2];
  const int *Ra = reg + 2*sa, *Rb = reg + 2*sb;
  if (Ra[0] == Rb[0]) { cr[nc] = Ra[0]; sg[nc] = 1.0; nc++; }
  else if (Ra[0] == Rb[1]) { cr[nc] = Ra[0]; sg[nc] = -1.0; nc++; }
  if (Ra[1] == Rb[0] && Ra[1] >= 0) { cr[nc] = Ra[1]; sg[nc] = -1.0; nc++; }
  else if (!pec[sa] && !pec[sb] && Ra[1] == Rb[1]) { cr[nc] = Ra[1]; sg[nc] = 1.0; nc++; }
  int sym = (sa == sb);
  int ca = a.c, cb = b.c;
  /* inside a diagonal 2x2 block of one edge the (1,0) entry is never
     stamped: it is the mirror of (0,1) */
  if (sym && a.e == b.e && ca == 1 && cb == 0) { ca = 0; cb = 1; }
  cplx v = 0.0;
  for (int r = 0; r < nc; r++) {
    cplx e = eps[2*cr[r]] + I*eps[2*cr[r]+1], m = mu[2*cr[r]] + I*mu[2*cr[r]+1];
    cplx kk = csqrt2(e*m) * omega;
    cplx PF1 = sg[r]*I*m*omega, PF2 = -sg[r]*I*kk, PF3 = -sg[r]*I*e*omega;
    cplx GC[2];
    ora_eei(S[sa], a.e, S[sb], b.e, kk, GC);
    if (pec[sa] && pec[sb]) v += PF1*GC[0];
    else if (pec[sa]) v += cb == 0 ? PF1*GC[0] : PF2*GC[1];
    else if (pec[sb]) v += ca == 0 ? PF1*GC[0] : PF2*GC[1];
    else if (ca == 0 && cb == 0) v += PF1*GC[0];
    else if (ca == 1 && cb == 1) v += PF3*GC[0];
    else v += PF2*GC[1];
  }
  return v;
}

void ora_assemble_cols(int ns, ora_surface **S, const int *reg, const int *pec,
                       double wr, double wi, const double *eps, const double *mu,
                       int ncols, const int *cols, double *Mout, int ldm)
{
  cplx omega = wr + I*wi;
  cplx *M = (cplx *)Mout;
  int off[64], N = 0;
  for (int s = 0; s < ns; s++) { off[s] = N; N += pec[s] ? S[s]->ne : 2*S[s]->ne; }
  for (int j = 0; j < ncols; j++) {
    const int C = cols[j];
    #pragma omp parallel for schedule(dynamic, 16)
    for (int R = 0; R < N; R++)
      M[R + (size_t)j*ldm] = R <= C ? entry_upper(ns, S, reg, pec, off, omega, eps, mu, R, C)
                                    : entry_upper(ns, S, reg, pec, off, omega, eps, mu, C, R);
  }
}

/* ------------------------------------------------------------------ */
/* The assembly loop of ora_assemble restricted to the column edges    */
/* [eb0, eb1) of one single-surface geometry (every edge pair ea <= eb */
/* with eb in the range, stamped into the full column-major M): the    */
/* bounded slices the CPU baseline times.  Over a partition of        */
/* [0, ne) the slices compute exactly ora_assemble's upper triangle.   */
/* ------------------------------------------------------------------ */
void ora_assemble_stripe(ora_surface *S, int reg_ext, int reg_int, int pec, double wr, double wi,
                         const double *eps, const double *mu, int eb0, int eb1, double *Mout, int N)
{
  cplx omega = wr + I*wi;
  cplx *M = (cplx *)Mout;
  /* CountCommonRegions of a surface with itself: its exterior region, and
     its interior one unless it is PEC (SurfaceSurfaceInteractions.cc:62-90) */
  int cr[2], nc = 0; double sg[2];
  cr[nc] = reg_ext; sg[nc] = 1.0; nc++;
  if (!pec && reg_int >= 0) { cr[nc] = reg_int; sg[nc] = 1.0; nc++; }
  cplx PF1[2], PF2[2], PF3[2], kk[2];
  for (int r = 0; r < nc; r++) {
    cplx e = eps[2*cr[r]] + I*eps[2*cr[r]+1], m = mu[2*cr[r]] + I*mu[2*cr[r]+1];
    kk[r] = csqrt2(e*m) * omega;
    PF1[r] = sg[r]*I*m*omega; PF2[r] = -sg[r]*I*kk[r]; PF3[r] = -sg[r]*I*e*omega;
  }
  #pragma omp parallel for schedule(dynamic, 4)
  for (int ea = 0; ea < eb1; ea++)
    for (int eb = ea > eb0 ? ea : eb0; eb < eb1; eb++)
      for (int r = 0; r < nc; r++) {
        cplx GC[2];
        ora_eei(S, ea, S, eb, kk[r], GC);
        if (pec) {
          M[ea + (size_t)eb*N] += PF1[r]*GC[0];
        } else {
          size_t X = 2*ea, Y = 2*eb;
          M[X + Y*N] += PF1[r]*GC[0];
          M[X + (Y+1)*N] += PF2[r]*GC[1];
          if (ea != eb) M[X+1 + Y*N] += PF2[r]*GC[1];
          M[X+1 + (Y+1)*N] += PF3[r]*GC[0];
        }
      }
}

/* Fill a surface's memo of static near-pair integrals (the warm state of */
/* the reference's FIPPI cache, FIPPICache.cc:135-187) for every ordered  */
/* near pair the assembly of this surface looks up.                      */
long long ora_warm_near(ora_surface *S)
{
  long long n = 0;
  #pragma omp parallel for schedule(dynamic, 8) reduction(+:n)
  for (int pa = 0; pa < S->np; pa++)
    for (int pb = 0; pb < S->np; pb++) {
      const double *Va[3], *Vb[3];
      double rrel;
      int ncv = assess_pair(S, pa, S, pb, &rrel, Va, Vb);
      if (rrel > 4.0 || ncv == 3) continue;
      cplx H[2];
      ora_ppi(S, pa, 0, S, pb, 0, 1.0, H, 0);
      n++;
    }
  return n;
}
