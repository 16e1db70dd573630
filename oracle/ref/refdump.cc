// refdump: a small driver linked against the reference implementation built
// from its own sources (oracle/ref/Makefile).  It exists only to produce golden
// vectors for the tests and to time the reference's CPU path; nothing in the
// product links it.
//
// Commands (all output is plain text or raw little-endian binary):
//   refdump geom   GEO OUT                   panels and RWG edges of every surface
//   refdump matrix GEO wr wi OUT             full BEM matrix (int32 N, then N*N complex128, column-major)
//   refdump cache  GEO wr wi OUT             assemble, then write the FIPPI cache file (StoreCache)
//   refdump cachematrix GEO wr wi CACHE OUT  PreloadCache(CACHE), assemble, write the matrix
//                                            (both print the cache's hits and misses)
//   refdump ppi    GEO ns LIST OUT           panel-panel integrals for "npa iQa npb iQb kr ki" lines
//   refdump fippi  GEO ns LIST OUT           Q-independent FIPPI data for "npa npb" lines
//   refdump rhs    GEO wr wi E0x E0y E0z nx ny nz OUT   plane-wave RHS (int32 N, N complex128)
//   refdump pft    GEO wr wi E0x E0y E0z nx ny nz OUT   assemble, LU, solve, EMT power; KN vector
//   refdump time   GEO wr wi NREP            wall time of AssembleBEMMatrix, LUFactorize, LUSolve
//   refdump gradblock GEO wr wi nsa nsb OUT  block (nsa,nsb) and its three gradients d/dx_mu
//                                            (per matrix: int32 NR NC, then NR*NC complex128 column-major)
//   refdump torqueblock GEO wr wi nsa nsb OUT  block (nsa,nsb) and its derivatives dM/dtheta for
//                                            rotations about the x, y and z axes through the origin
//                                            (GammaMatrix = the cross-product matrix of each axis)
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include <omp.h>
#include <complex>

#include <libhrutil.h>
#include <libhmat.h>
#include <libIncField.h>
#include <libscuff.h>
#include <libscuffInternals.h>

using namespace scuff;

static double now() { return omp_get_wtime(); }

static void write_matrix(const char *fn, HMatrix *M) {
  FILE *f = fopen(fn, "wb");
  int N = M->NR;
  fwrite(&N, sizeof(int), 1, f);
  for (int c = 0; c < N; c++)
    for (int r = 0; r < N; r++) {
      cdouble z = M->GetEntry(r, c);
      double d[2] = {real(z), imag(z)};
      fwrite(d, sizeof(double), 2, f);
    }
  fclose(f);
}

static void append_rect(FILE *f, HMatrix *M) {
  int nr = M->NR, nc = M->NC;
  fwrite(&nr, sizeof(int), 1, f);
  fwrite(&nc, sizeof(int), 1, f);
  for (int c = 0; c < nc; c++)
    for (int r = 0; r < nr; r++) {
      cdouble z = M->GetEntry(r, c);
      double d[2] = {real(z), imag(z)};
      fwrite(d, sizeof(double), 2, f);
    }
}

static void write_vector(const char *fn, HVector *V) {
  FILE *f = fopen(fn, "wb");
  int N = V->N;
  fwrite(&N, sizeof(int), 1, f);
  for (int r = 0; r < N; r++) {
    cdouble z = V->GetEntry(r);
    double d[2] = {real(z), imag(z)};
    fwrite(d, sizeof(double), 2, f);
  }
  fclose(f);
}

int main(int argc, char **argv) {
  if (argc < 3) { fprintf(stderr, "usage: refdump CMD GEO ...\n"); return 2; }
  const char *cmd = argv[1];
  RWGGeometry *G = new RWGGeometry(argv[2]);

  if (!strcmp(cmd, "geom")) {
    FILE *f = fopen(argv[3], "w");
    fprintf(f, "surfaces %d totalbfs %d\n", G->NumSurfaces, G->TotalBFs);
    for (int ns = 0; ns < G->NumSurfaces; ns++) {
      RWGSurface *S = G->Surfaces[ns];
      fprintf(f, "surface %d pec %d nv %d np %d ne %d offset %d\n", ns, S->IsPEC ? 1 : 0,
              S->NumVertices, S->NumPanels, S->NumEdges, G->BFIndexOffset[ns]);
      for (int np = 0; np < S->NumPanels; np++) {
        RWGPanel *P = S->Panels[np];
        fprintf(f, "P %d %d %d %.17e %.17e\n", P->VI[0], P->VI[1], P->VI[2], P->Radius, P->Area);
      }
      for (int ne = 0; ne < S->NumEdges; ne++) {
        RWGEdge *E = S->Edges[ne];
        fprintf(f, "E %d %d %d %d %d %d %d %d %d %.17e\n", E->iV1, E->iV2, E->iQP, E->iQM,
                E->iPPanel, E->iMPanel, E->PIndex, E->MIndex, E->Index, E->Length);
      }
    }
    fclose(f);
    return 0;
  }

  if (!strcmp(cmd, "cache")) {
    // assemble once (every near pair's FIPPI record goes to the global cache),
    // then write the cache file (StoreCache, FIPPICache.cc:223-293)
    cdouble Omega(atof(argv[3]), atof(argv[4]));
    HMatrix *M = G->AllocateBEMMatrix();
    G->AssembleBEMMatrix(Omega, M);
    StoreCache(argv[5]);
    printf("%d %d\n", (int)GlobalFIPPICache.Hits, (int)GlobalFIPPICache.Misses);
    return 0;
  }

  if (!strcmp(cmd, "cachematrix")) {
    // PreloadCache(CACHE), assemble, write the matrix; prints the cache hits and misses
    PreloadCache(argv[5]);
    cdouble Omega(atof(argv[3]), atof(argv[4]));
    HMatrix *M = G->AllocateBEMMatrix();
    G->AssembleBEMMatrix(Omega, M);
    write_matrix(argv[6], M);
    printf("%d %d\n", (int)GlobalFIPPICache.Hits, (int)GlobalFIPPICache.Misses);
    return 0;
  }

  if (!strcmp(cmd, "matrix")) {
    cdouble Omega(atof(argv[3]), atof(argv[4]));
    HMatrix *M = G->AllocateBEMMatrix();
    G->AssembleBEMMatrix(Omega, M);
    write_matrix(argv[5], M);
    return 0;
  }

  if (!strcmp(cmd, "ppi") || !strcmp(cmd, "fippi")) {
    int ns = atoi(argv[3]);
    RWGSurface *S = G->Surfaces[ns];
    FILE *in = fopen(argv[4], "r");
    FILE *out = fopen(argv[5], "w");
    char line[512];
    while (fgets(line, sizeof line, in)) {
      if (!strcmp(cmd, "ppi")) {
        int npa, iQa, npb, iQb;
        double kr, ki;
        if (sscanf(line, "%d %d %d %d %le %le", &npa, &iQa, &npb, &iQb, &kr, &ki) != 6) continue;
        GetPPIArgStruct A;
        InitGetPPIArgs(&A);
        A.Sa = A.Sb = S;
        A.npa = npa; A.iQa = iQa; A.npb = npb; A.iQb = iQb;
        A.k = cdouble(kr, ki);
        GetPanelPanelInteractions(&A);
        double rRel;
        int ncv = AssessPanelPair(S, npa, S, npb, &rRel);
        fprintf(out, "%.17e %.17e %.17e %.17e %d %d %.17e\n", real(A.H[0]), imag(A.H[0]),
                real(A.H[1]), imag(A.H[1]), A.WhichAlgorithm, ncv, rRel);
      } else {
        int npa, npb;
        if (sscanf(line, "%d %d", &npa, &npb) != 2) continue;
        double *Va[3], *Vb[3], rRel;
        int ncv = AssessPanelPair(S, npa, S, npb, &rRel, Va, Vb);
        QIFIPPIData Q;
        ComputeQIFIPPIData(Va, Vb, ncv, &Q);
        fprintf(out, "%d", ncv);
        for (int i = 0; i < 3; i++) fprintf(out, " %.17e", Q.xMxpRM3[i]);
        for (int i = 0; i < 3; i++) fprintf(out, " %.17e", Q.xXxpRM3[i]);
        for (int i = 0; i < 9; i++) fprintf(out, " %.17e", Q.uvupvpRM1[i]);
        for (int i = 0; i < 9; i++) fprintf(out, " %.17e", Q.uvupvpR1[i]);
        for (int i = 0; i < 9; i++) fprintf(out, " %.17e", Q.uvupvpR2[i]);
        // the vertex order AssessPanelPair chose (as vertex indices)
        RWGPanel *Pa = S->Panels[npa], *Pb = S->Panels[npb];
        for (int i = 0; i < 3; i++) fprintf(out, " %d", (int)((Va[i] - S->Vertices) / 3));
        for (int i = 0; i < 3; i++) fprintf(out, " %d", (int)((Vb[i] - S->Vertices) / 3));
        (void)Pa; (void)Pb;
        fprintf(out, "\n");
      }
    }
    fclose(in);
    fclose(out);
    return 0;
  }

  if (!strcmp(cmd, "rhs") || !strcmp(cmd, "pft")) {
    cdouble Omega(atof(argv[3]), atof(argv[4]));
    cdouble E0[3] = {atof(argv[5]), atof(argv[6]), atof(argv[7])};
    double nHat[3] = {atof(argv[8]), atof(argv[9]), atof(argv[10])};
    PlaneWave PW(E0, nHat);
    HVector *KN = G->AllocateRHSVector();
    G->AssembleRHSVector(Omega, &PW, KN);
    if (!strcmp(cmd, "rhs")) {
      write_vector(argv[11], KN);
      return 0;
    }
    HVector *RHS = G->AllocateRHSVector();
    RHS->Copy(KN);
    HMatrix *M = G->AllocateBEMMatrix();
    G->AssembleBEMMatrix(Omega, M);
    int info = M->LUFactorize();
    M->LUSolve(KN);
    write_vector(argv[11], KN);
    PFTOptions Opts;
    InitPFTOptions(&Opts);
    Opts.IF = &PW;
    Opts.RHSVector = RHS;
    double PFT[NUMPFT];
    G->GetPFT(0, KN, Omega, PFT, &Opts);
    printf("info %d PAbs %.17e PScat %.17e Fz %.17e\n", info, PFT[PFT_PABS], PFT[PFT_PSCAT], PFT[PFT_ZFORCE]);
    return 0;
  }

  if (!strcmp(cmd, "time")) {
    cdouble Omega(atof(argv[3]), atof(argv[4]));
    int nrep = argc > 5 ? atoi(argv[5]) : 1;
    HMatrix *M = G->AllocateBEMMatrix();
    double t0 = now();
    G->AssembleBEMMatrix(Omega, M);  // cold: fills the FIPPI cache
    double tcold = now() - t0;
    double twarm = 1e30, tlu = 1e30, tsolve = 1e30;
    HVector *B = G->AllocateRHSVector();
    for (int r = 0; r < nrep; r++) {
      t0 = now();
      G->AssembleBEMMatrix(Omega, M);
      twarm = fmin(twarm, now() - t0);
      t0 = now();
      M->LUFactorize();
      tlu = fmin(tlu, now() - t0);
      for (int i = 0; i < B->N; i++) B->SetEntry(i, 1.0);
      t0 = now();
      M->LUSolve(B);
      tsolve = fmin(tsolve, now() - t0);
    }
    printf("N %d threads %d assemble_cold %.6f assemble_warm %.6f lu %.6f solve1 %.6f\n", G->TotalBFs,
           omp_get_max_threads(), tcold, twarm, tlu, tsolve);
    return 0;
  }

  if (!strcmp(cmd, "gradblock")) {
    cdouble Omega(atof(argv[3]), atof(argv[4]));
    int nsa = atoi(argv[5]), nsb = atoi(argv[6]);
    int NR = G->Surfaces[nsa]->NumBFs, NC = G->Surfaces[nsb]->NumBFs;
    HMatrix *M = new HMatrix(NR, NC, LHM_COMPLEX);
    HMatrix *GradM[3];
    for (int mu = 0; mu < 3; mu++) GradM[mu] = new HMatrix(NR, NC, LHM_COMPLEX);
    M->Zero();
    for (int mu = 0; mu < 3; mu++) GradM[mu]->Zero();
    G->AssembleBEMMatrixBlock(nsa, nsb, Omega, 0, M, GradM, 0, 0);
    FILE *f = fopen(argv[7], "wb");
    append_rect(f, M);
    for (int mu = 0; mu < 3; mu++) append_rect(f, GradM[mu]);
    fclose(f);
    return 0;
  }

  if (!strcmp(cmd, "torqueblock")) {
    cdouble Omega(atof(argv[3]), atof(argv[4]));
    int nsa = atoi(argv[5]), nsb = atoi(argv[6]);
    int NR = G->Surfaces[nsa]->NumBFs, NC = G->Surfaces[nsb]->NumBFs;
    HMatrix *M = new HMatrix(NR, NC, LHM_COMPLEX);
    HMatrix *dMdT[3];
    for (int a = 0; a < 3; a++) dMdT[a] = new HMatrix(NR, NC, LHM_COMPLEX);
    M->Zero();
    for (int a = 0; a < 3; a++) dMdT[a]->Zero();
    // dX = n x X for axis n: Gamma[9 a + Mu + 3 Nu] = (n x e_Nu)_Mu
    double Gamma[27];
    memset(Gamma, 0, sizeof Gamma);
    for (int a = 0; a < 3; a++)
      for (int nu = 0; nu < 3; nu++) {
        double n[3] = {0, 0, 0}, e[3] = {0, 0, 0}, c[3];
        n[a] = 1.0; e[nu] = 1.0;
        c[0] = n[1] * e[2] - n[2] * e[1]; c[1] = n[2] * e[0] - n[0] * e[2]; c[2] = n[0] * e[1] - n[1] * e[0];
        for (int mu = 0; mu < 3; mu++) Gamma[9 * a + mu + 3 * nu] = c[mu];
      }
    G->AssembleBEMMatrixBlock(nsa, nsb, Omega, 0, M, 0, 0, 0, 0, false, 3, dMdT, Gamma);
    FILE *f = fopen(argv[7], "wb");
    append_rect(f, M);
    for (int a = 0; a < 3; a++) append_rect(f, dMdT[a]);
    fclose(f);
    return 0;
  }

  fprintf(stderr, "unknown command %s\n", cmd);
  return 2;
}
