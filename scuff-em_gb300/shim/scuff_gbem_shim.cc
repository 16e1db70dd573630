// scuff_gbem_shim.cc -- the drop-in boundary for SCUFF-EM's own C++ drivers.
//
// Defines, in a shared library of its own, the reference's hot-path entry
// points with their reference signatures:
//   RWGGeometry::AssembleBEMMatrix (both overloads)   libscuff.h:364-365,
//                                                    AssembleBEMMatrix.cc:684-775
//   RWGGeometry::AssembleBEMMatrixBlock               libscuff.h:500-505,
//                                                    AssembleBEMMatrix.cc:349-391
//   HMatrix::LUFactorize, HMatrix::LUSolve (5 forms)  libhmat.h:311-316,
//                                                    LBWrappers.cc:151-248
// and forwards them to the C ABI of include/gbem.h.  A driver (scuff-scatter,
// scuff-cas3D, unchanged) linked with this library ahead of the reference's
// libscuff/libhmat binds those calls here: ELF symbol interposition, the
// first definition in load order wins, so no reference source is edited.
// Everything else (geometry parsing, materials, incident fields, power
// post-processing) stays the reference's.
//
// Semantics kept from the reference:
//  * M == NULL or of the wrong size -> a new matrix from AllocateBEMMatrix
//    (with the reference's warning); the full matrix is symmetric and filled
//    in both triangles for LHM_NORMAL storage, the upper triangle only for
//    packed LHM_SYMMETRIC storage (AssembleBEMMatrix.cc:700-760);
//  * a nonzero Bloch vector on a compact geometry is an error with the
//    reference's message; periodic geometries (LBasis != 0) and the
//    Accelerator/TransposeAccelerator options are not part of this path and
//    stop the program (ErrExit), like the reference's own unsupported cases;
//  * LUFactorize returns LAPACK's info and keeps the factors and 1-based
//    pivots in ZM/DM and ipiv (drivers read M->GetEntry(n,n) after it,
//    CasimirIntegrand.cc:58-62); LHM_REAL matrices factor with dgetrf's
//    pivots (the library factors them as complex128 with zero imaginary
//    parts), LHM_SYMMETRIC with dsptrf/zsptrf's; LHM_HERMITIAN (zhptrf) is
//    outside this library and stops the program;
//  * LUSolve's argument checks and messages are the reference's.
// Library errors map to ErrExit with the library's message, as the
// reference's own fatal errors do (libhrutil.h:136).
#include <complex>
#include <cstring>
#include <map>
#include <mutex>
#include <vector>

#include "libhrutil.h"
#include "libhmat.h"
#include "libscuff.h"
#include "gbem.h"

using namespace scuff;

namespace {

std::mutex g_mu;
std::map<const RWGGeometry *, gbem_geometry *> g_geo;

void check(gbem_status st, const char *what) {
  if (st != GBEM_OK) ErrExit("%s: %s", what, gbem_last_error());
}

int gbem_device() {
  const char *d = getenv("GBEM_DEVICE");
  return d ? atoi(d) : 0;
}

// the library's geometry for a reference geometry (made on first use)
gbem_geometry *geometry_of(RWGGeometry *G) {
  std::lock_guard<std::mutex> l(g_mu);
  auto it = g_geo.find(G);
  if (it != g_geo.end()) return it->second;
  std::vector<gbem_surface_desc> d(G->NumSurfaces);
  std::vector<std::vector<int>> pv(G->NumSurfaces);
  for (int ns = 0; ns < G->NumSurfaces; ns++) {
    RWGSurface *S = G->Surfaces[ns];
    pv[ns].resize(3 * (size_t)S->NumPanels);
    for (int np = 0; np < S->NumPanels; np++)
      for (int i = 0; i < 3; i++) pv[ns][3 * np + i] = S->Panels[np]->VI[i];
    d[ns].num_vertices = S->NumVertices;
    d[ns].vertices = S->Vertices;
    d[ns].num_panels = S->NumPanels;
    d[ns].panel_vertices = pv[ns].data();
    d[ns].exterior_region = S->RegionIndices[0];
    d[ns].interior_region = S->IsPEC ? -1 : S->RegionIndices[1];
    d[ns].is_pec = S->IsPEC ? 1 : 0;
  }
  gbem_geometry *g = nullptr;
  check(gbem_geometry_create(G->NumSurfaces, d.data(), G->NumRegions, gbem_device(), &g), "gbem_geometry_create");
  int N = 0;
  check(gbem_geometry_num_bfs(g, &N), "gbem_geometry_num_bfs");
  if (N != G->TotalBFs) ErrExit("gbem: %d basis functions where the reference counts %d", N, G->TotalBFs);
  g_geo[G] = g;
  return g;
}

// eps, mu of every region at Omega, interleaved (re, im)
void eps_mu(RWGGeometry *G, cdouble Omega, std::vector<double> &eps, std::vector<double> &mu) {
  G->UpdateCachedEpsMuValues(Omega);
  eps.resize(2 * G->NumRegions);
  mu.resize(2 * G->NumRegions);
  for (int r = 0; r < G->NumRegions; r++) {
    eps[2 * r] = real(G->EpsTF[r]); eps[2 * r + 1] = imag(G->EpsTF[r]);
    mu[2 * r] = real(G->MuTF[r]); mu[2 * r + 1] = imag(G->MuTF[r]);
  }
}

void compact_only(RWGGeometry *G, double *kBloch) {
  if (G->LBasis != 0) ErrExit("gbem: periodic geometries are outside this library's path");
  if (kBloch != 0 && (kBloch[0] != 0.0 || kBloch[1] != 0.0))
    ErrExit("%s:%i: Bloch wavevector is undefined for compact geometries", __FILE__, __LINE__);
}

int dtype_of(const HMatrix *M) { return M->RealComplex == LHM_REAL ? GBEM_F64 : GBEM_C128; }
void *data_of(HMatrix *M) { return M->RealComplex == LHM_REAL ? (void *)M->DM : (void *)M->ZM; }

}  // namespace

namespace scuff {

void RWGGeometry::AssembleBEMMatrixBlock(int nsa, int nsb, cdouble Omega, double *kBloch, HMatrix *M,
                                         HMatrix **GradM, int RowOffset, int ColOffset, void *Accelerator,
                                         bool TransposeAccelerator, int NumTorqueAxes, HMatrix **dMdT,
                                         double *GammaMatrix) {
  compact_only(this, kBloch);
  if (Accelerator || TransposeAccelerator) ErrExit("gbem: block accelerators belong to periodic geometries");
  gbem_geometry *g = geometry_of(this);
  std::vector<double> eps, mu;
  eps_mu(this, Omega, eps, mu);
  const double wr = real(Omega), wi = imag(Omega);
  if (M) {
    if (M->StorageType == LHM_NORMAL) {
      check(gbem_assemble_block_host(g, nsa, nsb, wr, wi, eps.data(), mu.data(), data_of(M), M->NR, RowOffset,
                                     ColOffset, dtype_of(M)),
            "AssembleBEMMatrixBlock");
    } else if (M->StorageType == LHM_SYMMETRIC && nsa == nsb && RowOffset == 0 && ColOffset == 0 &&
               M->NR == Surfaces[nsa]->NumBFs) {
      check(gbem_assemble_block_packed_host(g, nsa, wr, wi, eps.data(), mu.data(), data_of(M), dtype_of(M)),
            "AssembleBEMMatrixBlock (packed)");
    } else {
      ErrExit("gbem: packed destinations hold one diagonal block at offset (0,0)");
    }
  }
  for (int m = 0; GradM && m < 3; m++)
    if (GradM[m]) {
      void *out[3] = {nullptr, nullptr, nullptr};
      out[m] = data_of(GradM[m]);
      check(gbem_assemble_block_gradient_host(g, nsa, nsb, wr, wi, eps.data(), mu.data(), out[0], out[1], out[2],
                                              GradM[m]->NR, RowOffset, ColOffset, dtype_of(GradM[m])),
            "AssembleBEMMatrixBlock (GradM)");
    }
  if (NumTorqueAxes > 0 && dMdT && GammaMatrix)
    for (int a = 0; a < NumTorqueAxes; a++)
      if (dMdT[a]) {
        void *out[1] = {data_of(dMdT[a])};
        check(gbem_assemble_block_dmdt_host(g, nsa, nsb, wr, wi, eps.data(), mu.data(), 1, GammaMatrix + 9 * a, out,
                                            dMdT[a]->NR, RowOffset, ColOffset, dtype_of(dMdT[a])),
              "AssembleBEMMatrixBlock (dMdT)");
      }
}

HMatrix *RWGGeometry::AssembleBEMMatrix(cdouble Omega, double *kBloch, HMatrix *M) {
  compact_only(this, kBloch);
  if (M == NULL)
    M = AllocateBEMMatrix();
  else if (M->NR != TotalBFs || M->NC != TotalBFs) {
    Warn("wrong-size matrix passed to AssembleBEMMatrix; reallocating...");
    M = AllocateBEMMatrix();
  }
  Log("Assembling BEM matrix at Omega=%s (GPU)", z2s(Omega));
  gbem_geometry *g = geometry_of(this);
  std::vector<double> eps, mu;
  eps_mu(this, Omega, eps, mu);
  const int N = TotalBFs, dt = dtype_of(M);
  if (M->StorageType == LHM_NORMAL && dt == GBEM_C128) {
    check(gbem_assemble_host(g, real(Omega), imag(Omega), eps.data(), mu.data(), (double *)M->ZM, N),
          "AssembleBEMMatrix");
    return M;
  }
  // real storage, or packed storage: the surface blocks of the upper block
  // triangle into a full array, the lower blocks mirrored from them
  const size_t es = dt == GBEM_C128 ? 16 : 8;
  std::vector<char> tmp;
  char *full = (char *)data_of(M);
  if (M->StorageType != LHM_NORMAL) {
    tmp.assign((size_t)N * N * es, 0);
    full = tmp.data();
  }
  for (int ns = 0; ns < NumSurfaces; ns++)
    for (int nsp = ns; nsp < NumSurfaces; nsp++)
      check(gbem_assemble_block_host(g, ns, nsp, real(Omega), imag(Omega), eps.data(), mu.data(), full, N,
                                     BFIndexOffset[ns], BFIndexOffset[nsp], dt),
            "AssembleBEMMatrix");
  for (int c = 0; c < N; c++)
    for (int r = c + 1; r < N; r++)
      memcpy(full + ((size_t)r + (size_t)c * N) * es, full + ((size_t)c + (size_t)r * N) * es, es);
  if (M->StorageType != LHM_NORMAL)
    for (int c = 0; c < N; c++)
      memcpy((char *)data_of(M) + (size_t)c * (c + 1) / 2 * es, full + (size_t)c * N * es, (size_t)(c + 1) * es);
  return M;
}

HMatrix *RWGGeometry::AssembleBEMMatrix(cdouble Omega, HMatrix *M) { return AssembleBEMMatrix(Omega, 0, M); }

}  // namespace scuff

// ---- LU (HMatrix lives in the global namespace) ----------------------------

int HMatrix::LUFactorize() {
  if (ipiv == 0) ipiv = (int *)mallocEC(NR * sizeof(int));
  int info = 0;
  gbem_status st;
  if (StorageType == LHM_NORMAL && RealComplex == LHM_COMPLEX) {
    st = gbem_lu_factor_host((double *)ZM, NR, NR, ipiv, &info);
  } else if (StorageType == LHM_NORMAL) {
    // real: factored as complex128 with zero imaginary parts (dgetrf's pivots)
    std::vector<cdouble> z((size_t)NR * NR);
    for (size_t i = 0; i < z.size(); i++) z[i] = DM[i];
    st = gbem_lu_factor_host((double *)z.data(), NR, NR, ipiv, &info);
    for (size_t i = 0; i < z.size(); i++) DM[i] = real(z[i]);
  } else if (StorageType == LHM_SYMMETRIC) {
    st = gbem_sp_factor_host(RealComplex == LHM_REAL ? (void *)DM : (void *)ZM, NR,
                             RealComplex == LHM_REAL ? GBEM_F64 : GBEM_C128, ipiv, &info);
  } else {
    ErrExit("gbem: LHM_HERMITIAN packed storage (zhptrf) is outside this library");
  }
  if (st != GBEM_OK && st != GBEM_ESINGULAR) check(st, "LUFactorize");
  return info;
}

int HMatrix::LUSolve(HMatrix *X, char Trans, int nrhs) {
  if (RealComplex != X->RealComplex) ErrExit("type mismatch in LUSolve");
  if (NR != NC || NR != X->NR) ErrExit("dimension mismatch in LUSolve");
  if (nrhs > X->NC) ErrExit("too many RHSs requested in LUSolve");
  if (ipiv == 0) ErrExit("LUFactorize() must be called before LUSolve()");
  if (Trans != 'N' && StorageType != LHM_NORMAL) ErrExit("transposed LU-solves not available for packed matrices");
  if (StorageType == LHM_SYMMETRIC) {
    check(gbem_sp_solve_host(RealComplex == LHM_REAL ? (void *)DM : (void *)ZM, NR,
                             RealComplex == LHM_REAL ? GBEM_F64 : GBEM_C128, ipiv, nrhs,
                             RealComplex == LHM_REAL ? (void *)X->DM : (void *)X->ZM, X->NR),
          "LUSolve");
  } else if (StorageType != LHM_NORMAL) {
    ErrExit("gbem: LHM_HERMITIAN packed storage (zhptrs) is outside this library");
  } else if (RealComplex == LHM_COMPLEX) {
    check(gbem_lu_solve_host((const double *)ZM, NR, NR, ipiv, Trans, nrhs, (double *)X->ZM, X->NR), "LUSolve");
  } else {
    std::vector<cdouble> z((size_t)NR * NR), b((size_t)NR * nrhs);
    for (size_t i = 0; i < z.size(); i++) z[i] = DM[i];
    for (int c = 0; c < nrhs; c++)
      for (int r = 0; r < NR; r++) b[r + (size_t)c * NR] = X->DM[r + (size_t)c * X->NR];
    check(gbem_lu_solve_host((const double *)z.data(), NR, NR, ipiv, Trans, nrhs, (double *)b.data(), NR),
          "LUSolve");
    for (int c = 0; c < nrhs; c++)
      for (int r = 0; r < NR; r++) X->DM[r + (size_t)c * X->NR] = real(b[r + (size_t)c * NR]);
  }
  return 0;
}

int HMatrix::LUSolve(HVector *X) {
  if (RealComplex != X->RealComplex) ErrExit("type mismatch in LUSolve");
  if (NR != NC || NR != X->N) ErrExit("dimension mismatch in LUSolve");
  HMatrix XM(X->N, 1, X->RealComplex, X->RealComplex == LHM_REAL ? (void *)X->DV : (void *)X->ZV);
  return LUSolve(&XM, 'N', 1);
}

int HMatrix::LUSolve(HMatrix *X) { return LUSolve(X, 'N', X->NC); }
int HMatrix::LUSolve(HMatrix *X, int nrhs) { return LUSolve(X, 'N', nrhs); }
int HMatrix::LUSolve(HMatrix *X, char Trans) { return LUSolve(X, Trans, X->NC); }
