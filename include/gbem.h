/*
 * gbem.h -- C ABI of the GB300-native BEM hot path (matrix assembly and dense
 * complex LU factor/solve) that stands in for SCUFF-EM's
 *   RWGGeometry::AssembleBEMMatrix / AssembleBEMMatrixBlock   (libs/libscuff)
 *   HMatrix::LUFactorize / HMatrix::LUSolve                  (libs/libhmat)
 *
 * Plain C types only; every call returns a gbem_status; no call aborts the
 * process.  Matrices are column-major (entry (r,c) at r + c*ld), complex
 * entries interleaved (re, im), as in HMatrix's ZM array
 * (libs/libhmat/HMatrix.cc:333).  Pivots are LAPACK-style, 1-based.
 *
 * Threading: distinct handles may be used from distinct host threads; a
 * handle is not re-entrant.  Each handle owns one CUDA stream.
 */
#ifndef GBEM_H
#define GBEM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  GBEM_OK = 0,
  GBEM_EINVAL = 1,    /* bad argument (the analogue of LAPACK info < 0) */
  GBEM_ENOMEM = 2,    /* device or host allocation failed */
  GBEM_ECUDA = 3,     /* a CUDA runtime error; see gbem_last_error() */
  GBEM_ENOTSUP = 4,   /* valid request outside what this build implements */
  GBEM_ESINGULAR = 5, /* zero pivot met (info > 0 is also returned) */
  GBEM_ENOCONV = 6,   /* iterative refinement did not reach its tolerance */
  GBEM_EMESH = 7,     /* non-manifold mesh topology */
  GBEM_ETIMEOUT = 8   /* a bounded device-side wait gave up */
} gbem_status;

/* arithmetic of a matrix / of an assembly */
typedef enum {
  GBEM_C128 = 0,      /* complex double (the reference's ZM) */
  GBEM_C64 = 1,       /* complex float */
  GBEM_F64 = 2        /* real double (imaginary frequency; the reference's DM) */
} gbem_dtype;

/* precision of the far-field panel-pair cubature in an assembly */
typedef enum {
  GBEM_PREC_FP64 = 0, /* plain: everything in FP64 */
  GBEM_PREC_MIXED = 1 /* far field in FP32, near/singular pairs in FP64 */
} gbem_precision;

typedef struct gbem_geometry gbem_geometry;
typedef struct gbem_matrix gbem_matrix;

/* A closed or open triangulated surface (one OBJECT of a .scuffgeo file). */
typedef struct {
  int num_vertices;
  const double *vertices;      /* 3*num_vertices, already displaced/rotated */
  int num_panels;
  const int *panel_vertices;   /* 3*num_panels, 0-based vertex indices */
  int exterior_region;         /* index of the region the normals point into */
  int interior_region;         /* region inside; -1 for a PEC body */
  int is_pec;
} gbem_surface_desc;

/* last error message of the calling thread (never NULL) */
const char *gbem_last_error(void);
/* library version string */
const char *gbem_version(void);

/* ---- geometry ---------------------------------------------------------- */
/* Replaces RWGGeometry(const char *GeoFile) (libs/libscuff/RWGGeometry.cc:353)
 * for the parts the hot path needs: panels (RWGSurface.cc:55-100), RWG edges
 * (InitEdgeList.cc:47-371), basis-function offsets (RWGGeometry.cc:708-724),
 * and the frequency-independent near-pair classification
 * (AssessPanelPair.cc:52-172).  device: CUDA ordinal. */
gbem_status gbem_geometry_create(int num_surfaces, const gbem_surface_desc *surfaces,
                                 int num_regions, int device, gbem_geometry **out);
gbem_status gbem_geometry_destroy(gbem_geometry *g);
/* Total basis functions (RWGGeometry::TotalBFs, libscuff.h:555). */
gbem_status gbem_geometry_num_bfs(const gbem_geometry *g, int *N);
/* Per-surface edge table: 8 ints per edge (iV1 iV2 iQP iQM iPPanel iMPanel
 * PIndex MIndex, libscuff.h:124-146) and edge lengths. */
gbem_status gbem_geometry_edges(const gbem_geometry *g, int surface, int *num_edges,
                                int *edge_table, double *lengths);
/* Run this geometry's device work on a caller-owned CUDA stream (a
 * cudaStream_t passed as void*; NULL restores the library's own stream).
 * No counterpart in the reference (host-only); lets a caller order the
 * library's kernels with its own work and time them with its own events. */
gbem_status gbem_geometry_set_stream(gbem_geometry *g, void *stream);
/* Counts of near panel pairs by common-vertex number (0..3), for logging. */
gbem_status gbem_geometry_near_counts(const gbem_geometry *g, long long counts[4]);

/* ---- matrices ------------------------------------------------------------ */
/* A device-resident N x N matrix (replaces AllocateBEMMatrix,
 * AssembleBEMMatrix.cc:778-783). */
gbem_status gbem_matrix_create(const gbem_geometry *g, int dtype, gbem_matrix **out);
gbem_status gbem_matrix_destroy(gbem_matrix *m);
gbem_status gbem_matrix_device_ptr(gbem_matrix *m, void **dptr, int *ld);
gbem_status gbem_matrix_download(gbem_matrix *m, void *host, int ldh);
gbem_status gbem_matrix_upload(gbem_matrix *m, const void *host, int ldh);

/* Replaces RWGGeometry::AssembleBEMMatrix(cdouble Omega, HMatrix *M)
 * (AssembleBEMMatrix.cc:684-765, compact geometries, kBloch = NULL).
 * eps/mu: 2*num_regions doubles each (re, im) at this frequency (the values
 * RWGGeometry::UpdateCachedEpsMuValues caches, RWGGeometry.cc:1093-1113).
 * precision: gbem_precision.  The matrix dtype must be C128 or F64 for FP64
 * and C64 for MIXED; F64 (the reference's real storage, used at purely
 * imaginary Omega where the matrix is real) keeps the real part. */
gbem_status gbem_assemble(gbem_geometry *g, double omega_re, double omega_im,
                          const double *eps, const double *mu, int precision,
                          gbem_matrix *M);

/* Host-buffer variant with the reference's drop-in semantics: fills a host
 * column-major complex128 N x N array (HMatrix::ZM) with leading dimension ld. */
gbem_status gbem_assemble_host(gbem_geometry *g, double omega_re, double omega_im,
                               const double *eps, const double *mu, double *ZM, int ld);

/* Replaces RWGGeometry::AssembleBEMMatrixBlock(nsa, nsb, Omega, kBloch=NULL, M,
 * GradM=NULL, RowOffset, ColOffset) (AssembleBEMMatrix.cc:349-391, compact
 * geometries): the block of rows of surface nsa's basis functions and columns
 * of surface nsb's, written to the device array dst (column-major, leading
 * dimension ld) at (row0, col0).  dtype C128 or F64 with GBEM_PREC_FP64 (F64:
 * real storage, the reference's LHM_REAL at imaginary frequency, where the
 * block is real), C64 with GBEM_PREC_MIXED.  Gradient blocks (GradM) come
 * from gbem_assemble_block_gradient, torque blocks (dMdT) from
 * gbem_assemble_block_dmdt. */
gbem_status gbem_assemble_block(gbem_geometry *g, int nsa, int nsb, double omega_re, double omega_im,
                                const double *eps, const double *mu, int precision, void *dst, int ld,
                                int row0, int col0, int dtype);
/* The gradient blocks GradM[mu] = dM/dx_mu of the (nsa, nsb) block under a
 * rigid displacement of surface nsa (AssembleBEMMatrixBlock's GradM,
 * AssembleBEMMatrix.cc:349-391 with PanelPanelInteractions.cc:166-181):
 * device arrays gx, gy, gz (any may be NULL to skip that component), same
 * layout as gbem_assemble_block; FP64, dtype C128 or F64.  Far pairs use the
 * 6x6 rule, near pairs a high-order rule without desingularisation, and
 * pairs on the Taylor-Duffy branch contribute zero, as in the reference. */
gbem_status gbem_assemble_block_gradient(gbem_geometry *g, int nsa, int nsb, double omega_re,
                                         double omega_im, const double *eps, const double *mu,
                                         void *gx, void *gy, void *gz, int ld, int row0, int col0,
                                         int dtype);
/* The torque blocks dMdT[a] = dM/dtheta_a of the (nsa, nsb) block under a
 * rotation of surface nsa generated by gamma + 9a (dX = Gamma X, with
 * gamma[9a + mu + 3 nu] = Gamma_{mu nu}; the GammaMatrix of
 * AssembleBEMMatrixBlock(..., NumTorqueAxes, dMdT, GammaMatrix),
 * AssembleBEMMatrix.cc:341-400, integrand PanelPanelInteractions.cc:183-199):
 * naxes (1..3) device arrays out[a], same layout, rules and branches as
 * gbem_assemble_block_gradient; dtype C128 or F64. */
gbem_status gbem_assemble_block_dmdt(gbem_geometry *g, int nsa, int nsb, double omega_re, double omega_im,
                                     const double *eps, const double *mu, int naxes, const double *gamma,
                                     void *const *out, int ld, int row0, int col0, int dtype);
/* Host-buffer variant of gbem_assemble_block_dmdt. */
gbem_status gbem_assemble_block_dmdt_host(gbem_geometry *g, int nsa, int nsb, double omega_re,
                                          double omega_im, const double *eps, const double *mu, int naxes,
                                          const double *gamma, void *const *out, int ld, int row0, int col0,
                                          int dtype);
/* Host-buffer variant of gbem_assemble_block_gradient. */
gbem_status gbem_assemble_block_gradient_host(gbem_geometry *g, int nsa, int nsb, double omega_re,
                                              double omega_im, const double *eps, const double *mu,
                                              void *gx, void *gy, void *gz, int ld, int row0, int col0,
                                              int dtype);
/* Host-buffer variant of gbem_assemble_block (FP64; dtype C128 or F64): fills
 * rows row0.. and columns col0.. of the host column-major array host. */
gbem_status gbem_assemble_block_host(gbem_geometry *g, int nsa, int nsb, double omega_re, double omega_im,
                                     const double *eps, const double *mu, void *host, int ld, int row0,
                                     int col0, int dtype);

/* ---- dense LU ------------------------------------------------------------ */
/* Replaces HMatrix::LUFactorize (libs/libhmat/LBWrappers.cc:151-171):
 * in-place LU with partial pivoting of a C128 (zgetrf semantics), F64
 * (dgetrf semantics, computed as complex128 with zero imaginary parts) or C64
 * matrix.  ipiv (optional, host, N ints) receives 1-based pivots; info is 0,
 * or k > 0 if U(k,k) is exactly zero. */
gbem_status gbem_lu_factor(gbem_matrix *M, int *ipiv, int *info);

/* Replaces HMatrix::LUSolve(HMatrix *X, char Trans, int nrhs)
 * (LBWrappers.cc:208-236): solves op(M) X = B in place on a host
 * column-major array B (N x nrhs, ldb) of the factor's type (C128, C64, or
 * real F64); trans is 'N', 'T' or 'C' (conjugate transpose, as zgetrs). */
gbem_status gbem_lu_solve(gbem_matrix *M, char trans, int nrhs, void *B, int ldb);

/* Trace of M^-1 B over the first ncols diagonal entries, for a factored M
 * (gbem_lu_factor) and B of M's size and element type (F64, C128 or C64)
 * whose first ncols columns hold the derivative blocks of the BEM matrix:
 * trace[0] = Re, trace[1] = Im.  Replaces the M->LUSolve(dM) + diagonal sum
 * of GetTraceMInvdM (applications/scuff-cas3D/CasimirIntegrand.cc:100-146),
 * whose force is -2 Re(trace) / (2 pi).  B on the device (a gbem_matrix) or
 * on the host (leading dimension ldb >= N). */
gbem_status gbem_lu_trace(gbem_matrix *M, const gbem_matrix *B, int ncols, double *trace);
gbem_status gbem_lu_trace_host(gbem_matrix *M, const void *B, int ldb, int ncols, double *trace);

/* log|det M| of a factored M (gbem_lu_factor): the sum of log|U(n,n)| over
 * the diagonal of its LU factor, the quantity GetLNDetMInvMInf sums from the
 * factors of M and of its diagonal T blocks for the Casimir energy
 * integrand (applications/scuff-cas3D/CasimirIntegrand.cc:50-63); -inf if a
 * pivot is exactly zero. */
gbem_status gbem_lu_log_abs_det(gbem_matrix *M, double *logdet);

/* The LU tuning choices made so far on device `device` (no reference
 * counterpart; LAPACK has no tunables here), as JSON: the register leaf's
 * threads per 64-row bucket of rows per CTA, and the complex-FP32 panel width
 * per 1024-row bucket of N.  Writes at most cap bytes including the
 * terminating NUL; returns GBEM_EINVAL if the text does not fit. */
gbem_status gbem_lu_tuning(int device, char *buf, int cap);

/* gbem_lu_solve without any device allocation.  No counterpart in the
 * reference (HMatrix::LUSolve runs LAPACK on host memory).  Same arguments
 * and results as gbem_lu_solve for complex128 and complex64 matrices; a real
 * F64 matrix (imaginary frequency) returns GBEM_EINVAL, since its solve runs
 * through a complex128 copy of the whole factor that no fixed scratch could
 * hold -- use gbem_lu_solve there.  It serves callers that cannot allocate GPU
 * memory at solve time: a process whose HBM is already taken by its
 * matrices or held by another allocator's pool (a PyTorch caching allocator,
 * say), where a cudaMalloc/cudaMallocAsync inside the solve would fail.
 * Its workspace is one 16 MiB device array of the library, reserved when the
 * library's LU code first loads on a device, so N is limited: N <= 13088
 * for a complex128 matrix, N <= 14528 for complex64; larger N returns
 * GBEM_EINVAL with the limit in gbem_last_error().  The first call on each
 * device looks up that array's device address (with the device current);
 * make that first call before any stream capture begins.  Every call on a
 * device shares the one array and leaves its last contents there; nothing
 * in it has to start at zero, since each call writes every scratch byte
 * before reading it.  Calls that overlap in time on one device (other host
 * threads, other matrices) race on the array and must be serialised by the
 * caller; each call synchronises the matrix's stream before returning, on
 * success and on error alike. */
gbem_status gbem_lu_solve_noalloc(gbem_matrix *M, char trans, int nrhs, void *B, int ldb);

/* Host-buffer drop-in for LUFactorize on a whole HMatrix: factors the host
 * column-major C128 array ZM (N x N, ld) in place and writes 1-based ipiv. */
gbem_status gbem_lu_factor_host(double *ZM, int N, int ld, int *ipiv, int *info);
/* Drop-in for LUSolve with host factors from gbem_lu_factor_host. */
gbem_status gbem_lu_solve_host(const double *ZM, int N, int ld, const int *ipiv,
                               char trans, int nrhs, double *B, int ldb);

/* ---- symmetric matrices in packed storage --------------------------------
 * HMatrix's LHM_SYMMETRIC storage (libs/libhmat/HMatrix.cc:333): the upper
 * triangle by columns, entry (i, j), i <= j, at i + j (j + 1) / 2, real (F64)
 * or complex symmetric (C128, A = A^T). */
/* The diagonal block (ns, ns) of AssembleBEMMatrixBlock
 * (AssembleBEMMatrix.cc:349-391) into a packed LHM_SYMMETRIC destination, as
 * scuff-cas3D allocates its T blocks (applications/scuff-cas3D/
 * CreateSC3Data.cc:110): AP holds NumBFs(ns) (NumBFs(ns) + 1) / 2 entries;
 * FP64; dtype F64 (imaginary frequency) or C128. */
gbem_status gbem_assemble_block_packed_host(gbem_geometry *g, int ns, double omega_re, double omega_im,
                                            const double *eps, const double *mu, void *AP, int dtype);
/* Replaces HMatrix::LUFactorize for LHM_SYMMETRIC storage
 * (LBWrappers.cc:159-166: dsptrf_ / zsptrf_ with UPLO = 'U'): Bunch-Kaufman
 * A = U D U^T in place on the host packed array AP, LAPACK's pivot codes in
 * ipiv (1-based; a 2 x 2 block at k-1, k has ipiv[k-1] = ipiv[k] < 0) and
 * its INFO (k > 0: D(k,k) exactly zero, GBEM_ESINGULAR). */
gbem_status gbem_sp_factor_host(void *AP, int N, int dtype, int *ipiv, int *info);
/* Replaces the LHM_SYMMETRIC branch of HMatrix::LUSolve (LBWrappers.cc:
 * 175-236: dsptrs_ / zsptrs_ 'U'): solves A X = B in place on the host
 * column-major B (N x nrhs, ldb) with the factor and pivots of
 * gbem_sp_factor_host. */
gbem_status gbem_sp_solve_host(const void *AP, int N, int dtype, const int *ipiv, int nrhs, void *B, int ldb);

/* ---- mixed-precision solve ----------------------------------------------- */
/* One BEM solve in the mixed form: assemble the matrix with an FP32 far
 * field and FP64 near field into C64, factor it in complex FP32 with pivoting
 * and tensor-core trailing updates, then refine x with FP64 residuals against
 * the assembled matrix until ||b - M x|| <= tol ||b|| (or max_iter).
 * B, X: host column-major C128 N x nrhs.  iters (optional) receives the
 * refinement sweeps taken, resid the final relative residual. */
gbem_status gbem_solve_mixed(gbem_geometry *g, double omega_re, double omega_im,
                             const double *eps, const double *mu, int nrhs,
                             const double *B, int ldb, double *X, int ldx,
                             double tol, int max_iter, int *iters, double *resid);

/* The FP64 solve by mixed-precision refinement (the gbem_solve_refined of the
 * replacement's C ABI; the reference solves with zgetrf/zgetrs on the FP64
 * matrix, LBWrappers.cc:151-236): the matrix is assembled in FP64
 * (complex128), its complex64 rounding is factored (tensor-core LU), and x
 * is refined with FP64 residuals against the complex128 matrix until
 * ||b - M x|| <= tol ||b||, so x is the FP64 solve's to that tolerance.
 * Arguments as gbem_solve_mixed. */
gbem_status gbem_solve_refined(gbem_geometry *g, double omega_re, double omega_im, const double *eps,
                               const double *mu, int nrhs, const double *B, int ldb, double *X, int ldx,
                               double tol, int max_iter, int *iters, double *resid);

/* A batch of independent mixed-precision solves (frequency sweeps and
 * multi-geometry jobs of uneven N; no counterpart in the reference, whose
 * drivers loop over frequencies and geometries one solve at a time).  Up to
 * max_concurrent jobs run at once, each on its geometry's own CUDA stream
 * from its own host thread, so the kernels of small jobs share the GPU;
 * jobs on the same geometry run one after another (a geometry holds one
 * stream and one set of cached buffers).  Largest N first.  Each job's
 * status, sweeps and residual are written to its own fields. */
typedef struct {
  gbem_geometry *g;
  double omega_re, omega_im;
  const double *eps, *mu;  /* per region, interleaved complex (as gbem_assemble) */
  int nrhs;
  const double *B;         /* host N x nrhs complex128, column-major */
  int ldb;
  double *X;               /* host N x nrhs complex128 */
  int ldx;
  double tol;
  int max_iter;
  int iters;               /* out */
  double resid;            /* out */
  gbem_status status;      /* out */
} gbem_batch_job;
gbem_status gbem_solve_mixed_batch(int njobs, gbem_batch_job *jobs, int max_concurrent);

/* Device-resident variant of gbem_solve_mixed: dB and dX are device
 * pointers (N x nrhs complex128, column-major).  No counterpart in the
 * reference, whose solves run on host arrays; it serves callers whose
 * right-hand sides already live in GPU memory.  The C64 matrix, its factor
 * and the refinement workspace are cached on the geometry between calls. */
gbem_status gbem_solve_mixed_device(gbem_geometry *g, double omega_re, double omega_im,
                                    const double *eps, const double *mu, int nrhs,
                                    const void *dB, int ldb, void *dX, int ldx,
                                    double tol, int max_iter, int *iters, double *resid);

/* Process-wide stage statistics (no counterpart in the reference, whose
 * stage timings are log lines, SurfaceSurfaceInteractions.cc:550-558):
 * returns the device milliseconds (CUDA events on the launching stream) and
 * kernel-launch counts accumulated since the previous call, per stage
 * [0] far-field tiles, [1] near/singular pairs, [2] LU panels, [3] LU
 * trailing updates, [4] triangular solves, [5] FP64 residuals, [6] other,
 * [7] reserved; then resets them.  enable != 0 turns event timing on for
 * subsequent calls (launch counts are always kept). */
gbem_status gbem_stats(int enable, double ms[8], long long counts[8]);

/* ---- power (EMT) ------------------------------------------------------------ */
/* Scattered and extinguished power of nrhs solutions (the EMT method of
 * GetPFT, EMTPFT.cc:468-700; absorbed power = extinction - scattered).  KN:
 * host N x nrhs complex128 solution vectors in the reference's layout (K and
 * -N/ZVAC interleaved on dielectric surfaces); rhs (optional, for pext): the
 * matching plane-wave right-hand sides.  P_scat is a quadratic form of K, N
 * with the exterior region's own matrix, assembled here with `precision`.
 * Every surface must face region 0; nrhs <= 8.  Powers in the reference's
 * units (W for |E0| = 1 V/um). */
gbem_status gbem_power_emt(gbem_geometry *g, double omega_re, double omega_im, const double *eps,
                           const double *mu, int precision, int nrhs, const double *KN, int ldkn,
                           const double *rhs, int ldr, double *pscat, double *pext);

/* ---- cache of the static near-pair integrals ----------------------------------
 * Replaces PreloadCache / StoreCache (libscuff.h:662-663) and reads and writes
 * their file format (FIPPICache.cc:195-400: "FIPPICACHE" + records of a
 * 15-float key and the reference's QIFIPPIData), so a cache written by the
 * reference warms this library's near field and the other way round.  The
 * cache is process-wide, like the reference's GlobalFIPPICache: preloaded
 * records are used by every later cold near-field pass (pairs not found are
 * computed as usual); gbem_cache_store writes the preloaded records and the
 * tables of every live geometry whose near field has been computed. */
gbem_status gbem_cache_preload(const char *path);
gbem_status gbem_cache_store(const char *path);
gbem_status gbem_cache_clear(void);
gbem_status gbem_cache_size(long long *nrecords);
/* near pairs of g (common-triangle pairs excepted) found / not found in the
 * cache (host only; no GPU needed) */
gbem_status gbem_cache_lookup_stats(const gbem_geometry *g, long long *hits, long long *misses);

/* ---- shape derivatives (adjoint) -------------------------------------------
 * No reference counterpart: the reference differentiates rigid motions of
 * whole surfaces only (GradM, dMdT of AssembleBEMMatrixBlock, libscuff.h:500-505).
 * Vertices are numbered surface by surface (surface 0's first); grad holds
 * 3 doubles per vertex and is overwritten.
 *
 * gbem_vertex_vjp_matrix: grad[3 v + c] = Re sum_r sum_ij conj(lam_ir)
 * dM_ij/dV_vc x_jr for the full matrix of gbem_assemble at this frequency;
 * lam, x: N x nrhs complex128 (host, column-major).  Far pairs are
 * differentiated analytically; near and common-vertex pairs by central
 * differences of their FP64 evaluation with displacement rel_step times the
 * pair's larger panel radius (1e-4 keeps both truncation and rounding near
 * 1e-9 of the derivative). */
gbem_status gbem_vertex_vjp_matrix(gbem_geometry *g, double omega_re, double omega_im, const double *eps,
                                   const double *mu, int nrhs, const double *lam, int ldl, const double *x,
                                   int ldx, double rel_step, double *grad);
/* gbem_vertex_vjp_matrix for one region's matrix alone, with the signs of an
 * exterior region (KK = i mu w GC0, KN = NK = -i k GC1, NN = -i eps w GC0):
 * region 0 gives the matrix of the EMT scattered power's quadratic form
 * (gbem_power_emt), whose explicit shape derivative this contracts. */
gbem_status gbem_vertex_vjp_region(gbem_geometry *g, double omega_re, double omega_im, const double *eps,
                                   const double *mu, int region, int nrhs, const double *lam, int ldl,
                                   const double *x, int ldx, double rel_step, double *grad);
/* Gradient of gbem_power_emt's scattered power with respect to the solution
 * vectors: G[:, r] = dP_r/dRe KN[:, r] + i dP_r/dIm KN[:, r] (FP64; host
 * N x nrhs complex128; nrhs <= 8).  No reference counterpart (the shape
 * derivative of absorbed power). */
gbem_status gbem_power_emt_grad(gbem_geometry *g, double omega_re, double omega_im, const double *eps,
                                const double *mu, int nrhs, const double *KN, int ldkn, double *G, int ldg);
/* grad[3 v + c] = Re sum_w sum_i conj(gb_iw) d b_iw/dV_vc for the plane-wave
 * right-hand sides of gbem_rhs_planewave (E0: 6 doubles, nhat: 3 per wave). */
gbem_status gbem_vertex_vjp_rhs_planewave(gbem_geometry *g, double omega_re, double omega_im, const double *eps,
                                          const double *mu, int nwaves, const double *E0, const double *nhat,
                                          const double *gb, int ldg, double *grad);
/* total vertices over all surfaces */
gbem_status gbem_geometry_num_vertices(const gbem_geometry *g, int *nv);

/* ---- right-hand sides ----------------------------------------------------- */
/* Plane-wave right-hand side (AssembleRHSVector.cc:145-255 with a PlaneWave
 * incident field, libs/libIncField/PlaneWave.cc): E0 (complex, 6 doubles),
 * nhat (3 doubles); writes N complex128 entries to host rhs. */
gbem_status gbem_rhs_planewave(gbem_geometry *g, double omega_re, double omega_im,
                               const double *eps, const double *mu,
                               const double *E0, const double *nhat, double *rhs);

#ifdef __cplusplus
}
#endif
#endif /* GBEM_H */
