/* The reference's Casimir driver declares dgetrf_/zgetrf_ itself
   (CasimirIntegrand.cc:39-42) instead of going through F77_FUNC; scipy's
   bundled OpenBLAS exports them with a scipy_ prefix.  Forwarders only. */
int scipy_dgetrf_(int *m, int *n, double *a, int *lda, int *ipiv, int *info);
int scipy_zgetrf_(int *m, int *n, void *a, int *lda, int *ipiv, int *info);
int dgetrf_(int *m, int *n, double *a, int *lda, int *ipiv, int *info) { return scipy_dgetrf_(m, n, a, lda, ipiv, info); }
int zgetrf_(int *m, int *n, void *a, int *lda, int *ipiv, int *info) { return scipy_zgetrf_(m, n, a, lda, ipiv, info); }
