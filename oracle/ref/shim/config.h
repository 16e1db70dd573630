/* Hand-written stand-in for the autoconf-generated config.h of the reference
 * build (used only to compile the reference sources into the test oracle).
 * LAPACK/BLAS symbols resolve to scipy's bundled LP64 OpenBLAS, whose exported
 * names carry a "scipy_" prefix. */
#ifndef GBEM_REF_CONFIG_H
#define GBEM_REF_CONFIG_H
#define HAVE_CXX11 1
#define USE_OPENMP 1
#define F77_FUNC(name,NAME) scipy_##name##_
#define F77_FUNC_(name,NAME) scipy_##name##_
#define PACKAGE_VERSION "0.96"
#define VERSION "0.96"
#endif
