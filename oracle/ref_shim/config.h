/* Minimal build configuration for compiling a few of the reference's header-only
 * spline sources in place (oracle/build_ref.sh); test infrastructure only. */
#ifndef QMCG_REF_SHIM_CONFIG_H
#define QMCG_REF_SHIM_CONFIG_H
#define OHMMS_DIM 3
#define OHMMS_INDEXTYPE int
#define OHMMS_PRECISION double
#define OHMMS_PRECISION_FULL double
#define QMC_SIMD_ALIGNMENT 64
#define HAVE_POSIX_MEMALIGN 1
#endif
