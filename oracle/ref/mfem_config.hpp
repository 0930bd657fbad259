// Hand-written configuration header for building the unmodified MFEM sources
// as a serial, CPU-only, double-precision library. It supplies the handful of
// macros that MFEM's config/config.hpp expects from its configuration step
// (MFEM_CONFIG_FILE hook, config/config.hpp:20-24); every optional third-party
// package is left disabled. OpenMP is enabled when the Makefile passes
// -DGB_REF_OPENMP so that Device("omp") can use every host core.
#ifndef MFEM_CONFIG_HEADER
#define MFEM_CONFIG_HEADER
#define MFEM_VERSION 40901
#define MFEM_VERSION_STRING "4.9.1"
#define MFEM_VERSION_TYPE ((MFEM_VERSION)%2)
#define MFEM_VERSION_TYPE_RELEASE 0
#define MFEM_VERSION_TYPE_DEVELOPMENT 1
#define MFEM_VERSION_MAJOR ((MFEM_VERSION)/10000)
#define MFEM_VERSION_MINOR (((MFEM_VERSION)/100)%100)
#define MFEM_VERSION_PATCH ((MFEM_VERSION)%100)
#define MFEM_SOURCE_DIR "reference"
#define MFEM_INSTALL_DIR "unused"
#define MFEM_GIT_STRING "(unknown)"
#define MFEM_USE_DOUBLE
#define MFEM_USE_MEMALLOC
#define MFEM_TIMER_TYPE 2
#ifdef GB_REF_OPENMP
#define MFEM_USE_OPENMP
#endif
#endif
