/* Hand-written stand-in for the reference's configure-time header.
 * The reference fills this in with CMake (config.h.cmake.in); the oracle
 * recipe runs no CMake and supplies the few facts the hot-path sources read.
 * Test infrastructure only: nothing in the product includes it. */
#ifndef ODE_CONFIG_H
#define ODE_CONFIG_H
#define HAVE_ALLOCA_H 1
#define HAVE_GETTIMEOFDAY 1
#define HAVE_INTTYPES_H 1
#define HAVE_ISNAN 1
#define HAVE_ISNANF 1
#define HAVE_MALLOC_H 1
#define HAVE_STDINT_H 1
#define HAVE_SYS_TIME_H 1
#define HAVE_SYS_TYPES_H 1
#define HAVE_UNISTD_H 1
#if defined(__linux__)
#define ODE_PLATFORM_LINUX
#else
#error "oracle reference build supports Linux only"
#endif
#include <alloca.h>
#include <malloc.h>
#include <stdint.h>
#include <inttypes.h>
#include "typedefs.h"
#endif
