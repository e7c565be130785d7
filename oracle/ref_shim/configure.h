/* Stand-in for the reference's generated configure.h (configure.h.in): only
 * the two macros its header-only face kernels read.  Used by oracle/Makefile
 * to compile those headers, unmodified, into oracle/_ref/libsnapref.so. */
#pragma once
#define NMASS 0
#ifdef __CUDACC__
#define DISPATCH_MACRO __host__ __device__
#else
#define DISPATCH_MACRO
#endif
