/*
 * Stand-in for the CUDA 4.0 SDK's cutil_inline.h, which the reference's host
 * sources include through kernel/cuda_header.h.  Only oracle/_ref uses it: the
 * host sources are compiled for the CPU, so the error-check macros pass their
 * argument through and the timers are no-ops.  Test infrastructure.
 */
#ifndef ORACLE_SHIM_CUTIL_INLINE_H
#define ORACLE_SHIM_CUTIL_INLINE_H
#include <stdio.h>
#define cutilSafeCall(x) (x)
#define cutilCheckMsg(x) ((void)0)
#define CUT_SAFE_CALL(x) (x)
static inline int cutCreateTimer(unsigned int*) { return 0; }
static inline int cutStartTimer(unsigned int) { return 0; }
static inline int cutStopTimer(unsigned int) { return 0; }
static inline int cutDeleteTimer(unsigned int) { return 0; }
static inline float cutGetTimerValue(unsigned int) { return 0.f; }
#endif
