/*
 * Stand-in for MATLAB's mex.h, used only to compile the reference sampler
 * (source/c/LibRJMCMC.cpp) outside MATLAB as a test oracle.  The sampler
 * uses two MEX calls: mexPrintf (diagnostics on caught exceptions and odd
 * prior lookups) and mexEvalString("drawnow;").  Messages are counted by the
 * driver so a test can see whether any were raised.
 */
#ifndef BAMF_ORACLE_STUB_MEX_H
#define BAMF_ORACLE_STUB_MEX_H
#include <stdio.h>
#ifdef __cplusplus
extern "C" {
#endif
int bamf_ref_mex_printf(const char *fmt, ...);
static inline int mexEvalString(const char *s) { (void)s; return 0; }
#ifdef __cplusplus
}
#endif
#define mexPrintf bamf_ref_mex_printf
#endif
