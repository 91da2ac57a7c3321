/*
 * Forced include (-include) for building the UNMODIFIED reference sampler
 * source/c/LibRJMCMC.cpp as a CPU oracle.  It does two things, both by
 * preprocessor renaming after the standard headers are in, so the reference
 * source text is compiled as is:
 *
 *  1. rand -> bamf_ref_rand: the reference draws every uniform through
 *     urand() = (float)rand()/((float)RAND_MAX+1) (LibRJMCMCreturn.hpp:17)
 *     from glibc's never-seeded global rand().  The driver feeds it the
 *     Philox stream of include/bamf_philox.h instead, so the GPU sampler can
 *     consume the very same uniforms.
 *
 *  2. (only with -DBAMF_REF_PARITY_MATH) erf/log/exp/pow on float arguments
 *     -> the project's parity math (include/bamf_parity_math.h), so the
 *     oracle's float results do not depend on glibc's last-ulp behaviour.
 *     The double overloads are deleted: the reference never calls them on
 *     the sampler path, and a compile error would say so if it did.
 */
#ifndef BAMF_REF_SHIM_H
#define BAMF_REF_SHIM_H
#include <cmath>
#include <math.h>
#include <stdlib.h>
#include <stdio.h>
#include <vector>
#include <stdexcept>

extern "C" int bamf_ref_rand(void);
#define rand bamf_ref_rand

#ifdef BAMF_REF_PARITY_MATH
#include "bamf_parity_math.h"
static inline float bamf_ref_erf(float x) { return bamf_pm_erff(x); }
double bamf_ref_erf(double) = delete;
static inline float bamf_ref_log(float x) { return bamf_pm_logf(x); }
double bamf_ref_log(double) = delete;
static inline float bamf_ref_exp(float x) { return bamf_pm_expf(x); }
double bamf_ref_exp(double) = delete;
static inline double bamf_ref_pow(float x, int n) { return bamf_pm_pow_fi(x, n); }
static inline float bamf_ref_pow(float x, float y) { return bamf_pm_powf(x, y); }
double bamf_ref_pow(double, double) = delete;
double bamf_ref_pow(double, int) = delete;
#define erf bamf_ref_erf
#define log bamf_ref_log
#define exp bamf_ref_exp
#define pow bamf_ref_pow
#endif

#endif
