// Host shim for compiling CUDA-style user hook files (and, for the pinned
// reference build, the reference's per-thread solver header) with g++.
//
// TEST INFRASTRUCTURE ONLY: used by the CPU oracle and by the CPU build of the
// reference under oracle/_ref. Nothing in the product links this.
#pragma once

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <algorithm>

#define __device__
#define __host__
#define __forceinline__ inline

using std::abs;
using std::cos;
using std::fabs;
using std::isfinite;
using std::pow;
using std::sin;
using std::sqrt;

#ifndef MPGOS_HOST_PI
#define MPGOS_HOST_PI 3.14159265358979323846
#endif

// sincospi has no glibc counterpart; sin(pi x), cos(pi x) by definition.
inline void sincospi(double x, double* s, double* c)
{
    *s = std::sin(MPGOS_HOST_PI * x);
    *c = std::cos(MPGOS_HOST_PI * x);
}
inline void sincospi(float x, float* s, float* c)
{
    *s = std::sin(static_cast<float>(MPGOS_HOST_PI) * x);
    *c = std::cos(static_cast<float>(MPGOS_HOST_PI) * x);
}
