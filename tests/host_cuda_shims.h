// Host stand-ins for the CUDA qualifiers and intrinsics that the device
// tree code (chipmunk2d_gb300/csrc/cpg_tree.cuh, cpg_mark.cuh) uses, so that
// tests can compile it for the host.  The directed-rounding intrinsics are
// built from round-to-nearest operations and an exact error term, so they
// do not depend on the host's rounding mode or on the compiler keeping
// operations in order around a rounding-mode change.
#pragma once
#define __device__
#define __host__
#define __forceinline__ inline
#define __constant__
#include <cmath>
#include <cstring>
static inline long long __double_as_longlong(double x) { long long b; memcpy(&b, &x, sizeof(b)); return b; }
static inline float __uint_as_float(unsigned u) { float f; memcpy(&f, &u, sizeof(f)); return f; }

// x rounded to a float downwards / upwards (x exact as a double)
static inline float host_down(double x) { float r = (float)x; return ((double)r > x) ? std::nextafterf(r, -INFINITY) : r; }
static inline float host_up(double x) { float r = (float)x; return ((double)r < x) ? std::nextafterf(r, INFINITY) : r; }
static inline float __double2float_rd(double x) { return std::isnan(x) ? (float)x : host_down(x); }
static inline float __double2float_ru(double x) { return std::isnan(x) ? (float)x : host_up(x); }
// products of two floats are exact in double
static inline float __fmul_rd(float a, float b) { return host_down((double)a*(double)b); }
static inline float __fmul_ru(float a, float b) { return host_up((double)a*(double)b); }
// sums: the rounded sum and its exact error (TwoSum, round to nearest)
static inline void host_two_sum(float a, float b, float &s, float &e)
{
	volatile float vs = a + b;
	s = vs;
	volatile float bb = s - a;
	e = (a - (s - bb)) + (b - bb);
}
static inline float __fadd_rd(float a, float b)
{
	float s, e; host_two_sum(a, b, s, e);
	if(std::isinf(s) || std::isnan(s)) return s;
	return e < 0.0f ? std::nextafterf(s, -INFINITY) : s;
}
static inline float __fadd_ru(float a, float b)
{
	float s, e; host_two_sum(a, b, s, e);
	if(std::isinf(s) || std::isnan(s)) return s;
	return e > 0.0f ? std::nextafterf(s, INFINITY) : s;
}
static inline float __fsub_rd(float a, float b) { return __fadd_rd(a, -b); }
static inline float __fsub_ru(float a, float b) { return __fadd_ru(a, -b); }
