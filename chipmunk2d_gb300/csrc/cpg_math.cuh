/*
 * cpg_math.cuh -- FP64 vector helpers for the device code.
 *
 * Every helper evaluates the same expression tree, in the same order, as
 * the reference's inline math (include/chipmunk/cpVect.h:35-225,
 * cpBB.h:35-190, cpTransform.h:30-140, chipmunk_types.h:137-168), and the
 * library is compiled with --fmad=false, so each operation rounds exactly
 * as the host code does.  cpfmin/cpfmax are comparisons, not fmin/fmax.
 */
#pragma once
#include <cfloat>
#include <cstring>

struct V2 { double x, y; };

__device__ __forceinline__ V2 v2(double x, double y) { V2 r; r.x = x; r.y = y; return r; }
__device__ __forceinline__ V2 vadd(V2 a, V2 b) { return v2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ V2 vsub(V2 a, V2 b) { return v2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ V2 vneg(V2 a) { return v2(-a.x, -a.y); }
__device__ __forceinline__ V2 vmul(V2 a, double s) { return v2(a.x*s, a.y*s); }
__device__ __forceinline__ double vdot(V2 a, V2 b) { return a.x*b.x + a.y*b.y; }
__device__ __forceinline__ double vcross(V2 a, V2 b) { return a.x*b.y - a.y*b.x; }
__device__ __forceinline__ V2 vperp(V2 a) { return v2(-a.y, a.x); }
__device__ __forceinline__ V2 vrperp(V2 a) { return v2(a.y, -a.x); }
__device__ __forceinline__ V2 vrotate(V2 a, V2 b) { return v2(a.x*b.x - a.y*b.y, a.x*b.y + a.y*b.x); }
__device__ __forceinline__ double vlensq(V2 a) { return vdot(a, a); }
__device__ __forceinline__ double vlen(V2 a) { return sqrt(vdot(a, a)); }
__device__ __forceinline__ V2 vnormalize(V2 a) { return vmul(a, 1.0/(vlen(a) + DBL_MIN)); }
__device__ __forceinline__ V2 vlerp(V2 a, V2 b, double t) { return vadd(vmul(a, 1.0 - t), vmul(b, t)); }
__device__ __forceinline__ bool veql(V2 a, V2 b) { return a.x == b.x && a.y == b.y; }

__device__ __forceinline__ double dmax(double a, double b) { return (a > b) ? a : b; }
__device__ __forceinline__ double dmin(double a, double b) { return (a < b) ? a : b; }
__device__ __forceinline__ double dabs(double f) { return (f < 0) ? -f : f; }
__device__ __forceinline__ double dclamp(double f, double lo, double hi) { return dmin(dmax(f, lo), hi); }
__device__ __forceinline__ double dclamp01(double f) { return dmax(0.0, dmin(f, 1.0)); }
__device__ __forceinline__ V2 vclamp(V2 v, double len) { return (vdot(v, v) > len*len) ? vmul(vnormalize(v), len) : v; }

/* ---- the solver's clamps on the bit patterns ----
 * A DSETP takes the FP64 pipe like a multiply, and the contact iteration
 * needs three per contact (cpfmax(jn, 0) and the friction cone's
 * cpfclamp, cpArbiter.c:486-492).  These return what the compares return,
 * for every input including NaN and signed zeros, with integer compares
 * and selects only. */
__device__ __forceinline__ long long dbits(double x)
{
#ifdef __CUDA_ARCH__
	return __double_as_longlong(x);
#else
	long long b; memcpy(&b, &x, sizeof(b)); return b;
#endif
}
__device__ __forceinline__ double dfrombits(long long b)
{
#ifdef __CUDA_ARCH__
	return __longlong_as_double(b);
#else
	double x; memcpy(&x, &b, sizeof(x)); return x;
#endif
}
#define CPG_DBL_SIGN ((long long)0x8000000000000000ull)
#define CPG_DBL_INF 0x7FF0000000000000ll

/* a > b as IEEE compares it: false when either is NaN, -0 equal to +0.
 * Ordered images: -0 folds to +0, negative magnitudes are inverted. */
__device__ __forceinline__ bool dgt_bits(double a, double b)
{
	long long x = dbits(a), y = dbits(b);
	bool nan = ((x & ~CPG_DBL_SIGN) > CPG_DBL_INF) || ((y & ~CPG_DBL_SIGN) > CPG_DBL_INF);
	if(x == CPG_DBL_SIGN) x = 0;
	if(y == CPG_DBL_SIGN) y = 0;
	x = (x < 0) ? (x ^ ~CPG_DBL_SIGN) : x;
	y = (y < 0) ? (y ^ ~CPG_DBL_SIGN) : y;
	return !nan && x > y;
}

/* cpfmax(x, 0.0): x when x > 0, else +0.  The doubles above zero (NaN
 * excluded) are exactly the bit patterns in (0, +inf]. */
__device__ __forceinline__ double dmax0(double x)
{
	long long b = dbits(x);
	return (b > 0 && b <= CPG_DBL_INF) ? x : 0.0;
}

/* cpfclamp(f, -m, m) = cpfmin(cpfmax(f, -m), m).  For m in [+0, +inf]:
 * f when |f| < m; otherwise m, or -m when m > 0 and f is negative or NaN
 * (NaN fails f > -m).  Any other m takes the general compares. */
__device__ __forceinline__ double dclamp_sym(double f, double m)
{
	long long mb = dbits(m), fb = dbits(f);
	double negm = dfrombits(mb ^ CPG_DBL_SIGN);
	if(mb < 0 || mb > CPG_DBL_INF){
		double t = dgt_bits(f, negm) ? f : negm;
		return dgt_bits(m, t) ? t : m;
	}
	long long fmag = fb & ~CPG_DBL_SIGN;
	if(fmag < mb) return f;
	bool low = (fb < 0) || (fmag > CPG_DBL_INF);
	return (mb != 0 && low) ? negm : m;
}

struct BB { double l, b, r, t; };
__device__ __forceinline__ BB bbnew(double l, double b, double r, double t) { BB o; o.l = l; o.b = b; o.r = r; o.t = t; return o; }
__device__ __forceinline__ bool bbintersects(BB a, BB b) { return (a.l <= b.r && b.l <= a.r && a.b <= b.t && b.b <= a.t); }
__device__ __forceinline__ bool bbcontains(BB bb, BB o) { return (bb.l <= o.l && bb.r >= o.r && bb.b <= o.b && bb.t >= o.t); }
__device__ __forceinline__ BB bbmerge(BB a, BB b) { return bbnew(dmin(a.l, b.l), dmin(a.b, b.b), dmax(a.r, b.r), dmax(a.t, b.t)); }
__device__ __forceinline__ double bbarea(BB a) { return (a.r - a.l)*(a.t - a.b); }
__device__ __forceinline__ double bbmergedarea(BB a, BB b) { return (dmax(a.r, b.r) - dmin(a.l, b.l))*(dmax(a.t, b.t) - dmin(a.b, b.b)); }
__device__ __forceinline__ double bbproximity(BB a, BB b) { return dabs(a.l + a.r - b.l - b.r) + dabs(a.b + a.t - b.b - b.t); }
__device__ __forceinline__ V2 bbcenter(BB bb) { return vlerp(v2(bb.l, bb.b), v2(bb.r, bb.t), 0.5); }

#define CPG_HASH_COEF 3344921057ull
__device__ __forceinline__ unsigned long long hash_pair(unsigned long long a, unsigned long long b)
{
	return a*CPG_HASH_COEF ^ b*CPG_HASH_COEF;
}
