// Host check of the solver's integer clamps (chipmunk2d_gb300/csrc/cpg_math.cuh):
// dmax0, dclamp_sym and dgt_bits must return, bit for bit, what the FP64
// compares of cpfmax / cpfclamp (chipmunk_types.h:137-168) return, for
// special values (signed zeros, denormals, infinities, NaNs of both signs)
// and for random bit patterns and random impulses.
// Prints one line and exits non-zero on a failure.
#define __device__
#define __host__
#define __forceinline__ inline
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>
#include "cpg_math.cuh"

static unsigned long long rng_state = 0x2545F4914F6CDD1Dull;
static unsigned long long next_bits()
{
	rng_state ^= rng_state << 13; rng_state ^= rng_state >> 7; rng_state ^= rng_state << 17;
	return rng_state;
}

static long long bits_of(double x) { long long b; memcpy(&b, &x, sizeof(b)); return b; }

/* the reference's definitions, as compares */
static double ref_max(double a, double b) { return (a > b) ? a : b; }
static double ref_min(double a, double b) { return (a < b) ? a : b; }
static double ref_clamp(double f, double lo, double hi) { return ref_min(ref_max(f, lo), hi); }

static long failures = 0, cases = 0;

static void check_pair(double f, double m)
{
	cases++;
	if(bits_of(dclamp_sym(f, m)) != bits_of(ref_clamp(f, -m, m))){
		if(failures < 10) printf("  FAIL clamp(%a, %a): %a vs %a\n", f, m, dclamp_sym(f, m), ref_clamp(f, -m, m));
		failures++;
	}
	if(dgt_bits(f, m) != (f > m)){
		if(failures < 10) printf("  FAIL gt(%a, %a)\n", f, m);
		failures++;
	}
}

static void check_one(double x)
{
	cases++;
	if(bits_of(dmax0(x)) != bits_of(ref_max(x, 0.0))){
		if(failures < 10) printf("  FAIL max0(%a): %a vs %a\n", x, dmax0(x), ref_max(x, 0.0));
		failures++;
	}
}

int main()
{
	std::vector<double> special = {
		0.0, -0.0, 1.0, -1.0, 0.5, -0.5, 2.0, -2.0, 1e-300, -1e-300,
		4.9e-324, -4.9e-324, 2.2250738585072014e-308, -2.2250738585072014e-308,
		1.7976931348623157e308, -1.7976931348623157e308, INFINITY, -INFINITY,
		NAN, -NAN, 3.0, -3.0, 1e10, -1e10,
	};
	double qnan_payload; long long qb = 0x7FF8000000000123ll; memcpy(&qnan_payload, &qb, 8);
	double snan; long long sb = 0x7FF0000000000001ll; memcpy(&snan, &sb, 8);
	double nnan; long long nb = (long long)0xFFF0000000000001ull; memcpy(&nnan, &nb, 8);
	special.push_back(qnan_payload); special.push_back(snan); special.push_back(nnan);
	/* neighbours of each value */
	size_t n0 = special.size();
	for(size_t i = 0; i < n0; i++){
		double x = special[i];
		if(std::isfinite(x)){ special.push_back(nextafter(x, INFINITY)); special.push_back(nextafter(x, -INFINITY)); }
	}
	for(double f : special){
		check_one(f);
		for(double m : special) check_pair(f, m);
	}
	/* equal magnitudes with both signs, and m near f */
	for(int i = 0; i < 200000; i++){
		double m = ldexp((double)(next_bits() >> 11)*(1.0/9007199254740992.0), (int)(next_bits()%80) - 40);
		double f = (next_bits() & 1) ? m : -m;
		if(next_bits() & 2) f = nextafter(f, (next_bits() & 4) ? INFINITY : -INFINITY);
		check_pair(f, m);
		check_one(f);
	}
	/* random bit patterns */
	for(int i = 0; i < 2000000; i++){
		long long a = (long long)next_bits(), b = (long long)next_bits();
		double f, m; memcpy(&f, &a, 8); memcpy(&m, &b, 8);
		check_pair(f, m);
		check_one(f);
		double mpos = fabs(m);
		check_pair(f, mpos);
	}
	/* impulses as the solver sees them */
	for(int i = 0; i < 2000000; i++){
		double old = (double)(next_bits() >> 11)*(1.0/9007199254740992.0)*10.0;
		double j = ((double)(next_bits() >> 11)*(1.0/9007199254740992.0) - 0.5)*20.0;
		double acc = dmax0(old + j);
		check_one(old + j);
		double u = (double)(next_bits() >> 11)*(1.0/9007199254740992.0);
		double jt = ((double)(next_bits() >> 11)*(1.0/9007199254740992.0) - 0.5)*20.0;
		check_pair(jt, u*acc);
	}
	printf("integer clamps: %ld cases, %ld mismatches\n", cases, failures);
	return failures ? 1 : 0;
}
