// Host check of the AABB tree's float brackets (chipmunk2d_gb300/csrc/
// cpg_tree.cuh).  Every decision the brackets settle must equal the one
// taken on the doubles:
//   - f32_bracket(x) gives floats lo <= x <= hi;
//   - bmin/bmax/bmerge return the same doubles (bit for bit) as
//     tmin/tmax/tmerge, and the merged brackets enclose the merged box;
//   - the insertion cost test: when the FP32 intervals of the two costs
//     are apart, the side they pick is the side the double costs pick.
// Inputs: uniform boxes, boxes one to three double ulps apart, exact ties
// (mirrored boxes), signed zeros, float-subnormal and out-of-float-range
// magnitudes.  Prints the counts and " N wrong"; exits non-zero if N > 0.
#include <cstdio>
#include <cstdlib>
#include <vector>
#include "host_cuda_shims.h"
#include "cpg_tree.cuh"

static unsigned long long rng = 0x2545F4914F6CDD1Dull;
static unsigned long long next_u64()
{
	rng ^= rng << 13; rng ^= rng >> 7; rng ^= rng << 17;
	return rng;
}
static double urand() { return (double)(next_u64() >> 11)*(1.0/9007199254740992.0); }

static double ulp_step(double x, int k)
{
	for(int i = 0; i < k; i++) x = std::nextafter(x, INFINITY);
	for(int i = 0; i > k; i--) x = std::nextafter(x, -INFINITY);
	return x;
}

/* a coordinate from one of several regimes */
static double coord(int regime)
{
	switch(regime){
		case 0: return (urand() - 0.5)*4000.0;
		case 1: return (double)(float)((urand() - 0.5)*4000.0);          // exactly a float
		case 2: return (urand() - 0.5)*1e-39;                              // float-subnormal range
		case 3: return (urand() - 0.5)*1e40;                               // beyond float range
		case 4: return (next_u64() & 1) ? 0.0 : -0.0;
		default: return (urand() - 0.5)*8.0;
	}
}

static bool same_bits(double a, double b) { return memcmp(&a, &b, sizeof(double)) == 0; }

static BB make_box(int regime)
{
	double x0 = coord(regime), y0 = coord(regime);
	double w = std::fabs(coord(regime == 4 ? 5 : regime))*(next_u64() & 3 ? 0.01 : 1.0);
	double h = std::fabs(coord(regime == 4 ? 5 : regime))*(next_u64() & 3 ? 0.01 : 1.0);
	if(next_u64() % 8 == 0) w = 0.0;
	return bbnew(x0, y0, x0 + w, y0 + h);
}

/* a box close to another: each coordinate moved by -3..3 ulps, kept valid */
static BB near_box(BB a)
{
	BB b = bbnew(ulp_step(a.l, (int)(next_u64() % 7) - 3), ulp_step(a.b, (int)(next_u64() % 7) - 3),
	             ulp_step(a.r, (int)(next_u64() % 7) - 3), ulp_step(a.t, (int)(next_u64() % 7) - 3));
	if(b.r < b.l) b.r = b.l;
	if(b.t < b.b) b.t = b.b;
	return b;
}

int main()
{
	long long wrong = 0, cmp = 0, certain = 0, exactPath = 0, merges = 0;
	/* brackets and comparisons */
	for(int it = 0; it < 2000000; it++){
		int regime = (int)(next_u64() % 6);
		double a = coord(regime);
		double b = (next_u64() & 1) ? ulp_step(a, (int)(next_u64() % 7) - 3) : coord(regime);
		float alo, ahi, blo, bhi;
		f32_bracket(a, alo, ahi);
		f32_bracket(b, blo, bhi);
		if(!((double)alo <= a && a <= (double)ahi) || !((double)blo <= b && b <= (double)bhi)){
			if(wrong < 10) printf("bracket %.17g -> [%.9g, %.9g]\n", a, alo, ahi);
			wrong++;
		}
		cmp++;
		if(!same_bits(bmin(a, alo, ahi, b, blo, bhi), tmin(a, b)) ||
		   !same_bits(bmax(a, alo, ahi, b, blo, bhi), tmax(a, b))){
			if(wrong < 10) printf("min/max %.17g %.17g\n", a, b);
			wrong++;
		}
	}
	/* merges and the insertion cost test */
	for(int it = 0; it < 1000000; it++){
		int regime = (int)(next_u64() % 6);
		BB A = make_box(regime), L = make_box(regime), B;
		int kind = (int)(next_u64() % 4);
		if(kind == 0) B = near_box(A);
		else if(kind == 1){
			/* B mirrors A about L's centre: equal costs, the tie-break decides */
			double cx = L.l + L.r, cy = L.b + L.t;
			B = bbnew(cx - A.r, cy - A.t, cx - A.l, cy - A.b);
			if(B.r < B.l || B.t < B.b) B = A;
		} else B = make_box(regime);
		FBox fa = fbox_of(A), fb = fbox_of(B), fl = fbox_of(L);
		BB m; FBox fm;
		bmerge(A, fa, L, fl, m, fm);
		BB t = tmerge(A, L);
		merges++;
		if(!same_bits(m.l, t.l) || !same_bits(m.b, t.b) || !same_bits(m.r, t.r) || !same_bits(m.t, t.t) ||
		   !((double)fm.llo <= m.l && m.l <= (double)fm.lhi) || !((double)fm.blo <= m.b && m.b <= (double)fm.bhi) ||
		   !((double)fm.rlo <= m.r && m.r <= (double)fm.rhi) || !((double)fm.tlo <= m.t && m.t <= (double)fm.thi)){
			if(wrong < 10) printf("merge\n");
			wrong++;
		}
		/* the decision of subtree_insert, both ways */
		float aLo, aHi, bLo, bHi, maLo, maHi, mbLo, mbHi;
		fbox_area(fa, aLo, aHi);
		fbox_area(fb, bLo, bHi);
		fmerged_area(fa, fl, maLo, maHi);
		fmerged_area(fb, fl, mbLo, mbHi);
		float caLo = __fadd_rd(bLo, maLo), caHi = __fadd_ru(bHi, maHi);
		float cbLo = __fadd_rd(aLo, mbLo), cbHi = __fadd_ru(aHi, mbHi);
		double cost_a = bbarea(B) + tmergedarea(A, L);
		double cost_b = bbarea(A) + tmergedarea(B, L);
		bool tie = (tkey(cost_a) == tkey(cost_b));
		bool exactB = tie ? (tkey(bbproximity(B, L)) < tkey(bbproximity(A, L))) : (tkey(cost_b) < tkey(cost_a));
		if(cbHi < caLo){
			certain++;
			if(tie || !exactB){ if(wrong < 10) printf("cost: B certain, doubles %.17g %.17g\n", cost_a, cost_b); wrong++; }
		} else if(caHi < cbLo){
			certain++;
			if(tie || exactB){ if(wrong < 10) printf("cost: A certain, doubles %.17g %.17g\n", cost_a, cost_b); wrong++; }
		} else {
			exactPath++;
		}
	}
	printf("%lld comparisons, %lld merges, %lld cost tests settled in FP32, %lld by doubles; %lld wrong\n",
	       cmp, merges, certain, exactPath, wrong);
	return wrong ? 1 : 0;
}
