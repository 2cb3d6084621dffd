/*
 * cpg_colored.cuh -- the graph-coloured solver mode for large spaces.
 *
 * Broadphase: sweep-and-prune over the dynamic shapes.  Each shape's AABB
 * left edge, rounded down to float, is the sort key; the order (key, shape
 * index) is repaired from the previous step's or rebuilt by a stable radix
 * sort (k_sap_sort).  The sweep from shape i visits the following
 * shapes while their key is <= i's right edge rounded up, and keeps the
 * pairs whose double-precision boxes intersect (cpBBIntersects, cpBB.h:47).
 * Rounding the keys outward keeps the sweep exact: a pair whose boxes
 * overlap always has the later key <= the earlier box's rounded-up right
 * edge.  Shapes on static bodies are found by querying the device static
 * AABB tree.  The resulting pair set equals the set of pairs the
 * reference's tree hands to cpSpaceCollideShapes that pass its box test
 * (cpSpaceStep.c:219-232).
 *
 * Colouring: units (arbiters, joints) that share a dynamic body conflict.
 * Rounds of Jones-Plassmann selection with hashed priorities pick
 * independent sets; each selected unit takes the lowest colour free on both
 * of its bodies (64-bit per-body masks).  Units of one colour run in
 * parallel; colours run in sequence.  The sweep order therefore differs
 * from the reference's, and results are judged by residual and
 * penetration, not bit agreement.
 */
#pragma once
#include <cooperative_groups.h>
#include "cpg_device.h"
#include "cpg_math.cuh"

namespace cg = cooperative_groups;

__device__ __forceinline__ unsigned float_order_key(float f)
{
	unsigned u = __float_as_uint(f);
	return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

/* Exclusive scan of `n` counts by one block.  Each thread takes a
 * contiguous run of ceil(n / blockDim) counts: it sums them, the block
 * scans the per-thread sums once, and the thread writes its run's
 * prefixes.  Two block barriers in all, whatever n. */
__global__ void k_scan_excl(unsigned *data, int n, unsigned *total)
{
	__shared__ unsigned warpSums[32];
	int t = threadIdx.x, lane = t & 31, warp = t >> 5, nwarps = blockDim.x >> 5;
	int per = (n + (int)blockDim.x - 1)/(int)blockDim.x;
	int i0 = min(n, t*per), i1 = min(n, i0 + per);
	unsigned sum = 0;
	for(int i = i0; i < i1; i++) sum += data[i];
	unsigned x = sum;
	for(int o = 1; o < 32; o <<= 1){
		unsigned y = __shfl_up_sync(0xffffffffu, x, o);
		if(lane >= o) x += y;
	}
	if(lane == 31) warpSums[warp] = x;
	__syncthreads();
	if(warp == 0){
		unsigned s = (lane < nwarps) ? warpSums[lane] : 0u;
		for(int o = 1; o < 32; o <<= 1){
			unsigned y = __shfl_up_sync(0xffffffffu, s, o);
			if(lane >= o) s += y;
		}
		if(lane < nwarps) warpSums[lane] = s;
	}
	__syncthreads();
	unsigned run = ((warp > 0) ? warpSums[warp - 1] : 0u) + x - sum;
	for(int i = i0; i < i1; i++){
		unsigned v = data[i];
		data[i] = run;
		run += v;
	}
	if(t == (int)blockDim.x - 1 && total) *total = run;
}

/* ---- sweep-and-prune ----
 *
 * Box tests run on ordered integer images of the doubles: -0 is folded to
 * +0 and negative values have their magnitude bits inverted, so that
 * okey(a) <= okey(b) exactly when a <= b for every non-NaN pair.  The
 * cpBBIntersects test (cpBB.h:47) then takes integer compares instead of
 * FP64 compares, which issue at a small fraction of the integer rate on
 * this part. */
__device__ __forceinline__ long long okey(double x)
{
	long long b = __double_as_longlong(x);
	if(b == (long long)0x8000000000000000ull) b = 0;
	return b < 0 ? (b ^ 0x7FFFFFFFFFFFFFFFll) : b;
}

struct KBB { long long l, b, r, t; };

__device__ __forceinline__ KBB kbb(double l, double b, double r, double t)
{
	KBB k; k.l = okey(l); k.b = okey(b); k.r = okey(r); k.t = okey(t);
	return k;
}

__device__ __forceinline__ bool kbb_intersects(const KBB &a, const KBB &b)
{
	return a.l <= b.r && b.l <= a.r && a.b <= b.t && b.b <= a.t;
}

struct SapCtx {
	const unsigned *keys;     /* sorted left-edge keys */
	const int *vals;          /* sorted shape indices (world-local) */
	const unsigned *rkeys;    /* right-edge keys by shape */
	const longlong4_32a *sbb; /* box keys (okey of l, b, r, t) in sorted order */
	int n;                    /* dynamic shapes */
};

__device__ __forceinline__ KBB gshape_kbb(const cpgSet &s, int g) { return kbb(s.bbl[g], s.bbb[g], s.bbr[g], s.bbt[g]); }

/* Static-tree hits of sorted shape i (one thread). */
template<class F>
__device__ void sap_static(const cpgSet &s, const cpgWorld &W, const cpgTree &T, const SapCtx &c, int i, F f)
{
	if(T.statRoot < 0) return;
	int sa = c.vals[i];
	KBB ba = gshape_kbb(s, W.shapeOff + sa);
	const cpgNode *nodes = s.nodes + W.nodeOff;
	int stack[64];
	int sp = 0;
	stack[sp++] = T.statRoot;
	while(sp > 0){
		int nidx = stack[--sp];
		const cpgNode &nd = nodes[nidx];
		if(!kbb_intersects(kbb(nd.l, nd.b, nd.r, nd.t), ba)) continue;
		if(nd.obj >= 0){
			if(kbb_intersects(ba, gshape_kbb(s, W.shapeOff + nd.obj))) f(sa, nd.obj);
		} else if(sp + 2 <= 64){
			stack[sp++] = nd.B;
			stack[sp++] = nd.A;
		}
	}
}

/* Sweep of sorted shape i by one warp: lane l tests box i+1+l, i+33+l, ...
 * while keys stay <= the shape's high key (keys are sorted, so the first
 * lane past the bound ends the sweep).  f(lane_rank, total, hit, a, b) is
 * called once per 32-box window by every lane; hits are ranked in box
 * order, so output positions are deterministic. */
template<class F>
__device__ void sap_sweep_warp(const SapCtx &c, int i, const KBB &ba, int sa, F f)
{
	int lane = threadIdx.x & 31;
	unsigned rk = c.rkeys[sa];
	for(int j0 = i + 1; j0 < c.n; j0 += 32){
		int j = j0 + lane;
		bool inside = (j < c.n) && (c.keys[j] <= rk);
		bool hit = false;
		int sb = -1;
		if(inside){
			longlong4_32a bj = c.sbb[j];
			KBB kb; kb.l = bj.x; kb.b = bj.y; kb.r = bj.z; kb.t = bj.w;
			hit = kbb_intersects(ba, kb);
			if(hit) sb = c.vals[j];
		}
		unsigned hits = __ballot_sync(0xffffffffu, hit);
		f(__popc(hits & ((1u << lane) - 1u)), __popc(hits), hit, sa, sb);
		if(__ballot_sync(0xffffffffu, inside) != 0xffffffffu) break;
	}
}
