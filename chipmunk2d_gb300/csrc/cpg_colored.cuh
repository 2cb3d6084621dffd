/*
 * cpg_colored.cuh -- the graph-coloured solver mode for large spaces.
 *
 * Broadphase: sweep-and-prune over the dynamic shapes.  Each shape's AABB
 * left edge, rounded down to float, is the sort key (LSD radix sort, 8-bit
 * digits, stable multi-block).  The sweep from shape i visits the following
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

#define RS_THREADS 256
#define RS_ITEMS 8
#define RS_TILE (RS_THREADS*RS_ITEMS)

__device__ __forceinline__ unsigned float_order_key(float f)
{
	unsigned u = __float_as_uint(f);
	return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

/* Per-digit counts of one tile; hist is digit-major: hist[d*nblocks + b]. */
__global__ void k_rs_hist(const unsigned *keys, int n, int shift, unsigned *hist)
{
	__shared__ unsigned h[256];
	h[threadIdx.x] = 0;
	__syncthreads();
	int base = blockIdx.x*RS_TILE;
	for(int k = 0; k < RS_ITEMS; k++){
		int i = base + k*RS_THREADS + threadIdx.x;
		if(i < n) atomicAdd(&h[(keys[i] >> shift) & 0xFF], 1u);
	}
	__syncthreads();
	hist[threadIdx.x*gridDim.x + blockIdx.x] = h[threadIdx.x];
}

/* Exclusive scan of `n` counts by one block. */
__global__ void k_scan_excl(unsigned *data, int n, unsigned *total)
{
	__shared__ unsigned warpSums[32];
	__shared__ unsigned carry;
	if(threadIdx.x == 0) carry = 0;
	__syncthreads();
	int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
	for(int c0 = 0; c0 < n; c0 += blockDim.x){
		int i = c0 + threadIdx.x;
		unsigned v = (i < n) ? data[i] : 0u;
		unsigned x = v;
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
		unsigned warpPrefix = (warp > 0) ? warpSums[warp - 1] : 0u;
		if(i < n) data[i] = carry + warpPrefix + x - v;
		__syncthreads();
		if(threadIdx.x == 0) carry += warpSums[nwarps - 1];
		__syncthreads();
	}
	if(threadIdx.x == 0 && total) *total = carry;
}

/* Stable scatter of one tile: item order is round-major, then thread. */
__global__ void k_rs_scatter(const unsigned *kin, const int *vin, unsigned *kout, int *vout, int n, int shift, const unsigned *hist)
{
	__shared__ unsigned base[256];
	__shared__ unsigned roundTotal[256];
	__shared__ unsigned warpCount[RS_THREADS/32][256];
	int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	base[threadIdx.x] = hist[threadIdx.x*gridDim.x + blockIdx.x];
	int tile = blockIdx.x*RS_TILE;
	for(int k = 0; k < RS_ITEMS; k++){
		for(int w = 0; w < RS_THREADS/32; w++) warpCount[w][threadIdx.x] = 0;
		__syncthreads();
		int i = tile + k*RS_THREADS + threadIdx.x;
		bool valid = i < n;
		unsigned key = valid ? kin[i] : 0u;
		unsigned d = valid ? ((key >> shift) & 0xFF) : 256u;
		unsigned peers = __match_any_sync(0xffffffffu, d);
		unsigned rank = __popc(peers & ((1u << lane) - 1u));
		if(valid && rank == 0) warpCount[warp][d] = __popc(peers);
		__syncthreads();
		{
			unsigned s = 0;
			for(int w = 0; w < RS_THREADS/32; w++){ unsigned t = warpCount[w][threadIdx.x]; warpCount[w][threadIdx.x] = s; s += t; }
			roundTotal[threadIdx.x] = s;
		}
		__syncthreads();
		if(valid){
			unsigned pos = base[d] + warpCount[warp][d] + rank;
			kout[pos] = key;
			vout[pos] = vin[i];
		}
		__syncthreads();
		base[threadIdx.x] += roundTotal[threadIdx.x];
		__syncthreads();
	}
}

/* ---- sweep-and-prune ---- */

struct SapCtx {
	const unsigned *keys;     /* sorted left-edge keys */
	const int *vals;          /* sorted shape indices (world-local) */
	const unsigned *rkeys;    /* right-edge keys by shape */
	const double4_32a *sbb;   /* boxes in sorted order */
	int n;                    /* dynamic shapes */
};

__device__ __forceinline__ BB gshape_bb(const cpgSet &s, int g) { return bbnew(s.bbl[g], s.bbb[g], s.bbr[g], s.bbt[g]); }

/* Static-tree hits of sorted shape i (one thread). */
template<class F>
__device__ void sap_static(const cpgSet &s, const cpgWorld &W, const cpgTree &T, const SapCtx &c, int i, F f)
{
	if(T.statRoot < 0) return;
	int sa = c.vals[i];
	BB ba = gshape_bb(s, W.shapeOff + sa);
	const cpgNode *nodes = s.nodes + W.nodeOff;
	int stack[64];
	int sp = 0;
	stack[sp++] = T.statRoot;
	while(sp > 0){
		int nidx = stack[--sp];
		const cpgNode &nd = nodes[nidx];
		if(!bbintersects(bbnew(nd.l, nd.b, nd.r, nd.t), ba)) continue;
		if(nd.obj >= 0){
			if(bbintersects(ba, gshape_bb(s, W.shapeOff + nd.obj))) f(sa, nd.obj);
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
__device__ void sap_sweep_warp(const SapCtx &c, int i, BB ba, int sa, F f)
{
	int lane = threadIdx.x & 31;
	unsigned rk = c.rkeys[sa];
	for(int j0 = i + 1; j0 < c.n; j0 += 32){
		int j = j0 + lane;
		bool inside = (j < c.n) && (c.keys[j] <= rk);
		bool hit = false;
		int sb = -1;
		if(inside){
			double4_32a bj = c.sbb[j];
			hit = bbintersects(ba, bbnew(bj.x, bj.y, bj.z, bj.w));
			if(hit) sb = c.vals[j];
		}
		unsigned hits = __ballot_sync(0xffffffffu, hit);
		f(__popc(hits & ((1u << lane) - 1u)), __popc(hits), hit, sa, sb);
		if(__ballot_sync(0xffffffffu, inside) != 0xffffffffu) break;
	}
}
