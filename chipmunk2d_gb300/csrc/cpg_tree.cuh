/*
 * cpg_tree.cuh -- device mirror of the reference's incremental AABB tree
 * (src/cpBBTree.c) for one world, run by one thread (the containment
 * scan of the leaves, which has no order to keep, by the whole block).
 *
 * The tree, its per-leaf pair cache and the leaf hash set determine the
 * order in which cpSpaceStep visits shape pairs, and that order is the
 * Gauss-Seidel order of the solver.  The GPU path reproduces it exactly by
 * keeping the same incremental structure on the device: the same insertion
 * cost function and tie-breaks (cpBBTree.c:325-350), the same pair
 * threading (:150-205), the same marking traversal (:418-480) and the same
 * leaf re-index order (hash-bin order, src/cpHashSet.c:87-229).
 * Recursion is replaced by explicit stacks; node and pair pools are
 * world-local index ranges with LIFO free lists.
 *
 * The traversal only *emits* candidate pairs (cpgCand) in visit order; the
 * narrow phase then runs on all candidates in parallel, which is exact
 * because the reference's query callback never modifies the tree.
 */
#pragma once
#include "cpg_device.h"
#include "cpg_math.cuh"

#define CPG_STACK 512

struct TreeCtx {
	cpgNode *nodes;
	cpgPair *pairs;
	int nodeCap, pairCap;
	cpgTree *T;
	int *dbins, *sbins;
	int dbinCap, sbinCap;
	/* shape data, world base */
	const double *bbl, *bbb, *bbr, *bbt;
	const int *sbody;
	const unsigned long long *shash;
	const double *vx, *vy;   /* body velocity, world base */
	/* candidate output */
	cpgCand *cands;
	int candCap;
	int ncand;
	int collide;            /* 1: emit candidates; 0: the void query */
};

/* Comparisons on ordered integer images of the doubles: -0 folds to +0
 * and negative magnitudes are inverted, so tkey(a) < tkey(b) exactly when
 * a < b for every non-NaN pair.  The tree runs on one thread per world and
 * its box tests, min and max would each be an FP64 instruction (64 cycles
 * of the sub-partition's FP64 pipe, shared with the other worlds' threads);
 * as integer compares and selects they return the same values. */
__device__ __forceinline__ long long tkey(double x)
{
	long long b = __double_as_longlong(x);
	if(b == (long long)0x8000000000000000ull) b = 0;
	return b < 0 ? (b ^ 0x7FFFFFFFFFFFFFFFll) : b;
}
__device__ __forceinline__ double tmin(double a, double b) { return (tkey(a) < tkey(b)) ? a : b; }
__device__ __forceinline__ double tmax(double a, double b) { return (tkey(a) > tkey(b)) ? a : b; }
__device__ __forceinline__ bool tintersects(BB a, BB b)
{
	return tkey(a.l) <= tkey(b.r) && tkey(b.l) <= tkey(a.r) && tkey(a.b) <= tkey(b.t) && tkey(b.b) <= tkey(a.t);
}
__device__ __forceinline__ bool tcontains(BB bb, BB o)
{
	return tkey(bb.l) <= tkey(o.l) && tkey(bb.r) >= tkey(o.r) && tkey(bb.b) <= tkey(o.b) && tkey(bb.t) >= tkey(o.t);
}
__device__ __forceinline__ BB tmerge(BB a, BB b) { return bbnew(tmin(a.l, b.l), tmin(a.b, b.b), tmax(a.r, b.r), tmax(a.t, b.t)); }
__device__ __forceinline__ double tmergedarea(BB a, BB b) { return (tmax(a.r, b.r) - tmin(a.l, b.l))*(tmax(a.t, b.t) - tmin(a.b, b.b)); }

/* ---- float brackets of the boxes ----
 * A node keeps, beside each double coordinate x, the floats rounded down
 * and up from it (lo <= x <= hi, equal when x is a float).  Rounding is
 * monotone, so lo(min(a, b)) = min(lo(a), lo(b)) and likewise for hi and
 * max: a merged box's brackets are min/max of its children's, with no
 * conversion.  The brackets decide most comparisons and the insertion
 * cost test in FP32 (full rate), and only near-ties fall back to the exact
 * doubles.  The decisions are the exact ones: a_hi < b_lo implies a < b;
 * and a cost computed in doubles, each operation rounded to nearest,
 * lies inside the FP32 interval computed with the rounding directed
 * outwards, because a double rounded to nearest stays between any two
 * floats that bracket the exact value. */
struct FBox { float llo, lhi, blo, bhi, rlo, rhi, tlo, thi; };

__device__ __forceinline__ BB node_bb(const cpgNode &n) { return bbnew(n.l, n.b, n.r, n.t); }
__device__ __forceinline__ FBox node_fbox(const cpgNode &n)
{
	FBox f;
	f.llo = n.llo; f.lhi = n.lhi; f.blo = n.blo; f.bhi = n.bhi;
	f.rlo = n.rlo; f.rhi = n.rhi; f.tlo = n.tlo; f.thi = n.thi;
	return f;
}
__device__ __forceinline__ void set_node_box(cpgNode &n, BB bb, FBox f)
{
	n.l = bb.l; n.b = bb.b; n.r = bb.r; n.t = bb.t;
	n.llo = f.llo; n.lhi = f.lhi; n.blo = f.blo; n.bhi = f.bhi;
	n.rlo = f.rlo; n.rhi = f.rhi; n.tlo = f.tlo; n.thi = f.thi;
}

/* x rounded down (lo) and up (hi) to floats.  In the normal float range
 * by bit arithmetic: the truncated mantissa is the magnitude rounded
 * towards zero, and one more unit in its last place (a carry runs into
 * the exponent) the magnitude rounded away from zero; elsewhere (zero,
 * float-subnormal, out of range, NaN) by the conversion intrinsics. */
__device__ __forceinline__ void f32_bracket(double x, float &lo, float &hi)
{
	unsigned long long u = (unsigned long long)__double_as_longlong(x);
	unsigned h = (unsigned)(u >> 32);
	int e = (int)((h >> 20) & 0x7FFu);
	if(e < 1023 - 126 || e > 1023 + 127){
		lo = __double2float_rd(x);
		hi = __double2float_ru(x);
		return;
	}
	unsigned sign = h & 0x80000000u;
	unsigned mag = ((unsigned)(e - 1023 + 127) << 23) | (unsigned)((u >> 29) & 0x7FFFFFu);
	float tz = __uint_as_float(sign | mag);
	if((u & 0x1FFFFFFFull) == 0ull){ lo = hi = tz; return; }
	float away = __uint_as_float(sign | (mag + 1u));
	if(sign){ lo = away; hi = tz; } else { lo = tz; hi = away; }
}

__device__ __forceinline__ FBox fbox_of(BB bb)
{
	FBox f;
	f32_bracket(bb.l, f.llo, f.lhi); f32_bracket(bb.b, f.blo, f.bhi);
	f32_bracket(bb.r, f.rlo, f.rhi); f32_bracket(bb.t, f.tlo, f.thi);
	return f;
}

__device__ __forceinline__ void set_node_bb(cpgNode &n, BB bb) { set_node_box(n, bb, fbox_of(bb)); }

/* tmin/tmax decided by the brackets when they are apart */
__device__ __forceinline__ double bmin(double a, float alo, float ahi, double b, float blo, float bhi)
{
	if(ahi < blo) return a;
	if(bhi < alo) return b;
	return tmin(a, b);
}
__device__ __forceinline__ double bmax(double a, float alo, float ahi, double b, float blo, float bhi)
{
	if(alo > bhi) return a;
	if(blo > ahi) return b;
	return tmax(a, b);
}

__device__ __forceinline__ bool same_box_bits(BB a, BB b)
{
	return __double_as_longlong(a.l) == __double_as_longlong(b.l) && __double_as_longlong(a.b) == __double_as_longlong(b.b) &&
	       __double_as_longlong(a.r) == __double_as_longlong(b.r) && __double_as_longlong(a.t) == __double_as_longlong(b.t);
}

/* tmerge(a, b) and the merged brackets */
__device__ __forceinline__ void bmerge(BB a, const FBox &fa, BB b, const FBox &fb, BB &m, FBox &fm)
{
	m.l = bmin(a.l, fa.llo, fa.lhi, b.l, fb.llo, fb.lhi);
	m.b = bmin(a.b, fa.blo, fa.bhi, b.b, fb.blo, fb.bhi);
	m.r = bmax(a.r, fa.rlo, fa.rhi, b.r, fb.rlo, fb.rhi);
	m.t = bmax(a.t, fa.tlo, fa.thi, b.t, fb.tlo, fb.thi);
	fm.llo = fminf(fa.llo, fb.llo); fm.lhi = fminf(fa.lhi, fb.lhi);
	fm.blo = fminf(fa.blo, fb.blo); fm.bhi = fminf(fa.bhi, fb.bhi);
	fm.rlo = fmaxf(fa.rlo, fb.rlo); fm.rhi = fmaxf(fa.rhi, fb.rhi);
	fm.tlo = fmaxf(fa.tlo, fb.tlo); fm.thi = fmaxf(fa.thi, fb.thi);
}

/* Interval of bbarea over a box's brackets.  A box whose width or height
 * may be negative gets the unbounded interval (its cost test then runs
 * in doubles). */
__device__ __forceinline__ void farea(float llo, float lhi, float blo, float bhi,
                                      float rlo, float rhi, float tlo, float thi, float &lo, float &hi)
{
	float wlo = __fsub_rd(rlo, lhi), whi = __fsub_ru(rhi, llo);
	float hlo = __fsub_rd(tlo, bhi), hhi = __fsub_ru(thi, blo);
	if(wlo >= 0.0f && hlo >= 0.0f){
		lo = __fmul_rd(wlo, hlo);
		hi = __fmul_ru(whi, hhi);
	} else {
		lo = -INFINITY; hi = INFINITY;
	}
}
__device__ __forceinline__ void fbox_area(const FBox &f, float &lo, float &hi)
{
	farea(f.llo, f.lhi, f.blo, f.bhi, f.rlo, f.rhi, f.tlo, f.thi, lo, hi);
}
/* interval of tmergedarea(a, b) */
__device__ __forceinline__ void fmerged_area(const FBox &a, const FBox &b, float &lo, float &hi)
{
	farea(fminf(a.llo, b.llo), fminf(a.lhi, b.lhi), fminf(a.blo, b.blo), fminf(a.bhi, b.bhi),
	      fmaxf(a.rlo, b.rlo), fmaxf(a.rhi, b.rhi), fmaxf(a.tlo, b.tlo), fmaxf(a.thi, b.thi), lo, hi);
}
__device__ __forceinline__ bool is_leaf(const TreeCtx &c, int n) { return c.nodes[n].obj >= 0; }

__device__ __forceinline__ BB shape_bb(const TreeCtx &c, int s) { return bbnew(c.bbl[s], c.bbb[s], c.bbr[s], c.bbt[s]); }

/* cpBBTree.c:82-98: dynamic leaves are fattened by 10% of their size plus
 * 0.1 s of their body's velocity (both factors are the float literal 0.1f). */
__device__ BB fatten(BB bb, V2 vel)
{
	const double coef = (double)0.1f;
	double x = (bb.r - bb.l)*coef;
	double y = (bb.t - bb.b)*coef;
	V2 v = vmul(vel, (double)0.1f);
	return bbnew(bb.l + tmin(-x, v.x), bb.b + tmin(-y, v.y), bb.r + tmax(x, v.x), bb.t + tmax(y, v.y));
}

__device__ BB leaf_fat_bb(const TreeCtx &c, int s)
{
	int body = c.sbody[s];
	return fatten(shape_bb(c, s), v2(c.vx[body], c.vy[body]));
}

__device__ int node_alloc(TreeCtx &c)
{
	cpgTree *T = c.T;
	if(T->freeNode >= 0){
		int n = T->freeNode;
		T->freeNode = c.nodes[n].parent;
		return n;
	}
	if(T->nodeTop >= c.nodeCap){ T->error |= CPG_ERR_NODES; return -1; }
	return T->nodeTop++;
}

__device__ __forceinline__ void node_recycle(TreeCtx &c, int n)
{
	c.nodes[n].parent = c.T->freeNode;
	c.T->freeNode = n;
}

__device__ int pair_alloc(TreeCtx &c)
{
	cpgTree *T = c.T;
	if(T->freePair >= 0){
		int p = T->freePair;
		T->freePair = c.pairs[p].aNext;
		return p;
	}
	if(T->pairTop >= c.pairCap){ T->error |= CPG_ERR_PAIRS; return -1; }
	return T->pairTop++;
}

/* pad marks a pool slot live (1) or free (0) */
__device__ __forceinline__ void pair_recycle(TreeCtx &c, int p)
{
	c.pairs[p].pad = 0;
	c.pairs[p].aNext = c.T->freePair;
	c.T->freePair = p;
	c.T->pairsLive--;
}

/* cpBBTree.c:150-165 */
__device__ void thread_unlink(TreeCtx &c, int prev, int leaf, int next)
{
	if(next >= 0){
		cpgPair &np = c.pairs[next];
		if(np.aLeaf == leaf) np.aPrev = prev; else np.bPrev = prev;
	}
	if(prev >= 0){
		cpgPair &pp = c.pairs[prev];
		if(pp.aLeaf == leaf) pp.aNext = next; else pp.bNext = next;
	} else {
		c.nodes[leaf].pairs = next;
	}
}

/* cpBBTree.c:167-186 */
__device__ void pairs_clear(TreeCtx &c, int leaf)
{
	int p = c.nodes[leaf].pairs;
	c.nodes[leaf].pairs = -1;
	for(int guard = 0; p >= 0; guard++){
		if(guard > c.pairCap){ c.T->error |= CPG_ERR_PAIRS; return; }
		cpgPair pr = c.pairs[p];
		int next;
		if(pr.aLeaf == leaf){
			next = pr.aNext;
			thread_unlink(c, pr.bPrev, pr.bLeaf, pr.bNext);
		} else {
			next = pr.bNext;
			thread_unlink(c, pr.aPrev, pr.aLeaf, pr.aNext);
		}
		pair_recycle(c, p);
		p = next;
	}
}

/* cpBBTree.c:188-205 */
__device__ void pair_insert(TreeCtx &c, int a, int b)
{
	int nextA = c.nodes[a].pairs, nextB = c.nodes[b].pairs;
	int p = pair_alloc(c);
	if(p < 0) return;
	c.T->pairsLive++;
	cpgPair &pr = c.pairs[p];
	pr.aPrev = -1; pr.aLeaf = a; pr.aNext = nextA;
	pr.bPrev = -1; pr.bLeaf = b; pr.bNext = nextB;
	pr.id = 0;
	pr.pad = 1;
	c.nodes[a].pairs = p;
	c.nodes[b].pairs = p;
	if(nextA >= 0){
		cpgPair &q = c.pairs[nextA];
		if(q.aLeaf == a) q.aPrev = p; else q.bPrev = p;
	}
	if(nextB >= 0){
		cpgPair &q = c.pairs[nextB];
		if(q.aLeaf == b) q.aPrev = p; else q.bPrev = p;
	}
}

/* A node's box and links in registers. */
struct NodeRec {
	BB bb;
	FBox f;
	int parent, A, B, obj;
};

__device__ __forceinline__ NodeRec node_rec(const TreeCtx &c, int n)
{
	const cpgNode &nd = c.nodes[n];
	NodeRec r;
	r.bb = node_bb(nd);
	r.f = node_fbox(nd);
	r.parent = nd.parent; r.A = nd.A; r.B = nd.B; r.obj = nd.obj;
	return r;
}

/* cpBBTree.c:250-267, with the children's boxes passed in */
__device__ int node_new_bb(TreeCtx &c, int a, BB abb, const FBox &fa, int b, BB bbb, const FBox &fb)
{
	int n = node_alloc(c);
	if(n < 0) return -1;
	cpgNode &nd = c.nodes[n];
	nd.obj = -1;
	BB m; FBox fm;
	bmerge(abb, fa, bbb, fb, m, fm);
	set_node_box(nd, m, fm);
	nd.parent = -1;
	nd.A = a; c.nodes[a].parent = n;
	nd.B = b; c.nodes[b].parent = n;
	nd.pairs = -1; nd.binNext = -1; nd.stamp = 0;
	return n;
}

__device__ int node_new(TreeCtx &c, int a, int b)
{
	const cpgNode &na = c.nodes[a], &nb = c.nodes[b];
	return node_new_bb(c, a, node_bb(na), node_fbox(na), b, node_bb(nb), node_fbox(nb));
}

/* cpBBTree.c:281-299.  The refit from the parent up to the root is one
 * round of dependent loads per level: the child just refitted is known,
 * so a level loads its sibling's box and the next parent's links at once
 * (merged in the reference's A, B order). */
__device__ void node_replace_child(TreeCtx &c, int parent, int child, int value)
{
	cpgNode &pn = c.nodes[parent];
	BB fromBB = node_bb(c.nodes[value]);
	FBox fromF = node_fbox(c.nodes[value]);
	if(pn.A == child){
		node_recycle(c, pn.A);
		pn.A = value; c.nodes[value].parent = parent;
	} else {
		node_recycle(c, pn.B);
		pn.B = value; c.nodes[value].parent = parent;
	}
	int from = value, n = parent;
	int a = pn.A, b = pn.B, up = pn.parent;
	BB cur = node_bb(pn);
	for(int guard = 0;; guard++){
		if(guard > c.nodeCap){ c.T->error |= CPG_ERR_NODES; return; }
		bool fromA = (a == from);
		const cpgNode &sn = c.nodes[fromA ? b : a];
		BB sbb = node_bb(sn);
		FBox sf = node_fbox(sn);
		int na = -1, nb = -1, nup = -1;
		BB ncur = cur;
		if(up >= 0){
			const cpgNode &un = c.nodes[up];
			na = un.A; nb = un.B; nup = un.parent;
			ncur = node_bb(un);
		}
		BB m; FBox fm;
		if(fromA) bmerge(fromBB, fromF, sbb, sf, m, fm);
		else bmerge(sbb, sf, fromBB, fromF, m, fm);
		/* A box the refit leaves as it was ends the walk: every node's box
		 * is the merge of its children's (insertion merges the leaf into
		 * each box on its path, a refit recomputes it), so the ancestors'
		 * recomputed boxes equal their present ones.  Equal in value; the
		 * bits could differ only in the sign of a zero coordinate, which
		 * the comparisons fold and no cost, area or proximity turns into
		 * a different decision. */
		if(same_box_bits(m, cur)) return;
		set_node_box(c.nodes[n], m, fm);
		if(up < 0) return;
		from = n; fromBB = m; fromF = fm; n = up;
		a = na; b = nb; up = nup; cur = ncur;
	}
}

/* cpBBTree.c:325-350, iterative.  The reference merges each visited
 * node's box on the way back up; a node's own box is only read by its
 * parent's cost test, which has already run, so merging on the way down
 * gives the same tree and boxes.  Both children's records are loaded at
 * each level, so the chosen child's links are already in registers and
 * the descent costs one round of dependent loads per level. */
__device__ int subtree_insert(TreeCtx &c, int root, int leaf)
{
	if(root < 0) return leaf;
	NodeRec nd = node_rec(c, root);
	if(nd.obj >= 0) return node_new(c, leaf, root);
	const cpgNode &ln = c.nodes[leaf];
	BB lbb = node_bb(ln);
	FBox lf = node_fbox(ln);
	int cur = root;
	for(int guard = 0;; guard++){
		if(guard > c.nodeCap){ c.T->error |= CPG_ERR_NODES; return root; }
		NodeRec ra = node_rec(c, nd.A), rb = node_rec(c, nd.B);
		/* the cost test on intervals; doubles only when they overlap */
		float aLo, aHi, bLo, bHi, maLo, maHi, mbLo, mbHi;
		fbox_area(ra.f, aLo, aHi);
		fbox_area(rb.f, bLo, bHi);
		fmerged_area(ra.f, lf, maLo, maHi);
		fmerged_area(rb.f, lf, mbLo, mbHi);
		float caLo = __fadd_rd(bLo, maLo), caHi = __fadd_ru(bHi, maHi);
		float cbLo = __fadd_rd(aLo, mbLo), cbHi = __fadd_ru(aHi, mbHi);
		bool goB;
		if(cbHi < caLo) goB = true;
		else if(caHi < cbLo) goB = false;
		else {
			BB abb = ra.bb, bbb = rb.bb;
			double cost_a = bbarea(bbb) + tmergedarea(abb, lbb);
			double cost_b = bbarea(abb) + tmergedarea(bbb, lbb);
			if(tkey(cost_a) == tkey(cost_b)){
				cost_a = bbproximity(abb, lbb);
				cost_b = bbproximity(bbb, lbb);
			}
			goB = (tkey(cost_b) < tkey(cost_a));
		}
		int child = goB ? nd.B : nd.A;
		NodeRec rc = goB ? rb : ra;
		/* a box whose brackets already hold the leaf's strictly inside is
		 * its own merge with the leaf: nothing to compute or store */
		bool inside = nd.f.lhi < lf.llo && nd.f.bhi < lf.blo && nd.f.rlo > lf.rhi && nd.f.tlo > lf.thi;
		if(!inside){
			BB m; FBox fm;
			bmerge(nd.bb, nd.f, lbb, lf, m, fm);
			if(!same_box_bits(m, nd.bb)) set_node_box(c.nodes[cur], m, fm);
		}
		if(rc.obj >= 0){
			int nn = node_new_bb(c, leaf, lbb, lf, child, rc.bb, rc.f);
			if(nn < 0) return root;
			if(goB) c.nodes[cur].B = nn; else c.nodes[cur].A = nn;
			c.nodes[nn].parent = cur;
			return root;
		}
		cur = child;
		nd = rc;
	}
}

/* cpBBTree.c:397-415 */
__device__ int subtree_remove(TreeCtx &c, int root, int leaf)
{
	if(leaf == root) return -1;
	int parent = c.nodes[leaf].parent;
	if(parent == root){
		int other = (c.nodes[root].A == leaf ? c.nodes[root].B : c.nodes[root].A);
		c.nodes[other].parent = c.nodes[root].parent;
		node_recycle(c, root);
		return other;
	}
	int other = (c.nodes[parent].A == leaf ? c.nodes[parent].B : c.nodes[parent].A);
	node_replace_child(c, c.nodes[parent].parent, parent, other);
	return root;
}

__device__ __forceinline__ void emit(TreeCtx &c, int a, int b, int pair, unsigned id)
{
	if(c.ncand >= c.candCap){ c.T->error |= CPG_ERR_CANDS; return; }
	cpgCand cd; cd.a = a; cd.b = b; cd.pair = pair; cd.idIn = id;
	c.cands[c.ncand++] = cd;
}

/* cpBBTree.c:425-441 (MarkLeafQuery), depth-first A before B. */
__device__ void mark_leaf_query(TreeCtx &c, int subtree, int leaf, bool left)
{
	int stack[CPG_STACK];
	int sp = 0;
	stack[sp++] = subtree;
	BB lbb = node_bb(c.nodes[leaf]);
	while(sp > 0){
		int n = stack[--sp];
		const cpgNode &nd = c.nodes[n];
		if(!tintersects(lbb, node_bb(nd))) continue;
		if(nd.obj >= 0){
			if(left){
				pair_insert(c, leaf, n);
			} else {
				if(nd.stamp < c.nodes[leaf].stamp) pair_insert(c, n, leaf);
				if(c.collide) emit(c, c.nodes[leaf].obj, nd.obj, -1, 0u);
			}
		} else {
			if(sp + 2 > CPG_STACK){ c.T->error |= CPG_ERR_NODES; return; }
			stack[sp++] = nd.B;
			stack[sp++] = nd.A;
		}
	}
}

/* cpBBTree.c:443-469 */
__device__ void mark_leaf(TreeCtx &c, int leaf, int staticRoot)
{
	if(c.nodes[leaf].stamp == c.T->treeStamp){
		if(staticRoot >= 0) mark_leaf_query(c, staticRoot, leaf, false);
		int guard = 0;
		for(int n = leaf; c.nodes[n].parent >= 0; n = c.nodes[n].parent){
			if(++guard > c.nodeCap){ c.T->error |= CPG_ERR_NODES; return; }
			int parent = c.nodes[n].parent;
			if(n == c.nodes[parent].A){
				mark_leaf_query(c, c.nodes[parent].B, leaf, true);
			} else {
				mark_leaf_query(c, c.nodes[parent].A, leaf, false);
			}
		}
	} else {
		int p = c.nodes[leaf].pairs;
		for(int guard = 0; p >= 0; guard++){
			if(guard > c.pairCap){ c.T->error |= CPG_ERR_PAIRS; return; }
			const cpgPair &pr = c.pairs[p];
			if(leaf == pr.bLeaf){
				if(c.collide) emit(c, c.nodes[pr.aLeaf].obj, c.nodes[leaf].obj, p, pr.id);
				p = pr.bNext;
			} else {
				p = pr.aNext;
			}
		}
	}
}

/* cpBBTree.c:471-480 */
__device__ void mark_subtree(TreeCtx &c, int root, int staticRoot)
{
	int stack[CPG_STACK];
	int sp = 0;
	stack[sp++] = root;
	while(sp > 0){
		int n = stack[--sp];
		const cpgNode &nd = c.nodes[n];
		if(nd.obj >= 0){
			mark_leaf(c, n, staticRoot);
		} else {
			if(sp + 2 > CPG_STACK){ c.T->error |= CPG_ERR_NODES; return; }
			stack[sp++] = nd.B;
			stack[sp++] = nd.A;
		}
	}
}

/* src/prime.h:25-55: the leaf set's table sizes, roughly doubling primes. */
__device__ __constant__ int cpg_primes[] = {
	5, 13, 23, 47, 97, 193, 389, 769, 1543, 3079, 6151, 12289, 24593, 49157,
	98317, 196613, 393241, 786433, 1572869, 3145739, 6291469, 12582917,
	25165843, 50331653, 100663319, 201326611, 402653189, 805306457, 1610612741, 0,
};

__device__ unsigned next_prime_dev(unsigned n)
{
	int i = 0;
	while(n > (unsigned)cpg_primes[i] && cpg_primes[i + 1]) i++;
	return (unsigned)cpg_primes[i];
}

/* cpHashSet.c:87-114: rehash into next_prime(size + 1) bins, walking the
 * old bins in order and pushing each leaf on the head of its new chain. */
__device__ bool leafset_resize(TreeCtx &c, int *bins, int binCap, unsigned *size)
{
	unsigned newSize = next_prime_dev(*size + 1);
	if((int)newSize > binCap){ c.T->error |= CPG_ERR_BINS; return false; }
	int head = -1, tail = -1;
	int guard = 0;
	for(unsigned i = 0; i < *size; i++){
		int n = bins[i];
		while(n >= 0){
			if(++guard > c.nodeCap){ c.T->error |= CPG_ERR_BINS; return false; }
			int next = c.nodes[n].binNext;
			if(tail >= 0) c.nodes[tail].binNext = n; else head = n;
			tail = n;
			n = next;
		}
	}
	if(tail >= 0) c.nodes[tail].binNext = -1;
	for(unsigned i = 0; i < newSize; i++) bins[i] = -1;
	guard = 0;
	for(int n = head; n >= 0;){
		if(++guard > c.nodeCap){ c.T->error |= CPG_ERR_BINS; return false; }
		int next = c.nodes[n].binNext;
		unsigned idx = (unsigned)(c.shash[c.nodes[n].obj] % newSize);
		c.nodes[n].binNext = bins[idx];
		bins[idx] = n;
		n = next;
	}
	*size = newSize;
	return true;
}

/* cpBBTree.c:605-616 with LeafAddPairs (:521-537) and the leaf-set insert
 * (cpHashSet.c:152-176). */
__device__ void tree_insert(TreeCtx &c, const cpgOp &op)
{
	cpgTree *T = c.T;
	int shape = op.shape;
	bool isStatic = op.isStatic != 0;
	int leaf = node_alloc(c);
	if(leaf < 0) return;
	cpgNode &nd = c.nodes[leaf];
	nd.obj = shape;
	BB bb = bbnew(op.l, op.b, op.r, op.t);
	set_node_bb(nd, isStatic ? bb : fatten(bb, v2(op.vx, op.vy)));
	nd.parent = -1; nd.A = -1; nd.B = -1;
	nd.stamp = 0;
	nd.pairs = -1;
	int *bins = isStatic ? c.sbins : c.dbins;
	unsigned *size = isStatic ? &T->statSize : &T->dynSize;
	unsigned *entries = isStatic ? &T->statEntries : &T->dynEntries;
	unsigned idx = (unsigned)(c.shash[shape] % *size);
	nd.binNext = bins[idx];
	bins[idx] = leaf;
	(*entries)++;
	if(*entries >= *size) leafset_resize(c, bins, isStatic ? c.sbinCap : c.dbinCap, size);

	if(isStatic){
		T->statRoot = subtree_insert(c, T->statRoot, leaf);
		c.nodes[leaf].stamp = T->treeStamp;
		if(T->dynRoot >= 0) mark_leaf_query(c, T->dynRoot, leaf, true);
	} else {
		T->dynRoot = subtree_insert(c, T->dynRoot, leaf);
		c.nodes[leaf].stamp = T->treeStamp;
		mark_leaf(c, leaf, T->statRoot);
	}
	T->treeStamp++;
}

/* cpBBTree.c:619-630 (cpBBTreeRemove): the leaf leaves the hash set
 * (cpHashSet.c:209-233: unlinked from its bin, the other leaves keep
 * their order), then the tree, then every pair list, and is recycled. */
__device__ void tree_remove(TreeCtx &c, const cpgOp &op)
{
	cpgTree *T = c.T;
	int shape = op.shape;
	bool isStatic = op.isStatic != 0;
	int *bins = isStatic ? c.sbins : c.dbins;
	unsigned size = isStatic ? T->statSize : T->dynSize;
	unsigned *entries = isStatic ? &T->statEntries : &T->dynEntries;
	if(size == 0){ T->error |= CPG_ERR_BINS; return; }
	unsigned idx = (unsigned)(c.shash[shape] % size);
	int prev = -1, leaf = bins[idx];
	for(int guard = 0; leaf >= 0; guard++){
		if(guard > c.nodeCap){ T->error |= CPG_ERR_BINS; return; }
		if(c.nodes[leaf].obj == shape) break;
		prev = leaf;
		leaf = c.nodes[leaf].binNext;
	}
	if(leaf < 0){ T->error |= CPG_ERR_BINS; return; }
	if(prev >= 0) c.nodes[prev].binNext = c.nodes[leaf].binNext;
	else bins[idx] = c.nodes[leaf].binNext;
	(*entries)--;
	if(isStatic) T->statRoot = subtree_remove(c, T->statRoot, leaf);
	else T->dynRoot = subtree_remove(c, T->dynRoot, leaf);
	pairs_clear(c, leaf);
	node_recycle(c, leaf);
}

/* The leaf of `shape` in the dynamic or the static leaf set, -1 when it
 * is not there (cpHashSetFind). */
__device__ int leaf_find(const TreeCtx &c, int shape, bool isStatic)
{
	const int *bins = isStatic ? c.sbins : c.dbins;
	unsigned size = isStatic ? c.T->statSize : c.T->dynSize;
	if(size == 0) return -1;
	int leaf = bins[(unsigned)(c.shash[shape] % size)];
	for(int guard = 0; leaf >= 0; guard++){
		if(guard > c.nodeCap){ c.T->error |= CPG_ERR_BINS; return -1; }
		if(c.nodes[leaf].obj == shape) return leaf;
		leaf = c.nodes[leaf].binNext;
	}
	return -1;
}

/* LeafUpdate (cpBBTree.c:498-517) against a given box: a leaf whose box
 * no longer holds it is given the new (fattened when dynamic) box and
 * reinserted, its pairs dropped and its stamp set. */
__device__ bool leaf_update_to(TreeCtx &c, int leaf, BB bb, bool isStatic, V2 vel)
{
	cpgTree *T = c.T;
	if(tcontains(node_bb(c.nodes[leaf]), bb)) return false;
	set_node_bb(c.nodes[leaf], isStatic ? bb : fatten(bb, vel));
	if(isStatic){
		int root = subtree_remove(c, T->statRoot, leaf);
		T->statRoot = subtree_insert(c, root, leaf);
	} else {
		int root = subtree_remove(c, T->dynRoot, leaf);
		T->dynRoot = subtree_insert(c, root, leaf);
	}
	pairs_clear(c, leaf);
	c.nodes[leaf].stamp = T->treeStamp;
	return true;
}

/* cpBBTreeReindexObject (cpBBTree.c:676-684) for cpSpaceReindexShape: an
 * updated leaf gets its pairs back (LeafAddPairs, :521-537), and the
 * stamp advances whenever the leaf is found. */
__device__ void tree_reindex(TreeCtx &c, const cpgOp &op)
{
	cpgTree *T = c.T;
	bool isStatic = op.isStatic != 0;
	int leaf = leaf_find(c, op.shape, isStatic);
	if(leaf < 0) return;
	if(leaf_update_to(c, leaf, bbnew(op.l, op.b, op.r, op.t), isStatic, v2(op.vx, op.vy))){
		if(isStatic){
			if(T->dynRoot >= 0) mark_leaf_query(c, T->dynRoot, leaf, true);
		} else {
			mark_leaf(c, leaf, T->statRoot);
		}
	}
	T->treeStamp++;
}

/* cpSpaceReindexStatic (cpSpace.c:654-660): the static tree's
 * cpBBTreeReindexQuery with the void query (cpBBTree.c:638-654): every
 * static leaf, in hash-bin order, updated to its shape's box, then the
 * static tree marked (no static root of its own) and the stamp advanced. */
__device__ void tree_reindex_static(TreeCtx &c)
{
	cpgTree *T = c.T;
	if(T->statRoot < 0) return;
	for(unsigned i = 0; i < T->statSize && (int)i < c.sbinCap; i++){
		int guard = 0;
		for(int n = c.sbins[i]; n >= 0; guard++){
			if(guard > c.nodeCap){ T->error |= CPG_ERR_BINS; return; }
			int next = c.nodes[n].binNext;
			leaf_update_to(c, n, shape_bb(c, c.nodes[n].obj), true, v2(0.0, 0.0));
			n = next;
		}
	}
	mark_subtree(c, T->statRoot, -1);
	T->treeStamp++;
}

/* ------------------------------------------------------------------ */
/* Spatial hash (src/cpSpaceHash.c) for a space that called
 * cpSpaceUseSpatialHash: a single world.  Handles are nodes of the pool
 * and the handle sets are the leaf sets; each grid's cells hold lists of
 * bins (head insertion) from the grid's own bin pool. */
struct GridCtx {
	int *cells;
	int *bh, *bn;           /* bin handle, bin next */
	int cap;
	int *top, *freeBin;
	unsigned *stamp;
	int numcells;
	double celldim;
};

__device__ __forceinline__ GridCtx grid_ctx(const cpgSet &s, cpgTree *T, int which)
{
	GridCtx g;
	g.cells = s.gcells + (size_t)which*s.numcells;
	g.bh = s.gbinHandle + (size_t)which*s.gbinCap;
	g.bn = s.gbinNext + (size_t)which*s.gbinCap;
	g.cap = s.gbinCap;
	g.top = &T->gbinTop[which]; g.freeBin = &T->gbinFree[which];
	g.stamp = &T->gstamp[which];
	g.numcells = s.numcells;
	g.celldim = s.celldim;
	return g;
}

/* hash_func (cpSpaceHash.c:223-227) over cpHashValue */
__device__ __forceinline__ int hash_cell(int x, int y, int n)
{
	unsigned long long hx = (unsigned long long)(long long)x, hy = (unsigned long long)(long long)y;
	return (int)((hx*1640531513ull ^ hy*2654435789ull) % (unsigned long long)n);
}

/* floor_int (cpSpaceHash.c:229-235) */
__device__ __forceinline__ int floor_int(double f)
{
	int i = (int)f;
	return (f < 0.0 && f != (double)i) ? i - 1 : i;
}

__device__ __forceinline__ void grid_clear(GridCtx &g)
{
	for(int i = 0; i < g.numcells; i++) g.cells[i] = -1;
	*g.top = 0; *g.freeBin = -1;
}

__device__ __forceinline__ bool grid_contains(const GridCtx &g, int cell, int hand, int guardMax)
{
	int guard = 0;
	for(int b = g.cells[cell]; b >= 0 && guard <= guardMax; b = g.bn[b], guard++) if(g.bh[b] == hand) return true;
	return false;
}

__device__ __forceinline__ bool grid_push(GridCtx &g, cpgTree *T, int cell, int hand)
{
	int b;
	if(*g.freeBin >= 0){ b = *g.freeBin; *g.freeBin = g.bn[b]; }
	else if(*g.top < g.cap) b = (*g.top)++;
	else { T->error |= CPG_ERR_HASH; return false; }
	g.bh[b] = hand;
	g.bn[b] = g.cells[cell];
	g.cells[cell] = b;
	return true;
}

/* hashHandle (cpSpaceHash.c:237-265) */
__device__ void grid_hash_handle(GridCtx &g, cpgTree *T, int hand, BB bb)
{
	double dim = g.celldim;
	int l = floor_int(bb.l/dim), r = floor_int(bb.r/dim);
	int b = floor_int(bb.b/dim), t = floor_int(bb.t/dim);
	for(int i = l; i <= r; i++){
		for(int j = b; j <= t; j++){
			int cell = hash_cell(i, j, g.numcells);
			if(grid_contains(g, cell, hand, g.cap)) continue;
			if(!grid_push(g, T, cell, hand)) return;
		}
	}
}

/* A removed handle's bins leave every cell (the reference leaves them as
 * orphans that the next query through the cell unlinks,
 * cpSpaceHash.c:330-349; the other bins keep their order either way). */
__device__ void grid_unlink(GridCtx &g, int hand)
{
	for(int i = 0; i < g.numcells; i++){
		int prev = -1;
		int guard = 0;
		for(int b = g.cells[i]; b >= 0 && guard <= g.cap; guard++){
			int next = g.bn[b];
			if(g.bh[b] == hand){
				if(prev >= 0) g.bn[prev] = next; else g.cells[i] = next;
				g.bn[b] = *g.freeBin; *g.freeBin = b;
			} else prev = b;
			b = next;
		}
	}
}

/* cpSpaceHashInsert (cpSpaceHash.c:269-274): a new handle at the head of
 * its bin in the handle set, hashed into the cells of the shape's box */
__device__ void hash_insert(TreeCtx &c, const cpgSet &s, int shape, bool isStatic, BB bb)
{
	cpgTree *T = c.T;
	int hand = node_alloc(c);
	if(hand < 0) return;
	cpgNode &nd = c.nodes[hand];
	nd.obj = shape;
	set_node_bb(nd, bb);
	nd.parent = -1; nd.A = -1; nd.B = -1;
	nd.stamp = 0;
	nd.pairs = -1;
	int *bins = isStatic ? c.sbins : c.dbins;
	unsigned *size = isStatic ? &T->statSize : &T->dynSize;
	unsigned *entries = isStatic ? &T->statEntries : &T->dynEntries;
	unsigned idx = (unsigned)(c.shash[shape] % *size);
	nd.binNext = bins[idx];
	bins[idx] = hand;
	(*entries)++;
	if(*entries >= *size) leafset_resize(c, bins, isStatic ? c.sbinCap : c.dbinCap, size);
	GridCtx g = grid_ctx(s, T, isStatic ? 1 : 0);
	grid_hash_handle(g, T, hand, bb);
}

/* cpSpaceHashRemove (cpSpaceHash.c:300-309); returns whether found */
__device__ bool hash_remove(TreeCtx &c, const cpgSet &s, int shape, bool isStatic)
{
	cpgTree *T = c.T;
	int *bins = isStatic ? c.sbins : c.dbins;
	unsigned size = isStatic ? T->statSize : T->dynSize;
	unsigned *entries = isStatic ? &T->statEntries : &T->dynEntries;
	if(size == 0) return false;
	unsigned idx = (unsigned)(c.shash[shape] % size);
	int prev = -1, hand = bins[idx];
	for(int guard = 0; hand >= 0; guard++){
		if(guard > c.nodeCap){ T->error |= CPG_ERR_BINS; return false; }
		if(c.nodes[hand].obj == shape) break;
		prev = hand;
		hand = c.nodes[hand].binNext;
	}
	if(hand < 0) return false;
	if(prev >= 0) c.nodes[prev].binNext = c.nodes[hand].binNext;
	else bins[idx] = c.nodes[hand].binNext;
	(*entries)--;
	GridCtx g = grid_ctx(s, T, isStatic ? 1 : 0);
	grid_unlink(g, hand);
	node_recycle(c, hand);
	return true;
}

/* cpSpaceHashRehash (cpSpaceHash.c:282-287) of the static grid, each
 * handle hashed again in handle-set order with its shape's box */
__device__ void hash_rehash_static(TreeCtx &c, const cpgSet &s)
{
	cpgTree *T = c.T;
	GridCtx g = grid_ctx(s, T, 1);
	grid_clear(g);
	for(unsigned i = 0; i < T->statSize && (int)i < c.sbinCap; i++){
		int guard = 0;
		for(int n = c.sbins[i]; n >= 0; n = c.nodes[n].binNext){
			if(++guard > c.nodeCap){ T->error |= CPG_ERR_BINS; return; }
			BB bb = shape_bb(c, c.nodes[n].obj);
			set_node_bb(c.nodes[n], bb);
			grid_hash_handle(g, T, n, bb);
		}
	}
}

/* The index edits of a space on the spatial hash (k_apply_ops). */
__device__ void hash_apply_op(TreeCtx &c, const cpgSet &s, const cpgOp &op)
{
	bool isStatic = op.isStatic != 0;
	BB bb = bbnew(op.l, op.b, op.r, op.t);
	if(op.kind == CPG_OP_INSERT) hash_insert(c, s, op.shape, isStatic, bb);
	else if(op.kind == CPG_OP_REMOVE){ if(!hash_remove(c, s, op.shape, isStatic)) c.T->error |= CPG_ERR_BINS; }
	else if(op.kind == CPG_OP_REINDEX){
		/* cpSpaceHashRehashObject (cpSpaceHash.c:276-286): a new handle */
		if(hash_remove(c, s, op.shape, isStatic)) hash_insert(c, s, op.shape, isStatic, bb);
	}
	else if(op.kind == CPG_OP_REINDEX_STATIC) hash_rehash_static(c, s);
}

/* cpSpaceUseSpatialHash (cpSpace.c:687-701): the trees give way to two
 * hashes holding the same shapes, the static ones first, each in its leaf
 * set's order.  The order is kept in the candidate buffer meanwhile. */
__device__ void hash_switch(TreeCtx &c, const cpgSet &s)
{
	cpgTree *T = c.T;
	int *order = (int *)c.cands;
	int cap = c.candCap*(int)(sizeof(cpgCand)/sizeof(int));
	int n = 0, nstat = 0;
	for(int pass = 0; pass < 2; pass++){
		const int *bins = pass == 0 ? c.sbins : c.dbins;
		unsigned size = pass == 0 ? T->statSize : T->dynSize;
		int binCap = pass == 0 ? c.sbinCap : c.dbinCap;
		for(unsigned i = 0; i < size && (int)i < binCap; i++){
			int guard = 0;
			for(int l = bins[i]; l >= 0; l = c.nodes[l].binNext){
				if(++guard > c.nodeCap || n >= cap){ T->error |= CPG_ERR_BINS; return; }
				order[n++] = c.nodes[l].obj;
			}
		}
		if(pass == 0) nstat = n;
	}
	/* fresh pools, sets and grids */
	T->dynRoot = T->statRoot = -1;
	T->freeNode = -1; T->nodeTop = 0;
	T->freePair = -1; T->pairTop = 0;
	T->dynSize = T->statSize = (unsigned)cpg_primes[0];
	T->dynEntries = T->statEntries = 0;
	for(int i = 0; i < c.dbinCap; i++) c.dbins[i] = -1;
	for(int i = 0; i < c.sbinCap; i++) c.sbins[i] = -1;
	for(int w = 0; w < 2; w++){
		GridCtx g = grid_ctx(s, T, w);
		grid_clear(g);
		T->gstamp[w] = 1;
	}
	for(int k = 0; k < n; k++){
		int shape = order[k];
		hash_insert(c, s, shape, k < nstat, shape_bb(c, shape));
	}
}

#ifdef __CUDACC__
/* The nodes' handle fields as the hash step reads them: in the pool, or
 * staged in shared memory as three arrays. */
struct PoolNodes {
	cpgNode *n;
	__device__ __forceinline__ int obj(int i) const { return n[i].obj; }
	__device__ __forceinline__ int next(int i) const { return n[i].binNext; }
	__device__ __forceinline__ unsigned &stamp(int i) const { return n[i].stamp; }
	/* the cell range of a handle's box, computed here */
	__device__ __forceinline__ void range(const TreeCtx &c, int i, double dim, int &l, int &r, int &b, int &t) const
	{
		BB bb = shape_bb(c, n[i].obj);
		l = floor_int(bb.l/dim); r = floor_int(bb.r/dim);
		b = floor_int(bb.b/dim); t = floor_int(bb.t/dim);
	}
};
/* Staged: the ranges were computed by the whole block beforehand (the
 * divisions are the serial walk's slowest part on the FP64 pipe). */
struct StagedNodes {
	int *o, *nx;
	unsigned *st;
	int *rg;                /* 4 per node: l, r, b, t */
	__device__ __forceinline__ int obj(int i) const { return o[i]; }
	__device__ __forceinline__ int next(int i) const { return nx[i]; }
	__device__ __forceinline__ unsigned &stamp(int i) const { return st[i]; }
	__device__ __forceinline__ void range(const TreeCtx &c, int i, double dim, int &l, int &r, int &b, int &t) const
	{
		(void)c; (void)dim;
		l = rg[4*i]; r = rg[4*i + 1]; b = rg[4*i + 2]; t = rg[4*i + 3];
	}
};

/* cpSpaceHashReindexQuery (cpSpaceHash.c:394-441) with cpSpaceCollideShapes
 * as the candidate emitter: each dynamic handle in handle-set order meets
 * the handles already in the cells it covers, then joins them; then each
 * queries the static grid (cpSpatialIndexCollideStatic).  Collision ids
 * start at 0: the hash keeps none.  g and sg are the two grids, wherever
 * their cells and bins are held. */
template <typename Nodes>
__device__ void hash_reindex_query(TreeCtx &c, GridCtx &g, GridCtx &sg, const Nodes &nodes)
{
	cpgTree *T = c.T;
	grid_clear(g);
	for(int pass = 0; pass < 2; pass++){
		if(pass == 1 && T->statEntries == 0) break;
		GridCtx &q = pass == 0 ? g : sg;
		for(unsigned i = 0; i < T->dynSize && (int)i < c.dbinCap; i++){
			int guard = 0;
			for(int hand = c.dbins[i]; hand >= 0; hand = nodes.next(hand)){
				if(++guard > c.nodeCap){ T->error |= CPG_ERR_BINS; return; }
				int obj = nodes.obj(hand);
				int l, r, b, t;
				nodes.range(c, hand, q.celldim, l, r, b, t);
				for(int ci = l; ci <= r; ci++){
					for(int cj = b; cj <= t; cj++){
						int cell = hash_cell(ci, cj, q.numcells);
						if(pass == 0 && grid_contains(q, cell, hand, q.cap)) continue;
						int bguard = 0;
						for(int bn = q.cells[cell]; bn >= 0; bn = q.bn[bn]){
							if(++bguard > q.cap){ T->error |= CPG_ERR_HASH; return; }
							int other = q.bh[bn];
							if(nodes.stamp(other) == *q.stamp || nodes.obj(other) == obj) continue;
							emit(c, obj, nodes.obj(other), -1, 0u);
							nodes.stamp(other) = *q.stamp;
						}
						if(pass == 0 && !grid_push(q, T, cell, hand)) return;
					}
				}
				(*q.stamp)++;
			}
		}
	}
}
#endif

/* cpBBTree.c:498-517: a leaf whose shape left its fattened box */
__device__ __forceinline__ bool leaf_moved(const TreeCtx &c, int leaf)
{
	return !tcontains(node_bb(c.nodes[leaf]), shape_bb(c, c.nodes[leaf].obj));
}

/* clearPairs false: the pairs stay threaded; the parallel marking drops
 * those of every moved leaf at once (cpg_mark.cuh) */
__device__ void leaf_reinsert(TreeCtx &c, int leaf, bool clearPairs = true)
{
	cpgTree *T = c.T;
	set_node_bb(c.nodes[leaf], leaf_fat_bb(c, c.nodes[leaf].obj));
	int root = subtree_remove(c, T->dynRoot, leaf);
	T->dynRoot = subtree_insert(c, root, leaf);
	if(clearPairs) pairs_clear(c, leaf);
	c.nodes[leaf].stamp = T->treeStamp;
}

#ifdef __CUDACC__
/* cpBBTree.c:638-654 (cpBBTreeReindexQuery): every leaf of the hash set,
 * in bin order, is updated (reinserted when its shape left its box), then
 * the tree is marked and the stamp advanced.  A leaf's containment test
 * reads only its own box and its shape's, and the reinsertion of another
 * leaf changes neither, so the threads first test every hash bin and list
 * the leaves that moved, in hash-bin order; thread 0 then reinserts them
 * in that order, which is the serial loop's sequence of tree changes, and
 * marks the tree.  The list lives in the candidate buffer, which
 * marking fills only afterwards (its capacity, 4 ints per candidate, is
 * far above the leaf count).  The whole scan runs before the first
 * reinsertion, so its loads do not evict the tree's top nodes from thread
 * 0's L1 between reinsertions.  Every thread of the block calls it. */
__device__ void tree_reindex_query_block(TreeCtx &c, bool parallelMark = false)
{
	__shared__ int warpTot[32];
	__shared__ int carry, stop;
	__shared__ cpgTree hdr;
	cpgTree *T = c.T;
	int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, warp = tid >> 5, nw = (nt + 31) >> 5;
	int *list = (int *)c.cands;
	long long listCap = 4ll*(long long)c.candCap;
	if(tid == 0){ stop = (T->dynRoot < 0) || (T->error != 0); carry = 0; }
	__syncthreads();
	if(stop){
		if(tid == 0 && T->dynRoot >= 0) T->error |= CPG_ERR_BINS;
		return;
	}
	unsigned size = T->dynSize;
	for(unsigned base = 0; base < size; base += (unsigned)nt){
		unsigned i = base + (unsigned)tid;
		int cnt = 0;
		if(i < size){
			int guard = 0;
			for(int n = c.dbins[i]; n >= 0; n = c.nodes[n].binNext){
				if(++guard > c.nodeCap){ atomicOr(&T->error, CPG_ERR_BINS); break; }
				if(leaf_moved(c, n)) cnt++;
			}
		}
		/* exclusive block scan of the moved counts, after the running total */
		int x = cnt;
		for(int o = 1; o < 32; o <<= 1){
			int y = __shfl_up_sync(0xffffffffu, x, o);
			if(lane >= o) x += y;
		}
		if(lane == 31) warpTot[warp] = x;
		__syncthreads();
		if(tid == 0){
			int acc = carry;
			for(int k = 0; k < nw; k++){ int t = warpTot[k]; warpTot[k] = acc; acc += t; }
			carry = acc;
		}
		__syncthreads();
		if(cnt > 0){
			long long off = (long long)warpTot[warp] + x - cnt;
			int guard = 0;
			for(int n = c.dbins[i]; n >= 0; n = c.nodes[n].binNext){
				if(++guard > c.nodeCap) break;
				if(leaf_moved(c, n)){
					if(off < listCap) list[off] = n;
					off++;
				}
			}
		}
		__syncthreads();
	}
	if(tid == 0){
		/* thread 0 reads and writes the tree header at every reinsertion
		 * and node or pair allocation: it works on a shared-memory copy */
		hdr = *T;
		c.T = &hdr;
		int moved = carry;
		hdr.moved = moved;
		if((long long)moved > listCap) hdr.error |= CPG_ERR_CANDS;
		/* with parallelMark the pairs of moved leaves stay threaded and
		 * k_tree_mark marks the tree (cpg_mark.cuh) */
		for(int k = 0; k < moved && !hdr.error; k++) leaf_reinsert(c, list[k], !parallelMark);
		if(!hdr.error && !parallelMark){
			mark_subtree(c, hdr.dynRoot, hdr.statRoot);
			hdr.treeStamp++;
		}
		*T = hdr;
		c.T = T;
	}
}
#endif
