/*
 * cpg_mark.cuh -- the tree's marking pass (src/cpBBTree.c:418-480,
 * MarkLeafQuery / MarkLeaf / MarkSubtree) in parallel phases that give
 * exactly the serial pass's candidates and pair lists.
 *
 * What makes it possible:
 *  - marking never changes the tree, only the pair lists;
 *  - a leaf's pair list is its pairs newest first (PairInsert threads a pair
 *    at the head of both leaves' lists and PairsClear keeps the order of
 *    the others, cpBBTree.c:150-205);
 *  - a moved leaf (stamp == the tree's stamp) emits its queries' hits of
 *    the "right" kind in traversal order and creates pairs, a leaf that
 *    did not move emits the pairs of its list where it is the second leaf.
 *    Every new pair where a leaf is second comes from a moved leaf before
 *    it in depth-first order, so it is already in the list when the serial
 *    pass visits that leaf.
 *
 * The phases, each over independent items (leaves, pair slots):
 *   1. the reinsertions (serial, by the caller) leave the pairs of moved
 *      leaves in place; mark_filter_list drops them from every list;
 *   2. depth-first ranks of the dynamic leaves (mark_count_up, mark_rank);
 *   3. each moved leaf counts its hits (mark_count_moved), each other leaf
 *      its emissions (mark_count_still);
 *   4. prefix sums in rank order give each leaf its candidate offset and
 *      the creation number of its first new pair (done by the caller);
 *   5. moved leaves write their candidates and new pairs (mark_write_moved);
 *   6. each leaf threads its new pairs, highest creation number first, in
 *      front of its surviving list (mark_link);
 *   7. leaves that did not move emit from their lists (mark_emit_still).
 * Every function writes only its own item's fields (a leaf only its own
 * side of a pair), or counters through MARK_ADD.  Compiled for the device
 * and, by the tests, for the host, where the phases run as plain loops.
 */
#pragma once
#include "cpg_tree.cuh"

#ifdef __CUDA_ARCH__
#define MARK_ADD(p, v) atomicAdd((p), (v))
#define MARK_LOAD(p) __ldcg(p)
#define MARK_FENCE() __threadfence()
#else
static inline int mark_add_host(int *p, int v) { int o = *p; *p += v; return o; }
#define MARK_ADD(p, v) mark_add_host((p), (v))
#define MARK_LOAD(p) (*(p))
#define MARK_FENCE() do {} while(0)
#endif

struct MarkScratch {
	int *cnt;       /* [nodeCap] leaves under an internal node */
	int *arrive;    /* [nodeCap] bottom-up arrivals at an internal node (zeroed) */
	int *rank;      /* [nodeCap] depth-first rank of a dynamic leaf */
	int *oldB;      /* [nodeCap] surviving pairs where the leaf is the second */
	int *inc;       /* [nodeCap] new pairs where the leaf is the second (zeroed) */
	int *incid;     /* [nodeCap + 1] new pairs per leaf, both ends (zeroed) -> offsets */
	int *incCur;    /* [nodeCap] fill cursors (zeroed) */
	int *incEnt;    /* [2 * incCap] (creation number, slot) per incidence */
	int *emit;      /* [leafCap + 1] candidates per leaf by rank -> offsets */
	int *ins;       /* [leafCap + 1] new pairs per leaf by rank -> offsets */
	int *freeSlot;  /* [pairCap] free pair slots, ascending */
	int nFree;      /* free slots below pairTop */
	int pairTop;    /* pairTop before the new pairs */
	int incCap;     /* incidences incEnt holds */
	int rankCap;    /* entries of emit and ins */
};

/* a leaf's rank, or -1 (with the error latched) when out of range */
__device__ __forceinline__ int mark_rank_of(const TreeCtx &c, const MarkScratch &m, int leaf)
{
	int r = m.rank[leaf];
	if(r < 0 || r >= m.rankCap){ c.T->error |= CPG_ERR_NODES; return -1; }
	return r;
}

__device__ __forceinline__ bool mark_moved(const TreeCtx &c, int leaf)
{
	return c.nodes[leaf].stamp == c.T->treeStamp;
}

/* Own side of a pair for leaf x: the prev / next links x's list uses. */
__device__ __forceinline__ void mark_set_links(cpgPair &pr, int x, int prev, int next)
{
	if(MARK_LOAD(&pr.aLeaf) == x){ pr.aPrev = prev; pr.aNext = next; }
	else { pr.bPrev = prev; pr.bNext = next; }
}

/* Phase 1, every leaf (dynamic and static): PairsClear of every moved
 * leaf at once (cpBBTree.c:167-186).  A moved leaf's list empties; any
 * other list keeps, in order, the pairs whose other leaf did not move.
 * Dropped pairs are marked free (pad = 0). */
__device__ void mark_filter_list(TreeCtx &c, MarkScratch &m, int x)
{
	bool xm = mark_moved(c, x);
	int head = -1, prev = -1, ob = 0;
	int p = c.nodes[x].pairs;
	for(int guard = 0; p >= 0; guard++){
		if(guard > c.pairCap){ c.T->error |= CPG_ERR_PAIRS; break; }
		cpgPair &pr = c.pairs[p];
		int pa = MARK_LOAD(&pr.aLeaf), pb = MARK_LOAD(&pr.bLeaf);
		bool isA = (pa == x);
		int next = isA ? MARK_LOAD(&pr.aNext) : MARK_LOAD(&pr.bNext);
		int other = isA ? pb : pa;
		if(xm || mark_moved(c, other)){
			pr.pad = 0;
		} else {
			if(isA) pr.aPrev = prev; else pr.bPrev = prev;
			if(prev >= 0){
				cpgPair &pp = c.pairs[prev];
				if(MARK_LOAD(&pp.aLeaf) == x) pp.aNext = p; else pp.bNext = p;
			} else {
				head = p;
			}
			prev = p;
			if(!isA) ob++;
		}
		p = next;
	}
	if(prev >= 0){
		cpgPair &pp = c.pairs[prev];
		if(MARK_LOAD(&pp.aLeaf) == x) pp.aNext = -1; else pp.bNext = -1;
	}
	c.nodes[x].pairs = head;
	m.oldB[x] = ob;
}

/* Phase 2a, every dynamic leaf: leaf counts of the internal nodes, bottom
 * up; the second child to arrive at a node goes on. */
__device__ void mark_count_up(const TreeCtx &c, MarkScratch &m, int leaf)
{
	int n = leaf;
	for(int guard = 0; guard <= c.nodeCap; guard++){
		int par = c.nodes[n].parent;
		if(par < 0) return;
		MARK_FENCE();
		if(MARK_ADD(&m.arrive[par], 1) == 0) return;
		MARK_FENCE();
		int a = c.nodes[par].A, b = c.nodes[par].B;
		int ca = is_leaf(c, a) ? 1 : MARK_LOAD(&m.cnt[a]);
		int cb = is_leaf(c, b) ? 1 : MARK_LOAD(&m.cnt[b]);
		m.cnt[par] = ca + cb;
		n = par;
	}
}

/* Phase 2b, every dynamic leaf: its rank in MarkSubtree's order (A before
 * B), the leaves under every A sibling on the way up. */
__device__ void mark_rank(const TreeCtx &c, MarkScratch &m, int leaf)
{
	int r = 0, n = leaf;
	for(int guard = 0; guard <= c.nodeCap; guard++){
		int par = c.nodes[n].parent;
		if(par < 0) break;
		if(n == c.nodes[par].B){
			int a = c.nodes[par].A;
			r += is_leaf(c, a) ? 1 : MARK_LOAD(&m.cnt[a]);
		}
		n = par;
	}
	m.rank[leaf] = r;
}

/* The hits of MarkLeaf's queries for moved leaf `leaf`, in the serial
 * pass's order (cpBBTree.c:425-458): the static tree first (left false),
 * then at each ancestor the sibling subtree, left when the leaf came up
 * from the A side.  f(hit, left). */
template<class F>
__device__ void mark_query_hits(const TreeCtx &c, int subtree, int leaf, bool left, F &f)
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
			f(n, left);
		} else {
			if(sp + 2 > CPG_STACK){ c.T->error |= CPG_ERR_NODES; return; }
			stack[sp++] = nd.B;
			stack[sp++] = nd.A;
		}
	}
}

template<class F>
__device__ void mark_hits(const TreeCtx &c, int leaf, int staticRoot, F &f)
{
	if(staticRoot >= 0) mark_query_hits(c, staticRoot, leaf, false, f);
	int guard = 0;
	for(int n = leaf; c.nodes[n].parent >= 0; n = c.nodes[n].parent){
		if(++guard > c.nodeCap){ c.T->error |= CPG_ERR_NODES; return; }
		int par = c.nodes[n].parent;
		if(n == c.nodes[par].A) mark_query_hits(c, c.nodes[par].B, leaf, true, f);
		else mark_query_hits(c, c.nodes[par].A, leaf, false, f);
	}
}

/* Phase 3, every moved leaf: its candidates (hits with left false) and the
 * pairs it creates (every left hit, and right hits on leaves of an older
 * stamp); the new pairs' incidences on both leaves, and on the second
 * leaf of a left hit the new pair it will emit. */
struct MarkCounter {
	const TreeCtx *c;
	MarkScratch *m;
	int leaf, ne, ni;
	__device__ void operator()(int x, bool left)
	{
		if(left){
			ni++;
			MARK_ADD(&m->inc[x], 1);
			MARK_ADD(&m->incid[x], 1);
		} else {
			ne++;
			if(c->nodes[x].stamp < c->nodes[leaf].stamp){
				ni++;
				MARK_ADD(&m->incid[x], 1);
			}
		}
	}
};

__device__ void mark_count_moved(const TreeCtx &c, MarkScratch &m, int leaf, int staticRoot)
{
	MarkCounter f;
	f.c = &c; f.m = &m; f.leaf = leaf; f.ne = 0; f.ni = 0;
	mark_hits(c, leaf, staticRoot, f);
	if(f.ni) MARK_ADD(&m.incid[leaf], f.ni);
	int r = mark_rank_of(c, m, leaf);
	if(r < 0) return;
	m.emit[r] = f.ne;
	m.ins[r] = f.ni;
}

/* Phase 3, every dynamic leaf that did not move: it will emit the new pairs
 * where it is second, then its surviving ones. */
__device__ void mark_count_still(const TreeCtx &c, MarkScratch &m, int leaf)
{
	int r = mark_rank_of(c, m, leaf);
	if(r < 0) return;
	m.emit[r] = MARK_LOAD(&m.inc[leaf]) + m.oldB[leaf];
	m.ins[r] = 0;
}

/* Slot of the new pair with creation number g: the free slots below the
 * old pairTop in ascending order, then fresh ones. */
__device__ __forceinline__ int mark_slot(const MarkScratch &m, int g)
{
	return g < m.nFree ? MARK_LOAD(&m.freeSlot[g]) : m.pairTop + (g - m.nFree);
}

__device__ __forceinline__ void mark_incidence(MarkScratch &m, int x, int g, int slot)
{
	int k = MARK_LOAD(&m.incid[x]) + MARK_ADD(&m.incCur[x], 1);
	if(k < m.incCap){ m.incEnt[2*k] = g; m.incEnt[2*k + 1] = slot; }
}

/* Phase 5, every moved leaf, after the prefix sums (m.emit and m.ins hold
 * offsets, m.incid the incidence offsets): the same hits again, now
 * writing the candidates and the new pairs. */
struct MarkWriter {
	TreeCtx *c;
	MarkScratch *m;
	int leaf, e, g;
	__device__ void make_pair(int a, int b)
	{
		int slot = mark_slot(*m, g);
		cpgPair &pr = c->pairs[slot];
		pr.aPrev = -1; pr.aLeaf = a; pr.aNext = -1;
		pr.bPrev = -1; pr.bLeaf = b; pr.bNext = -1;
		pr.id = 0; pr.pad = 1;
		mark_incidence(*m, a, g, slot);
		mark_incidence(*m, b, g, slot);
		g++;
	}
	__device__ void operator()(int x, bool left)
	{
		if(left){
			make_pair(leaf, x);
		} else {
			if(e < c->candCap){
				cpgCand cd; cd.a = c->nodes[leaf].obj; cd.b = c->nodes[x].obj; cd.pair = -1; cd.idIn = 0u;
				c->cands[e] = cd;
			}
			e++;
			if(c->nodes[x].stamp < c->nodes[leaf].stamp) make_pair(x, leaf);
		}
	}
};

__device__ void mark_write_moved(TreeCtx &c, MarkScratch &m, int leaf, int staticRoot)
{
	MarkWriter f;
	int r = mark_rank_of(c, m, leaf);
	if(r < 0) return;
	f.c = &c; f.m = &m; f.leaf = leaf; f.e = MARK_LOAD(&m.emit[r]); f.g = MARK_LOAD(&m.ins[r]);
	mark_hits(c, leaf, staticRoot, f);
}

/* Phase 6, every leaf with new pairs: they go in front of its surviving
 * list, the last created first, as PairInsert's head insertions leave
 * them. */
__device__ void mark_link(TreeCtx &c, MarkScratch &m, int x)
{
	int k = MARK_LOAD(&m.incCur[x]);
	if(k <= 0) return;
	int lo = MARK_LOAD(&m.incid[x]);
	if(lo + k > m.incCap){ c.T->error |= CPG_ERR_PAIRS; return; }
	int *ent = m.incEnt + 2*lo;
	/* written by other leaves' threads: read past the L1 once */
	for(int i = 0; i < 2*k; i++) ent[i] = MARK_LOAD(&ent[i]);
	/* insertion sort by creation number, descending (lists are short) */
	for(int i = 1; i < k; i++){
		int g = ent[2*i], s = ent[2*i + 1], j = i - 1;
		while(j >= 0 && ent[2*j] < g){ ent[2*j + 2] = ent[2*j]; ent[2*j + 3] = ent[2*j + 1]; j--; }
		ent[2*j + 2] = g; ent[2*j + 3] = s;
	}
	int oldHead = c.nodes[x].pairs;
	for(int i = 0; i < k; i++){
		int prev = i > 0 ? ent[2*i - 1] : -1;
		int next = i + 1 < k ? ent[2*i + 3] : oldHead;
		mark_set_links(c.pairs[ent[2*i + 1]], x, prev, next);
	}
	if(oldHead >= 0){
		cpgPair &oh = c.pairs[oldHead];
		if(MARK_LOAD(&oh.aLeaf) == x) oh.aPrev = ent[2*k - 1]; else oh.bPrev = ent[2*k - 1];
	}
	c.nodes[x].pairs = ent[1];
}

/* Phase 7, every dynamic leaf that did not move: MarkLeaf's list walk
 * (cpBBTree.c:459-468), at its offset. */
__device__ void mark_emit_still(TreeCtx &c, const MarkScratch &m, int leaf)
{
	int r = mark_rank_of(c, m, leaf);
	if(r < 0) return;
	int e = MARK_LOAD(&m.emit[r]);
	int p = c.nodes[leaf].pairs;
	for(int guard = 0; p >= 0; guard++){
		if(guard > c.pairCap){ c.T->error |= CPG_ERR_PAIRS; return; }
		const cpgPair &pr = c.pairs[p];
		int pa = MARK_LOAD(&pr.aLeaf), pb = MARK_LOAD(&pr.bLeaf);
		if(pb == leaf){
			if(e < c.candCap){
				cpgCand cd; cd.a = c.nodes[pa].obj; cd.b = c.nodes[leaf].obj; cd.pair = p; cd.idIn = MARK_LOAD(&pr.id);
				c.cands[e] = cd;
			}
			e++;
			p = MARK_LOAD(&pr.bNext);
		} else {
			p = MARK_LOAD(&pr.aNext);
		}
	}
}
