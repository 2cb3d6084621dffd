// Host check of the tree's parallel marking (chipmunk2d_gb300/csrc/cpg_mark.cuh)
// against the serial marking of the device tree (cpg_tree.cuh), both compiled
// for the host.  A world of moving boxes (plus static walls) is stepped in two
// copies of the tree: one re-indexes and marks serially (the reference's
// cpBBTreeReindexQuery order), the other reinserts the moved leaves with their
// pairs kept and then runs the parallel phases as plain loops.  After every
// step the candidates (shape pair and cached id, in order) and every leaf's
// pair list (as shape pairs and ids, in order) must be identical; pair slot
// numbers may differ.  Prints one line and exits non-zero on a mismatch.
#include <cstdio>
#include <cstdlib>
#include <vector>
#include "host_cuda_shims.h"
#include "cpg_mark.cuh"

static unsigned long long rng = 0x9E3779B97F4A7C15ull;
static double urand()
{
	rng ^= rng << 13; rng ^= rng >> 7; rng ^= rng << 17;
	return (double)(rng >> 11)*(1.0/9007199254740992.0);
}

struct Shapes {
	int n;                          // shapes; the first nstat are static
	int nstat;
	std::vector<double> l, b, r, t, cx, cy, hw, hh, vx, vy;   // boxes, centres, half sizes, velocities
	std::vector<int> body;
	std::vector<unsigned long long> hash;
};

struct Tree {
	std::vector<cpgNode> nodes;
	std::vector<cpgPair> pairs;
	cpgTree T;
	std::vector<int> dbins, sbins;
	std::vector<cpgCand> cands;
};

static TreeCtx ctx(Tree &tr, Shapes &sh)
{
	TreeCtx c;
	c.nodes = tr.nodes.data(); c.pairs = tr.pairs.data();
	c.nodeCap = (int)tr.nodes.size(); c.pairCap = (int)tr.pairs.size();
	c.T = &tr.T;
	c.dbins = tr.dbins.data(); c.sbins = tr.sbins.data();
	c.dbinCap = (int)tr.dbins.size(); c.sbinCap = (int)tr.sbins.size();
	c.bbl = sh.l.data(); c.bbb = sh.b.data(); c.bbr = sh.r.data(); c.bbt = sh.t.data();
	c.sbody = sh.body.data(); c.shash = sh.hash.data();
	c.vx = sh.vx.data(); c.vy = sh.vy.data();
	c.cands = tr.cands.data(); c.candCap = (int)tr.cands.size();
	c.ncand = 0; c.collide = 0;
	return c;
}

static void set_box(Shapes &sh, int i)
{
	sh.l[i] = sh.cx[i] - sh.hw[i]; sh.r[i] = sh.cx[i] + sh.hw[i];
	sh.b[i] = sh.cy[i] - sh.hh[i]; sh.t[i] = sh.cy[i] + sh.hh[i];
}

/* the serial re-index and marking, as the tree kernel did it before the
 * block scan: every leaf in hash-bin order, then MarkSubtree */
static void serial_step(TreeCtx &c)
{
	cpgTree *T = c.T;
	if(T->dynRoot < 0) return;
	for(unsigned i = 0; i < T->dynSize; i++){
		for(int n = c.dbins[i]; n >= 0;){
			int next = c.nodes[n].binNext;
			if(leaf_moved(c, n)) leaf_reinsert(c, n, true);
			n = next;
		}
	}
	c.collide = 1;
	c.ncand = 0;
	mark_subtree(c, T->dynRoot, T->statRoot);
	T->ncand = c.ncand;
	T->treeStamp++;
}

/* the leaves of a hash set, in bin order */
static std::vector<int> leaves_of(const TreeCtx &c, const int *bins, unsigned size)
{
	std::vector<int> out;
	for(unsigned i = 0; i < size; i++) for(int n = bins[i]; n >= 0; n = c.nodes[n].binNext) out.push_back(n);
	return out;
}

static void excl_scan(int *a, int n, int *total)
{
	int acc = 0;
	for(int i = 0; i < n; i++){ int v = a[i]; a[i] = acc; acc += v; }
	if(total) *total = acc;
}

/* the items of a phase in a random order: the phases claim their items are
 * independent, so any order (as threads would run them) gives the same */
static std::vector<int> shuffled(std::vector<int> v)
{
	for(size_t i = v.size(); i > 1; i--){
		size_t j = (size_t)(urand()*(double)i);
		if(j >= i) j = i - 1;
		int t = v[i - 1]; v[i - 1] = v[j]; v[j] = t;
	}
	return v;
}

/* the same step with the moved leaves' pairs kept through the reinsertions
 * and the parallel marking phases run as loops, in phase order, each over
 * its items in a fresh random order */
static void parallel_step(TreeCtx &c)
{
	cpgTree *T = c.T;
	if(T->dynRoot < 0) return;
	std::vector<int> dyn = leaves_of(c, c.dbins, T->dynSize);
	std::vector<int> stat = leaves_of(c, c.sbins, T->statSize);
	std::vector<int> moved;
	for(int n : dyn) if(leaf_moved(c, n)) moved.push_back(n);
	for(int n : moved) leaf_reinsert(c, n, false);

	int nodeCap = c.nodeCap, pairCap = c.pairCap;
	std::vector<int> cnt(nodeCap, 0), arrive(nodeCap, 0), rank(nodeCap, -1), oldB(nodeCap, 0), inc(nodeCap, 0);
	std::vector<int> incid(nodeCap + 1, 0), incCur(nodeCap, 0);
	std::vector<int> emit(dyn.size() + 1, 0), ins(dyn.size() + 1, 0), freeSlot(pairCap, 0);
	MarkScratch m;
	m.cnt = cnt.data(); m.arrive = arrive.data(); m.rank = rank.data(); m.oldB = oldB.data(); m.inc = inc.data();
	m.incid = incid.data(); m.incCur = incCur.data(); m.emit = emit.data(); m.ins = ins.data();
	m.freeSlot = freeSlot.data();
	m.rankCap = (int)dyn.size() + 1;

	/* 1: drop the moved leaves' pairs from every list */
	for(int n : shuffled(dyn)) mark_filter_list(c, m, n);
	for(int n : shuffled(stat)) mark_filter_list(c, m, n);
	/* free slots below pairTop, ascending */
	m.nFree = 0; m.pairTop = T->pairTop;
	for(int p = 0; p < T->pairTop; p++) if(c.pairs[p].pad == 0) freeSlot[m.nFree++] = p;
	/* 2: depth-first ranks */
	for(int n : shuffled(dyn)) mark_count_up(c, m, n);
	for(int n : shuffled(dyn)) mark_rank(c, m, n);
	/* 3: counts (every moved leaf before any leaf that did not move) */
	for(int n : shuffled(moved)) mark_count_moved(c, m, n, T->statRoot);
	for(int n : shuffled(dyn)) if(!mark_moved(c, n)) mark_count_still(c, m, n);
	/* 4: prefix sums */
	int ne = 0, ni = 0, nin = 0;
	excl_scan(emit.data(), (int)dyn.size(), &ne);
	excl_scan(ins.data(), (int)dyn.size(), &ni);
	excl_scan(incid.data(), T->nodeTop, &nin);
	std::vector<int> ent(2*(size_t)(nin > 0 ? nin : 1));
	m.incEnt = ent.data(); m.incCap = nin;
	int fresh = ni > m.nFree ? ni - m.nFree : 0;
	if(ne > c.candCap || T->pairTop + fresh > pairCap){ T->error |= CPG_ERR_CANDS; return; }
	/* 5: candidates and new pairs of the moved leaves */
	for(int n : shuffled(moved)) mark_write_moved(c, m, n, T->statRoot);
	/* 6, 7: new pairs in front of every list, then the leaves that did not
	 * move emit (one phase on the device: a leaf links, then emits) */
	for(int n : shuffled(dyn)){
		mark_link(c, m, n);
		if(!mark_moved(c, n)) mark_emit_still(c, m, n);
	}
	for(int n : shuffled(stat)) mark_link(c, m, n);
	/* the pool: slots past the used free ones stay free, in a list again */
	int left = m.nFree > ni ? m.nFree - ni : 0;
	for(int k = 0; k < left; k++){
		int p = freeSlot[ni + k];
		c.pairs[p].aNext = (k + 1 < left) ? freeSlot[ni + k + 1] : -1;
	}
	T->freePair = left > 0 ? freeSlot[ni] : -1;
	T->pairTop += fresh;
	T->pairsLive = T->pairTop - left;
	T->ncand = ne;
	T->treeStamp++;
}

static long mismatches = 0;
static void fail(const char *what, int step, int k)
{
	if(mismatches < 10) printf("  FAIL step %d: %s (index %d)\n", step, what, k);
	mismatches++;
}

/* each leaf's list as (first shape, second shape, id) in order */
static std::vector<long long> lists_of(const TreeCtx &c, const std::vector<int> &leaves)
{
	std::vector<long long> out;
	for(int x : leaves){
		out.push_back(-1000 - c.nodes[x].obj);
		int p = c.nodes[x].pairs;
		for(int guard = 0; p >= 0 && guard <= c.pairCap; guard++){
			const cpgPair &pr = c.pairs[p];
			out.push_back(((long long)c.nodes[pr.aLeaf].obj << 40) ^ ((long long)c.nodes[pr.bLeaf].obj << 20) ^ (long long)pr.id);
			p = (pr.aLeaf == x) ? pr.aNext : pr.bNext;
		}
	}
	return out;
}

/* the narrow phase's write-back of a cached id into the pair */
static void write_ids(TreeCtx &c, int step)
{
	for(int k = 0; k < c.T->ncand && k < c.candCap; k++){
		const cpgCand &cd = c.cands[k];
		if(cd.pair >= 0) c.pairs[cd.pair].id = (unsigned)(cd.a*7919 + cd.b*104729 + step*31) & 0xFFFFFu;
	}
}

static int run(int ndyn, int nstat, int steps, double speed, unsigned long long seed, double gravity = 0.0)
{
	rng = seed;
	Shapes sh;
	int n = ndyn + nstat;
	sh.n = n; sh.nstat = nstat;
	sh.l.resize(n); sh.b.resize(n); sh.r.resize(n); sh.t.resize(n);
	sh.cx.resize(n); sh.cy.resize(n); sh.hw.resize(n); sh.hh.resize(n);
	sh.body.resize(n); sh.hash.resize(n);
	sh.vx.assign(n, 0.0); sh.vy.assign(n, 0.0);
	double side = 12.0*std::sqrt((double)ndyn);
	for(int i = 0; i < n; i++){
		sh.body[i] = i;
		sh.hash[i] = 1000003ull*(unsigned long long)(i + 1);
		if(i < nstat){
			/* walls of a box, one long bar across the middle */
			int w = i % 5;
			sh.cx[i] = (w == 0) ? 0.5*side : (w == 1) ? 0.5*side : (w == 2) ? 0.0 : (w == 3) ? side : 0.5*side;
			sh.cy[i] = (w == 0) ? 0.0 : (w == 1) ? side : 0.5*side;
			sh.hw[i] = (w <= 1 || w == 4) ? 0.5*side : 1.0;
			sh.hh[i] = (w <= 1 || w == 4) ? 1.0 : 0.5*side;
		} else {
			sh.cx[i] = side*urand(); sh.cy[i] = side*urand();
			sh.hw[i] = 1.0 + 4.0*urand(); sh.hh[i] = 1.0 + 4.0*urand();
			sh.vx[i] = speed*(urand() - 0.5); sh.vy[i] = speed*(urand() - 0.5);
		}
		set_box(sh, i);
	}
	Tree A;
	A.nodes.assign(2*n + 4, cpgNode());
	A.pairs.assign(16*n + 256, cpgPair());
	memset(&A.T, 0, sizeof(A.T));
	A.T.dynRoot = -1; A.T.statRoot = -1; A.T.freeNode = -1; A.T.freePair = -1;
	A.T.dynSize = 5; A.T.statSize = 5;
	A.dbins.assign(49157, -1); A.sbins.assign(49157, -1);
	A.cands.assign(16*n + 256, cpgCand());
	{
		TreeCtx c = ctx(A, sh);
		/* insertions in a mixed order, static and dynamic */
		for(int k = 0; k < n; k++){
			int i = (k*7 + 3) % n;
			cpgOp op; memset(&op, 0, sizeof(op));
			op.shape = i; op.isStatic = (i < nstat);
			op.l = sh.l[i]; op.b = sh.b[i]; op.r = sh.r[i]; op.t = sh.t[i];
			op.vx = sh.vx[i]; op.vy = sh.vy[i];
			tree_insert(c, op);
		}
		if(A.T.error){ printf("  setup error 0x%x\n", A.T.error); return 1; }
	}
	Tree B = A;
	long totalCands = 0, totalMoved = 0;
	for(int step = 1; step <= steps; step++){
		for(int i = nstat; i < n; i++){
			/* wander, bounce off the walls, sometimes stop or jump */
			double u = urand();
			if(u < 0.05){ sh.vx[i] = 0.0; sh.vy[i] = 0.0; }
			else if(u < 0.10){ sh.vx[i] = 4.0*speed*(urand() - 0.5); sh.vy[i] = 4.0*speed*(urand() - 0.5); }
			else { sh.vx[i] += 0.2*speed*(urand() - 0.5); sh.vy[i] += 0.2*speed*(urand() - 0.5); }
			sh.vy[i] -= gravity*0.1;
			sh.cx[i] += sh.vx[i]*0.1; sh.cy[i] += sh.vy[i]*0.1;
			if(sh.cx[i] < 0.0 || sh.cx[i] > side) sh.vx[i] = -sh.vx[i];
			if(gravity > 0.0 && sh.cy[i] < 1.0 + sh.hh[i]){
				/* a pile on the floor: resting boxes keep still */
				sh.cy[i] = 1.0 + sh.hh[i]; sh.vy[i] = 0.0; sh.vx[i] *= 0.5;
				if(urand() < 0.9){ sh.vx[i] = 0.0; }
			} else if(sh.cy[i] < 0.0 || sh.cy[i] > side) sh.vy[i] = -sh.vy[i];
			set_box(sh, i);
		}
		TreeCtx ca = ctx(A, sh), cb = ctx(B, sh);
		for(unsigned i = 0; i < A.T.dynSize; i++) for(int x = ca.dbins[i]; x >= 0; x = ca.nodes[x].binNext) totalMoved += leaf_moved(ca, x);
		serial_step(ca);
		parallel_step(cb);
		if(A.T.error || B.T.error){ printf("  step %d: error flags 0x%x / 0x%x\n", step, A.T.error, B.T.error); return 1; }
		if(A.T.ncand != B.T.ncand){ fail("candidate count", step, A.T.ncand - B.T.ncand); continue; }
		for(int k = 0; k < A.T.ncand; k++){
			const cpgCand &x = A.cands[k], &y = B.cands[k];
			if(x.a != y.a || x.b != y.b || x.idIn != y.idIn || (x.pair < 0) != (y.pair < 0)){ fail("candidate", step, k); break; }
		}
		totalCands += A.T.ncand;
		/* the trees themselves: the same nodes */
		for(int k = 0; k < A.T.nodeTop; k++){
			const cpgNode &x = A.nodes[k], &y = B.nodes[k];
			if(x.parent != y.parent || x.A != y.A || x.B != y.B || x.obj != y.obj || x.stamp != y.stamp ||
				memcmp(&x.l, &y.l, 4*sizeof(double))){ fail("node", step, k); break; }
		}
		std::vector<int> leaves = leaves_of(ca, ca.dbins, A.T.dynSize), sl = leaves_of(ca, ca.sbins, A.T.statSize);
		leaves.insert(leaves.end(), sl.begin(), sl.end());
		if(lists_of(ca, leaves) != lists_of(cb, leaves)) fail("pair lists", step, 0);
		if(A.T.pairsLive != B.T.pairsLive) fail("live pairs", step, A.T.pairsLive - B.T.pairsLive);
		write_ids(ca, step);
		write_ids(cb, step);
	}
	printf("  %d dynamic + %d static shapes, %d steps: %ld candidates, %ld reinsertions\n", ndyn, nstat, steps, totalCands, totalMoved);
	return 0;
}

int main()
{
	int bad = 0;
	bad |= run(300, 5, 60, 2.0, 1);
	bad |= run(2000, 5, 40, 6.0, 2);
	bad |= run(800, 0, 40, 1.0, 3);
	bad |= run(1500, 10, 30, 20.0, 4);
	bad |= run(3000, 5, 80, 3.0, 5, 2.0);
	printf("parallel marking: %ld mismatches\n", mismatches);
	return (bad || mismatches) ? 1 : 0;
}
